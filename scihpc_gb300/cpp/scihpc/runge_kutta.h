// runge_kutta.h -- TVD-RK3 and Euler integrators (reference scihpc/runge_kutta.h:14-22).
// The known (flux, rhs) pairs map to fused GPU stages of the device session; any other pair
// is reported as SCIHPC_ERR_UNSUPPORTED (there is no CPU fallback).
#ifndef SCIHPC_GB300_RUNGE_KUTTA_H
#define SCIHPC_GB300_RUNGE_KUTTA_H

#include "global.h"
#include "scalar_data.h"
#include "wrapper.h"

class runge_kutta {
public:
    runge_kutta(int nx, int ny, int nz);

    DataType ***s1, ***s2, ***s3;   // unused on the GPU path (kept for source compatibility)

    void tvd_rk3(wrapper *f, wrapper *vel, void (*flux)(scalar_data *, vector_data *),
                 void (*rhs)(wrapper *, wrapper *, DataType ***, void (*)(scalar_data *, vector_data *))) const;

    void euler(wrapper *f, wrapper *vel, void (*flux)(scalar_data *, vector_data *),
               void (*rhs)(wrapper *, wrapper *, DataType ***, void (*)(scalar_data *, vector_data *))) const;
};

#endif
