// dummy_data.h -- shared scratch fields (reference scihpc/dummy_data.h:10-27).  heaviside,
// sign, delta, grad, curvature, density and viscosity mirror the GPU session's fields of the
// same meaning (downloaded on scihpc_sync_to_host and before VTK writes).
#ifndef SCIHPC_GB300_DUMMY_DATA_H
#define SCIHPC_GB300_DUMMY_DATA_H

#include "global.h"
#include "scalar_data.h"

struct dummy_data {
    DataType ***heaviside;
    DataType ***sign;
    DataType ***delta;
    DataType ***grad;
    DataType ***curvature;
    DataType ***tmp;
    DataType ***u_tmp, ***v_tmp, ***w_tmp;
    DataType ***a, ***b;
    DataType ***a_int, ***b_int;
    DataType ***density, ***viscosity;
};

dummy_data *dummy_data_alloc(scalar_data *f);

#endif
