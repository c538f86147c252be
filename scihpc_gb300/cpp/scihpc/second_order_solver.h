// second_order_solver.h -- second-order finite differences (reference
// scihpc/second_order_solver.h:11-40): central first and second derivatives with one-sided
// ends (find_fx/fy/fz(f)), the upwind-biased first derivative (find_fx/fy/fz(f, vel)) and the
// mixed derivatives.  Each call runs on the GPU on the scalar's host arrays (flux in; fx..,
// fxx.., fxy.. out; scihpc_sec_derivative / scihpc_sec_mixed) and returns with them updated.
// Inside projection_method::find_source_sec the GPU session uses the same stencils directly.
#ifndef SCIHPC_GB300_SECOND_ORDER_SOLVER_H
#define SCIHPC_GB300_SECOND_ORDER_SOLVER_H

#include "global.h"
#include "scalar_data.h"
#include "vector_data.h"

class second_order_solver {
public:
    DataType dx, dy, dz;

    void find_fx(scalar_data *f) const;
    void find_fy(scalar_data *f) const;
    void find_fz(scalar_data *f) const;
    void mixed_xy(scalar_data *f) const;
    void mixed_yz(scalar_data *f) const;
    void mixed_zx(scalar_data *f) const;
    void find_fx(scalar_data *f, vector_data *vel) const;
    void find_fy(scalar_data *f, vector_data *vel) const;
    void find_fz(scalar_data *f, vector_data *vel) const;
    void find_derivatives(scalar_data *f) const;
    void find_derivatives(scalar_data *f, vector_data *vel) const;
    void find_derivatives_all(scalar_data *f) const;

    second_order_solver(DataType _dx, DataType _dy, DataType _dz);
};

#endif
