// secorder.cuh -- the second-order finite differences of second_order_solver
// (second_order_solver.cpp:7-241), element-wise on the GPU (secorder.cu).
#pragma once

#include "common.cuh"

namespace scihpc {

// find_fx/fy/fz(f) (second_order_solver.cpp:14-88): central first and second derivatives of
// flux along axis a on every cell, second-order one-sided at the ends of the ghosted array
void launch_sec_central(const Dims &D, int a, const double *flux, double *f1, double *f2, cudaStream_t s);
// find_fx/fy/fz(f, vel) (:90-151): the second-order one-sided first derivative on the side the
// velocity comes from and the central second derivative, at the interior points of axis a
// (every point of the other axes); entries at axis a's ghost points are left as they are
void launch_sec_upwind(const Dims &D, int a, const double *flux, const double *vel_a, double *f1, double *f2,
                       cudaStream_t s);
// mixed_xy / mixed_yz / mixed_zx (:171-229): the derivative of src along axis b with the first-
// derivative stencils of launch_sec_central (b = 1 of fx, b = 2 of fy, b = 0 of fz)
void launch_sec_mixed(const Dims &D, int b, const double *src, double *out, cudaStream_t s);

}  // namespace scihpc
