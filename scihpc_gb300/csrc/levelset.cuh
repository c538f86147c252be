// levelset.cuh -- launchers of levelset.cu and the device helpers shared with the
// time-step kernels.
#pragma once

#include "common.cuh"

namespace scihpc {

void launch_weno5(const Dims &D, int a, const double *flux, const double *vel, double *out, cudaStream_t s);
void launch_godunov(const Dims &D, const double *phi, const double *sign, double *grad, cudaStream_t s);
// prm = {ls_width, density_ratio, viscosity_ratio, positive_ref}; outputs may be null.
void launch_lsf_fields(const Dims &D, const double *prm, const double *phi, double *H, double *De, double *Sg,
                       double *Rho, double *Mu, cudaStream_t s);
void launch_curvature(const Dims &D, const double *phi, const double *const d[9], double *curv, cudaStream_t s);
void launch_lsf_integral(const Dims &D, const double *prm, const double *phi, int which, double *work,
                         double *partial, double *out, cudaStream_t s);
// stabilized_upon_gradient: grad = Godunov |grad phi|, then phi /= max(grad) on every cell;
// partial: RED_MAX_BLOCKS doubles of scratch, mx: one double (device) receiving the maximum
void launch_stabilize(const Dims &D, double *phi, const double *sign, double *grad, double *partial, double *mx,
                      cudaStream_t s);
void launch_guess_from_history(const Dims &D, const double *old, const double *old2, double *flux, cudaStream_t s);

}  // namespace scihpc
