// transport.cu -- see transport.cuh.  Element-wise over the whole ghosted array, as the
// reference's loops are (they run over Nx x Ny x Nz); the sums follow the reference's order
// (x term, then minus the y term, then minus the z term) and the stage formulas its grouping.
#include "transport.cuh"

namespace scihpc {

namespace {

constexpr int TPB = 256;

__global__ void k_flux_fill(long long n, int kind, const double *__restrict__ phi, double *__restrict__ flux) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = phi[i];
    flux[i] = kind == 1 ? v * v * 0.5 : v;
}

struct Ptr3 {
    const double *p[3];
};

__global__ void k_rk3_stage(long long n, int ndim, int stage, int rhs_kind, double dt, double *__restrict__ phi,
                            Ptr3 d, Ptr3 vel, double *__restrict__ s1, double *__restrict__ s2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = rhs_kind == 0 ? -vel.p[0][i] * d.p[0][i] : -d.p[0][i];
    if (ndim > 1) s -= rhs_kind == 0 ? vel.p[1][i] * d.p[1][i] : d.p[1][i];
    if (ndim > 2) s -= rhs_kind == 0 ? vel.p[2][i] * d.p[2][i] : d.p[2][i];
    double f = phi[i];
    if (stage <= 1) {
        f += dt * s;
        if (stage == 1) s1[i] = s;
    } else if (stage == 2) {
        f += dt * (s - 3.0 * s1[i]) / 4.0;
        s2[i] = s;
    } else {
        f += dt * (-s1[i] - s2[i] + 8.0 * s) / 12.0;
    }
    phi[i] = f;
}

}  // namespace

void launch_flux_fill(const Dims &D, int kind, const double *phi, double *flux, cudaStream_t s) {
    const long long n = D.size();
    k_flux_fill<<<blocks_for(n, TPB), TPB, 0, s>>>(n, kind, phi, flux);
}

void launch_rk3_stage(const Dims &D, int stage, int rhs_kind, double dt, double *phi, const double *const d[3],
                      const double *const vel[3], double *s1, double *s2, cudaStream_t s) {
    const long long n = D.size();
    Ptr3 dp{{d[0], D.ndim > 1 ? d[1] : d[0], D.ndim > 2 ? d[2] : d[0]}};
    Ptr3 vp{{vel ? vel[0] : d[0], vel && D.ndim > 1 ? vel[1] : d[0], vel && D.ndim > 2 ? vel[2] : d[0]}};
    k_rk3_stage<<<blocks_for(n, TPB), TPB, 0, s>>>(n, D.ndim, stage, rhs_kind, dt, phi, dp, vp, s1, s2);
}

}  // namespace scihpc
