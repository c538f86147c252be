// secorder.cu -- see secorder.cuh.  The stencils and their evaluation order are those of
// second_order_solver.cpp (compiled without FMA contraction, like the reference's CPU build).
#include "secorder.cuh"

namespace scihpc {

namespace {

constexpr int TPB = 256;

// coordinate along axis a of flat cell q, and the stride of axis a
__device__ __forceinline__ int coord(const Dims &D, long long q, int a, long long &st) {
    st = D.s[a];
    if (a == 0) return int(q / D.s[0]);
    if (a == 1) return int((q % D.s[0]) / D.s[1]);
    return int(q % D.s[1]);
}

__global__ void k_sec_central(Dims D, int a, const double *__restrict__ f, double *__restrict__ f1,
                              double *__restrict__ f2) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= D.size()) return;
    long long st;
    const int i = coord(D, q, a, st), N = D.N[a];
    const double d = D.d[a];
    if (i == 0) {
        f1[q] = (-1.5 * f[q] + 2 * f[q + st] - 0.5 * f[q + 2 * st]) / d;
        f2[q] = (2 * f[q] - 5 * f[q + st] + 4 * f[q + 2 * st] - f[q + 3 * st]) / (d * d);
    } else if (i == N - 1) {
        f1[q] = (1.5 * f[q] - 2 * f[q - st] + 0.5 * f[q - 2 * st]) / d;
        f2[q] = (2 * f[q] - 5 * f[q - st] + 4 * f[q - 2 * st] - f[q - 3 * st]) / (d * d);
    } else {
        f1[q] = (f[q + st] - f[q - st]) / (2 * d);
        f2[q] = (f[q + st] - 2 * f[q] + f[q - st]) / (d * d);
    }
}

__global__ void k_sec_upwind(Dims D, int a, const double *__restrict__ f, const double *__restrict__ vel,
                             double *__restrict__ f1, double *__restrict__ f2) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= D.size()) return;
    long long st;
    const int i = coord(D, q, a, st);
    if (i < GHC || i >= GHC + D.n[a]) return;
    const double d = D.d[a];
    if (vel[q] > 0.0) f1[q] = (1.5 * f[q] - 2 * f[q - st] + 0.5 * f[q - 2 * st]) / d;
    else f1[q] = (-1.5 * f[q] + 2 * f[q + st] - 0.5 * f[q + 2 * st]) / d;
    f2[q] = (f[q + st] - 2 * f[q] + f[q - st]) / (d * d);
}

__global__ void k_sec_mixed(Dims D, int b, const double *__restrict__ f, double *__restrict__ out) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= D.size()) return;
    long long st;
    const int i = coord(D, q, b, st), N = D.N[b];
    const double d = D.d[b];
    if (i == 0) out[q] = (-1.5 * f[q] + 2 * f[q + st] - 0.5 * f[q + 2 * st]) / d;
    else if (i == N - 1) out[q] = (1.5 * f[q] - 2 * f[q - st] + 0.5 * f[q - 2 * st]) / d;
    else out[q] = (f[q + st] - f[q - st]) / (2 * d);
}

}  // namespace

void launch_sec_central(const Dims &D, int a, const double *flux, double *f1, double *f2, cudaStream_t s) {
    k_sec_central<<<blocks_for(D.size(), TPB), TPB, 0, s>>>(D, a, flux, f1, f2);
}

void launch_sec_upwind(const Dims &D, int a, const double *flux, const double *vel_a, double *f1, double *f2,
                       cudaStream_t s) {
    k_sec_upwind<<<blocks_for(D.size(), TPB), TPB, 0, s>>>(D, a, flux, vel_a, f1, f2);
}

void launch_sec_mixed(const Dims &D, int b, const double *src, double *out, cudaStream_t s) {
    k_sec_mixed<<<blocks_for(D.size(), TPB), TPB, 0, s>>>(D, b, src, out);
}

}  // namespace scihpc
