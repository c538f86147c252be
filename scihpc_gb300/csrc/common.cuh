// common.cuh -- grid description, index helpers and error plumbing shared by all kernels.
//
// Device fields use the reference's logical layout: one contiguous FP64 array per field,
// [Nx][Ny][Nz] with k fastest and ghost width 3 in every active dimension
// (scalar_data.h:12-17, global.cpp:7-19).  Keeping that order makes host<->device copies
// plain memcpys of the reference's data and keeps every boundary fill, line solve and
// stencil expressible in the reference's own indices.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "scihpc_gpu.h"

namespace scihpc {

constexpr int GHC = 3;
// streaming multiprocessors of a GB300 (two dies of 76); used to size small grids
constexpr int NUM_SMS = 152;

struct Dims {
    int ndim;
    int n[3];         // interior cells (1 on inactive axes)
    int N[3];         // with ghosts (1 on inactive axes)
    long long s[3];   // element strides
    double d[3];      // spacing (0 on inactive axes)
    double rd[3];     // 1.0 / d, rounded once on the host (0 on inactive axes)
    double h, dv;     // min spacing, cell volume (structured_grid.cpp:7-134)
    double lo[3];

    __host__ __device__ long long size() const { return (long long)N[0] * N[1] * N[2]; }
    __host__ __device__ long long at(int i, int j, int k) const { return i * s[0] + j * s[1] + k; }
    // array index of interior cell I along axis a (scalar_data.cpp:95-123)
    __host__ __device__ int ix(int a, int I) const { return a < ndim ? I + GHC : I; }
    __host__ __device__ long long interior() const { return (long long)n[0] * n[1] * n[2]; }
};

Dims make_dims(const scihpc_grid *g);

// Unsigned division by a run-time invariant d >= 1 as a multiply-high, an add and shifts
// (T. Granlund, P. Montgomery, "Division by invariant integers using multiplication", 1994):
// with l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1, for every 32-bit u,
// u / d = (t + ((u - t) >> 1)) >> (l - 1) with t = mulhi(m, u).  A hardware-free integer
// division is a long instruction sequence; this is four instructions.
struct FastDiv {
    uint32_t m = 0;
    int l = 0;   // 0: d == 1
    FastDiv() = default;
    explicit FastDiv(uint32_t d) {
        while ((1ull << l) < d) ++l;
        m = uint32_t(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    }
    __host__ __device__ uint32_t div(uint32_t u) const {
        if (l == 0) return u;
#if defined(__CUDA_ARCH__)
        const uint32_t t = __umulhi(m, u);
#else
        const uint32_t t = uint32_t((uint64_t(m) * u) >> 32);
#endif
        return (t + ((u - t) >> 1)) >> (l - 1);
    }
};

// Problem parameters that change from step to step live in device memory so that a
// captured CUDA graph replays correctly (problem_parameters, global.h:25-54).
struct StepScalars {
    double t, dt, dt_old, dt_old2;
    double stable_CFL;
    double lsf_mass0;
    double iter;
    double eta;          // mass-correction coefficient of the last mpls stage
    double mass;         // last lsf_mass
    double red[16];      // reduction results (maxima, sums)
};

#define SCIHPC_CUDA(call)                                                              \
    do {                                                                               \
        cudaError_t err__ = (call);                                                    \
        if (err__ != cudaSuccess) return ::scihpc::cuda_fail(err__, #call, __FILE__, __LINE__); \
    } while (0)

int cuda_fail(cudaError_t e, const char *what, const char *file, int line);
void set_last_error(const char *msg);

inline unsigned blocks_for(long long n, int threads) { return unsigned((n + threads - 1) / threads); }

// Programmatic dependent launch.  A kernel launched by launch_pdl may be scheduled while the
// kernel before it in the stream (or graph) is still finishing; it must call pdl_wait() before
// it touches memory that kernel writes (all kernels here call it first).  pdl_trigger() lets
// the next kernel be scheduled once every block of this one has started.  Both are no-ops for
// a kernel launched the ordinary way.
__device__ __forceinline__ void pdl_wait() {
#if defined(__CUDA_ARCH__)
    asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}
__device__ __forceinline__ void pdl_trigger() {
#if defined(__CUDA_ARCH__)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

// SCIHPC_PDL=0 turns the programmatic attribute off everywhere (ordinary launches of the same
// kernels)
bool pdl_enabled();

template <class... P>
inline void launch_pdl_args(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, bool on, P... a) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = on ? 1 : 0;
    void *args[] = {(void *)&a...};
    cudaLaunchKernelExC(&cfg, (const void *)k, args);
}

// k<<<grid, block, smem, s>>>(args...), as a programmatic dependent launch when `on`; the
// arguments are converted to the kernel's parameter types first
template <class... P, class... A>
inline void launch_pdl(bool on, void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A &&...args) {
    static_assert(sizeof...(P) == sizeof...(A), "argument count");
    launch_pdl_args<P...>(k, grid, block, smem, s, on, static_cast<P>(args)...);
}

// Interior linear index q -> (I, J, K) with K fastest, matching the reference loop nests.
// Linear index -> (I, J, K).  Indices below 2^31 (every grid of practical size) are split
// in 32-bit arithmetic: a 64-bit division is a long instruction sequence on the GPU.
__host__ __device__ inline void split3(long long q, const Dims &D, int &I, int &J, int &K) {
    if (q < (1LL << 31)) {
        const unsigned u = unsigned(q), r = u / unsigned(D.n[2]);
        K = int(u - r * unsigned(D.n[2]));
        J = int(r % unsigned(D.n[1]));
        I = int(r / unsigned(D.n[1]));
        return;
    }
    K = int(q % D.n[2]);
    long long r = q / D.n[2];
    J = int(r % D.n[1]);
    I = int(r / D.n[1]);
}

__host__ __device__ inline void split3_full(long long q, const Dims &D, int &i, int &j, int &k) {
    if (q < (1LL << 31)) {
        const unsigned u = unsigned(q), r = u / unsigned(D.N[2]);
        k = int(u - r * unsigned(D.N[2]));
        j = int(r % unsigned(D.N[1]));
        i = int(r / unsigned(D.N[1]));
        return;
    }
    k = int(q % D.N[2]);
    long long r = q / D.N[2];
    j = int(r % D.N[1]);
    i = int(r / D.N[1]);
}

// ---------------------------------------------------------------- kernels used across files
void launch_bc_fill(const Dims &D, int location, const int *types, const double *values, double *f, cudaStream_t s);
// nf (<= 3) independent fields filled together, one launch per axis: field q at location
// locations[q] with face types types[q][6]; `values` (the faces' bc values) are shared
void launch_bc_fill_many(const Dims &D, int nf, const int *locations, const int *const *types, const double *values,
                         double *const *f, cudaStream_t s);
void launch_extrapolate(const Dims &D, int location, const double *data, double *flux, cudaStream_t s);
void launch_zero_order(const Dims &D, double *f, cudaStream_t s);

}  // namespace scihpc
