// noalloc.cu -- enclosed mass / volume of a level set without any device allocation.
//
// Some callers cannot call cudaMalloc: plugins inside a host application that owns all
// device memory through its own pool (a stray cudaMalloc there can exceed the host's
// memory budget or fragment its pool), and real-time loops that must not touch the
// allocator (cudaMalloc and cudaFree can synchronise the device and take milliseconds).
// For them this file
// offers scihpc_lsf_integrals_noalloc, the same kernels as scihpc_lsf_integrals with their
// scratch (one product field plus the block partial sums) in a file-scope __device__
// array instead of a context allocation.
//
// Limits and sharing:
//   - The array holds NOALLOC_MAX_CELLS ghosted cells (8 MiB of FP64, held by every GPU that
//     loads this library until the process exits); larger grids are rejected.
//   - Every call uses the same array, so calls that overlap on the GPU (different streams,
//     or host threads) race on it and must be serialised by the caller.  Each call writes
//     every scratch entry it reads before reading it, so leftovers of a previous call do
//     not matter.
//   - The first call on each device resolves the array's device address with
//     cudaGetSymbolAddress (a host-side symbol is only a stand-in, never a device address).
#include <mutex>

#include "common.cuh"
#include "levelset.cuh"
#include "reduce.cuh"

namespace scihpc {

namespace {

constexpr long long NOALLOC_MAX_CELLS = 1LL << 20;
constexpr long long NOALLOC_SCRATCH = NOALLOC_MAX_CELLS + RED_MAX_BLOCKS + 8;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH];

constexpr int MAX_DEVICES = 64;
std::mutex g_mutex;
double *g_dev_ptr[MAX_DEVICES] = {};

// Device address of the scratch array on the current device (resolved once per device).
int scratch_address(double **out) {
    int dev = 0;
    SCIHPC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) {
        set_last_error("lsf_integrals_noalloc: device ordinal out of range");
        return SCIHPC_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_dev_ptr[dev]) {
        void *p = nullptr;
        SCIHPC_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_dev_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_dev_ptr[dev];
    return SCIHPC_OK;
}

}  // namespace

}  // namespace scihpc

using namespace scihpc;

extern "C" int scihpc_lsf_integrals_noalloc(const scihpc_grid *grid, const double prm[4], const double *phi,
                                            double out[2], void *stream) {
    if (!grid || !prm || !phi || !out || grid->ndim < 2 || grid->ndim > 3) {
        set_last_error("lsf_integrals_noalloc: NULL argument or ndim not 2 or 3");
        return SCIHPC_ERR_ARG;
    }
    for (int a = 0; a < grid->ndim; ++a) {
        if (grid->n[a] < 3 || !(grid->hi[a] > grid->lo[a])) {
            set_last_error("lsf_integrals_noalloc: every active axis needs n >= 3 and hi > lo");
            return SCIHPC_ERR_ARG;
        }
    }
    const Dims D = make_dims(grid);
    if (D.size() > NOALLOC_MAX_CELLS) {
        set_last_error("lsf_integrals_noalloc: grid exceeds the static scratch of 1048576 ghosted cells "
                       "(use scihpc_lsf_integrals with a context instead)");
        return SCIHPC_ERR_ARG;
    }
    double *base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    double *work = base, *partial = base + NOALLOC_MAX_CELLS, *red = partial + RED_MAX_BLOCKS;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    launch_lsf_integral(D, prm, phi, 0, work, partial, red, s);
    launch_lsf_integral(D, prm, phi, 1, work, partial, red + 1, s);
    SCIHPC_CUDA(cudaGetLastError());
    double h[2];
    SCIHPC_CUDA(cudaMemcpyAsync(h, red, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    SCIHPC_CUDA(cudaStreamSynchronize(s));
    out[0] = h[0] * D.dv;   // wrapper_func.cpp:510
    out[1] = h[1] * D.dv;   // wrapper_func.cpp:571
    return SCIHPC_OK;
}
