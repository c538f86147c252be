// conv.cu -- 3x3 convolution (stride 1, zero padding 1) as implicit GEMM on the 5th-generation
// tensor cores: BF16 operands in shared memory, FP32 accumulators in TMEM (tcgen05.mma issued
// by one thread, completion tracked by mbarriers), plus the weight-gradient GEMM.
//
// Activations are [pixels][channels] (channels fastest, a multiple of 16), pixels row-major
// over an H x W image.  Tap t = 3 * (dy + 1) + (dx + 1) reads pixel (y + dy, x + dx).
//   forward:   Y[p][co] = b[co] + sum_{t, ci} X[p + off(t)][ci] * W[co][t][ci]   (GEMM M = pixels,
//              N = Co, K = 9 Ci; optional ReLU; BF16 or FP32 output)
//   data grad: dX[p][ci] = sum_{t, co} dZ[p + off(t)][co] * Wt[ci][t][co] with
//              Wt[ci][t][co] = W[co][8 - t][ci] -- the forward kernel on transposed weights
//   weights:   dW[co][t][ci] = sum_p X[p + off(t)][ci] * dZ[p][co]   (GEMM M = 9 Ci rows
//              (t, ci), N = Co, K = pixels, split over blocks and reduced in fixed order)
#include "conv.cuh"
#include "tc.cuh"

namespace scihpc {

namespace {

constexpr int TILE_M = 128;   // pixels (forward) or (tap, ci) rows (weight gradient) per block
constexpr int THREADS = 128;  // four warps: one per 32-lane quarter of TMEM in the epilogue

__host__ __device__ inline uint32_t tmem_cols(int n) {
    uint32_t c = 32;
    while (c < uint32_t(n)) c <<= 1;
    return c;
}

// byte offset of the 16-byte chunk (row r, K half kb) of an operand tile with 16 K-elements
__device__ __forceinline__ uint32_t chunk_off(int r, int kb) { return uint32_t(((r >> 3) * 2 + kb) * 128 + (r & 7) * 16); }

// ------------------------------------------------------------------ forward / data gradient
// X [HW][Ci] bf16, Wk [N][9][Ci] bf16 (N output channels), bias [N] or null, out [HW][N]
template <bool OUT_BF16>
__global__ void __launch_bounds__(THREADS) k_conv3x3(const __nv_bfloat16 *__restrict__ X,
                                                     const __nv_bfloat16 *__restrict__ Wk,
                                                     const float *__restrict__ bias, void *__restrict__ out, int H,
                                                     int W, int Ci, int N, int relu, int *err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int stage_a = TILE_M * 32, stage_b = N * 32;   // bytes per stage
    unsigned char *sA[2] = {sm, sm + stage_a + stage_b};
    unsigned char *sB[2] = {sm + stage_a, sm + 2 * stage_a + stage_b};
    const long long HW = (long long)H * W;
    const long long p0 = (long long)blockIdx.x * TILE_M;
    const uint32_t ncols = tmem_cols(N);
    if (tid == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
    }
    if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = tc::idesc_bf16(TILE_M, N);
    // this thread's pixel for the A operand
    const long long p = p0 + tid;
    const int py = p < HW ? int(p / W) : 0, px = p < HW ? int(p % W) : 0;
    const int nch = Ci / 16, nk = 9 * nch;
    bool ok = true;
    for (int ks = 0; ks < nk; ++ks) {
        const int s = ks & 1;
        // the MMA two steps back read this stage; every thread must agree before reuse
        const bool freed = ks < 2 || tc::mbar_wait(&mbar[s], uint32_t(((ks >> 1) - 1) & 1));
        if (!__syncthreads_and(freed)) {
            ok = false;
            break;
        }
        const int tap = ks / nch, cc = ks - tap * nch;
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
        {   // A: 16 channels of the shifted pixel, zero outside the image
            const int ys = py + dy, xs = px + dx;
            const bool in = p < HW && ys >= 0 && ys < H && xs >= 0 && xs < W;
            const __nv_bfloat16 *src = in ? X + ((long long)ys * W + xs) * Ci + cc * 16 : X;
            tc::cp16(sA[s] + chunk_off(tid, 0), src, in ? 16u : 0u);
            tc::cp16(sA[s] + chunk_off(tid, 1), in ? src + 8 : X, in ? 16u : 0u);
        }
        for (int j = tid; j < 2 * N; j += THREADS) {   // B: 16 K-elements of each output channel
            const int n = j >> 1, kb = j & 1;
            tc::cp16(sB[s] + chunk_off(n, kb), Wk + ((long long)n * 9 + tap) * Ci + cc * 16 + kb * 8, 16u);
        }
        tc::cp_commit();
        tc::cp_wait_all();
        tc::fence_async_smem();
        tc::fence_before();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            const uint64_t ad = tc::sdesc(tc::smem_u32(sA[s]), 128, 256);
            const uint64_t bd = tc::sdesc(tc::smem_u32(sB[s]), 128, 256);
            tc::mma_bf16(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
            tc::commit(&mbar[s]);
        }
    }
    if (ok) ok = __syncthreads_and(tc::mbar_wait(&mbar[(nk - 1) & 1], uint32_t(((nk - 1) >> 1) & 1)));
    if (!ok) {
        if (lane == 0) atomicExch(err, 1);
    } else {
        tc::fence_after();
        const long long pr = p0 + warp * 32 + lane;   // this thread's row of D
        for (int c = 0; c < N; c += 8) {
            float v[8];
            tc::tmem_ld8(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c), v);
            if (pr < HW) {
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    if (bias) v[q] += bias[c + q];
                    if (relu) v[q] = fmaxf(v[q], 0.0f);
                }
                if (OUT_BF16) {
                    __nv_bfloat162 h[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) h[q] = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
                    *reinterpret_cast<uint4 *>(static_cast<__nv_bfloat16 *>(out) + pr * N + c) =
                        *reinterpret_cast<uint4 *>(h);
                } else {
                    float4 *o = reinterpret_cast<float4 *>(static_cast<float *>(out) + pr * N + c);
                    o[0] = make_float4(v[0], v[1], v[2], v[3]);
                    o[1] = make_float4(v[4], v[5], v[6], v[7]);
                }
            }
        }
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_free(tmem, ncols);
}

// ------------------------------------------------------------------ weight gradient
// partial[split][r][co] = sum over the split's pixels of X[p + off(t_r)][ci_r] * dZ[p][co],
// r = t * Ci + ci over the rows of this block's M tile
__global__ void __launch_bounds__(THREADS) k_conv3x3_wgrad(const __nv_bfloat16 *__restrict__ X,
                                                           const __nv_bfloat16 *__restrict__ dZ,
                                                           float *__restrict__ partial, int H, int W, int Ci, int N,
                                                           int pix_per_split, int *err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int stage_a = TILE_M * 32, stage_b = N * 32;
    unsigned char *sA[2] = {sm, sm + stage_a + stage_b};
    unsigned char *sB[2] = {sm + stage_a, sm + 2 * stage_a + stage_b};
    const long long HW = (long long)H * W;
    const int rows = 9 * Ci;
    const int r = blockIdx.x * TILE_M + tid;   // this thread's (tap, ci) row of A
    const int tap = r < rows ? r / Ci : 0, ci = r < rows ? r % Ci : 0;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const long long k0 = (long long)blockIdx.y * pix_per_split;
    const long long k1 = k0 + pix_per_split < HW ? k0 + pix_per_split : HW;
    const int nk = int((k1 - k0 + 15) / 16);
    const uint32_t ncols = tmem_cols(N);
    if (tid == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
    }
    if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = tc::idesc_bf16(TILE_M, N);
    bool ok = true;
    for (int ks = 0; ks < nk; ++ks) {
        const int s = ks & 1;
        const bool freed = ks < 2 || tc::mbar_wait(&mbar[s], uint32_t(((ks >> 1) - 1) & 1));
        if (!__syncthreads_and(freed)) {
            ok = false;
            break;
        }
        const long long kp = k0 + 16LL * ks;
        {   // A row: X[p + off][ci] for 16 pixels, transposed into K order
            __align__(16) __nv_bfloat16 v[16];
#pragma unroll
            for (int kk = 0; kk < 16; ++kk) {
                const long long pp = kp + kk;
                __nv_bfloat16 x = __float2bfloat16(0.0f);
                if (r < rows && pp < k1) {
                    const int y = int(pp / W) + dy, xx = int(pp % W) + dx;
                    if (y >= 0 && y < H && xx >= 0 && xx < W) x = X[((long long)y * W + xx) * Ci + ci];
                }
                v[kk] = x;
            }
            *reinterpret_cast<uint4 *>(sA[s] + chunk_off(tid, 0)) = reinterpret_cast<uint4 *>(v)[0];
            *reinterpret_cast<uint4 *>(sA[s] + chunk_off(tid, 1)) = reinterpret_cast<uint4 *>(v)[1];
        }
        for (int n = tid; n < N; n += THREADS) {   // B row: dZ[p][n] for 16 pixels
            __align__(16) __nv_bfloat16 v[16];
#pragma unroll
            for (int kk = 0; kk < 16; ++kk) {
                const long long pp = kp + kk;
                v[kk] = pp < k1 ? dZ[pp * N + n] : __float2bfloat16(0.0f);
            }
            *reinterpret_cast<uint4 *>(sB[s] + chunk_off(n, 0)) = reinterpret_cast<uint4 *>(v)[0];
            *reinterpret_cast<uint4 *>(sB[s] + chunk_off(n, 1)) = reinterpret_cast<uint4 *>(v)[1];
        }
        tc::fence_async_smem();
        tc::fence_before();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            const uint64_t ad = tc::sdesc(tc::smem_u32(sA[s]), 128, 256);
            const uint64_t bd = tc::sdesc(tc::smem_u32(sB[s]), 128, 256);
            tc::mma_bf16(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
            tc::commit(&mbar[s]);
        }
    }
    if (ok && nk > 0) ok = __syncthreads_and(tc::mbar_wait(&mbar[(nk - 1) & 1], uint32_t(((nk - 1) >> 1) & 1)));
    if (!ok) {
        if (lane == 0) atomicExch(err, 1);
    } else {
        tc::fence_after();
        const int rr = blockIdx.x * TILE_M + warp * 32 + lane;
        float *dst = partial + ((long long)blockIdx.y * rows + rr) * N;
        for (int c = 0; c < N; c += 8) {
            float v[8];
            if (nk > 0) tc::tmem_ld8(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c), v);
            else
                for (int q = 0; q < 8; ++q) v[q] = 0.0f;
            if (rr < rows)
#pragma unroll
                for (int q = 0; q < 8; ++q) dst[c + q] = v[q];
        }
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_free(tmem, ncols);
}

// dW[co][t][ci] = sum over splits (fixed order) of partial[split][t * Ci + ci][co]
__global__ void k_wgrad_reduce(const float *__restrict__ partial, float *__restrict__ dW, int Ci, int N, int splits) {
    const int rows = 9 * Ci;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)rows * N) return;
    const int co = int(i / rows), r = int(i % rows);
    float s = 0.0f;
    for (int k = 0; k < splits; ++k) s += partial[((long long)k * rows + r) * N + co];
    dW[i] = s;   // i = co * 9 Ci + t * Ci + ci
}

}  // namespace

size_t conv3x3_smem(int n) { return size_t(2) * (TILE_M * 32 + n * 32); }

int conv3x3_forward(const __nv_bfloat16 *X, const __nv_bfloat16 *Wk, const float *bias, void *out, bool out_bf16,
                    int H, int W, int Ci, int N, bool relu, int *err, cudaStream_t s) {
    if (Ci % 16 || N % 16 || N < 16 || N > 256) return SCIHPC_ERR_ARG;
    const long long HW = (long long)H * W;
    const unsigned blocks = unsigned((HW + TILE_M - 1) / TILE_M);
    const size_t smem = conv3x3_smem(N);
    if (out_bf16)
        k_conv3x3<true><<<blocks, THREADS, smem, s>>>(X, Wk, bias, out, H, W, Ci, N, relu ? 1 : 0, err);
    else
        k_conv3x3<false><<<blocks, THREADS, smem, s>>>(X, Wk, bias, out, H, W, Ci, N, relu ? 1 : 0, err);
    return SCIHPC_OK;
}

int conv3x3_wgrad(const __nv_bfloat16 *X, const __nv_bfloat16 *dZ, float *partial, float *dW, int H, int W, int Ci,
                  int N, int splits, int *err, cudaStream_t s) {
    if (Ci % 16 || N % 16 || N < 16 || N > 256 || splits < 1) return SCIHPC_ERR_ARG;
    const long long HW = (long long)H * W;
    long long per = (HW + splits - 1) / splits;
    per = (per + 15) / 16 * 16;
    const int used = int((HW + per - 1) / per);
    const dim3 grid(unsigned((9 * Ci + TILE_M - 1) / TILE_M), unsigned(used));
    k_conv3x3_wgrad<<<grid, THREADS, conv3x3_smem(N), s>>>(X, dZ, partial, H, W, Ci, N, int(per), err);
    const long long tot = 9LL * Ci * N;
    k_wgrad_reduce<<<unsigned((tot + 255) / 256), 256, 0, s>>>(partial, dW, Ci, N, used);
    return SCIHPC_OK;
}

int conv3x3_init(int max_n) {
    const int smem = int(conv3x3_smem(max_n));
    SCIHPC_CUDA(cudaFuncSetAttribute(k_conv3x3<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    SCIHPC_CUDA(cudaFuncSetAttribute(k_conv3x3<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    SCIHPC_CUDA(cudaFuncSetAttribute(k_conv3x3_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    return SCIHPC_OK;
}

}  // namespace scihpc
