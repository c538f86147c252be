// conv.cu -- 3x3 (2D) and 3x3x3 (3D) convolutions (stride 1, zero padding 1) as implicit GEMM on
// the 5th-generation tensor cores: BF16 operands in shared memory, FP32 accumulators in TMEM
// (tcgen05.mma issued by one thread, completion tracked by mbarriers), plus the weight-gradient
// GEMM.
//
// Activations are [pixels][channels] (channels fastest, a multiple of 16), pixels row-major
// over a D x H x W grid (D = 1 in 2D).  Tap t reads pixel (z + dz, y + dy, x + dx): in 2D
// t = 3 (dy + 1) + (dx + 1) (9 taps), in 3D t = 9 (dz + 1) + 3 (dy + 1) + (dx + 1) (27 taps).
//   forward:   Y[p][co] = b[co] + sum_{t, ci} X[p + off(t)][ci] * W[co][t][ci]   (GEMM M = pixels,
//              N = Co, K = taps Ci; optional ReLU; BF16 or FP32 output)
//   data grad: dX[p][ci] = sum_{t, co} dZ[p + off(t)][co] * Wt[ci][t][co] with
//              Wt[ci][t][co] = W[co][taps - 1 - t][ci] -- the forward kernel on transposed weights
//   weights:   dW[co][t][ci] = sum_p X[p + off(t)][ci] * dZ[p][co]   (GEMM M = taps Ci rows
//              (t, ci), N = Co, K = pixels, split over blocks and reduced in fixed order)
//
// Pipeline: a K-step is 16 K-elements (one tap x 16 channels forward, 16 pixels for the
// weights); a stage holds as many K-steps as fit in CONV_STAGE_BYTES, the threads fill one
// stage while the MMAs of the other run, and one thread issues the stage's MMAs back to back,
// so a copy round trip and a block barrier are paid once per stage rather than per MMA.
#include "conv.cuh"
#include "tc.cuh"

namespace scihpc {

namespace {

constexpr int TILE_M = 128;   // pixels (forward) or (tap, ci) rows (weight gradient) per block
constexpr int THREADS = 128;  // four warps: one per 32-lane quarter of TMEM in the epilogue
constexpr int CONV_STAGE_BYTES = 32 * 1024;   // per stage, two stages per block: three blocks per SM

__host__ __device__ inline uint32_t tmem_cols(int n) {
    uint32_t c = 32;
    while (c < uint32_t(n)) c <<= 1;
    return c;
}

// bytes of one K-step's operands (A: 128 rows x 16 K, B: N rows x 16 K) and K-steps per stage
// (no more than the nk steps of the whole reduction)
__host__ __device__ inline int step_bytes(int n) { return TILE_M * 32 + n * 32; }
inline int steps_per_stage(int n, int nk) {
    int s = CONV_STAGE_BYTES / step_bytes(n);
    if (s > nk) s = nk;
    return s < 1 ? 1 : s;
}

// byte offset of the 16-byte chunk (row r, K half kb) of an operand tile with 16 K-elements
__device__ __forceinline__ uint32_t chunk_off(int r, int kb) { return uint32_t(((r >> 3) * 2 + kb) * 128 + (r & 7) * 16); }

// tap t -> (dz, dy, dx)
__device__ __forceinline__ void tap_shift(int t, bool three, int &dz, int &dy, int &dx) {
    dz = 0;
    if (three) {
        dz = t / 9 - 1;
        t -= (dz + 1) * 9;
    }
    dy = t / 3 - 1;
    dx = t - (dy + 1) * 3 - 1;
}

// ------------------------------------------------------------------ forward / data gradient
// X [DHW][Ci] bf16, Wk [N][taps][Ci] bf16 (N output channels), bias [N] or null, out [DHW][N]
template <bool OUT_BF16>
__global__ void __launch_bounds__(THREADS) k_conv(const __nv_bfloat16 *__restrict__ X,
                                                  const __nv_bfloat16 *__restrict__ Wk,
                                                  const float *__restrict__ bias, void *__restrict__ out, int D,
                                                  int H, int W, int Ci, int N, int relu, int sk, int *err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int per = step_bytes(N);
    const long long HW = (long long)H * W, P = HW * D;
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
    int pz = 0, py = 0, px = 0;
    if (p < P) {
        pz = int(p / HW);
        const long long r = p - (long long)pz * HW;
        py = int(r / W);
        px = int(r - (long long)py * W);
    }
    const bool three = D > 1;
    const int taps = three ? 27 : 9;
    const int nch = Ci / 16, nk = taps * nch;
    const int ng = (nk + sk - 1) / sk;
    bool ok = true;
    for (int g = 0; g < ng; ++g) {
        const int s = g & 1;
        // the MMAs two stages back read this buffer; every thread must agree before reuse
        const bool freed = g < 2 || tc::mbar_wait(&mbar[s], uint32_t(((g >> 1) - 1) & 1));
        if (!__syncthreads_and(freed)) {
            ok = false;
            break;
        }
        unsigned char *base = sm + size_t(s) * sk * per;
        const int k0 = g * sk, kn = min(sk, nk - k0);
        for (int j = 0; j < kn; ++j) {
            const int ks = k0 + j;
            const int tap = ks / nch, cc = ks - tap * nch;
            int dz, dy, dx;
            tap_shift(tap, three, dz, dy, dx);
            unsigned char *a = base + j * per, *bt = a + TILE_M * 32;
            {   // A: 16 channels of the shifted pixel, zero outside the grid
                const int zs = pz + dz, ys = py + dy, xs = px + dx;
                const bool in = p < P && zs >= 0 && zs < D && ys >= 0 && ys < H && xs >= 0 && xs < W;
                const __nv_bfloat16 *src = in ? X + (((long long)zs * H + ys) * W + xs) * Ci + cc * 16 : X;
                tc::cp16(a + chunk_off(tid, 0), src, in ? 16u : 0u);
                tc::cp16(a + chunk_off(tid, 1), in ? src + 8 : X, in ? 16u : 0u);
            }
            for (int q = tid; q < 2 * N; q += THREADS) {   // B: 16 K-elements of each output channel
                const int n = q >> 1, kb = q & 1;
                tc::cp16(bt + chunk_off(n, kb), Wk + ((long long)n * taps + tap) * Ci + cc * 16 + kb * 8, 16u);
            }
        }
        tc::cp_commit();
        tc::cp_wait_all();
        tc::fence_async_smem();
        tc::fence_before();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            for (int j = 0; j < kn; ++j) {
                unsigned char *a = base + j * per;
                const uint64_t ad = tc::sdesc(tc::smem_u32(a), 128, 256);
                const uint64_t bd = tc::sdesc(tc::smem_u32(a + TILE_M * 32), 128, 256);
                tc::mma_bf16(tmem, ad, bd, idesc, (k0 + j) > 0 ? 1u : 0u);
            }
            tc::commit(&mbar[s]);
        }
    }
    if (ok) ok = __syncthreads_and(tc::mbar_wait(&mbar[(ng - 1) & 1], uint32_t(((ng - 1) >> 1) & 1)));
    if (!ok) {
        if (lane == 0) atomicExch(err, 1);
    } else {
        tc::fence_after();
        const long long pr = p0 + warp * 32 + lane;   // this thread's row of D
        for (int c = 0; c < N; c += 8) {
            float v[8];
            tc::tmem_ld8(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c), v);
            if (pr < P) {
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

// ------------------------------------------------------------------ forward, halo-tile form
// A block computes a 1 x HT_Y x HT_X tile of output pixels (z, y, x) = 128 rows of the GEMM.
// For each 16-channel chunk of the input it copies the tile's halo (HZ x (HT_Y + 2) x
// (HT_X + 2) pixels) once into shared memory, laid out [z][y][K half][x] x 16 bytes, so that
// the 8 pixels of a tile row are one 8 x 16-byte core matrix.  The A operand of tap
// (dz, dy, dx) is then the halo seen through a shared-memory descriptor that starts at the
// shifted row and column (core matrices 16 bytes apart along x, 160 bytes along K, one halo
// row along M): the taps' MMAs read the same halo and no per-tap copy is made.  The weights of
// all taps of the chunk are staged beside it.  Chunks are double-buffered.
constexpr int HT_X = 8, HT_Y = 16;                 // 8 x 16 = TILE_M pixels
constexpr int HX = HT_X + 2, HY = HT_Y + 2;        // halo extents in x and y
constexpr int HROW = 2 * HX * 16;                  // bytes of one halo row: two K halves of HX pixels
constexpr size_t HALO_SMEM_MAX = 200 * 1024;       // largest two-stage halo launch
static_assert(HT_X * HT_Y == TILE_M, "tile");

__host__ __device__ inline int halo_bytes(bool three) { return (three ? 3 : 1) * HY * HROW; }
__host__ __device__ inline int halo_stage_bytes(bool three, int n) { return halo_bytes(three) + (three ? 27 : 9) * n * 32; }

template <bool OUT_BF16, bool THREE>
__global__ void __launch_bounds__(THREADS) k_conv_halo(const __nv_bfloat16 *__restrict__ X,
                                                       const __nv_bfloat16 *__restrict__ Wk,
                                                       const float *__restrict__ bias, void *__restrict__ out, int D,
                                                       int H, int W, int Ci, int N, int relu, int *err) {
    constexpr int TAPS = THREE ? 27 : 9, HZ = THREE ? 3 : 1;
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int abytes = halo_bytes(THREE), per = halo_stage_bytes(THREE, N);
    const int tiles_x = (W + HT_X - 1) / HT_X, tiles_y = (H + HT_Y - 1) / HT_Y;
    const int tx = blockIdx.x % tiles_x, ty = (blockIdx.x / tiles_x) % tiles_y, z0 = blockIdx.x / (tiles_x * tiles_y);
    const int x0 = tx * HT_X, y0 = ty * HT_Y;
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
    const int nch = Ci / 16;
    bool ok = true;
    for (int g = 0; g < nch; ++g) {
        const int s = g & 1;
        const bool freed = g < 2 || tc::mbar_wait(&mbar[s], uint32_t(((g >> 1) - 1) & 1));
        if (!__syncthreads_and(freed)) {
            ok = false;
            break;
        }
        unsigned char *a = sm + size_t(s) * per, *bt = a + abytes;
        // halo of channels g*16 .. g*16+15: entry e = ((z * HY + y) * HX + x) * 2 + kb
        for (int e = tid; e < HZ * HY * HX * 2; e += THREADS) {
            const int kb = e & 1, v = e >> 1;
            const int x = v % HX, t2 = v / HX, y = t2 % HY, z = t2 / HY;
            const int gz = THREE ? z0 + z - 1 : z0, gy = y0 + y - 1, gx = x0 + x - 1;
            const bool in = gz >= 0 && gz < D && gy >= 0 && gy < H && gx >= 0 && gx < W;
            const __nv_bfloat16 *src = in ? X + (((long long)gz * H + gy) * W + gx) * Ci + g * 16 + kb * 8 : X;
            tc::cp16(a + (z * HY + y) * HROW + kb * (HX * 16) + x * 16, src, in ? 16u : 0u);
        }
        // weights of every tap of the chunk: tap t at t * N * 32, rows n, K halves kb
        for (int q = tid; q < TAPS * N * 2; q += THREADS) {
            const int t = q / (2 * N), r = q - t * 2 * N, n = r >> 1, kb = r & 1;
            tc::cp16(bt + t * N * 32 + chunk_off(n, kb), Wk + ((long long)n * TAPS + t) * Ci + g * 16 + kb * 8, 16u);
        }
        tc::cp_commit();
        tc::cp_wait_all();
        tc::fence_async_smem();
        tc::fence_before();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            for (int t = 0; t < TAPS; ++t) {
                int dz, dy, dx;
                tap_shift(t, THREE, dz, dy, dx);
                const int row = THREE ? (1 + dz) * HY + (1 + dy) : 1 + dy;
                const uint64_t ad = tc::sdesc(tc::smem_u32(a + row * HROW + (1 + dx) * 16), HX * 16, HROW);
                const uint64_t bd = tc::sdesc(tc::smem_u32(bt + t * N * 32), 128, 256);
                tc::mma_bf16(tmem, ad, bd, idesc, (g > 0 || t > 0) ? 1u : 0u);
            }
            tc::commit(&mbar[s]);
        }
    }
    if (ok) ok = __syncthreads_and(tc::mbar_wait(&mbar[(nch - 1) & 1], uint32_t(((nch - 1) >> 1) & 1)));
    if (!ok) {
        if (lane == 0) atomicExch(err, 1);
    } else {
        tc::fence_after();
        const int m = warp * 32 + lane;   // this thread's row of D: tile pixel (m / HT_X, m % HT_X)
        const int gy = y0 + m / HT_X, gx = x0 + m % HT_X;
        const bool inside = gy < H && gx < W;
        const long long pr = ((long long)z0 * H + gy) * W + gx;
        for (int c = 0; c < N; c += 8) {
            float v[8];
            tc::tmem_ld8(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c), v);
            if (inside) {
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
// r = t * Ci + ci over the rows of this block's M tile.
// K runs over pixels, and both operands are stored channels-fastest, so both are MN-major
// tiles for the MMA (transpose bits of the instruction descriptor): every 16-byte chunk of a
// tile is 8 consecutive channels of one pixel, copied straight from X (shifted by the row's
// tap, zero outside the grid) or dZ with cp.async -- no gather, no transpose.  MN-major
// layout without swizzle: a core matrix is 8 K-rows of 16 bytes (8 MN elements); the two core
// matrices along K of one 8-element MN group sit side by side, the MN groups 256 B apart.  As
// for the K-major tiles, the descriptor's leading byte offset is the K step between core
// matrices (128 B) and the stride byte offset the MN step (256 B) (checked against the CPU
// restatement by the weight-gradient tests).
__device__ __forceinline__ uint32_t mn_off(int m0, int k) { return uint32_t((m0 >> 3) * 256 + (k >> 3) * 128 + (k & 7) * 16); }

__global__ void __launch_bounds__(THREADS) k_conv_wgrad(const __nv_bfloat16 *__restrict__ X,
                                                        const __nv_bfloat16 *__restrict__ dZ,
                                                        float *__restrict__ partial, int D, int H, int W, int Ci,
                                                        int N, int pix_per_split, int sk, int *err) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int per = step_bytes(N);
    const long long HW = (long long)H * W, P = HW * D;
    const bool three = D > 1;
    const int taps = three ? 27 : 9;
    const int rows = taps * Ci;
    // this thread's two A chunks: pixel k_a of the K-step, MN groups g_a and g_a + 1 (8 rows each)
    const int k_a = tid >> 3, g_a = (tid & 7) * 2;
    int dzs[2], dys[2], dxs[2], ci0[2];
    bool rv[2];
    for (int u = 0; u < 2; ++u) {
        const int r0 = blockIdx.x * TILE_M + (g_a + u) * 8;
        rv[u] = r0 < rows;
        const int tap = rv[u] ? r0 / Ci : 0;
        ci0[u] = rv[u] ? r0 - tap * Ci : 0;
        tap_shift(tap, three, dzs[u], dys[u], dxs[u]);
    }
    const int ng8 = N >> 3;   // B chunks per K-row
    const long long k0 = (long long)blockIdx.y * pix_per_split;
    const long long k1 = k0 + pix_per_split < P ? k0 + pix_per_split : P;
    const int nk = k1 > k0 ? int((k1 - k0 + 15) / 16) : 0;
    const int ng = (nk + sk - 1) / sk;
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
    const uint32_t idesc = tc::idesc_bf16(TILE_M, N) | (1u << 15) | (1u << 16);   // A and B MN-major
    bool ok = true;
    for (int g = 0; g < ng; ++g) {
        const int s = g & 1;
        const bool freed = g < 2 || tc::mbar_wait(&mbar[s], uint32_t(((g >> 1) - 1) & 1));
        if (!__syncthreads_and(freed)) {
            ok = false;
            break;
        }
        unsigned char *base = sm + size_t(s) * sk * per;
        const int kn = min(sk, nk - g * sk);
        for (int j = 0; j < kn; ++j) {
            const long long kp = k0 + 16LL * (g * sk + j);
            unsigned char *a = base + j * per, *bt = a + TILE_M * 32;
            {   // A: X at the row's shifted pixel, 8 channels per chunk
                const long long p = kp + k_a;
                int z = 0, y = 0, x = 0;
                const bool pin = p < k1;
                if (pin) {
                    z = int(p / HW);
                    const long long rem = p - (long long)z * HW;
                    y = int(rem / W);
                    x = int(rem - (long long)y * W);
                }
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int zs = z + dzs[u], ys = y + dys[u], xs = x + dxs[u];
                    const bool in = pin && rv[u] && zs >= 0 && zs < D && ys >= 0 && ys < H && xs >= 0 && xs < W;
                    const __nv_bfloat16 *src = in ? X + (((long long)zs * H + ys) * W + xs) * Ci + ci0[u] : X;
                    tc::cp16(a + mn_off((g_a + u) * 8, k_a), src, in ? 16u : 0u);
                }
            }
            for (int c = tid; c < 16 * ng8; c += THREADS) {   // B: dZ, 8 output channels per chunk
                const int k = c / ng8, n0 = (c - k * ng8) * 8;
                const long long p = kp + k;
                const bool in = p < k1;
                tc::cp16(bt + mn_off(n0, k), in ? dZ + p * N + n0 : dZ, in ? 16u : 0u);
            }
        }
        tc::cp_commit();
        tc::cp_wait_all();
        tc::fence_async_smem();
        tc::fence_before();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            for (int j = 0; j < kn; ++j) {
                unsigned char *a = base + j * per;
                const uint64_t ad = tc::sdesc(tc::smem_u32(a), 128, 256);
                const uint64_t bd = tc::sdesc(tc::smem_u32(a + TILE_M * 32), 128, 256);
                tc::mma_bf16(tmem, ad, bd, idesc, (g * sk + j) > 0 ? 1u : 0u);
            }
            tc::commit(&mbar[s]);
        }
    }
    if (ok && ng > 0) ok = __syncthreads_and(tc::mbar_wait(&mbar[(ng - 1) & 1], uint32_t(((ng - 1) >> 1) & 1)));
    if (!ok) {
        if (lane == 0) atomicExch(err, 1);
    } else {
        tc::fence_after();
        const int rr = blockIdx.x * TILE_M + warp * 32 + lane;
        float *dst = partial + ((long long)blockIdx.y * rows + rr) * N;
        for (int c = 0; c < N; c += 8) {
            float v[8];
            if (ng > 0) tc::tmem_ld8(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c), v);
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
__global__ void k_wgrad_reduce(const float *__restrict__ partial, float *__restrict__ dW, int rows, int N,
                               int splits) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)rows * N) return;
    const int co = int(i / rows), r = int(i % rows);
    float s = 0.0f;
    for (int k = 0; k < splits; ++k) s += partial[((long long)k * rows + r) * N + co];
    dW[i] = s;   // i = co * taps Ci + t * Ci + ci
}

int forward_impl(const __nv_bfloat16 *X, const __nv_bfloat16 *Wk, const float *bias, void *out, bool out_bf16, int D,
                 int H, int W, int Ci, int N, bool relu, int *err, cudaStream_t s) {
    if (Ci % 16 || N % 16 || N < 16 || N > 256 || D < 1 || H < 1 || W < 1) return SCIHPC_ERR_ARG;
    const bool three = D > 1;
    const int stages = Ci / 16 >= 2 ? 2 : 1;
    const size_t hsm = size_t(stages) * halo_stage_bytes(three, N);
    if (hsm <= HALO_SMEM_MAX) {
        const unsigned tiles = unsigned((W + HT_X - 1) / HT_X) * unsigned((H + HT_Y - 1) / HT_Y) * unsigned(D);
        const int rl = relu ? 1 : 0;
        if (three) {
            if (out_bf16) k_conv_halo<true, true><<<tiles, THREADS, hsm, s>>>(X, Wk, bias, out, D, H, W, Ci, N, rl, err);
            else k_conv_halo<false, true><<<tiles, THREADS, hsm, s>>>(X, Wk, bias, out, D, H, W, Ci, N, rl, err);
        } else {
            if (out_bf16) k_conv_halo<true, false><<<tiles, THREADS, hsm, s>>>(X, Wk, bias, out, D, H, W, Ci, N, rl, err);
            else k_conv_halo<false, false><<<tiles, THREADS, hsm, s>>>(X, Wk, bias, out, D, H, W, Ci, N, rl, err);
        }
        return SCIHPC_OK;
    }
    // the halo and all taps' weights do not fit: one tap per K-step
    const long long P = (long long)D * H * W;
    const unsigned blocks = unsigned((P + TILE_M - 1) / TILE_M);
    const int sk = steps_per_stage(N, (D > 1 ? 27 : 9) * (Ci / 16));
    const size_t smem = size_t(2) * sk * step_bytes(N);
    if (out_bf16)
        k_conv<true><<<blocks, THREADS, smem, s>>>(X, Wk, bias, out, D, H, W, Ci, N, relu ? 1 : 0, sk, err);
    else
        k_conv<false><<<blocks, THREADS, smem, s>>>(X, Wk, bias, out, D, H, W, Ci, N, relu ? 1 : 0, sk, err);
    return SCIHPC_OK;
}

int wgrad_impl(const __nv_bfloat16 *X, const __nv_bfloat16 *dZ, float *partial, float *dW, int D, int H, int W,
               int Ci, int N, int splits, int *err, cudaStream_t s) {
    if (Ci % 16 || N % 16 || N < 16 || N > 256 || splits < 1 || D < 1 || H < 1 || W < 1) return SCIHPC_ERR_ARG;
    const long long P = (long long)D * H * W;
    const int rows = (D > 1 ? 27 : 9) * Ci;
    long long per = (P + splits - 1) / splits;
    per = (per + 15) / 16 * 16;
    const int used = int((P + per - 1) / per);
    const dim3 grid(unsigned((rows + TILE_M - 1) / TILE_M), unsigned(used));
    const int sk = steps_per_stage(N, int((per + 15) / 16));
    k_conv_wgrad<<<grid, THREADS, size_t(2) * sk * step_bytes(N), s>>>(X, dZ, partial, D, H, W, Ci, N, int(per), sk,
                                                                        err);
    const long long tot = (long long)rows * N;
    k_wgrad_reduce<<<unsigned((tot + 255) / 256), 256, 0, s>>>(partial, dW, rows, N, used);
    return SCIHPC_OK;
}

}  // namespace

size_t conv_smem(int n) { return size_t(2) * steps_per_stage(n, 1 << 20) * step_bytes(n); }

int conv3x3_forward(const __nv_bfloat16 *X, const __nv_bfloat16 *Wk, const float *bias, void *out, bool out_bf16,
                    int H, int W, int Ci, int N, bool relu, int *err, cudaStream_t s) {
    return forward_impl(X, Wk, bias, out, out_bf16, 1, H, W, Ci, N, relu, err, s);
}

int conv3x3x3_forward(const __nv_bfloat16 *X, const __nv_bfloat16 *Wk, const float *bias, void *out, bool out_bf16,
                      int D, int H, int W, int Ci, int N, bool relu, int *err, cudaStream_t s) {
    return forward_impl(X, Wk, bias, out, out_bf16, D, H, W, Ci, N, relu, err, s);
}

int conv3x3_wgrad(const __nv_bfloat16 *X, const __nv_bfloat16 *dZ, float *partial, float *dW, int H, int W, int Ci,
                  int N, int splits, int *err, cudaStream_t s) {
    return wgrad_impl(X, dZ, partial, dW, 1, H, W, Ci, N, splits, err, s);
}

int conv3x3x3_wgrad(const __nv_bfloat16 *X, const __nv_bfloat16 *dZ, float *partial, float *dW, int D, int H, int W,
                    int Ci, int N, int splits, int *err, cudaStream_t s) {
    return wgrad_impl(X, dZ, partial, dW, D, H, W, Ci, N, splits, err, s);
}

int conv3x3_init(int) {
    const int hs = int(HALO_SMEM_MAX);
    SCIHPC_CUDA(cudaFuncSetAttribute(k_conv_halo<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, hs));
    SCIHPC_CUDA(cudaFuncSetAttribute(k_conv_halo<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, hs));
    SCIHPC_CUDA(cudaFuncSetAttribute(k_conv_halo<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, hs));
    SCIHPC_CUDA(cudaFuncSetAttribute(k_conv_halo<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, hs));
    const int smem = 2 * CONV_STAGE_BYTES;
    SCIHPC_CUDA(cudaFuncSetAttribute(k_conv<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    SCIHPC_CUDA(cudaFuncSetAttribute(k_conv<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    SCIHPC_CUDA(cudaFuncSetAttribute(k_conv_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    return SCIHPC_OK;
}

}  // namespace scihpc
