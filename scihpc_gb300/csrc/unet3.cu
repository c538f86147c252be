// unet3.cu -- the learned initial guess for the 3D pressure equation: a 3-level U-Net (16, 32,
// 64 channels, two 3x3x3 convolutions per level, 2 x 2 x 2 average pooling down, nearest
// upsampling and skip concatenation up, ReLU) mapping (density, right-hand side, previous
// pressure) to a correction of the previous pressure.  The network runs at half the
// resolution of the pressure grid: each network voxel sees the average of its 2 x 2 x 2
// pressure cells, and the predicted correction is prolonged piecewise-constant (the multigrid
// that follows removes the high frequencies of the guess's error in its first sweeps).  Every
// convolution -- forward, data gradient and weight gradient -- runs on the tensor cores
// (conv.cu, 27 taps: BF16 operands, FP32 accumulation in TMEM); activations are BF16,
// gradients and master weights FP32, training by Adam.  Channel counts are multiples of 16,
// the K step of a BF16 tcgen05 MMA.
//
// Normalisation (per sample, over the pressure grid's interior): x = (rho - mean rho) /
// std rho, rhs / rms(rhs), pprev / s with s = rms(pprev); the network output o (channel 0 of
// the last layer) gives the guess p = pprev + s * P(o), and training fits o to the average
// over each voxel's cells of (p_solved - pprev) / s.  An untrained (zero) correction
// reproduces the warm start from the previous pressure, and the solve that follows iterates
// to the same tolerance either way.
#include <cmath>
#include <random>
#include <vector>

#include "conv.cuh"
#include "reduce.cuh"
#include "unet.cuh"

namespace scihpc {

namespace {

constexpr int C_IN = 16;   // packed input channels (3 used)
constexpr int TPB = 256;
constexpr int RED_NB = 256;   // blocks of the two-pass reductions
constexpr int BIAS_CHUNKS = 64;

struct LayerDef {
    int in, out, ci, co, relu, level;
};

enum T { X0, E1A, E1, P1, E2A, E2, P2, B1, B2, C2, D2A, D2, C1, D1A, D1, OUT, NT };
static_assert(NT == UNet3::NT, "tensor count");
const int T_LEVEL[NT] = {0, 0, 0, 1, 1, 1, 2, 2, 2, 1, 1, 1, 0, 0, 0, 0};
const int T_CH[NT] = {16, 16, 16, 16, 32, 32, 32, 64, 64, 96, 32, 32, 48, 16, 16, 16};

const LayerDef LAYERS[UNet3::NL] = {
    {X0, E1A, 16, 16, 1, 0}, {E1A, E1, 16, 16, 1, 0}, {P1, E2A, 16, 32, 1, 1}, {E2A, E2, 32, 32, 1, 1},
    {P2, B1, 32, 64, 1, 2},  {B1, B2, 64, 64, 1, 2},  {C2, D2A, 96, 32, 1, 1}, {D2A, D2, 32, 32, 1, 1},
    {C1, D1A, 48, 16, 1, 0}, {D1A, D1, 16, 16, 1, 0}, {D1, OUT, 16, 16, 0, 0}};

struct Grid3 {
    int d, h, w;   // extents of one level (voxel v = (z * h + y) * w + x)
};

__device__ __forceinline__ void decode(long long v, const Grid3 &g, int &z, int &y, int &x) {
    const long long hw = (long long)g.h * g.w;
    z = int(v / hw);
    const long long r = v - (long long)z * hw;
    y = int(r / g.w);
    x = int(r - (long long)y * g.w);
}

// parent voxel (one level coarser) of (z, y, x)
__device__ __forceinline__ long long parent(int z, int y, int x, const Grid3 &g) {
    return ((long long)(z >> 1) * (g.h >> 1) + (y >> 1)) * (g.w >> 1) + (x >> 1);
}

// ------------------------------------------------------------------ elementwise kernels
// y (level + 1) = average of the 8 children in x (level g)
__global__ void k3_pool(const __nv_bfloat16 *__restrict__ x, __nv_bfloat16 *__restrict__ y, Grid3 g, int C) {
    const Grid3 c{g.d / 2, g.h / 2, g.w / 2};
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)c.d * c.h * c.w * C) return;
    const int ch = int(i % C);
    int z, yy, xx;
    decode(i / C, c, z, yy, xx);
    float s = 0.0f;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int e = 0; e < 2; ++e)
                s += __bfloat162float(x[(((long long)(2 * z + a) * g.h + 2 * yy + b) * g.w + 2 * xx + e) * C + ch]);
    y[i] = __float2bfloat16(0.125f * s);
}

// y[v] = concat(u[parent(v)][0:cu], s[v][0:cs]) on level g
__global__ void k3_upcat(const __nv_bfloat16 *__restrict__ u, const __nv_bfloat16 *__restrict__ s,
                         __nv_bfloat16 *__restrict__ y, Grid3 g, int cu, int cs) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int C = cu + cs;
    if (i >= (long long)g.d * g.h * g.w * C) return;
    const int c = int(i % C);
    const long long v = i / C;
    int z, yy, xx;
    decode(v, g, z, yy, xx);
    y[i] = c < cu ? u[parent(z, yy, xx, g) * cu + c] : s[v * cs + (c - cu)];
}

// gu[q][c] = sum of the 8 children gy[..][c] (c < cu); gs[v][c] = gy[v][cu + c]
__global__ void k3_upcat_back(const float *__restrict__ gy, float *__restrict__ gu, float *__restrict__ gs, Grid3 g,
                              int cu, int cs) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int C = cu + cs;
    const Grid3 c{g.d / 2, g.h / 2, g.w / 2};
    const long long nu = (long long)c.d * c.h * c.w * cu, ns = (long long)g.d * g.h * g.w * cs;
    if (i < nu) {
        const int ch = int(i % cu);
        int z, yy, xx;
        decode(i / cu, c, z, yy, xx);
        float s = 0.0f;
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int e = 0; e < 2; ++e)
                    s += gy[(((long long)(2 * z + a) * g.h + 2 * yy + b) * g.w + 2 * xx + e) * C + ch];
        gu[i] = s;
    } else if (i < nu + ns) {
        const long long j = i - nu;
        gs[j] = gy[(j / cs) * C + cu + (j % cs)];
    }
}

// gx[v][c] = base[v][c] + gp[parent(v)][c] / 8
__global__ void k3_poolback_add(const float *__restrict__ gp, const float *__restrict__ base, float *__restrict__ gx,
                                Grid3 g, int C) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)g.d * g.h * g.w * C) return;
    const int c = int(i % C);
    int z, yy, xx;
    decode(i / C, g, z, yy, xx);
    gx[i] = base[i] + 0.125f * gp[parent(z, yy, xx, g) * C + c];
}

// dz = g * (y > 0) (ReLU backward; y null: no ReLU), in BF16 for the tensor-core GEMMs
__global__ void k3_mask(const float *__restrict__ g, const __nv_bfloat16 *__restrict__ y,
                        __nv_bfloat16 *__restrict__ dz, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = (!y || __bfloat162float(y[i]) > 0.0f) ? g[i] : 0.0f;
    dz[i] = __float2bfloat16(v);
}

// part[c][k] = sum of dz[p][c] over voxel chunk k; db[c] = sum over k in order
__global__ void k3_bias_part(const __nv_bfloat16 *__restrict__ dz, double *__restrict__ part, long long P, int C) {
    __shared__ double sh[TPB];
    const int c = blockIdx.x, k = blockIdx.y;
    const long long per = (P + BIAS_CHUNKS - 1) / BIAS_CHUNKS;
    const long long p0 = k * per, p1 = p0 + per < P ? p0 + per : P;
    double s = 0.0;
    for (long long p = p0 + threadIdx.x; p < p1; p += TPB) s += double(__bfloat162float(dz[p * C + c]));
    s = block_reduce<SumOp>(s, sh);
    if (threadIdx.x == 0) part[c * BIAS_CHUNKS + k] = s;
}

__global__ void k3_bias_fin(const double *__restrict__ part, float *__restrict__ db, int C) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    double s = 0.0;
    for (int k = 0; k < BIAS_CHUNKS; ++k) s += part[c * BIAS_CHUNKS + k];
    db[c] = float(s);
}

// per-sample statistics over the pressure grid's interior: sums of rho, rho^2, rhs^2, pprev^2
// per block (fixed order), then mean rho, std rho, rms rhs, rms pprev
__global__ void k3_stats_part(const double *__restrict__ rho, const double *__restrict__ rhs,
                              const double *__restrict__ pprev, Dims D, double *__restrict__ part) {
    __shared__ double sh[TPB];
    const long long n = D.interior();
    const Grid3 g{D.n[0], D.n[1], D.n[2]};
    double a[4] = {0, 0, 0, 0};
    for (long long q = (long long)blockIdx.x * TPB + threadIdx.x; q < n; q += (long long)RED_NB * TPB) {
        int i, j, k;
        decode(q, g, i, j, k);
        const long long c = D.at(i + GHC, j + GHC, k + GHC);
        a[0] += rho[c];
        a[1] += rho[c] * rho[c];
        a[2] += rhs[c] * rhs[c];
        a[3] += pprev ? pprev[c] * pprev[c] : 0.0;
    }
    for (int m = 0; m < 4; ++m) {
        const double r = block_reduce<SumOp>(a[m], sh);
        if (threadIdx.x == 0) part[m * RED_NB + blockIdx.x] = r;
        __syncthreads();
    }
}

__global__ void k3_stats_fin(const double *__restrict__ part, long long n, double *__restrict__ st) {
    if (threadIdx.x != 0) return;
    double r[4];
    for (int m = 0; m < 4; ++m) {
        r[m] = 0.0;
        for (int b = 0; b < RED_NB; ++b) r[m] += part[m * RED_NB + b];
    }
    const double mean = r[0] / n;
    st[0] = mean;
    st[1] = sqrt(fmax(r[1] / n - mean * mean, 0.0)) + 1e-12;
    st[2] = sqrt(r[2] / n) + 1e-300;
    st[3] = sqrt(r[3] / n);
}

// x0[v] = (rho', rhs', pprev', 0 ...) averaged over the 8 pressure cells of network voxel v;
// target t[v] = the average of (pnew - pprev) / s if pnew is given
__global__ void k3_pack(const double *__restrict__ rho, const double *__restrict__ rhs,
                        const double *__restrict__ pprev, const double *__restrict__ pnew, Dims D, Grid3 g,
                        const double *__restrict__ st, __nv_bfloat16 *__restrict__ x0, float *__restrict__ target) {
    const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= (long long)g.d * g.h * g.w) return;
    int z, y, x;
    decode(v, g, z, y, x);
    const double sp = st[3] > 0.0 ? st[3] : 1.0;
    double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int e = 0; e < 2; ++e) {
                const long long c = D.at(2 * z + a + GHC, 2 * y + b + GHC, 2 * x + e + GHC);
                const double pp = pprev ? pprev[c] : 0.0;
                a0 += rho[c];
                a1 += rhs[c];
                a2 += pp;
                if (pnew) a3 += pnew[c] - pp;
            }
    __nv_bfloat16 out[C_IN];
    for (int c = 0; c < C_IN; ++c) out[c] = __float2bfloat16(0.0f);
    out[0] = __float2bfloat16(float((0.125 * a0 - st[0]) / st[1]));
    out[1] = __float2bfloat16(float(0.125 * a1 / st[2]));
    out[2] = __float2bfloat16(float(0.125 * a2 / sp));
    for (int c = 0; c < C_IN; ++c) x0[v * C_IN + c] = out[c];
    if (target) target[v] = float(0.125 * a3 / sp);
}

// guess = pprev + s * out[parent][0] on the interior (other cells copied from pprev, or 0)
__global__ void k3_unpack(const float *__restrict__ out, const double *__restrict__ pprev, Dims D, Grid3 g,
                          const double *__restrict__ st, double *__restrict__ guess) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= D.size()) return;
    guess[q] = pprev ? pprev[q] : 0.0;
    const int i = int(q / D.s[0]) - GHC, j = int((q % D.s[0]) / D.s[1]) - GHC, k = int(q % D.s[1]) - GHC;
    if (i < 0 || i >= D.n[0] || j < 0 || j >= D.n[1] || k < 0 || k >= D.n[2]) return;
    const double sp = st[3] > 0.0 ? st[3] : 1.0;
    guess[q] += sp * double(out[(((long long)(i >> 1) * g.h + (j >> 1)) * g.w + (k >> 1)) * 16]);
}

// loss = mean over voxels of (out[v][0] - t[v])^2; gout = d loss / d out; block sums, then in order
__global__ void k3_loss_part(const float *__restrict__ out, const float *__restrict__ t, float *__restrict__ gout,
                             long long P, double *__restrict__ part) {
    __shared__ double sh[TPB];
    double a = 0.0;
    for (long long p = (long long)blockIdx.x * TPB + threadIdx.x; p < P; p += (long long)RED_NB * TPB) {
        const float d = out[p * 16] - t[p];
        a += double(d) * d;
        gout[p * 16] = 2.0f * d / float(P);
        for (int c = 1; c < 16; ++c) gout[p * 16 + c] = 0.0f;
    }
    a = block_reduce<SumOp>(a, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
}

__global__ void k3_loss_fin(const double *__restrict__ part, long long P, double *__restrict__ loss) {
    if (threadIdx.x != 0) return;
    double s = 0.0;
    for (int b = 0; b < RED_NB; ++b) s += part[b];
    *loss = s / double(P);
}

// BF16 copies of one layer's weights: forward [co][27][ci] and data-gradient [ci][27][co] with
// the taps flipped (t -> 26 - t)
__global__ void k3_weights_bf16(const float *__restrict__ w, __nv_bfloat16 *__restrict__ wb,
                                __nv_bfloat16 *__restrict__ wt, int ci, int co) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= co * 27 * ci) return;
    const int o = i / (27 * ci), r = i % (27 * ci), t = r / ci, c = r % ci;
    const __nv_bfloat16 v = __float2bfloat16(w[i]);
    wb[i] = v;
    wt[((long long)c * 27 + (26 - t)) * co + o] = v;
}

__global__ void k3_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                        float *__restrict__ v, long long n, float lr, float b1, float b2, float c1, float c2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi, vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
}

inline unsigned nblk(long long n, int t = TPB) { return unsigned((n + t - 1) / t); }

}  // namespace

int UNet3::create(int n0, int n1, int n2, unsigned seed) {
    if (n0 % 8 || n1 % 8 || n2 % 8 || n0 < 8 || n1 < 8 || n2 < 8) {
        set_last_error("unet3: grid sides must be multiples of 8");
        return SCIHPC_ERR_ARG;
    }
    const int n[3] = {n0, n1, n2};
    for (int l = 0; l < 3; ++l)
        for (int a = 0; a < 3; ++a) G[l][a] = n[a] >> (l + 1);
    SCIHPC_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    int rc = conv3x3_init(0);
    if (rc) return rc;
    nparam = 0;
    for (int l = 0; l < NL; ++l) {
        woff[l] = nparam;
        nparam += (long long)LAYERS[l].co * 27 * LAYERS[l].ci;
        boff[l] = nparam;
        nparam += LAYERS[l].co;
    }
    auto dalloc = [&](void **p, size_t bytes) -> int {
        SCIHPC_CUDA(cudaMalloc(p, bytes));
        SCIHPC_CUDA(cudaMemset(*p, 0, bytes));
        allocs.push_back(*p);
        return SCIHPC_OK;
    };
    if ((rc = dalloc((void **)&wmaster, nparam * 4)) || (rc = dalloc((void **)&grad, nparam * 4)) ||
        (rc = dalloc((void **)&adam_m, nparam * 4)) || (rc = dalloc((void **)&adam_v, nparam * 4)))
        return rc;
    long long wbf = 0;
    for (int l = 0; l < NL; ++l) wbf += (long long)LAYERS[l].co * 27 * LAYERS[l].ci;
    if ((rc = dalloc((void **)&wb, wbf * 2)) || (rc = dalloc((void **)&wt, wbf * 2))) return rc;
    long long maxact = 0, maxpart = 0;
    for (int t = 0; t < NT; ++t) {
        const long long e = vox(T_LEVEL[t]) * T_CH[t];
        if ((rc = dalloc(&act[t], t == OUT ? e * 4 : e * 2)) || (rc = dalloc((void **)&gact[t], e * 4))) return rc;
        maxact = e > maxact ? e : maxact;
    }
    for (int l = 0; l < NL; ++l) {
        const long long part = (long long)WGRAD_SPLITS * 27 * LAYERS[l].ci * LAYERS[l].co;
        maxpart = part > maxpart ? part : maxpart;
    }
    if ((rc = dalloc((void **)&gskip[0], vox(0) * T_CH[E1] * 4)) ||
        (rc = dalloc((void **)&gskip[1], vox(1) * T_CH[E2] * 4)) || (rc = dalloc((void **)&dz, maxact * 2)) ||
        (rc = dalloc((void **)&partial, maxpart * 4)) || (rc = dalloc((void **)&target, vox(0) * 4)) ||
        (rc = dalloc((void **)&stats, 8 * 8)) || (rc = dalloc((void **)&dred, size_t(4 * RED_NB + 64 * BIAS_CHUNKS) * 8)) ||
        (rc = dalloc((void **)&err, 16)))
        return rc;
    // He-normal weights, zero biases; the last layer starts near zero (guess = previous pressure)
    std::vector<float> hw(size_t(nparam), 0.0f);
    std::mt19937_64 gen(seed);
    for (int l = 0; l < NL; ++l) {
        const double sd = std::sqrt(2.0 / (27.0 * LAYERS[l].ci)) * (l == NL - 1 ? 0.01 : 1.0);
        std::normal_distribution<double> nd(0.0, sd);
        for (long long i = 0; i < (long long)LAYERS[l].co * 27 * LAYERS[l].ci; ++i)
            hw[size_t(woff[l] + i)] = float(nd(gen));
    }
    return set_weights(hw.data(), nparam);
}

void UNet3::destroy() {
    for (void *p : allocs) cudaFree(p);
    allocs.clear();
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
}

int UNet3::set_weights(const float *host, long long n) {
    if (n != nparam) {
        set_last_error("unet_set_weights: wrong parameter count");
        return SCIHPC_ERR_ARG;
    }
    SCIHPC_CUDA(cudaMemcpyAsync(wmaster, host, size_t(n) * 4, cudaMemcpyHostToDevice, stream));
    SCIHPC_CUDA(cudaMemsetAsync(adam_m, 0, size_t(n) * 4, stream));
    SCIHPC_CUDA(cudaMemsetAsync(adam_v, 0, size_t(n) * 4, stream));
    adam_t = 0;
    refresh_bf16();
    SCIHPC_CUDA(cudaStreamSynchronize(stream));
    return SCIHPC_OK;
}

int UNet3::get(float *host, long long n, bool gradient) {
    if (n != nparam) {
        set_last_error("unet: wrong parameter count");
        return SCIHPC_ERR_ARG;
    }
    SCIHPC_CUDA(cudaMemcpyAsync(host, gradient ? grad : wmaster, size_t(n) * 4, cudaMemcpyDeviceToHost, stream));
    SCIHPC_CUDA(cudaStreamSynchronize(stream));
    return SCIHPC_OK;
}

void UNet3::refresh_bf16() {
    long long off = 0;
    for (int l = 0; l < NL; ++l) {
        const int n = LAYERS[l].co * 27 * LAYERS[l].ci;
        k3_weights_bf16<<<nblk(n), TPB, 0, stream>>>(wmaster + woff[l], wb + off, wt + off, LAYERS[l].ci, LAYERS[l].co);
        wb_off[l] = off;
        off += n;
    }
}

int UNet3::forward() {
    auto grid = [&](int lv) { return Grid3{G[lv][0], G[lv][1], G[lv][2]}; };
    auto conv = [&](int l) {
        const LayerDef &L = LAYERS[l];
        const int lv = L.level;
        return conv3x3x3_forward((const __nv_bfloat16 *)act[L.in], wb + wb_off[l], wmaster + boff[l], act[L.out],
                                 L.out != OUT, G[lv][0], G[lv][1], G[lv][2], L.ci, L.co, L.relu != 0, err, stream);
    };
    auto pool = [&](int in, int out) {
        const int lv = T_LEVEL[in];
        const long long n = vox(lv + 1) * T_CH[in];
        k3_pool<<<nblk(n), TPB, 0, stream>>>((const __nv_bfloat16 *)act[in], (__nv_bfloat16 *)act[out], grid(lv),
                                            T_CH[in]);
    };
    auto upcat = [&](int u, int s, int out) {
        const int lv = T_LEVEL[s];
        const long long n = vox(lv) * T_CH[out];
        k3_upcat<<<nblk(n), TPB, 0, stream>>>((const __nv_bfloat16 *)act[u], (const __nv_bfloat16 *)act[s],
                                             (__nv_bfloat16 *)act[out], grid(lv), T_CH[u], T_CH[s]);
    };
    int rc = 0;
    if ((rc = conv(0)) || (rc = conv(1))) return rc;
    pool(E1, P1);
    if ((rc = conv(2)) || (rc = conv(3))) return rc;
    pool(E2, P2);
    if ((rc = conv(4)) || (rc = conv(5))) return rc;
    upcat(B2, E2, C2);
    if ((rc = conv(6)) || (rc = conv(7))) return rc;
    upcat(D2, E1, C1);
    if ((rc = conv(8)) || (rc = conv(9)) || (rc = conv(10))) return rc;
    SCIHPC_CUDA(cudaGetLastError());
    return SCIHPC_OK;
}

// gradient of the loss with respect to every parameter, from gact[OUT] (set by the loss)
int UNet3::backward() {
    auto grid = [&](int lv) { return Grid3{G[lv][0], G[lv][1], G[lv][2]}; };
    int rc = 0;
    // one layer: dZ = g_out * relu'(out); dW, db; g_in = data gradient (unless layer 0)
    auto layer = [&](int l) -> int {
        const LayerDef &L = LAYERS[l];
        const int lv = L.level;
        const long long P = vox(lv);
        const long long n = P * L.co;
        k3_mask<<<nblk(n), TPB, 0, stream>>>(gact[L.out], L.relu ? (const __nv_bfloat16 *)act[L.out] : nullptr, dz, n);
        int r = conv3x3x3_wgrad((const __nv_bfloat16 *)act[L.in], dz, partial, grad + woff[l], G[lv][0], G[lv][1],
                                G[lv][2], L.ci, L.co, WGRAD_SPLITS, err, stream);
        if (r) return r;
        k3_bias_part<<<dim3(unsigned(L.co), BIAS_CHUNKS), TPB, 0, stream>>>(dz, dred, P, L.co);
        k3_bias_fin<<<1, 64, 0, stream>>>(dred, grad + boff[l], L.co);
        if (l == 0) return SCIHPC_OK;
        return conv3x3x3_forward(dz, wt + wb_off[l], nullptr, gact[L.in], false, G[lv][0], G[lv][1], G[lv][2], L.co,
                                 L.ci, false, err, stream);
    };
    auto split = [&](int cat, int u, int s, float *gs) {
        const int lv = T_LEVEL[s];
        const long long n = vox(lv + 1) * T_CH[u] + vox(lv) * T_CH[s];
        k3_upcat_back<<<nblk(n), TPB, 0, stream>>>(gact[cat], gact[u], gs, grid(lv), T_CH[u], T_CH[s]);
    };
    auto poolback = [&](int p, int e, const float *gs) {
        const int lv = T_LEVEL[e];
        const long long n = vox(lv) * T_CH[e];
        k3_poolback_add<<<nblk(n), TPB, 0, stream>>>(gact[p], gs, gact[e], grid(lv), T_CH[e]);
    };
    if ((rc = layer(10)) || (rc = layer(9)) || (rc = layer(8))) return rc;
    split(C1, D2, E1, gskip[0]);
    if ((rc = layer(7)) || (rc = layer(6))) return rc;
    split(C2, B2, E2, gskip[1]);
    if ((rc = layer(5)) || (rc = layer(4))) return rc;
    poolback(P2, E2, gskip[1]);
    if ((rc = layer(3)) || (rc = layer(2))) return rc;
    poolback(P1, E1, gskip[0]);
    if ((rc = layer(1)) || (rc = layer(0))) return rc;
    SCIHPC_CUDA(cudaGetLastError());
    return SCIHPC_OK;
}

int UNet3::prepare(const Dims &D, const double *rho, const double *rhs, const double *pprev, const double *pnew) {
    if (D.ndim != 3 || D.n[0] != 2 * G[0][0] || D.n[1] != 2 * G[0][1] || D.n[2] != 2 * G[0][2]) {
        set_last_error("unet3: grid does not match the network's size");
        return SCIHPC_ERR_ARG;
    }
    k3_stats_part<<<RED_NB, TPB, 0, stream>>>(rho, rhs, pprev, D, dred);
    k3_stats_fin<<<1, 32, 0, stream>>>(dred, D.interior(), stats);
    const Grid3 g{G[0][0], G[0][1], G[0][2]};
    k3_pack<<<nblk(vox(0)), TPB, 0, stream>>>(rho, rhs, pprev, pnew, D, g, stats, (__nv_bfloat16 *)act[X0],
                                             pnew ? target : nullptr);
    return SCIHPC_OK;
}

int UNet3::check_err() {
    int h = 0;
    SCIHPC_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    SCIHPC_CUDA(cudaStreamSynchronize(stream));
    if (h) {
        set_last_error("unet3: a tensor-core barrier wait timed out");
        return SCIHPC_ERR_CUDA;
    }
    return SCIHPC_OK;
}

int UNet3::infer(const Dims &D, const double *rho, const double *rhs, const double *pprev, double *guess) {
    int rc = prepare(D, rho, rhs, pprev, nullptr);
    if (rc || (rc = forward())) return rc;
    const Grid3 g{G[0][0], G[0][1], G[0][2]};
    k3_unpack<<<nblk(D.size()), TPB, 0, stream>>>((const float *)act[OUT], pprev, D, g, stats, guess);
    SCIHPC_CUDA(cudaGetLastError());
    return check_err();
}

int UNet3::loss_grad(const Dims &D, const double *rho, const double *rhs, const double *pprev, const double *pnew,
                     double *loss) {
    int rc = prepare(D, rho, rhs, pprev, pnew);
    if (rc || (rc = forward())) return rc;
    k3_loss_part<<<RED_NB, TPB, 0, stream>>>((const float *)act[OUT], target, gact[OUT], vox(0), dred);
    k3_loss_fin<<<1, 32, 0, stream>>>(dred, vox(0), stats + 4);
    if ((rc = backward())) return rc;
    SCIHPC_CUDA(cudaMemcpyAsync(loss, stats + 4, sizeof(double), cudaMemcpyDeviceToHost, stream));
    return check_err();
}

int UNet3::train_step(const Dims &D, const double *rho, const double *rhs, const double *pprev, const double *pnew,
                      float lr, double *loss) {
    int rc = loss_grad(D, rho, rhs, pprev, pnew, loss);
    if (rc) return rc;
    ++adam_t;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, float(adam_t)), c2 = 1.0f - std::pow(b2, float(adam_t));
    k3_adam<<<nblk(nparam), TPB, 0, stream>>>(wmaster, grad, adam_m, adam_v, nparam, lr, b1, b2, c1, c2);
    refresh_bf16();
    SCIHPC_CUDA(cudaGetLastError());
    return SCIHPC_OK;
}

}  // namespace scihpc
