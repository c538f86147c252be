// unet.cu -- learned initial guess for the pressure equation: a 4-level 2D U-Net (16, 32, 64,
// 128 channels, two 3x3 convolutions per level, average pooling down, nearest upsampling and
// skip concatenation up, ReLU) mapping (density, right-hand side, previous pressure) to a
// correction of the previous pressure.  Every convolution -- forward, data gradient and weight
// gradient -- runs on the tensor cores (conv.cu: BF16 operands, FP32 accumulation in TMEM);
// activations are BF16, gradients and master weights FP32, training by Adam.
//
// Normalisation (per sample): x0 = (rho - mean rho) / std rho, rhs / rms(rhs), pprev / s with
// s = rms(pprev); the network output o (channel 0 of the last layer) gives the guess
// p = pprev + s * o, and training fits o to (p_solved - pprev) / s.  An untrained (zero)
// correction therefore reproduces the usual warm start from the previous pressure, and the
// multigrid solve that follows always iterates to the same tolerance: the network can only
// change how many cycles that takes.
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "conv.cuh"
#include "reduce.cuh"
#include "unet.cuh"

namespace scihpc {

namespace {

constexpr int C_IN = 16;   // packed input channels (3 used)
constexpr int TPB = 256;
constexpr int RED_NB = 256;   // blocks of the two-pass (block sums, then in block order) reductions

struct LayerDef {
    int in, out, ci, co, relu, level;
};

// activation tensors (BF16 unless noted)
enum T {
    X0, E1A, E1, P1, E2A, E2, P2, E3A, E3, P3, B1, B2, C3, D3A, D3, C2, D2A, D2, C1, D1A, D1, OUT, NT
};
const int T_LEVEL[NT] = {0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 2, 2, 2, 1, 1, 1, 0, 0, 0, 0};
const int T_CH[NT] = {16, 16, 16, 16, 32, 32, 32, 64, 64, 64, 128, 128, 192, 64, 64, 96, 32, 32, 48, 16, 16, 16};

const LayerDef LAYERS[UNet::NL] = {
    {X0, E1A, 16, 16, 1, 0},   {E1A, E1, 16, 16, 1, 0},   {P1, E2A, 16, 32, 1, 1},    {E2A, E2, 32, 32, 1, 1},
    {P2, E3A, 32, 64, 1, 2},   {E3A, E3, 64, 64, 1, 2},   {P3, B1, 64, 128, 1, 3},    {B1, B2, 128, 128, 1, 3},
    {C3, D3A, 192, 64, 1, 2},  {D3A, D3, 64, 64, 1, 2},   {C2, D2A, 96, 32, 1, 1},    {D2A, D2, 32, 32, 1, 1},
    {C1, D1A, 48, 16, 1, 0},   {D1A, D1, 16, 16, 1, 0},   {D1, OUT, 16, 16, 0, 0}};

// ------------------------------------------------------------------ elementwise kernels
__global__ void k_pool(const __nv_bfloat16 *__restrict__ x, __nv_bfloat16 *__restrict__ y, int H, int W, int C) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int h2 = H / 2, w2 = W / 2;
    if (i >= (long long)h2 * w2 * C) return;
    const int c = int(i % C);
    const long long q = i / C;
    const int yy = int(q / w2), xx = int(q % w2);
    const long long a = ((long long)(2 * yy) * W + 2 * xx) * C + c;
    const float s = __bfloat162float(x[a]) + __bfloat162float(x[a + C]) + __bfloat162float(x[a + (long long)W * C]) +
                    __bfloat162float(x[a + (long long)W * C + C]);
    y[i] = __float2bfloat16(0.25f * s);
}

// y[h][w] = concat(u[h/2][w/2][0:cu], s[h][w][0:cs])
__global__ void k_upcat(const __nv_bfloat16 *__restrict__ u, const __nv_bfloat16 *__restrict__ s,
                        __nv_bfloat16 *__restrict__ y, int H, int W, int cu, int cs) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int C = cu + cs;
    if (i >= (long long)H * W * C) return;
    const int c = int(i % C);
    const long long p = i / C;
    const int yy = int(p / W), xx = int(p % W);
    y[i] = c < cu ? u[((long long)(yy / 2) * (W / 2) + xx / 2) * cu + c] : s[p * cs + (c - cu)];
}

// gu[h2][w2][c] = sum of the four children gy[..][c] (c < cu); gs[p][c] = gy[p][cu + c]
__global__ void k_upcat_back(const float *__restrict__ gy, float *__restrict__ gu, float *__restrict__ gs, int H,
                             int W, int cu, int cs) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int C = cu + cs, h2 = H / 2, w2 = W / 2;
    const long long nu = (long long)h2 * w2 * cu, ns = (long long)H * W * cs;
    if (i < nu) {
        const int c = int(i % cu);
        const long long q = i / cu;
        const int yy = int(q / w2), xx = int(q % w2);
        const long long a = ((long long)(2 * yy) * W + 2 * xx) * C + c;
        gu[i] = gy[a] + gy[a + C] + gy[a + (long long)W * C] + gy[a + (long long)W * C + C];
    } else if (i < nu + ns) {
        const long long j = i - nu;
        gs[j] = gy[(j / cs) * C + cu + (j % cs)];
    }
}

// gx[p][c] = base[p][c] + gp[p/2][c] / 4
__global__ void k_poolback_add(const float *__restrict__ gp, const float *__restrict__ base, float *__restrict__ gx,
                               int H, int W, int C) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)H * W * C) return;
    const int c = int(i % C);
    const long long p = i / C;
    const int yy = int(p / W), xx = int(p % W);
    gx[i] = base[i] + 0.25f * gp[((long long)(yy / 2) * (W / 2) + xx / 2) * C + c];
}

// dz = g * (y > 0) (ReLU backward; y null: no ReLU), in BF16 for the tensor-core GEMMs
__global__ void k_mask(const float *__restrict__ g, const __nv_bfloat16 *__restrict__ y, __nv_bfloat16 *__restrict__ dz,
                       long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = (!y || __bfloat162float(y[i]) > 0.0f) ? g[i] : 0.0f;
    dz[i] = __float2bfloat16(v);
}

// db[c] = sum_p dz[p][c] (one block per channel, fixed order)
__global__ void k_bias_grad(const __nv_bfloat16 *__restrict__ dz, float *__restrict__ db, long long P, int C) {
    __shared__ double sh[TPB];
    const int c = blockIdx.x;
    double s = 0.0;
    for (long long p = threadIdx.x; p < P; p += TPB) s += double(__bfloat162float(dz[p * C + c]));
    s = block_reduce<SumOp>(s, sh);
    if (threadIdx.x == 0) db[c] = float(s);
}

// per-sample statistics over the interior: mean rho, std rho, rms rhs, rms pprev; block sums
// (pixels strided over the grid), then the sums in block order
__global__ void k_stats_part(const double *__restrict__ rho, const double *__restrict__ rhs,
                             const double *__restrict__ pprev, Dims D, double *__restrict__ part) {
    __shared__ double sh[TPB];
    const long long n = (long long)D.n[0] * D.n[1];
    double a[4] = {0, 0, 0, 0};
    for (long long q = (long long)blockIdx.x * TPB + threadIdx.x; q < n; q += (long long)RED_NB * TPB) {
        const int i = int(q / D.n[1]), j = int(q % D.n[1]);
        const long long g = D.at(i + GHC, j + GHC, 0);
        a[0] += rho[g];
        a[1] += rho[g] * rho[g];
        a[2] += rhs[g] * rhs[g];
        a[3] += pprev ? pprev[g] * pprev[g] : 0.0;
    }
    for (int m = 0; m < 4; ++m) {
        const double r = block_reduce<SumOp>(a[m], sh);
        if (threadIdx.x == 0) part[m * RED_NB + blockIdx.x] = r;
        __syncthreads();
    }
}

__global__ void k_stats_fin(const double *__restrict__ part, long long n, double *__restrict__ st) {
    if (threadIdx.x != 0) return;
    double r[4] = {0, 0, 0, 0};
    for (int m = 0; m < 4; ++m)
        for (int b = 0; b < RED_NB; ++b) r[m] += part[m * RED_NB + b];
    const double mean = r[0] / n;
    st[0] = mean;
    st[1] = sqrt(fmax(r[1] / n - mean * mean, 0.0)) + 1e-12;
    st[2] = sqrt(r[2] / n) + 1e-300;
    st[3] = sqrt(r[3] / n);
}

// x0[p] = (rho', rhs', pprev', 0 ...) for pixel p = i * ny + j; target t[p] if p_new given
__global__ void k_pack(const double *__restrict__ rho, const double *__restrict__ rhs, const double *__restrict__ pprev,
                       const double *__restrict__ pnew, Dims D, const double *__restrict__ st,
                       __nv_bfloat16 *__restrict__ x0, float *__restrict__ target) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)D.n[0] * D.n[1];
    if (q >= n) return;
    const int i = int(q / D.n[1]), j = int(q % D.n[1]);
    const long long g = D.at(i + GHC, j + GHC, 0);
    const double sp = st[3] > 0.0 ? st[3] : 1.0;
    const double pp = pprev ? pprev[g] : 0.0;
    __nv_bfloat16 v[C_IN];
    for (int c = 0; c < C_IN; ++c) v[c] = __float2bfloat16(0.0f);
    v[0] = __float2bfloat16(float((rho[g] - st[0]) / st[1]));
    v[1] = __float2bfloat16(float(rhs[g] / st[2]));
    v[2] = __float2bfloat16(float(pp / sp));
    for (int c = 0; c < C_IN; ++c) x0[q * C_IN + c] = v[c];
    if (target) target[q] = float((pnew[g] - pp) / sp);
}

// guess = pprev + s * out[p][0] on the interior (other cells copied from pprev, or 0)
__global__ void k_unpack(const float *__restrict__ out, const double *__restrict__ pprev, Dims D,
                         const double *__restrict__ st, double *__restrict__ guess) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= D.size()) return;
    guess[q] = pprev ? pprev[q] : 0.0;
    const int i = int(q / D.s[0]) - GHC, j = int((q % D.s[0]) / D.s[1]) - GHC;
    if (i < 0 || i >= D.n[0] || j < 0 || j >= D.n[1]) return;
    const double sp = st[3] > 0.0 ? st[3] : 1.0;
    guess[q] += sp * double(out[((long long)i * D.n[1] + j) * 16]);
}

// loss = mean (out[p][0] - t[p])^2; gout[p][c] = d loss / d out[p][c]; block sums, then in order
__global__ void k_loss_part(const float *__restrict__ out, const float *__restrict__ t, float *__restrict__ gout,
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

__global__ void k_loss_fin(const double *__restrict__ part, long long P, double *__restrict__ loss) {
    if (threadIdx.x != 0) return;
    double s = 0.0;
    for (int b = 0; b < RED_NB; ++b) s += part[b];
    *loss = s / double(P);
}

// ------------------------------------------------------------------ coarse-correction mode
// With factor F > 1 the network sees the pressure grid coarsened F x F: per coarse pixel the
// mean density, the mean residual of the previous pressure r = rhs - sum_f C_f (pprev_nb -
// pprev_c) (C_f = 2 / (rho_c + rho_nb) / d^2 on interior faces, the pressure equation's
// operator) and the mean previous pressure.  It predicts the mean of the error p - pprev over
// each coarse pixel, in units of s_e = 0.1 rms(r - mean r) (the error of a residual r on the
// unit square with density ~1-3 is about that size: e ~ rho r / k^2, k^2 >= 2 pi^2), and the
// guess is pprev + s_e times the prediction interpolated bilinearly to the cells.  The loss is
// on the coarse error -- the part of the error the multigrid cycle's coarse levels remove --
// and the interpolated correction is smooth, so it adds little high-frequency residual.
constexpr double COARSE_OUT_SCALE = 0.1;

__global__ void k_coarse_inputs(const double *__restrict__ rho, const double *__restrict__ rhs,
                                const double *__restrict__ pprev, Dims D, int fac, int Hc, int Wc,
                                float *__restrict__ cin) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (long long)Hc * Wc) return;
    const int I = int(p / Wc), J = int(p - (long long)I * Wc);
    const double w0 = 2.0 / (D.d[0] * D.d[0]), w1 = 2.0 / (D.d[1] * D.d[1]);
    double sr = 0.0, sres = 0.0, sp = 0.0;
    for (int a = 0; a < fac; ++a)
        for (int b = 0; b < fac; ++b) {
            const int i = I * fac + a, j = J * fac + b;
            const long long g = D.at(i + GHC, j + GHC, 0);
            const double rc = rho[g];
            sr += rc;
            double r = rhs[g];
            if (pprev) {
                const double pc = pprev[g];
                sp += pc;
                double lap = 0.0;
                if (i > 0) lap += w0 / (rc + rho[g - D.s[0]]) * (pprev[g - D.s[0]] - pc);
                if (i < D.n[0] - 1) lap += w0 / (rc + rho[g + D.s[0]]) * (pprev[g + D.s[0]] - pc);
                if (j > 0) lap += w1 / (rc + rho[g - D.s[1]]) * (pprev[g - D.s[1]] - pc);
                if (j < D.n[1] - 1) lap += w1 / (rc + rho[g + D.s[1]]) * (pprev[g + D.s[1]] - pc);
                r -= lap;
            }
            sres += r;
        }
    const double inv = 1.0 / double(fac * fac);
    cin[p * 3 + 0] = float(sr * inv);
    cin[p * 3 + 1] = float(sres * inv);
    cin[p * 3 + 2] = float(sp * inv);
}

// st = {mean rho, std rho, mean r, rms(r - mean r), rms pprev, s_e} over the coarse pixels
__global__ void k_stats_coarse_part(const float *__restrict__ cin, long long P, double *__restrict__ part) {
    __shared__ double sh[TPB];
    double a[5] = {0, 0, 0, 0, 0};
    for (long long p = (long long)blockIdx.x * TPB + threadIdx.x; p < P; p += (long long)RED_NB * TPB) {
        const double r0 = cin[p * 3], r1 = cin[p * 3 + 1], r2 = cin[p * 3 + 2];
        a[0] += r0, a[1] += r0 * r0, a[2] += r1, a[3] += r1 * r1, a[4] += r2 * r2;
    }
    for (int m = 0; m < 5; ++m) {
        const double r = block_reduce<SumOp>(a[m], sh);
        if (threadIdx.x == 0) part[m * RED_NB + blockIdx.x] = r;
        __syncthreads();
    }
}

__global__ void k_stats_coarse_fin(const double *__restrict__ part, long long P, double *__restrict__ st) {
    if (threadIdx.x != 0) return;
    double t[5] = {0, 0, 0, 0, 0};
    for (int m = 0; m < 5; ++m)
        for (int b = 0; b < RED_NB; ++b) t[m] += part[m * RED_NB + b];
    const double mr = t[0] / P, m1 = t[2] / P;
    st[0] = mr;
    st[1] = sqrt(fmax(t[1] / P - mr * mr, 0.0)) + 1e-12;
    st[2] = m1;
    st[3] = sqrt(fmax(t[3] / P - m1 * m1, 0.0)) + 1e-300;
    st[4] = sqrt(t[4] / P);
    st[5] = COARSE_OUT_SCALE * st[3];
}

// x0 from the coarse inputs; target: the mean of (pnew - pprev) over each coarse pixel / s_e
__global__ void k_pack_coarse(const float *__restrict__ cin, const double *__restrict__ st,
                              const double *__restrict__ pprev, const double *__restrict__ pnew, Dims D, int fac,
                              int Hc, int Wc, __nv_bfloat16 *__restrict__ x0, float *__restrict__ target) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (long long)Hc * Wc) return;
    const double sp = st[4] > 0.0 ? st[4] : 1.0;
    __nv_bfloat16 v[C_IN];
    for (int c = 0; c < C_IN; ++c) v[c] = __float2bfloat16(0.0f);
    v[0] = __float2bfloat16(float((double(cin[p * 3]) - st[0]) / st[1]));
    v[1] = __float2bfloat16(float((double(cin[p * 3 + 1]) - st[2]) / st[3]));
    v[2] = __float2bfloat16(float(double(cin[p * 3 + 2]) / sp));
    for (int c = 0; c < C_IN; ++c) x0[p * C_IN + c] = v[c];
    if (target) {
        const int I = int(p / Wc), J = int(p - (long long)I * Wc);
        double s = 0.0;
        for (int a = 0; a < fac; ++a)
            for (int b = 0; b < fac; ++b) {
                const long long g = D.at(I * fac + a + GHC, J * fac + b + GHC, 0);
                s += pnew[g] - (pprev ? pprev[g] : 0.0);
            }
        target[p] = float(s / double(fac * fac) / st[5]);
    }
}

// guess = pprev + s_e * (bilinear interpolation of out[.][0] from the coarse pixel centres),
// clamped at the walls; ghost cells copy pprev
__global__ void k_unpack_coarse(const float *__restrict__ out, const double *__restrict__ pprev, Dims D,
                                const double *__restrict__ st, int fac, int Hc, int Wc, double *__restrict__ guess) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= D.size()) return;
    guess[q] = pprev ? pprev[q] : 0.0;
    const int i = int(q / D.s[0]) - GHC, j = int((q % D.s[0]) / D.s[1]) - GHC;
    if (i < 0 || i >= D.n[0] || j < 0 || j >= D.n[1]) return;
    auto axis = [&](int k, int nc, int &k0, int &k1, double &w) {
        double x = (k + 0.5) / fac - 0.5;
        x = x < 0.0 ? 0.0 : (x > nc - 1 ? double(nc - 1) : x);
        k0 = int(x);
        k1 = k0 + 1 < nc ? k0 + 1 : k0;
        w = x - k0;
    };
    int i0, i1, j0, j1;
    double wi, wj;
    axis(i, Hc, i0, i1, wi);
    axis(j, Wc, j0, j1, wj);
    auto O = [&](int a, int b) { return double(out[((long long)a * Wc + b) * 16]); };
    const double v = (1.0 - wi) * ((1.0 - wj) * O(i0, j0) + wj * O(i0, j1)) + wi * ((1.0 - wj) * O(i1, j0) + wj * O(i1, j1));
    guess[q] += st[5] * v;
}

// BF16 copies of one layer's weights: forward [co][t][ci] and data-gradient [ci][t][co] with
// the taps flipped (t -> 8 - t)
__global__ void k_weights_bf16(const float *__restrict__ w, __nv_bfloat16 *__restrict__ wb,
                               __nv_bfloat16 *__restrict__ wt, int ci, int co) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= co * 9 * ci) return;
    const int o = i / (9 * ci), r = i % (9 * ci), t = r / ci, c = r % ci;
    const __nv_bfloat16 v = __float2bfloat16(w[i]);
    wb[i] = v;
    wt[((long long)c * 9 + (8 - t)) * co + o] = v;
}

__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       long long n, float lr, float b1, float b2, float c1, float c2) {
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

int UNet::create(int h, int w, unsigned seed, int factor) {
    if (factor < 1 || h % factor || w % factor) {
        set_last_error("unet: the coarsening factor must divide the grid");
        return SCIHPC_ERR_ARG;
    }
    fac = factor;
    PH = h, PW = w;
    h /= factor;
    w /= factor;
    if (h % 8 || w % 8 || h < 8 || w < 8) {
        set_last_error("unet: image sides (after coarsening) must be multiples of 8");
        return SCIHPC_ERR_ARG;
    }
    for (int l = 0; l < 4; ++l) H[l] = h >> l, W[l] = w >> l;
    SCIHPC_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    int rc = conv3x3_init(192);
    if (rc) return rc;
    // parameters: per layer co*9*ci weights then co biases
    nparam = 0;
    for (int l = 0; l < NL; ++l) {
        woff[l] = nparam;
        nparam += (long long)LAYERS[l].co * 9 * LAYERS[l].ci;
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
    for (int l = 0; l < NL; ++l) wbf += (long long)LAYERS[l].co * 9 * LAYERS[l].ci;
    if ((rc = dalloc((void **)&wb, wbf * 2)) || (rc = dalloc((void **)&wt, wbf * 2))) return rc;
    long long maxact = 0, maxpart = 0;
    for (int t = 0; t < NT; ++t) {
        const long long n = (long long)H[T_LEVEL[t]] * W[T_LEVEL[t]] * T_CH[t];
        const size_t bytes = t == OUT ? n * 4 : n * 2;
        if ((rc = dalloc(&act[t], bytes)) || (rc = dalloc((void **)&gact[t], n * 4))) return rc;
        maxact = n > maxact ? n : maxact;
    }
    for (int l = 0; l < NL; ++l) {
        const long long part = (long long)WGRAD_SPLITS * 9 * LAYERS[l].ci * LAYERS[l].co;
        maxpart = part > maxpart ? part : maxpart;
    }
    if ((rc = alloc_skip())) return rc;
    if ((rc = dalloc((void **)&dz, maxact * 2)) || (rc = dalloc((void **)&partial, maxpart * 4)) ||
        (rc = dalloc((void **)&target, (long long)H[0] * W[0] * 4)) || (rc = dalloc((void **)&stats, 8 * 8)) ||
        (rc = dalloc((void **)&dred, 5 * RED_NB * sizeof(double))) ||
        (rc = dalloc((void **)&err, 16)) || (rc = dalloc((void **)&cin, (long long)H[0] * W[0] * 3 * 4)))
        return rc;
    // He-normal weights, zero biases; the last layer starts near zero (guess = previous pressure)
    std::vector<float> hw(size_t(nparam), 0.0f);
    std::mt19937_64 gen(seed);
    for (int l = 0; l < NL; ++l) {
        const double sd = std::sqrt(2.0 / (9.0 * LAYERS[l].ci)) * (l == NL - 1 ? 0.01 : 1.0);
        std::normal_distribution<double> nd(0.0, sd);
        for (long long i = 0; i < (long long)LAYERS[l].co * 9 * LAYERS[l].ci; ++i) hw[size_t(woff[l] + i)] = float(nd(gen));
    }
    return set_weights(hw.data(), nparam);
}

void UNet::destroy() {
    for (void *p : allocs) cudaFree(p);
    allocs.clear();
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
}

int UNet::set_weights(const float *host, long long n) {
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

int UNet::get(float *host, long long n, bool gradient) {
    if (n != nparam) {
        set_last_error("unet: wrong parameter count");
        return SCIHPC_ERR_ARG;
    }
    SCIHPC_CUDA(cudaMemcpyAsync(host, gradient ? grad : wmaster, size_t(n) * 4, cudaMemcpyDeviceToHost, stream));
    SCIHPC_CUDA(cudaStreamSynchronize(stream));
    return SCIHPC_OK;
}

void UNet::refresh_bf16() {
    long long off = 0;
    for (int l = 0; l < NL; ++l) {
        const int n = LAYERS[l].co * 9 * LAYERS[l].ci;
        k_weights_bf16<<<nblk(n), TPB, 0, stream>>>(wmaster + woff[l], wb + off, wt + off, LAYERS[l].ci, LAYERS[l].co);
        wb_off[l] = off;
        off += n;
    }
}

int UNet::forward() {
    auto conv = [&](int l) {
        const LayerDef &L = LAYERS[l];
        const int lv = L.level;
        return conv3x3_forward((const __nv_bfloat16 *)act[L.in], wb + wb_off[l], wmaster + boff[l], act[L.out],
                               L.out != OUT, H[lv], W[lv], L.ci, L.co, L.relu != 0, err, stream);
    };
    auto pool = [&](int in, int out) {
        const int lv = T_LEVEL[in];
        const long long n = (long long)H[lv + 1] * W[lv + 1] * T_CH[in];
        k_pool<<<nblk(n), TPB, 0, stream>>>((const __nv_bfloat16 *)act[in], (__nv_bfloat16 *)act[out], H[lv], W[lv],
                                           T_CH[in]);
    };
    auto upcat = [&](int u, int s, int out) {
        const int lv = T_LEVEL[s];
        const long long n = (long long)H[lv] * W[lv] * T_CH[out];
        k_upcat<<<nblk(n), TPB, 0, stream>>>((const __nv_bfloat16 *)act[u], (const __nv_bfloat16 *)act[s],
                                            (__nv_bfloat16 *)act[out], H[lv], W[lv], T_CH[u], T_CH[s]);
    };
    int rc = 0;
    if ((rc = conv(0)) || (rc = conv(1))) return rc;
    pool(E1, P1);
    if ((rc = conv(2)) || (rc = conv(3))) return rc;
    pool(E2, P2);
    if ((rc = conv(4)) || (rc = conv(5))) return rc;
    pool(E3, P3);
    if ((rc = conv(6)) || (rc = conv(7))) return rc;
    upcat(B2, E3, C3);
    if ((rc = conv(8)) || (rc = conv(9))) return rc;
    upcat(D3, E2, C2);
    if ((rc = conv(10)) || (rc = conv(11))) return rc;
    upcat(D2, E1, C1);
    if ((rc = conv(12)) || (rc = conv(13)) || (rc = conv(14))) return rc;
    SCIHPC_CUDA(cudaGetLastError());
    return SCIHPC_OK;
}

// gradient of the loss with respect to every parameter, from gact[OUT] (set by the loss)
int UNet::backward() {
    int rc = 0;
    // one layer: dZ = g_out * relu'(out); dW, db; g_in = data gradient (unless layer 0)
    auto layer = [&](int l) -> int {
        const LayerDef &L = LAYERS[l];
        const int lv = L.level;
        const long long P = (long long)H[lv] * W[lv];
        const long long n = P * L.co;
        k_mask<<<nblk(n), TPB, 0, stream>>>(gact[L.out], L.relu ? (const __nv_bfloat16 *)act[L.out] : nullptr, dz, n);
        int r = conv3x3_wgrad((const __nv_bfloat16 *)act[L.in], dz, partial, grad + woff[l], H[lv], W[lv], L.ci, L.co,
                              WGRAD_SPLITS, err, stream);
        if (r) return r;
        k_bias_grad<<<L.co, TPB, 0, stream>>>(dz, grad + boff[l], P, L.co);
        if (l == 0) return SCIHPC_OK;
        return conv3x3_forward(dz, wt + wb_off[l], nullptr, gact[L.in], false, H[lv], W[lv], L.co, L.ci, false, err,
                               stream);
    };
    auto split = [&](int cat, int u, int s) {
        const int lv = T_LEVEL[s];
        const long long n = (long long)H[lv + 1] * W[lv + 1] * T_CH[u] + (long long)H[lv] * W[lv] * T_CH[s];
        k_upcat_back<<<nblk(n), TPB, 0, stream>>>(gact[cat], gact[u], gconcat(s), H[lv], W[lv], T_CH[u], T_CH[s]);
    };
    auto poolback = [&](int p, int e) {
        const int lv = T_LEVEL[e];
        const long long n = (long long)H[lv] * W[lv] * T_CH[e];
        k_poolback_add<<<nblk(n), TPB, 0, stream>>>(gact[p], gconcat(e), gact[e], H[lv], W[lv], T_CH[e]);
    };
    if ((rc = layer(14)) || (rc = layer(13)) || (rc = layer(12))) return rc;
    split(C1, D2, E1);
    if ((rc = layer(11)) || (rc = layer(10))) return rc;
    split(C2, D3, E2);
    if ((rc = layer(9)) || (rc = layer(8))) return rc;
    split(C3, B2, E3);
    if ((rc = layer(7)) || (rc = layer(6))) return rc;
    poolback(P3, E3);
    if ((rc = layer(5)) || (rc = layer(4))) return rc;
    poolback(P2, E2);
    if ((rc = layer(3)) || (rc = layer(2))) return rc;
    poolback(P1, E1);
    if ((rc = layer(1)) || (rc = layer(0))) return rc;
    SCIHPC_CUDA(cudaGetLastError());
    return SCIHPC_OK;
}

// gradient reaching a skip tensor (E1, E2, E3) through the concatenation; the pooling path
// is added to it in k_poolback_add
float *UNet::gconcat(int skip) {
    switch (skip) {
        case E1: return gskip[0];
        case E2: return gskip[1];
        default: return gskip[2];
    }
}

int UNet::prepare(const Dims &D, const double *rho, const double *rhs, const double *pprev, const double *pnew) {
    if (D.ndim != 2 || D.n[0] != PH || D.n[1] != PW) {
        set_last_error("unet: grid does not match the network's image size");
        return SCIHPC_ERR_ARG;
    }
    if (fac > 1) {
        const long long P = (long long)H[0] * W[0];
        k_coarse_inputs<<<nblk(P), TPB, 0, stream>>>(rho, rhs, pprev, D, fac, H[0], W[0], cin);
        k_stats_coarse_part<<<RED_NB, TPB, 0, stream>>>(cin, P, dred);
        k_stats_coarse_fin<<<1, 32, 0, stream>>>(dred, P, stats);
        k_pack_coarse<<<nblk(P), TPB, 0, stream>>>(cin, stats, pprev, pnew, D, fac, H[0], W[0],
                                                   (__nv_bfloat16 *)act[X0], pnew ? target : nullptr);
        return SCIHPC_OK;
    }
    k_stats_part<<<RED_NB, TPB, 0, stream>>>(rho, rhs, pprev, D, dred);
    k_stats_fin<<<1, 32, 0, stream>>>(dred, (long long)D.n[0] * D.n[1], stats);
    const long long P = (long long)H[0] * W[0];
    k_pack<<<nblk(P), TPB, 0, stream>>>(rho, rhs, pprev, pnew, D, stats, (__nv_bfloat16 *)act[X0],
                                       pnew ? target : nullptr);
    return SCIHPC_OK;
}

int UNet::check_err() {
    int h = 0;
    SCIHPC_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    SCIHPC_CUDA(cudaStreamSynchronize(stream));
    if (h) {
        set_last_error("unet: a tensor-core barrier wait timed out");
        return SCIHPC_ERR_CUDA;
    }
    return SCIHPC_OK;
}

int UNet::infer(const Dims &D, const double *rho, const double *rhs, const double *pprev, double *guess) {
    int rc = prepare(D, rho, rhs, pprev, nullptr);
    if (rc || (rc = forward())) return rc;
    if (fac > 1)
        k_unpack_coarse<<<nblk(D.size()), TPB, 0, stream>>>((const float *)act[OUT], pprev, D, stats, fac, H[0], W[0],
                                                            guess);
    else
        k_unpack<<<nblk(D.size()), TPB, 0, stream>>>((const float *)act[OUT], pprev, D, stats, guess);
    SCIHPC_CUDA(cudaGetLastError());
    return check_err();
}

int UNet::loss_grad(const Dims &D, const double *rho, const double *rhs, const double *pprev, const double *pnew,
                    double *loss) {
    int rc = prepare(D, rho, rhs, pprev, pnew);
    if (rc || (rc = forward())) return rc;
    const long long P = (long long)H[0] * W[0];
    k_loss_part<<<RED_NB, TPB, 0, stream>>>((const float *)act[OUT], target, gact[OUT], P, dred);
    k_loss_fin<<<1, 32, 0, stream>>>(dred, P, stats + 4);
    if ((rc = backward())) return rc;
    SCIHPC_CUDA(cudaMemcpyAsync(loss, stats + 4, sizeof(double), cudaMemcpyDeviceToHost, stream));
    return check_err();
}

int UNet::train_step(const Dims &D, const double *rho, const double *rhs, const double *pprev, const double *pnew,
                     float lr, double *loss) {
    int rc = loss_grad(D, rho, rhs, pprev, pnew, loss);
    if (rc) return rc;
    ++adam_t;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, float(adam_t)), c2 = 1.0f - std::pow(b2, float(adam_t));
    k_adam<<<nblk(nparam), TPB, 0, stream>>>(wmaster, grad, adam_m, adam_v, nparam, lr, b1, b2, c1, c2);
    refresh_bf16();
    SCIHPC_CUDA(cudaGetLastError());
    return SCIHPC_OK;
}

int UNet::alloc_skip() {
    for (int k = 0; k < 3; ++k) {
        const int t = k == 0 ? E1 : k == 1 ? E2 : E3;
        const size_t bytes = size_t(H[T_LEVEL[t]]) * W[T_LEVEL[t]] * T_CH[t] * 4;
        SCIHPC_CUDA(cudaMalloc(&gskip[k], bytes));
        SCIHPC_CUDA(cudaMemset(gskip[k], 0, bytes));
        allocs.push_back(gskip[k]);
    }
    return SCIHPC_OK;
}

}  // namespace scihpc
