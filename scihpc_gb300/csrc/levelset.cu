// levelset.cu -- WENO5 derivatives, Godunov gradient, smoothed level-set fields, curvature
// and the enclosed mass / volume integrals.  All FP64 (level-set transport and
// reinitialisation keep the reference's precision).
#include "common.cuh"
#include "levelset.cuh"
#include "lsm_device.cuh"
#include "reduce.cuh"

namespace scihpc {

namespace {

// WENO-Z face value from five cell values (weno_solver.cpp:16-66): `left` selects the
// left-biased reconstruction (indicators_m / interpolation_m), else the right-biased one.
__device__ __forceinline__ double weno_face(double a, double b, double c, double d, double e, bool left) {
    double b0, b1, b2, q0, q1, q2;
    const double sixth = 1.0 / 6.0;
    const double t1 = b - 2.0 * c + d;
    b1 = 13.0 * t1 * t1 + 3.0 * (b - d) * (b - d);
    if (left) {
        const double ta = a - 2.0 * b + c, tb = a - 4.0 * b + 3.0 * c;
        const double tc = c - 2.0 * d + e, td = 3.0 * c - 4.0 * d + e;
        b0 = 13.0 * ta * ta + 3.0 * tb * tb;
        b2 = 13.0 * tc * tc + 3.0 * td * td;
        q0 = (11.0 * c - 7.0 * b + 2.0 * a) * sixth;
        q1 = (2.0 * d + 5.0 * c - b) * sixth;
        q2 = (-e + 5.0 * d + 2.0 * c) * sixth;
    } else {
        const double ta = c - 2.0 * d + e, tb = 3.0 * c - 4.0 * d + e;
        const double tc = a - 2.0 * b + c, td = a - 4.0 * b + 3.0 * c;
        b0 = 13.0 * ta * ta + 3.0 * tb * tb;
        b2 = 13.0 * tc * tc + 3.0 * td * td;
        q0 = (11.0 * c - 7.0 * d + 2.0 * e) * sixth;
        q1 = (2.0 * b + 5.0 * c - d) * sixth;
        q2 = (-a + 5.0 * b + 2.0 * c) * sixth;
    }
    // WENO-Z weights a_k = d_k (1 + tau / g_k), g_k = eps + beta_k, multiplied through by
    // g0 g1 g2 so that one reciprocal remains (the refined hardware reciprocal: within about
    // an ulp of the reference's division)
    const double tau = fabs(b0 - b2);
    const double g0 = WENO_EPS + b0, g1 = WENO_EPS + b1, g2 = WENO_EPS + b2;
    const double a0 = (g0 + tau) * g1 * g2;
    const double a1 = 6.0 * (g1 + tau) * g0 * g2;
    const double a2 = 3.0 * (g2 + tau) * g0 * g1;
    return (a0 * q0 + a1 * q1 + a2 * q2) * rcp_refined(a0 + a1 + a2);
}

// Upwinded face value between cells i and i+1 (weno_solver.cpp:185-199).  The right-biased
// reconstruction is the left-biased one of the mirrored stencil (interpolation_p /
// indicators_p are interpolation_m / indicators_m read from the other side), so the face
// velocity only selects the five inputs and every thread runs the same instructions.
__device__ __forceinline__ double weno_upwind_face(const double *f, long long o, long long st, const double *vel) {
    const bool up = vel[o] + vel[o + st] > 0.0;
    const long long c = up ? o : o + st, dn = up ? st : -st;
    return weno_face(f[c - 2 * dn], f[c - dn], f[c], f[c + dn], f[c + 2 * dn], true);
}

// d/dx_a of the upwinded WENO flux (weno_solver.cpp:185-199): (h(i+1/2) - h(i-1/2)) / d_a.
// Every face is computed once and shared by the two cells beside it.
// Along the contiguous axis (a = ndim - 1): lane l of a warp computes the face between cells
// c0 + l - 1 and c0 + l of one line, and lanes 0..30 take their cell's derivative from their
// own face and the next lane's (31 cells per warp).
constexpr int WZ_SEG = 31;
__global__ void weno_kernel_lane(const double *__restrict__ f, const double *__restrict__ vel, double *__restrict__ out,
                                 Dims D, int a) {
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int na = D.n[a];
    const long long segs = (na + WZ_SEG - 1) / WZ_SEG;
    const long long lines = D.interior() / na;
    if (warp >= lines * segs) return;   // whole warps leave together
    const long long line = warp / segs;
    const int c0 = int(warp - line * segs) * WZ_SEG;
    // the line's cells: the other interior indices (axis 0 slowest)
    int I = 0, J = 0;
    if (D.ndim == 3) {
        I = int(line / D.n[1]);
        J = int(line - (long long)I * D.n[1]);
    } else {
        I = int(line);
    }
    const int c = c0 + lane - 1;   // this lane's face lies between cells c and c + 1
    const long long st = D.s[a];
    const long long o = D.ndim == 3 ? D.at(D.ix(0, I), D.ix(1, J), D.ix(2, c)) : D.at(D.ix(0, I), D.ix(1, c), 0);
    const double h = c < na ? weno_upwind_face(f, o, st, vel) : 0.0;
    const double hn = __shfl_down_sync(0xffffffffu, h, 1);
    if (lane < WZ_SEG && c + 1 < na) out[o + st] = (hn - h) / D.d[a];
}

// Along the other axes: a block of 32 x WZ_W threads, lanes along the contiguous axis, warp w
// computes the faces between cells a0 + w - 1 and a0 + w; warps 0 .. WZ_W - 2 then form the
// derivatives of cells a0 .. a0 + WZ_W - 2 from shared memory.
constexpr int WZ_W = 8;
__global__ void __launch_bounds__(32 * WZ_W)
    weno_kernel_tile(const double *__restrict__ f, const double *__restrict__ vel, double *__restrict__ out, Dims D,
                     int a) {
    __shared__ double H[WZ_W][33];
    const int lane = threadIdx.x, w = threadIdx.y;
    const int cl = D.ndim - 1;                  // contiguous axis
    const int ot = D.ndim == 3 ? 3 - a - cl : -1;   // the remaining axis (3D)
    const int q = blockIdx.x * 32 + lane;       // index along the contiguous axis
    const int c = blockIdx.y * (WZ_W - 1) + w - 1;   // the face lies between cells c and c + 1 along a
    const int r = blockIdx.z;                   // index along the remaining axis (3D)
    const bool live = q < D.n[cl] && c < D.n[a];
    int idx[3] = {0, 0, 0};
    idx[cl] = q;
    idx[a] = c;
    if (ot >= 0) idx[ot] = r;
    const long long st = D.s[a];
    const long long o = D.at(D.ix(0, idx[0]), D.ix(1, idx[1]), D.ndim == 3 ? D.ix(2, idx[2]) : 0);
    H[w][lane] = live ? weno_upwind_face(f, o, st, vel) : 0.0;
    __syncthreads();
    if (w < WZ_W - 1 && live && c + 1 < D.n[a]) out[o + st] = (H[w + 1][lane] - H[w][lane]) / D.d[a];
}

}  // namespace

namespace {

__global__ void godunov_kernel(const double *__restrict__ phi, const double *__restrict__ sign,
                               double *__restrict__ grad, Dims D) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= D.size()) return;
    int i, j, k;
    split3_full(q, D, i, j, k);
    const bool inside = (i >= GHC && i < D.N[0] - GHC) && (D.ndim < 2 || (j >= GHC && j < D.N[1] - GHC)) &&
                        (D.ndim < 3 || (k >= GHC && k < D.N[2] - GHC));
    grad[q] = inside ? godunov_at(phi, q, sign[q], D) : 0.0;
}

__global__ void fields_kernel(const double *__restrict__ phi, double *H, double *De, double *Sg, double *Rho,
                              double *Mu, long long n, double w, double dr, double vr, int pos) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const double x = phi[q];
    const double h = heaviside_d(x, w);
    if (H) H[q] = h;
    if (De) De[q] = delta_d(x, w);
    if (Sg) Sg[q] = sign_d(x, w);
    if (Rho) Rho[q] = pos ? h + (1.0 - h) * dr : (1.0 - h) + h * dr;   // wrapper_func.cpp:387-402
    if (Mu) Mu[q] = pos ? h + (1.0 - h) * vr : (1.0 - h) + h * vr;     // wrapper_func.cpp:404-418
}

__global__ void curvature_kernel(const double *__restrict__ phi, const double *fx, const double *fy,
                                 const double *fz, const double *fxx, const double *fyy, const double *fzz,
                                 const double *fxy, const double *fyz, const double *fzx, double *curv, long long n,
                                 int ndim) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    double k;
    if (ndim == 2) {
        const double x = fx[q], y = fy[q];
        k = (fxx[q] * y * y + fyy[q] * x * x - 2.0 * fxy[q] * x * y) / pow(x * x + y * y, 1.5);
        k = k > 0.0 ? 1.0 / (1.0 / k + phi[q]) : -1.0 / (-1.0 / k + phi[q]);
    } else {
        const double x = fx[q], y = fy[q], z = fz[q];
        k = (x * x * (fyy[q] + fzz[q]) + y * y * (fxx[q] + fzz[q]) + z * z * (fxx[q] + fyy[q]) -
             2.0 * (x * y * fxy[q] + x * z * fzx[q] + y * z * fyz[q])) /
            pow(x * x + y * y + z * z, 1.5);
        k = k > 0.0 ? 1.0 / (2.0 / k + phi[q]) : -1.0 / (-2.0 / k + phi[q]);
    }
    curv[q] = k;
}

// Per-cell contribution of lsf_mass (which = 0) or lsf_volume (which = 1) from the
// product field w (rho * H for mass, H for volume) (wrapper_func.cpp:450-572).
__device__ double integral_cell(const double *w, long long q, const Dims &D, int which) {
    int I, J, K;
    split3(q, D, I, J, K);
    const int i = D.ix(0, I), j = D.ix(1, J), k = D.ix(2, K);
    const long long o = D.at(i, j, k);
    if (D.ndim == 2) {
        const bool inner = I != 0 && I != D.n[0] - 1 && J != 0 && J != D.n[1] - 1;
        if (!inner) return w[o];
        double s = 15.0 * w[o];
        for (int a = -1; a < 2; ++a)
            for (int b = -1; b < 2; ++b) s += w[o + a * D.s[0] + b * D.s[1]];
        return s / 24.0;
    }
    const bool inner = I != 0 && I != D.n[0] - 1 && J != 0 && J != D.n[1] - 1 && K != 0 && K != D.n[2] - 1;
    double s = 50.0 * w[o];
    if (inner)
        for (int a = -1; a < 2; ++a)
            for (int b = -1; b < 2; ++b)
                for (int c = -1; c < 2; ++c) s += w[o + a * D.s[0] + b * D.s[1] + c];
    if (which == 0) return inner ? s * D.dv / 77.0 : w[o] * D.dv;
    return (inner ? s / 77.0 : w[o]) + s / 77.0;
}

__global__ void product_kernel(const double *__restrict__ phi, double *__restrict__ w, long long n, double lw,
                               double dr, int pos, int which) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const double h = heaviside_d(phi[q], lw);
    if (which == 1) {
        w[q] = h;
    } else {
        const double rho = pos ? h + (1.0 - h) * dr : (1.0 - h) + h * dr;
        w[q] = rho * h;
    }
}

__global__ void integral_kernel(const double *__restrict__ w, Dims D, int which, double *__restrict__ partial) {
    __shared__ double sh[RED_THREADS];
    const long long n = D.interior();
    const long long per_block = (n + gridDim.x - 1) / gridDim.x;
    const long long b0 = blockIdx.x * per_block;
    const long long b1 = b0 + per_block < n ? b0 + per_block : n;
    double s = 0.0;
    for (long long q = b0 + threadIdx.x; q < b1; q += blockDim.x) s += integral_cell(w, q, D, which);
    s = block_reduce<SumOp>(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// max over every cell of grad (>= 0; ghosts hold 0), block partials for finish_reduce<MaxOp>
// (godunov_gradient.cpp:161-170: fmax from 0.0, in any order the same value)
__global__ void max_kernel(const double *__restrict__ g, long long n, double *__restrict__ partial) {
    __shared__ double sh[RED_THREADS];
    const long long per_block = (n + gridDim.x - 1) / gridDim.x;
    const long long b0 = blockIdx.x * per_block;
    const long long b1 = b0 + per_block < n ? b0 + per_block : n;
    double m = 0.0;
    for (long long q = b0 + threadIdx.x; q < b1; q += blockDim.x) m = fmax(m, g[q]);
    m = block_reduce<MaxOp>(m, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = m;
}

// phi /= max |grad phi| on every cell (godunov_gradient.cpp:172-180)
__global__ void rescale_kernel(double *__restrict__ phi, long long n, const double *__restrict__ mx) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    phi[q] = __ddiv_rn(phi[q], *mx);
}

// guess_from_history (flux.cpp:653-662): flux = 2 old - old2 on every cell
__global__ void history_kernel(const double *__restrict__ old, const double *__restrict__ old2,
                               double *__restrict__ flux, long long n) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    flux[q] = __dsub_rn(__dmul_rn(2.0, old[q]), old2[q]);
}

}  // namespace

void launch_stabilize(const Dims &D, double *phi, const double *sign, double *grad, double *partial, double *mx,
                      cudaStream_t s) {
    launch_godunov(D, phi, sign, grad, s);
    const int nb = red_blocks(D.size());
    max_kernel<<<nb, RED_THREADS, 0, s>>>(grad, D.size(), partial);
    finish_reduce<MaxOp><<<1, 1024, 0, s>>>(partial, nb, mx);
    rescale_kernel<<<blocks_for(D.size(), 256), 256, 0, s>>>(phi, D.size(), mx);
}

void launch_guess_from_history(const Dims &D, const double *old, const double *old2, double *flux, cudaStream_t s) {
    history_kernel<<<blocks_for(D.size(), 256), 256, 0, s>>>(old, old2, flux, D.size());
}

void launch_weno5(const Dims &D, int a, const double *flux, const double *vel, double *out, cudaStream_t s) {
    if (a == D.ndim - 1) {
        const long long warps = D.interior() / D.n[a] * ((D.n[a] + WZ_SEG - 1) / WZ_SEG);
        weno_kernel_lane<<<blocks_for(warps * 32, 128), 128, 0, s>>>(flux, vel, out, D, a);
    } else {
        const int cl = D.ndim - 1, ot = D.ndim == 3 ? 3 - a - cl : -1;
        const dim3 grid(unsigned((D.n[cl] + 31) / 32), unsigned((D.n[a] + WZ_W - 2) / (WZ_W - 1)),
                        unsigned(ot >= 0 ? D.n[ot] : 1));
        weno_kernel_tile<<<grid, dim3(32, WZ_W), 0, s>>>(flux, vel, out, D, a);
    }
}

void launch_godunov(const Dims &D, const double *phi, const double *sign, double *grad, cudaStream_t s) {
    godunov_kernel<<<blocks_for(D.size(), 128), 128, 0, s>>>(phi, sign, grad, D);
}

void launch_lsf_fields(const Dims &D, const double *prm, const double *phi, double *H, double *De, double *Sg,
                       double *Rho, double *Mu, cudaStream_t s) {
    fields_kernel<<<blocks_for(D.size(), 256), 256, 0, s>>>(phi, H, De, Sg, Rho, Mu, D.size(), prm[0], prm[1], prm[2],
                                                             prm[3] != 0.0);
}

void launch_curvature(const Dims &D, const double *phi, const double *const d[9], double *curv, cudaStream_t s) {
    curvature_kernel<<<blocks_for(D.size(), 256), 256, 0, s>>>(phi, d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7],
                                                                d[8], curv, D.size(), D.ndim);
}

// lsf_mass (which 0) or lsf_volume (which 1) into *out (device), using `work` (one field)
// and `partial` (RED_MAX_BLOCKS doubles) as scratch.  The result still needs the final dv
// factor, applied by the caller (wrapper_func.cpp:510,571).
void launch_lsf_integral(const Dims &D, const double *prm, const double *phi, int which, double *work,
                         double *partial, double *out, cudaStream_t s) {
    product_kernel<<<blocks_for(D.size(), 256), 256, 0, s>>>(phi, work, D.size(), prm[0], prm[1], prm[3] != 0.0,
                                                             which);
    const int nb = red_blocks(D.interior());
    integral_kernel<<<nb, RED_THREADS, 0, s>>>(work, D, which, partial);
    finish_reduce<SumOp><<<1, 1024, 0, s>>>(partial, nb, out);
}

}  // namespace scihpc
