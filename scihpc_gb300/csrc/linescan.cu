// linescan.cu -- warp-cooperative line solves of the CCD / UCCD 2x2 block-tridiagonal
// systems (uccd_solver.cpp:14-209, ccd_solver.cpp:14-282, matrix_solver.cpp:56-83).
//
// The factored solve of one line is two first-order affine recurrences on 2-vectors:
//   forward   v_i = -L_i v_{i-1} + r_i                 (v_0 = r_0)
//   backward  x_i =  K_i x_{i+1} + Dinv_i v_i          (x_{n-1} = Dinv_{n-1} v_{n-1})
// with L_i the elimination multipliers, K_i = -Dinv_i U_i, Dinv_i the inverse of the
// reduced diagonal block (all fixed per axis, computed once on the host).  Affine maps
// x -> M x + c compose associatively, so one warp solves one line: each lane composes the
// maps of its contiguous chunk, a 5-step shuffle scan combines the 32 chunk maps, and each
// lane then replays its chunk from the value entering it.  The line lives in registers;
// nothing but the input and the outputs touches memory.  Lines up to 32 * CM points.
#include "common.cuh"
#include "compact.cuh"

namespace scihpc {

namespace {

struct Aff {
    double m00, m01, m10, m11, c0, c1;
};

__device__ __forceinline__ Aff aff_identity() { return {1.0, 0.0, 0.0, 1.0, 0.0, 0.0}; }

// b o a : x -> b(a(x))
__device__ __forceinline__ Aff compose(const Aff &b, const Aff &a) {
    Aff r;
    r.m00 = b.m00 * a.m00 + b.m01 * a.m10;
    r.m01 = b.m00 * a.m01 + b.m01 * a.m11;
    r.m10 = b.m10 * a.m00 + b.m11 * a.m10;
    r.m11 = b.m10 * a.m01 + b.m11 * a.m11;
    r.c0 = b.m00 * a.c0 + b.m01 * a.c1 + b.c0;
    r.c1 = b.m10 * a.c0 + b.m11 * a.c1 + b.c1;
    return r;
}

__device__ __forceinline__ Aff shfl_up(const Aff &a, int d) {
    return {__shfl_up_sync(0xffffffffu, a.m00, d), __shfl_up_sync(0xffffffffu, a.m01, d),
            __shfl_up_sync(0xffffffffu, a.m10, d), __shfl_up_sync(0xffffffffu, a.m11, d),
            __shfl_up_sync(0xffffffffu, a.c0, d), __shfl_up_sync(0xffffffffu, a.c1, d)};
}

__device__ __forceinline__ Aff shfl_down(const Aff &a, int d) {
    return {__shfl_down_sync(0xffffffffu, a.m00, d), __shfl_down_sync(0xffffffffu, a.m01, d),
            __shfl_down_sync(0xffffffffu, a.m10, d), __shfl_down_sync(0xffffffffu, a.m11, d),
            __shfl_down_sync(0xffffffffu, a.c0, d), __shfl_down_sync(0xffffffffu, a.c1, d)};
}

// One system: rhs r[k] (2-vectors) of the lane's points lo .. lo+cnt-1 in, solution out
// (in place).  tab: per point {L00 L01 L10 L11, K00 K01 K10 K11, D00 D01 D10 D11}.
template <int CM, int WPL>
__device__ __forceinline__ void solve_system(double (&r0)[CM], double (&r1)[CM], const double *__restrict__ tab,
                                             int lo, int cnt, int n, int lane, int warp, Aff *sh) {
    // forward: chunk map, warp inclusive scan, replay
    Aff F = aff_identity();
#pragma unroll
    for (int k = 0; k < CM; ++k) {
        if (k < cnt) {
            const int i = lo + k;
            if (i == 0) {
                F = {0.0, 0.0, 0.0, 0.0, r0[k], r1[k]};
            } else {
                const double *t = tab + (size_t)i * 12;
                const Aff f = {-t[0], -t[1], -t[2], -t[3], r0[k], r1[k]};
                F = compose(f, F);
            }
        }
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const Aff o = shfl_up(F, d);
        if (lane >= d) F = compose(F, o);
    }
    // with several warps per line, warp w enters with the composition of warps 0 .. w-1
    Aff Pw = aff_identity();
    if (WPL > 1) {
        if (lane == 31) sh[warp] = F;
        __syncthreads();
        for (int v = 0; v < warp; ++v) Pw = compose(sh[v], Pw);
        __syncthreads();
    }
    const Aff P = shfl_up(F, 1);
    double v0 = P.c0, v1 = P.c1;   // v at lo-1 (unused by the lane holding point 0)
    if (WPL > 1) {
        if (lane == 0) {
            v0 = Pw.c0, v1 = Pw.c1;
        } else {
            v0 = P.m00 * Pw.c0 + P.m01 * Pw.c1 + P.c0;
            v1 = P.m10 * Pw.c0 + P.m11 * Pw.c1 + P.c1;
        }
    }
#pragma unroll
    for (int k = 0; k < CM; ++k) {
        if (k < cnt) {
            const int i = lo + k;
            if (i == 0) {
                v0 = r0[k], v1 = r1[k];
            } else {
                const double *t = tab + (size_t)i * 12;
                const double a = r0[k] - (t[0] * v0 + t[1] * v1);
                const double b = r1[k] - (t[2] * v0 + t[3] * v1);
                v0 = a, v1 = b;
            }
            r0[k] = v0, r1[k] = v1;
        }
    }
    // backward: chunk map (applied from the chunk end down), reverse warp scan, replay
    Aff G = aff_identity();
#pragma unroll
    for (int k = CM - 1; k >= 0; --k) {
        if (k < cnt) {
            const int i = lo + k;
            const double *t = tab + (size_t)i * 12;
            const double e0 = t[8] * r0[k] + t[9] * r1[k], e1 = t[10] * r0[k] + t[11] * r1[k];
            if (i == n - 1) {
                G = {0.0, 0.0, 0.0, 0.0, e0, e1};
            } else {
                const Aff g = {t[4], t[5], t[6], t[7], e0, e1};
                G = compose(g, G);
            }
        }
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const Aff o = shfl_down(G, d);
        if (lane + d < 32) G = compose(G, o);
    }
    Aff Sw = aff_identity();   // composition of the warps after this one
    if (WPL > 1) {
        if (lane == 0) sh[warp] = G;
        __syncthreads();
        for (int v = WPL - 1; v > warp; --v) Sw = compose(sh[v], Sw);
        __syncthreads();
    }
    const Aff Q = shfl_down(G, 1);
    double x0 = Q.c0, x1 = Q.c1;   // x at lo+cnt (unused by the lane holding n-1)
    if (WPL > 1) {
        if (lane == 31) {
            x0 = Sw.c0, x1 = Sw.c1;
        } else {
            x0 = Q.m00 * Sw.c0 + Q.m01 * Sw.c1 + Q.c0;
            x1 = Q.m10 * Sw.c0 + Q.m11 * Sw.c1 + Q.c1;
        }
    }
#pragma unroll
    for (int k = CM - 1; k >= 0; --k) {
        if (k < cnt) {
            const int i = lo + k;
            const double *t = tab + (size_t)i * 12;
            const double e0 = t[8] * r0[k] + t[9] * r1[k], e1 = t[10] * r0[k] + t[11] * r1[k];
            if (i == n - 1) {
                x0 = e0, x1 = e1;
            } else {
                const double a = t[4] * x0 + t[5] * x1 + e0;
                const double b = t[6] * x0 + t[7] * x1 + e1;
                x0 = a, x1 = b;
            }
            r0[k] = x0, r1[k] = x1;
        }
    }
}

// MODE 0: CCD (f1 = f', f2 = f''); MODE 1: UCCD (f1 = upwind-selected f', f2 = mean f'');
// MODE 2: mixed derivative -- `io` is first zero-order extrapolated along the line in place,
// f1 = its CCD first derivative.
// WPL == 1: each warp of the block solves its own line.  WPL > 1: the block's WPL warps solve
// one line together (shorter chunks per lane, and the per-warp maps combined in shared memory).
template <int MODE, int CM, int WPL>
__global__ void __launch_bounds__(256) scan_kernel(double *__restrict__ io, const double *__restrict__ vel,
                                                   double *__restrict__ f1, double *__restrict__ f2,
                                                   const double *__restrict__ tabA, const double *__restrict__ tabB,
                                                   Dims D, int a, int fast, int slow) {
    __shared__ Aff sh[WPL > 1 ? WPL : 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long line = WPL > 1 ? (long long)blockIdx.x : (long long)blockIdx.x * (blockDim.x >> 5) + warp;
    const long long nf = D.N[fast], ns = D.N[slow];
    if (line >= nf * ns) return;   // uniform per warp (per block when WPL > 1)
    int idx[3];
    idx[a] = 0;
    idx[fast] = int(line % nf);
    idx[slow] = int(line / nf);
    const long long base = D.at(idx[0], idx[1], idx[2]);
    const long long st = D.s[a];
    const int n = D.N[a];
    const double ih = D.rd[a];
    const int C = (n + 32 * WPL - 1) / (32 * WPL);
    const int lo = (WPL > 1 ? int(threadIdx.x) : lane) * C;
    const int cnt = lo >= n ? 0 : (lo + C <= n ? C : n - lo);
    double *f = io + base;
    auto src = [&](int i) -> int {
        if (MODE != 2) return i;
        return i < GHC ? GHC : (i > n - 1 - GHC ? n - 1 - GHC : i);
    };
    auto F = [&](int i) { return f[(long long)src(i) * st]; };
    double r0[CM], r1[CM], q0[CM], q1[CM];
    const double c3 = -0.06096119008109, c2 = 1.99692238016218, c1 = -1.93596119008109;
    double fm = cnt > 0 && lo > 0 ? F(lo - 1) : 0.0;
    double fc = cnt > 0 ? F(lo) : 0.0;
#pragma unroll
    for (int k = 0; k < CM; ++k) {
        if (k < cnt) {
            const int i = lo + k;
            const double fp = i + 1 < n ? F(i + 1) : 0.0;
            if (i == 0 || i == n - 1) {
                // one-sided closures (uccd_solver.cpp:29-51, ccd_solver.cpp:31-40)
                double s, ss;
                if (i == 0) {
                    const double g0 = fc, g1 = fp, g2 = F(2);
                    s = (-3.5 * g0 + 4.0 * g1 - 0.5 * g2) * ih;
                    ss = (9.0 * g0 - 12.0 * g1 + 3.0 * g2) * ih * ih;
                } else {
                    const double g0 = fc, g1 = fm, g2 = F(n - 3);
                    s = -(-3.5 * g0 + 4.0 * g1 - 0.5 * g2) * ih;
                    ss = (9.0 * g0 - 12.0 * g1 + 3.0 * g2) * ih * ih;
                }
                r0[k] = s, r1[k] = ss;
                q0[k] = s, q1[k] = ss;
            } else {
                const double ss = (3.0 * fm - 6.0 * fc + 3.0 * fp) * ih * ih;
                if (MODE == 1) {
                    r0[k] = (c1 * fm + c2 * fc + c3 * fp) * ih;
                    q0[k] = -(c3 * fm + c2 * fc + c1 * fp) * ih;
                    q1[k] = ss;
                } else {
                    r0[k] = 15.0 / 16.0 * (fp - fm) * ih;
                }
                r1[k] = ss;
            }
            fm = fc;
            fc = fp;
        }
    }
    if (MODE == 2) {
        // the reference extrapolates the source in place (ccd_solver.cpp:151-155); every read
        // above went through the clamp, so the write-back order does not matter
#pragma unroll
        for (int k = 0; k < CM; ++k) {
            const int i = lo + k;
            if (k < cnt && (i < GHC || i > n - 1 - GHC)) f[(long long)i * st] = F(i);
        }
    }
    solve_system<CM, WPL>(r0, r1, tabA, lo, cnt, n, lane, warp, sh);
    if (MODE == 1) solve_system<CM, WPL>(q0, q1, tabB, lo, cnt, n, lane, warp, sh);
#pragma unroll
    for (int k = 0; k < CM; ++k) {
        if (k < cnt) {
            const long long o = base + (long long)(lo + k) * st;
            if (MODE == 1) {
                f1[o] = vel[o] > 0 ? r0[k] : q0[k];
                f2[o] = 0.5 * (r1[k] + q1[k]);
            } else if (MODE == 0) {
                f1[o] = r0[k];
                f2[o] = r1[k];
            } else {
                f1[o] = r0[k];
            }
        }
    }
}

template <int MODE>
bool launch_scan(const Dims &D, int a, double *io, const double *vel, double *f1, double *f2, const double *tA,
                 const double *tB, cudaStream_t s) {
    const int b = (a + 1) % 3, c = (a + 2) % 3;
    const int fast = b > c ? b : c, slow = b > c ? c : b;
    const long long lines = (long long)D.N[b] * D.N[c];
    const int n = D.N[a];
    // Each lane's chunk is an FP64 dependency chain.  When there are few lines (fewer than a
    // few per SM) several warps share a line: shorter chains and more warps in flight.
    int wpl = 1;
    if (lines < 4LL * NUM_SMS) wpl = n >= 192 ? 4 : (n >= 96 ? 2 : 1);
    const int C = (n + 32 * wpl - 1) / (32 * wpl);
    if (wpl > 1) {
        const unsigned blocks = unsigned(lines);
        const int tpb = 32 * wpl;
#define SCAN_WPL(W)                                                                                              \
    if (C <= 2) scan_kernel<MODE, 2, W><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, tA, tB, D, a, fast, slow);        \
    else if (C <= 4) scan_kernel<MODE, 4, W><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, tA, tB, D, a, fast, slow);   \
    else if (C <= 8) scan_kernel<MODE, 8, W><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, tA, tB, D, a, fast, slow);   \
    else if (C <= 16) scan_kernel<MODE, 16, W><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, tA, tB, D, a, fast, slow); \
    else return false;
        if (wpl == 2) {
            SCAN_WPL(2)
        } else {
            SCAN_WPL(4)
        }
#undef SCAN_WPL
        return true;
    }
    // many lines: one warp per line, up to eight lines per block
    int wpb = 1;
    while (wpb < 8 && lines >= (long long)wpb * 2 * 4 * NUM_SMS) wpb *= 2;
    const unsigned blocks = unsigned((lines + wpb - 1) / wpb);
    const int tpb = 32 * wpb;
    if (C <= 4) scan_kernel<MODE, 4, 1><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, tA, tB, D, a, fast, slow);
    else if (C <= 8) scan_kernel<MODE, 8, 1><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, tA, tB, D, a, fast, slow);
    else if (C <= 16) scan_kernel<MODE, 16, 1><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, tA, tB, D, a, fast, slow);
    else return false;
    return true;
}

}  // namespace

bool scan_uccd(const Dims &D, const CompactOps &ops, int a, const double *flux, const double *vel, double *f1,
               double *f2, cudaStream_t s) {
    return launch_scan<1>(D, a, const_cast<double *>(flux), vel, f1, f2, ops.scan_up[a], ops.scan_down[a], s);
}

bool scan_ccd(const Dims &D, const CompactOps &ops, int a, const double *flux, double *f1, double *f2,
              cudaStream_t s) {
    return launch_scan<0>(D, a, const_cast<double *>(flux), nullptr, f1, f2, ops.scan_ccd[a], nullptr, s);
}

bool scan_mixed(const Dims &D, const CompactOps &ops, int a, double *src, double *out, cudaStream_t s) {
    return launch_scan<2>(D, a, src, nullptr, out, nullptr, ops.scan_ccd[a], nullptr, s);
}

}  // namespace scihpc
