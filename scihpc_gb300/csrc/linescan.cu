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
// lane then replays its chunk from the value entering it.  Every matrix M met on the way
// (chunk products, scan partials) depends on the factorisation and the launch shape only and
// is precomputed per axis, so the kernel forms the vector halves c alone: about a third of the
// FP64 work of composing full maps, on a GPU whose FP64 rate bounds these solves.  The line
// lives in registers; nothing but the input and the outputs touches memory.  Lines up to
// 32 * 16 points with one warp, 128 * 16 with four.
#include "common.cuh"
#include "compact.cuh"

namespace scihpc {

namespace {

// One system: rhs r[k] (2-vectors) of the lane's points lo .. lo+cnt-1 in, solution out
// (in place).  lt: the line's tables for this launch shape (lane_table in compact.cu), thread
// index fastest so that every load of a warp is coalesced: per point of the chunk {-L00 -L01
// -L10 -L11, K00 K01 K10 K11, D00 D01 D10 D11} (L negated: each row of the forward step is two
// FMAs), then the matrix halves of the chunk and scan maps, so
// that only the vector halves are formed here; tid: the thread's index within its line.
template <int CM, int WPL>
__device__ __forceinline__ void solve_system(double (&r0)[CM], double (&r1)[CM], const double *__restrict__ lt, int tid,
                                             int lo, int cnt, int n, int C, int lane, int warp, double2 *sh) {
    constexpr unsigned FULL = 0xffffffffu;
    constexpr int T = 32 * WPL;
    const double *pt = lt + tid;                                 // [k][12][T]
    const double *me = lt + (size_t)C * 12 * T + tid;            // [48][T]
    const double *wt = lt + (size_t)C * 12 * T + (size_t)48 * T;  // [WPL][8]
    // forward: the chunk's map applied to a zero entry vector, inclusive warp scan, replay
    double c0 = 0.0, c1 = 0.0;
#pragma unroll
    for (int k = 0; k < CM; ++k) {
        if (k < cnt) {
            const int i = lo + k;
            if (i == 0) {
                c0 = r0[k], c1 = r1[k];
            } else {
                const double *t = pt + (size_t)k * 12 * T;
                const double a = fma(t[0 * T], c0, fma(t[1 * T], c1, r0[k]));   // t[0..3] = -L
                const double b = fma(t[2 * T], c0, fma(t[3 * T], c1, r1[k]));
                c0 = a, c1 = b;
            }
        }
    }
#pragma unroll
    for (int st = 0; st < 5; ++st) {
        const int d = 1 << st;
        const double o0 = __shfl_up_sync(FULL, c0, d), o1 = __shfl_up_sync(FULL, c1, d);
        if (lane >= d) {
            const double *ml = me + 4 * st * T;
            const double a = ml[0 * T] * o0 + ml[1 * T] * o1 + c0;
            const double b = ml[2 * T] * o0 + ml[3 * T] * o1 + c1;
            c0 = a, c1 = b;
        }
    }
    double v0 = __shfl_up_sync(FULL, c0, 1), v1 = __shfl_up_sync(FULL, c1, 1);   // v at lo-1
    if (WPL > 1) {
        // warp w enters with the composition of warps 0 .. w-1
        if (lane == 31) sh[warp] = make_double2(c0, c1);
        __syncthreads();
        double p0 = 0.0, p1 = 0.0;
        for (int w = 0; w < warp; ++w) {
            const double *m = wt + 8 * w;
            const double a = m[0] * p0 + m[1] * p1 + sh[w].x;
            const double b = m[2] * p0 + m[3] * p1 + sh[w].y;
            p0 = a, p1 = b;
        }
        __syncthreads();
        if (lane == 0) {
            v0 = p0, v1 = p1;
        } else {
            const double *ml = me + 20 * T;
            const double a = ml[0 * T] * p0 + ml[1 * T] * p1 + v0;
            const double b = ml[2 * T] * p0 + ml[3 * T] * p1 + v1;
            v0 = a, v1 = b;
        }
    }
#pragma unroll
    for (int k = 0; k < CM; ++k) {
        if (k < cnt) {
            const int i = lo + k;
            if (i == 0) {
                v0 = r0[k], v1 = r1[k];
            } else {
                const double *t = pt + (size_t)k * 12 * T;
                const double a = fma(t[0 * T], v0, fma(t[1 * T], v1, r0[k]));
                const double b = fma(t[2 * T], v0, fma(t[3 * T], v1, r1[k]));
                v0 = a, v1 = b;
            }
            r0[k] = v0, r1[k] = v1;
        }
    }
    // backward: e_i = Dinv_i v_i (kept in r), the chunk's map applied to a zero exit vector,
    // reverse warp scan, replay
    double g0 = 0.0, g1 = 0.0;
#pragma unroll
    for (int k = CM - 1; k >= 0; --k) {
        if (k < cnt) {
            const int i = lo + k;
            const double *t = pt + (size_t)k * 12 * T;
            const double e0 = t[8 * T] * r0[k] + t[9 * T] * r1[k], e1 = t[10 * T] * r0[k] + t[11 * T] * r1[k];
            r0[k] = e0, r1[k] = e1;
            if (i == n - 1) {
                g0 = e0, g1 = e1;
            } else {
                const double a = t[4 * T] * g0 + t[5 * T] * g1 + e0;
                const double b = t[6 * T] * g0 + t[7 * T] * g1 + e1;
                g0 = a, g1 = b;
            }
        }
    }
#pragma unroll
    for (int st = 0; st < 5; ++st) {
        const int d = 1 << st;
        const double o0 = __shfl_down_sync(FULL, g0, d), o1 = __shfl_down_sync(FULL, g1, d);
        if (lane + d < 32) {
            const double *ml = me + (24 + 4 * st) * T;
            const double a = ml[0 * T] * o0 + ml[1 * T] * o1 + g0;
            const double b = ml[2 * T] * o0 + ml[3 * T] * o1 + g1;
            g0 = a, g1 = b;
        }
    }
    double x0 = __shfl_down_sync(FULL, g0, 1), x1 = __shfl_down_sync(FULL, g1, 1);   // x at lo+cnt
    if (WPL > 1) {
        // composition of the warps after this one
        if (lane == 0) sh[warp] = make_double2(g0, g1);
        __syncthreads();
        double q0 = 0.0, q1 = 0.0;
        for (int w = WPL - 1; w > warp; --w) {
            const double *m = wt + 8 * w + 4;
            const double a = m[0] * q0 + m[1] * q1 + sh[w].x;
            const double b = m[2] * q0 + m[3] * q1 + sh[w].y;
            q0 = a, q1 = b;
        }
        __syncthreads();
        if (lane == 31) {
            x0 = q0, x1 = q1;
        } else {
            const double *ml = me + 44 * T;
            const double a = ml[0 * T] * q0 + ml[1 * T] * q1 + x0;
            const double b = ml[2 * T] * q0 + ml[3 * T] * q1 + x1;
            x0 = a, x1 = b;
        }
    }
#pragma unroll
    for (int k = CM - 1; k >= 0; --k) {
        if (k < cnt) {
            const int i = lo + k;
            if (i == n - 1) {
                x0 = r0[k], x1 = r1[k];
            } else {
                const double *t = pt + (size_t)k * 12 * T;
                const double a = t[4 * T] * x0 + t[5 * T] * x1 + r0[k];
                const double b = t[6 * T] * x0 + t[7 * T] * x1 + r1[k];
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
                                                   const double *__restrict__ ltA, const double *__restrict__ ltB,
                                                   Dims D, int a, int fast, int slow) {
    __shared__ double2 sh[WPL > 1 ? WPL : 1];
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
    const int tid = WPL > 1 ? int(threadIdx.x) : lane;
    solve_system<CM, WPL>(r0, r1, ltA, tid, lo, cnt, n, C, lane, warp, sh);
    if (MODE == 1) solve_system<CM, WPL>(q0, q1, ltB, tid, lo, cnt, n, C, lane, warp, sh);
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
bool launch_scan(const Dims &D, const CompactOps &ops, int a, double *io, const double *vel, double *f1, double *f2,
                 const double *ltA, const double *ltB, cudaStream_t s) {
    // the shape the matrix tables were built for (scan_shape); none for lines that are too long
    if (!ltA || ops.lane_n[a] != D.N[a]) return false;
    const int b = (a + 1) % 3, c = (a + 2) % 3;
    const int fast = b > c ? b : c, slow = b > c ? c : b;
    const long long lines = (long long)D.N[b] * D.N[c];
    const int wpl = ops.lane_wpl[a], C = ops.lane_c[a];
    if (wpl > 1) {
        const unsigned blocks = unsigned(lines);
        const int tpb = 32 * wpl;
#define SCAN_WPL(W)                                                                                              \
    if (C <= 2) scan_kernel<MODE, 2, W><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, ltA, ltB, D, a, fast, slow); \
    else if (C <= 4) scan_kernel<MODE, 4, W><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, ltA, ltB, D, a, fast,   \
                                                                      slow);                                        \
    else if (C <= 8) scan_kernel<MODE, 8, W><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, ltA, ltB, D, a, fast,   \
                                                                      slow);                                        \
    else if (C <= 16) scan_kernel<MODE, 16, W><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, ltA, ltB, D, a, fast, \
                                                                        slow);                                      \
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
    if (C <= 4) scan_kernel<MODE, 4, 1><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, ltA, ltB, D, a, fast, slow);
    else if (C <= 8) scan_kernel<MODE, 8, 1><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, ltA, ltB, D, a, fast, slow);
    else if (C <= 16)
        scan_kernel<MODE, 16, 1><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, ltA, ltB, D, a, fast, slow);
    else return false;
    return true;
}

}  // namespace

bool scan_uccd(const Dims &D, const CompactOps &ops, int a, const double *flux, const double *vel, double *f1,
               double *f2, cudaStream_t s) {
    return launch_scan<1>(D, ops, a, const_cast<double *>(flux), vel, f1, f2, ops.lane_up[a], ops.lane_down[a], s);
}

bool scan_ccd(const Dims &D, const CompactOps &ops, int a, const double *flux, double *f1, double *f2,
              cudaStream_t s) {
    return launch_scan<0>(D, ops, a, const_cast<double *>(flux), nullptr, f1, f2, ops.lane_ccd[a], nullptr, s);
}

bool scan_mixed(const Dims &D, const CompactOps &ops, int a, double *src, double *out, cudaStream_t s) {
    return launch_scan<2>(D, ops, a, src, nullptr, out, nullptr, ops.lane_ccd[a], nullptr, s);
}

}  // namespace scihpc
