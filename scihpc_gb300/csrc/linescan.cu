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
#include "tc.cuh"

namespace scihpc {

namespace {

// NS independent systems (UCCD's upwind and downwind pair, or one): rhs r[q][k] (2-vectors) of
// the lane's points lo .. lo+cnt-1 in, solutions out (in place), every phase run for all
// systems together (independent FP64 chains in flight, one barrier and one shuffle round for
// both).  lt[q]: the tables of system q for this launch shape (lane_table in compact.cu),
// thread index fastest so that every load of a warp is coalesced: per point of the chunk
// {-L00 -L01 -L10 -L11, K00 K01 K10 K11, D00 D01 D10 D11} (L negated: each row of the forward
// step is two FMAs), then the matrix halves of the chunk and scan maps, so that only the vector
// halves are formed here; tid: the thread's index within its line.
// SW: lanes per line within a warp (32, or 16 for two lines per warp when lines are many and
// moderately long: fewer idle lanes and one shuffle step less); lane is the lane within them.
template <int NS, int CM, int WPL, int SW = 32>
__device__ __forceinline__ void solve_systems(double (&r0)[2][CM], double (&r1)[2][CM], const double *__restrict__ ltA,
                                              const double *__restrict__ ltB, int tid, int lo, int cnt, int n, int C,
                                              int lane, int warp, double2 (*sh)[WPL > 1 ? WPL : 1]) {
    constexpr unsigned FULL = 0xffffffffu;
    static_assert(SW == 32 || (SW == 16 && WPL == 1), "half-warp lines have one segment");
    constexpr int T = SW * WPL;
    constexpr int STEPS = SW == 32 ? 5 : 4;
    const double *pt[2], *me[2], *wt[2];
#pragma unroll
    for (int q = 0; q < NS; ++q) {
        const double *lt = q == 0 ? ltA : ltB;
        pt[q] = lt + tid;                                       // [k][12][T]
        me[q] = lt + (size_t)C * 12 * T + tid;                  // [48][T]
        wt[q] = lt + (size_t)C * 12 * T + (size_t)48 * T;       // [WPL][8]
    }
    // forward: the chunk's map applied to a zero entry vector, inclusive warp scan, replay
    double c0[2] = {0.0, 0.0}, c1[2] = {0.0, 0.0};
#pragma unroll
    for (int k = 0; k < CM; ++k) {
        if (k < cnt) {
            const int i = lo + k;
#pragma unroll
            for (int q = 0; q < NS; ++q) {
                if (i == 0) {
                    c0[q] = r0[q][k], c1[q] = r1[q][k];
                } else {
                    const double *t = pt[q] + (size_t)k * 12 * T;
                    const double a = fma(t[0 * T], c0[q], fma(t[1 * T], c1[q], r0[q][k]));
                    const double b = fma(t[2 * T], c0[q], fma(t[3 * T], c1[q], r1[q][k]));
                    c0[q] = a, c1[q] = b;
                }
            }
        }
    }
#pragma unroll
    for (int st = 0; st < STEPS; ++st) {
        const int d = 1 << st;
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            const double o0 = __shfl_up_sync(FULL, c0[q], d, SW), o1 = __shfl_up_sync(FULL, c1[q], d, SW);
            if (lane >= d) {
                const double *ml = me[q] + 4 * st * T;
                const double a = fma(ml[0 * T], o0, fma(ml[1 * T], o1, c0[q]));
                const double b = fma(ml[2 * T], o0, fma(ml[3 * T], o1, c1[q]));
                c0[q] = a, c1[q] = b;
            }
        }
    }
    double v0[2], v1[2];   // v at lo-1
#pragma unroll
    for (int q = 0; q < NS; ++q) v0[q] = __shfl_up_sync(FULL, c0[q], 1, SW), v1[q] = __shfl_up_sync(FULL, c1[q], 1, SW);
    if (WPL > 1) {
        // warp w enters with the composition of warps 0 .. w-1
        if (lane == 31) {
#pragma unroll
            for (int q = 0; q < NS; ++q) sh[q][warp] = make_double2(c0[q], c1[q]);
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            double p0 = 0.0, p1 = 0.0;
            for (int w = 0; w < warp; ++w) {
                const double *m = wt[q] + 8 * w;
                const double a = fma(m[0], p0, fma(m[1], p1, sh[q][w].x));
                const double b = fma(m[2], p0, fma(m[3], p1, sh[q][w].y));
                p0 = a, p1 = b;
            }
            if (lane == 0) {
                v0[q] = p0, v1[q] = p1;
            } else {
                const double *ml = me[q] + 20 * T;
                const double a = fma(ml[0 * T], p0, fma(ml[1 * T], p1, v0[q]));
                const double b = fma(ml[2 * T], p0, fma(ml[3 * T], p1, v1[q]));
                v0[q] = a, v1[q] = b;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < CM; ++k) {
        if (k < cnt) {
            const int i = lo + k;
#pragma unroll
            for (int q = 0; q < NS; ++q) {
                if (i == 0) {
                    v0[q] = r0[q][k], v1[q] = r1[q][k];
                } else {
                    const double *t = pt[q] + (size_t)k * 12 * T;
                    const double a = fma(t[0 * T], v0[q], fma(t[1 * T], v1[q], r0[q][k]));
                    const double b = fma(t[2 * T], v0[q], fma(t[3 * T], v1[q], r1[q][k]));
                    v0[q] = a, v1[q] = b;
                }
                r0[q][k] = v0[q], r1[q][k] = v1[q];
            }
        }
    }
    // backward: e_i = Dinv_i v_i (kept in r), the chunk's map applied to a zero exit vector,
    // reverse warp scan, replay
    double g0[2] = {0.0, 0.0}, g1[2] = {0.0, 0.0};
#pragma unroll
    for (int k = CM - 1; k >= 0; --k) {
        if (k < cnt) {
            const int i = lo + k;
#pragma unroll
            for (int q = 0; q < NS; ++q) {
                const double *t = pt[q] + (size_t)k * 12 * T;
                const double e0 = fma(t[8 * T], r0[q][k], t[9 * T] * r1[q][k]);
                const double e1 = fma(t[10 * T], r0[q][k], t[11 * T] * r1[q][k]);
                r0[q][k] = e0, r1[q][k] = e1;
                if (i == n - 1) {
                    g0[q] = e0, g1[q] = e1;
                } else {
                    const double a = fma(t[4 * T], g0[q], fma(t[5 * T], g1[q], e0));
                    const double b = fma(t[6 * T], g0[q], fma(t[7 * T], g1[q], e1));
                    g0[q] = a, g1[q] = b;
                }
            }
        }
    }
#pragma unroll
    for (int st = 0; st < STEPS; ++st) {
        const int d = 1 << st;
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            const double o0 = __shfl_down_sync(FULL, g0[q], d, SW), o1 = __shfl_down_sync(FULL, g1[q], d, SW);
            if (lane + d < SW) {
                const double *ml = me[q] + (24 + 4 * st) * T;
                const double a = fma(ml[0 * T], o0, fma(ml[1 * T], o1, g0[q]));
                const double b = fma(ml[2 * T], o0, fma(ml[3 * T], o1, g1[q]));
                g0[q] = a, g1[q] = b;
            }
        }
    }
    double x0[2], x1[2];   // x at lo+cnt
#pragma unroll
    for (int q = 0; q < NS; ++q) x0[q] = __shfl_down_sync(FULL, g0[q], 1, SW), x1[q] = __shfl_down_sync(FULL, g1[q], 1, SW);
    if (WPL > 1) {
        // composition of the warps after this one
        if (lane == 0) {
#pragma unroll
            for (int q = 0; q < NS; ++q) sh[q][warp] = make_double2(g0[q], g1[q]);
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            double p0 = 0.0, p1 = 0.0;
            for (int w = WPL - 1; w > warp; --w) {
                const double *m = wt[q] + 8 * w + 4;
                const double a = fma(m[0], p0, fma(m[1], p1, sh[q][w].x));
                const double b = fma(m[2], p0, fma(m[3], p1, sh[q][w].y));
                p0 = a, p1 = b;
            }
            if (lane == 31) {
                x0[q] = p0, x1[q] = p1;
            } else {
                const double *ml = me[q] + 44 * T;
                const double a = fma(ml[0 * T], p0, fma(ml[1 * T], p1, x0[q]));
                const double b = fma(ml[2 * T], p0, fma(ml[3 * T], p1, x1[q]));
                x0[q] = a, x1[q] = b;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int k = CM - 1; k >= 0; --k) {
        if (k < cnt) {
            const int i = lo + k;
#pragma unroll
            for (int q = 0; q < NS; ++q) {
                if (i == n - 1) {
                    x0[q] = r0[q][k], x1[q] = r1[q][k];
                } else {
                    const double *t = pt[q] + (size_t)k * 12 * T;
                    const double a = fma(t[4 * T], x0[q], fma(t[5 * T], x1[q], r0[q][k]));
                    const double b = fma(t[6 * T], x0[q], fma(t[7 * T], x1[q], r1[q][k]));
                    x0[q] = a, x1[q] = b;
                }
                r0[q][k] = x0[q], r1[q][k] = x1[q];
            }
        }
    }
}

// MODE 0: CCD (f1 = f', f2 = f''); MODE 1: UCCD (f1 = upwind-selected f', f2 = mean f'');
// MODE 2: mixed derivative -- `io` is first zero-order extrapolated along the line in place,
// f1 = its CCD first derivative.
// WPL == 1: each warp of the block solves its own line.  WPL > 1: the block's WPL warps solve
// one line together (shorter chunks per lane, and the per-warp maps combined in shared memory).
template <int MODE, int CM, int WPL, int SW = 32>
__global__ void __launch_bounds__(256) scan_kernel(double *__restrict__ io, const double *__restrict__ vel,
                                                   double *__restrict__ f1, double *__restrict__ f2,
                                                   const double *__restrict__ ltA, const double *__restrict__ ltB,
                                                   Dims D, int a, int fast, int slow) {
    __shared__ double2 sh[2][WPL > 1 ? WPL : 1];
    // lane: the thread's lane within its line's SW lanes
    const int lane = threadIdx.x & (SW - 1), warp = threadIdx.x >> 5;
    const long long line = WPL > 1 ? (long long)blockIdx.x : (long long)blockIdx.x * (blockDim.x / SW) + threadIdx.x / SW;
    const long long nf = D.N[fast], ns = D.N[slow];
    // SW 32: uniform per warp (per block when WPL > 1); SW 16: the second half-warp of the
    // grid's last warp may have no line, and it still takes part in the shuffles (which stay
    // within each half)
    const bool has_line = line < nf * ns;
    if (SW == 32 && !has_line) return;
    int idx[3];
    idx[a] = 0;
    idx[fast] = int(line % nf);
    idx[slow] = int(line / nf);
    const long long base = D.at(idx[0], idx[1], idx[2]);
    const long long st = D.s[a];
    const int n = D.N[a];
    const double ih = D.rd[a], ih2 = ih * ih;
    const int C = (n + SW * WPL - 1) / (SW * WPL);
    const int lo = (WPL > 1 ? int(threadIdx.x) : lane) * C;
    const int cnt = !has_line || lo >= n ? 0 : (lo + C <= n ? C : n - lo);
    double *f = io + base;
    auto src = [&](int i) -> int {
        if (MODE != 2) return i;
        return i < GHC ? GHC : (i > n - 1 - GHC ? n - 1 - GHC : i);
    };
    auto F = [&](int i) { return f[(long long)src(i) * st]; };
    double r0[2][CM], r1[2][CM];   // [0]: the (upwind) system, [1]: UCCD's downwind system
    const double c3 = -0.06096119008109, c2 = 1.99692238016218, c1 = -1.93596119008109;
    const double k3 = 3.0 * ih2, k6 = -6.0 * ih2, k15 = 15.0 / 16.0 * ih;
    const double u1 = c1 * ih, u2 = c2 * ih, u3 = c3 * ih, w1 = -c3 * ih, w2 = -c2 * ih, w3 = -c1 * ih;
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
                r0[0][k] = s, r1[0][k] = ss;
                r0[1][k] = s, r1[1][k] = ss;
            } else {
                // interior stencils with the 1 / h factors folded into the coefficients
                const double ss = fma(k3, fm + fp, k6 * fc);
                if (MODE == 1) {
                    r0[0][k] = fma(u1, fm, fma(u2, fc, u3 * fp));
                    r0[1][k] = fma(w1, fm, fma(w2, fc, w3 * fp));
                    r1[1][k] = ss;
                } else {
                    r0[0][k] = k15 * (fp - fm);
                }
                r1[0][k] = ss;
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
    solve_systems<MODE == 1 ? 2 : 1, CM, WPL, SW>(r0, r1, ltA, ltB, tid, lo, cnt, n, C, lane, warp, sh);
#pragma unroll
    for (int k = 0; k < CM; ++k) {
        if (k < cnt) {
            const long long o = base + (long long)(lo + k) * st;
            if (MODE == 1) {
                f1[o] = vel[o] > 0 ? r0[0][k] : r0[1][k];
                f2[o] = 0.5 * (r1[0][k] + r1[1][k]);
            } else if (MODE == 0) {
                f1[o] = r0[0][k];
                f2[o] = r1[0][k];
            } else {
                f1[o] = r0[0][k];
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
    // many lines: one warp per line (two with 16-lane lines), up to eight warps per block
    const int lpw = ops.lane_seg[a] == 16 ? 2 : 1;
    int wpb = 1;
    while (wpb < 8 && lines >= (long long)wpb * lpw * 2 * 4 * NUM_SMS) wpb *= 2;
    const unsigned blocks = unsigned((lines + (long long)wpb * lpw - 1) / ((long long)wpb * lpw));
    const int tpb = 32 * wpb;
    if (lpw == 2) {
        if (C > 10) return false;
        scan_kernel<MODE, 10, 1, 16><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, ltA, ltB, D, a, fast, slow);
        return true;
    }
    if (C <= 4) scan_kernel<MODE, 4, 1><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, ltA, ltB, D, a, fast, slow);
    else if (C <= 8) scan_kernel<MODE, 8, 1><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, ltA, ltB, D, a, fast, slow);
    else if (C <= 16)
        scan_kernel<MODE, 16, 1><<<blocks, tpb, 0, s>>>(io, vel, f1, f2, ltA, ltB, D, a, fast, slow);
    else return false;
    return true;
}

// ------------------------------------------------------------ sequential solves (3D)
// One thread per line and system, in the order of the factored solve (forward elimination,
// then back substitution: matrix_solver.cpp:56-83), with the lines staged in shared memory.
// A scan composes and replays each chunk's maps and combines 32 of them: about 150 FP64
// operations per point for UCCD's two systems, where the recurrences themselves need 42.
// Which one is faster depends on the line count: a 3D grid has thousands of lines per axis
// (one warp per SM sub-partition at 128 x 64 x 64), enough to keep the FP64 pipes busy with
// one thread per line; a 2D grid has a few hundred, and keeps the scan.
// Block: LPB consecutive lines x NS systems (thread t: line t % LPB, system t / LPB).  Shared
// memory: the lines' values F[LPB][pf] (MODE 2: already extrapolated), for UCCD the upwinding
// velocity W[LPB][pf], then per system and line the forward values, overwritten by the
// solution, V[NS][LPB][pv] as (value, second) pairs; odd pitches keep a half-warp's 8-byte
// accesses on distinct banks.  The block copies its lines in with asynchronous copies, all in
// flight at once, in the order that is contiguous in memory (along the line when it is the
// fastest axis, across lines otherwise), and stores the results in the same order.
// op: per point {L (4), U (4), Dinv (4)} of the factored system, read through L1 (every
// thread of a warp reads the same point).
constexpr int SEQ_MAX_LPB = 32;

template <int MODE, int NS>
__global__ void __launch_bounds__(SEQ_MAX_LPB * 2) seq_kernel(double *__restrict__ io, const double *__restrict__ vel,
                                                              double *__restrict__ f1, double *__restrict__ f2,
                                                              const double *__restrict__ opA,
                                                              const double *__restrict__ opB, Dims D, int a, int fast,
                                                              int slow, int lpb, int pf, int pv) {
    extern __shared__ __align__(16) double seq_sm[];
    __shared__ long long bse[SEQ_MAX_LPB];
    double *F = seq_sm;
    double *W = F + (size_t)lpb * pf;   // UCCD only
    double *V = W + (MODE == 1 ? (size_t)lpb * pf : 0);
    const int n = D.N[a];
    const long long nf = D.N[fast], lines = nf * D.N[slow];
    const long long line0 = (long long)blockIdx.x * lpb;
    const int nl = int(lines - line0 < lpb ? lines - line0 : lpb);   // lines of this block
    const long long st = D.s[a];
    const int tid = threadIdx.x, nt = blockDim.x;
    if (tid < nl) {
        const long long line = line0 + tid;
        int idx[3];
        idx[a] = 0;
        idx[fast] = int(line % nf);
        idx[slow] = int(line / nf);
        bse[tid] = D.at(idx[0], idx[1], idx[2]);
    }
    __syncthreads();
    const int total = nl * n;
    auto src = [&](int i) -> int {
        if (MODE != 2) return i;
        return i < GHC ? GHC : (i > n - 1 - GHC ? n - 1 - GHC : i);
    };
    auto fetch = [&](int l, int i) {
        tc::cp8(&F[l * pf + i], &io[bse[l] + (long long)src(i) * st]);
        if (MODE == 1) tc::cp8(&W[l * pf + i], &vel[bse[l] + (long long)i * st]);
    };
    if (st == 1) {
        for (int e = tid; e < total; e += nt) {
            const int l = e / n;
            fetch(l, e - l * n);
        }
    } else {
        for (int e = tid; e < total; e += nt) {
            const int i = e / nl;
            fetch(e - i * nl, i);
        }
    }
    tc::cp_commit();
    tc::cp_wait_all();
    __syncthreads();
    const int l = tid % lpb, q = tid / lpb;
    if (l < nl && q < NS) {
        const double *f = F + l * pf;
        double *v = V + ((size_t)q * lpb + l) * pv;
        const double *op = q == 0 ? opA : opB;
        const double ih = D.rd[a], ih2 = ih * ih;
        const double c3 = -0.06096119008109, c2 = 1.99692238016218, c1 = -1.93596119008109;
        // interior stencils with the 1 / h factors folded into the coefficients; UCCD's
        // downwind system has the mirrored first-derivative stencil
        const double k3 = 3.0 * ih2, k6 = -6.0 * ih2, k15 = 15.0 / 16.0 * ih;
        const double s1c = (q == 0 ? c1 : -c3) * ih, s2c = (q == 0 ? c2 : -c2) * ih, s3c = (q == 0 ? c3 : -c1) * ih;
        // forward elimination; one-sided closures at both ends (uccd_solver.cpp:29-51,
        // ccd_solver.cpp:31-40), interior right-hand sides (uccd_solver.cpp:17-19,:33-41,
        // ccd_solver.cpp:22-28)
        double u_p = (-3.5 * f[0] + 4.0 * f[1] - 0.5 * f[2]) * ih;
        double uu_p = (9.0 * f[0] - 12.0 * f[1] + 3.0 * f[2]) * ih * ih;
        v[0] = u_p;
        v[1] = uu_p;
        double fm = f[0], f0 = f[1];
#pragma unroll 2
        for (int i = 1; i < n - 1; ++i) {
            const double fp = f[i + 1];
            double ssu = fma(k3, fm + fp, k6 * f0);
            double su;
            if (MODE == 1) su = fma(s1c, fm, fma(s2c, f0, s3c * fp));
            else su = k15 * (fp - fm);
            fm = f0;
            f0 = fp;
            const double *r = op + (size_t)i * 12;
            su = fma(-r[0], u_p, fma(-r[1], uu_p, su));
            ssu = fma(-r[2], u_p, fma(-r[3], uu_p, ssu));
            u_p = su, uu_p = ssu;
            v[2 * i] = su;
            v[2 * i + 1] = ssu;
        }
        {
            const int i = n - 1;
            double su = -(-3.5 * f[n - 1] + 4.0 * f[n - 2] - 0.5 * f[n - 3]) * ih;
            double ssu = (9.0 * f[n - 1] - 12.0 * f[n - 2] + 3.0 * f[n - 3]) * ih * ih;
            const double *r = op + (size_t)i * 12;
            su = fma(-r[0], u_p, fma(-r[1], uu_p, su));
            ssu = fma(-r[2], u_p, fma(-r[3], uu_p, ssu));
            // back substitution starts here
            double xu = r[8] * su + r[9] * ssu;
            double yu = r[10] * su + r[11] * ssu;
            v[2 * i] = xu;
            v[2 * i + 1] = yu;
#pragma unroll 2
            for (int k = n - 2; k >= 0; --k) {
                const double *rk = op + (size_t)k * 12;
                double sk = v[2 * k], ssk = v[2 * k + 1];
                sk = fma(-rk[4], xu, fma(-rk[5], yu, sk));
                ssk = fma(-rk[6], xu, fma(-rk[7], yu, ssk));
                xu = fma(rk[8], sk, rk[9] * ssk);
                yu = fma(rk[10], sk, rk[11] * ssk);
                v[2 * k] = xu;
                v[2 * k + 1] = yu;
            }
        }
    }
    __syncthreads();
    auto put = [&](int l2, int i) {
        const long long o = bse[l2] + (long long)i * st;
        const double *x0 = V + (size_t)l2 * pv + 2 * i;
        if (MODE == 1) {
            const double *x1 = V + ((size_t)lpb + l2) * pv + 2 * i;
            f1[o] = W[l2 * pf + i] > 0 ? x0[0] : x1[0];
            f2[o] = 0.5 * (x0[1] + x1[1]);
        } else if (MODE == 0) {
            f1[o] = x0[0];
            f2[o] = x0[1];
        } else {
            f1[o] = x0[0];
            // the reference extrapolates the source in place (ccd_solver.cpp:151-155)
            if (i < GHC || i > n - 1 - GHC) io[o] = F[l2 * pf + i];
        }
    };
    if (st == 1) {
        for (int e = tid; e < total; e += nt) {
            const int l2 = e / n;
            put(l2, e - l2 * n);
        }
    } else {
        for (int e = tid; e < total; e += nt) {
            const int i = e / nl;
            put(e - i * nl, i);
        }
    }
}

// Sequential solves for 3D grids with lines short enough; false (nothing launched) otherwise,
// and the scans run.
template <int MODE>
bool launch_seq(const Dims &D, int a, double *io, const double *vel, double *f1, double *f2, const double *opA,
                const double *opB, cudaStream_t s) {
    if (D.ndim != 3 || !opA) return false;
    constexpr int NS = MODE == 1 ? 2 : 1;
    const int n = D.N[a];
    const int pf = n | 1, pv = 2 * n + 1;
    auto bytes = [&](int lpb) {
        return size_t(lpb) * ((MODE == 1 ? 2 : 1) * size_t(pf) + size_t(NS) * pv) * sizeof(double);
    };
    // One thread per line keeps about a sixth of an SM's FP64 pipe busy per warp (the
    // recurrence is a dependency chain), so the sequential solve pays only with at least four
    // warps per SM; longer lines, whose blocks fill an SM's shared memory with fewer threads,
    // keep the scan (at 128 x 64 x 64: 88 us sequential against 185 us scanned along y and z,
    // 317 us against 167 us along x).
    const int lpb = SEQ_MAX_LPB;
    const size_t smem_sm = 228 * 1024, per_block = bytes(lpb) + 1024;
    if ((int)(smem_sm / per_block) * NS < 4) return false;
    static bool attr_set = false;   // one instantiation per MODE
    if (!attr_set) {
        if (cudaFuncSetAttribute(seq_kernel<MODE, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
            cudaSuccess)
            return false;
        attr_set = true;
    }
    const int b = (a + 1) % 3, c = (a + 2) % 3;
    const int fast = b > c ? b : c, slow = b > c ? c : b;
    const long long lines = (long long)D.N[b] * D.N[c];
    const unsigned blocks = unsigned((lines + lpb - 1) / lpb);
    seq_kernel<MODE, NS><<<blocks, lpb * NS, bytes(lpb), s>>>(io, vel, f1, f2, opA, opB, D, a, fast, slow, lpb, pf,
                                                               pv);
    return true;
}

}  // namespace

bool seq_uccd(const Dims &D, const CompactOps &ops, int a, const double *flux, const double *vel, double *f1,
              double *f2, cudaStream_t s) {
    return launch_seq<1>(D, a, const_cast<double *>(flux), vel, f1, f2, ops.up[a], ops.down[a], s);
}

bool seq_ccd(const Dims &D, const CompactOps &ops, int a, const double *flux, double *f1, double *f2,
             cudaStream_t s) {
    return launch_seq<0>(D, a, const_cast<double *>(flux), nullptr, f1, f2, ops.ccd[a], nullptr, s);
}

bool seq_mixed(const Dims &D, const CompactOps &ops, int a, double *src, double *out, cudaStream_t s) {
    return launch_seq<2>(D, a, src, nullptr, out, nullptr, ops.ccd[a], nullptr, s);
}

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
