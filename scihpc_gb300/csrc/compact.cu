// compact.cu -- combined compact difference (CCD) and upwind CCD (UCCD) line solves.
//
// Both schemes solve, along every grid line of one axis (ghosts included), a 2x2
// block-tridiagonal system for (f', f'') whose matrix depends only on the line length and
// spacing (uccd_base.cpp:7-118, ccd_base.cpp:7-105, matrix_solver.cpp:20-83).  The block LU
// factorisation is done once on the host per axis; the device keeps, per line position i,
// the elimination multipliers, the upper blocks and the inverse of the reduced diagonal
// block.  One thread owns one line: a forward sweep builds the right-hand side on the fly
// and eliminates, storing the partial results in the output arrays (and, for UCCD's second
// system, a scratch pair), then the backward sweep finishes the line holding only the i+1
// values in registers.  This sequential form serves lines longer than the warp-cooperative
// solver of linescan.cu handles (more than 512 points).
#include <algorithm>
#include <array>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "compact.cuh"

namespace scihpc {

namespace {

struct HostLineOp {
    int n = 0;
    std::vector<double> P[3], Q[3], R[3], S[3];
    void blank(int len) {
        n = len;
        for (int m = 0; m < 3; ++m) {
            P[m].assign(n, 0.0);
            Q[m].assign(n, 0.0);
            R[m].assign(n, 0.0);
            S[m].assign(n, 0.0);
        }
    }
};

// One-sided closure rows with alpha1 = 2, beta1 = -1, alpha2 = 5, beta2 = -6
// (ccd_base.cpp:63-101, uccd_base.cpp:165-221).
void closure_rows(HostLineOp &op, double h) {
    const int e = op.n - 1;
    op.P[0][0] = 0.0, op.P[1][0] = 1.0, op.P[2][0] = 2.0;
    op.Q[0][0] = 0.0, op.Q[1][0] = 0.0, op.Q[2][0] = -1.0 * h;
    op.R[0][0] = 0.0, op.R[1][0] = 0.0, op.R[2][0] = -6.0 / h;
    op.S[0][0] = 0.0, op.S[1][0] = 1.0, op.S[2][0] = 5.0;
    op.P[0][e] = 2.0, op.P[1][e] = 1.0, op.P[2][e] = 0.0;
    op.Q[0][e] = 1.0 * h, op.Q[1][e] = 0.0, op.Q[2][e] = 0.0;
    op.R[0][e] = 6.0 / h, op.R[1][e] = 0.0, op.R[2][e] = 0.0;
    op.S[0][e] = 5.0, op.S[1][e] = 1.0, op.S[2][e] = 0.0;
}

// Block LU of the 2x2 block-tridiagonal operator (the elimination of matrix_solver.cpp:20-54).
void factor(HostLineOp &op) {
    const int n = op.n;
    op.P[0][0] = 0.0, op.R[0][0] = 0.0, op.Q[0][0] = 1.0, op.S[0][0] = 1.0;
    op.P[2][n - 1] = 0.0, op.R[2][n - 1] = 0.0, op.Q[2][n - 1] = 1.0, op.S[2][n - 1] = 1.0;
    for (int i = 1; i < n; ++i) {
        const double den = op.P[1][i - 1] * op.S[1][i - 1] - op.R[1][i - 1] * op.Q[1][i - 1];
        double m1 = -(op.R[1][i - 1] * op.Q[0][i] - op.P[0][i] * op.S[1][i - 1]) / den;
        double m2 = (op.Q[0][i] * op.P[1][i - 1] - op.Q[1][i - 1] * op.P[0][i]) / den;
        op.P[0][i] = m1;
        op.P[1][i] = op.P[1][i] - (m1 * op.P[2][i - 1] + m2 * op.R[2][i - 1]);
        op.Q[0][i] = m2;
        op.Q[1][i] = op.Q[1][i] - (m1 * op.Q[2][i - 1] + m2 * op.S[2][i - 1]);
        m1 = -(op.R[1][i - 1] * op.S[0][i] - op.R[0][i] * op.S[1][i - 1]) / den;
        m2 = (op.S[0][i] * op.P[1][i - 1] - op.Q[1][i - 1] * op.R[0][i]) / den;
        op.R[0][i] = m1;
        op.R[1][i] = op.R[1][i] - (m1 * op.P[2][i - 1] + m2 * op.R[2][i - 1]);
        op.S[0][i] = m2;
        op.S[1][i] = op.S[1][i] - (m1 * op.Q[2][i - 1] + m2 * op.S[2][i - 1]);
    }
}

HostLineOp ccd_op(int n, double h) {
    HostLineOp op;
    op.blank(n);
    for (int i = 0; i < n; ++i) {   // ccd_base.cpp:45-61
        op.P[0][i] = 7.0 / 16.0, op.P[1][i] = 1.0, op.P[2][i] = 7.0 / 16.0;
        op.Q[0][i] = h / 16.0, op.Q[1][i] = 0.0, op.Q[2][i] = -h / 16.0;
        op.R[0][i] = -9.0 / 8.0 / h, op.R[1][i] = 0.0, op.R[2][i] = 9.0 / 8.0 / h;
        op.S[0][i] = -1.0 / 8.0, op.S[1][i] = 1.0, op.S[2][i] = -1.0 / 8.0;
    }
    closure_rows(op, h);
    factor(op);
    return op;
}

void uccd_ops(int n, double h, HostLineOp &up, HostLineOp &dn) {
    up.blank(n);
    dn.blank(n);
    const double a1 = 0.875;   // uccd_base.cpp:129-132
    const double b1 = 0.1251282341599089, b2 = -0.2487176584009104, b3 = 0.0001282341599089;
    for (int i = 0; i < n; ++i) {
        up.P[0][i] = a1, up.P[1][i] = 1.0, up.P[2][i] = 0.0;
        dn.P[0][i] = 0.0, dn.P[1][i] = 1.0, dn.P[2][i] = a1;
        up.Q[0][i] = b1 * h, up.Q[1][i] = b2 * h, up.Q[2][i] = b3 * h;
        dn.Q[0][i] = -b3 * h, dn.Q[1][i] = -b2 * h, dn.Q[2][i] = -b1 * h;
        for (HostLineOp *op : {&up, &dn}) {
            op->R[0][i] = -9.0 / 8.0 / h, op->R[1][i] = 0.0, op->R[2][i] = 9.0 / 8.0 / h;
            op->S[0][i] = -1.0 / 8.0, op->S[1][i] = 1.0, op->S[2][i] = -1.0 / 8.0;
        }
    }
    closure_rows(up, h);
    closure_rows(dn, h);
    factor(up);
    factor(dn);
}

// Device table of one factored operator, 12 doubles per line position:
// lower multipliers (P0 Q0 R0 S0), upper blocks (P2 Q2 R2 S2), inverse diagonal (a b c d)
// with [x; y] = [a b; c d] [s; ss].
std::vector<double> pack(const HostLineOp &op) {
    std::vector<double> t(size_t(op.n) * 12);
    for (int i = 0; i < op.n; ++i) {
        double *r = &t[size_t(i) * 12];
        r[0] = op.P[0][i], r[1] = op.Q[0][i], r[2] = op.R[0][i], r[3] = op.S[0][i];
        r[4] = op.P[2][i], r[5] = op.Q[2][i], r[6] = op.R[2][i], r[7] = op.S[2][i];
        const double den = op.P[1][i] * op.S[1][i] - op.R[1][i] * op.Q[1][i];
        r[8] = op.S[1][i] / den, r[9] = -op.Q[1][i] / den;
        r[10] = -op.R[1][i] / den, r[11] = op.P[1][i] / den;
    }
    return t;
}

// Scan form (linescan.cu): {L, K = -Dinv U, Dinv} per line position.
std::vector<double> pack_scan(const HostLineOp &op) {
    std::vector<double> t(size_t(op.n) * 12);
    for (int i = 0; i < op.n; ++i) {
        double *r = &t[size_t(i) * 12];
        const double den = op.P[1][i] * op.S[1][i] - op.R[1][i] * op.Q[1][i];
        const double a = op.S[1][i] / den, b = -op.Q[1][i] / den, c = -op.R[1][i] / den, d = op.P[1][i] / den;
        r[0] = op.P[0][i], r[1] = op.Q[0][i], r[2] = op.R[0][i], r[3] = op.S[0][i];
        r[4] = -(a * op.P[2][i] + b * op.R[2][i]);
        r[5] = -(a * op.Q[2][i] + b * op.S[2][i]);
        r[6] = -(c * op.P[2][i] + d * op.R[2][i]);
        r[7] = -(c * op.Q[2][i] + d * op.S[2][i]);
        r[8] = a, r[9] = b, r[10] = c, r[11] = d;
    }
    return t;
}

// Tables of the warp-cooperative solve (linescan.cu) for one launch shape: lines of n points,
// T = 32 * wpl threads per line, thread t holding points t*C .. t*C+C-1.  Thread index fastest,
// so that a warp's loads are coalesced:
//   [C][12][T]  the per-point factors {-L (4), K (4), Dinv (4)} of point t*C+k (zero past n);
//   [48][T]     the matrix halves of the scan maps.  A lane's chunk map and every partial map of
//               the shuffle scans are affine maps x -> M x + c whose matrices depend only on the
//               factorisation and the shape, so they are formed here once per axis and the kernel
//               carries the 2-vectors c alone: [0,20) the forward partial matrix of t before each
//               of the five shuffle steps, [20,24) the final forward matrix of thread t-1 of the
//               same warp, [24,44) and [44,48) the same for the backward scan (thread t+1);
//   [wpl][8]    per warp, the final forward matrix of its lane 31 and the final backward matrix
//               of its lane 0.
namespace {
using Mat2 = std::array<double, 4>;

// b a (row-major 2x2)
Mat2 mat_mul(const Mat2 &b, const Mat2 &a) {
    return {b[0] * a[0] + b[1] * a[2], b[0] * a[1] + b[1] * a[3], b[2] * a[0] + b[3] * a[2],
            b[2] * a[1] + b[3] * a[3]};
}
}  // namespace

std::vector<double> lane_table(const std::vector<double> &tab, int n, int wpl, int C, int seg) {
    const int T = seg * wpl;   // seg: lanes per line (32, or 16 with wpl 1)
    const size_t pts = size_t(C) * 12 * T;
    std::vector<double> out(pts + size_t(T) * 48 + size_t(wpl) * 8, 0.0);
    for (int t = 0; t < T; ++t)
        for (int k = 0; k < C && t * C + k < n; ++k)
            for (int q = 0; q < 12; ++q) {
                const double x = tab[size_t(t * C + k) * 12 + q];
                out[(size_t(k) * 12 + q) * T + t] = q < 4 ? -x : x;
            }
    const Mat2 I = {1.0, 0.0, 0.0, 1.0}, Z = {0.0, 0.0, 0.0, 0.0};
    std::vector<Mat2> F(T), G(T);
    for (int t = 0; t < T; ++t) {
        const int lo = t * C, cnt = lo >= n ? 0 : std::min(C, n - lo);
        Mat2 f = I, g = I;
        for (int k = 0; k < cnt; ++k) {
            const double *r = &tab[size_t(lo + k) * 12];
            f = lo + k == 0 ? Z : mat_mul({-r[0], -r[1], -r[2], -r[3]}, f);
        }
        for (int k = cnt - 1; k >= 0; --k) {
            const double *r = &tab[size_t(lo + k) * 12];
            g = lo + k == n - 1 ? Z : mat_mul({r[4], r[5], r[6], r[7]}, g);
        }
        F[t] = f;
        G[t] = g;
    }
    const int S = seg;   // lanes of one shuffle scan
    for (int w = 0; w < wpl; ++w) {
        Mat2 *f = &F[size_t(w) * S], *g = &G[size_t(w) * S];
        for (int st = 0, d = 1; d < S; ++st, d <<= 1) {
            const std::vector<Mat2> f0(f, f + S), g0(g, g + S);
            for (int l = 0; l < S; ++l) {
                double *e = &out[pts + size_t(w) * S + l];
                for (int q = 0; q < 4; ++q) {
                    e[size_t(4 * st + q) * T] = f0[l][q];
                    e[size_t(24 + 4 * st + q) * T] = g0[l][q];
                }
                if (l >= d) f[l] = mat_mul(f0[l], f0[l - d]);
                if (l + d < S) g[l] = mat_mul(g0[l], g0[l + d]);
            }
        }
        for (int l = 0; l < S; ++l) {
            double *e = &out[pts + size_t(w) * S + l];
            for (int q = 0; q < 4; ++q) {
                e[size_t(20 + q) * T] = l > 0 ? f[l - 1][q] : 0.0;
                e[size_t(44 + q) * T] = l < S - 1 ? g[l + 1][q] : 0.0;
            }
        }
        double *wt = &out[pts + size_t(T) * 48 + size_t(w) * 8];
        for (int q = 0; q < 4; ++q) {
            wt[q] = f[S - 1][q];
            wt[4 + q] = g[0][q];
        }
    }
    return out;
}

// Right-hand sides: one-sided three-point closures at both ends and the interior formulas
// (uccd_solver.cpp:21-51 and :17-19,:33-41; ccd_solver.cpp:22-46).
__device__ __forceinline__ void end_rhs(const double *f, long long st, int n, double ih, double &s0, double &ss0,
                                        double &sn, double &ssn) {
    const double f0 = f[0], f1 = f[st], f2 = f[2 * st];
    const double g0 = f[(long long)(n - 1) * st], g1 = f[(long long)(n - 2) * st], g2 = f[(long long)(n - 3) * st];
    s0 = (-3.5 * f0 + 4.0 * f1 - 0.5 * f2) * ih;
    ss0 = (9.0 * f0 - 12.0 * f1 + 3.0 * f2) * ih * ih;
    sn = -(-3.5 * g0 + 4.0 * g1 - 0.5 * g2) * ih;
    ssn = (9.0 * g0 - 12.0 * g1 + 3.0 * g2) * ih * ih;
}

// MODE 0: CCD (outputs f1, f2); MODE 1: UCCD (outputs f1 = upwind-selected first
// derivative, f2 = mean of the two second derivatives; t1/t2 hold the down system's partials).
template <int MODE>
__global__ void __launch_bounds__(128) line_kernel(const double *__restrict__ in, const double *__restrict__ vel,
                                                   double *__restrict__ f1, double *__restrict__ f2,
                                                   double *__restrict__ t1, double *__restrict__ t2,
                                                   const double *__restrict__ opA, const double *__restrict__ opB,
                                                   Dims D, int a, int fast, int slow) {
    const long long nf = D.N[fast], ns = D.N[slow];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nf * ns) return;
    int idx[3];
    idx[a] = 0;
    idx[fast] = int(t % nf);
    idx[slow] = int(t / nf);
    const long long base = D.at(idx[0], idx[1], idx[2]);
    const long long st = D.s[a];
    const int n = D.N[a];
    const double ih = D.rd[a];
    const double *f = in + base;
    double s0, ss0, sn, ssn;
    end_rhs(f, st, n, ih, s0, ss0, sn, ssn);
    const double c3 = -0.06096119008109, c2 = 1.99692238016218, c1 = -1.93596119008109;

    // forward elimination
    double u_p = 0.0, uu_p = 0.0, d_p = 0.0, dd_p = 0.0;   // previous eliminated values
    double fm = f[0], f0 = f[st];
    for (int i = 0; i < n; ++i) {
        double su, ssu, sd = 0.0, ssd = 0.0;
        if (i == 0) {
            su = s0, ssu = ss0;
            sd = s0, ssd = ss0;
        } else if (i == n - 1) {
            su = sn, ssu = ssn;
            sd = sn, ssd = ssn;
        } else {
            const double fp = f[(long long)(i + 1) * st];
            ssu = (3.0 * fm - 6.0 * f0 + 3.0 * fp) * ih * ih;
            if (MODE == 1) {
                su = (c1 * fm + c2 * f0 + c3 * fp) * ih;
                sd = -(c3 * fm + c2 * f0 + c1 * fp) * ih;
                ssd = ssu;
            } else {
                su = 15.0 / 16.0 * (fp - fm) * ih;
            }
            fm = f0;
            f0 = fp;
        }
        if (i > 0) {
            const double *r = opA + (size_t)i * 12;
            su = su - (r[0] * u_p + r[1] * uu_p);
            ssu = ssu - (r[2] * u_p + r[3] * uu_p);
            if (MODE == 1) {
                const double *q = opB + (size_t)i * 12;
                sd = sd - (q[0] * d_p + q[1] * dd_p);
                ssd = ssd - (q[2] * d_p + q[3] * dd_p);
            }
        }
        u_p = su, uu_p = ssu;
        const long long o = base + (long long)i * st;
        f1[o] = su;
        f2[o] = ssu;
        if (MODE == 1) {
            d_p = sd, dd_p = ssd;
            t1[o] = sd;
            t2[o] = ssd;
        }
    }
    // backward substitution
    double xu = 0.0, yu = 0.0, xd = 0.0, yd = 0.0;   // finished values at i+1
    for (int i = n - 1; i >= 0; --i) {
        const long long o = base + (long long)i * st;
        const double *r = opA + (size_t)i * 12;
        double su = f1[o], ssu = f2[o];
        if (i < n - 1) {
            su = su - (r[4] * xu + r[5] * yu);
            ssu = ssu - (r[6] * xu + r[7] * yu);
        }
        xu = r[8] * su + r[9] * ssu;
        yu = r[10] * su + r[11] * ssu;
        if (MODE == 1) {
            const double *q = opB + (size_t)i * 12;
            double sd = t1[o], ssd = t2[o];
            if (i < n - 1) {
                sd = sd - (q[4] * xd + q[5] * yd);
                ssd = ssd - (q[6] * xd + q[7] * yd);
            }
            xd = q[8] * sd + q[9] * ssd;
            yd = q[10] * sd + q[11] * ssd;
            f1[o] = vel[o] > 0 ? xu : xd;
            f2[o] = 0.5 * (yu + yd);
        } else {
            f1[o] = xu;
            f2[o] = yu;
        }
    }
}

}  // namespace

// Mixed derivatives: the source is extrapolated along the axis in place first; the second
// derivative is needed only to complete the elimination and goes to a scratch field.
namespace {
__global__ void __launch_bounds__(128) mixed_kernel(double *__restrict__ src, double *__restrict__ out,
                                                    double *__restrict__ tmp, const double *__restrict__ op, Dims D,
                                                    int a, int fast, int slow) {
    const long long nf = D.N[fast], ns = D.N[slow];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nf * ns) return;
    int idx[3];
    idx[a] = 0;
    idx[fast] = int(t % nf);
    idx[slow] = int(t / nf);
    const long long base = D.at(idx[0], idx[1], idx[2]);
    const long long st = D.s[a];
    const int n = D.N[a];
    const double ih = D.rd[a];
    double *f = src + base;
    const double lo = f[(long long)GHC * st], hi = f[(long long)(n - 1 - GHC) * st];
    for (int q = 0; q < GHC; ++q) {
        f[(long long)q * st] = lo;
        f[(long long)(n - 1 - q) * st] = hi;
    }
    double s0, ss0, sn, ssn;
    end_rhs(f, st, n, ih, s0, ss0, sn, ssn);
    double u_p = 0.0, uu_p = 0.0;
    double fm = f[0], f0 = f[st];
    for (int i = 0; i < n; ++i) {
        double su, ssu;
        if (i == 0) {
            su = s0, ssu = ss0;
        } else if (i == n - 1) {
            su = sn, ssu = ssn;
        } else {
            const double fp = f[(long long)(i + 1) * st];
            ssu = (3.0 * fm - 6.0 * f0 + 3.0 * fp) * ih * ih;
            su = 15.0 / 16.0 * (fp - fm) * ih;
            fm = f0;
            f0 = fp;
        }
        if (i > 0) {
            const double *r = op + (size_t)i * 12;
            su = su - (r[0] * u_p + r[1] * uu_p);
            ssu = ssu - (r[2] * u_p + r[3] * uu_p);
        }
        u_p = su, uu_p = ssu;
        const long long o = base + (long long)i * st;
        out[o] = su;
        tmp[o] = ssu;
    }
    double xu = 0.0, yu = 0.0;
    for (int i = n - 1; i >= 0; --i) {
        const long long o = base + (long long)i * st;
        const double *r = op + (size_t)i * 12;
        double su = out[o], ssu = tmp[o];
        if (i < n - 1) {
            su = su - (r[4] * xu + r[5] * yu);
            ssu = ssu - (r[6] * xu + r[7] * yu);
        }
        xu = r[8] * su + r[9] * ssu;
        yu = r[10] * su + r[11] * ssu;
        out[o] = xu;
    }
}
}  // namespace

int CompactOps::build(const Dims &D) {
    for (int a = 0; a < 3; ++a) {
        ccd[a] = up[a] = down[a] = nullptr;
        if (a >= D.ndim) continue;
        const int n = D.N[a];
        const double h = D.d[a];
        HostLineOp c = ccd_op(n, h), u, dn;
        uccd_ops(n, h, u, dn);
        std::vector<double> tc = pack(c), tu = pack(u), td = pack(dn);
        std::vector<double> sc = pack_scan(c), su = pack_scan(u), sd = pack_scan(dn);
        const size_t bytes = tc.size() * sizeof(double);
        SCIHPC_CUDA(cudaMalloc(&ccd[a], 3 * bytes));
        up[a] = ccd[a] + tc.size();
        down[a] = up[a] + tc.size();
        SCIHPC_CUDA(cudaMemcpy(ccd[a], tc.data(), bytes, cudaMemcpyHostToDevice));
        SCIHPC_CUDA(cudaMemcpy(up[a], tu.data(), bytes, cudaMemcpyHostToDevice));
        SCIHPC_CUDA(cudaMemcpy(down[a], td.data(), bytes, cudaMemcpyHostToDevice));
        int wpl, C, seg;
        if (scan_shape(D, a, wpl, C, seg)) {
            std::vector<double> lc = lane_table(sc, n, wpl, C, seg), lu = lane_table(su, n, wpl, C, seg),
                                ld = lane_table(sd, n, wpl, C, seg);
            const size_t lb = lc.size() * sizeof(double);
            SCIHPC_CUDA(cudaMalloc(&lane_ccd[a], 3 * lb));
            lane_up[a] = lane_ccd[a] + lc.size();
            lane_down[a] = lane_up[a] + lc.size();
            SCIHPC_CUDA(cudaMemcpy(lane_ccd[a], lc.data(), lb, cudaMemcpyHostToDevice));
            SCIHPC_CUDA(cudaMemcpy(lane_up[a], lu.data(), lb, cudaMemcpyHostToDevice));
            SCIHPC_CUDA(cudaMemcpy(lane_down[a], ld.data(), lb, cudaMemcpyHostToDevice));
            lane_wpl[a] = wpl, lane_c[a] = C, lane_n[a] = n, lane_seg[a] = seg;
        }
    }
    return SCIHPC_OK;
}

void CompactOps::release() {
    for (int a = 0; a < 3; ++a) {
        if (ccd[a]) cudaFree(ccd[a]);
        ccd[a] = up[a] = down[a] = nullptr;
        if (lane_ccd[a]) cudaFree(lane_ccd[a]);
        lane_ccd[a] = lane_up[a] = lane_down[a] = nullptr;
        lane_wpl[a] = lane_c[a] = lane_n[a] = 0;
        lane_seg[a] = 32;
    }
}

static void line_layout(const Dims &D, int a, int &fast, int &slow, long long &lines) {
    const int b = (a + 1) % 3, c = (a + 2) % 3;
    fast = b > c ? b : c;
    slow = b > c ? c : b;
    lines = (long long)D.N[b] * D.N[c];
}

void launch_uccd(const Dims &D, const CompactOps &ops, int a, const double *flux, const double *vel, double *f1,
                 double *f2, double *t1, double *t2, cudaStream_t s) {
    if (seq_uccd(D, ops, a, flux, vel, f1, f2, s) || scan_uccd(D, ops, a, flux, vel, f1, f2, s)) return;
    int fast, slow;
    long long lines;
    line_layout(D, a, fast, slow, lines);
    line_kernel<1><<<blocks_for(lines, 128), 128, 0, s>>>(flux, vel, f1, f2, t1, t2, ops.up[a],
                                                          ops.down[a], D, a, fast, slow);
}

void launch_ccd(const Dims &D, const CompactOps &ops, int a, const double *flux, double *f1, double *f2,
                cudaStream_t s) {
    if (seq_ccd(D, ops, a, flux, f1, f2, s) || scan_ccd(D, ops, a, flux, f1, f2, s)) return;
    int fast, slow;
    long long lines;
    line_layout(D, a, fast, slow, lines);
    line_kernel<0><<<blocks_for(lines, 128), 128, 0, s>>>(flux, nullptr, f1, f2, nullptr,
                                                          nullptr, ops.ccd[a], nullptr, D, a, fast, slow);
}

void launch_ccd_mixed(const Dims &D, const CompactOps &ops, int a, double *src, double *out, double *tmp,
                      cudaStream_t s) {
    if (seq_mixed(D, ops, a, src, out, s) || scan_mixed(D, ops, a, src, out, s)) return;
    int fast, slow;
    long long lines;
    line_layout(D, a, fast, slow, lines);
    mixed_kernel<<<blocks_for(lines, 128), 128, 0, s>>>(src, out, tmp, ops.ccd[a], D, a, fast, slow);
}

}  // namespace scihpc
