// bc.cu -- ghost fills (bc_factory + periodic/neumann/no_slip/slip/dirichlet) and the
// zero-order flux extrapolations.
//
// A boundary fill touches one 3-wide ghost slab per face, along the transverse interior
// lines of that face (bc_factory.cpp:123-437 and the per-face kernels).  One thread owns one
// transverse line and applies the right face then the left face, which reproduces the
// reference's sequential order inside each line; threads are laid out so that the
// memory-fastest transverse axis varies fastest across a warp.  Axes are filled x, then y,
// then z, one launch each: a later axis reads cells the earlier axis may have written
// (Dirichlet node fills overwrite the boundary cell, face fills the wall face).
#include "common.cuh"

namespace scihpc {

namespace {

__device__ __forceinline__ void fill_line(double *l, long long sa, int n, bool right, bool face, int type,
                                          double value, double dh) {
    const int L = n - 1 + GHC;
    const int F = GHC;
#define A(i) l[(long long)(i) * sa]
    switch (type) {
        case 0:   // periodic (periodic.cpp:7-161)
            if (right) {
                for (int q = 1; q <= GHC; ++q) A(L + q) = A(GHC + (q - 1));
            } else {
                for (int q = 1; q <= GHC; ++q) A(F - q) = A(L - (q - 1));
            }
            break;
        case 1:   // neumann (neumann.cpp:7-164)
            if (!face) {
                if (right) {
                    for (int q = 1; q <= GHC; ++q) A(L + q) = A(L + q - 1) + value * dh;
                } else {
                    for (int q = 1; q <= GHC; ++q) A(F - q) = A(F - q + 1) - value * dh;
                }
            } else {
                if (right) {
                    A(L) = A(L - 1) + value * dh;
                    for (int q = 1; q <= GHC; ++q) A(L + q) = A(L + q - 1) + value * dh;
                } else {
                    A(F - 1) = A(F) - value * dh;
                    for (int q = 1; q <= GHC - 1; ++q) A(F - 1 - q) = A(F - q) - value * dh;
                }
            }
            break;
        case 2:   // no_slip: odd reflection (no_slip.cpp:7-155)
        case 3: { // slip: even reflection (slip.cpp:7-155)
            const double sg = type == 2 ? -1.0 : 1.0;
            if (!face) {
                if (right) {
                    for (int q = 1; q <= GHC; ++q) A(L + q) = sg * A(L + 1 - q);
                } else {
                    for (int q = 1; q <= GHC; ++q) A(F - q) = sg * A(F - 1 + q);
                }
            } else {
                if (right) {
                    for (int q = 1; q <= GHC; ++q) A(L + q) = sg * A(L - q);
                    A(L) = 0.0;
                } else {
                    for (int q = 1; q <= GHC; ++q) A(F - q) = sg * A(F - 2 + q);
                    A(F - 1) = 0.0;
                }
            }
            break;
        }
        case 4:   // dirichlet (dirichlet.cpp:7-175)
            if (!face) {
                if (right) {
                    A(L) = A(L - 1) / 3.0 + 2.0 * value / 3.0;
                    for (int q = 1; q <= GHC; ++q) A(L + q) = 2.0 * A(L + q - 1) - A(L + q - 2);
                } else {
                    A(F) = A(F + 1) / 3.0 + 2.0 * value / 3.0;
                    for (int q = 1; q <= GHC; ++q) A(F - q) = 2.0 * A(F - q + 1) - A(F - q + 2);
                }
            } else {
                if (right) {
                    A(L) = value;
                    for (int q = 1; q <= GHC; ++q) A(L + q) = 2.0 * A(L + q - 1) - A(L + q - 2);
                } else {
                    A(F - 1) = value;
                    for (int q = 2; q <= GHC; ++q) A(F - q) = 2.0 * A(F - q + 1) - A(F - q + 2);
                }
            }
            break;
        default:
            break;
    }
#undef A
}

struct AxisFill {
    int a, fast, slow;
    bool face;
    int tl, tr;
    double vl, vr;
};

__global__ void bc_axis_kernel(double *__restrict__ f, Dims D, AxisFill P) {
    const long long nf = D.n[P.fast], ns = D.n[P.slow];
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nf * ns) return;
    int idx[3];
    idx[P.a] = 0;
    idx[P.fast] = D.ix(P.fast, int(t % nf));
    idx[P.slow] = D.ix(P.slow, int(t / nf));
    double *l = f + D.at(idx[0], idx[1], idx[2]);
    const long long sa = D.s[P.a];
    const double dh = D.d[P.a];
    fill_line(l, sa, D.n[P.a], true, P.face, P.tr, P.vr, dh);
    fill_line(l, sa, D.n[P.a], false, P.face, P.tl, P.vl, dh);
}

// The same fill for up to three independent fields in one launch per axis: thread t fills
// line t % lines of field t / lines (the fields are different arrays, so their lines never
// touch one another; the axes still go x, y, z, one launch each).
struct AxisFillMany {
    double *f[3];
    AxisFill P[3];
};

__global__ void bc_axis_many_kernel(AxisFillMany M, int nf, Dims D, int a, int fast, int slow) {
    const long long nfa = D.n[fast], ns = D.n[slow], lines = nfa * ns;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= lines * nf) return;
    const int fi = int(t / lines);
    const long long u = t - fi * lines;
    const AxisFill &P = M.P[fi];
    int idx[3];
    idx[a] = 0;
    idx[fast] = D.ix(fast, int(u % nfa));
    idx[slow] = D.ix(slow, int(u / nfa));
    double *l = M.f[fi] + D.at(idx[0], idx[1], idx[2]);
    const long long sa = D.s[a];
    const double dh = D.d[a];
    fill_line(l, sa, D.n[a], true, P.face, P.tr, P.vr, dh);
    fill_line(l, sa, D.n[a], false, P.face, P.tl, P.vl, dh);
}

// Clamp of an array index to the extrapolation source along one axis (flux.cpp:98-330,
// simple_bc.cpp:7-43): ghosts copy the boundary cell; on a staggered axis the left ghosts
// copy the wall face at index GHC-1.
__device__ __forceinline__ int clamp_src(int i, int N, bool active, bool face) {
    if (!active) return i;
    const int L = N - 1 - GHC;
    if (i > L) return L;
    const int F = face ? GHC - 1 : GHC;
    return i < F ? F : i;
}

__global__ void extrapolate_kernel(const double *__restrict__ data, double *__restrict__ flux, Dims D, int location) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= D.size()) return;
    int i, j, k;
    split3_full(q, D, i, j, k);
    const int si = clamp_src(i, D.N[0], D.ndim > 0, location == 1);
    const int sj = clamp_src(j, D.N[1], D.ndim > 1, location == 2);
    const int sk = clamp_src(k, D.N[2], D.ndim > 2, location == 3);
    flux[q] = data[D.at(si, sj, sk)];
}

// In place: every ghost reads a cell that is never written (an interior cell).
__global__ void zero_order_kernel(double *__restrict__ f, Dims D) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= D.size()) return;
    int i, j, k;
    split3_full(q, D, i, j, k);
    const int si = clamp_src(i, D.N[0], D.ndim > 0, false);
    const int sj = clamp_src(j, D.N[1], D.ndim > 1, false);
    const int sk = clamp_src(k, D.N[2], D.ndim > 2, false);
    if (si != i || sj != j || sk != k) f[q] = f[D.at(si, sj, sk)];
}

}  // namespace

void launch_bc_fill(const Dims &D, int location, const int *types, const double *values, double *f, cudaStream_t s) {
    for (int a = 0; a < D.ndim; ++a) {
        AxisFill P;
        P.a = a;
        const int b = (a + 1) % 3, c = (a + 2) % 3;
        P.fast = b > c ? b : c;
        P.slow = b > c ? c : b;
        P.face = location == a + 1;
        P.tl = types[2 * a];
        P.tr = types[2 * a + 1];
        P.vl = values[2 * a];
        P.vr = values[2 * a + 1];
        const long long lines = (long long)D.n[b] * D.n[c];
        bc_axis_kernel<<<blocks_for(lines, 128), 128, 0, s>>>(f, D, P);
    }
}

void launch_bc_fill_many(const Dims &D, int nf, const int *locations, const int *const *types, const double *values,
                         double *const *f, cudaStream_t s) {
    for (int a = 0; a < D.ndim; ++a) {
        AxisFillMany M{};
        const int b = (a + 1) % 3, c = (a + 2) % 3;
        for (int q = 0; q < nf; ++q) {
            AxisFill &P = M.P[q];
            P.a = a;
            P.fast = b > c ? b : c;
            P.slow = b > c ? c : b;
            P.face = locations[q] == a + 1;
            P.tl = types[q][2 * a];
            P.tr = types[q][2 * a + 1];
            P.vl = values[2 * a];
            P.vr = values[2 * a + 1];
            M.f[q] = f[q];
        }
        const long long lines = (long long)D.n[b] * D.n[c];
        bc_axis_many_kernel<<<blocks_for(lines * nf, 128), 128, 0, s>>>(M, nf, D, a, b > c ? b : c, b > c ? c : b);
    }
}

void launch_extrapolate(const Dims &D, int location, const double *data, double *flux, cudaStream_t s) {
    extrapolate_kernel<<<blocks_for(D.size(), 256), 256, 0, s>>>(data, flux, D, location);
}

void launch_zero_order(const Dims &D, double *f, cudaStream_t s) {
    zero_order_kernel<<<blocks_for(D.size(), 256), 256, 0, s>>>(f, D);
}

}  // namespace scihpc
