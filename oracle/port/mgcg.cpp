// mgcg.cpp -- TEST INFRASTRUCTURE (CPU restatement, see port.h).
//
// Preconditioner of the exact pressure solve (coef_cg_solve) on large grids, where the
// Jacobi-preconditioned CG needs thousands of iterations at density ratio 1000.  It only has
// to be a fixed symmetric positive-definite approximation of the operator's inverse: the
// answer is the CG's, checked against the operator itself (the residual is computed from the
// seven coefficient arrays, not from anything here).
//
// One V(1,1) cycle: symmetric Gauss-Seidel (a forward lexicographic sweep before the coarse
// correction, a backward one after), coarsening by 2 x 2 (x 2) aggregation with the
// Galerkin coarse operator of piecewise-constant prolongation -- for a face-coefficient
// operator again a face-coefficient operator whose coarse face carries the sum of the fine
// faces crossing it -- and a dense Cholesky solve on the coarsest level (its constant null
// space pinned by a rank-one term; the coarse right-hand sides sum to zero).
#include <cmath>
#include <vector>

#include "mg.h"

namespace port {

namespace {

struct PLevel {
    int ndim = 2;
    int n[3] = {1, 1, 1};
    std::vector<double> cf[3];   // coefficient of the +a face of each cell (0 on the wall)
    std::vector<double> diag, x, b, r;
    std::vector<double> chol;    // coarsest level: Cholesky factor of the pinned operator
    size_t size() const { return size_t(n[0]) * n[1] * n[2]; }
    size_t stride(int a) const { return a == 0 ? size_t(n[1]) * n[2] : a == 1 ? size_t(n[2]) : 1; }
    int coord(size_t q, int a) const {
        if (a == 2) return int(q % n[2]);
        if (a == 1) return int((q / n[2]) % n[1]);
        return int(q / (size_t(n[1]) * n[2]));
    }
};

// y = M x, M = -A: (M x)_q = diag_q x_q - sum over faces C (x_nb)
void apply(const PLevel &L, const std::vector<double> &x, std::vector<double> &y) {
    const size_t N = L.size();
    for (size_t q = 0; q < N; ++q) y[q] = L.diag[q] * x[q];
    for (int a = 0; a < L.ndim; ++a) {
        const size_t s = L.stride(a);
        for (size_t q = 0; q < N; ++q) {
            const double c = L.cf[a][q];
            if (c == 0.0) continue;
            y[q] -= c * x[q + s];
            y[q + s] -= c * x[q];
        }
    }
}

// one Gauss-Seidel sweep in lexicographic order (forward) or its reverse
void sweep(PLevel &L, bool forward) {
    const size_t N = L.size();
    for (size_t t = 0; t < N; ++t) {
        const size_t q = forward ? t : N - 1 - t;
        if (L.diag[q] == 0.0) continue;
        double s = L.b[q];
        for (int a = 0; a < L.ndim; ++a) {
            const size_t st = L.stride(a);
            const int c = L.coord(q, a);
            if (c < L.n[a] - 1) s += L.cf[a][q] * L.x[q + st];
            if (c > 0) s += L.cf[a][q - st] * L.x[q - st];
        }
        L.x[q] = s / L.diag[q];
    }
}

void factor_coarsest(PLevel &L) {
    const int N = int(L.size());
    std::vector<double> M(size_t(N) * N, 0.0);
    double dsum = 0.0;
    for (int q = 0; q < N; ++q) {
        M[size_t(q) * N + q] = L.diag[q];
        dsum += L.diag[q];
        for (int a = 0; a < L.ndim; ++a) {
            if (L.coord(q, a) == L.n[a] - 1) continue;
            const int nb = q + int(L.stride(a));
            M[size_t(q) * N + nb] -= L.cf[a][q];
            M[size_t(nb) * N + q] -= L.cf[a][q];
        }
    }
    const double pin = dsum / N / N;
    for (auto &e : M) e += pin;
    for (int j = 0; j < N; ++j) {
        double d = M[size_t(j) * N + j];
        for (int k = 0; k < j; ++k) d -= M[size_t(j) * N + k] * M[size_t(j) * N + k];
        d = std::sqrt(d);
        M[size_t(j) * N + j] = d;
        for (int i = j + 1; i < N; ++i) {
            double s = M[size_t(i) * N + j];
            for (int k = 0; k < j; ++k) s -= M[size_t(i) * N + k] * M[size_t(j) * N + k];
            M[size_t(i) * N + j] = s / d;
        }
    }
    L.chol = std::move(M);
}

void solve_coarsest(PLevel &L) {
    const int N = int(L.size());
    const double *C = L.chol.data();
    std::vector<double> y(N);
    for (int i = 0; i < N; ++i) {
        double s = L.b[i];
        for (int k = 0; k < i; ++k) s -= C[size_t(i) * N + k] * y[k];
        y[i] = s / C[size_t(i) * N + i];
    }
    for (int i = N - 1; i >= 0; --i) {
        double s = y[i];
        for (int k = i + 1; k < N; ++k) s -= C[size_t(k) * N + i] * L.x[k];
        L.x[i] = s / C[size_t(i) * N + i];
    }
}

bool coarsenable(const PLevel &L) {
    if (L.size() <= 512) return false;
    for (int a = 0; a < L.ndim; ++a)
        if (L.n[a] % 2 != 0 || L.n[a] < 4) return false;
    return true;
}

PLevel coarsen(const PLevel &F) {
    PLevel C;
    C.ndim = F.ndim;
    for (int a = 0; a < 3; ++a) C.n[a] = a < F.ndim ? F.n[a] / 2 : 1;
    const size_t N = C.size();
    for (int a = 0; a < 3; ++a) C.cf[a].assign(N, 0.0);
    C.diag.assign(N, 0.0);
    for (size_t q = 0; q < F.size(); ++q) {
        int c[3] = {F.coord(q, 0), F.coord(q, 1), F.coord(q, 2)};
        size_t Q = 0;
        for (int a = 0; a < 3; ++a) Q = Q * C.n[a] + size_t(a < F.ndim ? c[a] / 2 : 0);
        for (int a = 0; a < F.ndim; ++a) {
            // a fine +a face leaving the 2-cell block crosses the coarse +a face
            if (c[a] % 2 == 1 && c[a] < F.n[a] - 1) C.cf[a][Q] += F.cf[a][q];
        }
    }
    for (size_t Q = 0; Q < N; ++Q)
        for (int a = 0; a < C.ndim; ++a) {
            C.diag[Q] += C.cf[a][Q];
            if (C.coord(Q, a) > 0) C.diag[Q] += C.cf[a][Q - C.stride(a)];
        }
    return C;
}

void vcycle(std::vector<PLevel> &Ls, size_t l) {
    PLevel &L = Ls[l];
    std::fill(L.x.begin(), L.x.end(), 0.0);
    if (l + 1 == Ls.size()) {
        solve_coarsest(L);
        return;
    }
    sweep(L, true);
    apply(L, L.x, L.r);
    for (size_t q = 0; q < L.size(); ++q) L.r[q] = L.b[q] - L.r[q];
    PLevel &C = Ls[l + 1];
    std::fill(C.b.begin(), C.b.end(), 0.0);
    auto block = [&](size_t q) {
        size_t Q = 0;
        for (int a = 0; a < 3; ++a) Q = Q * C.n[a] + size_t(a < L.ndim ? L.coord(q, a) / 2 : 0);
        return Q;
    };
    for (size_t q = 0; q < L.size(); ++q) C.b[block(q)] += L.r[q];
    vcycle(Ls, l + 1);
    for (size_t q = 0; q < L.size(); ++q) L.x[q] += C.x[block(q)];
    sweep(L, false);
}

}  // namespace

// z = V-cycle(r) for the face operator given by the +x, +y, +z coefficient arrays of the
// interior cells (compact, K fastest); built once per call of coef_cg_solve
struct MGPrecond::Impl {
    std::vector<PLevel> Ls;
};

MGPrecond::MGPrecond(int ndim, const int *n, const std::vector<double> *cf) : impl(new Impl) {
    PLevel L0;
    L0.ndim = ndim;
    for (int a = 0; a < 3; ++a) L0.n[a] = a < ndim ? n[a] : 1;
    for (int a = 0; a < 3; ++a) L0.cf[a] = a < ndim ? cf[a] : std::vector<double>(L0.size(), 0.0);
    L0.diag.assign(L0.size(), 0.0);
    for (size_t q = 0; q < L0.size(); ++q)
        for (int a = 0; a < ndim; ++a) {
            L0.diag[q] += L0.cf[a][q];
            if (L0.coord(q, a) > 0) L0.diag[q] += L0.cf[a][q - L0.stride(a)];
        }
    impl->Ls.push_back(std::move(L0));
    while (coarsenable(impl->Ls.back())) impl->Ls.push_back(coarsen(impl->Ls.back()));
    for (auto &L : impl->Ls) {
        L.x.assign(L.size(), 0.0);
        L.b.assign(L.size(), 0.0);
        L.r.assign(L.size(), 0.0);
    }
    factor_coarsest(impl->Ls.back());
}

MGPrecond::~MGPrecond() { delete impl; }

void MGPrecond::apply(const std::vector<double> &r, std::vector<double> &z) {
    PLevel &L0 = impl->Ls[0];
    L0.b = r;
    vcycle(impl->Ls, 0);
    z = L0.x;
}

}  // namespace port
