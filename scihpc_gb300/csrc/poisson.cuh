// poisson.cuh -- multigrid-preconditioned solver of the pressure equation.
#pragma once

#include <type_traits>
#include <vector>

#include <cuda.h>

#include "common.cuh"

namespace scihpc {

// One multigrid level in a padded layout with a one-cell halo that is kept at zero:
// (nx+2) x (ny+2) [x (nz+2)], k fastest.  `coef` holds, for levels >= 1, the face
// coefficients C = k / d^2 of the +x, +y, +z faces of every padded cell (three arrays).
template <class T>
struct Level {
    int n[3] = {1, 1, 1};   // interior cells
    int P[3] = {1, 1, 1};   // padded extents
    long long s[3] = {0, 0, 0};
    long long cells = 0;    // padded size
    int ratio = 2;          // coarsening factor to the next level
    double d[3] = {0, 0, 0};
    T *x = nullptr, *b = nullptr;
    T *x2 = nullptr;   // second iterate buffer for out-of-place fused sweeps (same allocation as x)
    T *cx = nullptr, *cy = nullptr, *cz = nullptr;
    T *idg = nullptr;   // 1 / sum of the face coefficients (levels with stored coefficients)
    // divisions by n[1], n[2] and by the cells of one colour along the last axis,
    // (n[ndim - 1] + 1) / 2, used to decode cell indices
    FastDiv f1, f2, fh;
};

struct PcgScalars {
    double bb;        // ||g||^2 of the projected right-hand side
    double rr;        // ||r||^2
    double rz, rz_prev, r_zold;
    double dq;
    double relres;
    double mean;
    double best;      // smallest relative residual seen
    double rr_in, rr_in0;   // FP32 inner solve: ||r||^2 now and at its start
    double in_tol, in_target;   // inner relative tolerance: floor and current target
    double rr_in_min;           // smallest inner ||r||^2 of the current inner solve
    int it, done, diverged, since_best;
    int in_it, pending;     // inner iterations since the last refinement; refinement due
    int in_break;           // the inner recurrence broke down (FP32 round-off)
    int restart;            // FP64 CG: the residual was replaced, next direction restarts
    int sweep_err;          // a staged sweep timed out waiting for its planes
    double abs_tol;         // absolute residual target (0: none)
    double tol;             // relative target in force: max(rel_tol, abs_tol / ||g||), set at begin
};

class Poisson {
public:
    // bc: 0 Neumann walls, 1 Dirichlet walls with zero ghost-centre value.
    // density: 1 coefficients from a density field, 0 constant 1/d^2.
    // fp32: V-cycles in single precision.
    int create(const scihpc_grid *g, int bc, int density, int fp32);
    void destroy();
    int set_density(const double *rho, cudaStream_t s);
    // Device-side pieces of one solve (no host synchronisation; usable in graph capture).
    void begin(const double *rhs, double *p, int use_guess, cudaStream_t s);
    void iterate(cudaStream_t s);   // one outer iteration incl. convergence test
    void finish(double *p, cudaStream_t s);
    // Whole solve.  When the same inputs come back (repeated solves of a time loop or a
    // benchmark) it runs as one CUDA graph: begin, a conditional while-node over iterate,
    // finish, captured once and replayed, with one host synchronisation at the end.  A solve
    // with new inputs, SCIHPC_PPE_GRAPH=0 or SCIHPC_PPE_TRACE runs the host loop instead
    // (synchronising once per iteration).
    int solve(const double *rhs, double *p, int use_guess, double rel_tol, int max_iter, int *iters, double *relres,
              cudaStream_t s);
    int levels(int *out, int max_levels) const;
    // ||rhs - A p|| over the interior (rhs minus its mean for Neumann walls), FP64, synchronising.
    int residual(const double *rhs, const double *p, double *norm, cudaStream_t s);
    // Times n V-cycles (the preconditioner alone) on the residual of p = 0 for rhs.
    int time_vcycles(const double *rhs, double *p, int n, float *ms, cudaStream_t s);
    int fp32() const { return fp32_; }

    double rel_tol = 1e-10;
    // absolute target: the solve also stops once ||g - L p|| <= abs_tol (2-norm over the
    // interior; 0 = relative target only).  The reference's multigrid loops stop on this
    // absolute residual (projection_method.cpp:695-697).
    double abs_tol = 0.0;
    int max_iter = 200;
    PcgScalars *dev_state = nullptr;    // device
    PcgScalars *host_state = nullptr;   // pinned mirror
    unsigned long long *cond_handle = nullptr;   // graph conditional handle slot (device), 0 when unused
    bool use_conditional = false;
    int prolong_linear = 0;   // 0: piecewise-constant prolongation (default), 1: (bi/tri)linear
    // FP32 mode: each inner solve stops at this relative residual or after inner_max iterations
    double inner_tol = 1e-4;
    int inner_max = 12;
    unsigned long long conditional = 0;

private:
    template <class T>
    std::vector<Level<T>> &levs() {
        if constexpr (std::is_same_v<T, float>) return Lf;
        else return Ld;
    }
    template <class T>
    bool vcycle(cudaStream_t s, double *dot = nullptr);
    template <class T>
    int alloc_levels();
    template <class T>
    void build_coarse(cudaStream_t s);
    bool make_level0_maps(const std::vector<Level<float>> &Ls);
    template <int DIM>
    void begin_dim(const double *rhs, double *p, int use_guess, cudaStream_t s);
    template <int DIM>
    void iterate_dim(cudaStream_t s);
    template <int DIM>
    void finish_dim(double *p, cudaStream_t s);
    int capture_solve(const double *rhs, double *p, int use_guess);
    bool use_pdl(cudaStream_t s) const;
    void drop_solve_graph();

    // the captured solve and what it was captured for (set_density rewrites the coefficient
    // arrays in place, so a new density needs no new capture)
    struct SolveKey {
        const double *rhs = nullptr;
        double *p = nullptr;
        int use_guess = 0, max_iter = 0, inner_max = 0, prolong_linear = 0;
        double rel_tol = 0.0, inner_tol = 0.0, abs_tol = 0.0;
        bool operator==(const SolveKey &o) const {
            return rhs == o.rhs && p == o.p && use_guess == o.use_guess && max_iter == o.max_iter &&
                   inner_max == o.inner_max && prolong_linear == o.prolong_linear && rel_tol == o.rel_tol &&
                   inner_tol == o.inner_tol && abs_tol == o.abs_tol;
        }
    };
    cudaGraphExec_t solve_exec = nullptr;
    SolveKey solve_key{};
    SolveKey last_key{};   // inputs of the previous solve call
    cudaStream_t cap_stream = nullptr;   // private stream the solve is captured on

    Dims D{};
    int bc_ = 0, density_ = 1, fp32_ = 0;
    int nlev = 0;
    std::vector<Level<float>> Lf;
    std::vector<Level<double>> Ld;
    // FP64 outer iteration vectors (interior, compact, K fastest)
    double *r = nullptr, *dvec = nullptr, *q = nullptr;
    void *zold = nullptr;       // previous preconditioned residual, level-0 padded, T
    float *d32 = nullptr, *q32 = nullptr, *e32 = nullptr;   // FP32 inner solve vectors, level-0 padded
    void *rho_pad = nullptr;    // level-0 density, padded, T, +inf halo
    const double *rho64 = nullptr;   // caller's ghosted density (FP64 operator)
    double *partial = nullptr;       // reduction scratch (2 x RED_MAX_BLOCKS)
    double *oc = nullptr;            // FP64 +face coefficients of the outer operator (3 compact arrays)
    double *dense = nullptr;         // coarsest-level inverse (n x n, FP64)
    // TMA descriptors of the FP32 level 0 (3D): x, x2, padded density, b; level 1's x; the
    // inner conjugate-gradient direction
    CUtensorMap tmap[6];
    bool tma_ready = false, tma_pro_ready = false;
    int tma_enable = 1;
    int ncoarse = 0;
    const double *rhs_ = nullptr;
    double *p_ = nullptr;
};

}  // namespace scihpc
