// twophase.cuh -- one two-phase problem resident on the GPU.
#pragma once

#include <string>
#include <vector>

#include "common.cuh"
#include "compact.cuh"
#include "poisson.cuh"

namespace scihpc {

// The arrays of one scalar_data that the step uses (scalar_data.h:14-17).
struct DevScalar {
    double *data = nullptr, *flux = nullptr, *old = nullptr, *old2 = nullptr;
    double *d1[3] = {nullptr, nullptr, nullptr};   // fx, fy, fz
    double *d2[3] = {nullptr, nullptr, nullptr};   // fxx, fyy, fzz
    double *mixed[3] = {nullptr, nullptr, nullptr};   // fxy, fyz, fzx
};

// Neumann ghost fill fused into the kernels that write a scalar's interior (twophase.cu).
struct GhostFill {
    int on;
    double v[6];   // bc values xl, xr, yl, yr, zl, zr
};

struct HostParams {
    double density_ratio, viscosity_ratio, Re, Fr, We, ls_width, rdt, max_CFL, min_CFL;
    int positive_ref;
    double ppe_tol;
    int ppe_max_iter;
    int ppe_initer;
};

class TwoPhaseGpu {
public:
    int create(const scihpc_grid *g, const int *vel_bc, const int *scalar_bc, const double *prm, const int *opt);
    void destroy();
    double *field(const std::string &name);
    int get_scalars(double *out);
    // every field of the session and the step scalars to / from a file (restart)
    int checkpoint(const char *path);
    int restore(const char *path);
    int set_scalars(const double *in);

    // stages (asynchronous on `stream`)
    void find_dt();
    void advect();
    void mpls(int count);
    int reinit();            // returns RK3 steps
    void find_sign();        // find_sign (wrapper_func.cpp:387-402) into the sign field
    void reinit_step(int lambda);   // one TVD-RK3 step of the redistance equation
    void set_scheme(int s);  // convection: 0 UCCD (source.cpp:8-40), 1 WENO5
    // find_source's derivatives: 0 the compact schemes (projection_method.cpp:244-312),
    // 1 second_order_solver (find_source_sec, projection_method.cpp:314-382)
    void set_source_scheme(int s);
    void find_source();
    // pressure schedule: 0 the projection equation solved every step (default); 1 the
    // reference's ab_solve schedule (projection_method.cpp:755-777): the projection equation
    // while iter < 5, then pressure_guess_solution, init_ppe_fpc_coefficients and
    // fast_pressure_correction, each repeated ppe_initer times.  tol_mode 0: ppe_tol is the
    // relative residual; 1: the absolute residual 2-norm, as the reference's loops test it.
    int set_ppe_schedule(int schedule, int tol_mode);
    bool fpc_step() const { return ppe_schedule == 1 && iter_host >= 5.0; }
    void ab_solve_pre(bool fpc);    // store, find_source, AB2, PPE right-hand side, solver begin
    void ab_solve_post(bool fpc);   // solver finish, pressure BC, velocity correction, node velocity
    int ab_solve(int *iters, double *relres);   // host-driven pressure iteration
    // the stages of ab_solve one at a time (projection_method.cpp:384-402, 544-657; the
    // node velocity of wrapper_func.cpp:177-293)
    int intermediate_velocity();
    int projection(int *iters, double *relres);
    int node_from_face();
    // the stages of the fast pressure correction (projection_method.cpp:467-541, 659-753,
    // 803-815): pressure_guess_solution into the pressure's flux array, the right-hand side
    // term of init_ppe_fpc_coefficients from it, and the correction itself
    int pressure_guess();
    int fpc_coefficients();
    int fast_pressure_correction(int *iters, double *relres);
    void ab2_part();
    void projection_begin();
    void projection_end();
    void fpc_begin();
    void fpc_end();
    void node_part();
    int run_ppe(Poisson &ps, int *iters, double *relres);
    int init();
    int step(int nsteps, bool graph);
    int diagnostics(double *out);
    int graph_stats(long long *out);   // kernel nodes {pre, body, post}, PPE iterations summed over steps
    int time_reinit_gradient(int n, float *ms);   // ms per launch of the reinit gradient kernel

    cudaStream_t stream = nullptr;
    Dims D{};
    double last_iters = 0, last_relres = 0, last_ms = 0;
    double iter_host = 0.0;   // host copy of StepScalars::iter (selects the pressure stage)

private:
    void scalar_bc(double *f);
    void vel_bc(DevScalar *v, int location_for_all);
    void rk_stage_update(int stage);
    void convection_rhs(double *s);
    void reinit_stage(int stage);
    int capture_step(int fpc);
    void drop_graphs();
    int ensure_fpc();
    void set_solver_tol(Poisson &ps, int cap);

    // independent work of one stage runs as parallel branches on side streams (fork/join by
    // events; the branches become parallel nodes when the step is captured as a graph)
    void fork(int n);
    void join(int n);
    void sub_fork(int g, int n, cudaStream_t s);
    void sub_join(int g, int k, cudaStream_t s);
    // Programmatic dependent launches (in 2D, as for the multigrid) for the two chains of
    // small kernels that run back to back on the main stream: the reinitialisation stages and
    // the mass correction (451 -> 475 steps/s on the bubble step).  Measured on the same box:
    // giving the kernel before such a chain an early trigger as well (k_sign before the
    // reinitialisation) took the step to 366 steps/s, so only these kernels carry one.
    bool pdl_step() const { return D.ndim == 2 && pdl_enabled(); }
    cudaStream_t side[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t ev_fork = nullptr, ev_join[3] = {nullptr, nullptr, nullptr};
    // the pressure operator's density setup (Poisson::set_density: coefficients of every level
    // and the coarsest level's inverse) runs on its own stream from the density's computation
    // in find_source to the start of the pressure solve, beside the source terms' line solves;
    // dens_async asks find_source for it, dens_pending says that projection_begin must join it
    cudaStream_t dens_stream = nullptr;
    cudaEvent_t ev_dens = nullptr;
    bool dens_async = false, dens_pending = false;
    // per-direction face-averaged velocities of find_source for the directions other than the
    // last (that one uses nvel, as before), their extrapolation scratch and line-solve scratch
    double *fv[3][3] = {}, *fv_flux[3] = {}, *tb1[3] = {}, *tb2[3] = {};
    // Inside find_source's branches the line solves that do not depend on one another run as
    // parallel branches of their own (sub[a][k], a = velocity direction, 3 = the level set);
    // each concurrent UCCD solve has its own scratch (used only by the long-line fallback).
    // Measured: bubble step 553 -> 559 steps/s; 3D dam break 182.9 -> 187.7 steps/s with FP32
    // V-cycles, 150.7 -> 148.1 with FP64 ones.
    bool split_source() const { return source_scheme != 1; }
    cudaStream_t sub[4][2] = {};
    cudaEvent_t ev_sub[4] = {}, ev_subj[4][2] = {};
    double *tbs1[3][2] = {}, *tbs2[3][2] = {}, *mtmp[2] = {};

    HostParams P{};
    int scheme = 1, n_mpls = 5, reinit_every = 1, fp32 = 0, reinit_lambda = 1;
    int source_scheme = 0;
    int step_count = 0;
    int vel_types[3][6];
    int scalar_types[6];
    CompactOps ops;
    Poisson ppe;
    Poisson fpc;               // constant-coefficient solver of the fast pressure correction
    bool fpc_ready = false;
    int ppe_schedule = 0, ppe_tol_mode = 0;
    double *RHS_fpc = nullptr;   // init_ppe_fpc_coefficients' RHS array
    DevScalar phi, pres, vel[3], nvel[3];
    double *H = nullptr, *delta = nullptr, *sign = nullptr, *grad = nullptr, *curv = nullptr, *a_f = nullptr,
           *b_f = nullptr, *rho = nullptr, *mu = nullptr;
    double *src[3] = {nullptr, nullptr, nullptr}, *src_old[3] = {nullptr, nullptr, nullptr};
    double *RHS = nullptr, *s1 = nullptr, *s2 = nullptr, *s3 = nullptr, *t1 = nullptr, *t2 = nullptr, *work = nullptr;
    double *partial = nullptr;
    unsigned *mpls_counter = nullptr;   // blocks of k_mpls_sums done (the last one resets it)
    StepScalars *sc = nullptr;        // device
    StepScalars *sc_host = nullptr;   // pinned
    std::vector<void *> allocs;
    size_t nfield_allocs = 0;   // allocs[0 .. nfield_allocs) are whole ghosted fields
    cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};   // step graphs: projection, fast correction
    cudaGraph_t graph[2] = {nullptr, nullptr};
    int reinit_steps = 0;
    GhostFill phi_fill{};
    long long nodes_pre = 0, nodes_body = 0, nodes_post = 0;
};

}  // namespace scihpc
