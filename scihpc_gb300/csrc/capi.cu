// capi.cu -- the extern "C" entry points declared in include/scihpc_gpu.h.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>

#include "common.cuh"
#include "compact.cuh"
#include "levelset.cuh"
#include "poisson.cuh"
#include "reduce.cuh"
#include "secorder.cuh"
#include "transport.cuh"
#include "twophase.cuh"
#include "conv.cuh"
#include "unet.cuh"

namespace scihpc {

static thread_local std::string g_last_error;

void set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    g_last_error = buf;
    return e == cudaErrorMemoryAllocation ? SCIHPC_ERR_NOMEM : SCIHPC_ERR_CUDA;
}

// Programmatic dependent launch for the multigrid kernels (on unless SCIHPC_PDL=0).
bool pdl_enabled() {
    static const bool on = [] {
        const char *e = std::getenv("SCIHPC_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

// structured_grid.cpp:7-134 -- d = (end - start) / n, h = min d, dv = prod d.
Dims make_dims(const scihpc_grid *g) {
    Dims D{};
    D.ndim = g->ndim;
    for (int a = 0; a < 3; ++a) {
        const bool act = a < g->ndim;
        D.n[a] = act ? g->n[a] : 1;
        D.N[a] = act ? g->n[a] + 2 * GHC : 1;
        D.d[a] = act ? (g->hi[a] - g->lo[a]) / static_cast<double>(g->n[a]) : 0.0;
        D.rd[a] = act ? 1.0 / D.d[a] : 0.0;
        D.lo[a] = act ? g->lo[a] : 0.0;
    }
    D.s[2] = 1;
    D.s[1] = D.N[2];
    D.s[0] = (long long)D.N[1] * D.N[2];
    if (D.ndim == 1) {
        D.h = D.d[0];
        D.dv = D.d[0];
    } else if (D.ndim == 2) {
        D.h = D.d[0] < D.d[1] ? D.d[0] : D.d[1];
        D.dv = D.d[0] * D.d[1];
    } else {
        D.h = D.d[0] < D.d[1] ? D.d[0] : D.d[1];
        D.h = D.h < D.d[2] ? D.h : D.d[2];
        D.dv = D.d[0] * D.d[1] * D.d[2];
    }
    return D;
}

static int check_grid(const scihpc_grid *g) {
    if (!g || g->ndim < 1 || g->ndim > 3) {
        set_last_error("grid: ndim must be 1, 2 or 3");
        return SCIHPC_ERR_ARG;
    }
    for (int a = 0; a < g->ndim; ++a) {
        if (g->n[a] < 3 || !(g->hi[a] > g->lo[a])) {
            set_last_error("grid: every active axis needs n >= 3 and hi > lo");
            return SCIHPC_ERR_ARG;
        }
    }
    return SCIHPC_OK;
}

}  // namespace scihpc

using namespace scihpc;

struct scihpc_ctx {
    Dims D;
    CompactOps ops;
    double *t1 = nullptr, *t2 = nullptr, *work = nullptr, *partial = nullptr, *red = nullptr;
};

struct scihpc_poisson {
    Poisson ps;
};

struct scihpc_twophase {
    TwoPhaseGpu tp;
};

static inline cudaStream_t S(void *s) { return static_cast<cudaStream_t>(s); }

#define CHECK_LAUNCH()                                             \
    do {                                                           \
        cudaError_t e_ = cudaGetLastError();                       \
        if (e_ != cudaSuccess) return cuda_fail(e_, "kernel launch", __FILE__, __LINE__); \
    } while (0)

#define REQUIRE(cond, msg)           \
    do {                             \
        if (!(cond)) {               \
            set_last_error(msg);     \
            return SCIHPC_ERR_ARG;   \
        }                            \
    } while (0)

extern "C" {

const char *scihpc_last_error(void) { return g_last_error.c_str(); }

const char *scihpc_version(void) { return "scihpc_gb300 0.1 (sm_103a)"; }

int scihpc_ctx_create(const scihpc_grid *grid, scihpc_ctx **out) {
    REQUIRE(out, "ctx_create: out is NULL");
    int rc = check_grid(grid);
    if (rc) return rc;
    auto *c = new (std::nothrow) scihpc_ctx;
    if (!c) return SCIHPC_ERR_NOMEM;
    c->D = make_dims(grid);
    rc = c->ops.build(c->D);
    if (rc) {
        delete c;
        return rc;
    }
    const size_t bytes = size_t(c->D.size()) * sizeof(double);
    SCIHPC_CUDA(cudaMalloc(&c->t1, 3 * bytes));
    c->t2 = c->t1 + c->D.size();
    c->work = c->t2 + c->D.size();
    SCIHPC_CUDA(cudaMalloc(&c->partial, (RED_MAX_BLOCKS + 8) * sizeof(double)));
    c->red = c->partial + RED_MAX_BLOCKS;
    *out = c;
    return SCIHPC_OK;
}

int scihpc_ctx_destroy(scihpc_ctx *ctx) {
    if (!ctx) return SCIHPC_OK;
    ctx->ops.release();
    cudaFree(ctx->t1);
    cudaFree(ctx->partial);
    delete ctx;
    return SCIHPC_OK;
}

int scihpc_bc_fill(scihpc_ctx *ctx, int location, const int types[6], const double values[6], double *f,
                   void *stream) {
    REQUIRE(ctx && f && types && values, "bc_fill: NULL argument");
    REQUIRE(location >= 0 && location <= ctx->D.ndim, "bc_fill: location out of range");
    for (int a = 0; a < ctx->D.ndim; ++a) {
        REQUIRE(types[2 * a] >= 0 && types[2 * a] <= 4 && types[2 * a + 1] >= 0 && types[2 * a + 1] <= 4,
                "bc_fill: boundary type out of range");
        // bc_factory::check_bc (bc_factory.cpp:8-21): periodic on both faces or neither
        REQUIRE((types[2 * a] == 0) == (types[2 * a + 1] == 0), "bc_fill: periodic must be set on both faces");
    }
    launch_bc_fill(ctx->D, location, types, values, f, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_flux_extrapolate(scihpc_ctx *ctx, int location, const double *data, double *flux, void *stream) {
    REQUIRE(ctx && data && flux, "flux_extrapolate: NULL argument");
    REQUIRE(location >= 0 && location <= ctx->D.ndim, "flux_extrapolate: location out of range");
    launch_extrapolate(ctx->D, location, data, flux, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_zero_order_extrapolation(scihpc_ctx *ctx, double *f, void *stream) {
    REQUIRE(ctx && f, "zero_order_extrapolation: NULL argument");
    launch_zero_order(ctx->D, f, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_uccd(scihpc_ctx *ctx, int axis, const double *flux, const double *vel_axis, double *f1, double *f2,
                void *stream) {
    REQUIRE(ctx && flux && vel_axis && f1 && f2, "uccd: NULL argument");
    REQUIRE(axis >= 0 && axis < ctx->D.ndim, "uccd: axis out of range");
    launch_uccd(ctx->D, ctx->ops, axis, flux, vel_axis, f1, f2, ctx->t1, ctx->t2, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_flux_fill(scihpc_ctx *ctx, int kind, const double *phi, double *flux, void *stream) {
    REQUIRE(ctx && phi && flux, "flux_fill: NULL argument");
    REQUIRE(kind == 0 || kind == 1, "flux_fill: kind must be 0 (identity) or 1 (Burgers)");
    launch_flux_fill(ctx->D, kind, phi, flux, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_rk3_stage(scihpc_ctx *ctx, int stage, int rhs_kind, double dt, double *phi, const double *const d[3],
                     const double *const vel[3], double *s1, double *s2, void *stream) {
    REQUIRE(ctx && phi && d, "rk3_stage: NULL argument");
    REQUIRE(stage >= 0 && stage <= 3, "rk3_stage: stage must be 0 (Euler) or 1..3");
    REQUIRE(rhs_kind == 0 || rhs_kind == 1, "rk3_stage: rhs_kind must be 0 (convection) or 1 (Hamilton-Jacobi)");
    for (int a = 0; a < ctx->D.ndim; ++a) {
        REQUIRE(d[a], "rk3_stage: NULL derivative");
        REQUIRE(rhs_kind == 1 || (vel && vel[a]), "rk3_stage: convection needs the velocity");
    }
    REQUIRE(stage == 0 || s1, "rk3_stage: stages 1-3 need s1");
    REQUIRE(stage <= 1 || s2, "rk3_stage: stages 2-3 need s2");
    launch_rk3_stage(ctx->D, stage, rhs_kind, dt, phi, d, rhs_kind == 0 ? vel : nullptr, s1, s2, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_sec_derivative(scihpc_ctx *ctx, int axis, const double *flux, const double *vel_axis, double *f1,
                          double *f2, void *stream) {
    REQUIRE(ctx && flux && f1 && f2, "sec_derivative: NULL argument");
    REQUIRE(axis >= 0 && axis < ctx->D.ndim, "sec_derivative: axis out of range");
    if (vel_axis) launch_sec_upwind(ctx->D, axis, flux, vel_axis, f1, f2, S(stream));
    else launch_sec_central(ctx->D, axis, flux, f1, f2, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_sec_mixed(scihpc_ctx *ctx, int axis, const double *src, double *out, void *stream) {
    REQUIRE(ctx && src && out, "sec_mixed: NULL argument");
    REQUIRE(axis >= 0 && axis < ctx->D.ndim, "sec_mixed: axis out of range");
    launch_sec_mixed(ctx->D, axis, src, out, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_ccd(scihpc_ctx *ctx, int axis, const double *flux, double *f1, double *f2, void *stream) {
    REQUIRE(ctx && flux && f1 && f2, "ccd: NULL argument");
    REQUIRE(axis >= 0 && axis < ctx->D.ndim, "ccd: axis out of range");
    launch_ccd(ctx->D, ctx->ops, axis, flux, f1, f2, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_ccd_mixed(scihpc_ctx *ctx, int axis, double *src, double *out, void *stream) {
    REQUIRE(ctx && src && out, "ccd_mixed: NULL argument");
    REQUIRE(axis >= 0 && axis < ctx->D.ndim, "ccd_mixed: axis out of range");
    launch_ccd_mixed(ctx->D, ctx->ops, axis, src, out, ctx->work, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_weno5(scihpc_ctx *ctx, int axis, const double *flux, const double *vel_axis, double *fa, void *stream) {
    REQUIRE(ctx && flux && vel_axis && fa, "weno5: NULL argument");
    REQUIRE(axis >= 0 && axis < ctx->D.ndim, "weno5: axis out of range");
    launch_weno5(ctx->D, axis, flux, vel_axis, fa, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_godunov_gradient(scihpc_ctx *ctx, const double *phi, const double *sign, double *grad, void *stream) {
    REQUIRE(ctx && phi && sign && grad, "godunov_gradient: NULL argument");
    launch_godunov(ctx->D, phi, sign, grad, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_stabilized_upon_gradient(scihpc_ctx *ctx, double *phi, const double *sign, double *grad, void *stream) {
    REQUIRE(ctx && phi && sign && grad, "stabilized_upon_gradient: NULL argument");
    launch_stabilize(ctx->D, phi, sign, grad, ctx->partial, ctx->red + 2, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_guess_from_history(scihpc_ctx *ctx, const double *old, const double *old2, double *flux, void *stream) {
    REQUIRE(ctx && old && old2 && flux, "guess_from_history: NULL argument");
    launch_guess_from_history(ctx->D, old, old2, flux, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_lsf_fields(scihpc_ctx *ctx, const double prm[4], const double *phi, double *heaviside, double *delta,
                      double *sign, double *density, double *viscosity, void *stream) {
    REQUIRE(ctx && prm && phi, "lsf_fields: NULL argument");
    launch_lsf_fields(ctx->D, prm, phi, heaviside, delta, sign, density, viscosity, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_curvature(scihpc_ctx *ctx, const double *phi, const double *const d[9], double *curv, void *stream) {
    REQUIRE(ctx && phi && d && curv, "curvature: NULL argument");
    REQUIRE(ctx->D.ndim >= 2, "curvature: ndim must be 2 or 3");
    launch_curvature(ctx->D, phi, d, curv, S(stream));
    CHECK_LAUNCH();
    return SCIHPC_OK;
}

int scihpc_lsf_integrals(scihpc_ctx *ctx, const double prm[4], const double *phi, double out[2], void *stream) {
    REQUIRE(ctx && prm && phi && out, "lsf_integrals: NULL argument");
    REQUIRE(ctx->D.ndim >= 2, "lsf_integrals: ndim must be 2 or 3");
    launch_lsf_integral(ctx->D, prm, phi, 0, ctx->work, ctx->partial, ctx->red, S(stream));
    launch_lsf_integral(ctx->D, prm, phi, 1, ctx->work, ctx->partial, ctx->red + 1, S(stream));
    CHECK_LAUNCH();
    double h[2];
    SCIHPC_CUDA(cudaMemcpyAsync(h, ctx->red, 2 * sizeof(double), cudaMemcpyDeviceToHost, S(stream)));
    SCIHPC_CUDA(cudaStreamSynchronize(S(stream)));
    out[0] = h[0] * ctx->D.dv;   // wrapper_func.cpp:510
    out[1] = h[1] * ctx->D.dv;   // wrapper_func.cpp:571
    return SCIHPC_OK;
}

// ------------------------------------------------------------------ pressure Poisson
int scihpc_poisson_create(const scihpc_grid *grid, int bc, int density_mode, int precision, scihpc_poisson **out) {
    REQUIRE(out, "poisson_create: out is NULL");
    int rc = check_grid(grid);
    if (rc) return rc;
    REQUIRE(grid->ndim >= 2, "poisson_create: ndim must be 2 or 3");
    REQUIRE(bc == 0 || bc == 1, "poisson_create: bc must be 0 (Neumann) or 1 (Dirichlet)");
    REQUIRE(precision == 0 || precision == 1, "poisson_create: precision must be 0 (FP64) or 1 (FP32 inner)");
    REQUIRE(!(density_mode && bc == 1), "poisson_create: density coefficients are supported with Neumann walls");
    auto *p = new (std::nothrow) scihpc_poisson;
    if (!p) return SCIHPC_ERR_NOMEM;
    rc = p->ps.create(grid, bc, density_mode ? 1 : 0, precision);
    if (rc) {
        p->ps.destroy();
        delete p;
        return rc;
    }
    *out = p;
    return SCIHPC_OK;
}

int scihpc_poisson_destroy(scihpc_poisson *ps) {
    if (!ps) return SCIHPC_OK;
    ps->ps.destroy();
    delete ps;
    return SCIHPC_OK;
}

int scihpc_poisson_set_density(scihpc_poisson *ps, const double *rho, void *stream) {
    REQUIRE(ps && rho, "poisson_set_density: NULL argument");
    return ps->ps.set_density(rho, S(stream));
}

int scihpc_poisson_solve(scihpc_poisson *ps, const double *rhs, double *p, int use_guess, double rel_tol, int max_iter,
                         int *iters, double *relres, void *stream) {
    REQUIRE(ps && rhs && p, "poisson_solve: NULL argument");
    REQUIRE(rel_tol > 0.0 && max_iter > 0, "poisson_solve: rel_tol and max_iter must be positive");
    return ps->ps.solve(rhs, p, use_guess, rel_tol, max_iter, iters, relres, S(stream));
}

int scihpc_poisson_residual(scihpc_poisson *ps, const double *rhs, const double *p, double *norm, void *stream) {
    REQUIRE(ps && rhs && p && norm, "poisson_residual: NULL argument");
    return ps->ps.residual(rhs, p, norm, S(stream));
}

int scihpc_poisson_set_inner(scihpc_poisson *ps, double inner_tol, int inner_max) {
    REQUIRE(ps && inner_tol > 0.0 && inner_tol < 1.0 && inner_max >= 1, "poisson_set_inner: bad argument");
    ps->ps.inner_tol = inner_tol;
    ps->ps.inner_max = inner_max;
    return SCIHPC_OK;
}

int scihpc_poisson_time_vcycles(scihpc_poisson *ps, const double *rhs, double *p, int ncycles, float *ms,
                                void *stream) {
    REQUIRE(ps && rhs && p && ms && ncycles > 0, "poisson_time_vcycles: bad argument");
    return ps->ps.time_vcycles(rhs, p, ncycles, ms, S(stream));
}

int scihpc_poisson_levels(scihpc_poisson *ps, int *level_n, int max_levels) {
    if (!ps || !level_n) return -SCIHPC_ERR_ARG;
    return ps->ps.levels(level_n, max_levels);
}

// ------------------------------------------------------------------ two-phase step
int scihpc_twophase_create(const scihpc_grid *grid, const int vel_bc[6], const int scalar_bc[6], const double prm[16],
                           const int opt[5], scihpc_twophase **out) {
    REQUIRE(out && vel_bc && scalar_bc && prm && opt, "twophase_create: NULL argument");
    int rc = check_grid(grid);
    if (rc) return rc;
    REQUIRE(grid->ndim >= 2, "twophase_create: ndim must be 2 or 3");
    REQUIRE(opt[0] == 0 || opt[0] == 1, "twophase_create: scheme must be 0 (UCCD) or 1 (WENO5)");
    REQUIRE(opt[3] == 0 || opt[3] == 1, "twophase_create: pressure precision must be 0 or 1");
    for (int f = 0; f < 2 * grid->ndim; ++f)
        REQUIRE(vel_bc[f] >= 0 && vel_bc[f] <= 4 && scalar_bc[f] >= 0 && scalar_bc[f] <= 4,
                "twophase_create: boundary type out of range");
    for (int f = 0; f < 2 * grid->ndim; ++f)
        REQUIRE(scalar_bc[f] == 1 && (vel_bc[f] == 2 || vel_bc[f] == 3),
                "twophase_create: the multigrid pressure solve supports walls (no_slip/slip velocity, neumann scalars)");
    auto *t = new (std::nothrow) scihpc_twophase;
    if (!t) return SCIHPC_ERR_NOMEM;
    rc = t->tp.create(grid, vel_bc, scalar_bc, prm, opt);
    if (rc) {
        t->tp.destroy();
        delete t;
        return rc;
    }
    *out = t;
    return SCIHPC_OK;
}

int scihpc_twophase_destroy(scihpc_twophase *tp) {
    if (!tp) return SCIHPC_OK;
    tp->tp.destroy();
    delete tp;
    return SCIHPC_OK;
}

int scihpc_twophase_upload(scihpc_twophase *tp, const char *name, const double *host) {
    REQUIRE(tp && name && host, "twophase_upload: NULL argument");
    double *d = tp->tp.field(name);
    REQUIRE(d, "twophase_upload: unknown field name");
    SCIHPC_CUDA(cudaMemcpyAsync(d, host, size_t(tp->tp.D.size()) * sizeof(double), cudaMemcpyHostToDevice, tp->tp.stream));
    SCIHPC_CUDA(cudaStreamSynchronize(tp->tp.stream));
    return SCIHPC_OK;
}

int scihpc_twophase_download(scihpc_twophase *tp, const char *name, double *host) {
    REQUIRE(tp && name && host, "twophase_download: NULL argument");
    double *d = tp->tp.field(name);
    REQUIRE(d, "twophase_download: unknown field name");
    SCIHPC_CUDA(cudaMemcpyAsync(host, d, size_t(tp->tp.D.size()) * sizeof(double), cudaMemcpyDeviceToHost, tp->tp.stream));
    SCIHPC_CUDA(cudaStreamSynchronize(tp->tp.stream));
    return SCIHPC_OK;
}

int scihpc_twophase_upload_many(scihpc_twophase *tp, int n, const char *const *names, const double *const *host) {
    REQUIRE(tp && n >= 0 && (n == 0 || (names && host)), "twophase_upload_many: bad argument");
    for (int f = 0; f < n; ++f) {
        REQUIRE(names[f] && host[f], "twophase_upload_many: NULL name or buffer");
        REQUIRE(tp->tp.field(names[f]), "twophase_upload_many: unknown field name");
    }
    const size_t bytes = size_t(tp->tp.D.size()) * sizeof(double);
    for (int f = 0; f < n; ++f)
        SCIHPC_CUDA(cudaMemcpyAsync(tp->tp.field(names[f]), host[f], bytes, cudaMemcpyHostToDevice, tp->tp.stream));
    SCIHPC_CUDA(cudaStreamSynchronize(tp->tp.stream));
    return SCIHPC_OK;
}

int scihpc_twophase_download_many(scihpc_twophase *tp, int n, const char *const *names, double *const *host) {
    REQUIRE(tp && n >= 0 && (n == 0 || (names && host)), "twophase_download_many: bad argument");
    for (int f = 0; f < n; ++f) {
        REQUIRE(names[f] && host[f], "twophase_download_many: NULL name or buffer");
        REQUIRE(tp->tp.field(names[f]), "twophase_download_many: unknown field name");
    }
    const size_t bytes = size_t(tp->tp.D.size()) * sizeof(double);
    for (int f = 0; f < n; ++f)
        SCIHPC_CUDA(cudaMemcpyAsync(host[f], tp->tp.field(names[f]), bytes, cudaMemcpyDeviceToHost, tp->tp.stream));
    SCIHPC_CUDA(cudaStreamSynchronize(tp->tp.stream));
    return SCIHPC_OK;
}

int scihpc_twophase_field(scihpc_twophase *tp, const char *name, double **dev) {
    REQUIRE(tp && name && dev, "twophase_field: NULL argument");
    double *d = tp->tp.field(name);
    REQUIRE(d, "twophase_field: unknown field name");
    *dev = d;
    return SCIHPC_OK;
}

int scihpc_twophase_checkpoint(scihpc_twophase *tp, const char *path) {
    REQUIRE(tp && path, "twophase_checkpoint: NULL argument");
    return tp->tp.checkpoint(path);
}

int scihpc_twophase_restore(scihpc_twophase *tp, const char *path) {
    REQUIRE(tp && path, "twophase_restore: NULL argument");
    return tp->tp.restore(path);
}

int scihpc_twophase_get_scalars(scihpc_twophase *tp, double out[7]) {
    REQUIRE(tp && out, "twophase_get_scalars: NULL argument");
    return tp->tp.get_scalars(out);
}

int scihpc_twophase_set_scalars(scihpc_twophase *tp, const double in[7]) {
    REQUIRE(tp && in, "twophase_set_scalars: NULL argument");
    return tp->tp.set_scalars(in);
}

int scihpc_twophase_init(scihpc_twophase *tp) {
    REQUIRE(tp, "twophase_init: NULL argument");
    return tp->tp.init();
}

#define TP_SYNC(tp)                                                 \
    do {                                                            \
        CHECK_LAUNCH();                                             \
        SCIHPC_CUDA(cudaStreamSynchronize((tp)->tp.stream));        \
    } while (0)

int scihpc_twophase_find_dt(scihpc_twophase *tp) {
    REQUIRE(tp, "twophase_find_dt: NULL argument");
    tp->tp.find_dt();
    TP_SYNC(tp);
    return SCIHPC_OK;
}

int scihpc_twophase_advect(scihpc_twophase *tp) {
    REQUIRE(tp, "twophase_advect: NULL argument");
    tp->tp.advect();
    TP_SYNC(tp);
    return SCIHPC_OK;
}

int scihpc_twophase_mpls(scihpc_twophase *tp, int count) {
    REQUIRE(tp && count >= 0, "twophase_mpls: bad argument");
    tp->tp.mpls(count);
    TP_SYNC(tp);
    return SCIHPC_OK;
}

int scihpc_twophase_reinit(scihpc_twophase *tp, int *steps) {
    REQUIRE(tp, "twophase_reinit: NULL argument");
    const int n = tp->tp.reinit();
    TP_SYNC(tp);
    if (steps) *steps = n;
    return SCIHPC_OK;
}

int scihpc_twophase_find_sign(scihpc_twophase *tp) {
    REQUIRE(tp, "twophase_find_sign: NULL argument");
    tp->tp.find_sign();
    TP_SYNC(tp);
    return SCIHPC_OK;
}

int scihpc_twophase_reinit_step(scihpc_twophase *tp, int lambda) {
    REQUIRE(tp && (lambda == 0 || lambda == 1), "twophase_reinit_step: bad argument");
    tp->tp.reinit_step(lambda);
    TP_SYNC(tp);
    return SCIHPC_OK;
}

int scihpc_twophase_set_scheme(scihpc_twophase *tp, int scheme) {
    REQUIRE(tp && (scheme == 0 || scheme == 1), "twophase_set_scheme: scheme must be 0 (UCCD) or 1 (WENO5)");
    tp->tp.set_scheme(scheme);
    return SCIHPC_OK;
}

int scihpc_twophase_set_source_scheme(scihpc_twophase *tp, int scheme) {
    REQUIRE(tp && (scheme == 0 || scheme == 1),
            "twophase_set_source_scheme: scheme must be 0 (compact) or 1 (second order)");
    tp->tp.set_source_scheme(scheme);
    return SCIHPC_OK;
}

int scihpc_twophase_find_source(scihpc_twophase *tp) {
    REQUIRE(tp, "twophase_find_source: NULL argument");
    tp->tp.find_source();
    TP_SYNC(tp);
    return SCIHPC_OK;
}

int scihpc_twophase_ab_solve(scihpc_twophase *tp, int *iters, double *relres) {
    REQUIRE(tp, "twophase_ab_solve: NULL argument");
    return tp->tp.ab_solve(iters, relres);
}

int scihpc_twophase_intermediate_velocity(scihpc_twophase *tp) {
    REQUIRE(tp, "twophase_intermediate_velocity: NULL argument");
    return tp->tp.intermediate_velocity();
}

int scihpc_twophase_projection(scihpc_twophase *tp, int *iters, double *relres) {
    REQUIRE(tp, "twophase_projection: NULL argument");
    return tp->tp.projection(iters, relres);
}

int scihpc_twophase_node_from_face(scihpc_twophase *tp) {
    REQUIRE(tp, "twophase_node_from_face: NULL argument");
    return tp->tp.node_from_face();
}

int scihpc_twophase_set_ppe_schedule(scihpc_twophase *tp, int schedule, int tol_mode) {
    REQUIRE(tp, "twophase_set_ppe_schedule: NULL argument");
    REQUIRE(schedule == 0 || schedule == 1, "twophase_set_ppe_schedule: schedule must be 0 (projection) or 1 (stock)");
    REQUIRE(tol_mode == 0 || tol_mode == 1, "twophase_set_ppe_schedule: tol_mode must be 0 (relative) or 1 (absolute)");
    return tp->tp.set_ppe_schedule(schedule, tol_mode);
}

int scihpc_twophase_pressure_guess(scihpc_twophase *tp) {
    REQUIRE(tp, "twophase_pressure_guess: NULL argument");
    return tp->tp.pressure_guess();
}

int scihpc_twophase_fpc_coefficients(scihpc_twophase *tp) {
    REQUIRE(tp, "twophase_fpc_coefficients: NULL argument");
    return tp->tp.fpc_coefficients();
}

int scihpc_twophase_fast_pressure_correction(scihpc_twophase *tp, int *iters, double *relres) {
    REQUIRE(tp, "twophase_fast_pressure_correction: NULL argument");
    return tp->tp.fast_pressure_correction(iters, relres);
}

int scihpc_twophase_step(scihpc_twophase *tp, int nsteps, int use_graph, int sync) {
    REQUIRE(tp && nsteps >= 0, "twophase_step: bad argument");
    int rc = tp->tp.step(nsteps, use_graph != 0);
    if (rc) return rc;
    if (sync) SCIHPC_CUDA(cudaStreamSynchronize(tp->tp.stream));
    return SCIHPC_OK;
}

int scihpc_twophase_diagnostics(scihpc_twophase *tp, double out[3]) {
    REQUIRE(tp && out, "twophase_diagnostics: NULL argument");
    return tp->tp.diagnostics(out);
}

int scihpc_twophase_stream(scihpc_twophase *tp, void **stream) {
    REQUIRE(tp && stream, "twophase_stream: NULL argument");
    *stream = tp->tp.stream;
    return SCIHPC_OK;
}

int scihpc_twophase_time_reinit_gradient(scihpc_twophase *tp, int n, float *ms) {
    REQUIRE(tp && ms && n > 0, "twophase_time_reinit_gradient: bad argument");
    return tp->tp.time_reinit_gradient(n, ms);
}

// FP64 roof of this GPU: independent chains of fused multiply-adds per thread, enough
// blocks for every SM; 2 flops per FMA.
namespace {
constexpr int FP64_CHAINS = 8;
__global__ void k_fp64_fma_chains(double *out, int iters, double b, double c) {
    double a[FP64_CHAINS];
    for (int k = 0; k < FP64_CHAINS; ++k) a[k] = double(threadIdx.x + k);
    for (int it = 0; it < iters; ++it)
#pragma unroll
        for (int k = 0; k < FP64_CHAINS; ++k) a[k] = fma(a[k], b, c);
    double s = 0.0;
    for (int k = 0; k < FP64_CHAINS; ++k) s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

int scihpc_measure_fp64_peak(double *tflops) {
    REQUIRE(tflops, "measure_fp64_peak: NULL argument");
    const int blocks = NUM_SMS * 8, threads = 256, iters = 4096;
    double *out = nullptr;
    SCIHPC_CUDA(cudaMalloc(&out, size_t(blocks) * threads * sizeof(double)));
    cudaEvent_t e0, e1;
    SCIHPC_CUDA(cudaEventCreate(&e0));
    SCIHPC_CUDA(cudaEventCreate(&e1));
    // b slightly below 1 keeps the chains finite; c breaks any algebraic shortcut
    for (int w = 0; w < 2; ++w) k_fp64_fma_chains<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(e0);
        k_fp64_fma_chains<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float t = 0.0f;
        cudaEventElapsedTime(&t, e0, e1);
        best = t < best ? t : best;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return cuda_fail(err, "fp64 peak kernel", __FILE__, __LINE__);
    const double flops = 2.0 * double(blocks) * threads * iters * FP64_CHAINS;
    *tflops = flops / (double(best) * 1e-3) / 1e12;
    return SCIHPC_OK;
}

int scihpc_twophase_graph_stats(scihpc_twophase *tp, long long out[4]) {
    REQUIRE(tp && out, "twophase_graph_stats: NULL argument");
    return tp->tp.graph_stats(out);
}

int scihpc_twophase_ppe_stats(scihpc_twophase *tp, double out[3]) {
    REQUIRE(tp && out, "twophase_ppe_stats: NULL argument");
    out[0] = tp->tp.last_iters;
    out[1] = tp->tp.last_relres;
    out[2] = tp->tp.last_ms;
    return SCIHPC_OK;
}

// ------------------------------------------------------------------ tensor-core convolutions
int scihpc_conv3x3(const void *x, const void *w, const float *bias, float *out, int h, int w_, int ci, int co, int relu,
                   void *stream) {
    REQUIRE(x && w && out && h > 0 && w_ > 0, "conv3x3: bad argument");
    REQUIRE(ci % 16 == 0 && co % 16 == 0 && co >= 16 && co <= 256, "conv3x3: channels must be multiples of 16, co <= 256");
    static int *err = nullptr;
    if (!err) {
        SCIHPC_CUDA(cudaMalloc(&err, sizeof(int)));
        SCIHPC_CUDA(cudaMemset(err, 0, sizeof(int)));
        int rc = conv3x3_init(256);
        if (rc) return rc;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc = conv3x3_forward(static_cast<const __nv_bfloat16 *>(x), static_cast<const __nv_bfloat16 *>(w), bias, out,
                             false, h, w_, ci, co, relu != 0, err, s);
    if (rc) return rc;
    CHECK_LAUNCH();
    int herr = 0;
    SCIHPC_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    SCIHPC_CUDA(cudaStreamSynchronize(s));
    if (herr) {
        set_last_error("conv3x3: a tensor-core barrier wait timed out");
        return SCIHPC_ERR_CUDA;
    }
    return SCIHPC_OK;
}

int scihpc_conv3x3_wgrad(const void *x, const void *dz, float *dw, float *partial, int splits, int h, int w_, int ci,
                         int co, void *stream) {
    REQUIRE(x && dz && dw && partial && splits > 0 && h > 0 && w_ > 0, "conv3x3_wgrad: bad argument");
    REQUIRE(ci % 16 == 0 && co % 16 == 0 && co >= 16 && co <= 256, "conv3x3_wgrad: channels must be multiples of 16");
    static int *err = nullptr;
    if (!err) {
        SCIHPC_CUDA(cudaMalloc(&err, sizeof(int)));
        SCIHPC_CUDA(cudaMemset(err, 0, sizeof(int)));
        int rc = conv3x3_init(256);
        if (rc) return rc;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc = conv3x3_wgrad(static_cast<const __nv_bfloat16 *>(x), static_cast<const __nv_bfloat16 *>(dz), partial, dw, h,
                           w_, ci, co, splits, err, s);
    if (rc) return rc;
    CHECK_LAUNCH();
    int herr = 0;
    SCIHPC_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    SCIHPC_CUDA(cudaStreamSynchronize(s));
    if (herr) {
        set_last_error("conv3x3_wgrad: a tensor-core barrier wait timed out");
        return SCIHPC_ERR_CUDA;
    }
    return SCIHPC_OK;
}

// the 3x3x3 convolution and its weight gradient (same conventions, 27 taps, d x h x w voxels)
int scihpc_conv3x3x3(const void *x, const void *w, const float *bias, float *out, int d, int h, int w_, int ci, int co,
                     int relu, void *stream) {
    REQUIRE(x && w && out && d > 0 && h > 0 && w_ > 0, "conv3x3x3: bad argument");
    REQUIRE(ci % 16 == 0 && co % 16 == 0 && co >= 16 && co <= 256, "conv3x3x3: channels must be multiples of 16, co <= 256");
    static int *err = nullptr;
    if (!err) {
        SCIHPC_CUDA(cudaMalloc(&err, sizeof(int)));
        SCIHPC_CUDA(cudaMemset(err, 0, sizeof(int)));
        int rc = conv3x3_init(256);
        if (rc) return rc;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc = conv3x3x3_forward(static_cast<const __nv_bfloat16 *>(x), static_cast<const __nv_bfloat16 *>(w), bias, out,
                               false, d, h, w_, ci, co, relu != 0, err, s);
    if (rc) return rc;
    CHECK_LAUNCH();
    int herr = 0;
    SCIHPC_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    SCIHPC_CUDA(cudaStreamSynchronize(s));
    if (herr) {
        set_last_error("conv3x3x3: a tensor-core barrier wait timed out");
        return SCIHPC_ERR_CUDA;
    }
    return SCIHPC_OK;
}

int scihpc_conv3x3x3_wgrad(const void *x, const void *dz, float *dw, float *partial, int splits, int d, int h, int w_,
                           int ci, int co, void *stream) {
    REQUIRE(x && dz && dw && partial && splits > 0 && d > 0 && h > 0 && w_ > 0, "conv3x3x3_wgrad: bad argument");
    REQUIRE(ci % 16 == 0 && co % 16 == 0 && co >= 16 && co <= 256, "conv3x3x3_wgrad: channels must be multiples of 16");
    static int *err = nullptr;
    if (!err) {
        SCIHPC_CUDA(cudaMalloc(&err, sizeof(int)));
        SCIHPC_CUDA(cudaMemset(err, 0, sizeof(int)));
        int rc = conv3x3_init(256);
        if (rc) return rc;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int rc = conv3x3x3_wgrad(static_cast<const __nv_bfloat16 *>(x), static_cast<const __nv_bfloat16 *>(dz), partial, dw,
                             d, h, w_, ci, co, splits, err, s);
    if (rc) return rc;
    CHECK_LAUNCH();
    int herr = 0;
    SCIHPC_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    SCIHPC_CUDA(cudaStreamSynchronize(s));
    if (herr) {
        set_last_error("conv3x3x3_wgrad: a tensor-core barrier wait timed out");
        return SCIHPC_ERR_CUDA;
    }
    return SCIHPC_OK;
}

// ------------------------------------------------------------------ learned pressure guess
// one handle for both networks: the 2D UNet, or the 3D UNet3 when net3 is set
struct scihpc_unet {
    UNet net;
    UNet3 *net3 = nullptr;
};

int scihpc_unet_create(int h, int w, unsigned seed, scihpc_unet **out) {
    REQUIRE(out, "unet_create: out is NULL");
    auto *u = new (std::nothrow) scihpc_unet;
    if (!u) return SCIHPC_ERR_NOMEM;
    int rc = u->net.create(h, w, seed);
    if (rc) {
        u->net.destroy();
        delete u;
        return rc;
    }
    *out = u;
    return SCIHPC_OK;
}

int scihpc_unet_create_coarse(int h, int w, int factor, unsigned seed, scihpc_unet **out) {
    REQUIRE(out, "unet_create_coarse: out is NULL");
    REQUIRE(factor >= 1 && factor <= 16, "unet_create_coarse: factor must be 1 .. 16");
    auto *u = new (std::nothrow) scihpc_unet;
    if (!u) return SCIHPC_ERR_NOMEM;
    int rc = u->net.create(h, w, seed, factor);
    if (rc) {
        u->net.destroy();
        delete u;
        return rc;
    }
    *out = u;
    return SCIHPC_OK;
}

int scihpc_unet_create3(int n0, int n1, int n2, unsigned seed, scihpc_unet **out) {
    REQUIRE(out, "unet_create3: out is NULL");
    auto *u = new (std::nothrow) scihpc_unet;
    if (!u) return SCIHPC_ERR_NOMEM;
    u->net3 = new (std::nothrow) UNet3;
    if (!u->net3) {
        delete u;
        return SCIHPC_ERR_NOMEM;
    }
    int rc = u->net3->create(n0, n1, n2, seed);
    if (rc) {
        u->net3->destroy();
        delete u->net3;
        delete u;
        return rc;
    }
    *out = u;
    return SCIHPC_OK;
}

int scihpc_unet_destroy(scihpc_unet *u) {
    if (u) {
        if (u->net3) {
            u->net3->destroy();
            delete u->net3;
        } else {
            u->net.destroy();
        }
        delete u;
    }
    return SCIHPC_OK;
}

int scihpc_unet_num_params(scihpc_unet *u, long long *n) {
    REQUIRE(u && n, "unet_num_params: NULL argument");
    *n = u->net3 ? u->net3->num_params() : u->net.num_params();
    return SCIHPC_OK;
}

int scihpc_unet_set_weights(scihpc_unet *u, const float *host, long long n) {
    REQUIRE(u && host, "unet_set_weights: NULL argument");
    return u->net3 ? u->net3->set_weights(host, n) : u->net.set_weights(host, n);
}

int scihpc_unet_get_weights(scihpc_unet *u, float *host, long long n) {
    REQUIRE(u && host, "unet_get_weights: NULL argument");
    return u->net3 ? u->net3->get(host, n, false) : u->net.get(host, n, false);
}

int scihpc_unet_get_gradient(scihpc_unet *u, float *host, long long n) {
    REQUIRE(u && host, "unet_get_gradient: NULL argument");
    return u->net3 ? u->net3->get(host, n, true) : u->net.get(host, n, true);
}

int scihpc_unet_infer(scihpc_unet *u, const scihpc_grid *grid, const double *rho, const double *rhs,
                      const double *pprev, double *guess) {
    REQUIRE(u && grid && rho && rhs && guess, "unet_infer: NULL argument");
    const Dims D = make_dims(grid);
    return u->net3 ? u->net3->infer(D, rho, rhs, pprev, guess) : u->net.infer(D, rho, rhs, pprev, guess);
}

int scihpc_unet_loss_grad(scihpc_unet *u, const scihpc_grid *grid, const double *rho, const double *rhs,
                          const double *pprev, const double *p, double *loss) {
    REQUIRE(u && grid && rho && rhs && p && loss, "unet_loss_grad: NULL argument");
    const Dims D = make_dims(grid);
    return u->net3 ? u->net3->loss_grad(D, rho, rhs, pprev, p, loss) : u->net.loss_grad(D, rho, rhs, pprev, p, loss);
}

int scihpc_unet_train_step(scihpc_unet *u, const scihpc_grid *grid, const double *rho, const double *rhs,
                           const double *pprev, const double *p, float lr, double *loss) {
    REQUIRE(u && grid && rho && rhs && p && loss && lr > 0.0f, "unet_train_step: bad argument");
    const Dims D = make_dims(grid);
    return u->net3 ? u->net3->train_step(D, rho, rhs, pprev, p, lr, loss)
                   : u->net.train_step(D, rho, rhs, pprev, p, lr, loss);
}

int scihpc_unet_stream(scihpc_unet *u, void **stream) {
    REQUIRE(u && stream, "unet_stream: NULL argument");
    *stream = u->net3 ? u->net3->stream : u->net.stream;
    return SCIHPC_OK;
}

}  // extern "C"
