// ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Exposes selected functions of the reference implementation (luisleo526/SciHPC,
// compiled from its own sources by oracle/Makefile) over flat arrays, so that the
// oracle tests can call them through ctypes and compare them with this project's CPU
// restatement (oracle/port) and write golden fixtures.  Nothing in the product
// links this file; it is built only where the reference sources are present.
//
// Flat array layout: [Nx][Ny][Nz], k fastest -- the reference's own logical
// data[i][j][k] order (scalar_data.h:14, global.cpp:7-19).  Multigrid vectors use the
// reference's x-fastest order of multigrid_base::of (multigrid_base.cpp:8-14).
//
// Boundary-condition codes: 0 periodic, 1 neumann, 2 no_slip, 3 slip, 4 dirichlet
// (the strings of bc_factory.h:18-22).  Face order: xl, xr, yl, yr, zl, zr (the
// argument order of the wrapper/bc_factory constructors, wrapper.h:18-22).

#include <cstring>
#include <cmath>
#include <string>
#include <vector>

#include "wrapper.h"
#include "structured_grid.h"
#include "flux.h"
#include "wrapper_func.h"
#include "runge_kutta.h"
#include "projection_method.h"
#include "bc_factory.h"
#include "source.h"
#include "simple_bc.h"
#include "godunov_gradient.h"
#include "multigrid.h"
#include "second_order_solver.h"
#include "vtkWriter.h"

namespace {

struct Dims {
    int ndim, nx, ny, nz, Nx, Ny, Nz;
};

Dims dims_of(int ndim, const int *n) {
    Dims d{};
    d.ndim = ndim;
    d.nx = n[0];
    d.ny = ndim > 1 ? n[1] : 1;
    d.nz = ndim > 2 ? n[2] : 1;
    d.Nx = d.nx + 6;
    d.Ny = ndim > 1 ? d.ny + 6 : 1;
    d.Nz = ndim > 2 ? d.nz + 6 : 1;
    return d;
}

structured_grid *make_grid(int ndim, const int *n, const double *lo, const double *hi) {
    if (ndim == 1) return new structured_grid(axis{lo[0], hi[0], n[0]});
    if (ndim == 2) return new structured_grid(axis{lo[0], hi[0], n[0]}, axis{lo[1], hi[1], n[1]});
    return new structured_grid(axis{lo[0], hi[0], n[0]}, axis{lo[1], hi[1], n[1]}, axis{lo[2], hi[2], n[2]});
}

scalar_data *make_scalar(const Dims &d) {
    if (d.ndim == 1) return new scalar_data(d.nx);
    if (d.ndim == 2) return new scalar_data(d.nx, d.ny);
    return new scalar_data(d.nx, d.ny, d.nz);
}

vector_data *make_vector(const Dims &d) {
    if (d.ndim == 1) return new vector_data(d.nx);
    if (d.ndim == 2) return new vector_data(d.nx, d.ny);
    return new vector_data(d.nx, d.ny, d.nz);
}

void load(DataType ***a, const double *src, const Dims &d) {
    for (int i = 0; i < d.Nx; ++i)
        for (int j = 0; j < d.Ny; ++j)
            for (int k = 0; k < d.Nz; ++k) a[i][j][k] = src[(size_t(i) * d.Ny + j) * d.Nz + k];
}

void save(double *dst, DataType ***a, const Dims &d) {
    for (int i = 0; i < d.Nx; ++i)
        for (int j = 0; j < d.Ny; ++j)
            for (int k = 0; k < d.Nz; ++k) dst[(size_t(i) * d.Ny + j) * d.Nz + k] = a[i][j][k];
}

bc_info bc_of(int code, double value) {
    static const std::string names[5] = {PERIODIC, NEUMANN, NO_SLIP, SLIP, DIRICHLET};
    bc_info b;
    b.type = names[code];
    b.value = value;
    return b;
}

bc_factory *make_factory(structured_grid *geo, int ndim, const int *t, const double *v) {
    if (ndim == 1) return new bc_factory(geo, bc_of(t[0], v[0]), bc_of(t[1], v[1]));
    if (ndim == 2)
        return new bc_factory(geo, bc_of(t[0], v[0]), bc_of(t[1], v[1]), bc_of(t[2], v[2]), bc_of(t[3], v[3]));
    return new bc_factory(geo, bc_of(t[0], v[0]), bc_of(t[1], v[1]), bc_of(t[2], v[2]), bc_of(t[3], v[3]),
                          bc_of(t[4], v[4]), bc_of(t[5], v[5]));
}

wrapper *make_wrapper(bool scalar, structured_grid *geo, int ndim, const int *t, const double *v) {
    if (ndim == 1) return new wrapper(scalar, geo, bc_of(t[0], v[0]), bc_of(t[1], v[1]));
    if (ndim == 2)
        return new wrapper(scalar, geo, bc_of(t[0], v[0]), bc_of(t[1], v[1]), bc_of(t[2], v[2]), bc_of(t[3], v[3]));
    return new wrapper(scalar, geo, bc_of(t[0], v[0]), bc_of(t[1], v[1]), bc_of(t[2], v[2]), bc_of(t[3], v[3]),
                       bc_of(t[4], v[4]), bc_of(t[5], v[5]));
}

// Convection right-hand side with the WENO5 derivative: the same body as the reference's
// convection (source.cpp:8-40) with the WENO call that is commented out there (source.cpp:11).
void convection_weno(wrapper *f, wrapper *vel, DataType ***s, void (*flux)(scalar_data *, vector_data *)) {
    flux(f->scalar, vel->vector);
    f->solvers->weno->weno5_find_derivatives(f->scalar, vel->vector);
    for (int i = 0; i < f->scalar->Nx; ++i)
        for (int j = 0; j < f->scalar->Ny; ++j)
            for (int k = 0; k < f->scalar->Nz; ++k) s[i][j][k] = -vel->vector->x.data[i][j][k] * f->scalar->fx[i][j][k];
    if (f->scalar->ndim > 1)
        for (int i = 0; i < f->scalar->Nx; ++i)
            for (int j = 0; j < f->scalar->Ny; ++j)
                for (int k = 0; k < f->scalar->Nz; ++k) s[i][j][k] -= vel->vector->y.data[i][j][k] * f->scalar->fy[i][j][k];
    if (f->scalar->ndim > 2)
        for (int i = 0; i < f->scalar->Nx; ++i)
            for (int j = 0; j < f->scalar->Ny; ++j)
                for (int k = 0; k < f->scalar->Nz; ++k) s[i][j][k] -= vel->vector->z.data[i][j][k] * f->scalar->fz[i][j][k];
}

typedef void (*flux_fn)(scalar_data *, vector_data *);
const flux_fn IDENTITY = static_cast<flux_fn>(&identity_flux);

}  // namespace

extern "C" {

// ---------------------------------------------------------------- boundary fills
// location: 0 node-centred, 1/2/3 staggered in x/y/z (bc_factory.cpp:123-437).
int ref_bc_fill(int ndim, const int *n, const double *lo, const double *hi, int location, const int *types,
                const double *values, double *f) {
    Dims d = dims_of(ndim, n);
    structured_grid *geo = make_grid(ndim, n, lo, hi);
    bc_factory *fac = make_factory(geo, ndim, types, values);
    scalar_data *s = make_scalar(d);
    load(s->data, f, d);
    if (location == 0) fac->apply_node_centered(s);
    else if (location == 1) fac->apply_node_staggered_x(s);
    else if (location == 2) fac->apply_node_staggered_y(s);
    else fac->apply_node_staggered_z(s);
    save(f, s->data, d);
    return 0;
}

// identity_with_extrapolation[_face_x/y/z] (flux.cpp:98-330): flux <- data, ghosts zero-order.
int ref_flux_extrapolate(int ndim, const int *n, int location, const double *data, double *flux) {
    Dims d = dims_of(ndim, n);
    scalar_data *s = make_scalar(d);
    load(s->data, data, d);
    if (location == 0) identity_with_extrapolation(s);
    else if (location == 1) identity_with_extrapolation_face_x(s);
    else if (location == 2) identity_with_extrapolation_face_y(s);
    else identity_with_extrapolation_face_z(s);
    save(flux, s->flux, d);
    return 0;
}

// zero_order_extrapolation on a raw ghosted array (simple_bc.cpp:7-43).
int ref_zero_order_extrapolation(int ndim, const int *n, double *f) {
    Dims d = dims_of(ndim, n);
    DataType ***a = init_array(d.Nx, d.Ny, d.Nz);
    load(a, f, d);
    zero_order_extrapolation(a, d.Nx, d.Ny, d.Nz, 3);
    save(f, a, d);
    return 0;
}

// uccd_solver::find_derivatives (uccd_solver.cpp:211-216).  out: fx, fy, fz, fxx, fyy, fzz.
int ref_uccd(int ndim, const int *n, const double *lo, const double *hi, const double *flux, const double *u,
             const double *v, const double *w, double *out) {
    Dims d = dims_of(ndim, n);
    size_t N = size_t(d.Nx) * d.Ny * d.Nz;
    structured_grid *geo = make_grid(ndim, n, lo, hi);
    scalar_data *f = make_scalar(d);
    vector_data *vel = make_vector(d);
    load(f->flux, flux, d);
    load(vel->x.data, u, d);
    load(vel->y.data, v, d);
    load(vel->z.data, w, d);
    uccd_solver solver(f, geo);
    solver.find_derivatives(f, vel);
    save(out + 0 * N, f->fx, d);
    save(out + 1 * N, f->fy, d);
    save(out + 2 * N, f->fz, d);
    save(out + 3 * N, f->fxx, d);
    save(out + 4 * N, f->fyy, d);
    save(out + 5 * N, f->fzz, d);
    return 0;
}

// ccd_solver::find_derivatives[_all] (ccd_solver.cpp:284-305).
// out: fx, fy, fz, fxx, fyy, fzz, fxy, fyz, fzx.
int ref_ccd(int ndim, const int *n, const double *lo, const double *hi, int mixed, const double *flux, double *out) {
    Dims d = dims_of(ndim, n);
    size_t N = size_t(d.Nx) * d.Ny * d.Nz;
    structured_grid *geo = make_grid(ndim, n, lo, hi);
    scalar_data *f = make_scalar(d);
    load(f->flux, flux, d);
    ccd_solver solver(f, geo);
    if (mixed) solver.find_derivatives_all(f);
    else solver.find_derivatives(f);
    DataType ***arr[9] = {f->fx, f->fy, f->fz, f->fxx, f->fyy, f->fzz, f->fxy, f->fyz, f->fzx};
    for (int q = 0; q < 9; ++q) save(out + q * N, arr[q], d);
    return 0;
}

// weno_solver::weno5_find_derivatives (weno_solver.cpp:270-278).  out: fx, fy, fz (interior).
int ref_weno5(int ndim, const int *n, const double *lo, const double *hi, const double *flux, const double *u,
              const double *v, const double *w, double *out) {
    Dims d = dims_of(ndim, n);
    size_t N = size_t(d.Nx) * d.Ny * d.Nz;
    structured_grid *geo = make_grid(ndim, n, lo, hi);
    scalar_data *f = make_scalar(d);
    vector_data *vel = make_vector(d);
    load(f->flux, flux, d);
    load(vel->x.data, u, d);
    load(vel->y.data, v, d);
    load(vel->z.data, w, d);
    weno_solver solver(f, geo);
    solver.weno5_find_derivatives(f, vel);
    save(out + 0 * N, f->fx, d);
    save(out + 1 * N, f->fy, d);
    save(out + 2 * N, f->fz, d);
    return 0;
}

// godunov_gradient (godunov_gradient.cpp:7-157): grad from phi and sign.
int ref_godunov(int ndim, const int *n, const double *lo, const double *hi, const double *phi, const double *sign,
                double *grad) {
    Dims d = dims_of(ndim, n);
    structured_grid *geo = make_grid(ndim, n, lo, hi);
    int t[6] = {1, 1, 1, 1, 1, 1};
    double v[6] = {0, 0, 0, 0, 0, 0};
    wrapper *w = make_wrapper(true, geo, ndim, t, v);
    w->link_dummy(dummy_data_alloc(w->scalar));
    load(w->scalar->data, phi, d);
    load(w->dummy->sign, sign, d);
    godunov_gradient(w);
    save(grad, w->dummy->grad, d);
    return 0;
}

// stabilized_upon_gradient (godunov_gradient.cpp:159-181): grad, then phi /= max(grad), in place.
int ref_stabilize(int ndim, const int *n, const double *lo, const double *hi, double *phi, const double *sign,
                  double *grad) {
    Dims d = dims_of(ndim, n);
    structured_grid *geo = make_grid(ndim, n, lo, hi);
    int t[6] = {1, 1, 1, 1, 1, 1};
    double v[6] = {0, 0, 0, 0, 0, 0};
    wrapper *w = make_wrapper(true, geo, ndim, t, v);
    w->link_dummy(dummy_data_alloc(w->scalar));
    load(w->scalar->data, phi, d);
    load(w->dummy->sign, sign, d);
    stabilized_upon_gradient(w);
    save(grad, w->dummy->grad, d);
    save(phi, w->scalar->data, d);
    return 0;
}

// guess_from_history (flux.cpp:653-662): flux from old and old2.
int ref_guess_from_history(int ndim, const int *n, const double *old, const double *old2, double *flux) {
    Dims d = dims_of(ndim, n);
    scalar_data *f = make_scalar(d);
    load(f->old, old, d);
    load(f->old2, old2, d);
    guess_from_history(f);
    save(flux, f->flux, d);
    return 0;
}

// Level-set property fields (wrapper_func.cpp:9-58,387-418) and the curvature of
// find_source (projection_method.cpp:258-263 then wrapper_func.cpp:115-174).
// prm: ls_width, density_ratio, viscosity_ratio, positive_ref.
// out: heaviside, delta, sign, density, viscosity, curvature.
int ref_lsf_fields(int ndim, const int *n, const double *lo, const double *hi, const double *prm, const double *phi,
                   double *out) {
    Dims d = dims_of(ndim, n);
    size_t N = size_t(d.Nx) * d.Ny * d.Nz;
    structured_grid *geo = make_grid(ndim, n, lo, hi);
    int t[6] = {1, 1, 1, 1, 1, 1};
    double v[6] = {0, 0, 0, 0, 0, 0};
    wrapper *w = make_wrapper(true, geo, ndim, t, v);
    auto *param = new problem_parameters{};
    param->ls_width = prm[0];
    param->density_ratio = prm[1];
    param->viscosity_ratio = prm[2];
    param->positive_ref = prm[3] != 0.0;
    w->link_params(param);
    w->link_dummy(dummy_data_alloc(w->scalar));
    w->link_solvers(SharedSolvers_alloc(w->scalar, geo));
    load(w->scalar->data, phi, d);
    find_heavyside(w);
    find_delta(w);
    find_sign(w);
    find_density(w);
    find_viscosity(w);
    identity_with_extrapolation(w->scalar);
    w->solvers->ccd->find_derivatives_all(w->scalar);
    find_curvature(w);
    save(out + 0 * N, w->dummy->heaviside, d);
    save(out + 1 * N, w->dummy->delta, d);
    save(out + 2 * N, w->dummy->sign, d);
    save(out + 3 * N, w->dummy->density, d);
    save(out + 4 * N, w->dummy->viscosity, d);
    save(out + 5 * N, w->dummy->curvature, d);
    return 0;
}

// lsf_mass / lsf_volume (wrapper_func.cpp:450-572).  prm as ref_lsf_fields.  out: mass, volume.
int ref_lsf_integrals(int ndim, const int *n, const double *lo, const double *hi, const double *prm,
                      const double *phi, double *out) {
    Dims d = dims_of(ndim, n);
    structured_grid *geo = make_grid(ndim, n, lo, hi);
    int t[6] = {1, 1, 1, 1, 1, 1};
    double v[6] = {0, 0, 0, 0, 0, 0};
    wrapper *w = make_wrapper(true, geo, ndim, t, v);
    auto *param = new problem_parameters{};
    param->ls_width = prm[0];
    param->density_ratio = prm[1];
    param->viscosity_ratio = prm[2];
    param->positive_ref = prm[3] != 0.0;
    w->link_params(param);
    w->link_dummy(dummy_data_alloc(w->scalar));
    load(w->scalar->data, phi, d);
    out[0] = lsf_mass(w);
    out[1] = lsf_volume(w);
    return 0;
}

// ---------------------------------------------------------------- multigrid (constant coefficient)
// The reference's Poisson multigrid as its drivers use it
// (benchmarks_2d_multigrid_Poisson_Dirichlet.cpp:15-43): level hierarchy by multigrid::multigrid
// (multigrid.cpp:109-150), operators by init_DirichletBC / init_NeumannBC, zero initial guess,
// v_cycle() (or full_cycle()) until ||rhs - A sol|| / ||rhs|| <= rel_tol.
// rhs and sol are in the x-fastest order of multigrid_base::of.
// hist (optional, max_cycles+1 entries) receives the relative residual before each cycle.
int ref_mg_poisson(int ndim, const int *n, const double *lo, const double *hi, int dirichlet, int full,
                   const double *rhs, double *sol, double rel_tol, int max_cycles, int *cycles, double *hist) {
    Dims d = dims_of(ndim, n);
    structured_grid *geo = make_grid(ndim, n, lo, hi);
    scalar_data *s = make_scalar(d);
    multigrid mg(s, geo);
    for (unsigned l = 0; l < mg.level_num; ++l) {
        if (dirichlet) {
            mg.at[l]->no_compatibility = true;
            mg.at[l]->init_DirichletBC();
        } else {
            mg.at[l]->init_NeumannBC();
        }
        mg.at[l]->sol.setZero();
        mg.at[l]->rhs.setZero();
        mg.at[l]->res.setZero();
        mg.at[l]->buffer.setZero();
    }
    int N = mg.at[0]->n;
    for (int q = 0; q < N; ++q) mg.at[0]->rhs[q] = rhs[q];
    double bnorm = mg.at[0]->rhs.norm();
    int it = 0;
    double rel = mg.at[0]->residual() / bnorm;
    if (hist) hist[0] = rel;
    while (rel > rel_tol && it < max_cycles) {
        if (full) mg.full_cycle();
        else mg.v_cycle();
        ++it;
        rel = mg.at[0]->residual() / bnorm;
        if (hist) hist[it] = rel;
    }
    for (int q = 0; q < N; ++q) sol[q] = mg.at[0]->sol[q];
    *cycles = it;
    return 0;
}

int ref_mg_levels(int ndim, const int *n, int *level_n /* 3 per level */, int max_levels) {
    Dims d = dims_of(ndim, n);
    double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    structured_grid *geo = make_grid(ndim, n, lo, hi);
    scalar_data *s = make_scalar(d);
    multigrid mg(s, geo);
    int L = int(mg.level_num);
    for (int l = 0; l < L && l < max_levels; ++l) {
        level_n[3 * l] = mg.at[l]->nx;
        level_n[3 * l + 1] = mg.at[l]->ny;
        level_n[3 * l + 2] = mg.at[l]->nz;
    }
    return L;
}

// ---------------------------------------------------------------- two-phase state
// A complete two-phase problem built the way the reference drivers build it
// (benchmarks_2d_bubble_rising.cpp:19-89): phi/pressure scalars, vel (staggered) and
// nvel (node) vectors, shared solvers with Neumann multigrid, dummy scratch, one
// runge_kutta and one projection_method.
//
// prm[16]: density_ratio, viscosity_ratio, Re, Fr, We, ls_width, rdt, max_CFL, min_CFL,
//          positive_ref, ppe_tol, ppe_tol2, ppe_max_iter, ppe_omega, ppe_initer, dt0
// opt[5]:  convection scheme (0 uccd, 1 weno5), mpls Euler steps per step,
//          reinit every k steps (0 never), ppe mode (0 reference schedule: projection() for
//          iter<5 then fast_pressure_correction; 1 projection() every step),
//          reinit with the lambda correction (1) or without (0).
struct RefTP {
    Dims d;
    structured_grid *geo;
    wrapper *phi, *vel, *nvel, *pressure;
    runge_kutta *rk;
    projection_method *flow;
    problem_parameters *param;
    shared_solvers *solvers;
    dummy_data *dummy;
    int scheme, n_mpls, reinit_every, ppe_mode, reinit_lambda, step;
    int source_scheme;   // 1: find_source_sec / ab_solve_sec
};

void *ref_tp_create(int ndim, const int *n, const double *lo, const double *hi, const int *vel_bc,
                    const int *scalar_bc, const double *prm, const int *opt) {
    auto *tp = new RefTP{};
    tp->d = dims_of(ndim, n);
    tp->geo = make_grid(ndim, n, lo, hi);
    double zero[6] = {0, 0, 0, 0, 0, 0};
    tp->phi = make_wrapper(true, tp->geo, ndim, scalar_bc, zero);
    tp->pressure = make_wrapper(true, tp->geo, ndim, scalar_bc, zero);
    tp->vel = make_wrapper(false, tp->geo, ndim, vel_bc, zero);
    tp->nvel = make_wrapper(false, tp->geo, ndim, vel_bc, zero);
    tp->rk = new runge_kutta(tp->phi->scalar->Nx, tp->phi->scalar->Ny, tp->phi->scalar->Nz);
    tp->flow = new projection_method(tp->phi->scalar);
    tp->param = new problem_parameters{};
    tp->solvers = SharedSolvers_alloc(tp->phi->scalar, tp->geo);
    shared_solvers_mg_init_Neumann(tp->solvers);
    tp->dummy = dummy_data_alloc(tp->phi->scalar);
    for (wrapper *w : {tp->phi, tp->pressure, tp->vel, tp->nvel}) {
        w->link_params(tp->param);
        w->link_solvers(tp->solvers);
        w->link_dummy(tp->dummy);
    }
    problem_parameters *p = tp->param;
    p->density_ratio = prm[0];
    p->viscosity_ratio = prm[1];
    p->Reynolds_number = prm[2];
    p->Froude_number = prm[3];
    p->Weber_number = prm[4];
    p->ls_width = prm[5];
    p->rdt = prm[6];
    p->max_CFL = prm[7];
    p->min_CFL = prm[8];
    p->positive_ref = prm[9] != 0.0;
    p->ppe_tol = prm[10];
    p->ppe_tol2 = prm[11];
    p->ppe_max_iter = int(prm[12]);
    p->ppe_omega = prm[13];
    p->ppe_initer = int(prm[14]);
    p->dt = prm[15];
    tp->scheme = opt[0];
    tp->n_mpls = opt[1];
    tp->reinit_every = opt[2];
    tp->ppe_mode = opt[3];
    tp->reinit_lambda = opt[4];
    tp->step = 0;
    return tp;
}

static DataType ***tp_field(RefTP *tp, const char *name) {
    std::string s(name);
    if (s == "phi") return tp->phi->scalar->data;
    if (s == "p") return tp->pressure->scalar->data;
    if (s == "p_old") return tp->pressure->scalar->old;
    if (s == "p_old2") return tp->pressure->scalar->old2;
    if (s == "u") return tp->vel->vector->x.data;
    if (s == "v") return tp->vel->vector->y.data;
    if (s == "w") return tp->vel->vector->z.data;
    if (s == "nu") return tp->nvel->vector->x.data;
    if (s == "nv") return tp->nvel->vector->y.data;
    if (s == "nw") return tp->nvel->vector->z.data;
    if (s == "rho") return tp->dummy->density;
    if (s == "mu") return tp->dummy->viscosity;
    if (s == "delta") return tp->dummy->delta;
    if (s == "heaviside") return tp->dummy->heaviside;
    if (s == "curvature") return tp->dummy->curvature;
    if (s == "sign") return tp->dummy->sign;
    if (s == "grad") return tp->dummy->grad;
    if (s == "u_src") return tp->flow->u_src;
    if (s == "v_src") return tp->flow->v_src;
    if (s == "w_src") return tp->flow->w_src;
    if (s == "u_src_old") return tp->flow->u_src_old;
    if (s == "v_src_old") return tp->flow->v_src_old;
    if (s == "w_src_old") return tp->flow->w_src_old;
    if (s == "rhs") return tp->flow->RHS;
    return nullptr;
}

int ref_tp_set(void *h, const char *name, const double *src) {
    auto *tp = static_cast<RefTP *>(h);
    DataType ***a = tp_field(tp, name);
    if (!a) return -1;
    load(a, src, tp->d);
    return 0;
}

int ref_tp_get(void *h, const char *name, double *dst) {
    auto *tp = static_cast<RefTP *>(h);
    DataType ***a = tp_field(tp, name);
    if (!a) return -1;
    save(dst, a, tp->d);
    return 0;
}

// scalars: t, dt, dt_old, dt_old2, iter, stable_CFL, lsf_mass0
int ref_tp_scalars(void *h, double *out) {
    auto *tp = static_cast<RefTP *>(h);
    out[0] = tp->param->t;
    out[1] = tp->param->dt;
    out[2] = tp->param->dt_old;
    out[3] = tp->param->dt_old2;
    out[4] = tp->param->iter;
    out[5] = tp->param->stable_CFL;
    out[6] = tp->param->lsf_mass0;
    return 0;
}

int ref_tp_set_scalars(void *h, const double *in) {
    auto *tp = static_cast<RefTP *>(h);
    tp->param->t = in[0];
    tp->param->dt = in[1];
    tp->param->dt_old = in[2];
    tp->param->dt_old2 = in[3];
    tp->param->iter = int(in[4]);
    tp->param->stable_CFL = in[5];
    tp->param->lsf_mass0 = in[6];
    return 0;
}

// Start-up as in benchmarks_2d_bubble_rising.cpp:51,88-89: scalar BC, find_source, lsf_mass0.
int ref_tp_init(void *h) {
    auto *tp = static_cast<RefTP *>(h);
    tp->phi->apply_scalar_bc();
    tp->flow->find_source(tp->vel, tp->nvel, tp->phi);
    tp->param->lsf_mass0 = lsf_mass(tp->phi);
    return 0;
}

int ref_tp_find_dt(void *h) {
    auto *tp = static_cast<RefTP *>(h);
    find_dt(tp->vel);
    return 0;
}

int ref_tp_advect(void *h) {
    auto *tp = static_cast<RefTP *>(h);
    tp->rk->tvd_rk3(tp->phi, tp->nvel, IDENTITY, tp->scheme == 1 ? convection_weno : convection);
    return 0;
}

int ref_tp_mpls(void *h, int count) {
    auto *tp = static_cast<RefTP *>(h);
    for (int c = 0; c < count; ++c) tp->rk->euler(tp->phi, tp->nvel, IDENTITY, mpls);
    return 0;
}

// Reinitialisation block of benchmarks_2d_bubble_rising.cpp:122-129.  Returns the RK3 steps taken.
int ref_tp_reinit(void *h) {
    auto *tp = static_cast<RefTP *>(h);
    int instep = 0;
    while (instep * tp->param->rdt < 2.0 * tp->param->ls_width) {
        if (instep == 0) find_sign(tp->phi);
        instep++;
        tp->rk->tvd_rk3(tp->phi, tp->nvel, IDENTITY, tp->reinit_lambda ? lsf_redistance_lambda : lsf_redistance_no_lambda);
    }
    return instep;
}

int ref_tp_set_source_scheme(void *h, int scheme) {
    static_cast<RefTP *>(h)->source_scheme = scheme;
    return 0;
}

int ref_tp_find_source(void *h) {
    auto *tp = static_cast<RefTP *>(h);
    if (tp->source_scheme == 1) tp->flow->find_source_sec(tp->vel, tp->nvel, tp->phi);
    else tp->flow->find_source(tp->vel, tp->nvel, tp->phi);
    return 0;
}

int ref_tp_ab_solve(void *h) {
    auto *tp = static_cast<RefTP *>(h);
    const int saved = tp->param->iter;
    if (tp->ppe_mode == 1) tp->param->iter = 0;
    if (tp->source_scheme == 1) tp->flow->ab_solve_sec(tp->vel, tp->nvel, tp->pressure, tp->phi);
    else tp->flow->ab_solve(tp->vel, tp->nvel, tp->pressure, tp->phi);
    if (tp->ppe_mode == 1) tp->param->iter = saved;
    return 0;
}

// init_ppe_proj_coefficients + projection() alone on the current rho, vel and p
// (projection_method.cpp:404-465,544-657).
int ref_tp_projection(void *h) {
    auto *tp = static_cast<RefTP *>(h);
    tp->flow->init_ppe_proj_coefficients(tp->pressure);
    tp->flow->projection(tp->pressure, tp->phi, tp->vel);
    return 0;
}

// One time step of the reference drivers' loop (benchmarks_2d_bubble_rising.cpp:100-130).
int ref_tp_step(void *h, int nsteps) {
    auto *tp = static_cast<RefTP *>(h);
    for (int s = 0; s < nsteps; ++s) {
        find_dt(tp->vel);
        tp->param->t += tp->param->dt;
        tp->param->iter++;
        ref_tp_advect(h);
        ref_tp_mpls(h, tp->n_mpls);
        ref_tp_ab_solve(h);
        tp->step++;
        if (tp->reinit_every > 0 && tp->step % tp->reinit_every == 0) ref_tp_reinit(h);
    }
    return 0;
}

// Diagnostics: lsf_mass, lsf_volume, divergence (wrapper_func.cpp:295-333,450-572).
int ref_tp_diagnostics(void *h, double *out) {
    auto *tp = static_cast<RefTP *>(h);
    out[0] = lsf_mass(tp->phi);
    out[1] = lsf_volume(tp->phi);
    out[2] = divergence(tp->vel);
    return 0;
}

// runge_kutta::tvd_rk3 (runge_kutta.cpp:13-49), nsteps steps, with (identity_flux, convection)
// (flux_kind 0, rhs_kind 0; flux.cpp:7-20, source.cpp:8-40) or (burgers_flux, Hamilton_Jacobi)
// (flux_kind 1, rhs_kind 1; flux.cpp:86-96, source.cpp:75-107), or convection_sec (rhs_kind 2,
// source.cpp:42-73); t/v: the scalar's boundary
// types and values; u/vv/w: the velocity (whole arrays).  vel_from_phi: the velocity's x
// component is a copy of phi before every step, as benchmarks_1d_IBE.cpp does.
int ref_transport_rk3(int ndim, const int *n, const double *lo, const double *hi, const int *t, const double *v,
                      int flux_kind, int rhs_kind, double dt, int nsteps, int vel_from_phi, double *phi,
                      const double *u, const double *vv, const double *w) {
    typedef void (*rhs_fn)(wrapper *, wrapper *, DataType ***, flux_fn);
    Dims d = dims_of(ndim, n);
    structured_grid *geo = make_grid(ndim, n, lo, hi);
    wrapper *f = make_wrapper(true, geo, ndim, t, v);
    wrapper *vel = make_wrapper(false, geo, ndim, t, v);
    auto *param = new problem_parameters{};
    param->dt = dt;
    f->link_params(param);
    f->link_solvers(SharedSolvers_alloc(f->scalar, geo));
    load(f->scalar->data, phi, d);
    load(vel->vector->x.data, u, d);
    load(vel->vector->y.data, vv, d);
    load(vel->vector->z.data, w, d);
    runge_kutta rk(d.Nx, d.Ny, d.Nz);
    const flux_fn flux = flux_kind ? static_cast<flux_fn>(&burgers_flux) : IDENTITY;
    const rhs_fn rhs = rhs_kind == 1   ? static_cast<rhs_fn>(&Hamilton_Jacobi)
                       : rhs_kind == 2 ? static_cast<rhs_fn>(&convection_sec)
                                       : static_cast<rhs_fn>(&convection);
    for (int step = 0; step < nsteps; ++step) {
        if (vel_from_phi)
            for (int i = 0; i < d.Nx; ++i)
                for (int j = 0; j < d.Ny; ++j)
                    for (int k = 0; k < d.Nz; ++k) vel->vector->x.data[i][j][k] = f->scalar->data[i][j][k];
        rk.tvd_rk3(f, vel, flux, rhs);
    }
    save(phi, f->scalar->data, d);
    return 0;
}

// second_order_solver (second_order_solver.cpp:7-241) on flux: upwind 0 -- find_derivatives_all
// (central fx.., fxx.. and the mixed fxy, fyz, fzx); upwind 1 -- find_derivatives(f, vel).
// out: fx, fy, fz, fxx, fyy, fzz, fxy, fyz, fzx (entries a call does not write stay zero).
int ref_sec(int ndim, const int *n, const double *lo, const double *hi, int upwind, const double *flux,
            const double *u, const double *v, const double *w, double *out) {
    Dims d = dims_of(ndim, n);
    size_t N = size_t(d.Nx) * d.Ny * d.Nz;
    structured_grid *geo = make_grid(ndim, n, lo, hi);
    scalar_data *f = make_scalar(d);
    vector_data *vel = make_vector(d);
    load(f->flux, flux, d);
    load(vel->x.data, u, d);
    load(vel->y.data, v, d);
    load(vel->z.data, w, d);
    second_order_solver sec(geo->dx, geo->dy, geo->dz);
    if (upwind) sec.find_derivatives(f, vel);
    else sec.find_derivatives_all(f);
    DataType ***o[9] = {f->fx, f->fy, f->fz, f->fxx, f->fyy, f->fzz, f->fxy, f->fyz, f->fzx};
    for (int m = 0; m < 9; ++m) save(out + m * N, o[m], d);
    return 0;
}

// vtkWriter (vtkWriter.cpp:13-111): <prefix>0.vtk with a scalar, a raw array as a scalar, a
// vector and three raw arrays as a vector, on the grid [-0.5, 1.5] x [0.25, 2.0] (x [0, 1]);
// f, u, v, w: ghosted [Nx][Ny][Nz] arrays.
int ref_vtk_write(int ndim, const int *n, const double *f_in, const double *u, const double *v, const double *w,
                  const char *prefix) {
    Dims d = dims_of(ndim, n);
    const double lo[3] = {-0.5, 0.25, 0.0}, hi[3] = {1.5, 2.0, 1.0};
    structured_grid *geo = make_grid(ndim, n, lo, hi);
    scalar_data *f = make_scalar(d);
    vector_data *vel = make_vector(d);
    load(f->data, f_in, d);
    load(vel->x.data, u, d);
    load(vel->y.data, v, d);
    load(vel->z.data, w, d);
    vtkWriter vtk(geo, prefix);
    vtk.create(0);
    vtk.add_scalar(f, "phi");
    vtk.add_scalar(vel->x.data, f, "u_as_scalar");
    vtk.add_vector(vel, "vel");
    vtk.add_vector(vel->z.data, vel->y.data, vel->x.data, vel, "vel_swapped");
    vtk.close();
    return 0;
}

}  // extern "C"
