// scihpc_cpp.cpp -- the reference's C++ API for the two-phase projection step (structured_grid,
// scalar_data / vector_data, wrapper with bc_factory objects, runge_kutta, projection_method,
// the wrapper_func reductions, vtkWriter), implemented over the C ABI of scihpc_gpu.h.
//
// Device state.  The wrappers linked to one problem_parameters object form one problem; its
// GPU session (one scihpc_twophase) is created by the first stage call that names the level
// set and the velocities (projection_method::find_source / ab_solve, runge_kutta, find_dt).
// At creation the host arrays of phi, the face velocity, the node velocity and (when known)
// the pressure are uploaded; from then on the GPU holds the current values.  The scalar
// parameters that drivers change on the host between stages (t, iter, lsf_mass0, dt ...)
// are pushed before every stage and read back after it.  Host arrays are refreshed by
// scihpc_sync_to_host and before every VTK write.
//
// Errors: the reference reports nothing (asserts only); here every failing call records a
// status (scihpc_cpp_last_status) and prints the C ABI's message once.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "scihpc/bc_factory.h"
#include "scihpc/ccd_solver.h"
#include "scihpc/dummy_data.h"
#include "scihpc/flux.h"
#include "scihpc/global.h"
#include "scihpc/godunov_gradient.h"
#include "scihpc/gpu_session.h"
#include "scihpc/lsm.h"
#include "scihpc/multigrid.h"
#include "scihpc/projection_method.h"
#include "scihpc/runge_kutta.h"
#include "scihpc/scalar_data.h"
#include "scihpc/shared_solvers.h"
#include "scihpc/source.h"
#include "scihpc/structured_grid.h"
#include "scihpc/uccd_solver.h"
#include "scihpc/vector_data.h"
#include "scihpc/vtkWriter.h"
#include "scihpc/weno_solver.h"
#include "scihpc/wrapper.h"
#include "scihpc/wrapper_func.h"
#include "scihpc_gpu.h"

// ---------------------------------------------------------------- status
namespace {
int g_status = 0;
std::string g_message;
int g_pressure_fp32 = 1;
// pressure schedule and tolerance of sessions (scihpc_cpp_set_pressure_schedule): the
// reference's ab_solve schedule with its absolute residual test by default
int g_schedule = 1, g_tol_mode = 1;

void fail(int code, const std::string &msg) {
    g_status = code;
    g_message = msg;
    std::fprintf(stderr, "scihpc_gb300: %s\n", msg.c_str());
}

bool check(int rc, const char *what) {
    if (rc == SCIHPC_OK) return true;
    fail(rc, std::string(what) + ": " + scihpc_last_error());
    return false;
}

bool check_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    fail(SCIHPC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

size_t cells_of(const scalar_data *f) { return size_t(f->Nx) * size_t(f->Ny) * size_t(f->Nz); }
DataType *base_of(DataType ***a) { return a[0][0]; }   // init_array storage is contiguous
}  // namespace

int scihpc_cpp_last_status() { return g_status; }
const char *scihpc_cpp_last_message() { return g_message.c_str(); }
void scihpc_cpp_set_pressure_precision(int fp32) { g_pressure_fp32 = fp32 ? 1 : 0; }
void scihpc_cpp_set_pressure_schedule(int schedule, int tol_mode) {
    g_schedule = schedule ? 1 : 0;
    g_tol_mode = tol_mode ? 1 : 0;
}

// ---------------------------------------------------------------- global.h
DataType ***init_array(int Nx, int Ny, int Nz) {
    auto *block = new DataType[size_t(Nx) * Ny * Nz]();
    auto **rows = new DataType *[size_t(Nx) * Ny];
    auto ***arr = new DataType **[Nx];
    for (int i = 0; i < Nx; ++i) {
        arr[i] = rows + size_t(i) * Ny;
        for (int j = 0; j < Ny; ++j) arr[i][j] = block + (size_t(i) * Ny + j) * Nz;
    }
    return arr;
}

void delete3d(DataType ***arr, int, int) {
    if (!arr) return;
    delete[] arr[0][0];
    delete[] arr[0];
    delete[] arr;
}

// Nondimensionalisation of global.cpp:31-52: length scale L, velocity sqrt(g L) or given.
problem_parameters *set_parameters(DataType rho1, DataType rho2, DataType mu1, DataType mu2, DataType sigma,
                                   DataType g, DataType L, DataType U) {
    auto *p = new problem_parameters();
    p->density_ratio = rho2 / rho1;
    p->viscosity_ratio = mu2 / mu1;
    p->Lc = L;
    p->Uc = U;
    p->Tc = L / U;
    p->Reynolds_number = rho1 * U * L / mu1;
    p->Froude_number = U / std::sqrt(g * L);
    p->Weber_number = rho1 * U * U * L / sigma;
    return p;
}

problem_parameters *set_parameters(DataType rho1, DataType rho2, DataType mu1, DataType mu2, DataType sigma,
                                   DataType g, DataType L) {
    return set_parameters(rho1, rho2, mu1, mu2, sigma, g, L, std::sqrt(g * L));
}

// air and water at 20 C (global.cpp:72-80)
problem_parameters *set_air_water(DataType L) { return set_parameters(1000.0, 1.226, 1.137e-3, 1.78e-5, 0.0728, 9.81, L); }
problem_parameters *set_air_water(DataType L, DataType U) {
    return set_parameters(1000.0, 1.226, 1.137e-3, 1.78e-5, 0.0728, 9.81, L, U);
}

// ---------------------------------------------------------------- structured_grid
// Node coordinates x_i = start + i dx, centres x_i + dx/2, h = min spacing, dv = cell
// volume (structured_grid.cpp:7-134).
namespace {
void grid_axis(const axis &a, DataType *&x, DataType *&xc, DataType &d) {
    d = (a.end - a.start) / static_cast<DataType>(a.n);
    x = new DataType[a.n + 1];
    xc = new DataType[a.n];
    for (int i = 0; i <= a.n; ++i) {
        x[i] = a.start + static_cast<DataType>(i * d);
        if (i < a.n) xc[i] = x[i] + static_cast<DataType>(0.5 * d);
    }
}
void grid_unused(DataType *&x, DataType *&xc, DataType &d) {
    x = new DataType[1]();
    xc = new DataType[1]();
    d = 0.0;
}
}  // namespace

structured_grid::structured_grid(axis xa) {
    grid_axis(xa, x, xc, dx);
    grid_unused(y, yc, dy);
    grid_unused(z, zc, dz);
    h = dx;
    dv = dx;
    ndim = 1;
    x_axis = xa;
    y_axis = axis{0.0, 0.0, 1};
    z_axis = axis{0.0, 0.0, 1};
    vtk_info = {xa.start, 0.0, 0.0, xa.n + 1, 1, 1};
}

structured_grid::structured_grid(axis xa, axis ya) {
    grid_axis(xa, x, xc, dx);
    grid_axis(ya, y, yc, dy);
    grid_unused(z, zc, dz);
    h = std::fmin(dx, dy);
    dv = dx * dy;
    ndim = 2;
    x_axis = xa;
    y_axis = ya;
    z_axis = axis{0.0, 0.0, 1};
    vtk_info = {xa.start, ya.start, 0.0, xa.n + 1, ya.n + 1, 1};
}

structured_grid::structured_grid(axis xa, axis ya, axis za) {
    grid_axis(xa, x, xc, dx);
    grid_axis(ya, y, yc, dy);
    grid_axis(za, z, zc, dz);
    h = std::fmin(dx, std::fmin(dy, dz));
    dv = dx * dy * dz;
    ndim = 3;
    x_axis = xa;
    y_axis = ya;
    z_axis = za;
    vtk_info = {xa.start, ya.start, za.start, xa.n + 1, ya.n + 1, za.n + 1};
}

// ---------------------------------------------------------------- scalar_data / vector_data
void scalar_data::alloc() {
    DataType ****all[] = {&data, &flux, &old, &old2, &fx, &fy, &fz, &fxx, &fyy, &fzz, &fxy, &fyz, &fzx};
    for (auto *a : all) *a = init_array(Nx, Ny, Nz);
}

scalar_data::scalar_data(int _nx) : Nx(_nx + 2 * 3), Ny(1), Nz(1), nx(_nx), ny(1), nz(1), ndim(1) { alloc(); }
scalar_data::scalar_data(int _nx, int _ny)
    : Nx(_nx + 2 * 3), Ny(_ny + 2 * 3), Nz(1), nx(_nx), ny(_ny), nz(1), ndim(2) {
    alloc();
}
scalar_data::scalar_data(int _nx, int _ny, int _nz)
    : Nx(_nx + 2 * 3), Ny(_ny + 2 * 3), Nz(_nz + 2 * 3), nx(_nx), ny(_ny), nz(_nz), ndim(3) {
    alloc();
}

// 1-based interior index -> array index; axes of extent 1 are not ghosted (scalar_data.cpp:95-123)
indices scalar_data::index_mapping(int i, int j, int k) {
    indices r{i - 1, j - 1, k - 1};
    if (nx > 1) r.i += ghc;
    if (ny > 1) r.j += ghc;
    if (nz > 1) r.k += ghc;
    return r;
}

namespace {
bool session_store(const scalar_data *f);
}

// old2 <- old <- data (scalar_data.cpp:125-135); a pressure held by a GPU session moves its
// history on the device too (pressure_guess_solution reads it there)
void scalar_data::store() const {
    if (session_store(this)) return;
    const size_t n = cells_of(this);
    std::memcpy(base_of(old2), base_of(old), n * sizeof(DataType));
    std::memcpy(base_of(old), base_of(data), n * sizeof(DataType));
}

vector_data::vector_data(int _nx) : x(_nx), y(_nx), z(_nx) {}
vector_data::vector_data(int _nx, int _ny) : x(_nx, _ny), y(_nx, _ny), z(_nx, _ny) {}
vector_data::vector_data(int _nx, int _ny, int _nz) : x(_nx, _ny, _nz), y(_nx, _ny, _nz), z(_nx, _ny, _nz) {}
void vector_data::store() {
    x.store();
    y.store();
    z.store();
}

// ---------------------------------------------------------------- GPU sessions
namespace {
struct Session;

// where a host array lives on the GPU: a session field by name
struct Mirror {
    Session *s;
    std::string name;
};

struct Session {
    scihpc_twophase *tp = nullptr;
    problem_parameters *params = nullptr;
    wrapper *phi = nullptr, *vel = nullptr, *nvel = nullptr, *pressure = nullptr;
    int scheme = -1;
};

std::map<problem_parameters *, Session *> g_sessions;
std::map<DataType ***, Mirror> g_mirrors;   // host array -> session field

int code_of(const std::string &t) {
    if (t == PERIODIC) return 0;
    if (t == NEUMANN) return 1;
    if (t == NO_SLIP) return 2;
    if (t == SLIP) return 3;
    if (t == DIRICHLET) return 4;
    return -1;
}

scihpc_grid grid_of(const structured_grid *g) {
    scihpc_grid c{};
    c.ndim = g->ndim;
    const axis ax[3] = {g->x_axis, g->y_axis, g->z_axis};
    for (int a = 0; a < 3; ++a) {
        c.n[a] = a < g->ndim ? ax[a].n : 1;
        c.lo[a] = a < g->ndim ? ax[a].start : 0.0;
        c.hi[a] = a < g->ndim ? ax[a].end : 1.0;
    }
    return c;
}

bool upload(Session *s, const char *name, DataType ***a) {
    return check(scihpc_twophase_upload(s->tp, name, base_of(a)), "upload");
}

bool download(Session *s, const char *name, DataType ***a) {
    return check(scihpc_twophase_download(s->tp, name, base_of(a)), "download");
}

void attach_dummy(Session *s, dummy_data *d) {
    if (!d) return;
    const std::pair<DataType ***, const char *> m[] = {{d->heaviside, "heaviside"}, {d->delta, "delta"},
                                                       {d->sign, "sign"},           {d->grad, "grad"},
                                                       {d->curvature, "curvature"}, {d->density, "rho"},
                                                       {d->viscosity, "mu"}};
    for (auto &e : m) g_mirrors[e.first] = Mirror{s, e.second};
}

bool attach_pressure(Session *s, wrapper *p) {
    if (!p || s->pressure == p) return true;
    s->pressure = p;
    g_mirrors[p->scalar->data] = Mirror{s, "p"};
    return upload(s, "p", p->scalar->data);
}

// scalar_data::store of a pressure held by a session: the shift old2 <- old <- data on the
// device arrays, and the host arrays brought up to date with them
bool session_store(const scalar_data *f) {
    auto it = g_mirrors.find(f->data);
    if (it == g_mirrors.end() || it->second.name != "p") return false;
    Session *s = it->second.s;
    const size_t n = cells_of(f);
    if (!download(s, "p", f->data) || !download(s, "p_old", f->old)) return true;
    std::memcpy(base_of(f->old2), base_of(f->old), n * sizeof(DataType));
    std::memcpy(base_of(f->old), base_of(f->data), n * sizeof(DataType));
    upload(s, "p_old", f->old) && upload(s, "p_old2", f->old2);
    return true;
}

// host scalars -> device (the drivers advance t and iter and set lsf_mass0 on the host)
bool push_scalars(Session *s) {
    const problem_parameters *p = s->params;
    const double v[7] = {p->t, p->dt, p->dt_old, p->dt_old2, double(p->iter), p->stable_CFL, p->lsf_mass0};
    return check(scihpc_twophase_set_scalars(s->tp, v), "set_scalars");
}

bool pull_scalars(Session *s) {
    double v[7];
    if (!check(scihpc_twophase_get_scalars(s->tp, v), "get_scalars")) return false;
    problem_parameters *p = s->params;
    p->t = v[0];
    p->dt = v[1];
    p->dt_old = v[2];
    p->dt_old2 = v[3];
    p->iter = int(v[4]);
    p->stable_CFL = v[5];
    p->lsf_mass0 = v[6];
    return true;
}

// The session of the problem phi belongs to, created on first use.
Session *session_for(wrapper *phi, wrapper *vel, wrapper *nvel, wrapper *pressure) {
    if (!phi || !phi->is_scalar || !phi->params) {
        fail(SCIHPC_ERR_ARG, "the level-set wrapper must be a scalar wrapper linked to problem_parameters");
        return nullptr;
    }
    auto it = g_sessions.find(phi->params);
    if (it != g_sessions.end()) {
        Session *s = it->second;
        if (pressure && !attach_pressure(s, pressure)) return nullptr;
        return s;
    }
    if (!vel || vel->is_scalar || !nvel || nvel->is_scalar) {
        fail(SCIHPC_ERR_ARG, "the first stage call must name the face and node velocity wrappers");
        return nullptr;
    }
    auto *s = new Session();
    s->params = phi->params;
    s->phi = phi;
    s->vel = vel;
    s->nvel = nvel;
    const problem_parameters *p = phi->params;
    const scihpc_grid g = grid_of(phi->geo);
    int vbc[6], sbc[6];
    double vals[6];
    vel->bcFactory->codes(vbc, vals);
    phi->bcFactory->codes(sbc, vals);
    const double prm[16] = {p->density_ratio,  p->viscosity_ratio, p->Reynolds_number, p->Froude_number,
                            p->Weber_number,   p->ls_width,        p->rdt,             p->max_CFL,
                            p->min_CFL,        double(p->positive_ref), p->ppe_tol,     p->ppe_tol2,
                            double(p->ppe_max_iter), p->ppe_omega, double(p->ppe_initer), p->dt};
    const int opt[5] = {0, 0, 0, g_pressure_fp32, 1};
    if (!check(scihpc_twophase_create(&g, vbc, sbc, prm, opt, &s->tp), "twophase_create")) {
        delete s;
        return nullptr;
    }
    if (!check(scihpc_twophase_set_ppe_schedule(s->tp, g_schedule, g_tol_mode), "set_ppe_schedule")) {
        scihpc_twophase_destroy(s->tp);
        delete s;
        return nullptr;
    }
    s->scheme = 0;
    const char *vn[3] = {"u", "v", "w"}, *nn[3] = {"nu", "nv", "nw"};
    scalar_data *vc[3] = {&vel->vector->x, &vel->vector->y, &vel->vector->z};
    scalar_data *nc[3] = {&nvel->vector->x, &nvel->vector->y, &nvel->vector->z};
    bool ok = upload(s, "phi", phi->scalar->data);
    g_mirrors[phi->scalar->data] = Mirror{s, "phi"};
    for (int a = 0; a < g.ndim; ++a) {
        ok = ok && upload(s, vn[a], vc[a]->data) && upload(s, nn[a], nc[a]->data);
        g_mirrors[vc[a]->data] = Mirror{s, vn[a]};
        g_mirrors[nc[a]->data] = Mirror{s, nn[a]};
    }
    attach_dummy(s, phi->dummy);
    g_sessions[phi->params] = s;
    if (ok && pressure) ok = attach_pressure(s, pressure);
    return ok ? s : nullptr;
}

Session *session_of(wrapper *any) {
    if (!any || !any->params) return nullptr;
    auto it = g_sessions.find(any->params);
    return it == g_sessions.end() ? nullptr : it->second;
}

void sync_array(DataType ***a) {
    auto it = g_mirrors.find(a);
    if (it != g_mirrors.end()) download(it->second.s, it->second.name.c_str(), a);
}

// Device fill of one host field before a session owns it: a scratch context per grid.
struct Scratch {
    scihpc_ctx *ctx = nullptr;
    double *dev = nullptr;
    size_t cells = 0;
};
std::map<std::vector<double>, Scratch> g_scratch;

void host_fill(const structured_grid *geo, scalar_data *f, int location, const bc_factory *bf) {
    const scihpc_grid g = grid_of(geo);
    std::vector<double> key = {double(g.ndim)};
    for (int a = 0; a < 3; ++a) key.insert(key.end(), {double(g.n[a]), g.lo[a], g.hi[a]});
    Scratch &sc = g_scratch[key];
    const size_t n = cells_of(f);
    if (!sc.ctx && !check(scihpc_ctx_create(&g, &sc.ctx), "ctx_create")) return;
    if (sc.cells < n) {
        if (sc.dev) cudaFree(sc.dev);
        sc.dev = nullptr;
        if (!check_cuda(cudaMalloc(&sc.dev, n * sizeof(double)), "cudaMalloc")) return;
        sc.cells = n;
    }
    int types[6];
    double vals[6];
    bf->codes(types, vals);
    if (!check_cuda(cudaMemcpy(sc.dev, base_of(f->data), n * sizeof(double), cudaMemcpyHostToDevice), "upload"))
        return;
    if (!check(scihpc_bc_fill(sc.ctx, location, types, vals, sc.dev, nullptr), "bc_fill")) return;
    check_cuda(cudaMemcpy(base_of(f->data), sc.dev, n * sizeof(double), cudaMemcpyDeviceToHost), "download");
}

// A fill of a field a session owns runs on the session's device copy.
bool session_fill(scalar_data *f, int location, const bc_factory *bf) {
    auto it = g_mirrors.find(f->data);
    if (it == g_mirrors.end()) return false;
    Session *s = it->second.s;
    double *dev = nullptr;
    if (!check(scihpc_twophase_field(s->tp, it->second.name.c_str(), &dev), "field")) return true;
    int types[6];
    double vals[6];
    bf->codes(types, vals);
    scihpc_ctx *ctx = nullptr;
    const scihpc_grid g = grid_of(bf->geo);
    std::vector<double> key = {double(g.ndim)};
    for (int a = 0; a < 3; ++a) key.insert(key.end(), {double(g.n[a]), g.lo[a], g.hi[a]});
    Scratch &sc = g_scratch[key];
    if (!sc.ctx && !check(scihpc_ctx_create(&g, &sc.ctx), "ctx_create")) return true;
    ctx = sc.ctx;
    void *stream = nullptr;
    check(scihpc_twophase_stream(s->tp, &stream), "stream");
    check(scihpc_bc_fill(ctx, location, types, vals, dev, stream), "bc_fill");
    check_cuda(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "sync");
    return true;
}
}  // namespace

void scihpc_sync_to_host(wrapper *w) {
    if (!w) return;
    if (w->is_scalar) {
        sync_array(w->scalar->data);
    } else {
        sync_array(w->vector->x.data);
        sync_array(w->vector->y.data);
        sync_array(w->vector->z.data);
    }
    if (w->dummy) {
        DataType ***d[] = {w->dummy->heaviside, w->dummy->delta,     w->dummy->sign,   w->dummy->grad,
                           w->dummy->curvature, w->dummy->density,   w->dummy->viscosity};
        for (auto *a : d) sync_array(a);
    }
}

void scihpc_sync_to_device(wrapper *w) {
    if (!w) return;
    auto up = [](DataType ***a) {
        auto it = g_mirrors.find(a);
        if (it != g_mirrors.end()) upload(it->second.s, it->second.name.c_str(), a);
    };
    if (w->is_scalar) {
        up(w->scalar->data);
    } else {
        up(w->vector->x.data);
        up(w->vector->y.data);
        up(w->vector->z.data);
    }
}

// ---------------------------------------------------------------- bc_factory / wrapper
bc_factory::bc_factory(structured_grid *g, const bc_info &xl, const bc_info &xr)
    : xlbc(xl), xrbc(xr), ylbc(xl), yrbc(xr), zlbc(xl), zrbc(xr), dx(g->dx), dy(g->dy), dz(g->dz), geo(g) {}
bc_factory::bc_factory(structured_grid *g, const bc_info &xl, const bc_info &xr, const bc_info &yl, const bc_info &yr)
    : xlbc(xl), xrbc(xr), ylbc(yl), yrbc(yr), zlbc(yl), zrbc(yr), dx(g->dx), dy(g->dy), dz(g->dz), geo(g) {}
bc_factory::bc_factory(structured_grid *g, const bc_info &xl, const bc_info &xr, const bc_info &yl, const bc_info &yr,
                       const bc_info &zl, const bc_info &zr)
    : xlbc(xl), xrbc(xr), ylbc(yl), yrbc(yr), zlbc(zl), zrbc(zr), dx(g->dx), dy(g->dy), dz(g->dz), geo(g) {}

void bc_factory::codes(int types[6], double values[6]) const {
    const bc_info *b[6] = {&xlbc, &xrbc, &ylbc, &yrbc, &zlbc, &zrbc};
    for (int f = 0; f < 6; ++f) {
        types[f] = code_of(b[f]->type);
        values[f] = b[f]->value;
    }
}

namespace {
void fill_at(bc_factory *bf, scalar_data *f, int location) {
    if (!session_fill(f, location, bf)) host_fill(bf->geo, f, location, bf);
}
}  // namespace

void bc_factory::apply_node_centered(scalar_data *f) { fill_at(this, f, 0); }
void bc_factory::apply_node_staggered_x(scalar_data *f) { fill_at(this, f, 1); }
void bc_factory::apply_node_staggered_y(scalar_data *f) { fill_at(this, f, 2); }
void bc_factory::apply_node_staggered_z(scalar_data *f) { fill_at(this, f, 3); }

void wrapper::make_factories(const bc_info *b, int nb) {
    auto make = [&]() -> bc_factory * {
        if (nb == 2) return new bc_factory(geo, b[0], b[1]);
        if (nb == 4) return new bc_factory(geo, b[0], b[1], b[2], b[3]);
        return new bc_factory(geo, b[0], b[1], b[2], b[3], b[4], b[5]);
    };
    bcFactory = make();   // as given (for a vector: the faces of the problem, used by the session)
    bcFactoryU = bcFactoryV = bcFactoryW = nullptr;
    const int n[3] = {geo->x_axis.n, geo->y_axis.n, geo->z_axis.n};
    if (is_scalar) {
        scalar = nb == 2 ? new scalar_data(n[0]) : nb == 4 ? new scalar_data(n[0], n[1]) : new scalar_data(n[0], n[1], n[2]);
        vector = nullptr;
        return;
    }
    vector = nb == 2 ? new vector_data(n[0]) : nb == 4 ? new vector_data(n[0], n[1]) : new vector_data(n[0], n[1], n[2]);
    scalar = nullptr;
    bcFactoryU = make();
    bcFactoryV = make();
    bcFactoryW = make();
    // the wall-normal component of a slip wall is a no-slip (zero) wall (wrapper.cpp:159-181)
    if (b[0].type == SLIP) bcFactoryU->xlbc.type = NO_SLIP;
    if (b[1].type == SLIP) bcFactoryU->xrbc.type = NO_SLIP;
    if (nb >= 4 && b[2].type == SLIP) bcFactoryV->ylbc.type = NO_SLIP;
    if (nb >= 4 && b[3].type == SLIP) bcFactoryV->yrbc.type = NO_SLIP;
    if (nb >= 6 && b[4].type == SLIP) bcFactoryW->zlbc.type = NO_SLIP;
    if (nb >= 6 && b[5].type == SLIP) bcFactoryW->zrbc.type = NO_SLIP;
}

wrapper::wrapper(bool s, structured_grid *g, const bc_info &xl, const bc_info &xr) : is_scalar(s), geo(g) {
    const bc_info b[2] = {xl, xr};
    make_factories(b, 2);
}
wrapper::wrapper(bool s, structured_grid *g, const bc_info &xl, const bc_info &xr, const bc_info &yl, const bc_info &yr)
    : is_scalar(s), geo(g) {
    const bc_info b[4] = {xl, xr, yl, yr};
    make_factories(b, 4);
}
wrapper::wrapper(bool s, structured_grid *g, const bc_info &xl, const bc_info &xr, const bc_info &yl, const bc_info &yr,
                 const bc_info &zl, const bc_info &zr)
    : is_scalar(s), geo(g) {
    const bc_info b[6] = {xl, xr, yl, yr, zl, zr};
    make_factories(b, 6);
}

void wrapper::link_solvers(shared_solvers *s) { solvers = s; }
void wrapper::link_params(problem_parameters *p) { params = p; }
void wrapper::link_dummy(dummy_data *d) {
    dummy = d;
    if (Session *s = session_of(this)) attach_dummy(s, d);
}

void wrapper::apply_vel_bc() const {
    bcFactoryU->apply_node_staggered_x(&vector->x);
    bcFactoryV->apply_node_staggered_y(&vector->y);
    if (geo->ndim == 3) bcFactoryW->apply_node_staggered_z(&vector->z);
}
void wrapper::apply_nvel_bc() const {
    bcFactoryU->apply_node_centered(&vector->x);
    bcFactoryV->apply_node_centered(&vector->y);
    if (geo->ndim == 3) bcFactoryW->apply_node_centered(&vector->z);
}
void wrapper::apply_scalar_bc() const { bcFactory->apply_node_centered(scalar); }
void wrapper::apply_vel_x_bc() const {
    bcFactoryU->apply_node_staggered_x(&vector->x);
    bcFactoryV->apply_node_staggered_x(&vector->y);
    if (geo->ndim == 3) bcFactoryW->apply_node_staggered_x(&vector->z);
}
void wrapper::apply_vel_y_bc() const {
    bcFactoryU->apply_node_staggered_y(&vector->x);
    bcFactoryV->apply_node_staggered_y(&vector->y);
    if (geo->ndim == 3) bcFactoryW->apply_node_staggered_y(&vector->z);
}
void wrapper::apply_vel_z_bc() const {
    bcFactoryU->apply_node_staggered_z(&vector->x);
    bcFactoryV->apply_node_staggered_z(&vector->y);
    bcFactoryW->apply_node_staggered_z(&vector->z);
}

// ---------------------------------------------------------------- multigrid
DataType VectorX::norm() const {
    DataType s = 0.0;
    for (DataType x : v_) s += x * x;
    return std::sqrt(s);
}

multigrid_base::multigrid_base(int _nx, int _ny, int _degree, DataType _dx, DataType _dy)
    : nx(_nx), ny(_ny), nz(1), degree(_degree), ndim(2), n(_nx * _ny), dx(_dx), dy(_dy), dz(0.0) {
    rhs.resize(n), sol.resize(n), res.resize(n), buffer.resize(n);
}

multigrid_base::multigrid_base(int _nx, int _ny, int _nz, int _degree, DataType _dx, DataType _dy, DataType _dz)
    : nx(_nx), ny(_ny), nz(_nz), degree(_degree), ndim(3), n(_nx * _ny * _nz), dx(_dx), dy(_dy), dz(_dz) {
    rhs.resize(n), sol.resize(n), res.resize(n), buffer.resize(n);
}

int multigrid_base::of(int i, int j, int k) { return i + j * nx + k * nx * ny; }
int multigrid_base::of(int i, int j) { return i + j * nx; }

namespace {
void select_bc(multigrid_base *b, int code) {
    multigrid *m = b->owner;
    if (!m || b->level != 0 || m->bc == code) return;
    m->bc = code;
    if (m->gpu) {   // the operator changed: rebuild at the next cycle
        scihpc_poisson_destroy(m->gpu);
        m->gpu = nullptr;
    }
}
// recorded in the status; printed once per kind (drivers call these in their cycle loops)
void internal(const char *what) {
    static std::map<std::string, bool> said;
    const std::string msg = std::string(what) + ": the coarse levels and their transfers live inside the GPU cycle";
    g_status = SCIHPC_ERR_UNSUPPORTED;
    g_message = msg;
    if (!said[what]) std::fprintf(stderr, "scihpc_gb300: %s\n", msg.c_str());
    said[what] = true;
}
}  // namespace

void multigrid_base::init_NeumannBC() { select_bc(this, 0); }
void multigrid_base::init_DirichletBC() { select_bc(this, 1); }

// the mean removal of multigrid_base.cpp:47-67 (a host vector the caller owns)
void multigrid_base::compatibility_condition(VectorX &f) {
    if (no_compatibility || f.size() == 0) return;
    DataType s = 0.0;
    for (long i = 0; i < f.size(); ++i) s += f[i];
    s /= DataType(f.size());
    for (long i = 0; i < f.size(); ++i) f[i] -= s;
}

void multigrid_base::relax(int iter) {
    if (level != 0 || !owner) return internal("multigrid_base::relax on a coarse level");
    owner->iterate(iter);
}

DataType multigrid_base::residual() {
    if (level != 0 || !owner) {
        internal("multigrid_base::residual on a coarse level");
        return 0.0;
    }
    double r = 0.0;
    owner->residual(r);
    return r;
}

void multigrid_base::Ax(const VectorX &) { internal("multigrid_base::Ax"); }
void multigrid_base::restriction(multigrid_base *) { internal("multigrid_base::restriction"); }
void multigrid_base::prolongation(multigrid_base *) { internal("multigrid_base::prolongation"); }
void multigrid_base::solve() { internal("multigrid_base::solve"); }

// one coarsening step of multigrid.cpp:10-41: halve if every halved extent stays above 3,
// else divide by 3 likewise; returns the ratio (1: no further level)
int multigrid::check2d(std::vector<int> &nx, std::vector<int> &ny) {
    for (int r : {2, 3}) {
        const int a = nx.back(), b = ny.back();
        if (a % r == 0 && b % r == 0 && a / r > 3 && b / r > 3) {
            nx.push_back(a / r), ny.push_back(b / r);
            return r;
        }
    }
    return 1;
}

int multigrid::check3d(std::vector<int> &nx, std::vector<int> &ny, std::vector<int> &nz) {
    for (int r : {2, 3}) {
        const int a = nx.back(), b = ny.back(), c = nz.back();
        if (a % r == 0 && b % r == 0 && c % r == 0 && a / r > 3 && b / r > 3 && c / r > 3) {
            nx.push_back(a / r), ny.push_back(b / r), nz.push_back(c / r);
            return r;
        }
    }
    return 1;
}

multigrid::multigrid(scalar_data *var, structured_grid *g) : geo(g) {
    std::vector<int> nx{var->nx}, ny{var->ny}, nz{var->nz};
    while ((var->ndim == 3 ? check3d(nx, ny, nz) : check2d(nx, ny)) > 1) {
    }
    level_num = unsigned(nx.size());
    at = new multigrid_base *[level_num];
    for (unsigned l = 0; l < level_num; ++l) {
        const int deg = nx[0] / nx[l];
        if (var->ndim == 3)
            at[l] = new multigrid_base(nx[l], ny[l], nz[l], deg, g->dx * deg, g->dy * deg, g->dz * deg);
        else
            at[l] = new multigrid_base(nx[l], ny[l], deg, g->dx * deg, g->dy * deg);
        at[l]->owner = this;
        at[l]->level = int(l);
    }
}

namespace {
// interior vector (x fastest) <-> ghosted device field ([i][j][k], k fastest, ghost width 3)
void to_ghosted(const multigrid_base *b, const VectorX &v, std::vector<double> &out) {
    const int N1 = b->ny + 6, N2 = b->ndim == 3 ? b->nz + 6 : 1, g2 = b->ndim == 3 ? 3 : 0;
    out.assign(size_t(b->nx + 6) * N1 * N2, 0.0);
    for (int k = 0; k < b->nz; ++k)
        for (int j = 0; j < b->ny; ++j)
            for (int i = 0; i < b->nx; ++i)
                out[(size_t(i + 3) * N1 + (j + 3)) * N2 + (k + g2)] = v[i + j * b->nx + k * b->nx * b->ny];
}
void from_ghosted(const multigrid_base *b, const std::vector<double> &in, VectorX &v) {
    const int N1 = b->ny + 6, N2 = b->ndim == 3 ? b->nz + 6 : 1, g2 = b->ndim == 3 ? 3 : 0;
    for (int k = 0; k < b->nz; ++k)
        for (int j = 0; j < b->ny; ++j)
            for (int i = 0; i < b->nx; ++i)
                v[i + j * b->nx + k * b->nx * b->ny] = in[(size_t(i + 3) * N1 + (j + 3)) * N2 + (k + g2)];
}

bool mg_upload(multigrid *m) {
    multigrid_base *f = m->at[0];
    const scihpc_grid g = grid_of(m->geo);
    if (!m->gpu) {
        if (!check(scihpc_poisson_create(&g, m->bc, 0, g_pressure_fp32, &m->gpu), "poisson_create")) return false;
        const size_t cells = size_t(f->nx + 6) * (f->ny + 6) * (f->ndim == 3 ? f->nz + 6 : 1);
        if (!m->d_rhs && (!check_cuda(cudaMalloc(&m->d_rhs, cells * sizeof(double)), "cudaMalloc") ||
                          !check_cuda(cudaMalloc(&m->d_p, cells * sizeof(double)), "cudaMalloc")))
            return false;
    }
    std::vector<double> h;
    to_ghosted(f, f->rhs, h);
    if (!check_cuda(cudaMemcpy(m->d_rhs, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice), "upload"))
        return false;
    to_ghosted(f, f->sol, h);
    return check_cuda(cudaMemcpy(m->d_p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice), "upload");
}
}  // namespace

bool multigrid::iterate(int iters) {
    if (iters <= 0) return true;
    if (!mg_upload(this)) return false;
    int it = 0;
    double rr = 0.0;
    // a relative tolerance no residual reaches: exactly `iters` iterations (fewer if the
    // residual stops improving)
    const int rc = scihpc_poisson_solve(gpu, d_rhs, d_p, 1, 1e-300, iters, &it, &rr, nullptr);
    if (rc != SCIHPC_OK && rc != SCIHPC_ERR_MAXITER && !check(rc, "poisson_solve")) return false;
    multigrid_base *f = at[0];
    std::vector<double> h(size_t(f->nx + 6) * (f->ny + 6) * (f->ndim == 3 ? f->nz + 6 : 1));
    if (!check_cuda(cudaMemcpy(h.data(), d_p, h.size() * sizeof(double), cudaMemcpyDeviceToHost), "download"))
        return false;
    from_ghosted(f, h, f->sol);
    return true;
}

bool multigrid::residual(double &norm) {
    return mg_upload(this) && check(scihpc_poisson_residual(gpu, d_rhs, d_p, &norm, nullptr), "poisson_residual");
}

void multigrid::v_cycle() { iterate(1); }
void multigrid::full_cycle() { iterate(1); }

// ---------------------------------------------------------------- shared solvers, scratch
shared_solvers *SharedSolvers_alloc(scalar_data *f, structured_grid *geo) {
    auto *s = new shared_solvers();
    s->geo = geo;
    s->ccd = new ccd_solver(f, geo);
    s->uccd = new uccd_solver(f, geo);
    s->weno = new weno_solver(f, geo);
    s->secSol = new second_order_solver(geo->dx, geo->dy, geo->dz);
    s->mg = new multigrid(f, geo);
    return s;
}
void shared_solvers_mg_init_Neumann(shared_solvers *s) {
    s->mg_bc = 0;
    for (unsigned l = 0; l < s->mg->level_num; ++l) s->mg->at[l]->init_NeumannBC();
}
void shared_solvers_mg_init_Dirichlet(shared_solvers *s) {
    s->mg_bc = 1;
    for (unsigned l = 0; l < s->mg->level_num; ++l) s->mg->at[l]->init_DirichletBC();
}

dummy_data *dummy_data_alloc(scalar_data *f) {
    auto *d = new dummy_data();
    DataType ****all[] = {&d->heaviside, &d->sign,  &d->delta, &d->grad,  &d->curvature, &d->tmp,     &d->u_tmp,
                          &d->v_tmp,     &d->w_tmp, &d->a,     &d->b,     &d->a_int,     &d->b_int,   &d->density,
                          &d->viscosity};
    for (auto *a : all) *a = init_array(f->Nx, f->Ny, f->Nz);
    return d;
}

// ---------------------------------------------------------------- host-array GPU calls
namespace {
scihpc_ctx *ctx_for(const scihpc_grid &g) {
    std::vector<double> key = {double(g.ndim)};
    for (int a = 0; a < 3; ++a) key.insert(key.end(), {double(g.n[a]), g.lo[a], g.hi[a]});
    Scratch &sc = g_scratch[key];
    if (!sc.ctx && !check(scihpc_ctx_create(&g, &sc.ctx), "ctx_create")) return nullptr;
    return sc.ctx;
}

// a grid with the scalar's sizes (unit spacing) for calls that need no geometry
scihpc_grid grid_of_sizes(const scalar_data *f) {
    scihpc_grid c{};
    c.ndim = f->ndim;
    const int n[3] = {f->nx, f->ny, f->nz};
    for (int a = 0; a < 3; ++a) {
        c.n[a] = a < f->ndim ? n[a] : 1;
        c.lo[a] = 0.0;
        c.hi[a] = a < f->ndim ? double(n[a]) : 1.0;
    }
    return c;
}

// One GPU call on host arrays: inputs are brought up to date from a GPU session that owns
// them and uploaded; outputs are uploaded too (so that cells the call does not write keep
// their values), downloaded at finish() and pushed to the owning session, if any.
struct HostCall {
    scihpc_ctx *ctx = nullptr;
    size_t n = 0;
    bool ok = true;
    std::vector<std::pair<DataType ***, double *>> outs;
    std::vector<double *> bufs;

    HostCall(const scihpc_grid &g, const scalar_data *f) : ctx(ctx_for(g)), n(cells_of(f)) { ok = ctx != nullptr; }
    ~HostCall() {
        for (double *p : bufs) cudaFree(p);
    }
    double *in(DataType ***a) {
        if (!ok) return nullptr;
        sync_array(a);
        double *p = nullptr;
        if (!check_cuda(cudaMalloc(&p, n * sizeof(double)), "cudaMalloc")) return ok = false, nullptr;
        bufs.push_back(p);
        if (!check_cuda(cudaMemcpy(p, base_of(a), n * sizeof(double), cudaMemcpyHostToDevice), "upload")) ok = false;
        return p;
    }
    double *out(DataType ***a) {
        double *p = in(a);
        if (p) outs.emplace_back(a, p);
        return p;
    }
    bool run(int rc, const char *what) { return ok = ok && check(rc, what); }
    bool finish() {
        for (auto &o : outs) {
            if (!ok) break;
            ok = check_cuda(cudaMemcpy(base_of(o.first), o.second, n * sizeof(double), cudaMemcpyDeviceToHost),
                            "download");
            auto it = g_mirrors.find(o.first);
            if (ok && it != g_mirrors.end()) ok = upload(it->second.s, it->second.name.c_str(), o.first);
        }
        return ok;
    }
};

void host_copy(DataType ***dst, DataType ***src, const scalar_data *f) {
    sync_array(src);
    std::memcpy(base_of(dst), base_of(src), cells_of(f) * sizeof(DataType));
}

void extrapolate(scalar_data *f, DataType ***src, int location) {
    HostCall c(grid_of_sizes(f), f);
    double *s = c.in(src), *d = c.out(f->flux);
    if (c.ok) c.run(scihpc_flux_extrapolate(c.ctx, location, s, d, nullptr), "flux_extrapolate");
    c.finish();
}
void unsupported(const char *what, const char *why) { fail(SCIHPC_ERR_UNSUPPORTED, std::string(what) + ": " + why); }
}  // namespace

// ---------------------------------------------------------------- flux
void identity_flux(scalar_data *f, vector_data *) { host_copy(f->flux, f->data, f); }
void identity_flux(scalar_data *f) { host_copy(f->flux, f->data, f); }
void identity_flux(vector_data *v) {
    for (scalar_data *c : {&v->x, &v->y, &v->z}) host_copy(c->flux, c->data, c);
}
void identity_old_flux(scalar_data *f, vector_data *) { host_copy(f->flux, f->old, f); }
void identity_old_flux(scalar_data *f) { host_copy(f->flux, f->old, f); }
void identity_old_flux(vector_data *v) {
    for (scalar_data *c : {&v->x, &v->y, &v->z}) host_copy(c->flux, c->old, c);
}
void guess_from_history(scalar_data *f) {
    HostCall c(grid_of_sizes(f), f);
    double *o = c.in(f->old), *o2 = c.in(f->old2), *fl = c.out(f->flux);
    if (c.ok) c.run(scihpc_guess_from_history(c.ctx, o, o2, fl, nullptr), "guess_from_history");
    c.finish();
}

void burgers_flux(scalar_data *f, vector_data *) {
    HostCall c(grid_of_sizes(f), f);
    double *d = c.in(f->data), *fl = c.out(f->flux);
    if (c.ok) c.run(scihpc_flux_fill(c.ctx, 1, d, fl, nullptr), "flux_fill");
    c.finish();
}

void identity_with_extrapolation(scalar_data *f, vector_data *) { extrapolate(f, f->data, 0); }
void identity_with_extrapolation(scalar_data *f) { extrapolate(f, f->data, 0); }
void identity_with_extrapolation(vector_data *v) {
    for (scalar_data *c : {&v->x, &v->y, &v->z}) extrapolate(c, c->data, 0);
}
void identity_with_extrapolation_face_x(scalar_data *f) { extrapolate(f, f->data, 1); }
void identity_with_extrapolation_face_y(scalar_data *f) { extrapolate(f, f->data, 2); }
void identity_with_extrapolation_face_z(scalar_data *f) { extrapolate(f, f->data, 3); }
void identity_with_extrapolation_face_x(vector_data *v) {
    for (scalar_data *c : {&v->x, &v->y, &v->z}) extrapolate(c, c->data, 1);
}
void identity_with_extrapolation_face_y(vector_data *v) {
    for (scalar_data *c : {&v->x, &v->y, &v->z}) extrapolate(c, c->data, 2);
}
void identity_with_extrapolation_face_z(vector_data *v) {
    for (scalar_data *c : {&v->x, &v->y, &v->z}) extrapolate(c, c->data, 3);
}
void identity_with_extrapolation_face_x(scalar_data *f, vector_data *) { extrapolate(f, f->data, 1); }
void identity_with_extrapolation_face_y(scalar_data *f, vector_data *) { extrapolate(f, f->data, 2); }
void identity_with_extrapolation_face_z(scalar_data *f, vector_data *) { extrapolate(f, f->data, 3); }

void identity_old_with_extrapolation(scalar_data *f, vector_data *) { extrapolate(f, f->old, 0); }
void identity_old_with_extrapolation(scalar_data *f) { extrapolate(f, f->old, 0); }
void identity_old_with_extrapolation(vector_data *v) {
    for (scalar_data *c : {&v->x, &v->y, &v->z}) extrapolate(c, c->old, 0);
}
void identity_old_with_extrapolation_face_x(scalar_data *f) { extrapolate(f, f->old, 1); }
void identity_old_with_extrapolation_face_y(scalar_data *f) { extrapolate(f, f->old, 2); }
void identity_old_with_extrapolation_face_z(scalar_data *f) { extrapolate(f, f->old, 3); }
void identity_old_with_extrapolation_face_x(vector_data *v) {
    for (scalar_data *c : {&v->x, &v->y, &v->z}) extrapolate(c, c->old, 1);
}
void identity_old_with_extrapolation_face_y(vector_data *v) {
    for (scalar_data *c : {&v->x, &v->y, &v->z}) extrapolate(c, c->old, 2);
}
void identity_old_with_extrapolation_face_z(vector_data *v) {
    for (scalar_data *c : {&v->x, &v->y, &v->z}) extrapolate(c, c->old, 3);
}
void identity_old_with_extrapolation_face_x(scalar_data *f, vector_data *) { extrapolate(f, f->old, 1); }
void identity_old_with_extrapolation_face_y(scalar_data *f, vector_data *) { extrapolate(f, f->old, 2); }
void identity_old_with_extrapolation_face_z(scalar_data *f, vector_data *) { extrapolate(f, f->old, 3); }

// ---------------------------------------------------------------- compact / WENO solvers
namespace {
scalar_data *component(vector_data *v, int a) { return a == 0 ? &v->x : (a == 1 ? &v->y : &v->z); }
DataType ***first_of(scalar_data *f, int a) { return a == 0 ? f->fx : (a == 1 ? f->fy : f->fz); }
DataType ***second_of(scalar_data *f, int a) { return a == 0 ? f->fxx : (a == 1 ? f->fyy : f->fzz); }

void ccd_axis(const structured_grid *geo, scalar_data *f, int a) {
    HostCall c(grid_of(geo), f);
    double *fl = c.in(f->flux), *d1 = c.out(first_of(f, a)), *d2 = c.out(second_of(f, a));
    if (c.ok) c.run(scihpc_ccd(c.ctx, a, fl, d1, d2, nullptr), "ccd");
    c.finish();
}
// mixed derivative: src extrapolated in place along `a`, out = its CCD derivative along `a`
void ccd_mixed(const structured_grid *geo, scalar_data *f, DataType ***src, DataType ***out, int a) {
    HostCall c(grid_of(geo), f);
    double *sv = c.out(src), *ov = c.out(out);
    if (c.ok) c.run(scihpc_ccd_mixed(c.ctx, a, sv, ov, nullptr), "ccd_mixed");
    c.finish();
}
void uccd_axis(const structured_grid *geo, scalar_data *f, vector_data *vel, int a) {
    HostCall c(grid_of(geo), f);
    double *fl = c.in(f->flux), *u = c.in(component(vel, a)->data);
    double *d1 = c.out(first_of(f, a)), *d2 = c.out(second_of(f, a));
    if (c.ok) c.run(scihpc_uccd(c.ctx, a, fl, u, d1, d2, nullptr), "uccd");
    c.finish();
}
void weno_axis(const structured_grid *geo, scalar_data *f, vector_data *vel, int a) {
    HostCall c(grid_of(geo), f);
    double *fl = c.in(f->flux), *u = c.in(component(vel, a)->data), *d1 = c.out(first_of(f, a));
    if (c.ok) c.run(scihpc_weno5(c.ctx, a, fl, u, d1, nullptr), "weno5");
    c.finish();
}
}  // namespace

ccd_solver::ccd_solver(scalar_data *, structured_grid *g) : geo(g) {}
void ccd_solver::find_fx(scalar_data *f) const { ccd_axis(geo, f, 0); }
void ccd_solver::find_fy(scalar_data *f) const { ccd_axis(geo, f, 1); }
void ccd_solver::find_fz(scalar_data *f) const { ccd_axis(geo, f, 2); }
void ccd_solver::mixed_xy(scalar_data *f) const { ccd_mixed(geo, f, f->fx, f->fxy, 1); }
void ccd_solver::mixed_yz(scalar_data *f) const { ccd_mixed(geo, f, f->fy, f->fyz, 2); }
void ccd_solver::mixed_zx(scalar_data *f) const { ccd_mixed(geo, f, f->fz, f->fzx, 0); }
void ccd_solver::find_derivatives(scalar_data *f) const {
    find_fx(f);
    if (f->ndim > 1) find_fy(f);
    if (f->ndim > 2) find_fz(f);
}
void ccd_solver::find_derivatives(vector_data *f) const {
    find_derivatives(&f->x);
    find_derivatives(&f->y);
    find_derivatives(&f->z);
}
void ccd_solver::find_derivatives_all(scalar_data *f) const {
    find_derivatives(f);
    if (f->ndim > 1) mixed_xy(f);
    if (f->ndim > 2) {
        mixed_yz(f);
        mixed_zx(f);
    }
}
void ccd_solver::find_derivatives_all(vector_data *f) const {
    find_derivatives_all(&f->x);
    find_derivatives_all(&f->y);
    find_derivatives_all(&f->z);
}

uccd_solver::uccd_solver(scalar_data *, structured_grid *g) : geo(g) {}
void uccd_solver::find_fx(scalar_data *f, vector_data *vel) const { uccd_axis(geo, f, vel, 0); }
void uccd_solver::find_fy(scalar_data *f, vector_data *vel) const { uccd_axis(geo, f, vel, 1); }
void uccd_solver::find_fz(scalar_data *f, vector_data *vel) const { uccd_axis(geo, f, vel, 2); }
void uccd_solver::find_derivatives(scalar_data *f, vector_data *vel) const {
    find_fx(f, vel);
    if (f->ndim > 1) find_fy(f, vel);
    if (f->ndim > 2) find_fz(f, vel);
}

weno_solver::weno_solver(scalar_data *, structured_grid *g) : dx(g->dx), dy(g->dy), dz(g->dz), geo(g) {}
void weno_solver::weno5_flux_x(scalar_data *) { unsupported("weno5_flux_x", "face values are internal to the GPU kernel"); }
void weno_solver::weno5_flux_y(scalar_data *) { unsupported("weno5_flux_y", "face values are internal to the GPU kernel"); }
void weno_solver::weno5_flux_z(scalar_data *) { unsupported("weno5_flux_z", "face values are internal to the GPU kernel"); }
void weno_solver::weno5_find_fx(scalar_data *f, vector_data *vel) { weno_axis(geo, f, vel, 0); }
void weno_solver::weno5_find_fy(scalar_data *f, vector_data *vel) { weno_axis(geo, f, vel, 1); }
void weno_solver::weno5_find_fz(scalar_data *f, vector_data *vel) { weno_axis(geo, f, vel, 2); }
void weno_solver::weno5_find_derivatives(scalar_data *f, vector_data *vel) {
    weno5_find_fx(f, vel);
    if (f->ndim > 1) weno5_find_fy(f, vel);
    if (f->ndim > 2) weno5_find_fz(f, vel);
}

namespace {
void direct_call(const char *fn) {
    fail(SCIHPC_ERR_UNSUPPORTED, std::string(fn) + " runs on the GPU only inside runge_kutta::tvd_rk3 / euler");
}
}  // namespace

void convection(wrapper *, wrapper *, DataType ***, void (*)(scalar_data *, vector_data *)) { direct_call("convection"); }
void convection_weno(wrapper *, wrapper *, DataType ***, void (*)(scalar_data *, vector_data *)) {
    direct_call("convection_weno");
}
void Hamilton_Jacobi(wrapper *, wrapper *, DataType ***, void (*)(scalar_data *, vector_data *)) {
    direct_call("Hamilton_Jacobi");
}
void convection_sec(wrapper *, wrapper *, DataType ***, void (*)(scalar_data *, vector_data *)) {
    direct_call("convection_sec");
}

// ---------------------------------------------------------------- second_order_solver
second_order_solver::second_order_solver(DataType _dx, DataType _dy, DataType _dz) : dx(_dx), dy(_dy), dz(_dz) {}

namespace {
// the scalar's grid with the solver's spacing (the stencils divide by it)
scihpc_grid sec_grid(const scalar_data *f, const second_order_solver *so) {
    scihpc_grid c = grid_of_sizes(f);
    const double d[3] = {so->dx, so->dy, so->dz};
    for (int a = 0; a < f->ndim; ++a) c.hi[a] = c.lo[a] + d[a] * c.n[a];
    return c;
}

void sec_axis(const second_order_solver *so, scalar_data *f, int a, DataType ***vel_a) {
    if (a >= f->ndim) return;
    DataType ***d1[3] = {f->fx, f->fy, f->fz}, ***d2[3] = {f->fxx, f->fyy, f->fzz};
    HostCall c(sec_grid(f, so), f);
    double *fl = c.in(f->flux), *v = vel_a ? c.in(vel_a) : nullptr, *o1 = c.out(d1[a]), *o2 = c.out(d2[a]);
    if (c.ok) c.run(scihpc_sec_derivative(c.ctx, a, fl, v, o1, o2, nullptr), "sec_derivative");
    c.finish();
}

void sec_mix(const second_order_solver *so, scalar_data *f, int b, DataType ***src, DataType ***dst) {
    if (b >= f->ndim) return;
    HostCall c(sec_grid(f, so), f);
    double *in = c.in(src), *out = c.out(dst);
    if (c.ok) c.run(scihpc_sec_mixed(c.ctx, b, in, out, nullptr), "sec_mixed");
    c.finish();
}
}  // namespace

void second_order_solver::find_fx(scalar_data *f) const { sec_axis(this, f, 0, nullptr); }
void second_order_solver::find_fy(scalar_data *f) const { sec_axis(this, f, 1, nullptr); }
void second_order_solver::find_fz(scalar_data *f) const { sec_axis(this, f, 2, nullptr); }
void second_order_solver::find_fx(scalar_data *f, vector_data *vel) const { sec_axis(this, f, 0, vel->x.data); }
void second_order_solver::find_fy(scalar_data *f, vector_data *vel) const { sec_axis(this, f, 1, vel->y.data); }
void second_order_solver::find_fz(scalar_data *f, vector_data *vel) const { sec_axis(this, f, 2, vel->z.data); }
void second_order_solver::mixed_xy(scalar_data *f) const { sec_mix(this, f, 1, f->fx, f->fxy); }
void second_order_solver::mixed_yz(scalar_data *f) const { sec_mix(this, f, 2, f->fy, f->fyz); }
void second_order_solver::mixed_zx(scalar_data *f) const { sec_mix(this, f, 0, f->fz, f->fzx); }
void second_order_solver::find_derivatives(scalar_data *f) const {
    find_fx(f);
    if (f->ndim > 1) find_fy(f);
    if (f->ndim > 2) find_fz(f);
}
void second_order_solver::find_derivatives(scalar_data *f, vector_data *vel) const {
    find_fx(f, vel);
    if (f->ndim > 1) find_fy(f, vel);
    if (f->ndim > 2) find_fz(f, vel);
}
void second_order_solver::find_derivatives_all(scalar_data *f) const {
    find_derivatives(f);
    if (f->ndim > 1) mixed_xy(f);
    if (f->ndim > 2) {
        mixed_yz(f);
        mixed_zx(f);
    }
}
void mpls(wrapper *, wrapper *, DataType ***, void (*)(scalar_data *, vector_data *)) { direct_call("mpls"); }
void lsf_redistance_no_lambda(wrapper *, wrapper *, DataType ***, void (*)(scalar_data *, vector_data *)) {
    direct_call("lsf_redistance_no_lambda");
}
void lsf_redistance_lambda(wrapper *, wrapper *, DataType ***, void (*)(scalar_data *, vector_data *)) {
    direct_call("lsf_redistance_lambda");
}

// ---------------------------------------------------------------- runge_kutta
runge_kutta::runge_kutta(int, int, int) : s1(nullptr), s2(nullptr), s3(nullptr) {}

namespace {
typedef void (*rhs_fn)(wrapper *, wrapper *, DataType ***, void (*)(scalar_data *, vector_data *));
typedef void (*flux_fn)(scalar_data *, vector_data *);

bool stage_begin(Session *&s, wrapper *f, wrapper *vel, flux_fn flux) {
    if (flux != static_cast<flux_fn>(&identity_flux)) {
        fail(SCIHPC_ERR_UNSUPPORTED, "only identity_flux is implemented on the GPU path");
        return false;
    }
    // vel here is the node velocity the drivers pass to the transport stages
    Session *found = session_of(f);
    s = found ? found : session_for(f, vel, vel, nullptr);
    return s && push_scalars(s);
}
}  // namespace

// Transport of a scalar that no two-phase session owns (the 1D drivers, Hamilton-Jacobi /
// Burgers): the stages of runge_kutta.cpp:13-63 on device buffers kept per field between calls.
// Each stage: the flux on every cell (identity or Burgers), the UCCD first derivatives of every
// active axis upwinded by the velocity, the right-hand side (convection or Hamilton-Jacobi) with
// the stage's update of phi, and the fill of phi's ghosts with the field's boundary conditions.
namespace {
struct TransportBufs {
    scihpc_ctx *ctx = nullptr;
    size_t n = 0;
    double *phi = nullptr, *flux = nullptr, *s1 = nullptr, *s2 = nullptr;
    double *d1[3] = {}, *d2[3] = {}, *vel[3] = {};
};
std::map<const scalar_data *, TransportBufs> g_transport;

bool transport_case(wrapper *f, flux_fn flux, rhs_fn rhs) {
    const bool known_flux = flux == static_cast<flux_fn>(&identity_flux) || flux == &burgers_flux;
    const bool known_rhs = rhs == &convection || rhs == &Hamilton_Jacobi || rhs == &convection_sec;
    if (!known_flux || !known_rhs || !f->is_scalar || session_of(f)) return false;
    if (f->scalar->ndim == 1 || rhs == &Hamilton_Jacobi || rhs == &convection_sec || flux == &burgers_flux)
        return true;
    // a two-phase session serves scalars with Neumann walls; any other boundary goes here
    int types[6];
    double vals[6];
    f->bcFactory->codes(types, vals);
    for (int face = 0; face < 2 * f->scalar->ndim; ++face)
        if (types[face] != 1) return true;
    return false;
}

bool transport_run(wrapper *f, wrapper *vel, flux_fn flux, rhs_fn rhs, int first_stage, int last_stage) {
    if (!f->params) return fail(SCIHPC_ERR_ARG, "tvd_rk3: link_params first (dt)"), false;
    scalar_data *sc = f->scalar;
    TransportBufs &b = g_transport[sc];
    const size_t n = cells_of(sc);
    if (!b.ctx) {
        b.ctx = ctx_for(grid_of(f->geo));   // the derivatives need the grid's spacing
        if (!b.ctx) return false;
        b.n = n;
        double **all[] = {&b.phi, &b.flux, &b.s1, &b.s2, &b.d1[0], &b.d1[1], &b.d1[2], &b.d2[0], &b.d2[1], &b.d2[2],
                          &b.vel[0], &b.vel[1], &b.vel[2]};
        for (double **p : all) {
            if (!check_cuda(cudaMalloc(p, n * sizeof(double)), "cudaMalloc")) return false;
            if (!check_cuda(cudaMemset(*p, 0, n * sizeof(double)), "cudaMemset")) return false;
        }
    }
    const int ndim = sc->ndim;
    sync_array(sc->data);
    if (!check_cuda(cudaMemcpy(b.phi, base_of(sc->data), n * sizeof(double), cudaMemcpyHostToDevice), "upload"))
        return false;
    DataType ***vc[3] = {vel->vector->x.data, vel->vector->y.data, vel->vector->z.data};
    for (int a = 0; a < ndim; ++a) {
        sync_array(vc[a]);
        if (!check_cuda(cudaMemcpy(b.vel[a], base_of(vc[a]), n * sizeof(double), cudaMemcpyHostToDevice), "upload"))
            return false;
    }
    int types[6];
    double vals[6];
    f->bcFactory->codes(types, vals);
    const int fk = flux == &burgers_flux ? 1 : 0, rk = rhs == &Hamilton_Jacobi ? 1 : 0;
    const double *d1[3] = {b.d1[0], b.d1[1], b.d1[2]}, *vl[3] = {b.vel[0], b.vel[1], b.vel[2]};
    for (int st = first_stage; st <= last_stage; ++st) {
        if (!check(scihpc_flux_fill(b.ctx, fk, b.phi, b.flux, nullptr), "flux_fill")) return false;
        for (int a = 0; a < ndim; ++a) {
            // convection_sec: second_order_solver's upwind-biased derivative (source.cpp:42-73)
            const int rc = rhs == &convection_sec
                               ? scihpc_sec_derivative(b.ctx, a, b.flux, b.vel[a], b.d1[a], b.d2[a], nullptr)
                               : scihpc_uccd(b.ctx, a, b.flux, b.vel[a], b.d1[a], b.d2[a], nullptr);
            if (!check(rc, "derivative")) return false;
        }
        if (!check(scihpc_rk3_stage(b.ctx, st, rk, f->params->dt, b.phi, d1, vl, b.s1, b.s2, nullptr), "rk3_stage"))
            return false;
        if (!check(scihpc_bc_fill(b.ctx, 0, types, vals, b.phi, nullptr), "bc_fill")) return false;
    }
    return check_cuda(cudaMemcpy(base_of(sc->data), b.phi, n * sizeof(double), cudaMemcpyDeviceToHost), "download");
}
}  // namespace

void runge_kutta::tvd_rk3(wrapper *f, wrapper *vel, flux_fn flux, rhs_fn rhs) const {
    if (transport_case(f, flux, rhs)) {
        transport_run(f, vel, flux, rhs, 1, 3);
        return;
    }
    Session *s = nullptr;
    if (!stage_begin(s, f, vel, flux)) return;
    if (rhs == &convection || rhs == &convection_weno) {
        const int scheme = rhs == &convection ? 0 : 1;
        if (scheme != s->scheme && !check(scihpc_twophase_set_scheme(s->tp, scheme), "set_scheme")) return;
        s->scheme = scheme;
        if (!check(scihpc_twophase_advect(s->tp), "advect")) return;
    } else if (rhs == &lsf_redistance_lambda || rhs == &lsf_redistance_no_lambda) {
        if (!check(scihpc_twophase_reinit_step(s->tp, rhs == &lsf_redistance_lambda ? 1 : 0), "reinit_step")) return;
    } else {
        fail(SCIHPC_ERR_UNSUPPORTED, "tvd_rk3: right-hand side without a GPU stage");
        return;
    }
    pull_scalars(s);
}

void runge_kutta::euler(wrapper *f, wrapper *vel, flux_fn flux, rhs_fn rhs) const {
    if (transport_case(f, flux, rhs)) {
        transport_run(f, vel, flux, rhs, 0, 0);
        return;
    }
    Session *s = nullptr;
    if (!stage_begin(s, f, vel, flux)) return;
    if (rhs != &mpls) {
        fail(SCIHPC_ERR_UNSUPPORTED, "euler: right-hand side without a GPU stage");
        return;
    }
    if (check(scihpc_twophase_mpls(s->tp, 1), "mpls")) pull_scalars(s);
}

// ---------------------------------------------------------------- projection_method
projection_method::projection_method(scalar_data *) {}

void projection_method::find_source(wrapper *vel, wrapper *nvel, wrapper *lsf) const {
    Session *s = session_for(lsf, vel, nvel, nullptr);
    if (!s || !push_scalars(s)) return;
    if (!check(scihpc_twophase_set_source_scheme(s->tp, 0), "set_source_scheme")) return;
    if (check(scihpc_twophase_find_source(s->tp), "find_source")) pull_scalars(s);
}

void projection_method::ab_solve(wrapper *vel, wrapper *nvel, wrapper *pressure, wrapper *lsf) {
    Session *s = session_for(lsf, vel, nvel, pressure);
    if (!s || !push_scalars(s)) return;
    if (!check(scihpc_twophase_set_source_scheme(s->tp, 0), "set_source_scheme")) return;
    const int rc = scihpc_twophase_ab_solve(s->tp, &last_iterations, &last_relres);
    if (rc == SCIHPC_ERR_MAXITER) {
        fail(rc, "ab_solve: pressure solve stopped at ppe_max_iter above ppe_tol");
    } else if (!check(rc, "ab_solve")) {
        return;
    }
    pull_scalars(s);
}

namespace {
Session *stage_session(wrapper *any, const char *what) {
    Session *s = session_of(any);
    if (!s) fail(SCIHPC_ERR_ARG, std::string(what) + ": call find_source first (it starts the GPU session)");
    return s && push_scalars(s) ? s : nullptr;
}
}  // namespace

// the stages of ab_solve one at a time (projection_method.cpp:384-402, 544-657)
void projection_method::find_intermediate_velocity(wrapper *vel) const {
    Session *s = stage_session(vel, "find_intermediate_velocity");
    if (s && check(scihpc_twophase_intermediate_velocity(s->tp), "intermediate_velocity")) pull_scalars(s);
}

void projection_method::projection(wrapper *pressure, wrapper *lsf, wrapper *) const {
    Session *s = stage_session(lsf, "projection");
    if (!s || !attach_pressure(s, pressure)) return;
    int it = 0;
    double rr = 0.0;
    const int rc = scihpc_twophase_projection(s->tp, &it, &rr);
    if (rc == SCIHPC_ERR_MAXITER) fail(rc, "projection: pressure solve stopped at ppe_max_iter above ppe_tol");
    else if (!check(rc, "projection")) return;
    pull_scalars(s);
}

// the constant-coefficient equation with the extrapolated pressure's variable-density term
// on its right-hand side (projection_method.cpp:659-753), on the GPU multigrid
void projection_method::fast_pressure_correction(wrapper *pressure, wrapper *lsf, wrapper *) {
    Session *s = stage_session(lsf, "fast_pressure_correction");
    if (!s || !attach_pressure(s, pressure)) return;
    const int rc = scihpc_twophase_fast_pressure_correction(s->tp, &last_iterations, &last_relres);
    if (rc == SCIHPC_ERR_MAXITER) fail(rc, "fast_pressure_correction: stopped at 100 iterations above ppe_tol");
    else if (!check(rc, "fast_pressure_correction")) return;
    pull_scalars(s);
}

// the GPU builds projection()'s coefficients from the density inside projection()
void projection_method::init_ppe_proj_coefficients(wrapper *) {}

// the right-hand-side term of the fast correction from the extrapolated pressure and the
// density (projection_method.cpp:467-541)
void projection_method::init_ppe_fpc_coefficients(wrapper *pressure) {
    Session *s = stage_session(pressure, "init_ppe_fpc_coefficients");
    if (!s || !attach_pressure(s, pressure)) return;
    check(scihpc_twophase_fpc_coefficients(s->tp), "init_ppe_fpc_coefficients");
}

// flux = old + dt_old (old - old2) / dt_old2 (projection_method.cpp:803-815)
void projection_method::pressure_guess_solution(wrapper *pressure) {
    Session *s = stage_session(pressure, "pressure_guess_solution");
    if (!s || !attach_pressure(s, pressure)) return;
    check(scihpc_twophase_pressure_guess(s->tp), "pressure_guess_solution");
}
void projection_method::add_stress_x(wrapper *, wrapper *, wrapper *) const {
    unsupported("add_stress_x", "a stage inside the GPU find_source");
}
void projection_method::add_stress_y(wrapper *, wrapper *, wrapper *) const {
    unsupported("add_stress_y", "a stage inside the GPU find_source");
}
void projection_method::add_stress_z(wrapper *, wrapper *, wrapper *) const {
    unsupported("add_stress_z", "a stage inside the GPU find_source");
}
void projection_method::add_body_force(wrapper *) const {
    unsupported("add_body_force", "a stage inside the GPU find_source");
}
void projection_method::add_surface_force(wrapper *) const {
    unsupported("add_surface_force", "a stage inside the GPU find_source");
}
void projection_method::find_source_sec(wrapper *vel, wrapper *nvel, wrapper *lsf) const {
    Session *s = session_for(lsf, vel, nvel, nullptr);
    if (!s || !push_scalars(s)) return;
    if (!check(scihpc_twophase_set_source_scheme(s->tp, 1), "set_source_scheme")) return;
    if (check(scihpc_twophase_find_source(s->tp), "find_source_sec")) pull_scalars(s);
}

void projection_method::ab_solve_sec(wrapper *vel, wrapper *nvel, wrapper *pressure, wrapper *lsf) {
    Session *s = session_for(lsf, vel, nvel, pressure);
    if (!s || !push_scalars(s)) return;
    if (!check(scihpc_twophase_set_source_scheme(s->tp, 1), "set_source_scheme")) return;
    const int rc = scihpc_twophase_ab_solve(s->tp, &last_iterations, &last_relres);
    if (rc == SCIHPC_ERR_MAXITER) {
        fail(rc, "ab_solve_sec: pressure solve stopped at ppe_max_iter above ppe_tol");
    } else if (!check(rc, "ab_solve_sec")) {
        return;
    }
    pull_scalars(s);
}

// ---------------------------------------------------------------- wrapper_func
void node_from_face(wrapper *ref, wrapper *) {
    Session *s = stage_session(ref, "node_from_face");
    if (s && check(scihpc_twophase_node_from_face(s->tp), "node_from_face")) pull_scalars(s);
}
void all_to_face_x(wrapper *, wrapper *) { unsupported("all_to_face_x", "a stage inside the GPU find_source"); }
void all_to_face_y(wrapper *, wrapper *) { unsupported("all_to_face_y", "a stage inside the GPU find_source"); }
void all_to_face_z(wrapper *, wrapper *) { unsupported("all_to_face_z", "a stage inside the GPU find_source"); }
void find_gradient(wrapper *) { unsupported("find_gradient", "a stage inside the GPU find_source"); }

namespace {
// heaviside, delta, density or viscosity of the host level set, on the GPU
void lsf_field(wrapper *lsf, int which) {
    const problem_parameters *p = lsf->params;
    if (!p || !lsf->dummy) {
        fail(SCIHPC_ERR_ARG, "level-set fields: wrapper not linked to problem_parameters and dummy_data");
        return;
    }
    const double prm[4] = {p->ls_width, p->density_ratio, p->viscosity_ratio, double(p->positive_ref)};
    DataType ***dst[4] = {lsf->dummy->heaviside, lsf->dummy->delta, lsf->dummy->density, lsf->dummy->viscosity};
    HostCall c(grid_of(lsf->geo), lsf->scalar);
    double *phi = c.in(lsf->scalar->data), *out = c.out(dst[which]);
    if (c.ok)
        c.run(scihpc_lsf_fields(c.ctx, prm, phi, which == 0 ? out : nullptr, which == 1 ? out : nullptr, nullptr,
                                which == 2 ? out : nullptr, which == 3 ? out : nullptr, nullptr),
              "lsf_fields");
    c.finish();
}
}  // namespace

void find_heavyside(wrapper *lsf) { lsf_field(lsf, 0); }
void find_delta(wrapper *lsf) { lsf_field(lsf, 1); }
void find_density(wrapper *lsf) { lsf_field(lsf, 2); }
void find_viscosity(wrapper *lsf) { lsf_field(lsf, 3); }

// curvature from the level set and its CCD derivative arrays (wrapper_func.cpp:115-174)
void find_curvature(wrapper *lsf) {
    if (!lsf->dummy) {
        fail(SCIHPC_ERR_ARG, "find_curvature: wrapper not linked to dummy_data");
        return;
    }
    scalar_data *f = lsf->scalar;
    HostCall c(grid_of(lsf->geo), f);
    DataType ***src[9] = {f->fx, f->fy, f->fz, f->fxx, f->fyy, f->fzz, f->fxy, f->fyz, f->fzx};
    const double *d[9];
    for (int q = 0; q < 9; ++q) d[q] = c.in(src[q]);
    double *phi = c.in(f->data), *curv = c.out(lsf->dummy->curvature);
    if (c.ok) c.run(scihpc_curvature(c.ctx, phi, d, curv, nullptr), "curvature");
    c.finish();
}

// ---------------------------------------------------------------- godunov_gradient
// the scalar WENO-JS correction of godunov_gradient.cpp:183-198 (weights d = 1/10, 6/10,
// 3/10 on (eps + indicator)^-2)
DataType weno5_for_godunov(DataType a, DataType b, DataType c, DataType d) {
    const DataType eps = 1e-8;
    const DataType is0 = 13.0 * (a - b) * (a - b) + 3.0 * (a - 3.0 * b) * (a - 3.0 * b);
    const DataType is1 = 13.0 * (b - c) * (b - c) + 3.0 * (b + c) * (b + c);
    const DataType is2 = 13.0 * (c - d) * (c - d) + 3.0 * (3.0 * c - d) * (3.0 * c - d);
    const DataType a0 = 1.0 / ((eps + is0) * (eps + is0)), a1 = 6.0 / ((eps + is1) * (eps + is1)),
                   a2 = 3.0 / ((eps + is2) * (eps + is2));
    const DataType w0 = a0 / (a0 + a1 + a2), w2 = a2 / (a0 + a1 + a2);
    return w0 / 3.0 * (a - 2.0 * b + c) + (w2 - 0.5) / 6.0 * (b - 2.0 * c + d);
}

void godunov_gradient(wrapper *f) {
    if (!f->dummy) {
        fail(SCIHPC_ERR_ARG, "godunov_gradient: wrapper not linked to dummy_data");
        return;
    }
    HostCall c(grid_of(f->geo), f->scalar);
    double *phi = c.in(f->scalar->data), *sg = c.in(f->dummy->sign), *g = c.out(f->dummy->grad);
    if (c.ok) c.run(scihpc_godunov_gradient(c.ctx, phi, sg, g, nullptr), "godunov_gradient");
    c.finish();
}

// godunov_gradient, then phi /= max |grad phi| (godunov_gradient.cpp:159-181)
void stabilized_upon_gradient(wrapper *f) {
    if (!f->dummy) {
        fail(SCIHPC_ERR_ARG, "stabilized_upon_gradient: wrapper not linked to dummy_data");
        return;
    }
    HostCall c(grid_of(f->geo), f->scalar);
    double *phi = c.out(f->scalar->data), *sg = c.in(f->dummy->sign), *g = c.out(f->dummy->grad);
    if (c.ok) c.run(scihpc_stabilized_upon_gradient(c.ctx, phi, sg, g, nullptr), "stabilized_upon_gradient");
    c.finish();
}

void find_sign(wrapper *lsf) {
    Session *s = session_of(lsf);
    if (!s) {
        fail(SCIHPC_ERR_ARG, "find_sign: no GPU session for this level set yet");
        return;
    }
    check(scihpc_twophase_find_sign(s->tp), "find_sign");
}

void find_dt(wrapper *vel) {
    Session *s = session_of(vel);
    if (!s) {
        fail(SCIHPC_ERR_ARG, "find_dt: call find_source first (it starts the GPU session)");
        return;
    }
    if (push_scalars(s) && check(scihpc_twophase_find_dt(s->tp), "find_dt")) pull_scalars(s);
}

namespace {
// mass (which 0) or volume (which 1) of the level set on the GPU (wrapper_func.cpp:450-572)
DataType integral(wrapper *f, int which) {
    const problem_parameters *p = f->params;
    if (!p) {
        fail(SCIHPC_ERR_ARG, "lsf integral: wrapper not linked to problem_parameters");
        return 0.0;
    }
    const double prm[4] = {p->ls_width, p->density_ratio, p->viscosity_ratio, double(p->positive_ref)};
    double out[2] = {0.0, 0.0};
    Session *s = session_of(f);
    const scihpc_grid g = grid_of(f->geo);
    std::vector<double> key = {double(g.ndim)};
    for (int a = 0; a < 3; ++a) key.insert(key.end(), {double(g.n[a]), g.lo[a], g.hi[a]});
    Scratch &sc = g_scratch[key];
    if (!sc.ctx && !check(scihpc_ctx_create(&g, &sc.ctx), "ctx_create")) return 0.0;
    if (s) {
        double *dev = nullptr;
        if (!check(scihpc_twophase_field(s->tp, "phi", &dev), "field")) return 0.0;
        void *stream = nullptr;
        check(scihpc_twophase_stream(s->tp, &stream), "stream");
        check(scihpc_lsf_integrals(sc.ctx, prm, dev, out, stream), "lsf_integrals");
    } else {
        const size_t n = cells_of(f->scalar);
        if (sc.cells < n) {
            if (sc.dev) cudaFree(sc.dev);
            sc.dev = nullptr;
            if (!check_cuda(cudaMalloc(&sc.dev, n * sizeof(double)), "cudaMalloc")) return 0.0;
            sc.cells = n;
        }
        if (!check_cuda(cudaMemcpy(sc.dev, base_of(f->scalar->data), n * sizeof(double), cudaMemcpyHostToDevice),
                        "upload"))
            return 0.0;
        check(scihpc_lsf_integrals(sc.ctx, prm, sc.dev, out, nullptr), "lsf_integrals");
    }
    return out[which];
}
}  // namespace

DataType lsf_mass(wrapper *f) { return integral(f, 0); }
DataType lsf_volume(wrapper *f) { return integral(f, 1); }

DataType divergence(wrapper *vel) {
    Session *s = session_of(vel);
    if (!s) {
        fail(SCIHPC_ERR_ARG, "divergence: no GPU session for these velocities yet");
        return 0.0;
    }
    double d[3] = {0.0, 0.0, 0.0};
    check(scihpc_twophase_diagnostics(s->tp, d), "diagnostics");
    return d[2];
}

// l2norm / linfity against the store_tmp snapshot, over all cells (wrapper_func.cpp:60-113,
// 420-448; linfity keeps the reference's sqrt(max / N) normalisation)
void store_tmp(wrapper *f) {
    scihpc_sync_to_host(f);
    if (f->is_scalar) {
        std::memcpy(base_of(f->dummy->tmp), base_of(f->scalar->data), cells_of(f->scalar) * sizeof(DataType));
    } else {
        const size_t n = cells_of(&f->vector->x) * sizeof(DataType);
        std::memcpy(base_of(f->dummy->u_tmp), base_of(f->vector->x.data), n);
        std::memcpy(base_of(f->dummy->v_tmp), base_of(f->vector->y.data), n);
        std::memcpy(base_of(f->dummy->w_tmp), base_of(f->vector->z.data), n);
    }
}

namespace {
template <class Op>
DataType compare_tmp(wrapper *f, Op op) {
    scihpc_sync_to_host(f);
    DataType acc = 0.0;
    size_t n;
    if (f->is_scalar) {
        n = cells_of(f->scalar);
        const DataType *a = base_of(f->dummy->tmp), *b = base_of(f->scalar->data);
        for (size_t i = 0; i < n; ++i) acc = op(acc, a[i] - b[i]);
    } else {
        n = cells_of(&f->vector->x);
        const DataType *t[3] = {base_of(f->dummy->u_tmp), base_of(f->dummy->v_tmp), base_of(f->dummy->w_tmp)};
        const DataType *v[3] = {base_of(f->vector->x.data), base_of(f->vector->y.data), base_of(f->vector->z.data)};
        for (size_t i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c) acc = op(acc, t[c][i] - v[c][i]);
    }
    return std::sqrt(acc / DataType(n));
}
}  // namespace

DataType l2norm(wrapper *f) {
    return compare_tmp(f, [](DataType a, DataType d) { return a + d * d; });
}
DataType linfity(wrapper *f) {
    return compare_tmp(f, [](DataType a, DataType d) { return std::fmax(a, std::fabs(d)); });
}

// ---------------------------------------------------------------- lsm
DataType Heaviside(DataType x, DataType w) {
    if (x < -w) return 0;
    if (x > w) return 1;
    return 0.5 * (1 + x / w + std::sin(pi * x / w) / pi);
}
DataType Delta(DataType x, DataType w) {
    if (x < -w || x > w) return 0;
    return 0.5 * (1 + std::cos(pi * x / w)) / w;
}
DataType Sign(const DataType &x, const DataType &w) {
    if (x < -w) return -1;
    if (x > w) return 1;
    return x / std::sqrt(x * x + w * w);
}

// ---------------------------------------------------------------- vtkWriter
// Legacy VTK, STRUCTURED_POINTS with CELL_DATA, doubles big-endian, x fastest (the format the
// reference writes, vtkWriter.cpp:18-111).
namespace {
void put_be(std::vector<char> &buf, DataType v) {
    unsigned char b[sizeof(DataType)];
    std::memcpy(b, &v, sizeof v);
    for (int i = int(sizeof v) - 1; i >= 0; --i) buf.push_back(char(b[i]));
}
}  // namespace

vtkWriter::vtkWriter(structured_grid *g, std::string name) : grid(g), filename(std::move(name)) {}

void vtkWriter::create(unsigned int id) {
    file = std::ofstream(filename + std::to_string(id) + ".vtk", std::ios::binary);
    file << "# vtk DataFile Version 3.0\nvtk output\nBINARY\nDATASET STRUCTURED_POINTS\n";
    file << "DIMENSIONS " << grid->vtk_info.nx << " " << grid->vtk_info.ny << " " << grid->vtk_info.nz << "\n";
    file << "ORIGIN " << grid->vtk_info.xstart << " " << grid->vtk_info.ystart << " " << grid->vtk_info.zstart << "\n";
    file << "SPACING " << grid->dx << " " << grid->dy << " " << grid->dz << "\n";
    long cells = 1;
    for (int n : {grid->vtk_info.nx, grid->vtk_info.ny, grid->vtk_info.nz})
        if (n > 1) cells *= n - 1;
    file << "CELL_DATA " << cells << "\n";
}

void vtkWriter::add_scalar(DataType ***a, scalar_data *f, const std::string &name) {
    sync_array(a);
    file << "SCALARS " << name << " double 1\nLOOKUP_TABLE default\n";
    std::vector<char> buf;
    buf.reserve(size_t(f->nx) * f->ny * f->nz * sizeof(DataType));
    for (int k = 0; k < f->nz; ++k)
        for (int j = 0; j < f->ny; ++j)
            for (int i = 0; i < f->nx; ++i) {
                const indices ix = f->index_mapping(i + 1, j + 1, k + 1);
                put_be(buf, a[ix.i][ix.j][ix.k]);
            }
    file.write(buf.data(), std::streamsize(buf.size()));
}

void vtkWriter::add_scalar(scalar_data *f, const std::string &name) { add_scalar(f->data, f, name); }

void vtkWriter::add_vector(DataType ***u, DataType ***v, DataType ***w, vector_data *f, const std::string &name) {
    sync_array(u);
    sync_array(v);
    sync_array(w);
    file << "VECTORS " << name << " double\n";
    const scalar_data &x = f->x;
    std::vector<char> buf;
    buf.reserve(size_t(x.nx) * x.ny * x.nz * 3 * sizeof(DataType));
    for (int k = 0; k < x.nz; ++k)
        for (int j = 0; j < x.ny; ++j)
            for (int i = 0; i < x.nx; ++i) {
                const indices ix = f->x.index_mapping(i + 1, j + 1, k + 1);
                put_be(buf, u[ix.i][ix.j][ix.k]);
                put_be(buf, v[ix.i][ix.j][ix.k]);
                put_be(buf, w[ix.i][ix.j][ix.k]);
            }
    file.write(buf.data(), std::streamsize(buf.size()));
}

void vtkWriter::add_vector(vector_data *f, const std::string &name) {
    add_vector(f->x.data, f->y.data, f->z.data, f, name);
}

void vtkWriter::close() { file.close(); }
