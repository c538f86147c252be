/*
 * scihpc_gpu.h -- C ABI of the GB300 (sm_103a) two-phase projection-step library.
 *
 * The reference (luisleo526/SciHPC) has no FFI: its boundary is the C++ class API of
 * scihpc/*.h.  Each entry point below replaces one reference function or method on that
 * path and cites it.  Conventions:
 *
 *   - Every function returns an int status (SCIHPC_OK = 0).  scihpc_last_error() gives a
 *     message for the last failure on the calling thread.
 *   - Field arguments are DEVICE pointers to FP64 arrays laid out like the reference's
 *     scalar_data arrays: [Nx][Ny][Nz], k fastest, ghost width 3 on every active axis
 *     (Nx = nx + 6; Ny = ny + 6 when ndim >= 2, else 1; Nz = nz + 6 when ndim == 3, else 1).
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).  Calls are
 *     asynchronous unless their comment says they return a host value.
 *   - Boundary codes: 0 periodic, 1 neumann, 2 no_slip, 3 slip, 4 dirichlet
 *     (bc_factory.h:18-22).  Face order in 6-arrays: xl, xr, yl, yr, zl, zr
 *     (argument order of the bc_factory / wrapper constructors, bc_factory.h:42-48).
 *   - Locations: 0 cell-centred ("node"), 1/2/3 staggered in x/y/z ("face"), as in
 *     bc_factory::apply_node_centered / apply_node_staggered_{x,y,z} (bc_factory.h:53-56).
 */
#ifndef SCIHPC_GPU_H
#define SCIHPC_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define SCIHPC_OK 0
#define SCIHPC_ERR_ARG 1
#define SCIHPC_ERR_CUDA 2
#define SCIHPC_ERR_NONFINITE 3
#define SCIHPC_ERR_MAXITER 4
#define SCIHPC_ERR_UNSUPPORTED 5
#define SCIHPC_ERR_NOMEM 6

/* Uniform cell-centred grid (structured_grid.h:10-30): n interior cells on [lo, hi] per axis. */
typedef struct scihpc_grid {
    int ndim;       /* 1, 2 or 3 */
    int n[3];       /* interior cells per axis (ignored beyond ndim) */
    double lo[3];   /* axis start (axis::start, global.h:20-23) */
    double hi[3];   /* axis end   (axis::end) */
} scihpc_grid;

/* Message of the last failure on this thread (empty string when none). */
const char *scihpc_last_error(void);

/* Library version string. */
const char *scihpc_version(void);

/* ------------------------------------------------------------------ context
 * Per-grid device state shared by the kernel-level calls: factored compact-scheme line
 * operators for every axis (uccd_base.cpp:7-118, ccd_base.cpp:7-105), scratch fields and
 * reduction buffers.  Replaces the per-grid solver objects that SharedSolvers_alloc builds
 * (shared_solvers.cpp:7-15).  Allocates device memory; must not be called during capture. */
typedef struct scihpc_ctx scihpc_ctx;
int scihpc_ctx_create(const scihpc_grid *grid, scihpc_ctx **out);
int scihpc_ctx_destroy(scihpc_ctx *ctx);

/* ------------------------------------------------------------------ boundary fills
 * Ghost fill of one field: bc_factory::apply_node_centered (location 0) and
 * apply_node_staggered_{x,y,z} (locations 1..3) with the per-face kernels of periodic.cpp,
 * neumann.cpp, no_slip.cpp, slip.cpp and dirichlet.cpp (bc_factory.cpp:123-437).
 * values[f] is bc_info::value of face f (bc_factory.h:24-27). */
int scihpc_bc_fill(scihpc_ctx *ctx, int location, const int types[6], const double values[6], double *f,
                   void *stream);

/* flux <- data with zero-order ghost extrapolation: identity_with_extrapolation (location 0)
 * and identity_with_extrapolation_face_{x,y,z} (locations 1..3) (flux.cpp:98-330). */
int scihpc_flux_extrapolate(scihpc_ctx *ctx, int location, const double *data, double *flux, void *stream);

/* zero_order_extrapolation of a raw ghosted array, in place (simple_bc.cpp:7-43). */
int scihpc_zero_order_extrapolation(scihpc_ctx *ctx, double *f, void *stream);

/* ------------------------------------------------------------------ compact schemes
 * UCCD first/second derivative along `axis` (0..2) of every grid line, upwinded by the
 * sign of vel_axis: uccd_solver::find_fx / find_fy / find_fz (uccd_solver.cpp:14-209).
 * f1 receives f_axis, f2 receives f_axis,axis. */
int scihpc_uccd(scihpc_ctx *ctx, int axis, const double *flux, const double *vel_axis, double *f1, double *f2,
                void *stream);

/* Transport of a scalar by a velocity, one TVD-RK3 stage at a time (runge_kutta.cpp:13-63):
 * scihpc_flux_fill writes flux = phi (kind 0, identity_flux, flux.cpp:7-20) or phi^2 / 2
 * (kind 1, burgers_flux, flux.cpp:86-96) on every cell; after the caller's scihpc_uccd on
 * each axis (first derivatives d[a], upwinded by vel[a]), scihpc_rk3_stage forms the
 * right-hand side s = -sum_a vel[a] d[a] (rhs_kind 0, convection, source.cpp:8-40) or
 * -sum_a d[a] (rhs_kind 1, Hamilton_Jacobi, source.cpp:75-107) on every cell and applies the
 * stage: 1: phi += dt s (s -> s1); 2: phi += dt (s - 3 s1) / 4 (s -> s2); 3: phi += dt (-s1 - s2
 * + 8 s) / 12; 0: euler's phi += dt s.  The caller then refills phi's ghosts (scihpc_bc_fill). */
/* The second-order finite differences of second_order_solver (second_order_solver.cpp:7-241):
 * vel_axis NULL: find_fx/fy/fz(f) -- central first (f1) and second (f2) derivatives of flux
 * along axis on every cell, second-order one-sided at the ends of the ghosted array; vel_axis
 * given: find_fx/fy/fz(f, vel) -- the one-sided second-order first derivative on the side the
 * velocity comes from and the central second derivative, at the interior points of the axis
 * only (the axis's ghost points keep their values).  scihpc_sec_mixed: mixed_xy / mixed_yz /
 * mixed_zx, the derivative of src along axis with the central / one-sided stencils. */
int scihpc_sec_derivative(scihpc_ctx *ctx, int axis, const double *flux, const double *vel_axis, double *f1,
                          double *f2, void *stream);
int scihpc_sec_mixed(scihpc_ctx *ctx, int axis, const double *src, double *out, void *stream);
int scihpc_flux_fill(scihpc_ctx *ctx, int kind, const double *phi, double *flux, void *stream);
int scihpc_rk3_stage(scihpc_ctx *ctx, int stage, int rhs_kind, double dt, double *phi, const double *const d[3],
                     const double *const vel[3], double *s1, double *s2, void *stream);
/* Central CCD first/second derivative along `axis`: ccd_solver::find_fx / find_fy /
 * find_fz (ccd_solver.cpp:14-141). */
int scihpc_ccd(scihpc_ctx *ctx, int axis, const double *flux, double *f1, double *f2, void *stream);

/* Mixed derivative: src (a first derivative) is zero-order extrapolated along `axis` in
 * place, then out = its CCD derivative along `axis`.  axis 1 with src = f_x gives f_xy
 * (ccd_solver::mixed_xy), axis 2 with f_y gives f_yz (mixed_yz), axis 0 with f_z gives
 * f_zx (mixed_zx) (ccd_solver.cpp:143-282). */
int scihpc_ccd_mixed(scihpc_ctx *ctx, int axis, double *src, double *out, void *stream);

/* WENO5 (WENO-Z weights) derivative along `axis` on interior cells, faces upwinded by the
 * sign of vel_i + vel_{i+1}: weno_solver::weno5_find_fx / fy / fz
 * (weno_solver.cpp:68-268).  Ghost cells of fa are not written. */
int scihpc_weno5(scihpc_ctx *ctx, int axis, const double *flux, const double *vel_axis, double *fa, void *stream);

/* ------------------------------------------------------------------ level-set helpers
 * Godunov |grad phi| on interior cells, 0 on ghosts (godunov_gradient.cpp:7-157). */
int scihpc_godunov_gradient(scihpc_ctx *ctx, const double *phi, const double *sign, double *grad, void *stream);

/* stabilized_upon_gradient (godunov_gradient.cpp:159-181): grad = Godunov |grad phi| as
 * above, then phi /= max(grad) over every cell, in place.  The maximum is found on the
 * device (no host synchronisation). */
int scihpc_stabilized_upon_gradient(scihpc_ctx *ctx, double *phi, const double *sign, double *grad, void *stream);

/* guess_from_history (flux.cpp:653-662): flux = 2 old - old2 on every cell. */
int scihpc_guess_from_history(scihpc_ctx *ctx, const double *old, const double *old2, double *flux, void *stream);

/* Smoothed Heaviside, delta, sign, density and viscosity of phi on every cell
 * (lsm.cpp:8-43; wrapper_func.cpp:9-40,387-418).  prm = {ls_width, density_ratio,
 * viscosity_ratio, positive_ref}.  Any output may be NULL. */
int scihpc_lsf_fields(scihpc_ctx *ctx, const double prm[4], const double *phi, double *heaviside, double *delta,
                      double *sign, double *density, double *viscosity, void *stream);

/* Curvature from phi and its CCD derivatives d[9] = {fx, fy, fz, fxx, fyy, fzz, fxy, fyz,
 * fzx} with the reference's correction (wrapper_func.cpp:115-174). */
int scihpc_curvature(scihpc_ctx *ctx, const double *phi, const double *const d[9], double *curv, void *stream);

/* lsf_mass and lsf_volume of phi (wrapper_func.cpp:450-572); returns both on the host
 * (synchronises `stream`).  out[0] = mass, out[1] = volume. */
int scihpc_lsf_integrals(scihpc_ctx *ctx, const double prm[4], const double *phi, double out[2], void *stream);

/* The same integrals for callers that cannot allocate device memory: plugins whose host
 * application owns all device memory through its own pool, and real-time loops that must
 * not touch the allocator (cudaMalloc / cudaFree can synchronise the device).  No context:
 * its scratch lives in a static device array
 * of 1048576 ghosted cells (8 MiB, held by every GPU that loads the library until exit);
 * larger grids are rejected with SCIHPC_ERR_ARG.  All calls share that array: calls that
 * overlap on the GPU race and must be serialised by the caller.  The first call on each
 * device resolves the array's device address.  Synchronises `stream`.  This entry point has no counterpart in the reference. */
int scihpc_lsf_integrals_noalloc(const scihpc_grid *grid, const double prm[4], const double *phi, double out[2],
                                 void *stream);

/* ------------------------------------------------------------------ pressure Poisson
 * Multigrid solver of the pressure equation of projection_method::projection
 * (projection_method.cpp:404-465,544-627):
 *     sum_faces C_f (p_nb - p_c) = rhs   on interior cells,
 * C_f = 1 / (0.5 (rho_c + rho_nb)) / d^2 (density mode) or 1 / d^2 (constant mode).
 * Walls: bc = 0 Neumann (C_f = 0 at the wall, solution normalised to zero mean, as the
 * reference's SOR does every sweep); bc = 1 the reference multigrid's Dirichlet operator,
 * which keeps the wall term with a zero ghost-centre value (multigrid_base.cpp:293-345).
 * precision = 0: V-cycles in FP64; 1: V-cycles in FP32 inside the FP64 outer iteration
 * (the residual, the correction sum and the solution stay FP64).
 * Red-black Gauss-Seidel V(2,2) cycles, cell-average restriction, piecewise-constant
 * prolongation (its transpose, so the cycle is symmetric), FP64 dense direct solve on the
 * coarsest level (levels coarsened by the rule of multigrid.cpp:8-41), used as the
 * preconditioner of an FP64 flexible conjugate-gradient outer iteration that stops at the
 * tolerance, the iteration cap, or when the residual stops improving.  Replaces the reference's SOR sweep loop and multigrid::v_cycle /
 * full_cycle (multigrid.cpp:43-79).  Allocates device memory at creation. */
typedef struct scihpc_poisson scihpc_poisson;
int scihpc_poisson_create(const scihpc_grid *grid, int bc, int density_mode, int precision, scihpc_poisson **out);
int scihpc_poisson_destroy(scihpc_poisson *ps);
/* Coefficients from a ghosted density field (dummy_data::density); call again whenever it
 * changes (init_ppe_proj_coefficients, projection_method.cpp:404-465).  The solver keeps
 * reading `rho` in every solve: it must stay valid until the next set_density. */
int scihpc_poisson_set_density(scihpc_poisson *ps, const double *rho, void *stream);
/* Solve to ||rhs - A p|| <= rel_tol ||rhs|| (2-norms over interior cells) or max_iter
 * outer iterations.  rhs and p are ghosted fields; p holds the initial guess (use_guess = 1)
 * or is zeroed first (use_guess = 0); only interior cells of p are written.  Returns the
 * iterations and the final relative residual on the host (synchronises `stream`). */
int scihpc_poisson_solve(scihpc_poisson *ps, const double *rhs, double *p, int use_guess, double rel_tol,
                         int max_iter, int *iters, double *relres, void *stream);
/* ||rhs - A p|| (2-norm over interior cells; for Neumann walls rhs minus its mean) of the
 * solver's operator, on the GPU in FP64; synchronises `stream`.  The residual() of
 * multigrid_base (multigrid_base.cpp:69-72) for the finest level. */
int scihpc_poisson_residual(scihpc_poisson *ps, const double *rhs, const double *p, double *norm, void *stream);
/* FP32 mode (fp32 = 1): each inner FP32 conjugate-gradient solve stops once its residual has
 * dropped by inner_tol (0 < inner_tol < 1) or after inner_max (>= 1) iterations, and the FP64
 * refinement step follows.  Defaults 1e-4 and 12.  No reference counterpart (the reference
 * solves in FP64 only). */
int scihpc_poisson_set_inner(scihpc_poisson *ps, double inner_tol, int inner_max);
/* Times `ncycles` V-cycles (the preconditioner alone, on the residual of p = 0 for rhs)
 * with CUDA events on `stream`; *ms receives the total.  p is overwritten with zeros.
 * Synchronises `stream`.  Measurement hook with no reference counterpart. */
int scihpc_poisson_time_vcycles(scihpc_poisson *ps, const double *rhs, double *p, int ncycles, float *ms, void *stream);
/* Level sizes of the hierarchy (3 ints per level); returns the level count. */
int scihpc_poisson_levels(scihpc_poisson *ps, int *level_n, int max_levels);

/* ------------------------------------------------------------------ two-phase time step
 * One complete two-phase problem resident on the GPU, assembled like the reference drivers
 * (benchmarks_2d_bubble_rising.cpp:19-89): phi and pressure scalars, staggered velocity and
 * node velocity vectors, dummy scratch, projection sources and Runge-Kutta stages.
 * prm[16] = {density_ratio, viscosity_ratio, Re, Fr, We, ls_width, rdt, max_CFL, min_CFL,
 *            positive_ref, ppe_tol, ppe_tol2, ppe_max_iter, ppe_omega, ppe_initer, dt0}
 *            (problem_parameters, global.h:25-54; ppe_tol is the relative residual of the
 *            multigrid pressure solve, ppe_max_iter its outer-iteration cap).
 * opt[5]  = {convection scheme (0 UCCD, 1 WENO5), mass-correction Euler steps per step,
 *            reinitialise every k steps (0 never), pressure precision (0 FP64 V-cycles,
 *            1 FP32 V-cycles with FP64 refinement), reinit with lambda correction (1/0)}. */
typedef struct scihpc_twophase scihpc_twophase;
int scihpc_twophase_create(const scihpc_grid *grid, const int vel_bc[6], const int scalar_bc[6], const double prm[16],
                           const int opt[5], scihpc_twophase **out);
int scihpc_twophase_destroy(scihpc_twophase *tp);
/* Copy one named field between HOST memory and the device state (synchronous).  Names:
 * phi, p, p_old, p_old2, u, v, w (staggered velocity), nu, nv, nw (node velocity), rho,
 * mu, delta, heaviside, curvature, sign, grad, u_src, v_src, w_src, u_src_old, v_src_old,
 * w_src_old, rhs, p_flux (the pressure's flux array: pressure_guess_solution's output),
 * rhs_fpc (init_ppe_fpc_coefficients' right-hand-side term). */
int scihpc_twophase_upload(scihpc_twophase *tp, const char *name, const double *host);
int scihpc_twophase_download(scihpc_twophase *tp, const char *name, double *host);
/* The same for n fields at once: one asynchronous copy per field on the session's stream and a
 * single synchronisation before returning (the host buffers may be reused on return), instead
 * of one round trip per field.  Every name is checked before any copy starts.  Like the
 * single-field calls these have no counterpart in the reference, whose fields live in host
 * memory (scalar_data.h). */
int scihpc_twophase_upload_many(scihpc_twophase *tp, int n, const char *const *names, const double *const *host);
int scihpc_twophase_download_many(scihpc_twophase *tp, int n, const char *const *names, double *const *host);
/* Device pointer of a named field (for zero-copy use by callers). */
int scihpc_twophase_field(scihpc_twophase *tp, const char *name, double **dev);
/* Scalars {t, dt, dt_old, dt_old2, iter, stable_CFL, lsf_mass0}. */
int scihpc_twophase_get_scalars(scihpc_twophase *tp, double out[7]);
/* Checkpoint / restart: every device field of the session and its step scalars written to
 * `path`, or read back into a session created with the same grid (anything else is refused
 * with SCIHPC_ERR_ARG).  A restored session continues bit for bit.  Synchronise the
 * session's stream.  New: the reference writes only VTK output. */
int scihpc_twophase_checkpoint(scihpc_twophase *tp, const char *path);
int scihpc_twophase_restore(scihpc_twophase *tp, const char *path);
int scihpc_twophase_set_scalars(scihpc_twophase *tp, const double in[7]);
/* Start-up of the drivers: scalar BC, find_source, lsf_mass0
 * (benchmarks_2d_bubble_rising.cpp:51,88-89). */
int scihpc_twophase_init(scihpc_twophase *tp);
/* Pieces of the step, for parity checks of each stage:
 * find_dt (wrapper_func.cpp:335-385); tvd_rk3 with convection (runge_kutta.cpp:13-49,
 * source.cpp:8-40); `count` Euler steps with mpls (runge_kutta.cpp:51-63, source.cpp:109-154);
 * the reinitialisation loop with lsf_redistance_lambda (benchmarks_2d_bubble_rising.cpp:
 * 122-129, source.cpp:156-241), returning its RK3 step count in *steps; find_source
 * (projection_method.cpp:244-312); ab_solve with the multigrid pressure solve
 * (projection_method.cpp:755-777), returning the solver's iterations and relative
 * residual. */
int scihpc_twophase_find_dt(scihpc_twophase *tp);
int scihpc_twophase_advect(scihpc_twophase *tp);
int scihpc_twophase_mpls(scihpc_twophase *tp, int count);
int scihpc_twophase_reinit(scihpc_twophase *tp, int *steps);
int scihpc_twophase_find_source(scihpc_twophase *tp);
int scihpc_twophase_ab_solve(scihpc_twophase *tp, int *iters, double *relres);
/* The stages of ab_solve one at a time, for callers that compose them as the reference's
 * projection_method does: find_intermediate_velocity (AB2 predictor and velocity boundary
 * fill, projection_method.cpp:384-402); projection (right-hand side div(u*)/dt, the
 * pressure equation of init_ppe_proj_coefficients solved to ppe_tol, pressure boundary fill,
 * velocity correction, projection_method.cpp:404-465,544-657); node_from_face (node
 * velocity from the faces and its boundary fill, wrapper_func.cpp:177-293).  Each
 * synchronises the session's stream. */
int scihpc_twophase_intermediate_velocity(scihpc_twophase *tp);
int scihpc_twophase_projection(scihpc_twophase *tp, int *iters, double *relres);
int scihpc_twophase_node_from_face(scihpc_twophase *tp);
/* Pressure schedule of ab_solve and of the time step.  schedule 0 (default): the projection
 * equation above every step.  schedule 1: the reference's schedule (projection_method.cpp:
 * 755-777): the projection equation while iter < 5, then pressure_guess_solution,
 * init_ppe_fpc_coefficients and fast_pressure_correction, each solve repeated ppe_initer
 * times.  tol_mode 0: ppe_tol is a relative residual; 1: the absolute residual 2-norm, as the
 * reference's loops test it.  The fast correction is capped at 100 iterations as the
 * reference's loop is (:697); its solver is allocated here (not during capture). */
int scihpc_twophase_set_ppe_schedule(scihpc_twophase *tp, int schedule, int tol_mode);
/* The stages of the fast pressure correction one at a time:
 * pressure_guess_solution (projection_method.cpp:803-815): the pressure's flux array =
 * old + dt_old (old - old2) / dt_old2 on every cell;
 * init_ppe_fpc_coefficients (:467-541): the right-hand-side term sum_f C_f (ph_nb - ph_c),
 * C_f = (1 - density_ratio / rho_f) / d^2, from that flux array and the density;
 * fast_pressure_correction (:659-753): the constant-coefficient equation (the multigrid's
 * Neumann operator, multigrid_base.cpp:236-291) with right-hand side density_ratio / dt
 * div(u*) + that term, solved to ppe_tol (tol_mode of set_ppe_schedule) in at most 100
 * iterations, the pressure boundary fill and the velocity correction
 * u -= dt ((dp - dph) / density_ratio + dph / rho_f).  Each synchronises the session's
 * stream. */
int scihpc_twophase_pressure_guess(scihpc_twophase *tp);
int scihpc_twophase_fpc_coefficients(scihpc_twophase *tp);
int scihpc_twophase_fast_pressure_correction(scihpc_twophase *tp, int *iters, double *relres);
/* Finer-grained stages for callers that drive the reinitialisation loop themselves, as the
 * reference drivers do (benchmarks_2d_bubble_rising.cpp:122-129): find_sign
 * (wrapper_func.cpp:387-402); one runge_kutta::tvd_rk3 step (runge_kutta.cpp:13-49) with
 * lsf_redistance_lambda (lambda = 1) or lsf_redistance_no_lambda (lambda = 0)
 * (source.cpp:156-241); and the convection scheme advect() uses: 0 = convection with UCCD
 * (source.cpp:8-40), 1 = WENO5 (weno_solver.cpp:270-278). */
int scihpc_twophase_find_sign(scihpc_twophase *tp);
int scihpc_twophase_reinit_step(scihpc_twophase *tp, int lambda);
int scihpc_twophase_set_scheme(scihpc_twophase *tp, int scheme);
/* find_source's derivatives (and so ab_solve's): 0 the compact CCD / UCCD schemes (default,
 * projection_method.cpp:244-312), 1 second_order_solver -- find_source_sec / ab_solve_sec
 * (projection_method.cpp:314-382, 779-801; source.cpp:42-73). */
int scihpc_twophase_set_source_scheme(scihpc_twophase *tp, int scheme);
/* nsteps time steps of the drivers' loop (benchmarks_2d_bubble_rising.cpp:100-130):
 * find_dt, advection, mass correction, ab_solve, reinitialisation.  use_graph = 1 replays
 * a captured CUDA graph per step (the pressure solve iterates inside it under a device-side
 * convergence test).  Asynchronous on the problem's own stream unless `sync`. */
int scihpc_twophase_step(scihpc_twophase *tp, int nsteps, int use_graph, int sync);
/* lsf_mass, lsf_volume and the maximum |div u| (wrapper_func.cpp:295-333,450-572),
 * on the host (synchronises). */
int scihpc_twophase_diagnostics(scihpc_twophase *tp, double out[3]);
/* The problem's CUDA stream (cudaStream_t as void*). */
int scihpc_twophase_stream(scihpc_twophase *tp, void **stream);
/* Kernel nodes of the captured step graph {before the pressure loop, per pressure
 * iteration, after it} and the pressure iterations summed over all steps so far
 * (out[3]).  Measurement hook with no reference counterpart. */
int scihpc_twophase_graph_stats(scihpc_twophase *tp, long long out[4]);
/* Statistics of the last pressure solve: {iterations, relative residual, ms}. */
int scihpc_twophase_ppe_stats(scihpc_twophase *tp, double out[3]);
/* Measurement hooks with no reference counterpart.  time_reinit_gradient: ms per launch of
 * the reinitialisation's gradient kernel (Godunov |grad phi|, the redistance source and the
 * lambda fields, godunov_gradient.cpp:7-157 and source.cpp:157-198), n back-to-back launches
 * timed with CUDA events on the session's stream (synchronises).  measure_fp64_peak: FP64
 * TFLOP/s of chains of fused multiply-adds over all SMs (best of 5 launches; allocates and
 * synchronises the device). */
int scihpc_twophase_time_reinit_gradient(scihpc_twophase *tp, int n, float *ms);
int scihpc_measure_fp64_peak(double *tflops);

/* ------------------------------------------------------------------ tensor-core convolutions
 * 3x3 convolution, stride 1, zero padding 1, as implicit GEMM on the tcgen05 tensor cores
 * (BF16 operands, FP32 accumulation).  No reference counterpart: building blocks of the
 * learned pressure guess below.  x: BF16 [h*w][ci] (channels fastest), w: BF16 [co][9][ci]
 * (tap t = 3 (dy+1) + (dx+1)), bias: FP32 [co] or NULL, out: FP32 [h*w][co]; ci, co multiples
 * of 16, co <= 256.  conv3x3_wgrad: dw[co][9][ci] = sum_p x[p + off(t)][ci] dz[p][co], dz BF16
 * [h*w][co], partial: splits * 9 * ci * co floats of scratch.  Device pointers; synchronous. */
int scihpc_conv3x3(const void *x, const void *w, const float *bias, float *out, int h, int w_, int ci, int co, int relu,
                   void *stream);
int scihpc_conv3x3_wgrad(const void *x, const void *dz, float *dw, float *partial, int splits, int h, int w_, int ci,
                         int co, void *stream);
/* The same in 3D: x BF16 [d*h*w][ci], w BF16 [co][27][ci] (tap t = 9 (dz+1) + 3 (dy+1) +
 * (dx+1)), out FP32 [d*h*w][co]; wgrad: dw[co][27][ci], partial: splits * 27 * ci * co floats. */
int scihpc_conv3x3x3(const void *x, const void *w, const float *bias, float *out, int d, int h, int w_, int ci, int co,
                     int relu, void *stream);
int scihpc_conv3x3x3_wgrad(const void *x, const void *dz, float *dw, float *partial, int splits, int d, int h, int w_,
                           int ci, int co, void *stream);

/* ------------------------------------------------------------------ learned pressure guess
 * A 4-level 2D U-Net (16-32-64-128 channels) predicting the pressure of the variable-density
 * Poisson equation from (density, right-hand side, previous pressure) on an h x w grid (h, w
 * multiples of 8); every convolution, forward and backward, runs on the tensor cores.  No
 * reference counterpart (the reference has no learned component).  Fields are FP64 ghosted
 * 2D arrays of a grid with n = (h, w) (the pressure solver's layout); pprev may be NULL.
 * The network runs on its own stream (scihpc_unet_stream): inputs must be complete before
 * a call.  infer writes guess = pprev + s * net(...); the pressure solve then starts from
 * guess and iterates to its tolerance as usual.  loss_grad / train_step fit the network to a
 * solved pressure p (mean-squared error of the normalised correction; train_step adds one
 * Adam step with learning rate lr).  Weights and gradients move as FP32 host arrays of
 * scihpc_unet_num_params entries. */
typedef struct scihpc_unet scihpc_unet;
int scihpc_unet_create(int h, int w, unsigned seed, scihpc_unet **out);
/* The same 2D network run on the h x w pressure grid coarsened factor x factor (h / factor
 * and w / factor multiples of 8): its inputs are, per coarse pixel, the mean density, the
 * mean residual of pprev in the pressure equation (face coefficients 2 / (rho_c + rho_nb) /
 * d^2) and the mean pprev; it predicts the mean error p - pprev per coarse pixel (training
 * target and loss on the coarse grid, in units of a tenth of the residual's rms), and infer
 * adds that prediction, interpolated bilinearly to the cells, to pprev.  The other
 * scihpc_unet_* calls are unchanged. */
int scihpc_unet_create_coarse(int h, int w, int factor, unsigned seed, scihpc_unet **out);
/* The 3D network for an n0 x n1 x n2 pressure grid (each a multiple of 8): a 3-level U-Net
 * (16-32-64 channels, 3x3x3 convolutions on the tensor cores) at half the grid's resolution
 * (inputs averaged over 2 x 2 x 2 cells, the correction prolonged piecewise-constant).  The
 * other scihpc_unet_* functions take the same arguments for either network; fields are FP64
 * ghosted 3D arrays of the pressure grid. */
int scihpc_unet_create3(int n0, int n1, int n2, unsigned seed, scihpc_unet **out);
int scihpc_unet_destroy(scihpc_unet *u);
int scihpc_unet_num_params(scihpc_unet *u, long long *n);
int scihpc_unet_set_weights(scihpc_unet *u, const float *host, long long n);
int scihpc_unet_get_weights(scihpc_unet *u, float *host, long long n);
int scihpc_unet_get_gradient(scihpc_unet *u, float *host, long long n);
int scihpc_unet_infer(scihpc_unet *u, const scihpc_grid *grid, const double *rho, const double *rhs,
                      const double *pprev, double *guess);
int scihpc_unet_loss_grad(scihpc_unet *u, const scihpc_grid *grid, const double *rho, const double *rhs,
                          const double *pprev, const double *p, double *loss);
int scihpc_unet_train_step(scihpc_unet *u, const scihpc_grid *grid, const double *rho, const double *rhs,
                           const double *pprev, const double *p, float lr, double *loss);
int scihpc_unet_stream(scihpc_unet *u, void **stream);

#ifdef __cplusplus
}
#endif

#endif /* SCIHPC_GPU_H */
