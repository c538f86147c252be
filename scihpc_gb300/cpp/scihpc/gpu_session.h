// gpu_session.h -- control of the device state behind the reference-style API (no
// reference counterpart).  The wrappers of one problem (those linked to the same
// problem_parameters) share one GPU session, created by the first stage call.  Host arrays
// are copied to the GPU when the session starts; afterwards the GPU holds the current values.
#ifndef SCIHPC_GB300_GPU_SESSION_H
#define SCIHPC_GB300_GPU_SESSION_H

#include "wrapper.h"

// download the session's current values of this wrapper's field(s) into its host arrays
// (and the dummy_data mirrors of the same problem)
void scihpc_sync_to_host(wrapper *w);

// upload the host arrays of this wrapper (after the driver changed them on the host)
void scihpc_sync_to_device(wrapper *w);

// status of the last call of this layer (0 = ok; the codes of scihpc_gpu.h) and its message
int scihpc_cpp_last_status();
const char *scihpc_cpp_last_message();

// pressure precision of sessions created from now on: 1 = FP32 V-cycles in FP64 refinement
// (default), 0 = FP64 V-cycles
void scihpc_cpp_set_pressure_precision(int fp32);

// pressure schedule of sessions created from now on.  schedule 1 (default): ab_solve runs the
// reference's schedule -- projection() while iter < 5, then pressure_guess_solution,
// init_ppe_fpc_coefficients and fast_pressure_correction, ppe_initer times each
// (projection_method.cpp:755-777); schedule 0: projection()'s equation every step.
// tol_mode 1 (default): ppe_tol is an absolute residual 2-norm, as the reference's multigrid
// loop tests it (projection_method.cpp:697); tol_mode 0: a relative residual.  Either way the
// GPU solves run multigrid-preconditioned CG, not SOR sweeps or full_cycle iterations, so
// their iterates differ from the reference's; at convergence the fields agree.
void scihpc_cpp_set_pressure_schedule(int schedule, int tol_mode);

#endif
