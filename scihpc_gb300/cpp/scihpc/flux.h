// flux.h -- flux functions (reference scihpc/flux.h:12-49).  Passed to runge_kutta, only
// identity_flux has a GPU stage: the fused stage kernels read the level set itself.  Called
// directly on host arrays: identity_flux / identity_old_flux copy data (or old) into flux
// (after the current values of a GPU-owned array are brought to the host);
// identity_with_extrapolation and its face variants (and the _old_ ones) copy with the
// zero-order ghost extrapolation of flux.cpp:98-650 on the GPU (scihpc_flux_extrapolate).
// guess_from_history (2 old - old2) has no GPU stage and reports SCIHPC_ERR_UNSUPPORTED.
#ifndef SCIHPC_GB300_FLUX_H
#define SCIHPC_GB300_FLUX_H

#include "global.h"
#include "scalar_data.h"
#include "vector_data.h"

void identity_flux(scalar_data *f, vector_data *vel);
void identity_flux(scalar_data *f);
void identity_flux(vector_data *vel);

void identity_old_flux(scalar_data *f, vector_data *vel);
void identity_old_flux(scalar_data *f);
void identity_old_flux(vector_data *vel);

void guess_from_history(scalar_data *f);

// burgers_flux (flux.cpp:86-96): flux = data^2 / 2 on every cell.  Passed to runge_kutta it
// selects the GPU transport stages; called directly it runs on host arrays (scihpc_flux_fill).
void burgers_flux(scalar_data *f, vector_data *vel);

void identity_with_extrapolation(scalar_data *f, vector_data *vel);
void identity_with_extrapolation(scalar_data *f);
void identity_with_extrapolation(vector_data *vel);
void identity_with_extrapolation_face_x(scalar_data *f);
void identity_with_extrapolation_face_x(vector_data *f);
void identity_with_extrapolation_face_y(scalar_data *f);
void identity_with_extrapolation_face_y(vector_data *f);
void identity_with_extrapolation_face_z(scalar_data *f);
void identity_with_extrapolation_face_z(vector_data *f);
void identity_with_extrapolation_face_x(scalar_data *f, vector_data *vel);
void identity_with_extrapolation_face_y(scalar_data *f, vector_data *vel);
void identity_with_extrapolation_face_z(scalar_data *f, vector_data *vel);

void identity_old_with_extrapolation(scalar_data *f, vector_data *vel);
void identity_old_with_extrapolation(scalar_data *f);
void identity_old_with_extrapolation(vector_data *vel);
void identity_old_with_extrapolation_face_x(scalar_data *f);
void identity_old_with_extrapolation_face_x(vector_data *f);
void identity_old_with_extrapolation_face_y(scalar_data *f);
void identity_old_with_extrapolation_face_y(vector_data *f);
void identity_old_with_extrapolation_face_z(scalar_data *f);
void identity_old_with_extrapolation_face_z(vector_data *f);
void identity_old_with_extrapolation_face_x(scalar_data *f, vector_data *vel);
void identity_old_with_extrapolation_face_y(scalar_data *f, vector_data *vel);
void identity_old_with_extrapolation_face_z(scalar_data *f, vector_data *vel);

#endif
