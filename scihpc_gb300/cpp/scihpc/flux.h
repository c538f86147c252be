// flux.h -- flux functions passed to runge_kutta (reference scihpc/flux.h:12-49).  On the GPU
// the flux of the two-phase path is the level set itself (identity_flux), applied inside
// the fused stage kernels; the functions exist so that drivers can pass their addresses.
#ifndef SCIHPC_GB300_FLUX_H
#define SCIHPC_GB300_FLUX_H

#include "global.h"
#include "scalar_data.h"
#include "vector_data.h"

void identity_flux(scalar_data *f, vector_data *vel);
void identity_flux(scalar_data *f);
void identity_flux(vector_data *vel);

#endif
