// wrapper_func.h -- field operations on wrappers (reference scihpc/wrapper_func.h:14-48).
// Reductions (lsf_mass, lsf_volume, divergence) run on the GPU; l2norm / linfity / store_tmp
// compare against a host snapshot.  The property fields (find_heavyside, find_delta,
// find_density, find_viscosity, find_curvature) are computed on the GPU from the host level
// set (and, for the curvature, its CCD derivative arrays) and written to the wrapper's
// dummy arrays on the host.  node_from_face runs on the session of the velocities.
// find_gradient and all_to_face_{x,y,z} are stages inside the GPU find_source and report
// SCIHPC_ERR_UNSUPPORTED when called alone.
#ifndef SCIHPC_GB300_WRAPPER_FUNC_H
#define SCIHPC_GB300_WRAPPER_FUNC_H

#include "global.h"
#include "lsm.h"
#include "structured_grid.h"
#include "wrapper.h"

void find_heavyside(wrapper *lsf);

void find_delta(wrapper *lsf);

void find_sign(wrapper *lsf);

void find_gradient(wrapper *lsf);

void find_curvature(wrapper *lsf);

void find_density(wrapper *lsf);

void find_viscosity(wrapper *lsf);

void all_to_face_x(wrapper *ref, wrapper *tgt);

void all_to_face_y(wrapper *ref, wrapper *tgt);

void all_to_face_z(wrapper *ref, wrapper *tgt);

void node_from_face(wrapper *ref, wrapper *tgt);

void find_dt(wrapper *vel);

DataType lsf_mass(wrapper *f);

DataType lsf_volume(wrapper *f);

DataType divergence(wrapper *vel);

void store_tmp(wrapper *f);

DataType l2norm(wrapper *f);

DataType linfity(wrapper *f);

#endif
