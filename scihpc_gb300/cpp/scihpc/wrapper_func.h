// wrapper_func.h -- field operations on wrappers (reference scihpc/wrapper_func.h:14-48).
// Reductions (lsf_mass, lsf_volume, divergence) run on the GPU; l2norm / linfity / store_tmp
// compare against a host snapshot.
#ifndef SCIHPC_GB300_WRAPPER_FUNC_H
#define SCIHPC_GB300_WRAPPER_FUNC_H

#include "global.h"
#include "lsm.h"
#include "structured_grid.h"
#include "wrapper.h"

void find_sign(wrapper *lsf);

void find_dt(wrapper *vel);

DataType lsf_mass(wrapper *f);

DataType lsf_volume(wrapper *f);

DataType divergence(wrapper *vel);

void store_tmp(wrapper *f);

DataType l2norm(wrapper *f);

DataType linfity(wrapper *f);

#endif
