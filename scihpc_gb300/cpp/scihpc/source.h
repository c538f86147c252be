// source.h -- right-hand sides passed to runge_kutta (reference scihpc/source.h:14-19).
// runge_kutta recognises them by address and runs the matching fused GPU stages:
// convection (source.cpp:8-40, UCCD), mpls (source.cpp:109-154), lsf_redistance_lambda /
// lsf_redistance_no_lambda (source.cpp:156-241), Hamilton_Jacobi (source.cpp:75-107: s = -sum
// of the UCCD derivatives of the flux, upwinded by the velocity).  convection_weno is the WENO5
// (weno_solver.cpp:270-278) variant of convection, convection_sec (source.cpp:42-73) the
// second_order_solver one.  Called directly they report
// SCIHPC_ERR_UNSUPPORTED through scihpc_cpp_last_status(): the GPU path evaluates them only
// inside the time integrator.
#ifndef SCIHPC_GB300_SOURCE_H
#define SCIHPC_GB300_SOURCE_H

#include "flux.h"
#include "global.h"
#include "wrapper.h"

typedef void (*scihpc_flux_fn)(scalar_data *, vector_data *);

void convection(wrapper *f, wrapper *vel, DataType ***s, void (*flux)(scalar_data *, vector_data *));
void convection_weno(wrapper *f, wrapper *vel, DataType ***s, void (*flux)(scalar_data *, vector_data *));
void convection_sec(wrapper *f, wrapper *vel, DataType ***s, void (*flux)(scalar_data *, vector_data *));
void Hamilton_Jacobi(wrapper *f, wrapper *vel, DataType ***s, void (*flux)(scalar_data *, vector_data *));
void mpls(wrapper *phi, wrapper *vel, DataType ***s, void (*flux)(scalar_data *, vector_data *));
void lsf_redistance_no_lambda(wrapper *phi, wrapper *vel, DataType ***s, void (*flux)(scalar_data *, vector_data *));
void lsf_redistance_lambda(wrapper *phi, wrapper *vel, DataType ***s, void (*flux)(scalar_data *, vector_data *));

#endif
