// godunov_gradient.h -- Godunov |grad phi| (reference scihpc/godunov_gradient.h:12-16).
// godunov_gradient(f) writes f->dummy->grad from the level set and f->dummy->sign on the GPU
// (scihpc_godunov_gradient); weno5_for_godunov is the scalar WENO-JS correction of the
// fourth-order central gradient (godunov_gradient.cpp:183-198).
#ifndef SCIHPC_GB300_GODUNOV_GRADIENT_H
#define SCIHPC_GB300_GODUNOV_GRADIENT_H

#include "global.h"
#include "wrapper.h"

DataType weno5_for_godunov(DataType a, DataType b, DataType c, DataType d);

void godunov_gradient(wrapper *f);

// godunov_gradient followed by phi /= max |grad phi|; the rescale has no GPU stage and
// reports SCIHPC_ERR_UNSUPPORTED
void stabilized_upon_gradient(wrapper *f);

#endif
