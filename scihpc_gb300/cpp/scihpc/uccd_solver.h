// uccd_solver.h -- upwind combined compact difference derivatives (reference
// scihpc/uccd_solver.h:17-27) on the GPU: from the scalar's flux and the velocity
// component along the axis, fx (upwind-selected) and fxx (mean of the two biased solves) on
// the host arrays, computed by scihpc_uccd.
#ifndef SCIHPC_GB300_UCCD_SOLVER_H
#define SCIHPC_GB300_UCCD_SOLVER_H

#include "global.h"
#include "scalar_data.h"
#include "structured_grid.h"
#include "vector_data.h"

class uccd_solver {
public:
    uccd_solver(scalar_data *f, structured_grid *geo);

    void find_fx(scalar_data *f, vector_data *vel) const;
    void find_fy(scalar_data *f, vector_data *vel) const;
    void find_fz(scalar_data *f, vector_data *vel) const;
    void find_derivatives(scalar_data *f, vector_data *vel) const;

    structured_grid *geo;
};

#endif
