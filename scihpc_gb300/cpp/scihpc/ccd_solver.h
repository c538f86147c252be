// ccd_solver.h -- central combined compact difference derivatives (reference
// scihpc/ccd_solver.h:17-39) on the GPU.  Each call reads the scalar's host arrays (flux, or
// the first derivative for the mixed ones), runs the block-tridiagonal line solves on the
// device (scihpc_ccd / scihpc_ccd_mixed) and writes the derivative arrays back on the host.
// The coefficient tables live in the device context of the grid.
#ifndef SCIHPC_GB300_CCD_SOLVER_H
#define SCIHPC_GB300_CCD_SOLVER_H

#include "global.h"
#include "scalar_data.h"
#include "structured_grid.h"
#include "vector_data.h"

class ccd_solver {
public:
    ccd_solver(scalar_data *f, structured_grid *geo);

    void find_fx(scalar_data *f) const;
    void find_fy(scalar_data *f) const;
    void find_fz(scalar_data *f) const;
    void mixed_xy(scalar_data *f) const;
    void mixed_yz(scalar_data *f) const;
    void mixed_zx(scalar_data *f) const;
    void find_derivatives(scalar_data *f) const;
    void find_derivatives(vector_data *f) const;
    void find_derivatives_all(scalar_data *f) const;
    void find_derivatives_all(vector_data *f) const;

    structured_grid *geo;
};

#endif
