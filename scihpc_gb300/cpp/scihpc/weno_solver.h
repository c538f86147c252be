// weno_solver.h -- WENO5 (WENO-Z weights) derivatives (reference scihpc/weno_solver.h:30-47)
// on the GPU: from the scalar's flux and the velocity component along the axis, the upwinded
// face values and their difference on interior cells (scihpc_weno5), written to the host
// derivative array; ghost cells of the derivative keep their values.  The face-value
// stages weno5_flux_{x,y,z} and their fp / fm / fh arrays are internal to the GPU kernel.
#ifndef SCIHPC_GB300_WENO_SOLVER_H
#define SCIHPC_GB300_WENO_SOLVER_H

#include "global.h"
#include "scalar_data.h"
#include "structured_grid.h"
#include "vector_data.h"

class weno_solver {
public:
    weno_solver(scalar_data *f, structured_grid *geo);

    DataType dx, dy, dz;

    void weno5_flux_x(scalar_data *f);
    void weno5_flux_y(scalar_data *f);
    void weno5_flux_z(scalar_data *f);
    void weno5_find_fx(scalar_data *f, vector_data *vel);
    void weno5_find_fy(scalar_data *f, vector_data *vel);
    void weno5_find_fz(scalar_data *f, vector_data *vel);
    void weno5_find_derivatives(scalar_data *f, vector_data *vel);

    structured_grid *geo;
};

#endif
