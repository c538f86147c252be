// structured_grid.h -- uniform cell-centred grid (reference scihpc/structured_grid.h:10-30).
#ifndef SCIHPC_GB300_STRUCTURED_GRID_H
#define SCIHPC_GB300_STRUCTURED_GRID_H

#include "global.h"

class structured_grid {
public:
    explicit structured_grid(axis x_data);
    structured_grid(axis x_data, axis y_data);
    structured_grid(axis x_data, axis y_data, axis z_data);

    DataType *x, *xc;
    DataType *y, *yc;
    DataType *z, *zc;
    DataType dx, dy, dz, h, dv;

    axis x_axis, y_axis, z_axis;
    int ndim;

    struct {
        DataType xstart, ystart, zstart;
        int nx, ny, nz;
    } vtk_info;
};

#endif
