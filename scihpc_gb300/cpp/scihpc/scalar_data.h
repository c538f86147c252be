// scalar_data.h -- ghosted field storage (reference scihpc/scalar_data.h:10-32).  The host
// arrays mirror device fields once a GPU session owns the field: the session uploads them
// when it starts and downloads them on scihpc_sync_to_host (and before every VTK write).
#ifndef SCIHPC_GB300_SCALAR_DATA_H
#define SCIHPC_GB300_SCALAR_DATA_H

#include "global.h"

class scalar_data {
public:
    int ghc = 3;
    int Nx, Ny, Nz;
    int nx, ny, nz;
    int ndim;

    DataType ***data, ***flux, ***old, ***old2;
    DataType ***fx, ***fy, ***fz;
    DataType ***fxx, ***fyy, ***fzz;
    DataType ***fxy, ***fyz, ***fzx;

    explicit scalar_data(int _nx);
    scalar_data(int _nx, int _ny);
    scalar_data(int _nx, int _ny, int _nz);

    indices index_mapping(int i, int j, int k);

    void store() const;

private:
    void alloc();
};

#endif
