// vector_data.h -- three scalar_data components (reference scihpc/vector_data.h:10-21).
#ifndef SCIHPC_GB300_VECTOR_DATA_H
#define SCIHPC_GB300_VECTOR_DATA_H

#include "scalar_data.h"

class vector_data {
public:
    explicit vector_data(int _nx);
    vector_data(int _nx, int _ny);
    vector_data(int _nx, int _ny, int _nz);

    scalar_data x, y, z;

    void store();
};

#endif
