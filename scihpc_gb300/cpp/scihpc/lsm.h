// lsm.h -- smoothed level-set functions (reference scihpc/lsm.h:12-16; lsm.cpp:8-43).
#ifndef SCIHPC_GB300_LSM_H
#define SCIHPC_GB300_LSM_H

#include "global.h"

DataType Heaviside(DataType x, DataType ls_width);

DataType Delta(DataType x, DataType ls_width);

DataType Sign(const DataType &x, const DataType &ls_width);

#endif
