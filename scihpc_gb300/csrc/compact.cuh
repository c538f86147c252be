// compact.cuh -- factored CCD / UCCD line operators held on the device (see compact.cu).
#pragma once

#include "common.cuh"

namespace scihpc {

struct CompactOps {
    double *ccd[3] = {nullptr, nullptr, nullptr};
    double *up[3] = {nullptr, nullptr, nullptr};
    double *down[3] = {nullptr, nullptr, nullptr};
    // scan form for linescan.cu: per point {L (4), K = -Dinv U (4), Dinv (4)}
    double *scan_ccd[3] = {nullptr, nullptr, nullptr};
    double *scan_up[3] = {nullptr, nullptr, nullptr};
    double *scan_down[3] = {nullptr, nullptr, nullptr};
    int build(const Dims &D);
    void release();
};

// uccd_solver::find_f{x,y,z}: t1/t2 are scratch fields for the down-wind system.
void launch_uccd(const Dims &D, const CompactOps &ops, int a, const double *flux, const double *vel, double *f1,
                 double *f2, double *t1, double *t2, cudaStream_t s);
// ccd_solver::find_f{x,y,z}
void launch_ccd(const Dims &D, const CompactOps &ops, int a, const double *flux, double *f1, double *f2,
                cudaStream_t s);
// ccd_solver::mixed_{xy,yz,zx}: src extrapolated along a in place; tmp is a scratch field.
void launch_ccd_mixed(const Dims &D, const CompactOps &ops, int a, double *src, double *out, double *tmp,
                      cudaStream_t s);

// Warp-cooperative solves (linescan.cu); false when the line is too long for them.
bool scan_uccd(const Dims &D, const CompactOps &ops, int a, const double *flux, const double *vel, double *f1,
               double *f2, cudaStream_t s);
bool scan_ccd(const Dims &D, const CompactOps &ops, int a, const double *flux, double *f1, double *f2,
              cudaStream_t s);
bool scan_mixed(const Dims &D, const CompactOps &ops, int a, double *src, double *out, cudaStream_t s);

}  // namespace scihpc
