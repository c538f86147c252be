// compact.cuh -- factored CCD / UCCD line operators held on the device (see compact.cu).
#pragma once

#include "common.cuh"

namespace scihpc {

struct CompactOps {
    double *ccd[3] = {nullptr, nullptr, nullptr};
    double *up[3] = {nullptr, nullptr, nullptr};
    double *down[3] = {nullptr, nullptr, nullptr};
    // Tables of the warp-cooperative solves (linescan.cu; lane_table in compact.cu): per point
    // {-L (4), K = -Dinv U (4), Dinv (4)} and the matrix halves of the scan maps, laid out for
    // the launch shape scan_shape chose when they were built: lane_wpl warps per line, lane_c
    // points per lane, lines of lane_n points.
    double *lane_ccd[3] = {nullptr, nullptr, nullptr};
    double *lane_up[3] = {nullptr, nullptr, nullptr};
    double *lane_down[3] = {nullptr, nullptr, nullptr};
    int lane_wpl[3] = {0, 0, 0}, lane_c[3] = {0, 0, 0}, lane_n[3] = {0, 0, 0};
    int lane_seg[3] = {32, 32, 32};   // lanes per line: 32, or 16 (two lines per warp)
    int build(const Dims &D);
    void release();
};

// Launch shape of the warp-cooperative solves along axis a: each lane holds a contiguous chunk
// of C points; when there are few lines (fewer than four per SM) two or four warps share one
// line, for shorter FP64 dependency chains and more warps in flight.  False for lines longer
// than 16 points per lane.
inline bool scan_shape(const Dims &D, int a, int &wpl, int &C, int &seg) {
    const long long lines = (long long)D.N[(a + 1) % 3] * D.N[(a + 2) % 3];
    const int n = D.N[a];
    wpl = 1;
    if (lines < 4LL * NUM_SMS) wpl = n >= 192 ? 4 : (n >= 96 ? 2 : 1);
    // many lines of 65-160 points: 16 lanes per line, two lines per warp (chunks of up to 10
    // points: fewer idle lanes than 32 chunks of 3-5, and one shuffle step less); the FP64
    // work per point, not the parallelism, bounds these solves
    seg = wpl == 1 && n > 64 && n <= 160 && lines >= 8LL * NUM_SMS ? 16 : 32;
    C = (n + seg * wpl - 1) / (seg * wpl);
    return C <= 16;
}

// uccd_solver::find_f{x,y,z}: t1/t2 are scratch fields for the down-wind system.
void launch_uccd(const Dims &D, const CompactOps &ops, int a, const double *flux, const double *vel, double *f1,
                 double *f2, double *t1, double *t2, cudaStream_t s);
// ccd_solver::find_f{x,y,z}
void launch_ccd(const Dims &D, const CompactOps &ops, int a, const double *flux, double *f1, double *f2,
                cudaStream_t s);
// ccd_solver::mixed_{xy,yz,zx}: src extrapolated along a in place; tmp is a scratch field.
void launch_ccd_mixed(const Dims &D, const CompactOps &ops, int a, double *src, double *out, double *tmp,
                      cudaStream_t s);

// Sequential solves staged in shared memory, one thread per line and system (linescan.cu):
// 3D grids whose lines leave room for four warps per SM; false (nothing launched) otherwise.
bool seq_uccd(const Dims &D, const CompactOps &ops, int a, const double *flux, const double *vel, double *f1,
              double *f2, cudaStream_t s);
bool seq_ccd(const Dims &D, const CompactOps &ops, int a, const double *flux, double *f1, double *f2,
             cudaStream_t s);
bool seq_mixed(const Dims &D, const CompactOps &ops, int a, double *src, double *out, cudaStream_t s);
// Warp-cooperative solves (linescan.cu); false when the line is too long for them.
bool scan_uccd(const Dims &D, const CompactOps &ops, int a, const double *flux, const double *vel, double *f1,
               double *f2, cudaStream_t s);
bool scan_ccd(const Dims &D, const CompactOps &ops, int a, const double *flux, double *f1, double *f2,
              cudaStream_t s);
bool scan_mixed(const Dims &D, const CompactOps &ops, int a, double *src, double *out, cudaStream_t s);

}  // namespace scihpc
