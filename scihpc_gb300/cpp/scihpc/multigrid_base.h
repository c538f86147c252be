// multigrid_base.h -- one level of the reference's multigrid (scihpc/multigrid_base.h:17-55),
// GPU-backed.  The finest level's rhs / sol live on the host as in the reference (x fastest,
// of(i, j, k) = i + j nx + k nx ny); relax, residual and the cycles of the owning multigrid
// run on the GPU solver of scihpc_gpu.h (scihpc_poisson_*), which keeps the whole hierarchy
// on the device.  The coarser levels report their sizes; their vectors stay empty and their
// solver steps (restriction, prolongation, solve, Ax) are internal to the GPU cycle and report
// SCIHPC_ERR_UNSUPPORTED through scihpc_cpp_last_status().
#ifndef SCIHPC_GB300_MULTIGRID_BASE_H
#define SCIHPC_GB300_MULTIGRID_BASE_H

#include <algorithm>
#include <vector>

#include "global.h"

// dense vector with the element access of the reference's Eigen VectorX
class VectorX {
public:
    VectorX() = default;
    explicit VectorX(long n) : v_(size_t(n), 0.0) {}
    DataType &operator[](long i) { return v_[size_t(i)]; }
    const DataType &operator[](long i) const { return v_[size_t(i)]; }
    DataType &operator()(long i) { return v_[size_t(i)]; }
    const DataType &operator()(long i) const { return v_[size_t(i)]; }
    DataType &coeffRef(long i) { return v_[size_t(i)]; }
    long size() const { return long(v_.size()); }
    void resize(long n) { v_.assign(size_t(n), 0.0); }
    void setZero() { std::fill(v_.begin(), v_.end(), 0.0); }
    DataType norm() const;
    DataType *data() { return v_.data(); }
    const DataType *data() const { return v_.data(); }

private:
    std::vector<DataType> v_;
};

class multigrid;

class multigrid_base {
public:
    multigrid_base(int _nx, int _ny, int _degree, DataType _dx, DataType _dy);

    multigrid_base(int _nx, int _ny, int _nz, int _degree, DataType _dx, DataType _dy, DataType _dz);

    void init_NeumannBC();
    void init_DirichletBC();

    VectorX rhs, sol, res, buffer;

    int nx, ny, nz, degree, ndim, n;
    DataType dx, dy, dz;
    bool no_compatibility = false;

    int base_step = 10;

    int of(int i, int j, int k);

    int of(int i, int j);

    void Ax(const VectorX &x);

    void compatibility_condition(VectorX &f);

    // `iter` solver iterations on the GPU from the current sol (finest level)
    void relax(int iter);

    // ||rhs - A sol|| on the GPU (finest level)
    DataType residual();

    void restriction(multigrid_base *coarse);

    void prolongation(multigrid_base *dense);

    void solve();

    multigrid *owner = nullptr;   // set by multigrid
    int level = 0;
};

#endif
