// unet.cuh -- the learned pressure guess (unet.cu).
#pragma once

#include <vector>

#include <cuda_bf16.h>

#include "common.cuh"

namespace scihpc {

class UNet {
public:
    static constexpr int NL = 15;            // convolution layers
    static constexpr int NT = 22;            // activation tensors
    static constexpr int WGRAD_SPLITS = 64;  // pixel ranges of the weight-gradient GEMMs

    // h, w: the pressure grid; factor 1: the network runs on it; factor F > 1: the network
    // runs on the grid coarsened F x F (the coarse-correction mode of unet.cu)
    int create(int h, int w, unsigned seed, int factor = 1);
    void destroy();
    long long num_params() const { return nparam; }
    int set_weights(const float *host, long long n);
    int get(float *host, long long n, bool gradient);
    // guess = pprev + s * net(rho, rhs, pprev) on a 2D ghosted grid of the network's size
    int infer(const Dims &D, const double *rho, const double *rhs, const double *pprev, double *guess);
    // loss of the prediction against pnew and its gradient in grad (no update)
    int loss_grad(const Dims &D, const double *rho, const double *rhs, const double *pprev, const double *pnew,
                  double *loss);
    // loss_grad followed by one Adam step with learning rate lr
    int train_step(const Dims &D, const double *rho, const double *rhs, const double *pprev, const double *pnew,
                   float lr, double *loss);

    cudaStream_t stream = nullptr;

private:
    int forward();
    int backward();
    int prepare(const Dims &D, const double *rho, const double *rhs, const double *pprev, const double *pnew);
    int check_err();
    int alloc_skip();
    void refresh_bf16();
    float *gconcat(int skip);

    int H[4] = {0, 0, 0, 0}, W[4] = {0, 0, 0, 0};
    int fac = 1, PH = 0, PW = 0;   // coarsening factor and the pressure grid it applies to
    float *cin = nullptr;          // coarse inputs (density, residual, previous pressure) per pixel
    long long nparam = 0, woff[NL] = {}, boff[NL] = {}, wb_off[NL] = {};
    float *wmaster = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    __nv_bfloat16 *wb = nullptr, *wt = nullptr, *dz = nullptr;
    void *act[NT] = {};
    float *gact[NT] = {};
    float *gskip[3] = {nullptr, nullptr, nullptr};
    float *partial = nullptr, *target = nullptr;
    double *stats = nullptr, *dred = nullptr;   // dred: partial sums of the two-pass reductions
    int *err = nullptr;
    long long adam_t = 0;
    std::vector<void *> allocs;
};

// The 3D learned guess (unet3.cu): a 3-level U-Net (16, 32, 64 channels, two 3x3x3 convolutions
// per level) that runs at half the resolution of the pressure grid: the inputs are averaged
// over 2 x 2 x 2 cells and the predicted correction is prolonged piecewise-constant.  Same
// interface and normalisation as UNet.
class UNet3 {
public:
    static constexpr int NL = 11;            // convolution layers
    static constexpr int NT = 16;            // activation tensors
    static constexpr int WGRAD_SPLITS = 64;  // voxel ranges of the weight-gradient GEMMs

    // n0, n1, n2: the pressure grid (each a multiple of 8)
    int create(int n0, int n1, int n2, unsigned seed);
    void destroy();
    long long num_params() const { return nparam; }
    int set_weights(const float *host, long long n);
    int get(float *host, long long n, bool gradient);
    int infer(const Dims &D, const double *rho, const double *rhs, const double *pprev, double *guess);
    int loss_grad(const Dims &D, const double *rho, const double *rhs, const double *pprev, const double *pnew,
                  double *loss);
    int train_step(const Dims &D, const double *rho, const double *rhs, const double *pprev, const double *pnew,
                   float lr, double *loss);

    cudaStream_t stream = nullptr;

private:
    int forward();
    int backward();
    int prepare(const Dims &D, const double *rho, const double *rhs, const double *pprev, const double *pnew);
    int check_err();
    void refresh_bf16();
    long long vox(int level) const { return (long long)G[level][0] * G[level][1] * G[level][2]; }

    int G[3][3] = {};   // network grid of each level (level 0: half the pressure grid)
    long long nparam = 0, woff[NL] = {}, boff[NL] = {}, wb_off[NL] = {};
    float *wmaster = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    __nv_bfloat16 *wb = nullptr, *wt = nullptr, *dz = nullptr;
    void *act[NT] = {};
    float *gact[NT] = {};
    float *gskip[2] = {nullptr, nullptr};
    float *partial = nullptr, *target = nullptr;
    double *stats = nullptr, *dred = nullptr;   // dred: partial sums of the two-pass reductions
    int *err = nullptr;
    long long adam_t = 0;
    std::vector<void *> allocs;
};

}  // namespace scihpc
