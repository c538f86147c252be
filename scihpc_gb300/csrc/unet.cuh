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

    int create(int h, int w, unsigned seed);
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
    long long nparam = 0, woff[NL] = {}, boff[NL] = {}, wb_off[NL] = {};
    float *wmaster = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    __nv_bfloat16 *wb = nullptr, *wt = nullptr, *dz = nullptr;
    void *act[NT] = {};
    float *gact[NT] = {};
    float *gskip[3] = {nullptr, nullptr, nullptr};
    float *partial = nullptr, *target = nullptr;
    double *stats = nullptr;
    int *err = nullptr;
    long long adam_t = 0;
    std::vector<void *> allocs;
};

}  // namespace scihpc
