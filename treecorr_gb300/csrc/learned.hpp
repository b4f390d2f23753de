// learned.hpp -- host interface of the learned opening criterion (learned.cu).
#pragma once

#include <cuda_runtime.h>

#include "tc_internal.cuh"
#include "learned.cuh"

namespace tc {

// Inputs of the label kernel: the two fields' cell records, their points (the build's
// sorted buffer 0, cell c holds points [start[c], start[c] + n)) and the binning.
struct LabelParams {
    int coords, metric, nbins;
    double minsepsq, maxsepsq, logminsep, binsize;
    float finvminsepsq, finvbinsize, finvlogrange, fbinsize;
    long long max_point_pairs;   // larger pairs get no label (NaN target)
    const TCell *c1, *c2;
    const int *start1, *start2;
    const double *x1, *y1, *z1, *x2, *y2, *z2;
    const float *w1, *w2;
};

// FP32 parameters (MLP_NPARAM floats, host) -> packed FP16 fragments on the device
// (allocated on first use).
int mlp_pack(const float* h_params, MLPPacked** d_out, cudaStream_t st);
int launch_label(const LabelParams& L, const int2* pairs, long long n, float* feat,
                 float* target, cudaStream_t st);
// Host-array entry points (tests, training).
int mlp_grad_host(const float* P, const float* X, const float* Y, long long n, float* grad,
                  float* loss, cudaStream_t st);
int mlp_infer_host(const float* P, const float* X, long long n, float* Y, cudaStream_t st);
int mlp_train_host(float* P, const float* X, const float* Y, long long n, int steps, int batch,
                   float lr, unsigned seed, float* loss_out, cudaStream_t st);

}  // namespace tc
