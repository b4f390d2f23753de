// tc_host.hpp -- host-side error plumbing shared by the translation units.
#pragma once

#include <cstdio>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "tc_internal.cuh"

namespace tc {

void set_last_error(const std::string& msg);

// Number of kernels this library has launched (all devices, since load).
void count_launch();

// Evaluate a CUDA runtime call; on failure record the message and return TC_ERR_CUDA (2).
#define TC_CU(call)                                                                        \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            ::tc::set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));      \
            return 2;                                                                      \
        }                                                                                  \
    } while (0)

// Propagate a non-zero status.
#define TC_TRY(expr)                                                                       \
    do {                                                                                   \
        int s_ = (expr);                                                                   \
        if (s_ != 0) return s_;                                                            \
    } while (0)

// Device allocation that records a message and returns TC_ERR_NOMEM (5) on failure.
template <class T>
int dalloc(T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        set_last_error(std::string("cudaMalloc of ") + std::to_string(count * sizeof(T)) +
                       " bytes failed: " + cudaGetErrorString(e));
        return 5;
    }
    return 0;
}

template <class T>
void dfree(T*& p)
{
    if (p) cudaFree(p);
    p = nullptr;
}

// Tree build (tree_build.cu).
int build_tree(const BuildParams& BP, Points bufs[2], Cells C, int* d_tops, int* d_ntop,
               BuildScratch& S, cudaStream_t st, std::vector<int>& tops_out, int* d_err,
               int mintop, int maxtop);
int field_center(const BuildParams& BP, Points P, BuildScratch& S, cudaStream_t st,
                 double out[4]);
void launch_prepare(int n, int coords, int dkind, const double* x, const double* y,
                    const double* z, const double* d1, const double* d2, const double* w,
                    const double* wpos, Points P, cudaStream_t st);
int scratch_ensure_level(BuildScratch& S, int nt, int nc);
int tcgen05_selftest(const float* A, const float* B, float* C, int N, int K, cudaStream_t st);
void launch_validate_tree(int ncap, const Cells& C, const int* tops, int ntop, int* err,
                          cudaStream_t st);

}  // namespace tc
