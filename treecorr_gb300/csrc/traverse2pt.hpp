// traverse2pt.hpp -- parameters and launchers of the 2-point traversal.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "tc_internal.cuh"

namespace tc {

struct TravParams {
    int coords, metric, dkind, quick, nbins, autoc;
    int nqf;                      // FP32 bin quantities: weight, meanr, meanlogr, xi...
    // FP64 constants (escalation path), BaseCorr2 constructor src/Corr2.cpp:55-80.
    double minsep, maxsep, binsize, b, a, logminsep, halfminsep, minsepsq, maxsepsq, bsq, asq;
    // FP32 copies.
    float fminsep, fmaxsep, fbinsize, fb, fminsepsq, fmaxsepsq, fbsq, fasq, fbb, fmineff;
    float finvminsepsq, finvbinsize, flogminsep;
    // Cells.
    const TCell* c1;
    const TCell* c2;
    const double *x1, *y1, *z1, *x2, *y2, *z2;
    // Roots: ngen generated top pairs, then nin explicit items.
    const int* tops1;
    const int* tops2;
    long long ntop1, ntop2, ngen, nin;
    const int2* in_tasks;
    unsigned long long* root_next;
    // Spill list for the next launch.
    int2* out_tasks;
    unsigned long long* nout;
    long long out_cap;
    // Per-warp stacks and accumulators.
    int2* stacks;
    int stack_cap;
    int nwarps;
    int* idle;
    double* wacc;
    unsigned long long* wnp;
    unsigned long long* counters;   // [0] evaluated, [1] accepted, [2] escalated
    int* err;
};

void launch_pack_cells(int ncap, const Cells& C, TCell* out, cudaStream_t st);
size_t traverse_smem_bytes(int nq, int nb);
int traverse_grid(int nq, int nb, int* blocks, int* nwarps);
int launch_traverse(const TravParams& T, int blocks, cudaStream_t st);
int launch_reduce(int nwarps, int nq, int nb, const double* wacc, const unsigned long long* wnp,
                  double* out, unsigned long long* outnp, cudaStream_t st);

}  // namespace tc
