// multipole.hpp -- parameters and launchers of the GGG LogMultipole accumulation.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "tc_internal.cuh"

namespace tc {

enum MPErr : int {
    MP_ERR_ARENA = 11,   // a c2-list arena is full
    MP_ERR_JOBS = 12,    // the job list is full
    MP_ERR_SLOTS = 13,   // no free scratch slot for a c1 split
    MP_ERR_STACK = 14,   // a block-local stack is full
};

struct MPParams {
    int coords, metric, quick, nbins, maxn;
    double minsep, maxsep, binsize, b, a, logminsep, minsepsq, maxsepsq, bsq, asq, maxbsq_eff;
    // Cells (FP64 centres, float payloads) and their leaf sums (4 doubles per cell:
    // sum w^2, Re/Im sum (wz)^2, sum |wz|^2).
    const double *x, *y, *z;
    const float *size, *w, *d1, *d2;
    const int *n, *left, *right;
    const double* ls;
    const int* tops;
    int ntop;
    // Phase 1: per-block list arenas and the job list.
    int* arena1;
    long long arena1_cap;
    int4* jobs;
    long long jobs_cap;
    unsigned long long* njobs;
    long long njobs_val;
    // Phase 2: job counter, per-block arenas, accepted-pair buffers, scratch slots, outputs.
    unsigned long long* job_next;
    int* arena2;
    long long arena2_cap;
    int* acc_i;
    double* acc_d;
    int acc_cap;
    double* slots;
    int nslots;
    long long slot_doubles;
    double* out;
    long long out_stride;
    int* err;
};

// Device scratch of the multipole path, grown on demand and kept by the corr object.
struct MPScratch {
    int* arena1 = nullptr;
    long long arena1_cap = 0;
    long long ntop_alloc = 0;
    int4* jobs = nullptr;
    long long jobs_cap = 0;
    int* arena2 = nullptr;
    long long arena2_cap = 0;
    int* acc_i = nullptr;
    double* acc_d = nullptr;
    long long acc_cap = 0;
    double* slots = nullptr;
    int nslots = 0;
    long long slot_doubles = 0;
    double* out = nullptr;
    double* total = nullptr;
    long long out_stride = 0;
    int nblk = 0;
    unsigned long long* ctl = nullptr;
    int* err = nullptr;
    // Requested minimum capacities, raised after an overflow.
    long long want_a1 = 0, want_jobs = 0, want_a2 = 0, want_acc = 0;
    int want_slots = 0;
};

int launch_leaf_sums(int ncap, const Cells& C, double* ls, cudaStream_t st);
// Runs both phases and the reduction; h_out receives 15 arrays of nbins*nbins*(2*maxn+1)
// doubles: gam0r, gam0i, gam1r, gam1i, gam2r, gam2i, gam3r, gam3i, meand2, meanlogd2,
// meand3, meanlogd3, weight, weight_im, ntri.
int run_multipole(MPParams& P, MPScratch& X, int ntop, cudaStream_t st, double* h_out);
void free_mp_scratch(MPScratch& X);
size_t mp_slot_doubles(int nb, int M);

}  // namespace tc
