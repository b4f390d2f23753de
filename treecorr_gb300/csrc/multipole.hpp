// multipole.hpp -- parameters and launchers of the LogMultipole 3-point accumulation.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "tc_internal.cuh"

namespace tc {

// Floats per accepted-pair record of the G_n accumulation.
constexpr int MP_REC = 24;
// Largest nbins of the GPU multipole path (shared-memory bin counters).
constexpr int MP_MAXNB = 128;

enum MPErr : int {
    MP_ERR_ARENA = 11,   // a c2-list arena is full
    MP_ERR_JOBS = 12,    // the job list is full
    MP_ERR_SLOTS = 13,   // no free scratch slot for a c1 split
    MP_ERR_STACK = 14,   // a block-local stack is full
    MP_ERR_CHECK = 15,   // a consistency check failed (err[1] names the site)
};

struct MPParams {
    int coords, metric, quick, nbins, maxn;
    // 0: a spin-2 vertex (GGG: G_n up to n = max_n + 1, self-pair sums with z^2); 1: an N or
    // K vertex with G pairs (NGG, KGG: the record's vertex payload is (w1 or w1 k1, 0)).
    int vreal;
    // Bit 0: the vertex-2 (or only) pair list holds N or K cells whose payload is real (w or
    // w k): no spin-2 rotation; bit 1: the same for the vertex-3 list of a three-field cross.
    int pspin0;
    // Three-field cross (vertex 1, vertex-2 cells, vertex-3 cells): nbd is the number of
    // distance bins, nbins = 2 nbd the bins of the scratch and the records (vertex-3 pairs
    // land in [nbd, 2 nbd)); cells with id >= base3 are vertex-3 cells.  typo32: ordered = 1's
    // meanlogd3 second term as the reference writes it (mp3.sumw[k3], src/Corr3.cpp:2036).
    // Without a three-field cross nbd = nbins and three = 0.
    int three, nbd, base3, typo32;
    double minsep, maxsep, binsize, b, a, logminsep, minsepsq, maxsepsq, bsq, asq, maxbsq_eff;
    // FP32 copies for the FP32 decisions (the FP64 values decide whenever FP32 is too close).
    float f_minsepsq, f_minsep, f_maxsepsq, f_maxsep, f_asq, f_bsq, f_q25, f_logminsep, f_binsize, f_b,
        f_minba;
    // Cells (FP64 centres, float payloads) and their leaf sums (4 doubles per cell:
    // sum w^2, Re/Im sum (wz)^2, sum |wz|^2).
    const double *x, *y, *z;
    const float *size, *w, *d1, *d2;
    const int *n, *left, *right;
    const double* ls;
    const float4* lsf;   // the leaf sums as floats
    const TCell* tc;     // packed cells (float hi/lo positions and payload)
    const int* tops;     // vertex-1 top cells (one phase-1 block each)
    int ntop;
    const int* tops2;    // top cells that start every vertex's pair list
    int ntop2;
    int ncells;          // cell ids are 0 .. ncells-1
    // Phase 1: per-block list arenas and the job list.
    int* arena1;
    long long arena1_cap;
    int4* jobs;
    long long jobs_cap;
    unsigned long long* njobs;
    long long njobs_val;
    // Phase 2: job counter, per-block arenas, accepted-pair records, scratch slots, outputs.
    unsigned long long* job_next;
    int* arena2;
    long long arena2_cap;
    float* acc;          // per block: acc_cap records of MP_REC floats
    int* perm;           // per block: acc_cap ints (records in bin order)
    int acc_cap;
    double* slots;
    int nslots;
    long long slot_doubles;
    double* out;         // per block: 15 arrays of nbins^2 (2 maxn + 1) doubles
    long long out_stride;
    double* diag;        // per block: 9 x nbins self-pair corrections of the diagonal k2 == k3
    // Vertex records for the batched contraction: zcount counts them; records at index
    // >= zcap are contracted in place instead; jobs are not started once zcount >= zstop.
    float* zrec;
    long long zcap, zstop;
    int zrec_floats;
    unsigned long long* zcount;
    unsigned long long* zmaxjob;   // largest number of records of one job
    int* err;
    double* dbg;         // 32 doubles describing the first failed check
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
    float* acc = nullptr;
    int* perm = nullptr;
    long long acc_cap = 0;
    double* slots = nullptr;
    int nslots = 0;
    long long slot_doubles = 0;
    double* out = nullptr;
    double* diag = nullptr;
    double* total = nullptr;
    long long out_stride = 0;
    long long diag_stride = 0;
    float* zrec = nullptr;
    long long zcap = 0;
    int zrec_floats = 0;
    double* part = nullptr;     // per contraction group: 10 arrays of nbins^2 (2 maxn + 1)
    long long part_stride = 0;
    int ngroups = 0;
    double* spart = nullptr;    // per scalar group: 4 arrays of nbins^2 (meand2/3, meanlogd2/3)
    unsigned long long* ntp = nullptr;   // per scalar group: nbins^2 triangle counts
    long long spart_nb2 = 0;
    int nsg = 0;
    // Counters of the last run: vertex records, those contracted in place, waves.
    long long records = 0, overflow = 0, waves = 0;
    int nblk = 0;
    unsigned long long* ctl = nullptr;
    int* err = nullptr;
    double* dbg = nullptr;
    int* tcstatus = nullptr;    // set when a tensor-core contraction timed out
    // Requested minimum capacities, raised after an overflow.
    long long want_a1 = 0, want_jobs = 0, want_a2 = 0;
    int want_slots = 0;
};

int launch_leaf_sums(int ncap, const Cells& C, double* ls, float4* lsf, cudaStream_t st);
// N / K pair cells as the real payload (w or w k, 0) of GNN, GKK, NKK, KNN.
int launch_scalar_pairs(int ncap, int is_n, TCell* tc, float* d1, float* d2, double* ls,
                        float4* lsf, cudaStream_t st);
// Runs both phases and the reduction; h_out receives 15 arrays of nbins*nbins*(2*maxn+1)
// doubles: gam0r, gam0i, gam1r, gam1i, gam2r, gam2i, gam3r, gam3i, meand2, meanlogd2,
// meand3, meanlogd3, weight, weight_im, ntri.
int run_multipole(MPParams& P, MPScratch& X, int ntop, cudaStream_t st, double* h_out);
void free_mp_scratch(MPScratch& X);
size_t mp_slot_doubles(int nb, int M);

}  // namespace tc
