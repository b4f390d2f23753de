// traverse2pt.hpp -- parameters and launchers of the 2-point traversal.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "tc_internal.cuh"

namespace tc {

struct TravParams {
    int coords, metric, quick, nbins, autoc;
    int k1, k2, s1, s2;           // payload kind (DN/DK/DG) and spin of the two fields
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
    unsigned long long* counters;   // [0] evaluated, [1] accepted, [2] escalated,
                                    // [3] accepted by the learned criterion
    // Per-warp counter slots (when set; the expansion's and the tiles' warps, [warp][8]):
    // the counters above, then [4] tiles, [5] leaf pairs of tiles, [6] their FP64 decisions.
    // A warp adds to its own slot, so launches end without contended atomics.
    unsigned long long* wctr;
    int* err;
    // Learned opening criterion.  mode 0: the bin_slop rule; 1: the rule, and candidate pairs
    // are sampled into `samples`; 2: candidates go through the network.  A candidate is a
    // pair the rule splits with min_sep^2 <= rsq < max_sep^2, (s1+s2)^2 <= a^2 rsq and
    // (s1+s2)^2 <= cand_f2 rsq; the network accepts it when its output is <= mlp_thr.
    int mode;
    float cand_f2, mlp_thr, finvlogrange;
    const struct MLPPacked* mlp;
    int2* samples;
    unsigned long long* nsamples;
    long long sample_cap;
    unsigned sample_mod;
    // Patches (mode 3): one expansion over the cells of all patch fields, whose records
    // carry their patch in d.y; an accepted pair adds into the FP64 sums of its patch pair
    // (pacc: [pair][nqf][nbins], pnp: [pair][nbins]).
    int npatch;
    const int* pair_index;          // [npatch][npatch] -> pair id
    double* pacc;
    unsigned long long* pnp;
    // Mode 3 roots, generated on the device: pair p's top-level items are roots
    // proot_off[p] .. proot_off[p+1]-1; ptop[ptop_off[i] ..] are patch i's top cells.
    int npair;
    const long long* proot_off;
    const int2* ppairs;
    const int* ptop;
    const int* ptop_off;
    // Leaf-pair tiles (exact mode: every accepted pair is a pair of leaves, which holds for
    // angle_slop = 0 or two brute fields).  A cell pair that must be split while both cells
    // hold at most tile_leaf points becomes a tile (c1, c2), and a self item on such a cell a
    // self tile (c, -2 - c); k_tiles evaluates every leaf pair of a tile.  The leaf starting
    // at point p of field 1 (2) has cell id leaf_base1 (leaf_base2) + p.
    int tile_leaf;                  // 0: no tiles
    int leaf_base1, leaf_base2;
    int2* tiles;
    unsigned long long* tctl;       // [0] tiles waiting, [1] blocks of k_tiles done,
                                    // [2] tiles, [3] leaf pairs evaluated, [4] escalated
    long long tile_cap;
    int tile_blocks, tile_wbase;    // k_tiles grid; its warps' slots start at tile_wbase
    const float* tile_edge;         // [nbins+1]: 1 / (min_sep^2 exp(2 k bin_size))
    const float* tile_ledge;        // [nbins+1]: log(min_sep) + k bin_size
    // Fixed-order expansion (det != 0; modes 0 and 2): every warp of an expansion launch
    // writes its children and tiles into regions of its own (det_out + gw det_ccap,
    // det_tout + gw det_tcap) and their counts into det_cnt[gw] and det_cnt[det_nw + gw];
    // k_compact then joins the regions in warp order.  The level buffers and the tile list,
    // and with them the items every warp takes and the order of every floating-point sum,
    // are then the same from run to run.
    int det, det_nw;
    int2* det_out;
    int2* det_tout;
    int* det_cnt;
    long long det_ccap, det_tcap;
};

// Fixed traversal scratch of the allocation-free entry point (traverse2pt.cu).
static constexpr int NOALLOC_MAXW = 1024;           // warps launched at most
static constexpr int NOALLOC_SCAP = 2048;           // work items per warp stack
static constexpr int NOALLOC_MAXNB = 64;            // bins at most
static constexpr int NOALLOC_NQ = 7;                // FP32 bin quantities at most
static constexpr long long NOALLOC_SPILL = (long long)NOALLOC_MAXW * NOALLOC_SCAP;
static constexpr size_t NOALLOC_OFF_STACKS = 0;
static constexpr size_t NOALLOC_OFF_SPILL0 = NOALLOC_OFF_STACKS + sizeof(int2) * (size_t)NOALLOC_MAXW * NOALLOC_SCAP;
static constexpr size_t NOALLOC_OFF_SPILL1 = NOALLOC_OFF_SPILL0 + sizeof(int2) * (size_t)NOALLOC_SPILL;
static constexpr size_t NOALLOC_OFF_WACC = NOALLOC_OFF_SPILL1 + sizeof(int2) * (size_t)NOALLOC_SPILL;
static constexpr size_t NOALLOC_OFF_WNP = NOALLOC_OFF_WACC + sizeof(double) * (size_t)NOALLOC_MAXW * NOALLOC_NQ * NOALLOC_MAXNB;
static constexpr size_t NOALLOC_OFF_TOT = NOALLOC_OFF_WNP + 8 * (size_t)NOALLOC_MAXW * NOALLOC_MAXNB;
static constexpr size_t NOALLOC_OFF_TOTNP = NOALLOC_OFF_TOT + sizeof(double) * (size_t)NOALLOC_NQ * NOALLOC_MAXNB;
static constexpr size_t NOALLOC_OFF_CTL = NOALLOC_OFF_TOTNP + 8 * (size_t)NOALLOC_MAXNB;
static constexpr size_t NOALLOC_OFF_IDLE = NOALLOC_OFF_CTL + 8 * 8;
static constexpr size_t NOALLOC_OFF_ERR = NOALLOC_OFF_IDLE + 256;
static constexpr size_t NOALLOC_BYTES = NOALLOC_OFF_ERR + 256;

// Device address of the fixed scratch on the current device (looked up on first use).
int noalloc_scratch(void** base);

// Device-side schedule of the level-by-level expansion: a one-thread kernel picks the next
// chunk (the deepest non-empty level first) so that launches need no host round trip.
static constexpr int EXP_MAXLEV = 512;
struct ExpandSched {
    long long cnt[EXP_MAXLEV];     // items waiting per level (level 0: generated roots)
    int2* lev[EXP_MAXLEV];         // item buffers (level 0 has none)
    long long cap;                 // items per level buffer
    long long chunk_max;
    int nlev;                      // levels with a buffer
    int done, need_levels, out_level;
    const int2* in;                // current launch
    long long n_in, gen0, out_cap;
    int2* out;
    unsigned long long nout;
    long long launches;
    unsigned int warps_done;       // warps of the current expand launch that have finished
    int pending;                   // a picked chunk waits for its expand launch
};

void launch_pack_cells(int ncap, const Cells& C, TCell* out, cudaStream_t st);
size_t traverse_smem_bytes(int nq, int nb);
int traverse_grid(int nq, int nb, int* blocks, int* nwarps);
int launch_traverse(const TravParams& T, int blocks, cudaStream_t st);
int expand_grid(int nq, int nb, int* blocks, int* nwarps, int mode = 0);
// Enqueues `iters` (schedule, expand[, tiles]) launches on st without synchronising.  With
// ev (3 * iters events) it records events around them: ev[3 it] before the expansion launch,
// ev[3 it + 1] after it (= before the tiles), ev[3 it + 2] after the tiles.
int launch_expand_batch(const TravParams& T, int blocks, ExpandSched* dS, int iters,
                        cudaStream_t st, cudaEvent_t* ev = nullptr);
// Items an expansion warp takes at most in one launch of `chunk` items (the size of its
// fixed-order regions: 4 children and 1 tile per item at most).
long long det_items_per_warp(long long chunk, int nwarps);
// Leaf-pair tiles (tiles.cu): the leaf size of a tile side, the k_tiles grid for a traversal
// (its blocks fill every SM), and one k_tiles launch over the tiles waiting in T.tiles.
static constexpr int TILE_LEAF = 48;
int tiles_grid(const TravParams& T, int* blocks, int* nwarps);
int launch_tiles(const TravParams& T, cudaStream_t st);
int launch_reduce(int nwarps, int nq, int nb, const double* wacc, const unsigned long long* wnp,
                  double* out, unsigned long long* outnp, cudaStream_t st);

}  // namespace tc
