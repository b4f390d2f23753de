// kmeans.cu -- k-means patches on a field's tree (the reference's src/KMeans.cpp).
//
// KMeansRun alternates two steps until the rms centre shift drops below tol * field size:
// find the cells that lie wholly in one patch (FindCellsInPatches, src/KMeans.cpp:543-645),
// and move every centre to the weighted mean of its cells (UpdateCenters, 346-385); the
// alternate form first measures each patch's inertia (CalculateInertia, 387-463) and adds it
// as a penalty to the distances.
//
// GPU form.  FindCellsInPatches is a breadth-first pass over the tree: a work item is
// (cell, candidate list); one warp evaluates the cell against its candidates, prunes those
// that cannot hold any of its points, and either assigns the cell (one candidate left, or a
// cell of size 0) or hands the survivors to both children.  Children share the list, and a
// list that lost no candidate is not copied.  The per-patch sums then run over the cells in
// id order with per-warp accumulators in shared memory, block partials and a fixed-order
// final sum, so the result does not depend on scheduling.  All distances are FP64 with the
// reference's association and no contraction, so candidate decisions and nearest-centre
// choices are the reference's; sums differ from its OpenMP order only by rounding.
//
// The initialisations (KMeansInitTree / Rand / KMPP) draw from the C library's rand()
// stream exactly as the reference's urand() does, walking the few cells they visit from
// the host through a small cache filled by subtree gathers.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <ctime>
#include <set>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/tcgpu.h"
#include "tc_host.hpp"
#include "kmeans.hpp"

namespace tc {

namespace {

constexpr int KM_NQ = 5;            // per-patch sums: centres w x, w y, w z, w; inertia I, I_size, w
constexpr int KM_MAX_PATCH = 5000;  // per-warp shared accumulators must fit one warp at least
constexpr int KM_NBLK = 1216;       // accumulation blocks (fixed: the sum order depends on it)
constexpr int KM_LTB = 256;         // threads per block of the level kernel
constexpr int KM_LEVELS_PER_CHECK = 16;
// assign[cell] = tag * KM_TAG + patch for the cells assigned by the pass with that tag, so the
// array needs no clearing between passes (npatch <= KM_MAX_PATCH < KM_TAG).
constexpr int KM_TAG = 8192;
constexpr int KM_TAG_MAX = (1 << 30) / KM_TAG;

struct KMItem {
    int cell;
    int len;          // candidates
    long long off;    // first candidate in the pool
};

struct KMLevel {
    long long lo, hi;        // items of the current level
    long long total;         // items appended so far
    long long pool_top;
    unsigned blocks_done;
    int err;                 // 1: candidate pool full, 2: item array full
    int leaf_multi;          // leaves reached with more than one candidate
    int levels;              // levels that held items
};

__device__ __forceinline__ int km_patch_of(int v, int tag)
{
    return (v >= 0 && v / KM_TAG == tag) ? v % KM_TAG : -1;
}

// |a - b|^2 as the reference evaluates Position::normSq of a difference
// (include/Position.h:64-68, 159-163): ((dx dx + dy dy) + dz dz), no fused operations.
__device__ __forceinline__ double dsq3(double ax, double ay, double az, double bx, double by,
                                       double bz)
{
    const double dx = __dsub_rn(ax, bx), dy = __dsub_rn(ay, by), dz = __dsub_rn(az, bz);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__device__ __forceinline__ double sqd(double a) { return __dmul_rn(a, a); }

// Is candidate j of the list still possible for some point of the cell?  The pruning
// rule of FindCellsInPatches (src/KMeans.cpp:598-628).
__device__ __forceinline__ bool km_keep(double d, double s, double thresh, const double* inertia,
                                        int p)
{
    if (inertia) {
        const double dd = sqrt(d);
        if (s > dd) d = 0.;
        else d = __dadd_rn(sqd(__dsub_rn(dd, s)), inertia[p]);
    }
    return !(d > thresh);
}

__global__ void k_km_start(const int* tops, int ntop, int npatch, KMItem* items, int* pool,
                           KMLevel* L)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ntop) items[i] = KMItem{tops[i], npatch, 0};
    if (i < npatch) pool[i] = i;
    if (i == 0) {
        L->lo = 0; L->hi = ntop; L->total = ntop; L->pool_top = npatch;
        L->blocks_done = 0; L->err = 0; L->leaf_multi = 0; L->levels = 0;
    }
}

// A candidate list of at most KM_SMALL entries is handled by one thread; longer lists (the
// top levels) by a whole warp.
constexpr int KM_SMALL = 16;

// The whole-warp form for one item with a long candidate list.
__device__ void km_item_warp(const KMItem it, int lane, Cells C, const double* cen,
                             const double* inertia, KMItem* items, long long item_cap, int* pool,
                             long long pool_cap, int* assign, int tag, KMLevel* L)
{
    const int c = it.cell, m = it.len;
    const int* lst = pool + it.off;
    const double px = C.x[c], py = C.y[c], pz = C.z[c];
    const double s = (double)C.size[c];
    // The closest centre by the (penalised) distance: the first minimum in list order.
    double bmod = 0., bdsq = 0.;
    int bpos = INT_MAX;
    for (int j = lane; j < m; j += 32) {
        const int p = lst[j];
        const double d = dsq3(px, py, pz, cen[3 * p], cen[3 * p + 1], cen[3 * p + 2]);
        const double mod = inertia ? __dadd_rn(d, inertia[p]) : d;
        if (bpos == INT_MAX || mod < bmod) { bmod = mod; bdsq = d; bpos = j; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double om = __shfl_xor_sync(0xffffffffu, bmod, o);
        const double od = __shfl_xor_sync(0xffffffffu, bdsq, o);
        const int op = __shfl_xor_sync(0xffffffffu, bpos, o);
        if (op != INT_MAX && (bpos == INT_MAX || om < bmod || (om == bmod && op < bpos))) {
            bmod = om; bdsq = od; bpos = op;
        }
    }
    const int cp = lst[bpos];
    const double min_d = sqrt(bdsq);
    const double thresh = inertia ? __dadd_rn(sqd(__dadd_rn(min_d, s)), inertia[cp])
                                  : sqd(__dadd_rn(min_d, __dmul_rn(2., s)));
    int nkeep = 0;
    for (int j0 = 0; j0 < m; j0 += 32) {
        const int j = j0 + lane;
        bool keep = false;
        if (j < m && j != bpos) {
            const int p = lst[j];
            const double d = dsq3(px, py, pz, cen[3 * p], cen[3 * p + 1], cen[3 * p + 2]);
            keep = km_keep(d, s, thresh, inertia, p);
        }
        nkeep += __popc(__ballot_sync(0xffffffffu, keep));
    }
    const int ncand = nkeep + 1;
    const int left = C.left[c];
    if (ncand == 1 || s == 0. || left < 0) {
        if (lane == 0) {
            assign[c] = tag * KM_TAG + cp;
            if (ncand > 1 && s != 0.) atomicAdd(&L->leaf_multi, 1);
        }
        return;
    }
    long long off = it.off;
    if (ncand < m) {
        // The surviving candidates: the closest first, then the rest in list order.
        unsigned long long o = 0;
        if (lane == 0) o = atomicAdd((unsigned long long*)&L->pool_top, (unsigned long long)ncand);
        o = __shfl_sync(0xffffffffu, o, 0);
        if ((long long)o + ncand > pool_cap) {
            if (lane == 0) atomicCAS(&L->err, 0, 1);
            return;
        }
        off = (long long)o;
        if (lane == 0) pool[off] = cp;
        int base = 1;
        for (int j0 = 0; j0 < m; j0 += 32) {
            const int j = j0 + lane;
            bool keep = false;
            int p = 0;
            if (j < m && j != bpos) {
                p = lst[j];
                const double d = dsq3(px, py, pz, cen[3 * p], cen[3 * p + 1], cen[3 * p + 2]);
                keep = km_keep(d, s, thresh, inertia, p);
            }
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            if (keep) pool[off + base + __popc(bal & ((1u << lane) - 1u))] = p;
            base += __popc(bal);
        }
    }
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd((unsigned long long*)&L->total, 2ull);
    t = __shfl_sync(0xffffffffu, t, 0);
    if ((long long)t + 2 > item_cap) {
        if (lane == 0) atomicCAS(&L->err, 0, 2);
        return;
    }
    if (lane == 0) items[t] = KMItem{left, ncand, off};
    if (lane == 1) items[t + 1] = KMItem{C.right[c], ncand, off};
}

// One level of FindCellsInPatches.  cen: npatch x 3 (z = 0 for Flat).  Items with short
// lists are processed one per thread; their child items and new lists are reserved with one
// atomic per warp.
__global__ void __launch_bounds__(KM_LTB) k_km_level(Cells C, const double* cen,
                                                     const double* inertia, KMItem* items,
                                                     long long item_cap, int* pool,
                                                     long long pool_cap, int* assign,
                                                     int tag, KMLevel* L)
{
    const int lane = threadIdx.x & 31;
    const long long lo = *(volatile long long*)&L->lo;
    // After an error the level window may cover unwritten slots: process nothing.
    const long long hi = *(volatile int*)&L->err ? lo
                       : min(*(volatile long long*)&L->hi, item_cap);
    const long long stride = (long long)gridDim.x * KM_LTB;
    const long long nwarps = (long long)gridDim.x * (KM_LTB / 32);
    if (hi - lo <= 2 * nwarps) {
        // A small level (the top of the tree, long lists): one item per warp.
        for (long long i = lo + (long long)blockIdx.x * (KM_LTB / 32) + (threadIdx.x >> 5); i < hi;
             i += nwarps)
            km_item_warp(items[i], lane, C, cen, inertia, items, item_cap, pool, pool_cap, assign,
                         tag, L);
    } else
    for (long long base = lo + (long long)blockIdx.x * KM_LTB + (threadIdx.x & ~31); base < hi;
         base += stride) {
        const long long i = base + lane;
        KMItem it{0, 0, 0};
        if (i < hi) it = items[i];
        const bool small = i < hi && it.len <= KM_SMALL;
        int nout = 0, nlist = 0, cp = -1;
        unsigned kept = 0;            // bit j: candidate j survives (the closest excluded)
        if (small) {
            const int c = it.cell, m = it.len;
            const int* lst = pool + it.off;
            const double px = C.x[c], py = C.y[c], pz = C.z[c];
            const double s = (double)C.size[c];
            double dd[KM_SMALL];
            double bmod = 0., bdsq = 0.;
            int bpos = 0;
#pragma unroll
            for (int j = 0; j < KM_SMALL; ++j) {
                if (j < m) {
                    const int p = lst[j];
                    const double d = dsq3(px, py, pz, cen[3 * p], cen[3 * p + 1], cen[3 * p + 2]);
                    dd[j] = d;
                    const double mod = inertia ? __dadd_rn(d, inertia[p]) : d;
                    if (j == 0 || mod < bmod) { bmod = mod; bdsq = d; bpos = j; }
                }
            }
            cp = lst[bpos];
            const double min_d = sqrt(bdsq);
            const double thresh = inertia ? __dadd_rn(sqd(__dadd_rn(min_d, s)), inertia[cp])
                                          : sqd(__dadd_rn(min_d, __dmul_rn(2., s)));
            int nkeep = 0;
#pragma unroll
            for (int j = 0; j < KM_SMALL; ++j) {
                if (j < m && j != bpos && km_keep(dd[j], s, thresh, inertia, inertia ? lst[j] : 0)) {
                    kept |= 1u << j;
                    ++nkeep;
                }
            }
            const int ncand = nkeep + 1;
            if (ncand == 1 || s == 0. || C.left[c] < 0) {
                assign[c] = tag * KM_TAG + cp;
                if (ncand > 1 && s != 0.) atomicAdd(&L->leaf_multi, 1);
            } else {
                nout = 2;
                nlist = ncand < m ? ncand : 0;
            }
        }
        // Warp-aggregated reservations of child items and list space.
        int xo = nout, xl = nlist;
        for (int o = 1; o < 32; o <<= 1) {
            const int a = __shfl_up_sync(0xffffffffu, xo, o), b = __shfl_up_sync(0xffffffffu, xl, o);
            if (lane >= o) { xo += a; xl += b; }
        }
        const int tot_o = __shfl_sync(0xffffffffu, xo, 31), tot_l = __shfl_sync(0xffffffffu, xl, 31);
        xo -= nout; xl -= nlist;
        // List space first: on overflow no items are reserved (the pass is repeated).
        unsigned long long ob = 0, lb = 0;
        int ok = 1;
        if (lane == 0) {
            if (tot_l) {
                lb = atomicAdd((unsigned long long*)&L->pool_top, (unsigned long long)tot_l);
                if ((long long)lb + tot_l > pool_cap) { atomicCAS(&L->err, 0, 1); ok = 0; }
            }
            if (ok && tot_o) {
                ob = atomicAdd((unsigned long long*)&L->total, (unsigned long long)tot_o);
                if ((long long)ob + tot_o > item_cap) { atomicCAS(&L->err, 0, 2); ok = 0; }
            }
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        ob = __shfl_sync(0xffffffffu, ob, 0);
        lb = __shfl_sync(0xffffffffu, lb, 0);
        if (!ok) nout = 0;
        if (nout) {
            const int c = it.cell;
            long long off = it.off;
            int ncand = it.len;
            if (nlist) {
                off = (long long)lb + xl;
                const int* lst = pool + it.off;
                pool[off] = cp;
                int q = 1;
                for (unsigned k = kept; k; k &= k - 1) pool[off + q++] = lst[__ffs(k) - 1];
                ncand = nlist;
            }
            items[ob + xo] = KMItem{C.left[c], ncand, off};
            items[ob + xo + 1] = KMItem{C.right[c], ncand, off};
        }
        // Items with long lists: the whole warp takes them one by one.
        unsigned wide = __ballot_sync(0xffffffffu, i < hi && !small);
        while (wide) {
            const int l = __ffs(wide) - 1;
            wide &= wide - 1;
            KMItem w;
            w.cell = __shfl_sync(0xffffffffu, it.cell, l);
            w.len = __shfl_sync(0xffffffffu, it.len, l);
            w.off = __shfl_sync(0xffffffffu, it.off, l);
            km_item_warp(w, lane, C, cen, inertia, items, item_cap, pool, pool_cap, assign, tag, L);
        }
    }
    // The last block to finish moves the level window to the appended items.
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&L->blocks_done, 1u) == gridDim.x - 1) {
            __threadfence();
            L->blocks_done = 0;
            if (hi > lo) L->levels += 1;
            L->lo = hi;
            L->hi = *(volatile long long*)&L->total;
        }
    }
}

enum { KM_SUM_CENTERS = 0, KM_SUM_INERTIA = 1 };

// Per-patch sums over the assigned cells, in cell id order: block b takes a contiguous id
// range, each warp its own accumulators; lanes of one patch are combined in lane order.
//   centres: (w x, w y, w z, w)          (UpdateCenters::run, src/KMeans.cpp:355-359)
//   inertia: (|x - c|^2 w, 0.75 s^2 w, w) (CalculateInertia::run, 397-417)
__device__ __forceinline__ void km_cell_values(Cells C, long long id, int p, const double* cen,
                                               int mode, double (&v)[KM_NQ])
{
    const double w = (double)C.w[id];
    const double x = C.x[id], y = C.y[id], z = C.z[id];
    if (mode == KM_SUM_CENTERS) {
        v[0] = __dmul_rn(x, w); v[1] = __dmul_rn(y, w); v[2] = __dmul_rn(z, w);
        v[3] = w; v[4] = 0.;
    } else {
        const double s = (double)C.size[id], ssq = __dmul_rn(s, s);
        v[0] = __dmul_rn(dsq3(x, y, z, cen[3 * p], cen[3 * p + 1], cen[3 * p + 2]), w);
        v[1] = ssq > 0. ? __dmul_rn(__dmul_rn(0.75, ssq), w) : 0.;
        v[2] = w; v[3] = 0.; v[4] = 0.;
    }
}

// Per-patch sums over the cells assigned by pass `tag`, in cell id order: block b takes a
// contiguous id range (a multiple of 16 ids; each thread reads 16 consecutive assignments with
// four 16-byte loads in flight), each warp its own accumulators; lanes of one patch are
// combined in lane order.
//   centres: (w x, w y, w z, w)          (UpdateCenters::run, src/KMeans.cpp:355-359)
//   inertia: (|x - c|^2 w, 0.75 s^2 w, w) (CalculateInertia::run, 397-417)
__global__ void k_km_accum(Cells C, int ncap, const int* assign, int tag, const double* cen,
                           int npatch, int mode, double* partial)
{
    extern __shared__ __align__(16) double kmsm[];
    const int nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* my = kmsm + (size_t)wib * npatch * KM_NQ;
    double* stage = kmsm + (size_t)nw * npatch * KM_NQ + (size_t)wib * 32 * KM_NQ;
    for (int q = lane; q < npatch * KM_NQ; q += 32) my[q] = 0.;
    __syncwarp();
    long long per = ((long long)ncap + gridDim.x - 1) / gridDim.x;
    per = (per + 15) & ~15LL;
    const long long b0 = (long long)blockIdx.x * per;
    const long long b1 = min(b0 + per, (long long)ncap);
    for (long long base = b0; base < b1; base += 16LL * blockDim.x) {
        const long long id0 = base + 16LL * threadIdx.x;
        int a[16];
        if (id0 + 15 < b1) {
            const int4* a4 = reinterpret_cast<const int4*>(assign + id0);
            int4 q[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) q[r] = a4[r];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                a[4 * r] = q[r].x; a[4 * r + 1] = q[r].y; a[4 * r + 2] = q[r].z; a[4 * r + 3] = q[r].w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < 16; ++k) a[k] = id0 + k < b1 ? assign[id0 + k] : -1;
        }
        unsigned mine = 0;   // bit k: id0 + k is assigned in this pass
#pragma unroll
        for (int k = 0; k < 16; ++k)
            if (km_patch_of(a[k], tag) >= 0) mine |= 1u << k;
        if (!__ballot_sync(0xffffffffu, mine != 0)) continue;
        for (int k0 = 0; k0 < 16; k0 += 4) {
            if (!__ballot_sync(0xffffffffu, (mine >> k0) & 0xfu)) continue;
            // The cell values of four slots, loaded together.
            int pp[4];
            double vv[4][KM_NQ];
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                pp[kk] = ((mine >> (k0 + kk)) & 1u) ? km_patch_of(assign[id0 + k0 + kk], tag) : -1;
#pragma unroll
                for (int q = 0; q < KM_NQ; ++q) vv[kk][q] = 0.;
                if (pp[kk] >= 0) km_cell_values(C, id0 + k0 + kk, pp[kk], cen, mode, vv[kk]);
            }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
            const int p = pp[kk];
            if (!__ballot_sync(0xffffffffu, p >= 0)) continue;
#pragma unroll
            for (int q = 0; q < KM_NQ; ++q) stage[lane * KM_NQ + q] = vv[kk][q];
            __syncwarp();
            const unsigned grp = __match_any_sync(0xffffffffu, p);
            if (p >= 0 && lane == __ffs(grp) - 1) {
                double sum[KM_NQ] = {0., 0., 0., 0., 0.};
                for (unsigned g = grp; g; g &= g - 1) {
                    const int l = __ffs(g) - 1;
#pragma unroll
                    for (int q = 0; q < KM_NQ; ++q) sum[q] = __dadd_rn(sum[q], stage[l * KM_NQ + q]);
                }
#pragma unroll
                for (int q = 0; q < KM_NQ; ++q) my[p * KM_NQ + q] = __dadd_rn(my[p * KM_NQ + q], sum[q]);
            }
            __syncwarp();
            }
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < npatch * KM_NQ; q += blockDim.x) {
        double s = 0.;
        for (int w = 0; w < nw; ++w) s = __dadd_rn(s, kmsm[(size_t)w * npatch * KM_NQ + q]);
        partial[(size_t)blockIdx.x * npatch * KM_NQ + q] = s;
    }
}

// Block partials -> totals: one warp per summed quantity, lanes over the blocks, then a
// fixed-shape warp reduction (deterministic).
__global__ void k_km_total(int nq, int nblk, const double* partial, double* tot)
{
    const int q = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (q >= nq) return;
    double s = 0.;
    for (int b = lane; b < nblk; b += 32) s = __dadd_rn(s, partial[(size_t)b * nq + q]);
    for (int o = 16; o > 0; o >>= 1) s = __dadd_rn(s, __shfl_xor_sync(0xffffffffu, s, o));
    if (lane == 0) tot[q] = s;
}

// Fixed-shape block sum (the same tree of additions on every run).
__device__ double block_sum(double v, double* red)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double t = 0.;
    for (int w = 0; w < nw; ++w) t = __dadd_rn(t, red[w]);
    return t;
}

// The finalize step of the sums, one thread per patch.
__global__ void __launch_bounds__(1024) k_km_finish(int npatch, const double* tot, int mode,
                                                    int coords, double* cen, double* inertia,
                                                    double* shift)
{
    __shared__ double red[32];
    if (mode == KM_SUM_CENTERS) {
        // UpdateCenters::finalize (src/KMeans.cpp:370-380), CalculateShiftSq (689-706).
        double sh = 0.;
        for (int p = threadIdx.x; p < npatch; p += blockDim.x) {
            const double* t = tot + p * KM_NQ;
            double x = t[0], y = t[1], z = t[2];
            const double w = t[3];
            if (w > 0.) {
                x = __ddiv_rn(x, w); y = __ddiv_rn(y, w); z = __ddiv_rn(z, w);
                if (coords == SPHERE) {
                    const double nrm = sqrt(__dadd_rn(__dadd_rn(sqd(x), sqd(y)), sqd(z)));
                    if (nrm == 0.) { x = 1.; y = 0.; z = 0.; }
                    else { x = __ddiv_rn(x, nrm); y = __ddiv_rn(y, nrm); z = __ddiv_rn(z, nrm); }
                }
            }
            sh = __dadd_rn(sh, dsq3(cen[3 * p], cen[3 * p + 1], cen[3 * p + 2], x, y, z));
            cen[3 * p] = x; cen[3 * p + 1] = y; cen[3 * p + 2] = z;
        }
        sh = block_sum(sh, red);
        if (threadIdx.x == 0) *shift = sh;
    } else {
        // CalculateInertia::finalize (src/KMeans.cpp:419-446): I_i / (sum w / npatch / 3).
        double sw = 0.;
        for (int p = threadIdx.x; p < npatch; p += blockDim.x) sw = __dadd_rn(sw, tot[p * KM_NQ + 2]);
        const double sumw = block_sum(sw, red);
        const double meanw = __ddiv_rn(__ddiv_rn(sumw, (double)npatch), 3.);
        for (int p = threadIdx.x; p < npatch; p += blockDim.x)
            inertia[p] = __ddiv_rn(__dadd_rn(tot[p * KM_NQ], tot[p * KM_NQ + 1]), meanw);
    }
}

// AssignPatches::run (src/KMeans.cpp:482-510): every point of an assigned cell gets its
// patch.  Cells of up to 32 points are written by one thread, larger ones by a block.
__global__ void k_km_paint(Cells C, int ncap, const int* assign, int tag, const int* idx,
                           int64_t* out, int* big, int* nbig)
{
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ncap) return;
    const int p = km_patch_of(assign[id], tag);
    if (p < 0) return;
    const int n = C.n[id], s = C.start[id];
    if (n <= 32) {
        for (int k = s; k < s + n; ++k) out[idx[k]] = p;
    } else {
        big[atomicAdd(nbig, 1)] = (int)id;
    }
}

__global__ void k_km_paint_big(Cells C, const int* assign, int tag, const int* idx,
                               const int* big, const int* nbig, int64_t* out)
{
    const int nb = *nbig;
    for (int e = blockIdx.x; e < nb; e += gridDim.x) {
        const int id = big[e];
        const int p = km_patch_of(assign[id], tag), n = C.n[id], s = C.start[id];
        for (int k = s + threadIdx.x; k < s + n; k += blockDim.x) out[idx[k]] = p;
    }
}

// QuickAssign (mode 0, src/KMeans.cpp:890-942) and SelectPatch (mode 1, 944-1011).
// Distances are first taken in FP32 on coordinates shifted to an origin o (centre 0):
// with R the largest |coordinate - o| of the point and the centres and u = 2^-24, the FP32
// distance differs from the reference's FP64 one by at most 84 u R^2 (two roundings of each
// shifted coordinate, the squares and the sum), so E = 6e-6 R^2 bounds it.  Only centres
// within 4 E of the FP32 minimum can be the FP64 minimum or tie with it; those are compared
// in FP64 with the reference's expression, in index order, so the result is the reference's.
__global__ void k_quick_assign(const double* cen, const float4* cen32, float rc, int npatch,
                               int dim, const double* x, const double* y, const double* z,
                               int64_t n, int mode, int patch, int64_t* out, int cen_in_smem)
{
    extern __shared__ __align__(16) float4 qsm[];
    const float4* c32 = cen32;
    if (cen_in_smem) {
        for (int q = threadIdx.x; q < npatch; q += blockDim.x) qsm[q] = cen32[q];
        __syncthreads();
        c32 = qsm;
    }
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double px = x[i], py = y[i], pz = z ? z[i] : 0.;
    const double ox = cen[0], oy = cen[1], oz = dim == 3 ? cen[2] : 0.;
    const float qx = (float)(px - ox), qy = (float)(py - oy), qz = (float)(pz - oz);
    const float r = fmaxf(rc, fmaxf(fabsf(qx), fmaxf(fabsf(qy), fabsf(qz))));
    const float E = 6e-6f * r * r;
    auto d32 = [&](int k) {
        const float4 c = c32[k];
        const float dx = qx - c.x, dy = qy - c.y, dz = qz - c.z;
        return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    };
    auto d64 = [&](int k) {
        return dsq3(px, py, pz, cen[dim * k], cen[dim * k + 1], dim == 3 ? cen[dim * k + 2] : 0.);
    };
    if (mode == 0) {
        float mn = d32(0);
        for (int k = 1; k < npatch; ++k) mn = fminf(mn, d32(k));
        const float lim = mn + 4.f * E;
        int kmin = -1;
        double best = 0.;
        for (int k = 0; k < npatch; ++k) {
            if (d32(k) > lim) continue;
            const double d = d64(k);
            if (kmin < 0 || d < best) { kmin = k; best = d; }
        }
        out[i] = kmin;
    } else {
        const float p32 = d32(patch);
        double p64 = -1.;
        int64_t use = 1;
        for (int q = 0; q < npatch; ++q) {
            if (q == patch) continue;
            const float d = d32(q);
            if (d > p32 + 2.f * E) continue;
            if (d < p32 - 2.f * E) { use = 0; break; }
            if (p64 < 0.) p64 = d64(patch);
            if (d64(q) < p64) { use = 0; break; }
        }
        out[i] = use;
    }
}

struct KMCellRec {
    double x, y, z;
    float size;
    int n;
    int left, right;
    int start, id;
};

// Subtrees of the given roots down to depth levels, breadth first (id -1 where a leaf
// ends a branch): one thread per root, (2^(depth+1) - 1) records each.
__global__ void k_km_subtree(Cells C, const int* roots, int nroot, int depth, KMCellRec* out)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nroot) return;
    const int per = (1 << (depth + 1)) - 1;
    KMCellRec* o = out + (size_t)r * per;
    for (int k = 0; k < per; ++k) {
        int id;
        if (k == 0) id = roots[r];
        else {
            const int par = o[(k - 1) / 2].id;
            id = par < 0 ? -1 : ((k & 1) ? o[(k - 1) / 2].left : o[(k - 1) / 2].right);
        }
        KMCellRec rec;
        rec.id = id;
        if (id >= 0) {
            rec.x = C.x[id]; rec.y = C.y[id]; rec.z = C.z[id];
            rec.size = C.size[id]; rec.n = C.n[id];
            rec.left = C.left[id]; rec.right = C.right[id]; rec.start = C.start[id];
        } else {
            rec.x = rec.y = rec.z = 0.; rec.size = 0.f; rec.n = 0;
            rec.left = rec.right = -1; rec.start = 0;
        }
        o[k] = rec;
    }
}

// ---------------------------------------------------------------------------------------
// Host side.

struct V3 {
    double x = 0., y = 0., z = 0.;
};

inline bool v3_eq(const V3& a, const V3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// |a - b|^2 in the reference's association (the host compiler must not contract it: the
// library is built with -ffp-contract=off for host code).
inline double v3_dsq(const V3& a, const V3& b)
{
    const double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return (dx * dx + dy * dy) + dz * dz;
}

// Position<Sphere>::normalize (include/Position.h:251-256).
inline void v3_normalize(V3& v)
{
    const double n = std::sqrt((v.x * v.x + v.y * v.y) + v.z * v.z);
    if (n == 0.) { v.x = 1.; v.y = 0.; v.z = 0.; }
    else { v.x /= n; v.y /= n; v.z /= n; }
}

// urand (src/Cell.cpp:59-80): the C library's rand() over RAND_MAX; a non-zero seed reseeds
// the stream first, and that call also returns a draw.  Without a seed, the first call seeds
// from the clock (the reference prefers /dev/urandom; either is non-reproducible).
bool g_urand_first = true;
double urand(long long seed = 0)
{
    if (seed != 0) {
        srand((unsigned)seed);
        g_urand_first = false;
    } else if (g_urand_first) {
        srand((unsigned)time(nullptr) ^ (unsigned)clock());
        g_urand_first = false;
    }
    double r = rand();
    r /= RAND_MAX;
    return r;
}

}  // namespace

// The field constructor's seed (BaseField, src/Field.cpp:160): a non-zero seed reseeds the
// urand stream that the k-means initialisations draw from afterwards.
void km_seed(long long seed)
{
    if (seed != 0) urand(seed);
}

namespace {

// SelectRandomFrom (src/Corr2.cpp:622-661): n distinct values of [0, m) -- Floyd's
// algorithm with a set when m > 3 n, else a partial Fisher-Yates shuffle.
std::vector<long> select_random_from(long m, long n)
{
    std::vector<long> sel(n);
    if (m > 3 * n) {
        std::set<long> seen;
        while ((long)seen.size() < n) {
            long j = long(urand() * m);
            if (j == m) j = m - 1;
            if (seen.insert(j).second) sel[seen.size() - 1] = j;
        }
    } else {
        std::vector<long> full(m);
        for (long i = 0; i < m; ++i) full[i] = i;
        for (long i = 0; i < n; ++i) {
            long j = long(urand() * (m - i)) + i;
            if (j == m) j = m - 1;
            std::swap(full[i], full[j]);
        }
        std::copy(full.begin(), full.begin() + n, sel.begin());
    }
    return sel;
}

// Host view of the cells the initialisations visit, fetched as small subtrees.
class CellCache {
public:
    CellCache(const KMField& F, cudaStream_t st) : F_(F), st_(st) {}
    ~CellCache() { dfree(d_roots_); dfree(d_out_); }

    int get(int id, KMCellRec& r)
    {
        auto it = map_.find(id);
        if (it == map_.end()) {
            TC_TRY(fetch(std::vector<int>{id}, kDepth));
            it = map_.find(id);
            if (it == map_.end()) { set_last_error("k-means: cell fetch failed"); return TC_ERR_DEVICE; }
        }
        r = it->second;
        return 0;
    }

    // The top-level cells, in order.
    int tops(std::vector<KMCellRec>& out)
    {
        std::vector<int> ids(F_.ntop);
        TC_CU(cudaMemcpyAsync(ids.data(), F_.d_tops, sizeof(int) * F_.ntop, cudaMemcpyDeviceToHost, st_));
        TC_CU(cudaStreamSynchronize(st_));
        TC_TRY(fetch(ids, 0));
        out.resize(F_.ntop);
        for (int k = 0; k < F_.ntop; ++k) out[k] = map_[ids[k]];
        return 0;
    }

    // getLeafNumber (src/Cell.cpp:675-685).
    int leaf_number(int id, long m, KMCellRec& leaf)
    {
        KMCellRec r;
        TC_TRY(get(id, r));
        while (r.left >= 0) {
            KMCellRec L;
            TC_TRY(get(r.left, L));
            if (m < L.n) r = L;
            else { m -= L.n; TC_TRY(get(r.right, r)); }
        }
        leaf = r;
        return 0;
    }

private:
    static constexpr int kDepth = 5;

    int fetch(const std::vector<int>& roots, int depth)
    {
        const int per = (1 << (depth + 1)) - 1;
        const size_t nrec = roots.size() * (size_t)per;
        if ((long long)roots.size() > cap_roots_) {
            dfree(d_roots_);
            cap_roots_ = (long long)roots.size();
            TC_TRY(dalloc(&d_roots_, roots.size()));
        }
        if ((long long)nrec > cap_out_) {
            dfree(d_out_);
            cap_out_ = (long long)nrec;
            TC_TRY(dalloc(&d_out_, nrec));
        }
        TC_CU(cudaMemcpyAsync(d_roots_, roots.data(), sizeof(int) * roots.size(), cudaMemcpyHostToDevice, st_));
        count_launch();
        k_km_subtree<<<((int)roots.size() + 127) / 128, 128, 0, st_>>>(F_.cells, d_roots_, (int)roots.size(), depth, d_out_);
        TC_CU(cudaGetLastError());
        std::vector<KMCellRec> h(nrec);
        TC_CU(cudaMemcpyAsync(h.data(), d_out_, sizeof(KMCellRec) * nrec, cudaMemcpyDeviceToHost, st_));
        TC_CU(cudaStreamSynchronize(st_));
        for (const KMCellRec& r : h)
            if (r.id >= 0) map_[r.id] = r;
        return 0;
    }

    const KMField& F_;
    cudaStream_t st_;
    std::unordered_map<int, KMCellRec> map_;
    int* d_roots_ = nullptr;
    KMCellRec* d_out_ = nullptr;
    long long cap_roots_ = 0, cap_out_ = 0;
};

inline V3 rec_pos(const KMCellRec& r) { return V3{r.x, r.y, r.z}; }

void write_centers(const std::vector<V3>& c, double* out, int dim)
{
    for (size_t i = 0; i < c.size(); ++i) {
        out[dim * i] = c[i].x;
        out[dim * i + 1] = c[i].y;
        if (dim == 3) out[dim * i + 2] = c[i].z;
    }
}

int check_npatch(const KMField& F, int npatch)
{
    if (npatch < 1) { set_last_error("npatch must be at least 1"); return TC_ERR_ARG; }
    if (npatch > KM_MAX_PATCH) {
        set_last_error("npatch above " + std::to_string(KM_MAX_PATCH) + " is not supported by the GPU k-means");
        return TC_ERR_UNSUPPORTED;
    }
    if (F.n == 0 || F.ntop == 0) { set_last_error("k-means on an empty field"); return TC_ERR_ARG; }
    return 0;
}

// InitializeCentersTree, the recursive part (src/KMeans.cpp:28-59).
int init_tree_rec(CellCache& cc, int id, long first, int nc, std::vector<V3>& cen, bool sphere)
{
    KMCellRec r;
    TC_TRY(cc.get(id, r));
    if (nc == 1) {
        cen[first] = rec_pos(r);
    } else if (r.left >= 0) {
        int m1 = nc / 2, m2 = nc - m1;
        if (urand() < 0.5) std::swap(m1, m2);
        TC_TRY(init_tree_rec(cc, r.left, first, m1, cen, sphere));
        TC_TRY(init_tree_rec(cc, r.right, first + m1, m2, cen, sphere));
    } else {
        for (int i = 0; i < nc; ++i) {
            const double f = 1. + urand() * 1.e-8;
            V3 v{r.x * f, r.y * f, r.z * f};
            if (sphere) v3_normalize(v);
            cen[first + i] = v;
        }
    }
    return 0;
}

// InitializeCentersKMPP, the recursive part (src/KMeans.cpp:159-218).  Returns 0 with the
// new centre, 1 when every leaf below is already a centre (the reference's LeafAlreadyUsed).
int kmpp_rec(CellCache& cc, int id, const std::vector<V3>& cen, long ncen, V3& out)
{
    KMCellRec r;
    if (cc.get(id, r)) return -1;
    if (r.size == 0.f) {
        const V3 p = rec_pos(r);
        for (long j = 0; j < ncen; ++j)
            if (v3_eq(p, cen[j])) return 1;
        out = p;
        return 0;
    }
    if (r.left < 0) {
        set_last_error("k-means++ reached a leaf of non-zero size (min_size > 0)");
        return -1;
    }
    KMCellRec L, R;
    if (cc.get(r.left, L) || cc.get(r.right, R)) return -1;
    double d1 = v3_dsq(rec_pos(L), cen[0]), d2 = v3_dsq(rec_pos(R), cen[0]);
    for (long j = 1; j < ncen; ++j) {
        const double a = v3_dsq(rec_pos(L), cen[j]), b = v3_dsq(rec_pos(R), cen[j]);
        if (a < d1) d1 = a;
        if (b < d2) d2 = b;
    }
    if (d1 + d2 == 0.) return 1;
    const double u = urand() * (d1 + d2);
    const int first = u < d1 ? r.left : r.right, second = u < d1 ? r.right : r.left;
    int rc = kmpp_rec(cc, first, cen, ncen, out);
    if (rc == 1) rc = kmpp_rec(cc, second, cen, ncen, out);
    return rc;
}

// Device scratch of one KMeansRun / KMeansAssign call.
struct KMScratch {
    double *cen = nullptr, *inertia = nullptr, *partial = nullptr, *tot = nullptr, *shift = nullptr;
    KMItem* items = nullptr;
    int* pool = nullptr;
    int* assign = nullptr;
    KMLevel* lvl = nullptr;
    long long item_cap = 0, pool_cap = 0;
    int acc_threads = 0;
    size_t acc_smem = 0;
    int tag = 0;           // tag of the last tree pass (assignments of older passes are stale)
    int levels = 0;        // levels with items in the last tree pass
    ~KMScratch()
    {
        dfree(cen); dfree(inertia); dfree(partial); dfree(tot); dfree(shift); dfree(items);
        dfree(pool); dfree(assign); dfree(lvl);
    }
};

int scratch_alloc(const KMField& F, int npatch, KMScratch& S)
{
    TC_TRY(dalloc(&S.cen, 3 * (size_t)npatch));
    TC_TRY(dalloc(&S.inertia, npatch));
    TC_TRY(dalloc(&S.partial, (size_t)KM_NBLK * npatch * KM_NQ));
    TC_TRY(dalloc(&S.tot, (size_t)npatch * KM_NQ));
    TC_TRY(dalloc(&S.shift, 1));
    S.item_cap = std::max<long long>(F.ncap, F.ntop);
    TC_TRY(dalloc(&S.items, S.item_cap));
    S.pool_cap = std::max<long long>(1 << 22, 4LL * npatch + 2LL * F.ntop);
    TC_TRY(dalloc(&S.pool, S.pool_cap));
    TC_TRY(dalloc(&S.assign, F.ncap));
    TC_CU(cudaMemset(S.assign, 0xff, sizeof(int) * (size_t)F.ncap));
    TC_TRY(dalloc(&S.lvl, 1));
    // Accumulator warps per block: as many as fit (at most 8), each npatch x KM_NQ doubles
    // plus a 32-lane staging row.
    const size_t per_warp = ((size_t)npatch * KM_NQ + 32 * KM_NQ) * sizeof(double);
    int nw = (int)std::min<size_t>(8, (200 * 1024) / per_warp);
    if (nw < 1) { set_last_error("k-means: too many patches for the accumulators"); return TC_ERR_UNSUPPORTED; }
    S.acc_threads = 32 * nw;
    S.acc_smem = per_warp * nw;
    if (S.acc_smem > 48 * 1024)
        TC_CU(cudaFuncSetAttribute(k_km_accum, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S.acc_smem));
    return 0;
}

int upload_centers(const double* centers, int npatch, int coords, KMScratch& S, cudaStream_t st)
{
    const int dim = coords == FLAT ? 2 : 3;
    std::vector<double> h(3 * (size_t)npatch, 0.);
    for (int p = 0; p < npatch; ++p) {
        V3 v{centers[dim * p], centers[dim * p + 1], dim == 3 ? centers[dim * p + 2] : 0.};
        if (coords == SPHERE) v3_normalize(v);   // ReadCenters builds Position<Sphere>
        h[3 * p] = v.x; h[3 * p + 1] = v.y; h[3 * p + 2] = v.z;
    }
    TC_CU(cudaMemcpyAsync(S.cen, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, st));
    TC_CU(cudaStreamSynchronize(st));
    return 0;
}

// FindCellsInPatches over the whole field: assign[cell] = patch for the cells that lie in
// one patch.
int find_cells(const KMField& F, int npatch, const double* inertia, KMScratch& S, cudaStream_t st)
{
    static int nblocks = 0;
    if (!nblocks) {
        int dev = 0, sms = 0;
        TC_CU(cudaGetDevice(&dev));
        TC_CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        nblocks = 4 * std::max(sms, 1);
    }
    for (int attempt = 0; attempt < 6; ++attempt) {
        if (++S.tag >= KM_TAG_MAX) {
            TC_CU(cudaMemsetAsync(S.assign, 0xff, sizeof(int) * (size_t)F.ncap, st));
            S.tag = 1;
        }
        const int nstart = std::max(F.ntop, npatch);
        count_launch();
        k_km_start<<<(nstart + 255) / 256, 256, 0, st>>>(F.d_tops, F.ntop, npatch, S.items, S.pool, S.lvl);
        TC_CU(cudaGetLastError());
        KMLevel h{};
        bool done = false;
        // As many levels as the last pass needed (plus one to see the end), then batches.
        int batch = S.levels > 0 ? S.levels + 1 : KM_LEVELS_PER_CHECK;
        for (int lev = 0; lev < F.ncap + 2 && !done; lev += batch, batch = KM_LEVELS_PER_CHECK) {
            for (int k = 0; k < batch; ++k) {
                count_launch();
                k_km_level<<<nblocks, KM_LTB, 0, st>>>(F.cells, S.cen, inertia, S.items, S.item_cap,
                                                       S.pool, S.pool_cap, S.assign, S.tag, S.lvl);
            }
            TC_CU(cudaGetLastError());
            TC_CU(cudaMemcpyAsync(&h, S.lvl, sizeof(KMLevel), cudaMemcpyDeviceToHost, st));
            TC_CU(cudaStreamSynchronize(st));
            if (h.err || h.lo == h.hi) done = true;
        }
        S.levels = h.levels;
        if (!done) { set_last_error("k-means: tree pass did not end"); return TC_ERR_DEVICE; }
        if (h.err == 2) { set_last_error("k-means: work item array full (inconsistent tree)"); return TC_ERR_DEVICE; }
        if (h.err == 0) return 0;
        // Candidate pool full: grow it and repeat the pass.
        dfree(S.pool);
        S.pool_cap *= 4;
        TC_TRY(dalloc(&S.pool, S.pool_cap));
    }
    set_last_error("k-means: candidate pool could not be sized");
    return TC_ERR_NOMEM;
}

int sum_cells(const KMField& F, int npatch, int mode, KMScratch& S, cudaStream_t st)
{
    count_launch();
    k_km_accum<<<KM_NBLK, S.acc_threads, S.acc_smem, st>>>(F.cells, F.ncap, S.assign, S.tag, S.cen,
                                                           npatch, mode, S.partial);
    TC_CU(cudaGetLastError());
    const int nq = npatch * KM_NQ;
    count_launch();
    k_km_total<<<(nq + 7) / 8, 256, 0, st>>>(nq, KM_NBLK, S.partial, S.tot);
    count_launch();
    k_km_finish<<<1, 1024, 0, st>>>(npatch, S.tot, mode, F.coords, S.cen, S.inertia, S.shift);
    TC_CU(cudaGetLastError());
    return 0;
}

}  // namespace

// ---------------------------------------------------------------------------------------

int kmeans_init_tree(const KMField& F, double* centers, int npatch, long long seed, cudaStream_t st)
{
    TC_TRY(check_npatch(F, npatch));
    CellCache cc(F, st);
    std::vector<KMCellRec> tops;
    TC_TRY(cc.tops(tops));
    std::vector<V3> cen(npatch);
    const long ncells = (long)tops.size();
    urand(seed);
    if (ncells > npatch) {
        const std::vector<long> sel = select_random_from(ncells, npatch);
        for (int i = 0; i < npatch; ++i) cen[i] = rec_pos(tops[sel[i]]);
    } else {
        // InitializeCentersTree (src/KMeans.cpp:61-109): n1 or n1+1 centres per top cell,
        // the counts shuffled, then a recursive split of each count.
        const long n1 = npatch / ncells, k2 = npatch % ncells, k1 = ncells - k2;
        std::vector<long> nv(ncells);
        for (long k = 0; k < ncells; ++k) nv[k] = k < k1 ? n1 : n1 + 1;
        for (long k = ncells; k > 1; --k) {
            long j = int(urand() * k);
            if (j > k - 1) j = k - 1;   // urand() == 1 exactly
            if (j != k - 1) std::swap(nv[j], nv[k - 1]);
        }
        long first = 0;
        for (long k = 0; k < ncells; ++k) {
            TC_TRY(init_tree_rec(cc, tops[k].id, first, (int)nv[k], cen, F.coords == SPHERE));
            first += nv[k];
        }
    }
    write_centers(cen, centers, F.coords == FLAT ? 2 : 3);
    return 0;
}

int kmeans_init_rand(const KMField& F, double* centers, int npatch, long long seed, cudaStream_t st)
{
    // InitializeCentersRand (src/KMeans.cpp:111-157).
    TC_TRY(check_npatch(F, npatch));
    CellCache cc(F, st);
    std::vector<KMCellRec> tops;
    TC_TRY(cc.tops(tops));
    long ntot = 0;
    for (const KMCellRec& t : tops) ntot += t.n;
    if (npatch > ntot) { set_last_error("npatch larger than the number of points"); return TC_ERR_ARG; }
    urand(seed);
    const std::vector<long> index = select_random_from(ntot, npatch);
    std::vector<V3> cen(npatch);
    for (int i = 0; i < npatch; ++i) {
        long m = index[i];
        for (size_t k = 0; k < tops.size(); ++k) {
            if (m < tops[k].n) {
                KMCellRec leaf;
                TC_TRY(cc.leaf_number(tops[k].id, m, leaf));
                cen[i] = rec_pos(leaf);
                break;
            }
            m -= tops[k].n;
        }
        for (int i1 = 0; i1 < i; ++i1) {
            if (v3_eq(cen[i1], cen[i])) {
                const double f = 1. + urand() * 1.e-8;
                cen[i].x *= f; cen[i].y *= f; cen[i].z *= f;
            }
        }
    }
    write_centers(cen, centers, F.coords == FLAT ? 2 : 3);
    return 0;
}

int kmeans_init_kmpp(const KMField& F, double* centers, int npatch, long long seed, cudaStream_t st)
{
    // InitializeCentersKMPP (src/KMeans.cpp:220-315).
    TC_TRY(check_npatch(F, npatch));
    CellCache cc(F, st);
    std::vector<KMCellRec> tops;
    TC_TRY(cc.tops(tops));
    const long ncells = (long)tops.size();
    long ntot = 0;
    for (const KMCellRec& t : tops) ntot += t.n;
    if (npatch > ntot) { set_last_error("npatch larger than the number of points"); return TC_ERR_ARG; }
    urand(seed);
    std::vector<long> per_cell(ncells, 0);
    std::vector<V3> cen(npatch);
    long m = long(urand() * ntot);
    for (long k = 0; k < ncells; ++k) {
        if (m < tops[k].n) {
            KMCellRec leaf;
            TC_TRY(cc.leaf_number(tops[k].id, m, leaf));
            cen[0] = rec_pos(leaf);
            per_cell[k] += 1;
            break;
        }
        m -= tops[k].n;
    }
    const double coef = F.coords == THREED ? 0.6 : 0.5;
    std::vector<double> p(ncells);
    for (int i = 1; i < npatch; ++i) {
        double sump = 0.;
        for (long k = 0; k < ncells; ++k) {
            const V3 tp = rec_pos(tops[k]);
            double d1 = v3_dsq(cen[0], tp);
            for (int i1 = 1; i1 < i; ++i1) {
                const double d2 = v3_dsq(cen[i1], tp);
                if (d2 < d1) d1 = d2;
            }
            const double s = (double)tops[k].size;
            p[k] = double(tops[k].n - per_cell[k]) * (d1 + coef * (s * s));
            sump += p[k];
        }
        double u = urand();
        for (long k = 0; k < ncells; ++k) {
            p[k] /= sump;
            if (u < p[k]) {
                const int rc = kmpp_rec(cc, tops[k].id, cen, i, cen[i]);
                if (rc == 1) { set_last_error("k-means++: every leaf of the chosen cell is already a centre"); return TC_ERR_DEVICE; }
                if (rc < 0) return TC_ERR_DEVICE;
                per_cell[k] += 1;
                break;
            }
            u -= p[k];
        }
    }
    write_centers(cen, centers, F.coords == FLAT ? 2 : 3);
    return 0;
}

int kmeans_run(const KMField& F, double* centers, int npatch, int max_iter, double tol, bool alt,
               cudaStream_t st, int* iters_out)
{
    // KMeansRun1 (src/KMeans.cpp:773-833).
    TC_TRY(check_npatch(F, npatch));
    KMScratch S;
    TC_TRY(scratch_alloc(F, npatch, S));
    TC_TRY(upload_centers(centers, npatch, F.coords, S, st));
    const double tolsq = (tol * F.size) * (tol * F.size) * npatch;
    int it = 0;
    for (; it < max_iter; ++it) {
        if (alt) {
            TC_TRY(find_cells(F, npatch, nullptr, S, st));
            TC_TRY(sum_cells(F, npatch, KM_SUM_INERTIA, S, st));
        }
        TC_TRY(find_cells(F, npatch, alt ? S.inertia : nullptr, S, st));
        TC_TRY(sum_cells(F, npatch, KM_SUM_CENTERS, S, st));
        double shift = 0.;
        TC_CU(cudaMemcpyAsync(&shift, S.shift, sizeof(double), cudaMemcpyDeviceToHost, st));
        TC_CU(cudaStreamSynchronize(st));
        if (shift < tolsq) { ++it; break; }
    }
    if (iters_out) *iters_out = it;
    std::vector<double> h(3 * (size_t)npatch);
    TC_CU(cudaMemcpyAsync(h.data(), S.cen, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
    TC_CU(cudaStreamSynchronize(st));
    const int dim = F.coords == FLAT ? 2 : 3;
    for (int p = 0; p < npatch; ++p) {
        centers[dim * p] = h[3 * p];
        centers[dim * p + 1] = h[3 * p + 1];
        if (dim == 3) centers[dim * p + 2] = h[3 * p + 2];
    }
    return 0;
}

int kmeans_assign(const KMField& F, const double* centers, int npatch, int64_t* patches,
                  cudaStream_t st)
{
    // KMeansAssign1 (src/KMeans.cpp:835-849).
    TC_TRY(check_npatch(F, npatch));
    KMScratch S;
    TC_TRY(scratch_alloc(F, npatch, S));
    TC_TRY(upload_centers(centers, npatch, F.coords, S, st));
    TC_TRY(find_cells(F, npatch, nullptr, S, st));
    int64_t* d_out = nullptr;
    int *big = nullptr, *nbig = nullptr;
    int rc = 0;
    do {
        if ((rc = dalloc(&d_out, F.n))) break;
        if ((rc = dalloc(&big, F.n / 32 + 1))) break;
        if ((rc = dalloc(&nbig, 1))) break;
        cudaMemsetAsync(d_out, 0xff, sizeof(int64_t) * F.n, st);
        cudaMemsetAsync(nbig, 0, sizeof(int), st);
        count_launch();
        k_km_paint<<<(F.ncap + 255) / 256, 256, 0, st>>>(F.cells, F.ncap, S.assign, S.tag, F.idx, d_out,
                                                         big, nbig);
        count_launch();
        k_km_paint_big<<<1216, 256, 0, st>>>(F.cells, S.assign, S.tag, F.idx, big, nbig, d_out);
        if (cudaGetLastError() != cudaSuccess) { set_last_error("k-means assign launch failed"); rc = TC_ERR_CUDA; break; }
        if (cudaMemcpyAsync(patches, d_out, sizeof(int64_t) * F.n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            set_last_error("k-means assign copy failed"); rc = TC_ERR_CUDA; break;
        }
    } while (0);
    dfree(d_out); dfree(big); dfree(nbig);
    return rc;
}

namespace {

int quick_common(int mode, int patch, const double* centers, int npatch, const double* x,
                 const double* y, const double* z, int64_t n, int64_t* out, bool on_device,
                 cudaStream_t st)
{
    if (npatch < 1) { set_last_error("npatch must be at least 1"); return TC_ERR_ARG; }
    if (mode == 1 && (patch < 0 || patch >= npatch)) { set_last_error("patch out of range"); return TC_ERR_ARG; }
    if (n <= 0) return 0;
    const int dim = z ? 3 : 2;
    double *dc = nullptr, *dx = nullptr, *dy = nullptr, *dz = nullptr;
    float4* d32c = nullptr;
    int64_t* dout = nullptr;
    int rc = 0;
    do {
        if ((rc = dalloc(&dc, (size_t)npatch * dim))) break;
        if (cudaMemcpyAsync(dc, centers, sizeof(double) * npatch * dim, cudaMemcpyHostToDevice, st) != cudaSuccess) {
            set_last_error("centre copy failed"); rc = TC_ERR_CUDA; break;
        }
        const double *px = x, *py = y, *pz = z;
        int64_t* po = out;
        if (!on_device) {
            if ((rc = dalloc(&dx, n)) || (rc = dalloc(&dy, n)) || (z && (rc = dalloc(&dz, n))) ||
                (rc = dalloc(&dout, n)))
                break;
            cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dy, y, sizeof(double) * n, cudaMemcpyHostToDevice, st);
            if (z) cudaMemcpyAsync(dz, z, sizeof(double) * n, cudaMemcpyHostToDevice, st);
            px = dx; py = dy; pz = z ? dz : nullptr; po = dout;
        }
        // The centres shifted to centre 0, in FP32, and their largest |coordinate|.
        std::vector<float4> h32(npatch);
        float rmax = 0.f;
        for (int k = 0; k < npatch; ++k) {
            const float cx = (float)(centers[dim * k] - centers[0]);
            const float cy = (float)(centers[dim * k + 1] - centers[1]);
            const float cz = dim == 3 ? (float)(centers[dim * k + 2] - centers[2]) : 0.f;
            h32[k] = make_float4(cx, cy, cz, 0.f);
            rmax = std::max(rmax, std::max(std::fabs(cx), std::max(std::fabs(cy), std::fabs(cz))));
        }
        if ((rc = dalloc(&d32c, (size_t)npatch)) != 0) break;
        if (cudaMemcpyAsync(d32c, h32.data(), sizeof(float4) * npatch, cudaMemcpyHostToDevice, st) != cudaSuccess) {
            set_last_error("centre copy failed"); rc = TC_ERR_CUDA; break;
        }
        const size_t csm = sizeof(float4) * npatch;
        const int in_smem = csm <= 48 * 1024 ? 1 : 0;
        count_launch();
        k_quick_assign<<<(unsigned)((n + 255) / 256), 256, in_smem ? csm : 0, st>>>(
            dc, d32c, rmax, npatch, dim, px, py, pz, n, mode, patch, po, in_smem);
        if (cudaGetLastError() != cudaSuccess) { set_last_error("assign launch failed"); rc = TC_ERR_CUDA; break; }
        if (!on_device &&
            cudaMemcpyAsync(out, dout, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess) {
            set_last_error("assign copy failed"); rc = TC_ERR_CUDA; break;
        }
        if (cudaStreamSynchronize(st) != cudaSuccess) { set_last_error("assign failed"); rc = TC_ERR_CUDA; break; }
    } while (0);
    dfree(dc); dfree(d32c); dfree(dx); dfree(dy); dfree(dz); dfree(dout);
    return rc;
}

}  // namespace

int quick_assign(const double* centers, int npatch, const double* x, const double* y,
                 const double* z, int64_t n, int64_t* out, bool on_device, cudaStream_t st)
{
    return quick_common(0, 0, centers, npatch, x, y, z, n, out, on_device, st);
}

int select_patch(int patch, const double* centers, int npatch, const double* x, const double* y,
                 const double* z, int64_t n, int64_t* use, bool on_device, cudaStream_t st)
{
    return quick_common(1, patch, centers, npatch, x, y, z, n, use, on_device, st);
}

}  // namespace tc
