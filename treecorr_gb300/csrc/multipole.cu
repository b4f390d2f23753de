// multipole.cu -- 3-point correlations with LogMultipole binning on sm_103a (all N / K / G
// classes: GGG's contraction over the payloads each class needs, see MPParams).
//
// Semantics follow the reference's multipole algorithm (Porth et al.):
//   BaseCorr3::multipole (src/Corr3.cpp:1124-1175; cross12 1177-1237; three-field
//   1239-1305), multipoleSplit1 (1374-1449), splitC2Cells (1323-1372), multipoleFinish
//   (1548-1679), splitC2CellsOrCalculateGn (1452-1546), Corr3::calculateGn +
//   MultipoleScratch<GData>::calculateGn (1681-1704, 1767-1828), Corr3::calculateZeta
//   (1861-2087) and MultipoleHelper<1..6>::CalculateZeta (2108-3082); scratch layout
//   include/MultipoleScratch.h:36-125, 296-383.
//
// GB300 design:
//   * Phase 1: one block per top-level cell walks the c1 subtree of multipoleSplit1, refining
//     the c2 list with block-parallel decisions and a stable block scan, and emits one job
//     (c1, c2 list) per cell that is small enough to start multipoleFinish.
//   * Phase 2: persistent blocks take jobs from a counter.  A job runs multipoleFinish as a
//     depth-first loop: each pass over the c2 list is block-parallel; every accepted pair
//     becomes a record of its FP64-computed terms stored as FP32 (phase z, projected shear,
//     scalar sums).  The records are ranked stably by bin and split evenly over the warps;
//     a warp forms z^n for n = 1..max_n+1 with one multiplicative warp scan per record, sums
//     the G_n / W_n terms in FP32 and flushes them to the FP64 scratch.  When c1 must split,
//     the scratch is copied into a free slot and the right child is pushed, as the
//     reference's mp.duplicate() does.
//   * Rows of Zeta that are final become vertex records (FP32 copies of G_n and W_n).  The
//     contraction over vertices is a sum of outer products per n; k_mp_zeta runs it in
//     batches (waves) between runs of the finish kernel, FP32 products with FP64 sums.
//   * A last kernel sums the per-block outputs, the contraction partials and the diagonal
//     self-pair corrections in a fixed order.
//   * A three-field cross keeps vertex 3's pairs in scratch bins [nbd, 2 nbd), so the same
//     kernels produce both cross blocks of a (2 nbd)^2 matrix (MPParams::three).
// Geometry and the split/accept decisions are taken in FP32 with error margins
// (mp_decide32); an entry inside a margin is decided again in FP64 with the reference's
// arithmetic, so the decisions are the reference's.  The cell payloads are the tree's float
// values.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "tc_internal.cuh"
#include "tc_host.hpp"
#include "multipole.hpp"
#include "tc_mma.cuh"

namespace tc {

static constexpr int MB = 256;            // threads per multipole block
static constexpr int MW = MB / 32;        // warps per block
static constexpr int MSTACK = 128;        // depth of the block-local stacks

// ---------------------------------------------------------------------------------------
// Leaf sums of every cell: calculateSumWSq, calculateSumWZSq, calculateSumAbsWZSq
// (src/Cell.cpp:138-168).  A cell is a leaf of these sums if its size is 0, it holds one
// point, or it has no children; each such leaf adds w^2, (wz)^2 and |wz|^2 to itself and
// to every ancestor.

__global__ void k_leaf_sums(int ncap, Cells C, double* ls)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncap) return;
    if (C.n[i] <= 0) return;   // unused id
    const bool leaf = (C.size[i] == 0.f) || (C.n[i] == 1) || (C.left[i] < 0);
    if (!leaf) return;
    // Skip cells nested below another summation leaf (their sum is already counted there).
    for (int p = C.parent[i]; p >= 0; p = C.parent[p])
        if (C.size[p] == 0.f) return;
    const double w = C.w[i];
    const double gr = C.d1[i], gi = C.d2[i];
    const double v0 = w * w, v1 = gr * gr - gi * gi, v2 = 2. * gr * gi, v3 = gr * gr + gi * gi;
    for (int p = i; p >= 0; p = C.parent[p]) {
        atomicAdd(&ls[4 * (size_t)p + 0], v0);
        atomicAdd(&ls[4 * (size_t)p + 1], v1);
        atomicAdd(&ls[4 * (size_t)p + 2], v2);
        atomicAdd(&ls[4 * (size_t)p + 3], v3);
    }
}

__global__ void k_leaf_sums_f(int ncap, const double* ls, float4* lsf)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncap) return;
    const double* p = ls + 4 * (size_t)i;
    lsf[i] = make_float4((float)p[0], (float)p[1], (float)p[2], (float)p[3]);
}

// The cells of an N or K pair field as a real payload (GNN, GKK, NKK, KNN, KKK;
// MultipoleHelper<4> and <1>, src/Corr3.cpp:2462-2580, 2108-2214): (d1, d2) := (w, 0) for N
// (Sigma w z^n is its G_n), (w k, 0) for K; the leaf sums (sum w^2 or sum (w k)^2, 0) stand
// where the squared shear was.
__global__ void k_mp_scalar_pairs(int ncap, int is_n, TCell* tc, float* d1, float* d2,
                                  double* ls, float4* lsf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncap) return;
    TCell c = tc[i];
    if (is_n) c.c.x = c.b.w;
    c.c.y = 0.f;
    tc[i] = c;
    d1[i] = c.c.x;
    d2[i] = 0.f;
    double* l = ls + 4 * (size_t)i;
    if (is_n) l[1] = l[0];
    l[2] = 0.;
    lsf[i] = make_float4((float)l[0], (float)l[1], 0.f, (float)l[3]);
}

int launch_scalar_pairs(int ncap, int is_n, TCell* tc, float* d1, float* d2, double* ls,
                        float4* lsf, cudaStream_t st)
{
    if (ncap <= 0) return 0;
    count_launch();
    k_mp_scalar_pairs<<<(ncap + 255) / 256, 256, 0, st>>>(ncap, is_n, tc, d1, d2, ls, lsf);
    TC_CU(cudaGetLastError());
    return 0;
}

int launch_leaf_sums(int ncap, const Cells& C, double* ls, float4* lsf, cudaStream_t st)
{
    TC_CU(cudaMemsetAsync(ls, 0, 4 * sizeof(double) * (size_t)ncap, st));
    count_launch();
    k_leaf_sums<<<(ncap + 255) / 256, 256, 0, st>>>(ncap, C, ls);
    TC_CU(cudaGetLastError());
    count_launch();
    k_leaf_sums_f<<<(ncap + 255) / 256, 256, 0, st>>>(ncap, ls, lsf);
    TC_CU(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------------------
// FP64 geometry and rules.

struct C2 { double re, im; };
__device__ __forceinline__ C2 cmul(C2 a, C2 b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ C2 conj2(C2 a) { return {a.re, -a.im}; }
__device__ __forceinline__ C2 cadd(C2 a, C2 b) { return {a.re + b.re, a.im + b.im}; }

__device__ __forceinline__ void norm3(double& x, double& y, double& z)
{
    double n = sqrt(x * x + y * y + z * z);
    if (n == 0.) { x = 1.; y = 0.; z = 0.; } else { x /= n; y /= n; z /= n; }
}

__device__ __forceinline__ double mp_dist_sq(const MPParams& P, int i, int j)
{
    double dx = P.x[i] - P.x[j], dy = P.y[i] - P.y[j];
    if (P.coords == FLAT) return dx * dx + dy * dy;
    double dz = P.z[i] - P.z[j];
    double dsq = dx * dx + dy * dy + dz * dz;
    if (P.metric == ARC) { double th = 2. * asin(sqrt(dsq) / 2.); return th * th; }
    return dsq;
}

// BinTypeHelper<Log>::singleBin, include/BinType.h:93-151.
__device__ __forceinline__ bool mp_single_bin(const MPParams& P, double rsq, double s1ps2, int& ik,
                                              double& r, double& logr)
{
    if (s1ps2 == 0.) return true;
    double s2 = s1ps2 * s1ps2;
    if (s2 > P.asq * rsq) return false;
    if (s2 <= P.bsq * rsq) return true;
    if (s2 > 0.25 * (P.binsize + P.b) * (P.binsize + P.b) * rsq) return false;
    logr = 0.5 * log(rsq);
    double kk = (logr - P.logminsep) / P.binsize;
    ik = int(kk);
    double frac = kk - ik;
    double f = fmin(frac, 1. - frac);
    double t4 = f * P.binsize + P.b;
    if (s2 > t4 * t4 * rsq) return false;
    double t5 = frac * P.binsize + P.b - s2 / rsq;
    if (s2 > t5 * t5 * rsq) return false;
    r = sqrt(rsq);
    return true;
}

__device__ __forceinline__ bool mp_too_small(const MPParams& P, double rsq, double s)
{ return rsq < P.minsepsq && s < P.minsep && rsq < (P.minsep - s) * (P.minsep - s); }
__device__ __forceinline__ bool mp_too_large(const MPParams& P, double rsq, double s)
{ return rsq >= P.maxsepsq && rsq >= (P.maxsep + s) * (P.maxsep + s); }

// FP32 decisions.  Each comparison a < b is made with a relative margin: inside the margin
// the entry is left to the FP64 code above, so every decision taken here equals the FP64
// one.  Margins: 1e-5 for plain comparisons (FP32 rounding of rsq, s and the constants is
// below 1e-6), 2e-4 where the fractional bin position enters (its FP32 error is below 1e-5).
__device__ __forceinline__ int lt3(float a, float b, float m)
{
    const float d = m * (fabsf(a) + fabsf(b));
    if (a < b - d) return 1;
    if (a > b + d) return 0;
    return -1;
}

// One (c1, c2) entry of a multipoleFinish pass in FP32.  Returns -1 (undecided: use FP64),
// 0 (dropped: too small, too large, or accepted outside [min_sep, max_sep)), 1 (accepted
// into bin k; r and logr returned) or 2 (not accepted: split flags, any = split1 and
// r + s > thresh1, r returned).
__device__ __forceinline__ int mp_decide32(const MPParams& P, float rsq, float s1, float s2,
                                           float thresh1, int& k, float& r, float& logr,
                                           bool& split1, bool& split2, bool& any)
{
    constexpr float M5 = 1e-5f, ML = 2e-4f;
    const float s = s1 + s2;
    // tooSmallDist: rsq < min_sep^2 && s < min_sep && rsq < (min_sep - s)^2.  min_sep - s
    // loses relative accuracy when s is close to min_sep: those go to FP64.
    const int below_min = lt3(rsq, P.f_minsepsq, M5);
    if (below_min < 0) return -1;
    if (below_min == 1) {
        const int c2 = lt3(s, P.f_minsep, M5);
        if (c2 < 0) return -1;
        if (c2 == 1) {
            const float d = P.f_minsep - s;
            if (d < 0.01f * P.f_minsep) return -1;
            const int c3 = lt3(rsq, d * d, ML);
            if (c3 < 0) return -1;
            if (c3 == 1) return 0;
        }
    }
    const int below_max = lt3(rsq, P.f_maxsepsq, M5);
    if (below_max < 0) return -1;
    if (below_max == 0) {                       // tooLargeDist
        const float ms = P.f_maxsep + s;
        const int c = lt3(rsq, ms * ms, M5);
        if (c < 0) return -1;
        if (c == 0) return 0;
    }
    // BinTypeHelper<Log>::singleBin
    bool sb;
    int ik = -1;
    float lr = 0.f;
    if (s == 0.f) {
        sb = true;
    } else {
        const float s2q = s * s;
        int c = lt3(P.f_asq * rsq, s2q, M5);
        if (c < 0) return -1;
        if (c == 1) {
            sb = false;
        } else {
            c = lt3(P.f_bsq * rsq, s2q, M5);
            if (c < 0) return -1;
            if (c == 0) {
                sb = true;
            } else {
                c = lt3(P.f_q25 * rsq, s2q, M5);
                if (c < 0) return -1;
                if (c == 1) {
                    sb = false;
                } else {
                    lr = 0.5f * logf(rsq);
                    const float kk = (lr - P.f_logminsep) / P.f_binsize;
                    ik = (int)kk;
                    const float frac = kk - (float)ik;
                    const float af = fabsf(frac);      // kk < 0 below min_sep: frac <= 0
                    if (af < ML || af > 1.f - ML) return -1;
                    const float f = fminf(frac, 1.f - frac);
                    const float t4 = f * P.f_binsize + P.f_b;
                    c = lt3(t4 * t4 * rsq, s2q, ML);
                    if (c < 0) return -1;
                    if (c == 1) {
                        sb = false;
                    } else {
                        const float t5 = frac * P.f_binsize + P.f_b - s2q / rsq;
                        c = lt3(t5 * t5 * rsq, s2q, ML);
                        if (c < 0) return -1;
                        sb = (c != 1);
                    }
                }
            }
        }
    }
    r = sqrtf(rsq);
    if (sb) {
        if (below_max == 0 || below_min == 1) return 0;   // isRSqInRange fails
        if (ik < 0) {
            lr = logf(r);
            const float kk = (lr - P.f_logminsep) / P.f_binsize;
            ik = (int)kk;
            const float frac = kk - (float)ik;
            if (frac < ML || frac > 1.f - ML) return -1;
        }
        k = ik < P.nbd ? ik : P.nbd - 1;
        logr = lr;
        return 1;
    }
    // CalcSplitSq (include/Split.h:82-101); s1, s2 are the cells' float sizes, so the size
    // comparisons are exact.
    const float bsq_eff = rsq * P.f_minba;
    if (s2 > s1) {
        split2 = true;
        if (s2 > 2.f * s1) split1 = false;
        else {
            const int c = lt3(0.3422f * bsq_eff, s1 * s1, M5);
            if (c < 0) return -1;
            split1 = (c == 1);
        }
    } else {
        split1 = true;
        if (s1 > 2.f * s2) split2 = false;
        else {
            const int c = lt3(0.3422f * bsq_eff, s2 * s2, M5);
            if (c < 0) return -1;
            split2 = (c == 1);
        }
    }
    any = false;
    if (split1) {
        const int c = lt3(thresh1, r + s, M5);
        if (c < 0) return -1;
        any = (c == 1);
    }
    return 2;
}

// calculate_direction(p1, p2) of include/ProjectHelper.h:272-345 (unnormalised).
__device__ __forceinline__ C2 direction(double x1, double y1, double z1, double x2, double y2,
                                        double z2)
{
    double dsq = (x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2) + (z1 - z2) * (z1 - z2);
    double cosA = (z1 - z2) + 0.5 * z2 * dsq;
    double sinA = y1 * x2 - x1 * y2;
    return {sinA, -cosA};
}

// ExpIPhi (ProjectHelper.h:264-266, 526-535, 688-697) and the spin-2 projection factor
// conj(r^2)/|r|^2 of ProjectWithSq, for the pair (c1, c2).
__device__ __forceinline__ void phases(const MPParams& P, int i, int j, double r, C2& z, C2& e)
{
    if (P.coords == FLAT) {
        double dx = P.x[j] - P.x[i], dy = P.y[j] - P.y[i];
        z = {dx / r, dy / r};
        double n = dx * dx + dy * dy;
        if (!(n > 0.)) n = 1.;
        e = {(dx * dx - dy * dy) / n, -(2. * dx * dy) / n};
        return;
    }
    double x1 = P.x[i], y1 = P.y[i], z1 = P.z[i], x2 = P.x[j], y2 = P.y[j], z2 = P.z[j];
    if (P.coords == THREED) { norm3(x1, y1, z1); norm3(x2, y2, z2); }
    C2 d = direction(x2, y2, z2, x1, y1, z1);
    double n = d.re * d.re + d.im * d.im;
    if (!(n > 0.)) n = 1.;
    double sn = sqrt(n);
    z = {d.re / sn, d.im / sn};
    C2 q = direction(x1, y1, z1, x2, y2, z2);
    double m = q.re * q.re + q.im * q.im;
    if (!(m > 0.)) m = 1.;
    e = {(q.re * q.re - q.im * q.im) / m, -(2. * q.re * q.im) / m};
}

// ---------------------------------------------------------------------------------------
// Block helpers.

__device__ __forceinline__ int block_excl_scan(int v, int* sh, int& total)
{
    // sh: MW ints.
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[wid] = x;
    __syncthreads();
    int pre = 0;
    total = 0;
    for (int k = 0; k < MW; ++k) {
        if (k < wid) pre += sh[k];
        total += sh[k];
    }
    __syncthreads();
    return pre + x - v;
}

__device__ __forceinline__ void set_mp_err(int* err, int code) { atomicCAS(err, 0, code); }

// A consistency check that failed: record the site, the caller skips the item.
__device__ __forceinline__ void mp_check_fail(int* err, int site)
{
    atomicCAS(err, 0, MP_ERR_CHECK);
    atomicCAS(err + 1, 0, site);
}

__device__ __forceinline__ bool mp_valid_cell(const MPParams& P, int c)
{ return c >= 0 && c < P.ncells && P.n[c] > 0; }

// ---------------------------------------------------------------------------------------
// Phase 1: multipoleSplit1 + splitC2Cells, one block per vertex-1 top-level cell; its pair
// list starts as all top cells of the pair field (the same field for an auto-correlation,
// src/Corr3.cpp:1124-1175; field 2 for cross12, 1177-1237).

struct P1Entry { int c1, off, len, pad; };

__global__ void __launch_bounds__(MB) k_mp_split1(MPParams P)
{
    __shared__ P1Entry stk[MSTACK];
    __shared__ int sp, top_rel, scan_sh[MW], have_sh;
    __shared__ P1Entry cur;
    const int b = blockIdx.x;
    int* arena = P.arena1 + (size_t)b * P.arena1_cap;
    const int tid = threadIdx.x;
    for (int j = tid; j < P.ntop2; j += MB) arena[j] = P.tops2[j];
    if (tid == 0) {
        sp = 0;
        top_rel = P.ntop2;
        stk[sp++] = {P.tops[b], 0, P.ntop2, 0};
    }
    __syncthreads();
    int guard = 0;
    while (true) {
        // Thread 0 pops; everyone learns the outcome from a flag written before the barrier
        // (reading sp directly would race with the pop).
        __syncthreads();
        if (tid == 0) {
            have_sh = sp > 0;
            if (have_sh) cur = stk[--sp];
        }
        __syncthreads();
        if (!have_sh) break;
        if (++guard > (1 << 24)) {
            if (tid == 0) set_mp_err(P.err, MP_ERR_STACK);
            break;
        }
        const int c1 = cur.c1;
        const double s1 = P.size[c1];
        const int base = top_rel;
        int written = 0;
        for (int j0 = 0; j0 < cur.len; j0 += MB) {
            const int j = j0 + tid;
            int cnt = 0, ca = -1, cb = -1;
            const int c2 = j < cur.len ? __ldcg(arena + cur.off + j) : 0;
            if (j < cur.len && !mp_valid_cell(P, c2)) mp_check_fail(P.err, 1);
            else if (j < cur.len) {
                const double s2 = P.size[c2];
                const double rsq = mp_dist_sq(P, c1, c2);
                const double s = s1 + s2;
                if (!mp_too_small(P, rsq, s) && !mp_too_large(P, rsq, s)) {
                    int k = -1;
                    double r = 0., lr = 0.;
                    bool split = !mp_single_bin(P, rsq, s, k, r, lr);
                    if (split && s2 > s1) { ca = P.left[c2]; cb = P.right[c2]; cnt = 2; }
                    else { ca = c2; cnt = 1; }
                }
            }
            int total;
            int pos = block_excl_scan(cnt, scan_sh, total);
            if (base + written + total > P.arena1_cap) {
                if (tid == 0) set_mp_err(P.err, MP_ERR_ARENA);
            } else {
                if (cnt >= 1) arena[base + written + pos] = ca;
                if (cnt == 2) arena[base + written + pos + 1] = cb;
            }
            written += total;
        }
        __syncthreads();
        if (base + written > P.arena1_cap) break;   // overflow flagged: lists incomplete
        if (tid == 0) {
            top_rel = base + written;
            if ((double)s1 * (double)s1 > P.maxbsq_eff && P.left[c1] >= 0) {
                if (sp + 2 > MSTACK) set_mp_err(P.err, MP_ERR_STACK);
                else {
                    stk[sp++] = {P.right[c1], base, written, 0};
                    stk[sp++] = {P.left[c1], base, written, 0};
                }
            } else {
                unsigned long long jn = atomicAdd(P.njobs, 1ull);
                if ((long long)jn < P.jobs_cap) P.jobs[jn] = make_int4(c1, b, base, written);
                else set_mp_err(P.err, MP_ERR_JOBS);
            }
        }
    }
}

// ---------------------------------------------------------------------------------------
// Phase 2: multipoleFinish per job.

// maxr / maxr3: the previous pass's largest remaining r + s over the vertex-2 (or only)
// list and the vertex-3 list (multipoleFinish keeps them apart, src/Corr3.cpp:1616-1679).
struct P2Entry { int c1, len, slot, mink; long long goff; double maxr, maxr3; long long mark; };

// Scratch slot layout (doubles): W_n [n = 0 .. M][bin] complex, G_n [n + M + 1 = 0 .. 2M+2]
// [bin] complex, gg0/gg1/gg2 [bin] complex, then npairs, sumw, sumwr, sumwlogr, sumww,
// sumwwr, sumwwlogr [bin].  The [n][bin] order is the vertex record's order.
__device__ __forceinline__ size_t sW(int nb, int n, int k) { return 2 * ((size_t)n * nb + k); }
__device__ __forceinline__ size_t sG(int nb, int M, int n, int k)
{ return 2 * ((size_t)(n + M + 1) * nb + k); }
__device__ __forceinline__ double* slot_ptr(const MPParams& P, int blk, int s)
{ return P.slots + ((size_t)blk * P.nslots + s) * P.slot_doubles; }

// Accepted-pair record (MP_REC floats): z (2), wg = g2 * e (2), w2, n2 (int), k (int), pad,
// then the 14 scalar terms of calculateGn: w2, w2 r, w2 logr, sum w^2, (sum w^2) r,
// (sum w^2) logr, sumwwgg0 (2), sumwwgg1 (2), sumwwgg2 (2), wg (2).
static constexpr int REC_K = 6, REC_S = 8, NSCAL = 14;

// Bin-ordered G_n / W_n accumulation of the records [0, nrec) of this block into slot S.
// The records are ranked stably by bin (list order within a bin), then warp w takes the
// w-th contiguous share of the ranked records.  A warp walks its share one record at a time:
// lane l forms z^(l+1) (and z^(l+33)) by a multiplicative warp scan and adds the record's
// W_n, G_{+n}, G_{-n} terms in FP32; lanes 0..13 add the scalar terms, lane 14 counts n2.
// The FP32 partials go to FP64 registers every 32 records and to the slot (FP64 atomics,
// since two warps can share a bin) when the bin changes.
__device__ void mp_accumulate(const MPParams& P, const float* rec, int* perm, int nrec,
                              double* S, int* bh, int (*bw)[MP_MAXNB])
{
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int nb = P.nbins, M = P.maxn, gst = 2 * M + 3;
    // Stable ranking by bin: bh holds the per-bin counts on entry.
    if (tid == 0) {
        int s = 0;
        for (int k = 0; k < nb; ++k) { const int c = bh[k]; bh[k] = s; s += c; }
        if (s != nrec) mp_check_fail(P.err, 8);   // counts and records disagree
    }
    for (int q = tid; q < MW * MP_MAXNB; q += MB) bw[q / MP_MAXNB][q % MP_MAXNB] = 0;
    for (int a = tid; a < nrec; a += MB) perm[a] = -1;
    __syncthreads();
    for (int c0 = 0; c0 < nrec; c0 += MB) {
        const int a = c0 + tid;
        const int k = a < nrec ? __float_as_int(__ldcg(rec + (size_t)a * MP_REC + REC_K)) : nb;
        const unsigned peers = __match_any_sync(0xffffffffu, k);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (a < nrec && rank == 0) bw[wid][k] = __popc(peers);
        __syncthreads();
        if (a < nrec) {
            int pos = bh[k] + rank;
            for (int w = 0; w < wid; ++w) pos += bw[w][k];
            perm[pos] = a;
        }
        __syncthreads();
        if (tid < nb) {
            int t = 0;
            for (int w = 0; w < MW; ++w) { t += bw[w][tid]; bw[w][tid] = 0; }
            bh[tid] += t;
        }
        __syncthreads();
    }
    for (int k = tid; k < nb; k += MB) bh[k] = 0;   // counts of the next batch
    double* W = S;
    double* G = S + 2 * (size_t)nb * (M + 1);
    double* GG = G + 2 * (size_t)nb * gst;
    double* SC = GG + 6 * (size_t)nb;
    const int per = (nrec + MW - 1) / MW;
    const int p0 = wid * per, p1 = min(nrec, p0 + per);
    constexpr int KNONE = 0x7fffffff;
    __shared__ float4 bz[MW][32];
    __shared__ float2 bk[MW][32];
    // FP32 sums of the current bin: F over one batch, F2 over up to 32 batches; they reach
    // FP64 (D, then the slot) only every 32 batches and when the bin changes.
    float F[12], F2[12];
    double D[12];
#pragma unroll
    for (int q = 0; q < 12; ++q) { F[q] = 0.f; F2[q] = 0.f; D[q] = 0.; }
    int curk = -1, nbatch = 0;
    // Power sums of lane n = lane+1 (and lane+33) to the slot.
    auto flushp = [&](int k) {
#pragma unroll
        for (int q = 0; q < 12; ++q) { D[q] += (double)(F2[q] + F[q]); F[q] = 0.f; F2[q] = 0.f; }
        nbatch = 0;
        const int n = lane + 1, n1 = lane + 33;
        if (n <= M) { double* wp = W + sW(nb, n, k); atomicAdd(wp, D[0]); atomicAdd(wp + 1, D[1]); }
        if (n <= M + 1) {
            double* gpp = G + sG(nb, M, n, k);
            double* gmp = G + sG(nb, M, -n, k);
            atomicAdd(gpp, D[2]); atomicAdd(gpp + 1, D[3]);
            atomicAdd(gmp, D[4]); atomicAdd(gmp + 1, D[5]);
        }
        if (n1 <= M) { double* wp = W + sW(nb, n1, k); atomicAdd(wp, D[6]); atomicAdd(wp + 1, D[7]); }
        if (n1 <= M + 1) {
            double* gpp = G + sG(nb, M, n1, k);
            double* gmp = G + sG(nb, M, -n1, k);
            atomicAdd(gpp, D[8]); atomicAdd(gpp + 1, D[9]);
            atomicAdd(gmp, D[10]); atomicAdd(gmp + 1, D[11]);
        }
#pragma unroll
        for (int q = 0; q < 12; ++q) D[q] = 0.;
    };
    // Batches of 32 ranked records: lane l loads record base+l.  The scalar terms are summed
    // by a segmented warp scan over the lanes of equal bin (the bins ascend along the lanes);
    // the last lane of each run adds its run to the slot.  The powers walk the batch one
    // record at a time with the record's values taken from its lane.
    // Scalar sums of one run of bin kb to the slot.
    auto flush_scal = [&](int kb, const float* v, long long cnt) {
#pragma unroll
        for (int q = 0; q < 6; ++q) atomicAdd(&SC[(size_t)(q + 1) * nb + kb], (double)v[q]);
#pragma unroll
        for (int q = 0; q < 6; ++q) atomicAdd(&GG[(size_t)(q >> 1) * 2 * nb + 2 * kb + (q & 1)], (double)v[6 + q]);
        atomicAdd(&G[sG(nb, M, 0, kb)], (double)v[12]);
        atomicAdd(&G[sG(nb, M, 0, kb) + 1], (double)v[13]);
        atomicAdd(&W[sW(nb, 0, kb)], (double)v[0]);
        atomicAdd(&SC[kb], (double)cnt);
    };
    float cs[NSCAL];                  // carried run: FP32 scalar sums, count, bin, batches
    long long cn = 0;
    int ck = -1, cnum = 0;
#pragma unroll
    for (int q = 0; q < NSCAL; ++q) cs[q] = 0.f;
    for (int base = p0; base < p1; base += 32) {
        const int p = base + lane;
        bool ok = p < p1;
        const int pi = ok ? __ldcg(perm + p) : 0;
        if (ok && (pi < 0 || pi >= nrec)) {          // every rank is filled exactly once
            mp_check_fail(P.err, 4);
            ok = false;
        }
        const float4* r4 = reinterpret_cast<const float4*>(rec + (size_t)(ok ? pi : 0) * MP_REC);
        const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 h0 = ok ? __ldcg(r4) : zero4, h1 = ok ? __ldcg(r4 + 1) : zero4;
        const float4 q0 = ok ? __ldcg(r4 + 2) : zero4, q1 = ok ? __ldcg(r4 + 3) : zero4;
        const float4 q2 = ok ? __ldcg(r4 + 4) : zero4, q3 = ok ? __ldcg(r4 + 5) : zero4;
        int k = ok ? __float_as_int(h1.z) : KNONE;
        if (ok && (k < 0 || k >= nb)) { mp_check_fail(P.err, 5); k = KNONE; ok = false; }
        float sv[NSCAL] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w,
                           q2.x, q2.y, q2.z, q2.w, q3.x, q3.y};
        long long n2 = ok ? (long long)__float_as_int(h1.y) : 0;
        if (!ok) {
#pragma unroll
            for (int q = 0; q < NSCAL; ++q) sv[q] = 0.f;
        }
        // The run carried from the previous batch joins lane 0 when the bin continues, and
        // goes to the slot when it does not.
        if (lane == 0 && ck >= 0) {
            if (k == ck) {
#pragma unroll
                for (int q = 0; q < NSCAL; ++q) sv[q] += cs[q];
                n2 += cn;
            } else {
                flush_scal(ck, cs, cn);
            }
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int kk = __shfl_up_sync(0xffffffffu, k, o);
            const bool same = lane >= o && kk == k;
#pragma unroll
            for (int q = 0; q < NSCAL; ++q) {
                const float t = __shfl_up_sync(0xffffffffu, sv[q], o);
                if (same) sv[q] += t;
            }
            const long long tn = __shfl_up_sync(0xffffffffu, n2, o);
            if (same) n2 += tn;
        }
        const int kn = __shfl_down_sync(0xffffffffu, k, 1);
        // The last run of the batch is carried on while it stays short; runs that end inside
        // the batch, or at the end of the warp's range, go to the slot.
        const bool last_batch = base + 32 >= p1;
        const bool run_end = ok && (lane == 31 || kn != k);
        const bool carry = run_end && lane == 31 && !last_batch && cnum < 32;
        if (run_end && !carry) flush_scal(k, sv, n2);
        {
            const bool c31 = __shfl_sync(0xffffffffu, carry, 31);
            const int k31 = __shfl_sync(0xffffffffu, k, 31);
#pragma unroll
            for (int q = 0; q < NSCAL; ++q) cs[q] = __shfl_sync(0xffffffffu, sv[q], 31);
            cn = __shfl_sync(0xffffffffu, n2, 31);
            ck = c31 ? k31 : -1;
            cnum = c31 ? cnum + 1 : 0;
        }
        const int nv = min(32, p1 - base);
        // The batch's (z, wg) and (w2, k) go through shared memory: lane j's record is read
        // by the whole warp with broadcast loads.
        bz[wid][lane] = h0;
        bk[wid][lane] = make_float2(h1.x, __int_as_float(k));
        __syncwarp();
        const int m = lane + 1;
        for (int j = 0; j < nv; ++j) {
            const float4 hz = bz[wid][j];
            const float2 hk = bk[wid][j];
            const int kj = __float_as_int(hk.y);
            const float zr = hz.x, zi = hz.y, wgr = hz.z, wgi = hz.w, w2 = hk.x;
            if (kj == KNONE) continue;
            if (kj != curk) {
                if (curk >= 0) flushp(curk);
                curk = kj;
            }
            // z^(lane+1) by binary powering: every lane squares z up to z^32 and multiplies
            // the powers of the bits of lane+1.
            float pre = 1.f, pim = 0.f, br = zr, bi = zi;
#pragma unroll
            for (int t = 0; t < 6; ++t) {
                if (m & (1 << t)) { const float u = pre * br - pim * bi; pim = pre * bi + pim * br; pre = u; }
                if (t < 5) { const float u = br * br - bi * bi; bi = 2.f * br * bi; br = u; }
            }
            F[0] += w2 * pre; F[1] += w2 * pim;
            F[2] += wgr * pre - wgi * pim; F[3] += wgr * pim + wgi * pre;
            F[4] += wgr * pre + wgi * pim; F[5] += wgi * pre - wgr * pim;
            if (M + 1 > 32) {
                const float z32r = br, z32i = bi;     // z^32
                const float qr = z32r * pre - z32i * pim, qi = z32r * pim + z32i * pre;
                F[6] += w2 * qr; F[7] += w2 * qi;
                F[8] += wgr * qr - wgi * qi; F[9] += wgr * qi + wgi * qr;
                F[10] += wgr * qr + wgi * qi; F[11] += wgi * qr - wgr * qi;
            }
        }
#pragma unroll
        for (int q = 0; q < 12; ++q) { F2[q] += F[q]; F[q] = 0.f; }
        if (++nbatch == 32) {
#pragma unroll
            for (int q = 0; q < 12; ++q) { D[q] += (double)F2[q]; F2[q] = 0.f; }
            nbatch = 0;
        }
        __syncwarp();
    }
    if (curk >= 0) flushp(curk);
    __syncthreads();
}

// The n = 0 scalar outputs of calculateZeta for rows k2 in [ks, mk): ntri, meand2/3,
// meanlogd2/3 (FP64, into the block's outputs).
__device__ void zeta_scalars(const MPParams& P, int c1, const double* S, int ks, int mk,
                             double* out)
{
    const int nb = P.nbins, M = P.maxn, nn = 2 * M + 1;
    const int gst = 2 * M + 3;
    const size_t Z = (size_t)nb * nb * nn;
    const double* SC = S + 2 * (size_t)nb * (M + 1) + 2 * (size_t)nb * gst + 6 * (size_t)nb;
    // The slot was just updated by atomics: read it from L2.
    auto npairs = [&](int k) { return __ldcg(SC + k); };
    auto sumw = [&](int k) { return __ldcg(SC + nb + k); };
    auto sumwr = [&](int k) { return __ldcg(SC + 2 * nb + k); };
    auto sumwlogr = [&](int k) { return __ldcg(SC + 3 * nb + k); };
    auto sumwwr = [&](int k) { return __ldcg(SC + 5 * nb + k); };
    auto sumwwlogr = [&](int k) { return __ldcg(SC + 6 * nb + k); };
    const double w1 = P.w[c1];
    const double n1 = P.n[c1];
    const int rows = mk - ks;
    for (int t = threadIdx.x; t < rows * nb; t += MB) {
        const int k2 = ks + t / nb, k3 = t % nb;
        if (k3 < k2) continue;
        const int i23 = (k2 * nb + k3) * nn + M;
        if (k3 == k2) {
            out[14 * Z + i23] += n1 * npairs(k2) * (npairs(k2) - 1);
            double md = w1 * (sumw(k2) * sumwr(k2) - sumwwr(k2));
            double ml = w1 * (sumw(k2) * sumwlogr(k2) - sumwwlogr(k2));
            out[8 * Z + i23] += md; out[9 * Z + i23] += ml;
            out[10 * Z + i23] += md; out[11 * Z + i23] += ml;
        } else {
            const int i32 = (k3 * nb + k2) * nn + M;
            double nnn = n1 * npairs(k2) * npairs(k3);
            out[14 * Z + i23] += nnn; out[14 * Z + i32] += nnn;
            double ww12 = w1 * sumw(k2), ww13 = w1 * sumw(k3);
            out[8 * Z + i23] += ww13 * sumwr(k2);  out[10 * Z + i32] += ww13 * sumwr(k2);
            out[9 * Z + i23] += ww13 * sumwlogr(k2); out[11 * Z + i32] += ww13 * sumwlogr(k2);
            out[10 * Z + i23] += ww12 * sumwr(k3); out[8 * Z + i32] += ww12 * sumwr(k3);
            out[11 * Z + i23] += ww12 * sumwlogr(k3); out[9 * Z + i32] += ww12 * sumwlogr(k3);
        }
    }
}

// The self-pair corrections of the diagonal entries k2 == k3 (the same for every n), rows
// [ks, mk): gam0 -= wg1 sumwwgg0, gam1 -= conj(wg1) sumwwgg1, gam2, gam3 -= wg1 sumwwgg2,
// weight -= w1 sumww.  Stored positive in the block's diag array and subtracted at the end.
__device__ void zeta_diag(const MPParams& P, int c1, const double* S, int ks, int mk,
                          double* diag)
{
    const int nb = P.nbins, M = P.maxn, gst = 2 * M + 3;
    const double* GG = S + 2 * (size_t)nb * (M + 1) + 2 * (size_t)nb * gst;
    const double* sumww = GG + 6 * (size_t)nb + 4 * (size_t)nb;
    const double w1 = P.w[c1];
    const C2 wg1 = {(double)P.d1[c1], (double)P.d2[c1]};
    for (int a = ks + threadIdx.x; a < mk; a += MB) {
        const C2 t0 = cmul(wg1, {__ldcg(GG + 2 * a), __ldcg(GG + 2 * a + 1)});
        const C2 t1 = cmul(conj2(wg1), {__ldcg(GG + 2 * nb + 2 * a), __ldcg(GG + 2 * nb + 2 * a + 1)});
        const C2 t2 = cmul(wg1, {__ldcg(GG + 4 * nb + 2 * a), __ldcg(GG + 4 * nb + 2 * a + 1)});
        diag[0 * nb + a] += t0.re; diag[1 * nb + a] += t0.im;
        diag[2 * nb + a] += t1.re; diag[3 * nb + a] += t1.im;
        diag[4 * nb + a] += t2.re; diag[5 * nb + a] += t2.im;
        diag[6 * nb + a] += t2.re; diag[7 * nb + a] += t2.im;
        diag[8 * nb + a] += w1 * __ldcg(sumww + a);
    }
}

// The product terms of calculateZeta for the entries (a, b, n) with min(a, b) in [ks, mk),
// in FP64 directly into the block's outputs: the path for a vertex record that does not fit
// the record buffer.
__device__ void zeta_products(const MPParams& P, int c1, const double* S, int ks, int mk,
                              double* out, double* shG, double* shW)
{
    const int nb = P.nbins, M = P.maxn, nn = 2 * M + 1;
    const int gst = 2 * M + 3;
    const size_t Z = (size_t)nb * nb * nn;
    const double* W = S;
    const double* G = S + 2 * (size_t)nb * (M + 1);
    for (int q = threadIdx.x; q < 2 * nb * gst; q += MB) shG[q] = __ldcg(G + q);
    for (int q = threadIdx.x; q < 2 * nb * (M + 1); q += MB) shW[q] = __ldcg(W + q);
    __syncthreads();
    const double w1 = P.w[c1];
    const C2 wg1 = {(double)P.d1[c1], (double)P.d2[c1]};
    const C2 wg1c = conj2(wg1);
    auto Gv = [&](int k, int n) -> C2 {
        const double* p = shG + sG(nb, M, n, k);
        return {p[0], p[1]};
    };
    auto Wv = [&](int k, int n) -> C2 {
        const double* p = shW + sW(nb, n >= 0 ? n : -n, k);
        return n >= 0 ? C2{p[0], p[1]} : C2{p[0], -p[1]};
    };
    const int na = mk - ks;
    const long long cnt = (long long)na * nb * 2 * nn;   // pairs (a in rows, b >= a) and mirror
    for (long long t = threadIdx.x; t < cnt; t += MB) {
        const int n = (int)(t % nn) - M;
        long long rest = t / nn;
        const int mirror = (int)(rest % 2);
        rest /= 2;
        const int bb = (int)(rest % nb);
        const int aa = ks + (int)(rest / nb);
        if (bb < aa) continue;                     // (aa, bb) with bb >= aa; the mirror swaps
        if (bb == aa && mirror) continue;
        const int a = mirror ? bb : aa, b = mirror ? aa : bb;
        const size_t i = (size_t)(a * nb + b) * nn + M + n;
        // weight (Porth et al. eq. 27)
        if (a == b) {
            C2 wv = Wv(a, n);
            out[12 * Z + i] += w1 * (wv.re * wv.re + wv.im * wv.im);
        } else {
            C2 p = cmul(Wv(a, n), conj2(Wv(b, n)));
            out[12 * Z + i] += w1 * p.re;
            out[13 * Z + i] += w1 * p.im;
        }
        // gam0..3 (eqs. 21, 23-25)
        C2 g0 = cmul(cmul(wg1, Gv(a, n - 1)), Gv(b, -n - 1));
        C2 g1 = cmul(cmul(wg1c, Gv(a, n + 1)), Gv(b, -n + 1));
        C2 g2 = cmul(cmul(wg1, Gv(a, n - 1)), conj2(Gv(b, n + 1)));
        C2 g3 = cmul(cmul(wg1, conj2(Gv(a, -n + 1))), Gv(b, -n - 1));
        out[0 * Z + i] += g0.re; out[1 * Z + i] += g0.im;
        out[2 * Z + i] += g1.re; out[3 * Z + i] += g1.im;
        out[4 * Z + i] += g2.re; out[5 * Z + i] += g2.im;
        out[6 * Z + i] += g3.re; out[7 * Z + i] += g3.im;
    }
    __syncthreads();
}

// The in-place path of a three-field cross (Corr3::calculateZeta with mp2, mp3,
// src/Corr3.cpp:1976-2087): every entry (a, b) of the scratch's 2 nbd x 2 nbd bins whose
// row and column belong to different vertices and whose min(a mod nbd, b mod nbd) is in
// [ks, mk), with the auto-correlation's off-diagonal formulas; the caller keeps the
// vertex-3 x vertex-2 block (and, for ordered = 1, adds the other).
__device__ void zeta_inplace3(const MPParams& P, int c1, const double* S, int ks, int mk,
                              double* out, double* shG, double* shW)
{
    const int nb = P.nbins, nbd = P.nbd, M = P.maxn, nn = 2 * M + 1;
    const int gst = 2 * M + 3;
    const size_t Z = (size_t)nb * nb * nn;
    const double* W = S;
    const double* G = S + 2 * (size_t)nb * (M + 1);
    const double* SC = G + 2 * (size_t)nb * gst + 6 * (size_t)nb;
    for (int q = threadIdx.x; q < 2 * nb * gst; q += MB) shG[q] = __ldcg(G + q);
    for (int q = threadIdx.x; q < 2 * nb * (M + 1); q += MB) shW[q] = __ldcg(W + q);
    __syncthreads();
    const double w1 = P.w[c1];
    const double n1 = P.n[c1];
    const C2 wg1 = {(double)P.d1[c1], (double)P.d2[c1]};
    const C2 wg1c = conj2(wg1);
    const int sh = P.vreal ? 0 : 1;
    auto Gv = [&](int k, int n) -> C2 {
        const double* p = shG + sG(nb, M, n, k);
        return {p[0], p[1]};
    };
    auto Wv = [&](int k, int n) -> C2 {
        const double* p = shW + sW(nb, n >= 0 ? n : -n, k);
        return n >= 0 ? C2{p[0], p[1]} : C2{p[0], -p[1]};
    };
    const long long cnt = (long long)nb * nb * nn;
    for (long long t = threadIdx.x; t < cnt; t += MB) {
        const int n = (int)(t % nn) - M;
        const int b = (int)((t / nn) % nb), a = (int)(t / nn / nb);
        if ((a >= nbd) == (b >= nbd)) continue;
        const int m = min(a % nbd, b % nbd);
        if (m < ks || m >= mk) continue;
        const size_t i = (size_t)(a * nb + b) * nn + M + n;
        const C2 p = cmul(Wv(a, n), conj2(Wv(b, n)));
        out[12 * Z + i] += w1 * p.re;
        out[13 * Z + i] += w1 * p.im;
        const C2 g0 = cmul(cmul(wg1, Gv(a, n - sh)), Gv(b, -n - sh));
        const C2 g1 = cmul(cmul(wg1c, Gv(a, n + sh)), Gv(b, -n + sh));
        const C2 g2 = cmul(cmul(wg1, Gv(a, n - sh)), conj2(Gv(b, n + sh)));
        const C2 g3 = cmul(cmul(wg1, conj2(Gv(a, -n + sh))), Gv(b, -n - sh));
        out[0 * Z + i] += g0.re; out[1 * Z + i] += g0.im;
        out[2 * Z + i] += g1.re; out[3 * Z + i] += g1.im;
        out[4 * Z + i] += g2.re; out[5 * Z + i] += g2.im;
        out[6 * Z + i] += g3.re; out[7 * Z + i] += g3.im;
        if (n == 0 && !P.quick) {
            const size_t i0 = (size_t)(a * nb + b) * nn + M;
            const double npa = __ldcg(SC + a), npb = __ldcg(SC + b);
            const double swa = __ldcg(SC + nb + a), swb = __ldcg(SC + nb + b);
            const double sra = __ldcg(SC + 2 * nb + a), srb = __ldcg(SC + 2 * nb + b);
            const double sla = __ldcg(SC + 3 * nb + a), slb = __ldcg(SC + 3 * nb + b);
            // meanlogd3 of the vertex-3 x vertex-2 block for ordered = 1 as the reference
            // writes it: mp3.sumw at the column's bin.
            const double swl = (P.typo32 && a >= nbd) ? __ldcg(SC + nb + (b % nbd) + nbd) : swa;
            out[14 * Z + i0] += n1 * npa * npb;
            out[8 * Z + i0] += w1 * swb * sra;
            out[9 * Z + i0] += w1 * swb * sla;
            out[10 * Z + i0] += w1 * swa * srb;
            out[11 * Z + i0] += w1 * swl * slb;
        }
    }
    __syncthreads();
}

// calculateZeta for vertex c1, rows [ks, mk): the diagonal self-pair corrections now, the
// rest as one vertex record for the batched contraction kernels (k_mp_zeta, k_mp_zscal).
// Record (floats): header (c1, ks, mk, w1, Re/Im wg1, n1, pad), then G_n [n = -(M+1) ..
// M+1][bin] and W_n [n = 0 .. M][bin] complex, then npairs (int), sumw, sumwr, sumwlogr,
// sumwwr, sumwwlogr [bin].  A record that does not fit the buffer is contracted in place.
__device__ void zeta_emit(const MPParams& P, int c1, const double* S, int ks, int mk,
                          double* out, double* diag, double* shG, double* shW,
                          unsigned long long* zidx_sh, int* emits_sh)
{
    const int nb = P.nbins, M = P.maxn, gst = 2 * M + 3;
    // (a three-field cross has no self-pair corrections: getMP2 / getMP3 without ww)
    if (!P.three) zeta_diag(P, c1, S, ks, mk, diag);
    if (threadIdx.x == 0) {
        *zidx_sh = atomicAdd(P.zcount, 1ull);
        ++*emits_sh;
    }
    __syncthreads();
    const unsigned long long zi = *zidx_sh;
    if ((long long)zi < P.zcap) {
        float* R = P.zrec + (size_t)zi * P.zrec_floats;
        if (threadIdx.x == 0) {
            R[0] = __int_as_float(c1); R[1] = __int_as_float(ks); R[2] = __int_as_float(mk);
            R[3] = P.w[c1]; R[4] = P.d1[c1]; R[5] = P.d2[c1];
            R[6] = __int_as_float(P.n[c1]); R[7] = 0.f;
        }
        // G then W: the slot's first 2 nb (M+1) + 2 nb gst doubles, reordered G-first.
        const double* W = S;
        const double* G = S + 2 * (size_t)nb * (M + 1);
        float* RG = R + 8;
        float* RW = RG + 2 * (size_t)gst * nb;
        for (int q = threadIdx.x; q < 2 * gst * nb; q += MB) RG[q] = (float)__ldcg(G + q);
        for (int q = threadIdx.x; q < 2 * (M + 1) * nb; q += MB) RW[q] = (float)__ldcg(W + q);
        const double* SC = G + 2 * (size_t)nb * gst + 6 * (size_t)nb;
        float* RS = RW + 2 * (size_t)(M + 1) * nb;
        for (int q = threadIdx.x; q < nb; q += MB) {
            RS[q] = __int_as_float((int)__ldcg(SC + q));                // npairs
            RS[nb + q] = (float)__ldcg(SC + nb + q);                    // sumw
            RS[2 * nb + q] = (float)__ldcg(SC + 2 * nb + q);            // sumwr
            RS[3 * nb + q] = (float)__ldcg(SC + 3 * nb + q);            // sumwlogr
            RS[4 * nb + q] = (float)__ldcg(SC + 5 * nb + q);            // sumwwr
            RS[5 * nb + q] = (float)__ldcg(SC + 6 * nb + q);            // sumwwlogr
        }
    } else if (P.three) {
        zeta_inplace3(P, c1, S, ks, mk, out, shG, shW);
    } else {
        if (!P.quick) zeta_scalars(P, c1, S, ks, mk, out);
        zeta_products(P, c1, S, ks, mk, out, shG, shW);
    }
    __syncthreads();
}

// THREE: a three-field cross (two pair lists); compiled apart so that the auto and cross12
// paths carry none of its registers.
template <bool THREE>
__global__ void __launch_bounds__(MB, 2) k_mp_finish(MPParams P)
{
    extern __shared__ __align__(16) double mp_sh[];
    __shared__ P2Entry stk[MSTACK];
    __shared__ int sp, free_cnt, free_list[64], scan_sh[MW];
    __shared__ P2Entry cur;
    __shared__ unsigned long long job_sh, zidx_sh;
    __shared__ int acc_n, new_n, anysplit, alloc_ok, have_sh, job_emits;
    __shared__ double maxr_sh[MW], maxr3_sh[MW];
    __shared__ long long arena_top;
    __shared__ int bh[MP_MAXNB];
    __shared__ int bw[MW][MP_MAXNB];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int blk = blockIdx.x;
    const int nb = P.nbins, M = P.maxn;
    const int gst = 2 * M + 3;
    double* shG = mp_sh;
    double* shW = mp_sh + 2 * (size_t)nb * gst;
    int* arena = P.arena2 + (size_t)blk * P.arena2_cap;
    float* acc = P.acc + (size_t)blk * P.acc_cap * MP_REC;
    int* perm = P.perm + (size_t)blk * P.acc_cap;
    double* out = P.out + (size_t)blk * P.out_stride;
    double* diag = P.diag + (size_t)blk * 9 * nb;
    const int* arena1 = P.arena1;
    for (int k = tid; k < MP_MAXNB; k += MB) bh[k] = 0;

    while (true) {
        if (tid == 0) {
            // After an error the results are discarded and the call is retried: stop early.
            // With the vertex-record buffer nearly full, stop taking jobs until it is drained.
            if (*(volatile int*)P.err ||
                (long long)*(volatile unsigned long long*)P.zcount >= P.zstop)
                job_sh = (unsigned long long)P.njobs_val;
            else
                job_sh = atomicAdd(P.job_next, 1ull);
        }
        __syncthreads();
        const unsigned long long job = job_sh;
        if ((long long)job >= P.njobs_val) break;
        const int4 J = P.jobs[job];
        if (!mp_valid_cell(P, J.x) || J.y < 0 || J.y >= P.ntop || J.z < 0 || J.w < 0 ||
            (long long)J.z + J.w > P.arena1_cap) {
            if (tid == 0) mp_check_fail(P.err, 3);
            break;
        }
        if (tid == 0) {
            free_cnt = P.nslots;
            for (int s = 0; s < P.nslots; ++s) free_list[s] = P.nslots - 1 - s;
            arena_top = 0;
            sp = 0;
            job_emits = 0;
            int s0 = free_list[--free_cnt];
            P2Entry e;
            e.c1 = J.x; e.len = J.w; e.slot = s0; e.mink = P.nbd;
            e.goff = (long long)J.y * P.arena1_cap + J.z; e.maxr = 0.; e.maxr3 = 0.;
            e.mark = 0;
            stk[sp++] = e;
        }
        __syncthreads();
        int guard = 0, stall = 0, stall_c1 = -1;
        {
            double* S0 = slot_ptr(P, blk, stk[0].slot);
            for (int q = tid; q < P.slot_doubles; q += MB) S0[q] = 0.;
        }
        __syncthreads();
        while (true) {
            // Thread 0 pops (see k_mp_split1 for why the outcome goes through a flag).
            __syncthreads();
            if (tid == 0) {
                have_sh = sp > 0;
                if (have_sh) {
                    cur = stk[--sp];
                    arena_top = cur.mark;   // the finished left subtree's lists are dead
                }
            }
            __syncthreads();
            if (!have_sh) break;
            // multipoleFinish loop on cur (c1 changes to its left child, the list to the new
            // list, the slot stays).
            while (true) {
                if (++guard > (1 << 24)) {   // last-resort bound; the recursion is finite
                    if (tid == 0) mp_check_fail(P.err, 6);
                    break;
                }
                // Passes at one c1 refine its c2 list; their number is bounded by the depth
                // of the c2 trees.
                if (cur.c1 != stall_c1) { stall_c1 = cur.c1; stall = 0; }
                if (++stall > 4096) {
                    if (tid == 0 && atomicCAS(P.err + 1, 0, 7) == 0) {
                        atomicCAS(P.err, 0, MP_ERR_CHECK);
                        const int* l = (cur.goff >= 0) ? (arena1 + cur.goff) : (arena + (-cur.goff - 1));
                        double* d = P.dbg;
                        d[0] = cur.c1; d[1] = cur.len; d[2] = cur.maxr; d[3] = P.size[cur.c1];
                        d[4] = P.left[cur.c1]; d[5] = cur.goff; d[6] = arena_top; d[7] = sp;
                        d[8] = blk; d[9] = cur.mink;
                        for (int q = 0; q < 8 && q < cur.len; ++q) {
                            d[10 + 2 * q] = l[q];
                            d[11 + 2 * q] = sqrt(mp_dist_sq(P, cur.c1, l[q])) + P.size[l[q]];
                        }
                    }
                    break;
                }
                const int c1 = cur.c1;
                const double s1 = P.size[c1];
                // oneBinLessThan of each list's previous maximum
                const double thresh1_2 = (1. - P.binsize) * cur.maxr;
                const double thresh1_3 = (1. - P.binsize) * cur.maxr3;
                const int* list = (cur.goff >= 0) ? (arena1 + cur.goff) : nullptr;
                const int* list2 = (cur.goff < 0) ? (arena + (-cur.goff - 1)) : nullptr;
                const long long nbase = arena_top;
                double* S = slot_ptr(P, blk, cur.slot);
                if (tid == 0) { acc_n = 0; new_n = 0; anysplit = 0; }
                double mymax = 0., mymax3 = 0.;
                float run32 = 0.f, run32_3 = 0.f;
                int myany = 0;
                const float4 c1a = __ldg(reinterpret_cast<const float4*>(P.tc + c1));
                const float4 c1b = __ldg(reinterpret_cast<const float4*>(P.tc + c1) + 1);
                const float s1f = c1a.w;
                const float thresh1f_2 = (float)thresh1_2, thresh1f_3 = (float)thresh1_3;
                __syncthreads();
                for (int j0 = 0; j0 < cur.len; j0 += MB) {
                    const int j = j0 + tid;
                    int cnt = 0, ca = -1, cb = -1, acc_ok = 0, kacc = -1;
                    double racc = 0., lracc = 0.;
                    const int c2 = j < cur.len ? __ldcg(list ? list + j : list2 + j) : 0;
                    // A vertex-3 cell of a three-field cross: its own threshold, maximum and
                    // bins [nbd, 2 nbd).
                    const bool is3 = THREE && c2 >= P.base3;
                    const double thresh1 = is3 ? thresh1_3 : thresh1_2;
                    const float thresh1f = is3 ? thresh1f_3 : thresh1f_2;
                    bool dec32 = false;          // decided (and recorded) in FP32
                    float rs32 = 0.f;            // r + s of an FP32-decided unaccepted entry
                    float r32 = 0.f, lr32 = 0.f, dxf = 0.f, dyf = 0.f;
                    float4 ta, tb, tq, td;       // the packed cell c2
                    const bool inlist = j < cur.len && c2 >= 0 && c2 < P.ncells;
                    if (inlist) {
                        const float4* t4 = reinterpret_cast<const float4*>(P.tc + c2);
                        ta = __ldg(t4); tb = __ldg(t4 + 1); tq = __ldg(t4 + 2); td = __ldg(t4 + 3);
                    }
                    const bool valid = inlist && __float_as_int(tq.z) > 0;
                    if (j < cur.len && !valid) mp_check_fail(P.err, 2);
                    else if (j < cur.len) {
                        // Geometry from the hi/lo float positions, decisions in FP32.
                        const float s2f = ta.w;
                        dxf = (ta.x - c1a.x) + (tb.x - c1b.x);
                        dyf = (ta.y - c1a.y) + (tb.y - c1b.y);
                        float dsq = dxf * dxf + dyf * dyf;
                        if (P.coords != FLAT) {
                            const float dzf = (ta.z - c1a.z) + (tb.z - c1b.z);
                            dsq += dzf * dzf;
                        }
                        float rsqf = dsq;
                        if (P.metric == ARC) {
                            const float th = arc_from_chord_sq(dsq);
                            rsqf = th * th;
                        }
                        int k32 = -1;
                        bool sp1 = false, sp2 = false, any32 = false;
                        const int kind = mp_decide32(P, rsqf, s1f, s2f, thresh1f, k32, r32, lr32,
                                                     sp1, sp2, any32);
                        if (kind >= 0) {
                            dec32 = true;
                            if (kind == 1) {
                                acc_ok = 1; kacc = k32; ca = c2;
                            } else if (kind == 2) {
                                rs32 = r32 + (s1f + s2f);
                                if (any32) myany = 1;
                                if (sp2) { ca = __float_as_int(tq.w); cb = __float_as_int(td.x); cnt = 2; }
                                else { ca = c2; cnt = 1; }
                            }
                        }
                    }
                    if (j < cur.len && !dec32 && valid) {
                        const double s2 = P.size[c2];
                        const double rsq = mp_dist_sq(P, c1, c2);
                        const double s = s1 + s2;
                        if (!mp_too_small(P, rsq, s) && !mp_too_large(P, rsq, s)) {
                            int k = -1;
                            double r = sqrt(rsq), lr = 0.;
                            if (mp_single_bin(P, rsq, s, k, r, lr)) {
                                if (rsq >= P.minsepsq && rsq < P.maxsepsq) {
                                    if (k < 0) {
                                        lr = log(r);
                                        k = int((lr - P.logminsep) / P.binsize);
                                    }
                                    if (k >= P.nbd) k = P.nbd - 1;
                                    acc_ok = 1; kacc = k; racc = r; lracc = lr;
                                    ca = c2;
                                }
                            } else {
                                if (is3) mymax3 = fmax(mymax3, r + s);
                                else mymax = fmax(mymax, r + s);
                                // CalcSplitSq (include/Split.h:82-101)
                                double bsq_eff = rsq * fmin(P.bsq, P.asq);
                                bool split1, split2;
                                if (s2 > s1) {
                                    split2 = true;
                                    split1 = !(s2 > 2. * s1) && (s1 * s1 > 0.3422 * bsq_eff);
                                } else {
                                    split1 = true;
                                    split2 = !(s1 > 2. * s2) && (s2 * s2 > 0.3422 * bsq_eff);
                                }
                                if (split1 && r + s > thresh1) myany = 1;
                                if (split2) { ca = P.left[c2]; cb = P.right[c2]; cnt = 2; }
                                else { ca = c2; cnt = 1; }
                            }
                        }
                    }
                    // The maximum of r + s over the unaccepted entries is kept exact (it sets
                    // the next pass's thresholds): the warp's FP32 maximum is compared with its
                    // running FP32 maximum, and the entries within the FP32 error of the larger
                    // one get their FP64 value; all other entries are below an evaluated one.
                    // (per list for a three-field cross)
                    for (int li = 0; li < (THREE ? 2 : 1); ++li) {
                        const float rsl = (li == 1) == is3 ? rs32 : 0.f;
                        float& runl = li ? run32_3 : run32;
                        float wm = rsl;
                        for (int o = 16; o > 0; o >>= 1) wm = fmaxf(wm, __shfl_xor_sync(0xffffffffu, wm, o));
                        if (wm > runl * (1.f - 8e-6f)) {
                            if (rsl > 0.f && rsl > wm * (1.f - 8e-6f)) {
                                const double rs64 = sqrt(mp_dist_sq(P, c1, c2)) + (s1 + (double)ta.w);
                                if (li) mymax3 = fmax(mymax3, rs64);
                                else mymax = fmax(mymax, rs64);
                            }
                            runl = fmaxf(runl, wm);
                        }
                    }
                    if (acc_ok && is3) kacc += P.nbd;
                    int tot_new, tot_acc;
                    int pos = block_excl_scan(cnt, scan_sh, tot_new);
                    int apos = block_excl_scan(acc_ok, scan_sh, tot_acc);
                    const long long wbase = nbase + new_n;
                    if (wbase + tot_new > P.arena2_cap || acc_n + tot_acc > P.acc_cap) {
                        if (tid == 0) set_mp_err(P.err, MP_ERR_ARENA);
                    } else {
                        if (cnt >= 1) arena[wbase + pos] = ca;
                        if (cnt == 2) arena[wbase + pos + 1] = cb;
                        if (acc_ok && dec32 && P.coords == FLAT) {
                            // calculateGn's per-pair terms in FP32: ExpIPhi z = d / r, the
                            // spin-2 factor e = conj(d^2) / |d|^2, the projected shear wg and
                            // the scalar sums.
                            const float rr = r32 > 0.f ? r32 : 1.f;
                            const float zr = dxf / rr, zi = dyf / rr;
                            float nn2 = dxf * dxf + dyf * dyf;
                            if (!(nn2 > 0.f)) nn2 = 1.f;
                            // (no rotation for the real payload of N / K pairs)
                            const bool rl = (P.pspin0 >> (is3 ? 1 : 0)) & 1;
                            const float er = rl ? 1.f : (dxf * dxf - dyf * dyf) / nn2;
                            const float ei = rl ? 0.f : -(2.f * dxf * dyf) / nn2;
                            const float w2 = tb.w;
                            const float4 lf = __ldg(P.lsf + ca);
                            const float l0 = lf.x, l1 = lf.y, l2 = lf.z, l3 = lf.w;
                            const float g1 = tq.x, g2 = tq.y;
                            const float wgr = g1 * er - g2 * ei, wgi = g1 * ei + g2 * er;
                            const float e2r = er * er - ei * ei, e2i = 2.f * er * ei;
                            const float wsr = l1 * e2r - l2 * e2i, wsi = l1 * e2i + l2 * e2r;
                            // z^2 in the self-pair sums of a spin-2 vertex; 1 for an N or K
                            // vertex (MultipoleScratch<GData>::calculateGn, buffer 0).
                            const float zsr = P.vreal ? 1.f : zr * zr - zi * zi;
                            const float zsi = P.vreal ? 0.f : 2.f * zr * zi;
                            const float a0r = wsr * zsr + wsi * zsi, a0i = wsi * zsr - wsr * zsi;
                            const float a1r = wsr * zsr - wsi * zsi, a1i = wsr * zsi + wsi * zsr;
                            float* R = acc + (size_t)(acc_n + apos) * MP_REC;
                            *reinterpret_cast<float4*>(R) = make_float4(zr, zi, wgr, wgi);
                            *reinterpret_cast<float4*>(R + 4) =
                                make_float4(w2, tq.z, __int_as_float(kacc), 0.f);
                            *reinterpret_cast<float4*>(R + 8) = make_float4(w2, w2 * r32, w2 * lr32, l0);
                            *reinterpret_cast<float4*>(R + 12) = make_float4(l0 * r32, l0 * lr32, a0r, a0i);
                            *reinterpret_cast<float4*>(R + 16) = make_float4(a1r, a1i, l3 * zsr, -l3 * zsi);
                            *reinterpret_cast<float4*>(R + 20) = make_float4(wgr, wgi, 0.f, 0.f);
                            atomicAdd(&bh[kacc], 1);
                        } else if (acc_ok) {
                            // The same terms from FP64 (non-flat geometry, or decided in FP64).
                            if (dec32) { racc = r32; lracc = lr32; }
                            C2 z, e;
                            phases(P, c1, ca, racc, z, e);
                            if ((P.pspin0 >> (is3 ? 1 : 0)) & 1) e = C2{1., 0.};
                            const double w2 = P.w[ca];
                            const double* ls = P.ls + 4 * (size_t)ca;
                            const C2 wg = cmul({(double)P.d1[ca], (double)P.d2[ca]}, e);
                            const C2 wgsq = cmul({ls[1], ls[2]}, cmul(e, e));
                            const C2 zsq = P.vreal ? C2{1., 0.} : cmul(z, z);
                            const C2 a0 = cmul(wgsq, conj2(zsq)), a1 = cmul(wgsq, zsq);
                            float* R = acc + (size_t)(acc_n + apos) * MP_REC;
                            *reinterpret_cast<float4*>(R) =
                                make_float4((float)z.re, (float)z.im, (float)wg.re, (float)wg.im);
                            *reinterpret_cast<float4*>(R + 4) =
                                make_float4((float)w2, __int_as_float(P.n[ca]), __int_as_float(kacc), 0.f);
                            *reinterpret_cast<float4*>(R + 8) =
                                make_float4((float)w2, (float)(w2 * racc), (float)(w2 * lracc), (float)ls[0]);
                            *reinterpret_cast<float4*>(R + 12) =
                                make_float4((float)(ls[0] * racc), (float)(ls[0] * lracc), (float)a0.re, (float)a0.im);
                            *reinterpret_cast<float4*>(R + 16) =
                                make_float4((float)a1.re, (float)a1.im, (float)(ls[3] * zsq.re), (float)(-ls[3] * zsq.im));
                            *reinterpret_cast<float4*>(R + 20) =
                                make_float4((float)wg.re, (float)wg.im, 0.f, 0.f);
                            atomicAdd(&bh[kacc], 1);
                        }
                    }
                    __syncthreads();
                    if (tid == 0) { new_n += tot_new; acc_n += tot_acc; }
                    __syncthreads();
                    if (acc_n > P.acc_cap - MB) {      // record buffer full: accumulate now
                        mp_accumulate(P, acc, perm, acc_n, S, bh, bw);
                        if (tid == 0) acc_n = 0;
                        __syncthreads();
                    }
                }
                // An overflow of the arenas leaves the lists incomplete: stop this job (the
                // call is retried with larger arenas).
                if (tid == 0) alloc_ok = (*(volatile int*)P.err) ? 0 : 1;
                __syncthreads();
                if (!alloc_ok) break;
                if (acc_n > 0) mp_accumulate(P, acc, perm, acc_n, S, bh, bw);
                // Block max of the remaining separations and OR of anysplit1.
                for (int o = 16; o > 0; o >>= 1) {
                    mymax = fmax(mymax, __shfl_xor_sync(0xffffffffu, mymax, o));
                    mymax3 = fmax(mymax3, __shfl_xor_sync(0xffffffffu, mymax3, o));
                    myany |= __shfl_xor_sync(0xffffffffu, myany, o);
                }
                if (lane == 0) {
                    maxr_sh[wid] = mymax; maxr3_sh[wid] = mymax3;
                    if (myany) atomicOr(&anysplit, 1);
                }
                __syncthreads();
                double maxrem2 = 0., maxrem3 = 0.;
                for (int k = 0; k < MW; ++k) {
                    maxrem2 = fmax(maxrem2, maxr_sh[k]);
                    maxrem3 = fmax(maxrem3, maxr3_sh[k]);
                }
                const double maxrem = fmax(maxrem2, maxrem3);
                const int n_new = new_n;
                int mink = cur.mink;
                if (n_new == 0) {
                    zeta_emit(P, c1, S, 0, mink, out, diag, shG, shW, &zidx_sh, &job_emits);
                    break;
                }
                if (maxrem < P.maxsep) {
                    int k = 0;
                    if (lane == 0 && !(maxrem < P.minsep))
                        k = int((log(maxrem) - P.logminsep) / P.binsize) + 1;
                    k = __shfl_sync(0xffffffffu, k, 0);
                    if (k < mink) {
                        zeta_emit(P, c1, S, k, mink, out, diag, shG, shW, &zidx_sh, &job_emits);
                        mink = k;
                    }
                }
                const bool split1 = anysplit && P.left[c1] >= 0;
                __syncthreads();
                if (tid == 0) {
                    arena_top = nbase + n_new;
                    alloc_ok = 1;
                    if (split1) {
                        if (free_cnt == 0 || sp + 1 > MSTACK) {
                            set_mp_err(P.err, MP_ERR_SLOTS);
                            alloc_ok = 0;
                        } else {
                            P2Entry rgt;
                            rgt.c1 = P.right[c1]; rgt.len = n_new; rgt.slot = free_list[--free_cnt];
                            rgt.mink = mink; rgt.goff = -nbase - 1;
                            rgt.maxr = maxrem2; rgt.maxr3 = maxrem3;
                            rgt.mark = nbase + n_new;
                            stk[sp++] = rgt;
                        }
                    }
                }
                __syncthreads();
                if (!alloc_ok) break;
                if (split1) {
                    // The right child gets a copy of the scratch (mp.duplicate()).
                    const double* src = S;
                    double* dst = slot_ptr(P, blk, stk[sp - 1].slot);
                    for (int q = tid; q < P.slot_doubles; q += MB) dst[q] = __ldcg(src + q);
                }
                __syncthreads();
                // Without a split, the old list is dead unless a pushed entry still uses it:
                // move the new list down onto it, so a chain of passes reuses one region.
                long long newoff = nbase;
                const bool old_in2 = cur.goff < 0;
                const long long oo = old_in2 ? (-cur.goff - 1) : 0;
                const bool old_used = (sp > 0 && stk[sp - 1].goff == cur.goff);
                if (!split1 && old_in2 && !old_used && oo < nbase) {
                    for (long long i0 = 0; i0 < n_new; i0 += MB) {
                        const long long i = i0 + tid;
                        int v = 0;
                        if (i < n_new) v = __ldcg(arena + nbase + i);
                        __syncthreads();
                        if (i < n_new) arena[oo + i] = v;
                        __syncthreads();
                    }
                    newoff = oo;
                }
                __syncthreads();
                if (tid == 0) {
                    if (split1) cur.c1 = P.left[c1];
                    cur.len = n_new;
                    cur.goff = -newoff - 1;
                    cur.mink = mink;
                    cur.maxr = maxrem2;
                    cur.maxr3 = maxrem3;
                    arena_top = newoff + n_new;
                }
                __syncthreads();
            }
            __syncthreads();
            if (tid == 0) free_list[free_cnt++] = cur.slot;
            __syncthreads();
        }
        // The largest record count of one job sizes the stop margin of later waves.
        if (tid == 0) atomicMax(P.zmaxjob, (unsigned long long)job_emits);
    }
}

// ---------------------------------------------------------------------------------------
// Batched Zeta contraction over vertex records.  For one n and a group of records the
// block computes, for every entry (a, b) of the nbins x nbins tile,
//   gam0 += (wg1 G_a[n-1]) G_b[-n-1]        gam1 += (conj(wg1) G_a[n+1]) G_b[-n+1]
//   gam2 += (wg1 G_a[n-1]) conj(G_b[n+1])   gam3 += (wg1 conj(G_a[-n+1])) G_b[-n-1]
//   weight += (w1 W_a[n]) conj(W_b[n])
// over the records whose row range [ks, mk) holds min(a, b) -- a sum of outer products over
// vertices.  Operands are staged in shared memory per chunk of records; products and chunk
// sums are FP32, the running sums FP64; each group adds its sums to its own partial array.
// These are GGG's sums (MultipoleHelper<5>).  With shift 0 the G indices are n and -n and
// wg1 is the real w1 or w1 k1 of an N or K vertex, which makes gam0 and gam2 NGG's / KGG's
// zeta0 and zeta1 (MultipoleHelper<2>, src/Corr3.cpp:2216-2405).

struct ZParams {
    const float* rec;
    long long nrec;
    int rec_floats, nbins, maxn, chunk, ngroups;
    int shift;             // 1: G_n at n -+ 1 (a spin-2 vertex); 0: at n (an N or K vertex)
    int nbd;               // distance bins; a record's rows [ks, mk) hold min(a, b) mod nbd
    int typo32;            // see MPParams::typo32
    double* part;          // [group][10][Z]
    long long Z;
};

static constexpr int ZB = 256;   // threads per contraction block
static constexpr int ZE = 2;     // entries per thread

__global__ void __launch_bounds__(ZB) k_mp_zeta(ZParams Q)
{
    extern __shared__ float4 zsh[];    // [chunk][nb][4]: (A0, A1), (A3, AW), (B0, B1), (B2, BW)
    __shared__ int2 rows_sh[64];
    const int nb = Q.nbins, M = Q.maxn, nn = 2 * M + 1, gst = 2 * M + 3;
    const int n = (int)blockIdx.x - M;
    const int g = blockIdx.y;
    const int tid = threadIdx.x;
    int ea[ZE], eb[ZE], em[ZE];     // entry (a, b) and min(a, b) mod nbd (the row mask)
    bool ev[ZE];
#pragma unroll
    for (int j = 0; j < ZE; ++j) {
        const int e = ((int)blockIdx.z * ZE + j) * ZB + tid;
        ev[j] = e < nb * nb;
        ea[j] = ev[j] ? e / nb : 0;
        eb[j] = ev[j] ? e % nb : 0;
        em[j] = min(ea[j] % Q.nbd, eb[j] % Q.nbd);
    }
    // Sums: FP32 per chunk (F), FP32 over up to 16 chunks (F2), then FP64 (D) -- FP64 work is
    // kept rare (GB300 runs FP64 at 1/64 of the FP32 rate).
    double D[ZE][10];
    float F2[ZE][10];
#pragma unroll
    for (int j = 0; j < ZE; ++j)
#pragma unroll
        for (int q = 0; q < 10; ++q) { D[j][q] = 0.; F2[j][q] = 0.f; }
    int nchunk = 0;
    const long long r0 = Q.nrec * g / Q.ngroups, r1 = Q.nrec * (g + 1) / Q.ngroups;
    const int nw = (n >= 0) ? n : -n;
    for (long long c0 = r0; c0 < r1; c0 += Q.chunk) {
        const int nv = (int)min((long long)Q.chunk, r1 - c0);
        __syncthreads();
        for (int idx = tid; idx < nv * nb; idx += ZB) {
            const int v = idx / nb, a = idx % nb;
            const float* R = Q.rec + (size_t)(c0 + v) * Q.rec_floats;
            const float2* RG = reinterpret_cast<const float2*>(R + 8);
            const float2* RW = RG + (size_t)gst * nb;
            const float w1 = R[3], wr = R[4], wi = R[5];
            const int sh = Q.shift;
            const float2 gm1 = RG[(n - sh + M + 1) * nb + a];     // G[n-1]
            const float2 gmm1 = RG[(-n - sh + M + 1) * nb + a];   // G[-n-1]
            const float2 gp1 = RG[(n + sh + M + 1) * nb + a];     // G[n+1]
            const float2 gmp1 = RG[(-n + sh + M + 1) * nb + a];   // G[-n+1]
            float2 w = RW[nw * nb + a];
            if (n < 0) w.y = -w.y;
            float4 o0, o1, o2, o3;
            o0.x = wr * gm1.x - wi * gm1.y;  o0.y = wr * gm1.y + wi * gm1.x;     // A0
            o0.z = wr * gp1.x + wi * gp1.y;  o0.w = wr * gp1.y - wi * gp1.x;     // A1
            o1.x = wr * gmp1.x + wi * gmp1.y; o1.y = wi * gmp1.x - wr * gmp1.y;  // A3
            o1.z = w1 * w.x;                 o1.w = w1 * w.y;                    // AW
            o2 = make_float4(gmm1.x, gmm1.y, gmp1.x, gmp1.y);                   // B0, B1
            o3 = make_float4(gp1.x, -gp1.y, w.x, -w.y);                         // B2, BW
            float4* d = zsh + ((size_t)v * nb + a) * 4;
            d[0] = o0; d[1] = o1; d[2] = o2; d[3] = o3;
            if (a == 0) rows_sh[v] = make_int2(__float_as_int(R[1]), __float_as_int(R[2]));
        }
        __syncthreads();
        float F[ZE][10];
#pragma unroll
        for (int j = 0; j < ZE; ++j)
#pragma unroll
            for (int q = 0; q < 10; ++q) F[j][q] = 0.f;
        for (int v = 0; v < nv; ++v) {
            const int2 rw = rows_sh[v];
#pragma unroll
            for (int j = 0; j < ZE; ++j) {
                const int m = em[j];
                if (!ev[j] || m < rw.x || m >= rw.y) continue;
                const float4* pa = zsh + ((size_t)v * nb + ea[j]) * 4;
                const float4* pb = zsh + ((size_t)v * nb + eb[j]) * 4;
                const float4 a01 = pa[0], a3w = pa[1], b01 = pb[2], b2w = pb[3];
                F[j][0] += a01.x * b01.x - a01.y * b01.y;  F[j][1] += a01.x * b01.y + a01.y * b01.x;
                F[j][2] += a01.z * b01.z - a01.w * b01.w;  F[j][3] += a01.z * b01.w + a01.w * b01.z;
                F[j][4] += a01.x * b2w.x - a01.y * b2w.y;  F[j][5] += a01.x * b2w.y + a01.y * b2w.x;
                F[j][6] += a3w.x * b01.x - a3w.y * b01.y;  F[j][7] += a3w.x * b01.y + a3w.y * b01.x;
                F[j][8] += a3w.z * b2w.z - a3w.w * b2w.w;  F[j][9] += a3w.z * b2w.w + a3w.w * b2w.z;
            }
        }
#pragma unroll
        for (int j = 0; j < ZE; ++j)
#pragma unroll
            for (int q = 0; q < 10; ++q) F2[j][q] += F[j][q];
        if (++nchunk == 16) {
            nchunk = 0;
#pragma unroll
            for (int j = 0; j < ZE; ++j)
#pragma unroll
                for (int q = 0; q < 10; ++q) { D[j][q] += (double)F2[j][q]; F2[j][q] = 0.f; }
        }
    }
#pragma unroll
    for (int j = 0; j < ZE; ++j)
#pragma unroll
        for (int q = 0; q < 10; ++q) D[j][q] += (double)F2[j][q];
#pragma unroll
    for (int j = 0; j < ZE; ++j) {
        if (!ev[j]) continue;
        const size_t i = (size_t)(ea[j] * nb + eb[j]) * nn + M + n;
        double* p = Q.part + (size_t)g * 10 * Q.Z + i;
        if (ea[j] == eb[j]) D[j][9] = 0.;   // W_a conj(W_a) is real
#pragma unroll
        for (int q = 0; q < 10; ++q) p[(size_t)q * Q.Z] += D[j][q];
    }
}

// Tensor-core contraction (tcgen05, nbins <= 32).  Same sums as k_mp_zeta, as two real
// GEMMs per n over the vertex records (the K dimension):
//   region 0: rows [Re A0, Im A0, Re A3, Im A3] x cols [Re B0, Im B0, Re B2, Im B2]
//   region 1: rows [Re A1, Im A1, Re AW, Im AW] x cols [Re B1, Im B1, Re BW, Im BW]
// (each 4 nbins long, rows padded to M = 128, cols to NC = a multiple of 16), whose blocks
// combine into the complex gam0, gam3, gam2 (region 0) and gam1, weight (region 1).  The
// row-range mask min(a, b) in [ks, mk) is {a, b >= ks} minus {a, b >= mk}: every record
// enters as two K entries, the second with negated A and both masked at mk.  Operands are
// split into TF32 hi + lo parts and multiplied as hi*hi + hi*lo + lo*hi (FP32-level
// products); the FP32 accumulators in TMEM are drained to FP64 every TC_DRAIN chunks.
static constexpr int TCB = 128;        // threads (4 warps = the 128 TMEM lanes)
static constexpr int TC_REC = 16;      // records per chunk = 32 K entries = 4 K steps
// Chunks between FP64 drains: the TMEM accumulators add 3 MMAs x 4 K steps x 2 entries per
// record in FP32, and that error grows with the records per drain (at 20 bins / max_n 30,
// 1024 records per drain gave 1.6e-5 of max|gam|; 128 records keep it near 2e-6).
static constexpr int TC_DRAIN = 8;

__device__ __forceinline__ void tf32_split(float x, float& hi, float& lo)
{
    hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
    lo = x - hi;
}

__global__ void __launch_bounds__(TCB) k_mp_zeta_tc(ZParams Q, int* status)
{
    extern __shared__ __align__(1024) unsigned char zts[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t taddr_sh;
    const int nb = Q.nbins, M = Q.maxn, nn = 2 * M + 1, gst = 2 * M + 3;
    const int n = (int)blockIdx.x - M;
    const int g = blockIdx.y;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int NC = (4 * nb + 15) & ~15;
    const int aBytes = 4 * 4096, bBytes = 4 * NC * 32, rgBytes = aBytes + bBytes;
    // Operand tiles: [region][hi, lo][A (4 K steps of 128 rows) | B (4 K steps of NC rows)].
    auto tileA = [&](int r, int h, int st) { return zts + (r * 2 + h) * rgBytes + st * 4096; };
    auto tileB = [&](int r, int h, int st) { return zts + (r * 2 + h) * rgBytes + aBytes + st * NC * 32; };
    for (int q = tid; q < 4 * rgBytes / 16; q += TCB)
        reinterpret_cast<float4*>(zts)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (tid == 0) mbar_init(&mbar, 1);
    __syncthreads();
    if (wid == 0) tmem_alloc(&taddr_sh, 256);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tm = taddr_sh;
    const uint32_t idesc = umma_idesc_tf32(128, NC);
    const int nw = n >= 0 ? n : -n;
    const long long r0 = Q.nrec * g / Q.ngroups, r1 = Q.nrec * (g + 1) / Q.ngroups;
    uint32_t phase = 0;
    int nchunk = 0;
    bool fresh = true;     // the next MMA overwrites the accumulators
    bool failed = false;
    float* S = reinterpret_cast<float*>(zts);   // drain buffer [128][2 NC], over the tiles
    const size_t Zs = (size_t)Q.Z;
    auto drain = [&]() {
        __syncthreads();
        for (int r = 0; r < 2; ++r)
            for (int c0 = 0; c0 < NC; c0 += 8) {
                float v[8];
                tmem_ld8(tm + ((uint32_t)(32 * wid) << 16) + (uint32_t)(r * 128 + c0), v);
#pragma unroll
                for (int q = 0; q < 8; ++q) S[(32 * wid + lane) * (2 * NC) + r * NC + c0 + q] = v[q];
            }
        tc_fence_before();
        __syncthreads();
        double* part = Q.part + (size_t)g * 10 * Zs;
        for (int e = tid; e < nb * nb; e += TCB) {
            const int a = e / nb, b = e % nb;
            auto C0 = [&](int row, int col) { return S[row * (2 * NC) + col]; };
            auto C1 = [&](int row, int col) { return S[row * (2 * NC) + NC + col]; };
            // (Re X + i Im X)(Re Y + i Im Y) from the four real blocks.
            const float g0r = C0(a, b) - C0(nb + a, nb + b), g0i = C0(a, nb + b) + C0(nb + a, b);
            const float g2r = C0(a, 2 * nb + b) - C0(nb + a, 3 * nb + b);
            const float g2i = C0(a, 3 * nb + b) + C0(nb + a, 2 * nb + b);
            const float g3r = C0(2 * nb + a, b) - C0(3 * nb + a, nb + b);
            const float g3i = C0(2 * nb + a, nb + b) + C0(3 * nb + a, b);
            const float g1r = C1(a, b) - C1(nb + a, nb + b), g1i = C1(a, nb + b) + C1(nb + a, b);
            const float wr = C1(2 * nb + a, 2 * nb + b) - C1(3 * nb + a, 3 * nb + b);
            const float wi = a == b ? 0.f : C1(2 * nb + a, 3 * nb + b) + C1(3 * nb + a, 2 * nb + b);
            const size_t i = (size_t)(a * nb + b) * nn + M + n;
            // All ten loads first, then the stores: one round trip per entry instead of ten
            // (the compiler cannot reorder a load past a store to a possibly equal address).
            const float add[10] = {g0r, g0i, g1r, g1i, g2r, g2i, g3r, g3i, wr, wi};
            double o[10];
#pragma unroll
            for (int q = 0; q < 10; ++q) o[q] = part[q * Zs + i];
#pragma unroll
            for (int q = 0; q < 10; ++q) part[q * Zs + i] = o[q] + (double)add[q];
        }
        __syncthreads();
        // The tile area was overwritten: restore the zero padding before the next fill.
        for (int q = tid; q < 4 * rgBytes / 16; q += TCB)
            reinterpret_cast<float4*>(zts)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        fresh = true;
        nchunk = 0;
    };
    // The chunk's record data is loaded into registers one chunk ahead, so the loads of
    // chunk i+1 overlap the MMAs of chunk i.  A thread holds up to TC_IT fill items.
    const int nab = (nb + 7) >> 3;
    constexpr int TC_IT = 4;                 // nab * 8 * TC_REC / TCB <= 4 for nbins <= 32
    float2 ig[TC_IT][5];
    float4 ih[TC_IT];                        // w1, Re wg1, Im wg1, (ks, mk) packed
    auto load_items = [&](long long cb) {
        const int nvb = (int)min((long long)TC_REC, r1 - cb);
#pragma unroll
        for (int j = 0; j < TC_IT; ++j) {
            const int idx = tid + j * TCB;
            const int w = idx >> 5, l = idx & 31;
            const int a = (w % nab) * 8 + (l & 7);
            const int v = (w / nab) * 4 + (l >> 3);
            ih[j] = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
            if (idx >= nab * 8 * TC_REC || a >= nb || v >= nvb) continue;
            const float* R = Q.rec + (size_t)(cb + v) * Q.rec_floats;
            const float2* RG = reinterpret_cast<const float2*>(R + 8);
            const float2* RW = RG + (size_t)gst * nb;
            const int sh = Q.shift;
            ig[j][0] = RG[(n - sh + M + 1) * nb + a];    // G[n-1]
            ig[j][1] = RG[(-n - sh + M + 1) * nb + a];   // G[-n-1]
            ig[j][2] = RG[(n + sh + M + 1) * nb + a];    // G[n+1]
            ig[j][3] = RG[(-n + sh + M + 1) * nb + a];   // G[-n+1]
            ig[j][4] = RW[nw * nb + a];            // W[|n|]
            const int ks = __float_as_int(R[1]), mk = __float_as_int(R[2]);
            ih[j] = make_float4(R[3], R[4], R[5], __int_as_float((ks << 8) | mk));
        }
    };
    if (r0 < r1) load_items(r0);
    for (long long c0 = r0; c0 < r1 && !failed; c0 += TC_REC) {
        // Fill the K entries v (rows >= ks) and TC_REC + v (rows >= mk, A negated) of the
        // chunk.  A warp covers 8 consecutive bins x 4 consecutive records: its stores hit
        // the 8 rows x 4 k of core matrices, all 32 banks once.
#pragma unroll
        for (int j = 0; j < TC_IT; ++j) {
            const int idx = tid + j * TCB;
            const int w = idx >> 5, l = idx & 31;
            const int a = (w % nab) * 8 + (l & 7);
            const int v = (w / nab) * 4 + (l >> 3);
            if (idx >= nab * 8 * TC_REC || a >= nb) continue;
            float A0r = 0.f, A0i = 0.f, A1r = 0.f, A1i = 0.f, A3r = 0.f, A3i = 0.f, AWr = 0.f, AWi = 0.f;
            float B0r = 0.f, B0i = 0.f, B1r = 0.f, B1i = 0.f, B2r = 0.f, B2i = 0.f, BWr = 0.f, BWi = 0.f;
            int ks = nb, mk = nb;
            const int am = a % Q.nbd;    // the row mask's bin
            const int km = __float_as_int(ih[j].w);
            if (km >= 0) {
                const float w1 = ih[j].x, wr = ih[j].y, wi = ih[j].z;
                ks = km >> 8; mk = km & 255;
                const float2 gm1 = ig[j][0], gmm1 = ig[j][1], gp1 = ig[j][2], gmp1 = ig[j][3];
                float2 w = ig[j][4];
                if (n < 0) w.y = -w.y;
                A0r = wr * gm1.x - wi * gm1.y;   A0i = wr * gm1.y + wi * gm1.x;
                A1r = wr * gp1.x + wi * gp1.y;   A1i = wr * gp1.y - wi * gp1.x;
                A3r = wr * gmp1.x + wi * gmp1.y; A3i = wi * gmp1.x - wr * gmp1.y;
                AWr = w1 * w.x;                  AWi = w1 * w.y;
                B0r = gmm1.x; B0i = gmm1.y; B1r = gmp1.x; B1i = gmp1.y;
                B2r = gp1.x;  B2i = -gp1.y; BWr = w.x;    BWi = -w.y;
            }
#pragma unroll
            for (int t = 0; t < 2; ++t) {
                const int e = t * TC_REC + v, st = e >> 3, kk = e & 7;
                const bool on = am >= (t == 0 ? ks : mk);
                const float sg = on ? (t == 0 ? 1.f : -1.f) : 0.f, sb = on ? 1.f : 0.f;
                const float av[2][4] = {{A0r, A0i, A3r, A3i}, {A1r, A1i, AWr, AWi}};
                const float bv[2][4] = {{B0r, B0i, B2r, B2i}, {B1r, B1i, BWr, BWi}};
#pragma unroll
                for (int r = 0; r < 2; ++r)
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int row = q * nb + a;
                        float hi, lo;
                        tf32_split(sg * av[r][q], hi, lo);
                        *reinterpret_cast<float*>(tileA(r, 0, st) + umma_tile_off(row, kk)) = hi;
                        *reinterpret_cast<float*>(tileA(r, 1, st) + umma_tile_off(row, kk)) = lo;
                        tf32_split(sb * bv[r][q], hi, lo);
                        *reinterpret_cast<float*>(tileB(r, 0, st) + umma_tile_off(row, kk)) = hi;
                        *reinterpret_cast<float*>(tileB(r, 1, st) + umma_tile_off(row, kk)) = lo;
                    }
            }
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            for (int r = 0; r < 2; ++r) {
                const uint32_t d = tm + (uint32_t)(r * 128);
                for (int st = 0; st < 4; ++st) {
                    const uint64_t ah = umma_desc(smem_u32(tileA(r, 0, st)), 128, 256);
                    const uint64_t al = umma_desc(smem_u32(tileA(r, 1, st)), 128, 256);
                    const uint64_t bh = umma_desc(smem_u32(tileB(r, 0, st)), 128, 256);
                    const uint64_t bl = umma_desc(smem_u32(tileB(r, 1, st)), 128, 256);
                    umma_tf32(d, ah, bh, idesc, (fresh && st == 0) ? 0u : 1u);
                    umma_tf32(d, ah, bl, idesc, 1u);
                    umma_tf32(d, al, bh, idesc, 1u);
                }
            }
            umma_commit(&mbar);
        }
        if (c0 + TC_REC < r1) load_items(c0 + TC_REC);   // overlaps the MMAs
        const bool ok = mbar_wait(&mbar, phase, 1 << 24);
        phase ^= 1u;
        tc_fence_after();
        failed = __syncthreads_or(!ok) != 0;
        fresh = false;
        if (failed) break;
        if (++nchunk == TC_DRAIN) drain();
    }
    if (!failed && !fresh) drain();
    if (failed && tid == 0) atomicExch(status, 1);
    tc_fence_before();
    __syncthreads();
    if (wid == 0) tmem_dealloc(tm, 256);
}

// The n = 0 scalar outputs of calculateZeta over vertex records (ntri, meand2/3,
// meanlogd2/3): for every entry (a, b) whose min(a, b) lies in the record's rows,
//   a != b: ntri += n1 np_a np_b, meand2 += w1 sumw_b sumwr_a, meand3 += w1 sumw_a sumwr_b
//   a == b: ntri += n1 np_a (np_a - 1), meand2 = meand3 += w1 (sumw_a sumwr_a - sumwwr_a)
// (meanlogd likewise with sumwlogr).  ntri is an exact 64-bit integer sum; the means are FP32
// products with FP64 sums.  Block (g, tile) adds its sums to group g's partial arrays.
__global__ void __launch_bounds__(ZB) k_mp_zscal(ZParams Q, double* spart,
                                                 unsigned long long* ntp)
{
    extern __shared__ float4 zsh[];    // [chunk][nb][2]
    __shared__ int4 hdr_sh[64];
    const int nb = Q.nbins, M = Q.maxn, gst = 2 * M + 3;
    const int nb2 = nb * nb;
    const int g = blockIdx.x, tid = threadIdx.x;
    int ea[ZE], eb[ZE], em[ZE];     // entry (a, b) and min(a, b) mod nbd (the row mask)
    bool ev[ZE];
#pragma unroll
    for (int j = 0; j < ZE; ++j) {
        const int e = ((int)blockIdx.y * ZE + j) * ZB + tid;
        ev[j] = e < nb2;
        ea[j] = ev[j] ? e / nb : 0;
        eb[j] = ev[j] ? e % nb : 0;
        em[j] = min(ea[j] % Q.nbd, eb[j] % Q.nbd);
    }
    double D[ZE][4];
    unsigned long long C[ZE];
#pragma unroll
    for (int j = 0; j < ZE; ++j) { C[j] = 0ull; for (int q = 0; q < 4; ++q) D[j][q] = 0.; }
    const long long r0 = Q.nrec * g / gridDim.x, r1 = Q.nrec * (g + 1) / gridDim.x;
    for (long long c0 = r0; c0 < r1; c0 += Q.chunk) {
        const int nv = (int)min((long long)Q.chunk, r1 - c0);
        __syncthreads();
        for (int idx = tid; idx < nv * nb; idx += ZB) {
            const int v = idx / nb, a = idx % nb;
            const float* R = Q.rec + (size_t)(c0 + v) * Q.rec_floats;
            const float* RS = R + 8 + 2 * (size_t)gst * nb + 2 * (size_t)(M + 1) * nb;
            float4* d = zsh + ((size_t)v * nb + a) * 2;
            d[0] = make_float4(RS[a], RS[nb + a], RS[2 * nb + a], RS[3 * nb + a]);
            d[1] = make_float4(RS[4 * nb + a], RS[5 * nb + a], 0.f, 0.f);
            if (a == 0)
                hdr_sh[v] = make_int4(__float_as_int(R[1]), __float_as_int(R[2]),
                                      __float_as_int(R[6]), __float_as_int(R[3]));
        }
        __syncthreads();
        float F[ZE][4];
#pragma unroll
        for (int j = 0; j < ZE; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) F[j][q] = 0.f;
        for (int v = 0; v < nv; ++v) {
            const int4 h = hdr_sh[v];
            const float w1 = __int_as_float(h.w);
            const unsigned long long n1 = (unsigned long long)h.z;
#pragma unroll
            for (int j = 0; j < ZE; ++j) {
                const int m = em[j];
                if (!ev[j] || m < h.x || m >= h.y) continue;
                const float4 pa = zsh[((size_t)v * nb + ea[j]) * 2];
                const unsigned long long npa = (unsigned)__float_as_int(pa.x);
                if (ea[j] == eb[j]) {
                    const float4 pa2 = zsh[((size_t)v * nb + ea[j]) * 2 + 1];
                    C[j] += n1 * npa * (npa > 0 ? npa - 1 : 0);
                    const float md = w1 * (pa.y * pa.z - pa2.x);
                    const float ml = w1 * (pa.y * pa.w - pa2.y);
                    F[j][0] += md; F[j][1] += ml; F[j][2] += md; F[j][3] += ml;
                } else {
                    const float4 pb = zsh[((size_t)v * nb + eb[j]) * 2];
                    C[j] += n1 * npa * (unsigned long long)(unsigned)__float_as_int(pb.x);
                    // (ordered = 1's meanlogd3 in the vertex-3 x vertex-2 block takes
                    // mp3.sumw at the column's bin, as the reference writes it)
                    const float swl = (Q.typo32 && ea[j] >= Q.nbd)
                        ? zsh[((size_t)v * nb + eb[j] % Q.nbd + Q.nbd) * 2].y : pa.y;
                    F[j][0] += w1 * pb.y * pa.z; F[j][1] += w1 * pb.y * pa.w;
                    F[j][2] += w1 * pa.y * pb.z; F[j][3] += w1 * swl * pb.w;
                }
            }
        }
#pragma unroll
        for (int j = 0; j < ZE; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) D[j][q] += F[j][q];
    }
#pragma unroll
    for (int j = 0; j < ZE; ++j) {
        if (!ev[j]) continue;
        const int e = ea[j] * nb + eb[j];
#pragma unroll
        for (int q = 0; q < 4; ++q) spart[((size_t)g * 4 + q) * nb2 + e] += D[j][q];
        ntp[(size_t)g * nb2 + e] += C[j];
    }
}

// Final sums, in a fixed order: the per-block outputs, the contraction groups' partials and
// the diagonal corrections.
__global__ void k_mp_reduce(int nblk, long long stride, long long Z, int nb, int nn,
                            const double* in, const double* diag, long long diag_stride,
                            int ngroups, const double* part, int nsg, const double* spart,
                            const unsigned long long* ntp, double* out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 15 * Z) return;
    const int q = (int)(i / Z);
    const long long r = i % Z;
    double s = 0.;
    for (int b = 0; b < nblk; ++b) s += in[(size_t)b * stride + i];
    const int qp = q < 8 ? q : (q == 12 ? 8 : (q == 13 ? 9 : -1));
    if (qp >= 0)
        for (int g = 0; g < ngroups; ++g) s += part[((size_t)g * 10 + qp) * Z + r];
    const long long ab = r / nn;
    const int a = (int)(ab / nb), b = (int)(ab % nb);
    if (r % nn == nn / 2 && ((q >= 8 && q <= 11) || q == 14)) {
        const size_t nb2 = (size_t)nb * nb;
        if (q == 14) {
            unsigned long long c = 0ull;
            for (int g = 0; g < nsg; ++g) c += ntp[(size_t)g * nb2 + ab];
            s += (double)c;
        } else {
            for (int g = 0; g < nsg; ++g) s += spart[((size_t)g * 4 + (q - 8)) * nb2 + ab];
        }
    }
    if (a == b && (q < 8 || q == 12)) {
        const int d = q < 8 ? q : 8;
        for (int bl = 0; bl < nblk; ++bl) s -= diag[(size_t)bl * diag_stride + (size_t)d * nb + a];
    }
    out[i] = s;
}

// ---------------------------------------------------------------------------------------
// Host orchestration.

size_t mp_slot_doubles(int nb, int M)
{ return 2 * (size_t)nb * (M + 1) + 2 * (size_t)nb * (2 * M + 3) + 13 * (size_t)nb; }

static int mp_rec_floats(int nb, int M)
{ return (8 + 2 * nb * (2 * M + 3) + 2 * nb * (M + 1) + 6 * nb + 3) & ~3; }

int run_multipole(MPParams& P, MPScratch& X, int ntop, cudaStream_t st, double* h_out)
{
    const int nb = P.nbins, M = P.maxn, nn = 2 * M + 1;
    const long long Z = (long long)nb * nb * nn;
    int dev = 0, nsm = 0;
    TC_CU(cudaGetDevice(&dev));
    TC_CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const size_t shbytes = sizeof(double) * (2 * (size_t)nb * (2 * M + 3) + 2 * (size_t)nb * (M + 1));
    if (shbytes > 160 * 1024 || M + 1 > 64 || nb > MP_MAXNB) {
        set_last_error("the GPU multipole path needs max_n <= 63, nbins <= 128 and "
                       "nbins * max_n within its shared-memory staging");
        return 3;
    }
    auto* kfin = P.three ? k_mp_finish<true> : k_mp_finish<false>;
    TC_CU(cudaFuncSetAttribute(kfin, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shbytes));
    int per = 0;
    TC_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kfin, MB, shbytes));
    if (per < 1) per = 1;
    const int nblk = nsm * std::min(per, 2);
    P.slot_doubles = (long long)mp_slot_doubles(nb, M);
    P.out_stride = 15 * Z;
    // Contraction geometry: records per shared-memory chunk, entry tiles, record groups.
    const int chunk = (int)std::max<long long>(1, std::min<long long>(64, (96 * 1024) / (64LL * nb)));
    const size_t zsh = (size_t)chunk * nb * 64;
    TC_CU(cudaFuncSetAttribute(k_mp_zeta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zsh));
    const int etiles = (nb * nb + ZE * ZB - 1) / (ZE * ZB);
    // The tensor-core contraction (tcgen05) for nbins <= 32, unless TCGPU_MP_TENSOR=0.  Its
    // shared memory keeps at most two blocks on an SM (each holds 256 TMEM columns).
    bool use_tc = 4 * nb <= 128;
    if (const char* ev = std::getenv("TCGPU_MP_TENSOR")) use_tc = use_tc && std::atoi(ev) != 0;
    const int NCt = (4 * nb + 15) & ~15;
    const size_t tcsm = std::max<size_t>((size_t)4 * (16384 + 128 * NCt), 100 * 1024);
    if (use_tc)
        TC_CU(cudaFuncSetAttribute(k_mp_zeta_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tcsm));
    const int ngroups = std::max(1, (4 * nsm + nn * etiles - 1) / (nn * etiles));
    // Scalar outputs: records per chunk and record groups.
    const int chunk2 = (int)std::max<long long>(1, std::min<long long>(64, (48 * 1024) / (32LL * nb)));
    const size_t zsh2 = (size_t)chunk2 * nb * 32;
    // (with its static header array this can pass the 48 KB that needs no opt-in)
    TC_CU(cudaFuncSetAttribute(k_mp_zscal, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zsh2));
    const int nsg = std::max(1, 2 * nsm / etiles);
    const int recf = mp_rec_floats(nb, M);
    const long long acc_cap = 4096;
    X.want_a1 = std::max<long long>(X.want_a1, 4LL * std::max(ntop, P.ntop2) + (1 << 16));
    X.want_jobs = std::max<long long>(X.want_jobs, 1 << 18);
    X.want_a2 = std::max<long long>(X.want_a2, 1 << 20);
    X.want_slots = std::max(X.want_slots, 32);
    for (int attempt = 0; attempt < 4; ++attempt) {
        // Allocate what is requested (the requests grow after an overflow).
        if (X.arena1_cap < X.want_a1 || (long long)ntop > X.ntop_alloc) {
            dfree(X.arena1);
            X.arena1_cap = 0;
            TC_TRY(dalloc(&X.arena1, (size_t)X.want_a1 * ntop));
            X.arena1_cap = X.want_a1; X.ntop_alloc = ntop;
        }
        if (X.jobs_cap < X.want_jobs) {
            dfree(X.jobs);
            X.jobs_cap = 0;
            TC_TRY(dalloc(&X.jobs, (size_t)X.want_jobs));
            X.jobs_cap = X.want_jobs;
        }
        const bool grow_blk = nblk > X.nblk;
        if (X.arena2_cap < X.want_a2 || grow_blk) {
            dfree(X.arena2);
            X.arena2_cap = 0;
            TC_TRY(dalloc(&X.arena2, (size_t)X.want_a2 * nblk));
            X.arena2_cap = X.want_a2;
        }
        if (X.acc_cap < acc_cap || grow_blk) {
            dfree(X.acc); dfree(X.perm);
            X.acc_cap = 0;
            TC_TRY(dalloc(&X.acc, (size_t)MP_REC * acc_cap * nblk));
            TC_TRY(dalloc(&X.perm, (size_t)acc_cap * nblk));
            X.acc_cap = acc_cap;
        }
        if (X.nslots < X.want_slots || grow_blk || P.slot_doubles != X.slot_doubles) {
            dfree(X.slots);
            X.nslots = 0;
            TC_TRY(dalloc(&X.slots, (size_t)X.want_slots * P.slot_doubles * nblk));
            X.nslots = X.want_slots; X.slot_doubles = P.slot_doubles;
        }
        if (grow_blk || P.out_stride > X.out_stride || 9LL * nb > X.diag_stride) {
            dfree(X.out); dfree(X.total); dfree(X.diag);
            X.out_stride = 0; X.diag_stride = 0;
            TC_TRY(dalloc(&X.out, (size_t)P.out_stride * nblk));
            TC_TRY(dalloc(&X.total, (size_t)P.out_stride));
            TC_TRY(dalloc(&X.diag, (size_t)9 * nb * nblk));
            X.out_stride = P.out_stride; X.diag_stride = 9LL * nb;
        }
        {
            // The vertex-record buffer: up to 16 GiB and a quarter of the free memory, or the
            // byte count in TCGPU_MP_RECORD_BYTES (at least 16 records).
            size_t budget = (size_t)16 << 30;
            if (const char* ev = std::getenv("TCGPU_MP_RECORD_BYTES"))
                budget = (size_t)std::max(0LL, std::atoll(ev));
            const long long cap = std::max<long long>(16, (long long)(budget / (4ULL * recf)));
            if (!X.zrec || X.zrec_floats != recf || X.zcap != cap) {
                dfree(X.zrec);
                X.zcap = 0;
                size_t fr = 0, tot = 0;
                TC_CU(cudaMemGetInfo(&fr, &tot));
                const long long fit = std::max<long long>(16, (long long)(fr / 4 / (4ULL * recf)));
                const long long c2 = std::min(cap, fit);
                TC_TRY(dalloc(&X.zrec, (size_t)c2 * recf));
                X.zcap = c2; X.zrec_floats = recf;
            }
        }
        if (X.nsg < nsg || X.spart_nb2 < (long long)nb * nb) {
            dfree(X.spart); dfree(X.ntp);
            X.nsg = 0;
            TC_TRY(dalloc(&X.spart, (size_t)nsg * 4 * nb * nb));
            TC_TRY(dalloc(&X.ntp, (size_t)nsg * nb * nb));
            X.nsg = nsg; X.spart_nb2 = (long long)nb * nb;
        }
        if (X.ngroups < ngroups || X.part_stride < 10 * Z) {
            dfree(X.part);
            X.ngroups = 0;
            TC_TRY(dalloc(&X.part, (size_t)ngroups * 10 * Z));
            X.ngroups = ngroups; X.part_stride = 10 * Z;
        }
        if (!X.ctl) TC_TRY(dalloc(&X.ctl, 4));
        if (!X.tcstatus) TC_TRY(dalloc(&X.tcstatus, 1));
        if (!X.err) TC_TRY(dalloc(&X.err, 2));
        if (!X.dbg) TC_TRY(dalloc(&X.dbg, 32));
        X.nblk = std::max(X.nblk, nblk);
        P.arena1 = X.arena1; P.arena1_cap = X.arena1_cap;
        P.jobs = X.jobs; P.jobs_cap = X.jobs_cap;
        P.njobs = X.ctl; P.job_next = X.ctl + 1; P.zcount = X.ctl + 2; P.zmaxjob = X.ctl + 3;
        P.arena2 = X.arena2; P.arena2_cap = X.arena2_cap;
        P.acc = X.acc; P.perm = X.perm; P.acc_cap = (int)X.acc_cap;
        P.slots = X.slots; P.nslots = X.nslots;
        P.out = X.out;
        P.diag = X.diag;
        P.zrec = X.zrec; P.zcap = X.zcap; P.zrec_floats = recf;
        // Jobs are not started once the buffer holds zstop records; the blocks' jobs in
        // flight then fill at most nblk x (the largest job so far) more.
        auto set_zstop = [&](long long maxjob) {
            const long long margin = (long long)nblk * std::max<long long>(64, 2 * maxjob);
            P.zstop = std::max<long long>(X.zcap / 4, X.zcap - margin);
        };
        set_zstop(512);
        P.err = X.err;
        P.dbg = X.dbg;
        TC_CU(cudaMemsetAsync(X.ctl, 0, 4 * sizeof(unsigned long long), st));
        TC_CU(cudaMemsetAsync(X.tcstatus, 0, sizeof(int), st));
        X.overflow = 0; X.records = 0; X.waves = 0;
        TC_CU(cudaMemsetAsync(X.err, 0, 2 * sizeof(int), st));
        TC_CU(cudaMemsetAsync(X.out, 0, sizeof(double) * (size_t)P.out_stride * nblk, st));
        TC_CU(cudaMemsetAsync(X.diag, 0, sizeof(double) * (size_t)9 * nb * nblk, st));
        TC_CU(cudaMemsetAsync(X.part, 0, sizeof(double) * (size_t)ngroups * 10 * Z, st));
        TC_CU(cudaMemsetAsync(X.spart, 0, sizeof(double) * (size_t)nsg * 4 * nb * nb, st));
        TC_CU(cudaMemsetAsync(X.ntp, 0, sizeof(unsigned long long) * (size_t)nsg * nb * nb, st));
        count_launch();
        k_mp_split1<<<ntop, MB, 0, st>>>(P);
        TC_CU(cudaGetLastError());
        unsigned long long nj = 0;
        int e = 0;
        TC_CU(cudaMemcpyAsync(&nj, X.ctl, sizeof(nj), cudaMemcpyDeviceToHost, st));
        TC_CU(cudaMemcpyAsync(&e, X.err, sizeof(int), cudaMemcpyDeviceToHost, st));
        TC_CU(cudaStreamSynchronize(st));
        P.njobs_val = (long long)nj;
        // Waves: the finish kernel runs jobs until the record buffer is nearly full, then the
        // records are contracted and the buffer is reused.
        for (int wave = 0; e == 0; ++wave) {
            TC_CU(cudaMemsetAsync(X.ctl + 2, 0, sizeof(unsigned long long), st));
            count_launch();
            kfin<<<nblk, MB, shbytes, st>>>(P);
            TC_CU(cudaGetLastError());
            unsigned long long c[4] = {0, 0, 0, 0};
            TC_CU(cudaMemcpyAsync(c, X.ctl, sizeof(c), cudaMemcpyDeviceToHost, st));
            TC_CU(cudaMemcpyAsync(&e, X.err, sizeof(int), cudaMemcpyDeviceToHost, st));
            TC_CU(cudaStreamSynchronize(st));
            if (e) break;
            ZParams Q;
            Q.rec = X.zrec; Q.nrec = std::min<long long>((long long)c[2], X.zcap);
            Q.rec_floats = recf; Q.nbins = nb; Q.maxn = M; Q.chunk = chunk;
            Q.ngroups = ngroups; Q.part = X.part; Q.Z = Z;
            Q.shift = P.vreal ? 0 : 1;
            Q.nbd = P.nbd; Q.typo32 = P.typo32;
            if (Q.nrec > 0) {
                count_launch();
                if (use_tc) k_mp_zeta_tc<<<dim3(nn, ngroups), TCB, tcsm, st>>>(Q, X.tcstatus);
                else k_mp_zeta<<<dim3(nn, ngroups, etiles), ZB, zsh, st>>>(Q);
                TC_CU(cudaGetLastError());
                if (!P.quick) {
                    ZParams Q2 = Q;
                    Q2.chunk = chunk2;
                    count_launch();
                    k_mp_zscal<<<dim3(nsg, etiles), ZB, zsh2, st>>>(Q2, X.spart, X.ntp);
                    TC_CU(cudaGetLastError());
                }
            }
            X.overflow += std::max<long long>(0, (long long)c[2] - X.zcap);
            X.records += (long long)c[2];
            ++X.waves;
            set_zstop((long long)c[3]);
            if ((long long)c[1] >= P.njobs_val) break;
            if (wave > (1 << 24)) { e = MP_ERR_STACK; break; }
        }
        if (e == MP_ERR_ARENA || e == MP_ERR_JOBS || e == MP_ERR_SLOTS) {
            X.want_a1 = X.arena1_cap * 4; X.want_jobs = X.jobs_cap * 4;
            X.want_a2 = X.arena2_cap * 4;
            X.want_slots = std::min(X.nslots * 2, 64);
            continue;
        }
        if (e == MP_ERR_CHECK) {
            int site = 0;
            double d[32];
            TC_CU(cudaMemcpy(&site, X.err + 1, sizeof(int), cudaMemcpyDeviceToHost));
            TC_CU(cudaMemcpy(d, X.dbg, sizeof(d), cudaMemcpyDeviceToHost));
            std::string msg = "multipole: internal consistency check failed at site " +
                              std::to_string(site);
            if (site == 4 || site == 7) {
                msg += " [";
                for (int q = 0; q < 26; ++q) msg += std::to_string(d[q]) + " ";
                msg += "]";
            }
            set_last_error(msg);
            return 4;
        }
        if (e) {
            set_last_error("multipole: device stack overflow (tree too deep)");
            return 4;
        }
        {
            int tcs = 0;
            TC_CU(cudaMemcpyAsync(&tcs, X.tcstatus, sizeof(int), cudaMemcpyDeviceToHost, st));
            TC_CU(cudaStreamSynchronize(st));
            if (tcs) {
                set_last_error("multipole: a tensor-core contraction did not complete in time");
                return 4;
            }
        }
        count_launch();
        k_mp_reduce<<<(unsigned)((P.out_stride + 255) / 256), 256, 0, st>>>(
            nblk, P.out_stride, Z, nb, nn, X.out, X.diag, 9LL * nb, ngroups, X.part,
            P.quick ? 0 : nsg, X.spart, X.ntp, X.total);
        TC_CU(cudaGetLastError());
        TC_CU(cudaMemcpyAsync(h_out, X.total, sizeof(double) * (size_t)P.out_stride,
                              cudaMemcpyDeviceToHost, st));
        TC_CU(cudaStreamSynchronize(st));
        return 0;
    }
    set_last_error("multipole scratch still too small after retries");
    return 4;
}

void free_mp_scratch(MPScratch& X)
{
    dfree(X.arena1); dfree(X.jobs); dfree(X.arena2); dfree(X.acc); dfree(X.perm);
    dfree(X.slots); dfree(X.out); dfree(X.diag); dfree(X.total); dfree(X.zrec); dfree(X.part);
    dfree(X.spart); dfree(X.ntp);
    dfree(X.ctl); dfree(X.err); dfree(X.dbg); dfree(X.tcstatus);
    X = MPScratch();
}

}  // namespace tc
