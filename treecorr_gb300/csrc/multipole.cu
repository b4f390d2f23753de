// multipole.cu -- GGG 3-point correlation with LogMultipole binning on sm_103a.
//
// Semantics follow the reference's multipole algorithm (Porth et al.):
//   BaseCorr3::multipole (src/Corr3.cpp:1124-1175), multipoleSplit1 (1374-1408),
//   splitC2Cells (1323-1372), multipoleFinish (1548-1613), splitC2CellsOrCalculateGn
//   (1452-1546), Corr3::calculateGn + MultipoleScratch<GData>::calculateGn (1681-1704,
//   1767-1828), Corr3::calculateZeta (1861-1974) and MultipoleHelper<5>::CalculateZeta
//   (2585-2843); scratch layout include/MultipoleScratch.h:36-125, 296-383.
//
// GB300 design:
//   * Phase 1: one block per top-level cell walks the c1 subtree of multipoleSplit1, refining
//     the c2 list with block-parallel decisions and a stable block scan, and emits one job
//     (c1, c2 list) per cell that is small enough to start multipoleFinish.
//   * Phase 2: persistent blocks take jobs from a counter.  A job runs multipoleFinish as a
//     depth-first loop: each pass over the c2 list is block-parallel; the accepted c2 cells
//     are added to the G_n / W_n scratch by warps that own disjoint bins (so no atomics, and
//     each bin keeps the list order), with the powers z^n of a pair computed by one warp-wide
//     multiplicative scan.  When c1 must split, the scratch is copied into a free slot and
//     the right child is pushed, as the reference's mp.duplicate() does.  Rows of Zeta that
//     are final are contracted into the block's private copy of the outputs.
//   * A last kernel sums the private copies in block order.
// All arithmetic is FP64 (the reference's precision); the cell payloads are the tree's
// float values.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <vector>

#include "tc_internal.cuh"
#include "tc_host.hpp"
#include "multipole.hpp"

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

int launch_leaf_sums(int ncap, const Cells& C, double* ls, cudaStream_t st)
{
    TC_CU(cudaMemsetAsync(ls, 0, 4 * sizeof(double) * (size_t)ncap, st));
    count_launch();
    k_leaf_sums<<<(ncap + 255) / 256, 256, 0, st>>>(ncap, C, ls);
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

// ---------------------------------------------------------------------------------------
// Phase 1: multipoleSplit1 + splitC2Cells, one block per top-level cell.

struct P1Entry { int c1, off, len, pad; };

__global__ void __launch_bounds__(MB) k_mp_split1(MPParams P)
{
    __shared__ P1Entry stk[MSTACK];
    __shared__ int sp, top_rel, scan_sh[MW];
    __shared__ P1Entry cur;
    const int b = blockIdx.x;
    int* arena = P.arena1 + (size_t)b * P.arena1_cap;
    const int tid = threadIdx.x;
    for (int j = tid; j < P.ntop; j += MB) arena[j] = P.tops[j];
    if (tid == 0) {
        sp = 0;
        top_rel = P.ntop;
        stk[sp++] = {P.tops[b], 0, P.ntop, 0};
    }
    __syncthreads();
    int guard = 0;
    while (true) {
        __syncthreads();
        if (sp == 0) break;
        if (++guard > (1 << 24)) {
            if (tid == 0) set_mp_err(P.err, MP_ERR_STACK);
            break;
        }
        if (tid == 0) cur = stk[--sp];
        __syncthreads();
        const int c1 = cur.c1;
        const double s1 = P.size[c1];
        const int base = top_rel;
        int written = 0;
        for (int j0 = 0; j0 < cur.len; j0 += MB) {
            const int j = j0 + tid;
            int cnt = 0, ca = -1, cb = -1;
            if (j < cur.len) {
                const int c2 = arena[cur.off + j];
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

struct P2Entry { int c1, len, slot, mink; long long goff; double maxr; long long mark; };

// Scratch slot layout (doubles): Wn [nb][M+1] complex, Gn [nb][2M+3] complex (n = -(M+1) ..
// M+1), gg0/gg1/gg2 [nb] complex, then npairs, sumw, sumwr, sumwlogr, sumww, sumwwr,
// sumwwlogr [nb].
__device__ __forceinline__ double* slot_ptr(const MPParams& P, int blk, int s)
{ return P.slots + ((size_t)blk * P.nslots + s) * P.slot_doubles; }

// The Zeta contraction for rows k2 in [ks, mk) of vertex c1 (calculateZeta).
__device__ void zeta_rows(const MPParams& P, int c1, const double* S, int ks, int mk, double* out,
                          double* shG, double* shW)
{
    const int nb = P.nbins, M = P.maxn, nn = 2 * M + 1;
    const int gst = 2 * M + 3;          // complex entries per bin in Gn
    const size_t Z = (size_t)nb * nb * nn;
    const double* W = S;
    const double* G = S + 2 * (size_t)nb * (M + 1);
    const double* GG = G + 2 * (size_t)nb * gst;
    const double* SC = GG + 6 * (size_t)nb;
    const double* npairs = SC;
    const double* sumw = SC + nb;
    const double* sumwr = SC + 2 * nb;
    const double* sumwlogr = SC + 3 * nb;
    const double* sumww = SC + 4 * nb;
    const double* sumwwr = SC + 5 * nb;
    const double* sumwwlogr = SC + 6 * nb;
    // Stage G and W in shared memory.
    for (int q = threadIdx.x; q < 2 * nb * gst; q += MB) shG[q] = G[q];
    for (int q = threadIdx.x; q < 2 * nb * (M + 1); q += MB) shW[q] = W[q];
    __syncthreads();
    const double w1 = P.w[c1];
    const C2 wg1 = {(double)P.d1[c1], (double)P.d2[c1]};
    const C2 wg1c = conj2(wg1);
    auto Gv = [&](int k, int n) -> C2 {
        const double* p = shG + 2 * ((size_t)k * gst + (M + 1) + n);
        return {p[0], p[1]};
    };
    auto Wv = [&](int k, int n) -> C2 {
        const double* p = shW + 2 * ((size_t)k * (M + 1) + (n >= 0 ? n : -n));
        return n >= 0 ? C2{p[0], p[1]} : C2{p[0], -p[1]};
    };
    if (!P.quick) {
        const double n1 = P.n[c1];
        const int rows = mk - ks;
        for (int t = threadIdx.x; t < rows * nb; t += MB) {
            const int k2 = ks + t / nb, k3 = t % nb;
            if (k3 < k2) continue;
            const int i23 = (k2 * nb + k3) * nn + M;
            if (k3 == k2) {
                out[14 * Z + i23] += n1 * npairs[k2] * (npairs[k2] - 1);
                double md = w1 * (sumw[k2] * sumwr[k2] - sumwwr[k2]);
                double ml = w1 * (sumw[k2] * sumwlogr[k2] - sumwwlogr[k2]);
                out[8 * Z + i23] += md; out[9 * Z + i23] += ml;
                out[10 * Z + i23] += md; out[11 * Z + i23] += ml;
            } else {
                const int i32 = (k3 * nb + k2) * nn + M;
                double nnn = n1 * npairs[k2] * npairs[k3];
                out[14 * Z + i23] += nnn; out[14 * Z + i32] += nnn;
                double ww12 = w1 * sumw[k2], ww13 = w1 * sumw[k3];
                out[8 * Z + i23] += ww13 * sumwr[k2];  out[10 * Z + i32] += ww13 * sumwr[k2];
                out[9 * Z + i23] += ww13 * sumwlogr[k2]; out[11 * Z + i32] += ww13 * sumwlogr[k2];
                out[10 * Z + i23] += ww12 * sumwr[k3]; out[8 * Z + i32] += ww12 * sumwr[k3];
                out[11 * Z + i23] += ww12 * sumwlogr[k3]; out[9 * Z + i32] += ww12 * sumwlogr[k3];
            }
        }
    }
    // Entries (a, b, n) with min(a, b) in [ks, mk).
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
        const bool diag = (a == b);
        // weight (Porth et al. eq. 27)
        if (diag) {
            C2 wv = Wv(a, n);
            out[12 * Z + i] += w1 * ((wv.re * wv.re + wv.im * wv.im) - sumww[a]);
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
        if (diag) {
            C2 c0 = {GG[2 * a], GG[2 * a + 1]};
            C2 c1v = {GG[2 * nb + 2 * a], GG[2 * nb + 2 * a + 1]};
            C2 c2v = {GG[4 * nb + 2 * a], GG[4 * nb + 2 * a + 1]};
            C2 t0 = cmul(wg1, c0), t1 = cmul(wg1c, c1v), t2 = cmul(wg1, c2v);
            g0.re -= t0.re; g0.im -= t0.im;
            g1.re -= t1.re; g1.im -= t1.im;
            g2.re -= t2.re; g2.im -= t2.im;
            g3.re -= t2.re; g3.im -= t2.im;
        }
        out[0 * Z + i] += g0.re; out[1 * Z + i] += g0.im;
        out[2 * Z + i] += g1.re; out[3 * Z + i] += g1.im;
        out[4 * Z + i] += g2.re; out[5 * Z + i] += g2.im;
        out[6 * Z + i] += g3.re; out[7 * Z + i] += g3.im;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(MB) k_mp_finish(MPParams P)
{
    extern __shared__ __align__(16) double mp_sh[];
    __shared__ P2Entry stk[MSTACK];
    __shared__ int sp, free_cnt, free_list[64], scan_sh[MW];
    __shared__ P2Entry cur;
    __shared__ unsigned long long job_sh;
    __shared__ int acc_n, new_n, anysplit, alloc_ok;
    __shared__ double maxr_sh[MW];
    __shared__ long long arena_top;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int blk = blockIdx.x;
    const int nb = P.nbins, M = P.maxn;
    const int gst = 2 * M + 3;
    double* shG = mp_sh;
    double* shW = mp_sh + 2 * (size_t)nb * gst;
    int* arena = P.arena2 + (size_t)blk * P.arena2_cap;
    // Accepted records of the current pass: c2, k (ints) and r, logr (doubles).
    int* acc_c2 = P.acc_i + (size_t)blk * 2 * P.acc_cap;
    double* acc_r = P.acc_d + (size_t)blk * 2 * P.acc_cap;
    double* out = P.out + (size_t)blk * P.out_stride;
    const int* arena1 = P.arena1;

    while (true) {
        if (tid == 0) {
            job_sh = atomicAdd(P.job_next, 1ull);
            // After an error the results are discarded and the call is retried: stop early.
            if (*(volatile int*)P.err) job_sh = (unsigned long long)P.njobs_val;
        }
        __syncthreads();
        const unsigned long long job = job_sh;
        if ((long long)job >= P.njobs_val) break;
        const int4 J = P.jobs[job];
        if (tid == 0) {
            free_cnt = P.nslots;
            for (int s = 0; s < P.nslots; ++s) free_list[s] = P.nslots - 1 - s;
            arena_top = 0;
            sp = 0;
            int s0 = free_list[--free_cnt];
            P2Entry e;
            e.c1 = J.x; e.len = J.w; e.slot = s0; e.mink = nb;
            e.goff = (long long)J.y * P.arena1_cap + J.z; e.maxr = 0.;
            e.mark = 0;
            stk[sp++] = e;
        }
        __syncthreads();
        int guard = 0;
        {
            double* S0 = slot_ptr(P, blk, stk[0].slot);
            for (int q = tid; q < P.slot_doubles; q += MB) S0[q] = 0.;
        }
        __syncthreads();
        while (true) {
            __syncthreads();
            if (sp == 0) break;
            if (tid == 0) {
                cur = stk[--sp];
                arena_top = cur.mark;   // the finished left subtree's lists are dead
            }
            __syncthreads();
            // multipoleFinish loop on cur (c1 changes to its left child, the list to the new
            // list, the slot stays).
            while (true) {
                if (++guard > (1 << 24)) {   // last-resort bound; the recursion is finite
                    if (tid == 0) set_mp_err(P.err, MP_ERR_STACK);
                    break;
                }
                const int c1 = cur.c1;
                const double s1 = P.size[c1];
                const double thresh1 = (1. - P.binsize) * cur.maxr;   // oneBinLessThan
                const int* list = (cur.goff >= 0) ? (arena1 + cur.goff) : nullptr;
                const int* list2 = (cur.goff < 0) ? (arena + (-cur.goff - 1)) : nullptr;
                const long long nbase = arena_top;
                if (tid == 0) { acc_n = 0; new_n = 0; anysplit = 0; }
                double mymax = 0.;
                int myany = 0;
                __syncthreads();
                for (int j0 = 0; j0 < cur.len; j0 += MB) {
                    const int j = j0 + tid;
                    int cnt = 0, ca = -1, cb = -1, acc = 0, kacc = -1;
                    double racc = 0., lracc = 0.;
                    if (j < cur.len) {
                        const int c2 = list ? list[j] : list2[j];
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
                                    if (k >= nb) k = nb - 1;
                                    acc = 1; kacc = k; racc = r; lracc = lr;
                                    ca = c2;
                                }
                            } else {
                                mymax = fmax(mymax, r + s);
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
                    int tot_new, tot_acc;
                    int pos = block_excl_scan(cnt, scan_sh, tot_new);
                    int apos = block_excl_scan(acc, scan_sh, tot_acc);
                    const long long wbase = nbase + new_n;
                    if (wbase + tot_new > P.arena2_cap || acc_n + tot_acc > P.acc_cap) {
                        if (tid == 0) set_mp_err(P.err, MP_ERR_ARENA);
                    } else {
                        if (cnt >= 1) arena[wbase + pos] = ca;
                        if (cnt == 2) arena[wbase + pos + 1] = cb;
                        if (acc) {
                            const int a = acc_n + apos;
                            acc_c2[2 * a] = ca;
                            acc_c2[2 * a + 1] = kacc;
                            acc_r[2 * a] = racc;
                            acc_r[2 * a + 1] = lracc;
                        }
                    }
                    __syncthreads();
                    if (tid == 0) { new_n += tot_new; acc_n += tot_acc; }
                    __syncthreads();
                }
                // An overflow of the arenas leaves the lists incomplete: stop this job (the
                // call is retried with larger arenas).
                if (tid == 0) alloc_ok = (*(volatile int*)P.err) ? 0 : 1;
                __syncthreads();
                if (!alloc_ok) break;
                // Block max of the remaining separations and OR of anysplit1.
                for (int o = 16; o > 0; o >>= 1) {
                    mymax = fmax(mymax, __shfl_xor_sync(0xffffffffu, mymax, o));
                    myany |= __shfl_xor_sync(0xffffffffu, myany, o);
                }
                if (lane == 0) { maxr_sh[wid] = mymax; if (myany) atomicOr(&anysplit, 1); }
                __syncthreads();
                double maxrem = 0.;
                for (int k = 0; k < MW; ++k) maxrem = fmax(maxrem, maxr_sh[k]);
                const int n_acc = acc_n < P.acc_cap ? acc_n : P.acc_cap;
                const int n_new = new_n;
                // G_n / W_n accumulation: warp w owns the bins k with k % MW == w.
                double* S = slot_ptr(P, blk, cur.slot);
                {
                    double* W = S;
                    double* G = S + 2 * (size_t)nb * (M + 1);
                    double* GG = G + 2 * (size_t)nb * gst;
                    double* SC = GG + 6 * (size_t)nb;
                    for (int a = 0; a < n_acc; ++a) {
                        const int k = acc_c2[2 * a + 1];
                        if (k % MW != wid) continue;
                        const int c2 = acc_c2[2 * a];
                        const double r = acc_r[2 * a], lr = acc_r[2 * a + 1];
                        const double w2 = P.w[c2];
                        C2 z, e;
                        phases(P, c1, c2, r, z, e);
                        const C2 wz = {(double)P.d1[c2], (double)P.d2[c2]};
                        const C2 wg = cmul(wz, e);
                        if (lane == 0) {
                            const double* ls = P.ls + 4 * (size_t)c2;
                            SC[k] += (double)P.n[c2];
                            SC[nb + k] += w2;
                            SC[2 * nb + k] += w2 * r;
                            SC[3 * nb + k] += w2 * lr;
                            SC[4 * nb + k] += ls[0];
                            SC[5 * nb + k] += ls[0] * r;
                            SC[6 * nb + k] += ls[0] * lr;
                            const C2 wgsq = cmul({ls[1], ls[2]}, cmul(e, e));
                            const C2 zsq = cmul(z, z);
                            const C2 a0 = cmul(wgsq, conj2(zsq)), a1 = cmul(wgsq, zsq);
                            const C2 a2 = {ls[3] * zsq.re, -ls[3] * zsq.im};
                            GG[2 * k] += a0.re; GG[2 * k + 1] += a0.im;
                            GG[2 * nb + 2 * k] += a1.re; GG[2 * nb + 2 * k + 1] += a1.im;
                            GG[4 * nb + 2 * k] += a2.re; GG[4 * nb + 2 * k + 1] += a2.im;
                            W[2 * (size_t)k * (M + 1)] += w2;
                            double* g0 = G + 2 * ((size_t)k * gst + (M + 1));
                            g0[0] += wg.re; g0[1] += wg.im;
                        }
                        // z^(lane+1) by a multiplicative warp scan; chunks of 32 powers.
                        C2 p = z;
                        for (int o = 1; o < 32; o <<= 1) {
                            C2 q = {__shfl_up_sync(0xffffffffu, p.re, o), __shfl_up_sync(0xffffffffu, p.im, o)};
                            if (lane >= o) p = cmul(q, p);
                        }
                        const C2 z32 = {__shfl_sync(0xffffffffu, p.re, 31), __shfl_sync(0xffffffffu, p.im, 31)};
                        C2 base_pow = {1., 0.};
                        for (int c = 0; 32 * c < M + 1; ++c) {
                            const C2 pw = cmul(base_pow, p);     // z^(32c + lane + 1)
                            const int n = 32 * c + lane + 1;
                            if (n <= M) {
                                double* wp = W + 2 * ((size_t)k * (M + 1) + n);
                                wp[0] += w2 * pw.re; wp[1] += w2 * pw.im;
                            }
                            if (n <= M + 1) {
                                const C2 gp = cmul(wg, pw), gm = cmul(wg, conj2(pw));
                                double* gpp = G + 2 * ((size_t)k * gst + (M + 1) + n);
                                double* gmp = G + 2 * ((size_t)k * gst + (M + 1) - n);
                                gpp[0] += gp.re; gpp[1] += gp.im;
                                gmp[0] += gm.re; gmp[1] += gm.im;
                            }
                            base_pow = cmul(base_pow, z32);
                        }
                    }
                }
                __syncthreads();
                int mink = cur.mink;
                if (n_new == 0) {
                    zeta_rows(P, c1, S, 0, mink, out, shG, shW);
                    break;
                }
                if (maxrem < P.maxsep) {
                    int k = maxrem < P.minsep ? 0
                          : int((log(maxrem) - P.logminsep) / P.binsize) + 1;
                    if (k < mink) {
                        zeta_rows(P, c1, S, k, mink, out, shG, shW);
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
                            rgt.mink = mink; rgt.goff = -nbase - 1; rgt.maxr = maxrem;
                            rgt.mark = nbase + n_new;
                            stk[sp++] = rgt;
                        }
                    }
                }
                __syncthreads();
                if (!alloc_ok) break;
                if (split1) {
                    // The right child gets a copy of the scratch (mp.duplicate()).
                    const double* src = slot_ptr(P, blk, cur.slot);
                    double* dst = slot_ptr(P, blk, stk[sp - 1].slot);
                    for (int q = tid; q < P.slot_doubles; q += MB) dst[q] = src[q];
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
                        if (i < n_new) v = arena[nbase + i];
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
                    cur.maxr = maxrem;
                    arena_top = newoff + n_new;
                }
                __syncthreads();
            }
            __syncthreads();
            if (tid == 0) free_list[free_cnt++] = cur.slot;
            __syncthreads();
        }
    }
}

// Sum of the per-block output copies, in block order.
__global__ void k_mp_reduce(int nblk, long long stride, long long total, const double* in,
                            double* out)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    double s = 0.;
    for (int b = 0; b < nblk; ++b) s += in[(size_t)b * stride + i];
    out[i] = s;
}

// ---------------------------------------------------------------------------------------
// Host orchestration.

size_t mp_slot_doubles(int nb, int M)
{ return 2 * (size_t)nb * (M + 1) + 2 * (size_t)nb * (2 * M + 3) + 13 * (size_t)nb; }

int run_multipole(MPParams& P, MPScratch& X, int ntop, cudaStream_t st, double* h_out)
{
    const int nb = P.nbins, M = P.maxn;
    const long long Z = (long long)nb * nb * (2 * M + 1);
    int dev = 0, nsm = 0;
    TC_CU(cudaGetDevice(&dev));
    TC_CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const size_t shbytes = sizeof(double) * (2 * (size_t)nb * (2 * M + 3) + 2 * (size_t)nb * (M + 1));
    if (shbytes > 200 * 1024) {
        set_last_error("nbins * max_n too large for the multipole shared-memory staging");
        return 3;
    }
    TC_CU(cudaFuncSetAttribute(k_mp_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shbytes));
    int per = 0;
    TC_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mp_finish, MB, shbytes));
    if (per < 1) per = 1;
    const int nblk = nsm * std::min(per, 2);
    P.slot_doubles = (long long)mp_slot_doubles(nb, M);
    P.out_stride = 15 * Z;
    X.want_a1 = std::max<long long>(X.want_a1, 4LL * ntop + (1 << 16));
    X.want_jobs = std::max<long long>(X.want_jobs, 1 << 18);
    X.want_a2 = std::max<long long>(X.want_a2, 1 << 20);
    X.want_acc = std::max<long long>(X.want_acc, 1 << 16);
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
        if (X.acc_cap < X.want_acc || grow_blk) {
            dfree(X.acc_i); dfree(X.acc_d);
            X.acc_cap = 0;
            TC_TRY(dalloc(&X.acc_i, (size_t)2 * X.want_acc * nblk));
            TC_TRY(dalloc(&X.acc_d, (size_t)2 * X.want_acc * nblk));
            X.acc_cap = X.want_acc;
        }
        if (X.nslots < X.want_slots || grow_blk || P.slot_doubles != X.slot_doubles) {
            dfree(X.slots);
            X.nslots = 0;
            TC_TRY(dalloc(&X.slots, (size_t)X.want_slots * P.slot_doubles * nblk));
            X.nslots = X.want_slots; X.slot_doubles = P.slot_doubles;
        }
        if (grow_blk || P.out_stride > X.out_stride) {
            dfree(X.out); dfree(X.total);
            X.out_stride = 0;
            TC_TRY(dalloc(&X.out, (size_t)P.out_stride * nblk));
            TC_TRY(dalloc(&X.total, (size_t)P.out_stride));
            X.out_stride = P.out_stride;
        }
        if (!X.ctl) TC_TRY(dalloc(&X.ctl, 4));
        if (!X.err) TC_TRY(dalloc(&X.err, 1));
        X.nblk = std::max(X.nblk, nblk);
        P.arena1 = X.arena1; P.arena1_cap = X.arena1_cap;
        P.jobs = X.jobs; P.jobs_cap = X.jobs_cap;
        P.njobs = X.ctl; P.job_next = X.ctl + 1;
        P.arena2 = X.arena2; P.arena2_cap = X.arena2_cap;
        P.acc_i = X.acc_i; P.acc_d = X.acc_d; P.acc_cap = (int)X.acc_cap;
        P.slots = X.slots; P.nslots = X.nslots;
        P.out = X.out;
        P.err = X.err;
        TC_CU(cudaMemsetAsync(X.ctl, 0, 4 * sizeof(unsigned long long), st));
        TC_CU(cudaMemsetAsync(X.err, 0, sizeof(int), st));
        TC_CU(cudaMemsetAsync(X.out, 0, sizeof(double) * (size_t)P.out_stride * nblk, st));
        count_launch();
        k_mp_split1<<<ntop, MB, 0, st>>>(P);
        TC_CU(cudaGetLastError());
        unsigned long long nj = 0;
        int e = 0;
        TC_CU(cudaMemcpyAsync(&nj, X.ctl, sizeof(nj), cudaMemcpyDeviceToHost, st));
        TC_CU(cudaMemcpyAsync(&e, X.err, sizeof(int), cudaMemcpyDeviceToHost, st));
        TC_CU(cudaStreamSynchronize(st));
        if (e == 0) {
            P.njobs_val = (long long)nj;
            count_launch();
            k_mp_finish<<<nblk, MB, shbytes, st>>>(P);
            TC_CU(cudaGetLastError());
            TC_CU(cudaMemcpyAsync(&e, X.err, sizeof(int), cudaMemcpyDeviceToHost, st));
            TC_CU(cudaStreamSynchronize(st));
        }
        if (e == MP_ERR_ARENA || e == MP_ERR_JOBS || e == MP_ERR_SLOTS) {
            X.want_a1 = X.arena1_cap * 4; X.want_jobs = X.jobs_cap * 4;
            X.want_a2 = X.arena2_cap * 4; X.want_acc = X.acc_cap * 4;
            X.want_slots = std::min(X.nslots * 2, 64);
            continue;
        }
        if (e) {
            set_last_error("multipole: device stack overflow (tree too deep)");
            return 4;
        }
        count_launch();
        k_mp_reduce<<<(unsigned)((P.out_stride + 255) / 256), 256, 0, st>>>(
            nblk, P.out_stride, P.out_stride, X.out, X.total);
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
    dfree(X.arena1); dfree(X.jobs); dfree(X.arena2); dfree(X.acc_i); dfree(X.acc_d);
    dfree(X.slots); dfree(X.out); dfree(X.total); dfree(X.ctl); dfree(X.err);
    X = MPScratch();
}

}  // namespace tc
