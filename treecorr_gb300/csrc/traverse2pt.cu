// traverse2pt.cu -- dual-tree 2-point traversal and per-pair accumulation on sm_103a.
//
// Semantics follow the reference exactly:
//   BaseCorr2::process (auto src/Corr2.cpp:146-205, cross 207-288), process2 (290-306),
//   process11 (308-389), directProcess11 (476-525), finishProcess + DirectHelper (394-566),
//   BinTypeHelper<Log> (include/BinType.h:40-156), CalcSplitSq (include/Split.h:82-101),
//   MetricHelper<Euclidean> / <Arc> (include/Metric.h:119-258, 658-700) and the spin-2
//   projections (include/ProjectHelper.h:45-47, 84-136, 272-388).
//
// GB300 design:
//   * Work items are cell pairs (plus "self" items for process2).  A persistent grid of
//     warps takes 32 items at a time; each lane evaluates one item and pushes 0, 2, 3 or 4
//     children onto its warp's stack (LIFO, so the warp walks depth first and the stack
//     stays shallow).  Roots are the top-level pairs, generated on the fly from a counter.
//   * Decisions are taken in FP32 on cells stored as float hi/lo positions (differences of
//     nearby cells keep ~48 bits).  Every comparison carries an error bound; when a value
//     falls inside it, the whole decision for that pair is redone in FP64 from the FP64
//     centres with the reference's formulas.  So accept/split/bin choices are the
//     reference's, while almost all work runs at FP32 rate (GB300's FP64 rate is ~1/64).
//   * Accepted pairs are accumulated into per-warp FP32 shared-memory bins that are flushed
//     every few iterations into per-warp FP64 totals; npairs is an exact 64-bit integer.
//   * When the roots run out and many warps are idle, warps with deep stacks spill them to
//     a global list that the next launch redistributes (no inter-warp waiting anywhere).
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <vector>

#include "tc_internal.cuh"
#include "tc_host.hpp"
#include "traverse2pt.hpp"
#include "pair_math.cuh"
#include "learned.cuh"

namespace tc {

static constexpr int TB = 128;        // threads per traversal block
static constexpr int WPB = TB / 32;   // warps per block
static constexpr int FLUSH = 8;       // iterations between flushes of the FP32 bins

// ---------------------------------------------------------------------------------------
// Packing of the traversal records.

__global__ void k_pack_cells(int ncap, Cells C, TCell* out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncap) return;
    double x = C.x[i], y = C.y[i], z = C.z[i];
    float xh = float(x), yh = float(y), zh = float(z);
    TCell t;
    t.a = make_float4(xh, yh, zh, C.size[i]);
    t.b = make_float4(float(x - double(xh)), float(y - double(yh)), float(z - double(zh)), C.w[i]);
    t.c = make_float4(C.d1[i], C.d2[i], __int_as_float(C.n[i]), __int_as_float(C.left[i]));
    t.d = make_float4(__int_as_float(C.right[i]), 0.f, __int_as_float(C.start[i]), 0.f);
    out[i] = t;
}

void launch_pack_cells(int ncap, const Cells& C, TCell* out, cudaStream_t st)
{
    if (ncap <= 0) return;
    count_launch(); k_pack_cells<<<(ncap + 255) / 256, 256, 0, st>>>(ncap, C, out);
}

// ---------------------------------------------------------------------------------------
// Tri-state comparisons.  A value v known up to [lo, hi].

enum : int { NO = 0, YES = 1, UNSURE = 2 };

// Is a > b, given a in [alo, ahi] and b in [blo, bhi]?
__device__ __forceinline__ int gt3(float alo, float ahi, float blo, float bhi)
{ return alo > bhi ? YES : (ahi <= blo ? NO : UNSURE); }

// Square of an interval.
__device__ __forceinline__ void sq_iv(float lo, float hi, float& slo, float& shi)
{
    if (lo >= 0.f) { slo = lo * lo; shi = hi * hi; }
    else if (hi <= 0.f) { slo = hi * hi; shi = lo * lo; }
    else { slo = 0.f; shi = fmaxf(lo * lo, hi * hi); }
}

// Slack added to every bound to cover the FP32 rounding of the bound itself.
__device__ __forceinline__ float LOW(float v) { return v - fabsf(v) * 2e-6f - 1e-30f; }
__device__ __forceinline__ float HIGH(float v) { return v + fabsf(v) * 2e-6f + 1e-30f; }

// FP32 decision of process11 for one cell pair; ACT_UNSURE when any comparison is within
// its error bound.
__device__ __forceinline__ Decision decide32(const TravParams& T, float rsq, float s1, float s2,
                                             bool arc)
{
    Decision D;
    D.act = ACT_UNSURE; D.k = -1; D.r = 0.f; D.logr = 0.f;
    // Error bounds: rsq (relative), s1+s2 (relative).
    const float ER = arc ? 5e-6f : 2e-6f;
    const float ES = 1e-6f;
    const float Rlo = rsq * (1.f - ER), Rhi = rsq * (1.f + ER);
    const float s1ps2 = s1 + s2;
    const float Slo = s1ps2 * (1.f - ES), Shi = s1ps2 * (1.f + ES);

    // tooSmallDist, include/BinType.h:70-76 (the first clause decides most pairs).
    const int below = gt3(T.fminsepsq * (1.f - 1e-7f), T.fminsepsq * (1.f + 1e-7f), Rlo, Rhi);
    if (below != NO) {
        int c2 = gt3(T.fminsep, T.fminsep, Slo, Shi);                                    // s1ps2 < minsep
        float xlo = T.fminsep - Shi, xhi = T.fminsep - Slo, x2lo, x2hi;
        sq_iv(xlo, xhi, x2lo, x2hi);
        int c3 = gt3(LOW(x2lo), HIGH(x2hi), Rlo, Rhi);                                  // rsq < (minsep-s)^2
        if (below == YES && c2 == YES && c3 == YES) { D.act = ACT_DROP; return D; }
        if (!(c2 == NO || c3 == NO)) return D;
    }
    // tooLargeDist, include/BinType.h:77-82: rsq >= maxsepsq  <=>  !(maxsepsq > rsq).
    const int inside = gt3(T.fmaxsepsq * (1.f - 1e-7f), T.fmaxsepsq * (1.f + 1e-7f), Rlo, Rhi);
    if (inside != YES) {
        float ylo = T.fmaxsep + Slo, yhi = T.fmaxsep + Shi;
        float y2lo = LOW(ylo * ylo), y2hi = HIGH(yhi * yhi);
        int lt2 = gt3(y2lo, y2hi, Rlo, Rhi);   // (maxsep+s)^2 > rsq
        if (inside == NO && lt2 == NO) { D.act = ACT_DROP; return D; }
        if (lt2 != YES) return D;
    }
    // singleBin, include/BinType.h:93-151.
    int sb = UNSURE;
    int k = -1;
    float lr = 0.f;   // log(r/minsep), set once it is needed
    if (s1ps2 == 0.f) {
        sb = YES;
    } else {
        const float S2lo = LOW(Slo * Slo), S2hi = HIGH(Shi * Shi);
        int t1 = gt3(S2lo, S2hi, LOW(T.fasq * Rlo), HIGH(T.fasq * Rhi));
        if (t1 == UNSURE) return D;
        if (t1 == YES) sb = NO;
        else {
            int t2 = gt3(S2lo, S2hi, LOW(T.fbsq * Rlo), HIGH(T.fbsq * Rhi));   // > bsq*rsq
            if (t2 == UNSURE) return D;
            if (t2 == NO) sb = YES;
            else {
                int t3 = gt3(S2lo, S2hi, LOW(T.fbb * Rlo), HIGH(T.fbb * Rhi));
                if (t3 == UNSURE) return D;
                if (t3 == YES) sb = NO;
                else {
                    lr = 0.5f * logf(rsq * T.finvminsepsq);
                    float kk = lr * T.finvbinsize;
                    float ek = (0.5f * ER + 3e-7f * (1.f + fabsf(lr))) * T.finvbinsize + 1e-6f;
                    float klo = kk - ek, khi = kk + ek;
                    // int(kk) truncates toward zero, as in the reference (kk < 0 is possible).
                    float ik = truncf(kk);
                    if (truncf(klo) != ik || truncf(khi) != ik) return D;
                    float flo = klo - ik, fhi = khi - ik;
                    float mlo = fminf(flo, 1.f - fhi), mhi = fminf(fhi, 1.f - flo);
                    float alo = mlo * T.fbinsize + T.fb, ahi = mhi * T.fbinsize + T.fb;
                    float a2lo, a2hi;
                    sq_iv(alo, ahi, a2lo, a2hi);
                    int t4 = gt3(S2lo, S2hi, LOW(a2lo * Rlo), HIGH(a2hi * Rhi));
                    if (t4 == UNSURE) return D;
                    if (t4 == YES) sb = NO;
                    else {
                        float zlo = flo * T.fbinsize + T.fb - S2hi / Rlo;
                        float zhi = fhi * T.fbinsize + T.fb - S2lo / Rhi;
                        float z2lo, z2hi;
                        sq_iv(LOW(zlo) - 1e-7f, HIGH(zhi) + 1e-7f, z2lo, z2hi);
                        int t5 = gt3(S2lo, S2hi, LOW(z2lo * Rlo), HIGH(z2hi * Rhi));
                        if (t5 == UNSURE) return D;
                        if (t5 == YES) sb = NO;
                        else { sb = YES; k = int(ik); }
                    }
                }
            }
        }
    }
    if (sb == YES) {
        // isRSqInRange, include/BinType.h:61-66: minsepsq <= rsq < maxsepsq.
        if (below == UNSURE || inside == UNSURE) return D;
        if (below == YES || inside == NO) { D.act = ACT_DROP; return D; }
        float r = arc ? 0.f : sqrtf(rsq);
        if (k < 0) lr = 0.5f * logf(rsq * T.finvminsepsq);
        if (k < 0) {
            // directProcess11, src/Corr2.cpp:492-514.
            float kk = lr * T.finvbinsize;
            float ek = (0.5f * ER + 3e-7f * (1.f + fabsf(lr))) * T.finvbinsize + 1e-6f;
            float ik = truncf(kk);
            if (truncf(kk - ek) != ik || truncf(kk + ek) != ik) return D;
            k = int(ik);
        }
        if (k == T.nbins) k = T.nbins - 1;
        if (k < 0 || k >= T.nbins) return D;
        D.act = ACT_ACCEPT;
        D.k = k;
        D.r = r;
        D.logr = lr + T.flogminsep;
        return D;
    }
    // CalcSplitSq with bsq_eff = rsq*min(bsq,asq), include/Split.h:82-101 and
    // getEffectiveBSq, include/BinType.h:50-51.
    bool sw = s2 > s1;
    float big = sw ? s2 : s1, sml = sw ? s1 : s2;
    int which;
    if (big > 2.f * sml) {
        which = 1;
    } else {
        float m2lo = LOW(sml * sml), m2hi = HIGH(sml * sml);
        int t = gt3(m2lo, m2hi, LOW(0.3422f * T.fmineff * Rlo), HIGH(0.3422f * T.fmineff * Rhi));
        if (t == UNSURE) return D;
        which = (t == YES) ? 2 : 1;
    }
    D.act = which == 2 ? ACT_SPLIT12 : (sw ? ACT_SPLIT2 : ACT_SPLIT1);
    return D;
}

// ---------------------------------------------------------------------------------------
// Root generation.

// Row i of the upper triangle (self + pairs j > i) of n top cells starts at
// i*n - i*(i-1)/2; item g of that enumeration.
__device__ __forceinline__ void tri_index(long long n, long long g, long long& i, long long& j)
{
    double b = 2.0 * n + 1.0;
    i = (long long)((b - sqrt(b * b - 8.0 * (double)g)) * 0.5);
    if (i < 0) i = 0;
    if (i > n - 1) i = n - 1;
    while (i > 0 && i * n - i * (i - 1) / 2 > g) --i;
    while (i + 1 < n && (i + 1) * n - (i + 1) * i / 2 <= g) ++i;
    j = g - (i * n - i * (i - 1) / 2) + i;
}

// Patches: root g of all patch pairs (auto enumeration within a patch, all top pairs
// across two patches).
__device__ __forceinline__ int2 make_patch_root(const TravParams& T, long long g)
{
    int lo = 0, hi = T.npair;          // proot_off[lo] <= g < proot_off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (T.proot_off[mid] <= g) lo = mid; else hi = mid;
    }
    const int2 pr = T.ppairs[lo];
    const long long r = g - T.proot_off[lo];
    const int* ti = T.ptop + T.ptop_off[pr.x];
    if (pr.x == pr.y) {
        const long long n = T.ptop_off[pr.x + 1] - T.ptop_off[pr.x];
        long long i, j;
        tri_index(n, r, i, j);
        return j == i ? make_int2(ti[i], -1) : make_int2(ti[i], ti[j]);
    }
    const int* tj = T.ptop + T.ptop_off[pr.y];
    const long long nj = T.ptop_off[pr.y + 1] - T.ptop_off[pr.y];
    return make_int2(ti[r / nj], tj[r % nj]);
}

template <int MODE = 0>
__device__ __forceinline__ int2 make_root(const TravParams& T, long long g)
{
    if constexpr (MODE == 3) return make_patch_root(T, g);
    if (g >= T.ngen) return T.in_tasks[g - T.ngen];
    if (T.autoc) {
        // Row i of the upper triangle (self + pairs j>i) starts at i*n - i*(i-1)/2.
        long long n = T.ntop1;
        double b = 2.0 * n + 1.0;
        long long i = (long long)((b - sqrt(b * b - 8.0 * (double)g)) * 0.5);
        if (i < 0) i = 0;
        if (i > n - 1) i = n - 1;
        while (i > 0 && i * n - i * (i - 1) / 2 > g) --i;
        while (i + 1 < n && (i + 1) * n - (i + 1) * i / 2 <= g) ++i;
        long long j = g - (i * n - i * (i - 1) / 2) + i;
        if (j == i) return make_int2(T.tops1[i], -1);
        return make_int2(T.tops1[i], T.tops1[j]);
    }
    long long i = g / T.ntop2, j = g - i * T.ntop2;
    return make_int2(T.tops1[i], T.tops2[j]);
}

// ---------------------------------------------------------------------------------------
// The traversal kernel.

// FP32 bins (4 segment copies) -> the warp's double-float totals, all in shared memory.
__device__ __forceinline__ void flush_bins(int nqnb, float* fb, float2* fd, int lane)
{
    for (int q = lane; q < nqnb; q += 32) {
        float a = fb[q], b = fb[nqnb + q], c = fb[2 * nqnb + q], d = fb[3 * nqnb + q];
        if (a != 0.f || b != 0.f || c != 0.f || d != 0.f) {
            float2 f = fd[q];
            df_add(f, a); df_add(f, b); df_add(f, c); df_add(f, d);
            const float t = f.x + f.y;          // renormalise (|lo| <= ulp(hi) / 2)
            f.y -= t - f.x;
            f.x = t;
            fd[q] = f;
            fb[q] = 0.f; fb[nqnb + q] = 0.f; fb[2 * nqnb + q] = 0.f; fb[3 * nqnb + q] = 0.f;
        }
    }
}

// Adds the accepted pairs of this iteration to the warp's bins.  Each lane stages (7 values,
// k) in shared memory; then the warp works as 4 segments of 8 lanes: lane q < 7 of a segment
// owns quantity q and adds the segment's 8 staged entries, in order, to its segment's copy
// of the bins -- one read-modify-write per entry, the same instructions on every lane (an
// entry without a pair adds 0 to bin 0), so the warp never diverges here.  The exact integer
// npairs goes in with one 64-bit shared atomic per accepting lane (copy lane & 3).
static constexpr int STG = 9;    // staged words per lane (odd stride: no bank conflicts)

__host__ __device__ inline size_t traverse_warp_bytes(int nq, int nb)
{
    size_t b = (size_t)nq * nb * 8 + (size_t)4 * nb * 8 + (size_t)4 * nq * nb * 4 +
               (size_t)32 * STG * 4;
    return (b + 15) & ~(size_t)15;
}

__device__ __forceinline__ void stage_accumulate(int k, const float (&v)[7],
                                                 unsigned long long nn, int nq, bool quick,
                                                 float* stage, float* fb, unsigned long long* np,
                                                 int nb, int lane)
{
    if (!quick && k >= 0) atomicAdd(np + (lane & 3) * nb + k, nn);
    float* my = stage + lane * STG;
#pragma unroll
    for (int q = 0; q < 7; ++q) my[q] = v[q];
    my[7] = __int_as_float(k);
    __syncwarp();
    const int seg = lane >> 3, q = lane & 7;
    if (q < nq) {
        float* fbs = fb + seg * nq * nb + q * nb;
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const float* e = stage + (seg * 8 + t) * STG;
            const int kj = __float_as_int(e[7]);
            const float x = kj >= 0 ? e[q] : 0.f;
            fbs[kj >= 0 ? kj : 0] += x;
        }
    }
    __syncwarp();
}

// One work item: process2 for a self item (task.y < 0), else process11 for a cell pair.
// Writes the children to ch (nch of them) and, for an accepted pair, its bin and values.
// MODE 1 samples the candidate pairs of the learned criterion; MODE 2 marks them (cand),
// returns their features and prepares both outcomes: the children and, in acc_k / av, the
// values of accepting the pair into the bin of its separation.  MODE 4 is the bin_slop rule
// of MODE 0 in exact mode: a pair it would split whose cells both hold at most tile_leaf
// points becomes a leaf-pair tile (tl) instead (a separate instantiation, so that MODE 0
// carries none of the tile code).
template <int MODE>
__device__ __forceinline__ void eval_task(const TravParams& T, bool has, int2 task,
                                          int2 (&ch)[4], int& nch, int2& tl, int& acc_k,
                                          float (&av)[7],
                                          unsigned long long& acc_nn, long long& n_eval,
                                          long long& n_acc, long long& n_esc, bool& cand,
                                          float (&feat)[MLP_IN])
{
    const bool arc = (T.metric == ARC);
    const bool flat = (T.coords == FLAT);
    if (has) {
        ++n_eval;
        const int i = task.x;
        if (task.y < 0) {
            // process2, src/Corr2.cpp:290-306.
            const TCell A = T.c1[i];
            const float w = A.b.w, s = A.a.w;
            if (w != 0.f && !((double)s <= T.halfminsep)) {
                int L = __float_as_int(A.c.w), R = __float_as_int(A.d.x);
                if (MODE == 4 && __float_as_int(A.c.z) <= T.tile_leaf) {
                    tl = make_int2(i, -2 - i);      // every leaf pair of this cell
                } else if (L < 0 || R < 0) {
                    atomicCAS(T.err, 0, DEV_BAD_CHILD);
                } else {
                    ch[0] = make_int2(L, -1); ch[1] = make_int2(R, -1); ch[2] = make_int2(L, R);
                    nch = 3;
                }
            }
        } else {
            const int j = task.y;
            const TCell A = T.c1[i];
            const TCell B = T.c2[j];
            if (A.b.w != 0.f && B.b.w != 0.f) {
                const float dx = (A.a.x - B.a.x) + (A.b.x - B.b.x);
                const float dy = (A.a.y - B.a.y) + (A.b.y - B.b.y);
                const float dz = flat ? 0.f : (A.a.z - B.a.z) + (A.b.z - B.b.z);
                const float dsq = dx * dx + dy * dy + dz * dz;
                float rsq = dsq, theta = 0.f;
                if (arc) {
                    theta = arc_from_chord_sq(dsq);
                    rsq = theta * theta;
                }
                const float s1 = A.a.w, s2 = B.a.w;
                Decision D = decide32(T, rsq, s1, s2, arc);
                if (D.act == ACT_UNSURE) {
                    ++n_esc;
                    double ddx = T.x1[i] - T.x2[j], ddy = T.y1[i] - T.y2[j];
                    double ddsq = ddx * ddx + ddy * ddy;
                    if (!flat) { double ddz = T.z1[i] - T.z2[j]; ddsq += ddz * ddz; }
                    D = decide64(T, ddsq, (double)s1, (double)s2);
                    if (D.act == ACT_ACCEPT && arc) theta = D.r;
                } else if (D.act == ACT_ACCEPT && arc) {
                    D.r = theta;
                }
                if (D.act == ACT_ACCEPT) {
                    ++n_acc;
                    acc_k = D.k;
                    accept_values(T, A, B, i, j, dx, dy, dz, dsq, D.r, D.logr, av, acc_nn);
                } else if (MODE == 4 && D.act != ACT_DROP &&
                           __float_as_int(A.c.z) <= T.tile_leaf &&
                           __float_as_int(B.c.z) <= T.tile_leaf) {
                    tl = make_int2(i, j);               // every leaf pair of the two cells
                } else if (D.act != ACT_DROP) {
                    const int L1 = __float_as_int(A.c.w), R1 = __float_as_int(A.d.x);
                    const int L2 = __float_as_int(B.c.w), R2 = __float_as_int(B.d.x);
                    if (D.act == ACT_SPLIT12) {
                        if (L1 < 0 || L2 < 0) atomicCAS(T.err, 0, DEV_BAD_CHILD);
                        else {
                            ch[0] = make_int2(L1, L2); ch[1] = make_int2(L1, R2);
                            ch[2] = make_int2(R1, L2); ch[3] = make_int2(R1, R2);
                            nch = 4;
                        }
                    } else if (D.act == ACT_SPLIT1) {
                        if (L1 < 0) atomicCAS(T.err, 0, DEV_BAD_CHILD);
                        else { ch[0] = make_int2(L1, j); ch[1] = make_int2(R1, j); nch = 2; }
                    } else {
                        if (L2 < 0) atomicCAS(T.err, 0, DEV_BAD_CHILD);
                        else { ch[0] = make_int2(i, L2); ch[1] = make_int2(i, R2); nch = 2; }
                    }
                    if constexpr (MODE == 1 || MODE == 2) {
                        const float S = s1 + s2, S2 = S * S;
                        if (nch > 0 && rsq >= T.fminsepsq && rsq < T.fmaxsepsq &&
                            S2 <= T.fasq * rsq && S2 <= T.cand_f2 * rsq) {
                            const float lr = 0.5f * logf(rsq * T.finvminsepsq);
                            int k = (int)(lr * T.finvbinsize);
                            if (k >= T.nbins) k = T.nbins - 1;
                            if (k >= 0) {
                                cand = true;
                                if constexpr (MODE == 1) {
                                    // A fixed hash of the pair picks ~1/sample_mod of the candidates.
                                    unsigned h = (unsigned)i * 0x9E3779B1u ^ ((unsigned)j * 0x85EBCA77u);
                                    h ^= h >> 15; h *= 0x2C1B3C6Du; h ^= h >> 12;
                                    if (h % T.sample_mod == 0) {
                                        const unsigned long long o = atomicAdd(T.nsamples, 1ull);
                                        if ((long long)o < T.sample_cap) T.samples[o] = make_int2(i, j);
                                    }
                                } else {
                                    const float r = arc ? theta : sqrtf(rsq);
                                    mlp_features(s1, s2, r, lr, T.finvbinsize, T.finvlogrange,
                                                 T.fbinsize, feat);
                                    acc_k = k;
                                    accept_values(T, A, B, i, j, dx, dy, dz, dsq, r,
                                                  lr + T.flogminsep, av, acc_nn);
                                }
                            }
                        }
                    }
                }
            }
        }
    }
}

__global__ void __launch_bounds__(TB) k_traverse(TravParams T)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int gw = blockIdx.x * WPB + wib;
    const int nq = T.nqf, nb = T.nbins;
    // Per-warp bins: nq*nb FP64 totals, 4 segment copies of the npairs (u64) and of the
    // nq*nb FP32 partials, and the 32-lane staging area.
    const size_t wbytes = traverse_warp_bytes(nq, nb);
    float2* fd = (float2*)(smem + wib * wbytes);
    unsigned long long* np = (unsigned long long*)(fd + nq * nb);
    float* fb = (float*)(np + 4 * nb);
    float* stage = fb + 4 * nq * nb;
    for (int q = lane; q < nq * nb; q += 32) fd[q] = make_float2(0.f, 0.f);
    for (int q = lane; q < 4 * nb; q += 32) np[q] = 0ull;
    for (int q = lane; q < 4 * nq * nb; q += 32) fb[q] = 0.f;
    __syncwarp();

    int2* stk = T.stacks + (size_t)gw * T.stack_cap;
    int sp = 0;
    bool roots_done = false;
    int iter = 0;
    long long n_eval = 0, n_acc = 0, n_esc = 0;
    const long long total_roots = T.ngen + T.nin;
    const bool arc = (T.metric == ARC);
    const bool flat = (T.coords == FLAT);

    while (true) {
        if (sp < 32 && !roots_done) {
            // Take up to 32 roots; fewer when the pool is small, so that the last items of
            // a launch are spread over many warps.
            unsigned long long base = 0;
            int want = 32;
            if (lane == 0) {
                long long cur = (long long)*(volatile unsigned long long*)T.root_next;
                long long per = (total_roots - cur) / T.nwarps;
                want = per >= 32 ? 32 : (per < 1 ? 1 : (int)per);
                base = atomicAdd(T.root_next, (unsigned long long)want);
            }
            base = __shfl_sync(0xffffffffu, base, 0);
            want = __shfl_sync(0xffffffffu, want, 0);
            if ((long long)base >= total_roots) {
                roots_done = true;
            } else {
                long long g = (long long)base + lane;
                bool ok = lane < want && g < total_roots;
                int2 t = ok ? make_root(T, g) : make_int2(0, 0);
                unsigned m = __ballot_sync(0xffffffffu, ok);
                if (ok) stk[sp + __popc(m & ((1u << lane) - 1u))] = t;
                sp += __popc(m);
                __syncwarp();
            }
        }
        if (sp == 0) {
            if (roots_done) break;
            continue;
        }
        if (roots_done && (iter & 3) == 0) {
            // Spill when many warps are idle, so the next launch can spread this stack.
            int idle = 0;
            if (lane == 0) idle = *(volatile int*)T.idle;
            idle = __shfl_sync(0xffffffffu, idle, 0);
            if (idle * 4 > T.nwarps) {
                unsigned long long o = 0;
                if (lane == 0) o = atomicAdd(T.nout, (unsigned long long)sp);
                o = __shfl_sync(0xffffffffu, o, 0);
                if ((long long)(o + sp) > T.out_cap) {
                    if (lane == 0) atomicCAS(T.err, 0, DEV_SPILL_OVERFLOW);
                } else {
                    for (int q = lane; q < sp; q += 32) T.out_tasks[o + q] = stk[q];
                }
                sp = 0;
                break;
            }
        }
        // Keep room for the children of 32 items: spill the bottom of a full stack.
        if (sp + 160 > T.stack_cap) {
            const int keep = 256;
            int mv = sp - keep;
            unsigned long long o = 0;
            if (lane == 0) o = atomicAdd(T.nout, (unsigned long long)mv);
            o = __shfl_sync(0xffffffffu, o, 0);
            if ((long long)(o + mv) > T.out_cap) {
                if (lane == 0) atomicCAS(T.err, 0, DEV_SPILL_OVERFLOW);
                break;
            }
            for (int q = lane; q < mv; q += 32) T.out_tasks[o + q] = stk[q];
            __syncwarp();
            for (int q = lane; q < keep; q += 32) {
                int2 v = stk[mv + q];
                __syncwarp();
                stk[q] = v;
            }
            sp = keep;
            __syncwarp();
        }
        if (iter >= (1 << 30)) {   // last-resort bound; a valid tree never gets here
            if (lane == 0) atomicCAS(T.err, 0, DEV_STACK_OVERFLOW);
            break;
        }
        const int nt = sp < 32 ? sp : 32;
        sp -= nt;
        int2 task = make_int2(0, 0);
        const bool has = lane < nt;
        if (has) task = stk[sp + lane];
        __syncwarp();
        ++iter;

        int nch = 0;
        int2 ch[4];
        int2 tl = make_int2(-1, 0);   // k_traverse runs without tiles (tile_leaf = 0)
        int acc_k = -1;
        float av[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        unsigned long long acc_nn = 0ull;
        bool cand = false;
        float feat[MLP_IN];
        eval_task<0>(T, has, task, ch, nch, tl, acc_k, av, acc_nn, n_eval, n_acc, n_esc, cand,
                     feat);
        // Accumulate this iteration's accepted pairs (warp-converged here).
        if (__any_sync(0xffffffffu, acc_k >= 0))
            stage_accumulate(acc_k, av, acc_nn, nq, T.quick, stage, fb, np, nb, lane);
        // Push the children: exclusive warp scan of the counts.
        int off = nch;
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, off, o);
            if (lane >= o) off += v;
        }
        const int tot = __shfl_sync(0xffffffffu, off, 31);
        off -= nch;
        for (int c = 0; c < nch; ++c) stk[sp + off + c] = ch[c];
        sp += tot;
        __syncwarp();
        if ((iter % FLUSH) == 0) {
            __syncwarp();
            flush_bins(nq * nb, fb, fd, lane);
            __syncwarp();
        }
    }
    __syncwarp();
    flush_bins(nq * nb, fb, fd, lane);
    __syncwarp();
    {
        // The warp's totals: added to its global slot (kept across relaunches).
        double* wa = T.wacc + (size_t)gw * nq * nb;
        warp_add_totals(wa, fd, nq * nb, lane);
        unsigned long long* wn = T.wnp + (size_t)gw * nb;
        for (int q = lane; q < nb; q += 32) wn[q] += (np[q] + np[nb + q]) + (np[2 * nb + q] + np[3 * nb + q]);
    }
    // Counters.
    for (int o = 16; o > 0; o >>= 1) {
        n_eval += __shfl_xor_sync(0xffffffffu, n_eval, o);
        n_acc += __shfl_xor_sync(0xffffffffu, n_acc, o);
        n_esc += __shfl_xor_sync(0xffffffffu, n_esc, o);
    }
    if (lane == 0) {
        atomicAdd(&T.counters[0], (unsigned long long)n_eval);
        atomicAdd(&T.counters[1], (unsigned long long)n_acc);
        atomicAdd(&T.counters[2], (unsigned long long)n_esc);
        atomicAdd(T.idle, 1);
    }
}

// One level of the breadth-first expansion: every thread takes one work item of the input
// array (or a generated root when in == nullptr), and the children of the whole launch are
// appended to out.  The grid is fixed; warps stride over the input, so all lanes stay busy
// and the launch is balanced.  Bins live in shared memory for the whole launch and are added
// to the warp's global FP64 slot at the end (the slots persist across launches).
// Patches: the warp's bins (all of one patch pair) go to that pair's FP64 sums.
__device__ __forceinline__ void patch_flush(const TravParams& T, int pair, int nq, int nb,
                                            float* fb, float2* fd, unsigned long long* np,
                                            int lane)
{
    __syncwarp();
    flush_bins(nq * nb, fb, fd, lane);
    __syncwarp();
    if (pair >= 0) {
        double* pa = T.pacc + (size_t)pair * nq * nb;
        for (int q = lane; q < nq * nb; q += 32) {
            const double v = df_value(fd[q]);
            if (v != 0.) atomicAdd(&pa[q], v);
        }
        unsigned long long* pn = T.pnp + (size_t)pair * nb;
        for (int q = lane; q < nb; q += 32) {
            const unsigned long long v = (np[q] + np[nb + q]) + (np[2 * nb + q] + np[3 * nb + q]);
            if (v) atomicAdd(&pn[q], v);
        }
    }
    __syncwarp();
    for (int q = lane; q < nq * nb; q += 32) fd[q] = make_float2(0.f, 0.f);
    for (int q = lane; q < 4 * nb; q += 32) np[q] = 0ull;
    for (int q = lane; q < 4 * nq * nb; q += 32) fb[q] = 0.f;
    __syncwarp();
}

// Patches: a lane whose pair is not the warp's current one adds directly.
__device__ __forceinline__ void patch_add(const TravParams& T, int pair, int k, int nq, int nb,
                                          const float (&v)[7], unsigned long long nn)
{
    double* pa = T.pacc + (size_t)pair * nq * nb;
    for (int q = 0; q < nq; ++q) atomicAdd(&pa[q * nb + k], (double)v[q]);
    atomicAdd(&T.pnp[(size_t)pair * nb + k], nn);
}

__device__ void sched_step(ExpandSched* S);

// The last warp of a scheduled launch to finish runs the schedule step for the next one.
__device__ __forceinline__ void expand_warp_done(const ExpandSched* S, int lane)
{
    if (!S) return;
    if (lane == 0) {
        ExpandSched* W = const_cast<ExpandSched*>(S);
        __threadfence();
        const unsigned total = gridDim.x * (blockDim.x >> 5);
        if (atomicAdd(&W->warps_done, 1u) == total - 1) {
            __threadfence();
            W->warps_done = 0;
            sched_step(W);
        }
    }
}

// A warp's counters: into its own slot when the launch has slots, else by atomics.
__device__ __forceinline__ void add_counters(const TravParams& T, int gw, long long ev,
                                             long long acc, long long esc, long long learn)
{
    if (T.wctr) {
        unsigned long long* w = T.wctr + (size_t)gw * 8;
        const unsigned long long o0 = w[0], o1 = w[1], o2 = w[2], o3 = w[3];
        w[0] = o0 + (unsigned long long)ev;
        w[1] = o1 + (unsigned long long)acc;
        w[2] = o2 + (unsigned long long)esc;
        w[3] = o3 + (unsigned long long)learn;
        return;
    }
    if (ev) atomicAdd(&T.counters[0], (unsigned long long)ev);
    if (acc) atomicAdd(&T.counters[1], (unsigned long long)acc);
    if (esc) atomicAdd(&T.counters[2], (unsigned long long)esc);
    if (learn) atomicAdd(&T.counters[3], (unsigned long long)learn);
}

// End of an expansion warp: the fixed-order mode records the warp's region counts (k_compact
// commits them and takes the schedule step); otherwise the completion count above.
template <bool DET>
__device__ __forceinline__ void expand_finish(const TravParams& T, const ExpandSched* S, int gw,
                                              long long lo_ch, long long lo_tl, int lane)
{
    if constexpr (DET) {
        if (lane == 0) {
            T.det_cnt[gw] = (int)(lo_ch < T.det_ccap ? lo_ch : T.det_ccap);
            T.det_cnt[T.det_nw + gw] = (int)(lo_tl < T.det_tcap ? lo_tl : T.det_tcap);
        }
        return;
    }
    expand_warp_done(S, lane);
}

#ifndef EXPAND_MINB
#define EXPAND_MINB 7   // resident blocks per SM the register budget is sized for (72 registers)
#endif
template <int MODE, bool DET = false>
__global__ void __launch_bounds__(TB, EXPAND_MINB) k_expand(TravParams T, const int2* in, long long n_in,
                                               long long gen0, int2* out,
                                               unsigned long long* nout, long long out_cap,
                                               const ExpandSched* S)
{
    if (S) {   // scheduled launch: the chunk comes from the device-side schedule
        in = S->in; n_in = S->n_in; gen0 = S->gen0; out = S->out; out_cap = S->out_cap;
        nout = const_cast<unsigned long long*>(&S->nout);
        if (n_in <= 0) return;
    }
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int gw = blockIdx.x * WPB + wib;
    const int nq = T.nqf, nb = T.nbins;
    const size_t wbytes = traverse_warp_bytes(nq, nb);
    float2* fd = (float2*)(smem + wib * wbytes);
    unsigned long long* np = (unsigned long long*)(fd + nq * nb);
    float* fb = (float*)(np + 4 * nb);
    float* stage = fb + 4 * nq * nb;
    for (int q = lane; q < nq * nb; q += 32) fd[q] = make_float2(0.f, 0.f);
    for (int q = lane; q < 4 * nb; q += 32) np[q] = 0ull;
    for (int q = lane; q < 4 * nq * nb; q += 32) fb[q] = 0.f;
    // MODE 2: the network in shared memory after the bins, then per-warp staging.
    MLPPacked* mlpW = nullptr;
    __half* msx = nullptr;
    float* msy = nullptr;
    if constexpr (MODE == 2) {
        unsigned char* mb = smem + ((WPB * wbytes + 15) & ~(size_t)15);
        mlpW = reinterpret_cast<MLPPacked*>(mb);
        msx = reinterpret_cast<__half*>(mb + sizeof(MLPPacked)) + wib * 32 * 8;
        msy = reinterpret_cast<float*>(mb + sizeof(MLPPacked) + WPB * 32 * 8 * sizeof(__half)) + wib * 32;
        for (int q = threadIdx.x; q < (int)(sizeof(MLPPacked) / 4); q += TB)
            reinterpret_cast<uint32_t*>(mlpW)[q] = reinterpret_cast<const uint32_t*>(T.mlp)[q];
        __syncthreads();
    }
    __syncwarp();
    long long n_eval = 0, n_acc = 0, n_esc = 0, n_learn = 0;
    long long lo_ch = 0, lo_tl = 0;   // fixed-order mode: children and tiles in the regions
    int cur_pair = -1;   // mode 3: the patch pair the warp's bins hold
    const long long stride = (long long)gridDim.x * TB;
    int iter = 0;
    for (long long base = (long long)gw * 32; base < n_in; base += stride) {
        const long long idx = base + lane;
        const bool has = idx < n_in;
        int2 task = make_int2(0, 0);
        if (has) task = in ? in[idx] : make_root<MODE>(T, gen0 + idx);
        int nch = 0;
        int2 ch[4];
        int2 tl = make_int2(-1, 0);
        int acc_k = -1;
        float av[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        unsigned long long acc_nn = 0ull;
        bool cand = false;
        float feat[MLP_IN];
        eval_task<MODE>(T, has, task, ch, nch, tl, acc_k, av, acc_nn, n_eval, n_acc, n_esc, cand,
                        feat);
        if constexpr (MODE == 2) {
            // The learned criterion for the warp's candidate pairs: accept (drop the
            // children) or split (drop the prepared accept values).
            if (__any_sync(0xffffffffu, cand)) {
                if (!cand) {
#pragma unroll
                    for (int q = 0; q < MLP_IN; ++q) feat[q] = 0.f;
                }
                const float y = mlp_warp_eval(*mlpW, feat, msx, msy);
                if (cand) {
                    if (y <= T.mlp_thr) { nch = 0; ++n_acc; ++n_learn; }
                    else acc_k = -1;
                }
            }
        }
        if constexpr (MODE == 3) {
            // The warp's bins hold one patch pair.  When every accepted lane is of another
            // pair, the bins move to it; lanes of a pair other than the current one (mixed
            // iterations) add directly.
            int pr = -1;
            if (acc_k >= 0) {
                const int p1 = __float_as_int(T.c1[task.x].d.y), p2 = __float_as_int(T.c2[task.y].d.y);
                pr = T.pair_index[p1 * T.npatch + p2];
            }
            const unsigned am = __ballot_sync(0xffffffffu, acc_k >= 0);
            if (am) {
                const int p0 = __shfl_sync(0xffffffffu, pr, __ffs(am) - 1);
                const bool same = __all_sync(0xffffffffu, acc_k < 0 || pr == p0);
                if (cur_pair < 0) cur_pair = p0;
                if (same && p0 != cur_pair) {
                    patch_flush(T, cur_pair, nq, nb, fb, fd, np, lane);
                    cur_pair = p0;
                    iter = 0;
                }
                if (acc_k >= 0 && pr != cur_pair) {
                    if (pr >= 0) patch_add(T, pr, acc_k, nq, nb, av, acc_nn);
                    acc_k = -1;
                }
            }
        }
        if (__any_sync(0xffffffffu, acc_k >= 0))
            stage_accumulate(acc_k, av, acc_nn, nq, T.quick, stage, fb, np, nb, lane);
        // Append the children: warp scan, one atomic per warp.
        int off = nch;
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, off, o);
            if (lane >= o) off += v;
        }
        const int tot = __shfl_sync(0xffffffffu, off, 31);
        off -= nch;
        if (DET && tot > 0) {
            // Fixed order: the warp's own region, in iteration and lane order.
            if (lo_ch + tot > T.det_ccap) {
                if (lane == 0) atomicCAS(T.err, 0, DEV_SPILL_OVERFLOW);
            } else {
                int2* o = T.det_out + (size_t)gw * T.det_ccap + lo_ch + off;
                for (int c = 0; c < nch; ++c) o[c] = ch[c];
            }
            lo_ch += tot;
        } else if (tot > 0) {
            unsigned long long o0 = 0;
            if (lane == 0) o0 = atomicAdd(nout, (unsigned long long)tot);
            o0 = __shfl_sync(0xffffffffu, o0, 0);
            if ((long long)(o0 + tot) > out_cap) {
                if (lane == 0) atomicCAS(T.err, 0, DEV_SPILL_OVERFLOW);
            } else {
                for (int c = 0; c < nch; ++c) out[o0 + off + c] = ch[c];
            }
        }
        if constexpr (MODE == 4) {
            // Tiles go to the tile list that k_tiles, launched after this kernel, drains.
            const unsigned tm = __ballot_sync(0xffffffffu, tl.x >= 0);
            const int before = __popc(tm & ((1u << lane) - 1u));
            if (DET && tm) {
                if (lo_tl + __popc(tm) > T.det_tcap) {
                    if (lane == 0) atomicCAS(T.err, 0, DEV_SPILL_OVERFLOW);
                } else if (tl.x >= 0) {
                    T.det_tout[(size_t)gw * T.det_tcap + lo_tl + before] = tl;
                }
                lo_tl += __popc(tm);
            } else if (tm) {
                unsigned long long t0 = 0;
                if (lane == 0) t0 = atomicAdd(&T.tctl[0], (unsigned long long)__popc(tm));
                t0 = __shfl_sync(0xffffffffu, t0, 0);
                if ((long long)(t0 + __popc(tm)) > T.tile_cap) {
                    if (lane == 0) atomicCAS(T.err, 0, DEV_SPILL_OVERFLOW);
                } else if (tl.x >= 0) {
                    T.tiles[t0 + before] = tl;
                }
            }
        }
        if ((++iter % FLUSH) == 0) {
            __syncwarp();
            flush_bins(nq * nb, fb, fd, lane);
            __syncwarp();
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        n_eval += __shfl_xor_sync(0xffffffffu, n_eval, o);
        n_acc += __shfl_xor_sync(0xffffffffu, n_acc, o);
        n_esc += __shfl_xor_sync(0xffffffffu, n_esc, o);
        if constexpr (MODE == 2) n_learn += __shfl_xor_sync(0xffffffffu, n_learn, o);
    }
    if (n_acc == 0) {   // nothing accumulated by this warp in this launch
        if (lane == 0 && n_eval) add_counters(T, gw, n_eval, 0, n_esc, 0);
        expand_finish<DET>(T, S, gw, lo_ch, lo_tl, lane);
        return;
    }
    if constexpr (MODE == 3) {
        patch_flush(T, cur_pair, nq, nb, fb, fd, np, lane);
        if (lane == 0) {
            atomicAdd(&T.counters[0], (unsigned long long)n_eval);
            atomicAdd(&T.counters[1], (unsigned long long)n_acc);
            atomicAdd(&T.counters[2], (unsigned long long)n_esc);
        }
        expand_warp_done(S, lane);
        return;
    }
    __syncwarp();
    flush_bins(nq * nb, fb, fd, lane);
    __syncwarp();
    double* wa = T.wacc + (size_t)gw * nq * nb;
    warp_add_totals(wa, fd, nq * nb, lane);
    unsigned long long* wn = T.wnp + (size_t)gw * nb;
    for (int q = lane; q < nb; q += 32) wn[q] += (np[q] + np[nb + q]) + (np[2 * nb + q] + np[3 * nb + q]);
    if (lane == 0) add_counters(T, gw, n_eval, n_acc, n_esc, MODE == 2 ? n_learn : 0);
    expand_finish<DET>(T, S, gw, lo_ch, lo_tl, lane);
}

// The schedule step: commits the previous launch's children and picks the next chunk.
__device__ void sched_step(ExpandSched* S)
{
    if (S->out_level >= 0) {
        S->cnt[S->out_level] += (long long)S->nout;
        S->out_level = -1;
    }
    S->nout = 0;
    S->n_in = 0;
    S->pending = 0;
    if (S->done || S->need_levels) return;
    int L = S->nlev - 1;
    while (L >= 0 && S->cnt[L] == 0) --L;
    if (L < 0) { S->done = 1; return; }
    if (L + 1 >= S->nlev) { S->need_levels = 1; return; }
    const long long chunk = S->cnt[L] < S->chunk_max ? S->cnt[L] : S->chunk_max;
    const long long start = S->cnt[L] - chunk;
    S->cnt[L] = start;
    S->in = (L == 0) ? nullptr : S->lev[L] + start;
    S->n_in = chunk;
    S->gen0 = start;
    S->out = S->lev[L + 1] + S->cnt[L + 1];
    S->out_cap = S->cap - S->cnt[L + 1];
    S->out_level = L + 1;
    S->launches += 1;
    S->pending = 1;
}

// Start of a batch: a step only if no picked chunk is waiting (the last warp of the
// previous batch's final launch may already have picked one).
__global__ void k_expand_sched(ExpandSched* S)
{
    if (!S->pending) sched_step(S);
}

// Fixed-order expansion: joins the child and tile regions of the expansion launch that just
// ran, in warp order, into the level buffer (S->out) and the tile list; then the last block
// commits the children and takes the schedule step, which the last warp of an expansion
// launch does otherwise.  Block b copies the regions of warps CPB b .. CPB b + CPB - 1, one
// per warp; every count is an integer, so the offsets do not depend on timing.
static constexpr int CPB = 8;

__device__ __forceinline__ long long warp_sum_ll(long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Copies n items from src to dst with 8 loads in flight per lane.
__device__ __forceinline__ void copy_items(int2* dst, const int2* src, int n, int lane)
{
    for (int i0 = 0; i0 < n; i0 += 256) {
        int2 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = i0 + 32 * u + lane;
            if (i < n) v[u] = src[i];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = i0 + 32 * u + lane;
            if (i < n) dst[i] = v[u];
        }
    }
}

__global__ void __launch_bounds__(CPB * 32) k_compact(const __grid_constant__ TravParams T,
                                                      ExpandSched* S)
{
    if (S->n_in <= 0) return;   // the expansion launch had nothing to do
    __shared__ long long red[2][CPB];
    __shared__ int last;
    const int nw = T.det_nw, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int* cc = T.det_cnt;
    const int* ct = T.det_cnt + nw;
    const int r0 = blockIdx.x * CPB;
    // Counts of the regions before this block's, four at a time (nw and r0 are multiples of
    // 4, so both count arrays are 16-byte aligned).
    long long pc = 0, pt = 0;
    const int4* cc4 = reinterpret_cast<const int4*>(cc);
    const int4* ct4 = reinterpret_cast<const int4*>(ct);
    for (int q = tid; q < r0 / 4; q += CPB * 32) {
        const int4 a = cc4[q], b = ct4[q];
        pc += (long long)a.x + a.y + a.z + a.w;
        pt += (long long)b.x + b.y + b.z + b.w;
    }
    pc = warp_sum_ll(pc);
    pt = warp_sum_ll(pt);
    if (lane == 0) { red[0][w] = pc; red[1][w] = pt; }
    __syncthreads();
    long long oc = 0, ot = 0;
    for (int q = 0; q < CPB; ++q) { oc += red[0][q]; ot += red[1][q]; }
    const int r = r0 + w;
    if (r < nw) {
        for (int q = r0; q < r; ++q) { oc += cc[q]; ot += ct[q]; }
        const int n = cc[r], m = ct[r];
        if (oc + n > S->out_cap) {
            if (lane == 0) atomicCAS(T.err, 0, DEV_SPILL_OVERFLOW);
        } else {
            copy_items(S->out + oc, T.det_out + (size_t)r * T.det_ccap, n, lane);
        }
        if (m > 0 && ot + m > T.tile_cap) {
            if (lane == 0) atomicCAS(T.err, 0, DEV_SPILL_OVERFLOW);
        } else if (m > 0) {
            copy_items(T.tiles + ot, T.det_tout + (size_t)r * T.det_tcap, m, lane);
        }
    }
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        last = atomicAdd(&S->warps_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    long long tc = 0, tt = 0;
    for (int q = tid; q < nw / 4; q += CPB * 32) {
        const int4 a = cc4[q], b = ct4[q];
        tc += (long long)a.x + a.y + a.z + a.w;
        tt += (long long)b.x + b.y + b.z + b.w;
    }
    tc = warp_sum_ll(tc);
    tt = warp_sum_ll(tt);
    if (lane == 0) { red[0][w] = tc; red[1][w] = tt; }
    __syncthreads();
    if (tid == 0) {
        tc = 0; tt = 0;
        for (int q = 0; q < CPB; ++q) { tc += red[0][q]; tt += red[1][q]; }
        S->warps_done = 0;
        S->nout = (unsigned long long)(tc < S->out_cap ? tc : S->out_cap);
        if (T.tile_leaf > 0) T.tctl[0] = (unsigned long long)(tt < T.tile_cap ? tt : T.tile_cap);
        sched_step(S);
    }
}

long long det_items_per_warp(long long chunk, int nwarps)
{
    const long long per = 32LL * nwarps;
    return 32LL * ((chunk + per - 1) / per);
}

// Sum of the per-warp totals in a fixed order: out[q*nb+k] (double), outnp[k] (u64).
__global__ void k_reduce_acc(int nwarps, int nq, int nb, const double* wacc,
                             const unsigned long long* wnp, double* out,
                             unsigned long long* outnp)
{
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nq * nb) {
        double s = 0.;
        for (int w = 0; w < nwarps; ++w) s += wacc[(size_t)w * nq * nb + q];
        out[q] = s;
    }
    if (q < nb) {
        unsigned long long s = 0;
        for (int w = 0; w < nwarps; ++w) s += wnp[(size_t)w * nb + q];
        outnp[q] = s;
    }
}

// ---------------------------------------------------------------------------------------
// Host side.

size_t traverse_smem_bytes(int nq, int nb)
{
    return traverse_warp_bytes(nq, nb) * WPB;
}

int traverse_grid(int nq, int nb, int* blocks, int* nwarps)
{
    int dev = 0, nsm = 0, per = 0;
    TC_CU(cudaGetDevice(&dev));
    TC_CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    size_t sm = traverse_smem_bytes(nq, nb);
    if (sm > 48 * 1024)
        TC_CU(cudaFuncSetAttribute(k_traverse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    TC_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_traverse, TB, sm));
    if (per < 1) per = 1;
    *blocks = nsm * per;
    *nwarps = *blocks * WPB;
    return 0;
}

// Shared memory of k_expand<mode>: the warps' bins, and for mode 2 the network and the
// warps' staging areas.
static size_t expand_smem_bytes(int nq, int nb, int mode)
{
    size_t sm = traverse_smem_bytes(nq, nb);
    if (mode == 2)
        sm = ((sm + 15) & ~(size_t)15) + sizeof(MLPPacked) +
             WPB * 32 * (8 * sizeof(__half) + sizeof(float));
    return sm;
}

template <int MODE, bool DET = false>
static int set_expand_attr(size_t sm)
{
    if (sm > 48 * 1024)
        TC_CU(cudaFuncSetAttribute(k_expand<MODE, DET>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    return 0;
}

int launch_expand_batch(const TravParams& T, int blocks, ExpandSched* dS, int iters,
                        cudaStream_t st, cudaEvent_t* ev)
{
    const size_t sm = expand_smem_bytes(T.nqf, T.nbins, T.mode);
    // One schedule step starts the batch (the host may have changed the schedule); every
    // expand launch ends with the next step, run by its last warp.
    count_launch();
    k_expand_sched<<<1, 1, 0, st>>>(dS);
    for (int it = 0; it < iters; ++it) {
        if (ev) TC_CU(cudaEventRecord(ev[3 * it], st));
        count_launch();
        // The fixed-order mode (T.det: modes 0 and 2) and the tiles (mode 0 in exact mode,
        // run as instantiation 4) are compiled in only where they are used.
        if (T.mode == 3) k_expand<3><<<blocks, TB, sm, st>>>(T, nullptr, 0, 0, nullptr, nullptr, 0, dS);
        else if (T.mode == 2 && T.det) k_expand<2, true><<<blocks, TB, sm, st>>>(T, nullptr, 0, 0, nullptr, nullptr, 0, dS);
        else if (T.mode == 2) k_expand<2><<<blocks, TB, sm, st>>>(T, nullptr, 0, 0, nullptr, nullptr, 0, dS);
        else if (T.mode == 1) k_expand<1><<<blocks, TB, sm, st>>>(T, nullptr, 0, 0, nullptr, nullptr, 0, dS);
        else if (T.tile_leaf > 0 && T.det) k_expand<4, true><<<blocks, TB, sm, st>>>(T, nullptr, 0, 0, nullptr, nullptr, 0, dS);
        else if (T.tile_leaf > 0) k_expand<4><<<blocks, TB, sm, st>>>(T, nullptr, 0, 0, nullptr, nullptr, 0, dS);
        else if (T.det) k_expand<0, true><<<blocks, TB, sm, st>>>(T, nullptr, 0, 0, nullptr, nullptr, 0, dS);
        else k_expand<0><<<blocks, TB, sm, st>>>(T, nullptr, 0, 0, nullptr, nullptr, 0, dS);
        if (T.det) {
            count_launch();
            k_compact<<<(T.det_nw + CPB - 1) / CPB, CPB * 32, 0, st>>>(T, dS);
        }
        if (ev) TC_CU(cudaEventRecord(ev[3 * it + 1], st));
        if (T.mode == 0 && T.tile_leaf > 0) TC_TRY(launch_tiles(T, st));
        if (ev) TC_CU(cudaEventRecord(ev[3 * it + 2], st));
    }
    TC_CU(cudaGetLastError());
    return 0;
}

int expand_grid(int nq, int nb, int* blocks, int* nwarps, int mode)
{
    int dev = 0, nsm = 0, per = 0;
    TC_CU(cudaGetDevice(&dev));
    TC_CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const size_t sm = expand_smem_bytes(nq, nb, mode);
    if (mode == 3) {
        TC_TRY(set_expand_attr<3>(sm));
        TC_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_expand<3>, TB, sm));
    } else if (mode == 2) {
        TC_TRY(set_expand_attr<2>(sm));
        TC_TRY((set_expand_attr<2, true>(sm)));
        TC_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_expand<2>, TB, sm));
    } else if (mode == 1) {
        TC_TRY(set_expand_attr<1>(sm));
        TC_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_expand<1>, TB, sm));
    } else {
        // Mode 0 runs as k_expand<0>, or as k_expand<4> when it hands leaf-pair tiles to
        // k_tiles; both have the same register bound and shared memory.
        TC_TRY(set_expand_attr<0>(sm));
        TC_TRY((set_expand_attr<0, true>(sm)));
        TC_TRY(set_expand_attr<4>(sm));
        TC_TRY((set_expand_attr<4, true>(sm)));
        TC_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_expand<0>, TB, sm));
    }
    if (per < 1) per = 1;
    *blocks = nsm * per;
    *nwarps = *blocks * WPB;
    return 0;
}

int launch_traverse(const TravParams& T, int blocks, cudaStream_t st)
{
    size_t sm = traverse_smem_bytes(T.nqf, T.nbins);
    count_launch(); k_traverse<<<blocks, TB, sm, st>>>(T);
    TC_CU(cudaGetLastError());
    return 0;
}

int launch_reduce(int nwarps, int nq, int nb, const double* wacc, const unsigned long long* wnp,
                  double* out, unsigned long long* outnp, cudaStream_t st)
{
    int n = nq * nb > nb ? nq * nb : nb;
    count_launch(); k_reduce_acc<<<(n + 127) / 128, 128, 0, st>>>(nwarps, nq, nb, wacc, wnp, out, outnp);
    TC_CU(cudaGetLastError());
    return 0;
}


// ---------------------------------------------------------------------------------------
// Fixed traversal scratch for callers that cannot allocate device memory.
//
// One file-scope device array holds everything one traversal needs: the per-warp stacks,
// the two spill lists, the per-warp FP64 bins, the reduced totals and the control words.
// Its size is fixed at NOALLOC_BYTES (about 52 MiB); every GPU that loads this library holds
// it until the process exits.  The host code must not use the array's name as an address
// (that is only a host-side stand-in): noalloc_scratch() looks its device address up with
// cudaGetSymbolAddress, once per device, with that device current.

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

static void* g_noalloc_ptr[64] = {nullptr};

int noalloc_scratch(void** base)
{
    int dev = 0;
    TC_CU(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_last_error("device index out of range for the fixed traversal scratch");
        return 1;
    }
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        TC_CU(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = p;
    }
    *base = g_noalloc_ptr[dev];
    return 0;
}

}  // namespace tc
