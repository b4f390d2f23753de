// tiles.cu -- leaf-pair tiles of the exact mode (angle_slop 0, or two brute fields).
//
// In that mode the reference accepts only pairs of leaves (src/Corr2.cpp:308-389:
// BinTypeHelper<Log>::singleBin, include/BinType.h:93-151, needs s1 + s2 <= a r, which
// a = 0 allows only for leaves, whose size is 0), so below a cell pair it visits every leaf
// pair, keeps those in range (isRSqInRange, include/BinType.h:61-66) and adds each into the
// bin of its own separation (directProcess11 and finishProcess with DirectHelper,
// src/Corr2.cpp:394-566).  The traversal stops at cell pairs of at most TILE_LEAF points per
// side and hands them here as tiles; k_tiles does the rest with one warp per tile and no tree
// walk:
//   * both sides' leaves are staged in shared memory as FP32 offsets from cell B's FP64 centre
//     (hi + lo parts), so a separation is one FP32 difference of offsets whose error is a few
//     ulps of the tile's extent;
//   * the tile is classified once from the centres and the cells' sizes: when every pair
//     certainly lies inside the separation range and inside one bin (margins far above the
//     FP32 errors), the per-pair range and bin work is skipped (tile_fast); when the pairs lie
//     in range and on either side of one bin edge, one comparison with that edge decides the
//     bin (tile_two); otherwise each pair gets its range test and its bin from log2 of its
//     squared separation over the squared edge of the tile's lowest bin (tile_general).  Both
//     decisions carry a band that covers every FP32 error; a pair inside the band is decided
//     again in FP64 from the FP64 positions with the reference's formulas, in a second pass
//     over the tile, so that the main pair loops have no call and keep their registers;
//   * lanes take the tile's leaf pairs in order (pair p: leaf p / nB of A, p % nB of B), and
//     keep running sums for the tile's lowest two bins in registers; pairs in other bins (tiles
//     that span three or more bins, at separations comparable with the cell sizes) and the
//     FP64-decided pairs go to the warp's shared-memory bins in ascending lane order (through
//     a staging area in leaf arrays the pass does not read, or by shuffles), so every sum is
//     formed in the same order in every run;
//   * at the end of a tile the lanes' sums are combined by a reduce-scatter butterfly (one
//     shuffle per value and step, halving the values each step) and added to the warp's FP32
//     bins, which go into double-float totals every few tiles and into the warp's FP64 slot
//     at the end, like the traversal's.
// The kernel is compiled per geometry (flat, sphere with Arc, sphere or 3-d with Euclidean)
// and per class family (NN; NK and KK; GG; the others through the generic projection code).
// Measured on the 10M-point curved-sky catalog (bin_slop 0, angle_slop 0): the single-bin
// loop runs at ~3.6e11 leaf pairs/s, the two-bin loop at ~2.4e11; tiles of up to 48 points
// per side (TILE_LEAF; 64 with the autotuner on that catalog) balance the pair loops against
// the per-tile work (staging, bounds, the final butterfly): 32-point tiles took 22.5 s, 48
// 17.5 s before the two-pass loops, 15.3 s after.  A variant that staged the next tile's
// leaves with bulk copies (cp.async.bulk + mbarrier) while the current one ran was 6% slower:
// the per-tile cost is instruction issue, not load latency, with 24 warps per SM.
#include <cfloat>
#include <cmath>
#include <cstdint>

#include "tc_internal.cuh"
#include "tc_host.hpp"
#include "traverse2pt.hpp"
#include "pair_math.cuh"

namespace tc {

namespace {

constexpr int TPB = 128;          // threads per block
constexpr int TWPB = TPB / 32;    // warps per block
constexpr int TFLUSH = 8;         // tiles between flushes of the FP32 bins
#ifndef TILES_MINB
#define TILES_MINB 6
#endif
constexpr int TMINB = TILES_MINB; // resident blocks per SM the registers are sized for
#ifndef TILE_CAP
#define TILE_CAP 64
#endif
constexpr int TCAP = TILE_CAP;    // most leaves per tile side (>= the traversal's tile_leaf)
static_assert(TCAP * 4 >= 32 * 8, "a tile side's X array doubles as the 32 x 8 staging area");

enum { TG_FLAT = 0, TG_ARC = 1, TG_SPHEUC = 2, TG_3D = 3 };   // geometry
enum { TK_NN = 0, TK_SC = 1, TK_GEN = 2, TK_GG = 3 };           // class family

// One side of a tile: its valid leaves (n > 0, w != 0) in point order.  Pair loops read P and
// W of both sides (two 16-byte shared loads per side) and X only where it is needed.
struct TileLeaves {
    float4 P[TCAP];   // (ox, oy, oz, z / 2): offset from B's centre, half the z coordinate
    float4 W[TCAP];   // (w, p1, p2, n bits): weight, payload (p1 = w for N, w k for K, w g for
                      // complex kinds), point count
    float4 X[TCAP];   // (x, y, id bits, 0): FP32 position (sphere projections), leaf cell id
};

__host__ __device__ inline size_t bins_bytes(int nq, int nb)
{
    return ((size_t)nq * nb * 8 + (size_t)nb * 8 + (size_t)nq * nb * 4 + 15) & ~(size_t)15;
}

__host__ __device__ inline size_t edges_bytes(int nb)
{
    return ((size_t)2 * (nb + 1) * 4 + 15) & ~(size_t)15;
}

__host__ __device__ inline size_t warp_bytes(int nq, int nb)
{
    return bins_bytes(nq, nb) + 2 * sizeof(TileLeaves);
}

// Stages the valid leaves of cell c (points [start, start + n), leaf ids base + p) with their
// offsets from the centre (ch + cl), in point order.  Returns the count; *single is false when
// a staged leaf holds more than one point.  on1 / on2: the largest L1 norm and length of the
// lane's offsets (used only when the cells' sizes are not finite bounds, i.e. brute cells).
__device__ __forceinline__ int stage(const TCell* cells, int base, float4 cc, float4 cd,
                                     float chx, float chy, float chz, float clx, float cly,
                                     float clz, int kind, TileLeaves& S, int lane, bool norms,
                                     float& on1, float& on2, bool& single)
{
    const int start = __float_as_int(cd.z), n = __float_as_int(cc.z);
    int cnt = 0;
    bool all1 = true;
    on1 = 0.f; on2 = 0.f;
#pragma unroll
    for (int h = 0; h < TCAP / 32; ++h) {
        const int p0 = lane + 32 * h;
        bool v = false;
        float4 P = make_float4(0.f, 0.f, 0.f, 0.f), W = P, X = P;
        int nn = 0;
        if (p0 < n) {
            const int id = base + start + p0;
            const float4 a = cells[id].a, b = cells[id].b, c = cells[id].c;
            nn = __float_as_int(c.z);
            v = nn > 0 && b.w != 0.f;
            if (v) {
                P = make_float4((a.x - chx) + (b.x - clx), (a.y - chy) + (b.y - cly),
                                (a.z - chz) + (b.z - clz), 0.5f * a.z);
                W = make_float4(b.w, kind == DN ? b.w : c.x, c.y, __int_as_float(nn));
                X = make_float4(a.x, a.y, __int_as_float(id), 0.f);
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, v);
        all1 = all1 && __all_sync(0xffffffffu, !v || nn == 1);
        if (v) {
            const int p = cnt + __popc(m & ((1u << lane) - 1u));
            S.P[p] = P; S.W[p] = W; S.X[p] = X;
        }
        cnt += __popc(m);
        if (norms) {
            on1 = fmaxf(on1, fabsf(P.x) + fabsf(P.y) + fabsf(P.z));
            on2 = fmaxf(on2, sqrtf(P.x * P.x + P.y * P.y + P.z * P.z));
        }
        if (32 * (h + 1) >= n) break;
    }
    single = all1;
    return cnt;
}

__device__ __forceinline__ float warp_max(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Sums v[0..7] over the warp: after the reduce-scatter each group of 4 lanes holds one value's
// total; lane 4 q + 0 returns value q's total in *out (q = 0..7) and true.
__device__ __forceinline__ bool warp_sum8(float (&v)[8], int lane, float& out)
{
    // xor 16: keep 4 of 8.
    const bool h16 = lane & 16;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float send = h16 ? v[q] : v[q + 4];
        const float got = __shfl_xor_sync(0xffffffffu, send, 16);
        v[q] = (h16 ? v[q + 4] : v[q]) + got;
    }
    // xor 8: keep 2 of 4.
    const bool h8 = lane & 8;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const float send = h8 ? v[q] : v[q + 2];
        const float got = __shfl_xor_sync(0xffffffffu, send, 8);
        v[q] = (h8 ? v[q + 2] : v[q]) + got;
    }
    // xor 4: keep 1 of 2.
    const bool h4 = lane & 4;
    {
        const float send = h4 ? v[0] : v[1];
        const float got = __shfl_xor_sync(0xffffffffu, send, 4);
        v[0] = (h4 ? v[1] : v[0]) + got;
    }
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 2);
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
    out = v[0];
    return (lane & 3) == 0;
}

// Which value a lane holds after warp_sum8: bit 4 picks the upper half, bit 3 the upper
// quarter of that, bit 2 the upper one of the last two.
__device__ __forceinline__ int warp_sum8_index(int lane)
{
    return ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
}

// A leaf pair decided in FP64 with the reference's formulas: decide64 (the reference's
// process11 for s1 = s2 = 0) on the FP64 leaf positions.  Out of line: it runs for about one
// pair in 10^5, and keeping it out of the loop keeps the loop's registers low.
__device__ __noinline__ int leaf_pair64(const TravParams& T, int ida, int idb, bool self,
                                        float* r, float* logr)
{
    const double* x2 = self ? T.x1 : T.x2;
    const double* y2 = self ? T.y1 : T.y2;
    const double* z2 = self ? T.z1 : T.z2;
    const double dx = T.x1[ida] - x2[idb], dy = T.y1[ida] - y2[idb];
    double dsq = dx * dx + dy * dy;
    if (T.coords != FLAT) {
        const double dz = T.z1[ida] - z2[idb];
        dsq += dz * dz;
    }
    const Decision D = decide64(T, dsq, 0., 0.);
    if (D.act != ACT_ACCEPT) return -1;
    *r = D.r;
    *logr = D.logr;
    return D.k;
}

// The generic values of an accepted leaf pair (every class, with the projections of
// accept_values); x = the correlation products.  Out of line: it serves the rarer classes.
__device__ __noinline__ void leaf_values_generic(const TravParams& T, float4 Pa, float4 Wa,
                                                 float4 Xa, float4 Pb, float4 Wb, float4 Xb,
                                                 float dx, float dy, float dz, float dsq,
                                                 float r, float logr, float* x)
{
    TCell A, B;
    A.a = make_float4(Xa.x, Xa.y, 2.f * Pa.w, 0.f);
    A.b = make_float4(0.f, 0.f, 0.f, Wa.x);
    A.c = make_float4(Wa.y, Wa.z, Wa.w, 0.f);
    A.d = make_float4(0.f, 0.f, 0.f, 0.f);
    B.a = make_float4(Xb.x, Xb.y, 2.f * Pb.w, 0.f);
    B.b = make_float4(0.f, 0.f, 0.f, Wb.x);
    B.c = make_float4(Wb.y, Wb.z, Wb.w, 0.f);
    B.d = A.d;
    float av[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    unsigned long long nn = 0;
    accept_values(T, A, B, __float_as_int(Xa.z), __float_as_int(Xb.z), dx, dy, dz, dsq, r, logr,
                  av, nn);
#pragma unroll
    for (int q = 3; q < 7; ++q) x[q - 3] = av[q];
}

// The correlation products of one leaf pair (quantities 3.. of the bins) as x * sc.
template <int GEO, int KIND>
__device__ __forceinline__ void pair_products(const TravParams& T, const TileLeaves& LA,
                                              const TileLeaves& SB, int i, int j, float4 Pa,
                                              float4 Wa, float4 Pb, float4 Wb, float dx,
                                              float dy, float dz, float dsq, float r, float logr,
                                              float (&x)[4], float& sc)
{
    sc = 1.f;
    if constexpr (KIND == TK_SC) {
        x[0] = Wa.y * Wb.y;                                  // wk1 wk2 (DirectHelper<1>)
    } else if constexpr (KIND == TK_GG && GEO == TG_FLAT) {
        // ProjectHelper<Flat>: both shears rotated by exp(-2i alpha) of r = p2 - p1, so
        // g1 conj(g2) is unchanged and g1 g2 turns by exp(-4i alpha) = conj(r)^4 / |r|^4.
        const float g1r = Wa.y, g1i = Wa.z, g2r = Wb.y, g2i = Wb.z;
        x[0] = fmaf(g1r, g2r, g1i * g2i);                    // xi+ = g1 conj(g2)
        x[1] = fmaf(g1i, g2r, -g1r * g2i);
        const float er = fmaf(dx, dx, -dy * dy), ei = -2.f * dx * dy;   // conj(r)^2, r = -d
        const float e2r = fmaf(er, er, -ei * ei), e2i = 2.f * er * ei;
        const float inv = __fdividef(1.f, dsq * dsq);
        const float pr = fmaf(g1r, g2r, -g1i * g2i), pi = fmaf(g1r, g2i, g1i * g2r);   // g1 g2
        x[2] = fmaf(pr, e2r, -pi * e2i) * inv;               // xi-
        x[3] = fmaf(pr, e2i, pi * e2r) * inv;
    } else if constexpr (KIND == TK_GG && (GEO == TG_ARC || GEO == TG_SPHEUC)) {
        // ProjectHelper<Sphere>, include/ProjectHelper.h:272-388: directions at p2
        // (sinA, -cosA) and at p1 (-sinA, -cosB) on accurate differences (d = p1 - p2):
        // y1 x2 - x1 y2 = x1 dy - y1 dx.  Spin 2: exp(-2i a) = conj(u)^2 / |u|^2; the two
        // normalisations are one reciprocal, applied as the scale sc.
        const float4 Xa = LA.X[i];
        const float sinA = fmaf(Xa.x, dy, -Xa.y * dx);
        const float cosA = fmaf(Pb.w, dsq, dz);
        const float cosB = fmaf(Pa.w, dsq, -dz);
        const float s2 = sinA * sinA;
        const float n2 = fmaf(cosA, cosA, s2), n1 = fmaf(cosB, cosB, s2);
        const float e2r = fmaf(-cosA, cosA, s2), e2i = 2.f * sinA * cosA;
        const float e1r = fmaf(-cosB, cosB, s2), e1i = -2.f * sinA * cosB;
        sc = __fdividef(1.f, n1 * n2);
        const float a2r = fmaf(Wb.y, e2r, -Wb.z * e2i), a2i = fmaf(Wb.y, e2i, Wb.z * e2r);
        const float a1r = fmaf(Wa.y, e1r, -Wa.z * e1i), a1i = fmaf(Wa.y, e1i, Wa.z * e1r);
        // both_complex_prod(g2, g1), include/ProjectHelper.h:84-101.
        x[0] = fmaf(a2r, a1r, a2i * a1i);     // xi+
        x[1] = fmaf(a2r, a1i, -a2i * a1r);
        x[2] = fmaf(a2r, a1r, -a2i * a1i);    // xi-
        x[3] = fmaf(a2r, a1i, a2i * a1r);
    } else if constexpr (KIND == TK_GG || KIND == TK_GEN) {
        leaf_values_generic(T, Pa, Wa, LA.X[i], Pb, Wb, SB.X[j], dx, dy, dz, dsq, r, logr, x);
    }
}

// The great-circle angle from a chord c < 0.25 (the tile checks it): the Maclaurin series
// of 2 asin(c / 2) to x^7, x = c / 2 (the first omitted term is below 2e-9 of x).
__device__ __forceinline__ float arc_series(float c)
{
    const float x = 0.5f * c, x2 = x * x;
    return 2.f * x * fmaf(x2, fmaf(x2, fmaf(x2, 5.f / 112.f, 3.f / 40.f), 1.f / 6.f), 1.f);
}

// Adds a tile's per-lane sums of one bin into the warp's FP32 bins.  acc: weight, sum w w r,
// sum w w lr (lr = log2(r^2 / edge^2) of the tile's reference edge), products; the bin's
// meanlogr sum is (ln 2 / 2) sum w w lr + log(edge) sum w w.
__device__ __forceinline__ void tile_bin_out(float (&acc)[8], unsigned cn, int kb, int nq, int nb,
                                             float ledge, float* fb, unsigned long long* np,
                                             bool quick, bool single, int lane)
{
    if (!__any_sync(0xffffffffu, cn != 0u) || kb >= nb) return;
    acc[2] = fmaf(acc[2], 0.5f * 0.69314718f, acc[0] * ledge);
    float tot;
    const bool holder = warp_sum8(acc, lane, tot);
    const int q = warp_sum8_index(lane);
    if (holder && q < nq) fb[q * nb + kb] += tot;
    if (!quick) {
        if (single) {
            const unsigned ct = __reduce_add_sync(0xffffffffu, cn);
            if (lane == 0) np[kb] += ct;
        } else if (cn) {
            atomicAdd(&np[kb], (unsigned long long)cn);
        }
    }
    __syncwarp();
}

// Everything a tile's pair loop needs besides its leaves.
struct TileCtx {
    int na, nbl, kref;
    float inv_edge, ledge, emax, band_e, band_0;
    bool self, interior, small_chord;
};

// The leaf pairs of a tile whose pairs all lie in range and in bin kref (and, on the sphere,
// whose chords are below 0.25): no range test, no bin, no FP64.
template <int GEO, int KIND>
__device__ __forceinline__ void tile_fast(const TravParams& T, const TileLeaves& LA,
                                          const TileLeaves& SB, const TileCtx& C, int lane,
                                          float (&acc)[8], unsigned& cnt)
{
    const int nbl = C.nbl, npt = C.na * nbl;
    int ii = lane / nbl, jj = lane - ii * nbl;
    const int di = 32 / nbl, dj = 32 - di * nbl;
    for (int p = lane; p < npt; p += 32) {
        const int i = ii, j = jj;
        jj += dj; ii += di;
        if (jj >= nbl) { jj -= nbl; ++ii; }
        const float4 Pa = LA.P[i], Wa = LA.W[i], Pb = SB.P[j], Wb = SB.W[j];
        const float dx = Pa.x - Pb.x, dy = Pa.y - Pb.y;
        const float dz = GEO == TG_FLAT ? 0.f : Pa.z - Pb.z;
        const float dsq = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const float c = dsq * rsqrtf(dsq);
        const float r = GEO == TG_ARC ? arc_series(c) : c;
        const float lr = __log2f(r * r * C.inv_edge);
        const float ww = Wa.x * Wb.x;
        acc[0] += ww;
        acc[1] = fmaf(ww, r, acc[1]);
        acc[2] = fmaf(ww, lr, acc[2]);
        if constexpr (KIND != TK_NN) {
            float x[4] = {0.f, 0.f, 0.f, 0.f}, sc;
            pair_products<GEO, KIND>(T, LA, SB, i, j, Pa, Wa, Pb, Wb, dx, dy, dz, dsq, r,
                                     fmaf(lr, 0.5f * 0.69314718f, C.ledge), x, sc);
            constexpr int NX = KIND == TK_SC ? 1 : 4;
#pragma unroll
            for (int q = 0; q < NX; ++q) acc[3 + q] = fmaf(x[q], sc, acc[3 + q]);
        }
        cnt += (unsigned)__float_as_int(Wa.w) * (unsigned)__float_as_int(Wb.w);
    }
}

// Adds the pairs that lanes hold for the shared bins (kx >= 0, values v) in ascending lane
// order: lane q < nq adds quantity q of each, so the sums do not depend on the order in which
// conflicting shared atomics would land.
__device__ __forceinline__ void shared_bins_in_order(int kx, const float (&v)[8], float* fb,
                                                     int nq, int nb, int lane)
{
    unsigned m = __ballot_sync(0xffffffffu, kx >= 0);
    while (m) {
        const int t = __ffs(m) - 1;
        m &= m - 1u;
        const int kt = __shfl_sync(0xffffffffu, kx, t);
        float x = 0.f;
#pragma unroll
        for (int q = 0; q < 7; ++q) {
            const float y = __shfl_sync(0xffffffffu, v[q], t);
            x = lane == q ? y : x;
        }
        if (lane < nq) fb[lane * nb + kt] += x;
    }
}

// The same through a staging area of 32 x 8 floats in shared memory (a part of the tile's
// leaf arrays that the pass does not read): each lane writes its values and bin, then lane
// q < nq adds quantity q of the staged pairs in ascending lane order -- a few instructions
// per pair instead of a round of shuffles.
__device__ __forceinline__ void shared_bins_staged(int kx, const float (&v)[8], float* stg,
                                                   float* fb, int nq, int nb, int lane)
{
    unsigned m = __ballot_sync(0xffffffffu, kx >= 0);
    if (!m) return;
    if (kx >= 0) {
        float4* my = reinterpret_cast<float4*>(stg + lane * 8);
        my[0] = make_float4(v[0], v[1], v[2], v[3]);
        my[1] = make_float4(v[4], v[5], v[6], __int_as_float(kx));
    }
    __syncwarp();
    if (lane < nq) {
        while (m) {
            const int t = __ffs(m) - 1;
            m &= m - 1u;
            const float* e = stg + t * 8;
            fb[lane * nb + __float_as_int(e[7])] += e[lane];
        }
    }
    __syncwarp();
}

// Pairs inside the FP32 error band of a bin or range decision are decided in FP64 from the
// FP64 positions (leaf_pair64).  The pair loops below run twice when a tile has such pairs:
// the main pass (ESC = false) skips them and has no call in its loop, which keeps its
// registers free of the call's saves; the escalation pass (ESC = true) takes only them.

// The pair loop of a cross tile whose pairs all lie in range and in bins kref and kref + 1
// (the common general case at large separations, where a tile straddles one bin edge): no
// range test, one comparison with the middle edge (in units of bins, d = kk - 1, with the
// same FP32 error band as the general loop), both bins summed branch-free in registers.
template <int GEO, int KIND, bool ESC>
__device__ __forceinline__ bool tile_two(const TravParams& T, const TileLeaves& LA,
                                         const TileLeaves& SB, const TileCtx& C, int lane,
                                         float (&acc0)[8], float (&acc1)[8], unsigned& c0,
                                         unsigned& c1, float* fb, unsigned long long* np,
                                         unsigned& n_drop, unsigned& n_esc)
{
    const int nbl = C.nbl, npt = C.na * nbl, nq = T.nqf, nb = T.nbins;
    const float ln2h = 0.5f * 0.69314718f;
    const float ckk = ln2h * T.finvbinsize;
    int ii = lane / nbl, jj = lane - ii * nbl;
    const int di = 32 / nbl, dj = 32 - di * nbl;
    bool seen = false;   // main pass: a pair was left for the escalation pass
    for (int p0 = 0; p0 < npt; p0 += 32) {
        const int i = ii, j = jj;
        jj += dj; ii += di;
        if (jj >= nbl) { jj -= nbl; ++ii; }
        int kx = -1;
        float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        do {
            if (p0 + lane >= npt) break;
            const float4 Pa = LA.P[i], Pb = SB.P[j];
            const float dx = Pa.x - Pb.x, dy = Pa.y - Pb.y;
            const float dz = GEO == TG_FLAT ? 0.f : Pa.z - Pb.z;
            const float dsq = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const float invc = rsqrtf(dsq);
            float r = dsq * invc;
            if (GEO == TG_ARC) r = arc_series(r);
            const float lr = __log2f(r * r * C.inv_edge);
            const float d = fmaf(lr, ckk, -1.f);
            const bool unsure = fabsf(d) < fmaf(C.band_e, invc, C.band_0);
            if (unsure != ESC) {
                seen = seen || unsure;
                break;
            }
            float logr = fmaf(lr, ln2h, C.ledge);
            int k = C.kref + (d >= 0.f ? 1 : 0);
            if constexpr (ESC) {
                ++n_esc;
                k = leaf_pair64(T, __float_as_int(LA.X[i].z), __float_as_int(SB.X[j].z), false,
                                &r, &logr);
                if (k < 0) { ++n_drop; break; }
            }
            const float4 Wa = LA.W[i], Wb = SB.W[j];
            const float ww = Wa.x * Wb.x;
            v[0] = ww; v[1] = ww * r; v[2] = ww * (ESC ? logr : lr);
            if constexpr (KIND != TK_NN) {
                float x[4] = {0.f, 0.f, 0.f, 0.f}, sc;
                pair_products<GEO, KIND>(T, LA, SB, i, j, Pa, Wa, Pb, Wb, dx, dy, dz, dsq, r,
                                         logr, x, sc);
#pragma unroll
                for (int q = 0; q < 4; ++q) v[3 + q] = x[q] * sc;
            }
            const unsigned nn = (unsigned)__float_as_int(Wa.w) * (unsigned)__float_as_int(Wb.w);
            if constexpr (ESC) {
                kx = k;
                if (!T.quick) atomicAdd(&np[k], (unsigned long long)nn);   // exact integer
            } else {
                const float m1 = d >= 0.f ? 1.f : 0.f, m0 = 1.f - m1;
#pragma unroll
                for (int q = 0; q < 7; ++q) {
                    acc0[q] = fmaf(m0, v[q], acc0[q]);
                    acc1[q] = fmaf(m1, v[q], acc1[q]);
                }
                if (d >= 0.f) c1 += nn; else c0 += nn;
            }
        } while (false);
        if constexpr (ESC) shared_bins_in_order(kx, v, fb, nq, nb, lane);
    }
    __syncwarp();
    return __any_sync(0xffffffffu, seen);
}

// The general pair loop: range test near min_sep / max_sep, the bin of every pair with its
// FP32 error band, self tiles (j > i).  Bins kref and kref + 1 are summed in registers; other
// bins go to the warp's shared-memory bins in lane order (through stg when it is given);
// pairs inside an error band are left to the escalation pass (ESC = true), which decides
// them in FP64.
template <int GEO, int KIND, bool ESC>
__device__ __forceinline__ bool tile_general(const TravParams& T, const TileLeaves& LA,
                                             const TileLeaves& SB, const TileCtx& C, int lane,
                                             float (&acc0)[8], float (&acc1)[8], unsigned& c0,
                                             unsigned& c1, float* fb, unsigned long long* np,
                                             unsigned& n_acc, unsigned& n_pairs,
                                             unsigned& n_esc, float* stg)
{
    const int nbl = C.nbl, npt = C.na * nbl, nb = T.nbins, nq = T.nqf;
    const float ln2h = 0.5f * 0.69314718f;
    const float ckk = ln2h * T.finvbinsize;
    int ii = lane / nbl, jj = lane - ii * nbl;
    const int di = 32 / nbl, dj = 32 - di * nbl;
    bool seen = false;
    for (int p0 = 0; p0 < npt; p0 += 32) {
        const int i = ii, j = jj;
        jj += dj; ii += di;
        if (jj >= nbl) { jj -= nbl; ++ii; }
        int kx = -1;             // the shared-memory bin of this lane's pair, if it has one
        float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        do {                     // (break: no pair to add)
            if (p0 + lane >= npt || (C.self && j <= i)) break;
            if (!ESC) ++n_pairs;
            const float4 Pa = LA.P[i], Pb = SB.P[j];
            const float dx = Pa.x - Pb.x, dy = Pa.y - Pb.y;
            const float dz = GEO == TG_FLAT ? 0.f : Pa.z - Pb.z;
            const float dsq = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const float invc = rsqrtf(dsq);
            float r = dsq * invc;
            if (GEO == TG_ARC) r = C.small_chord ? arc_series(r) : arc_from_chord_sq(dsq);
            float lr = __log2f(r * r * C.inv_edge);
            bool unsure = false;
            int k = C.kref;
            if (!C.interior) {
                const float dr = C.emax + 4e-7f * r;
                if (r + dr < T.fminsep || r - dr >= T.fmaxsep) break;
                unsure = !(r - dr >= T.fminsep && r + dr < T.fmaxsep);
            }
            if (!unsure) {
                const float kk = lr * ckk;
                const float fk = floorf(kk);
                const float fr = kk - fk;
                const float band = fmaf(C.band_e, invc, C.band_0);
                k = C.kref + (int)fk;
                unsure = fr < band || fr > 1.f - band || k < 0;
                if (k >= nb) k = nb - 1;                    // the clamp of src/Corr2.cpp:514
            }
            if (unsure != ESC) {
                seen = seen || unsure;
                break;
            }
            float logr = fmaf(lr, ln2h, C.ledge);
            if constexpr (ESC) {
                ++n_esc;
                k = leaf_pair64(T, __float_as_int(LA.X[i].z), __float_as_int(SB.X[j].z), C.self,
                                &r, &logr);
                if (k < 0) break;
            }
            ++n_acc;
            const float4 Wa = LA.W[i], Wb = SB.W[j];
            const float ww = Wa.x * Wb.x;
            v[0] = ww; v[1] = ww * r; v[2] = ww * lr;
            if constexpr (KIND != TK_NN) {
                float x[4] = {0.f, 0.f, 0.f, 0.f}, sc;
                pair_products<GEO, KIND>(T, LA, SB, i, j, Pa, Wa, Pb, Wb, dx, dy, dz, dsq, r,
                                         logr, x, sc);
#pragma unroll
                for (int q = 0; q < 4; ++q) v[3 + q] = x[q] * sc;
            }
            const unsigned nn = (unsigned)__float_as_int(Wa.w) * (unsigned)__float_as_int(Wb.w);
            if (!ESC && k == C.kref) {
#pragma unroll
                for (int q = 0; q < 7; ++q) acc0[q] += v[q];
                c0 += nn;
            } else if (!ESC && k == C.kref + 1) {
#pragma unroll
                for (int q = 0; q < 7; ++q) acc1[q] += v[q];
                c1 += nn;
            } else {
                v[2] = ww * logr;   // the FP64 pair's own log r, or the tile edge's
                kx = k;
                if (!T.quick) atomicAdd(&np[k], (unsigned long long)nn);   // exact integer
            }
        } while (false);
        if (!ESC && stg) shared_bins_staged(kx, v, stg, fb, nq, nb, lane);
        else shared_bins_in_order(kx, v, fb, nq, nb, lane);
    }
    __syncwarp();
    return __any_sync(0xffffffffu, seen);
}

template <int GEO, int KIND>
__global__ void __launch_bounds__(TPB, TMINB) k_tiles(const __grid_constant__ TravParams T)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int gw = blockIdx.x * TWPB + wib;
    const int nq = T.nqf, nb = T.nbins;
    // Tiles waiting; an expansion launch that ran out of room counted past the capacity (and
    // raised DEV_SPILL_OVERFLOW), so never read beyond it.
    long long nt = (long long)*(volatile unsigned long long*)&T.tctl[0];
    if (nt > T.tile_cap) nt = T.tile_cap;
    // The bin edges (1 / edge^2 and log edge, nb + 1 each) for the whole block, then the
    // warps' areas.
    float* edge_sh = reinterpret_cast<float*>(smem);
    for (int q = threadIdx.x; q < 2 * (nb + 1); q += TPB)
        edge_sh[q] = q <= nb ? T.tile_edge[q] : T.tile_ledge[q - nb - 1];
    __syncthreads();
    unsigned char* wb = smem + edges_bytes(nb) + (size_t)wib * warp_bytes(nq, nb);
    float2* fd = reinterpret_cast<float2*>(wb);
    unsigned long long* np = reinterpret_cast<unsigned long long*>(fd + nq * nb);
    float* fb = reinterpret_cast<float*>(np + nb);
    TileLeaves& SA = *reinterpret_cast<TileLeaves*>(wb + bins_bytes(nq, nb));
    TileLeaves& SB = *(&SA + 1);
    const long long nwt = (long long)gridDim.x * TWPB;
    // Per-lane counters: at most ~10^8 pairs per lane in a launch, so 32 bits suffice.
    unsigned n_acc = 0, n_pairs = 0, n_esc = 0, n_tiles = 0, n_drop = 0;
    if ((long long)gw < nt) {
        for (int q = lane; q < nq * nb; q += 32) { fd[q] = make_float2(0.f, 0.f); fb[q] = 0.f; }
        for (int q = lane; q < nb; q += 32) np[q] = 0ull;
        __syncwarp();
        const float ckk = 0.5f * 0.69314718f * T.finvbinsize;   // bins per unit of log2(r^2)
        const bool quick = T.quick != 0;
        int since_flush = 0;
        for (long long t = gw; t < nt; t += nwt) {
            const int2 tile = T.tiles[t];
            TileCtx C;
            C.self = tile.y < 0;
            const int ia = tile.x, ib = C.self ? -2 - tile.y : tile.y;
            const TCell* cB = C.self ? T.c1 : T.c2;
            const int baseB = C.self ? T.leaf_base1 : T.leaf_base2;
            const float4 Aa = T.c1[ia].a, Ab = T.c1[ia].b, Ac = T.c1[ia].c, Ad = T.c1[ia].d;
            const float4 Ba = cB[ib].a, Bb = cB[ib].b, Bc = cB[ib].c, Bd = cB[ib].d;
            ++n_tiles;
            // Bounds of the tile's separations from the two cells' sizes (each point lies
            // within size of its cell's FP64 centre; 1e-6 covers the size's FP32 rounding).
            // Brute cells have infinite sizes: then the staged leaves give the bounds.
            const bool sized = Aa.w < 1e30f && Ba.w < 1e30f;
            float eA = 0.f, rA = 0.f, eB = 0.f, rB = 0.f;
            bool sA, sB;
            C.nbl = stage(cB, baseB, Bc, Bd, Ba.x, Ba.y, Ba.z, Bb.x, Bb.y, Bb.z, T.k2, SB, lane,
                          !sized, eB, rB, sB);
            C.na = C.nbl;
            // A's offsets are also taken from B's centre; D = centre A - centre B.
            const float Dx = (Aa.x - Ba.x) + (Ab.x - Bb.x), Dy = (Aa.y - Ba.y) + (Ab.y - Bb.y);
            const float Dz = GEO == TG_FLAT ? 0.f : (Aa.z - Ba.z) + (Ab.z - Bb.z);
            if (!C.self) {
                float on2;
                C.na = stage(T.c1, T.leaf_base1, Ac, Ad, Ba.x, Ba.y, Ba.z, Bb.x, Bb.y, Bb.z, T.k1,
                             SA, lane, !sized, eA, on2, sA);
                if (!sized) {
                    // Distance of A's leaves from A's centre.
                    __syncwarp();
                    for (int p = lane; p < C.na; p += 32) {
                        const float4 P = SA.P[p];
                        const float ux = P.x - Dx, uy = P.y - Dy, uz = P.z - Dz;
                        rA = fmaxf(rA, sqrtf(ux * ux + uy * uy + uz * uz));
                    }
                }
            } else {
                eA = eB; rA = rB; sA = sB;
            }
            __syncwarp();
            if (C.na == 0 || C.nbl == 0) continue;
            const TileLeaves& LA = C.self ? SB : SA;
            const float Dsq = Dx * Dx + Dy * Dy + Dz * Dz;
            const float Dn = Dsq > 0.f ? Dsq * rsqrtf(Dsq) : 0.f;    // |D| within 2 ulps
            float rAB;
            if (sized) {
                // emax bounds |FP32 d - d| of every pair: each offset within 2 ulps of its L1
                // size, the difference one more (a 1.5x margin), and L1 <= sqrt(3) L2.
                rAB = (Aa.w + Ba.w) * (1.f + 1e-6f) + 1e-30f;
                C.emax = 4.7e-7f * (Dn + rAB) + 1e-30f;
            } else {
                C.emax = 2.7e-7f * (warp_max(eA) + warp_max(eB)) + 1e-30f;
                rAB = warp_max(rA) + warp_max(rB);
            }
            // Every pair's separation lies within |D| +- rAB, up to the FP32 errors (slack).
            const float slack = C.emax + 2e-6f * (Dn + rAB);
            float lo = fmaxf(Dn - rAB - slack, 0.f), hi = Dn + rAB + slack;
            C.small_chord = hi < 0.25f;
            if (GEO == TG_ARC) {
                if (C.small_chord) { lo = arc_series(lo); hi = arc_series(hi); }
                else { lo = arc_from_chord_sq(lo * lo); hi = arc_from_chord_sq(hi * hi); }
            }
            lo *= 1.f - 1e-5f;
            hi *= 1.f + 1e-5f;
            if (lo >= T.fmaxsep || hi < T.fminsep) continue;   // no pair in range
            C.interior = lo >= T.fminsep && hi < T.fmaxsep;
            // Bins of the bounds: __log2f is within 2^-22 (or 2 ulps of a result <= 17) of
            // log2, far inside the 1e-5 margins above.
            const float lb = fmaxf(lo, T.fminsep), hb = fminf(hi, T.fmaxsep);
            int klo = (int)floorf(__log2f(lb * lb * T.finvminsepsq) * ckk);
            int khi = (int)floorf(__log2f(hb * hb * T.finvminsepsq) * ckk);
            klo = klo < 0 ? 0 : (klo > nb - 1 ? nb - 1 : klo);
            khi = khi < 0 ? 0 : (khi > nb - 1 ? nb - 1 : khi);
            C.kref = klo;
            C.inv_edge = edge_sh[klo];         // 1 / (lower edge of kref)^2
            C.ledge = edge_sh[nb + 1 + klo];   // log of that edge
            // Band (in bins) outside which the FP32 bin is certain: r's relative error
            // (emax / chord + 4e-7) and __log2f's (2^-22 absolute on [0.5, 2], else 2 ulps;
            // |log2| <= lmax here), the roundings of its argument and of kk.
            const float lmax = fmaxf(fabsf(__log2f(hi * hi * C.inv_edge)), 1.f);
            C.band_e = C.emax * T.finvbinsize;
            C.band_0 = 4e-7f * T.finvbinsize + (5e-7f + 4.2e-7f * lmax) * ckk + 1e-7f;
            float acc0[8], acc1[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) { acc0[q] = 0.f; acc1[q] = 0.f; }
            unsigned c0 = 0u, c1 = 0u;
            const bool fast = C.interior && klo == khi && !C.self &&
                              (GEO != TG_ARC || C.small_chord);
            const bool two = C.interior && khi == klo + 1 && !C.self &&
                             (GEO != TG_ARC || C.small_chord);
            if (fast) {
                tile_fast<GEO, KIND>(T, LA, SB, C, lane, acc0, c0);
                if (lane == 0) { n_pairs += C.na * C.nbl; n_acc += C.na * C.nbl; }
            } else if (two) {
                if (tile_two<GEO, KIND, false>(T, LA, SB, C, lane, acc0, acc1, c0, c1, fb, np,
                                               n_drop, n_esc))
                    tile_two<GEO, KIND, true>(T, LA, SB, C, lane, acc0, acc1, c0, c1, fb, np,
                                              n_drop, n_esc);
                if (lane == 0) { n_pairs += C.na * C.nbl; n_acc += C.na * C.nbl; }
            } else {
                // Staging for the shared bins: the A side's arrays of a self tile (unused), or
                // B's X array of a cross tile when the pair products do not read it (only the
                // generic projection does: the other class families, and GG in 3-d): B's
                // leaves are staged again before an escalation pass, which reads their ids.
                constexpr bool reads_xb = KIND == TK_GEN || (KIND == TK_GG && GEO == TG_3D);
                float* stg = C.self ? reinterpret_cast<float*>(SA.P)
                                    : (reads_xb ? nullptr : reinterpret_cast<float*>(SB.X));
                if (tile_general<GEO, KIND, false>(T, LA, SB, C, lane, acc0, acc1, c0, c1, fb, np,
                                                   n_acc, n_pairs, n_esc, stg)) {
                    if (!C.self && stg) {
                        const float4 Ba2 = cB[ib].a, Bb2 = cB[ib].b, Bc2 = cB[ib].c,
                                     Bd2 = cB[ib].d;
                        float u1, u2;
                        bool u3;
                        stage(cB, baseB, Bc2, Bd2, Ba2.x, Ba2.y, Ba2.z, Bb2.x, Bb2.y, Bb2.z,
                              T.k2, SB, lane, false, u1, u2, u3);
                        __syncwarp();
                    }
                    tile_general<GEO, KIND, true>(T, LA, SB, C, lane, acc0, acc1, c0, c1, fb, np,
                                                  n_acc, n_pairs, n_esc, nullptr);
                }
            }
            // The tile's register bins into the warp's FP32 bins.  With single-point leaves a
            // lane counts at most 32 pairs, so the warp's u32 sum is exact; list leaves add
            // their per-lane counts (n1 n2 each) one by one.
            const bool single = sA && sB;
            tile_bin_out(acc0, c0, C.kref, nq, nb, C.ledge, fb, np, quick, single, lane);
            if (!fast)
                tile_bin_out(acc1, c1, C.kref + 1, nq, nb, C.ledge, fb, np, quick, single, lane);
            if (++since_flush >= TFLUSH) {
                since_flush = 0;
                __syncwarp();
                for (int q = lane; q < nq * nb; q += 32) {
                    const float x = fb[q];
                    if (x != 0.f) {
                        float2 f = fd[q];
                        df_add(f, x);
                        fd[q] = f;
                        fb[q] = 0.f;
                    }
                }
            }
            __syncwarp();
        }
        __syncwarp();
        for (int q = lane; q < nq * nb; q += 32) {
            float2 f = fd[q];
            df_add(f, fb[q]);
            fd[q] = f;
        }
        __syncwarp();
        double* wa = T.wacc + (size_t)(T.tile_wbase + gw) * nq * nb;
        warp_add_totals(wa, fd, nq * nb, lane);
        unsigned long long* wn = T.wnp + (size_t)(T.tile_wbase + gw) * nb;
        for (int q = lane; q < nb; q += 32) wn[q] += np[q];
    }
    unsigned long long a64 = n_acc, p64 = n_pairs, e64 = n_esc, t64 = n_tiles, d64 = n_drop;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a64 += __shfl_xor_sync(0xffffffffu, a64, o);
        d64 += __shfl_xor_sync(0xffffffffu, d64, o);
        p64 += __shfl_xor_sync(0xffffffffu, p64, o);
        e64 += __shfl_xor_sync(0xffffffffu, e64, o);
    }
    a64 -= d64;   // pairs of two-bin tiles that the FP64 decision put out of range
    if (lane == 0 && t64) {
        if (T.wctr) {
            unsigned long long* w = T.wctr + (size_t)(T.tile_wbase + gw) * 8;
            const unsigned long long o1 = w[1], o4 = w[4], o5 = w[5], o6 = w[6];
            w[1] = o1 + a64;
            w[4] = o4 + t64;
            w[5] = o5 + p64;
            w[6] = o6 + e64;
        } else {
            atomicAdd(&T.counters[1], a64);
            atomicAdd(&T.tctl[2], t64);
            atomicAdd(&T.tctl[3], p64);
            atomicAdd(&T.tctl[4], e64);
        }
    }
    // The last block to finish empties the tile list for the next expansion launch.
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned long long prev = atomicAdd(&T.tctl[1], 1ull);
        if (prev == (unsigned long long)gridDim.x - 1) {
            T.tctl[0] = 0ull;
            T.tctl[1] = 0ull;
            __threadfence();
        }
    }
}

using TileKernel = void (*)(TravParams);

template <int GEO>
TileKernel pick_kind(const TravParams& T)
{
    if (T.k1 == DN && T.k2 == DN) return k_tiles<GEO, TK_NN>;
    if (T.k2 != DG) return k_tiles<GEO, TK_SC>;
    if (T.k1 == DG && T.s1 == 2 && T.s2 == 2) return k_tiles<GEO, TK_GG>;
    return k_tiles<GEO, TK_GEN>;
}

TileKernel pick(const TravParams& T)
{
    if (T.coords == FLAT) return pick_kind<TG_FLAT>(T);
    if (T.coords == SPHERE) return T.metric == ARC ? pick_kind<TG_ARC>(T) : pick_kind<TG_SPHEUC>(T);
    return pick_kind<TG_3D>(T);
}

}  // namespace

int tiles_grid(const TravParams& T, int* blocks, int* nwarps)
{
    if (T.tile_leaf > TCAP) {
        set_last_error("tile leaf size above the tile kernel's staging capacity");
        return 1;
    }
    int dev = 0, nsm = 0, per = 0;
    TC_CU(cudaGetDevice(&dev));
    TC_CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const size_t sm = edges_bytes(T.nbins) + warp_bytes(T.nqf, T.nbins) * TWPB;
    const TileKernel k = pick(T);
    if (sm > 48 * 1024)
        TC_CU(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    TC_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, TPB, sm));
    if (per < 1) per = 1;
    *blocks = nsm * per;
    *nwarps = *blocks * TWPB;
    return 0;
}

int launch_tiles(const TravParams& T, cudaStream_t st)
{
    const size_t sm = edges_bytes(T.nbins) + warp_bytes(T.nqf, T.nbins) * TWPB;
    count_launch();
    pick(T)<<<T.tile_blocks, TPB, sm, st>>>(T);
    return 0;
}

}  // namespace tc
