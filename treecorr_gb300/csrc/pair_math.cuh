// pair_math.cuh -- per-pair arithmetic shared by the traversal (traverse2pt.cu) and the
// leaf-pair tiles (tiles.cu): the reference's FP64 decision for one pair, the spin-s
// projections and the values an accepted pair adds, and double-float running sums.
#pragma once

#include <cmath>
#include <cstdint>

#include "tc_internal.cuh"
#include "traverse2pt.hpp"

namespace tc {

struct Decision {
    int act;         // ACT_*
    int k;           // bin (accept)
    float r, logr;   // separation and its log (accept)
};
enum : int { ACT_DROP = 0, ACT_ACCEPT = 1, ACT_SPLIT1 = 2, ACT_SPLIT2 = 3, ACT_SPLIT12 = 4,
             ACT_UNSURE = 5 };

// FP64 decision of process11, the reference's arithmetic on the FP64 centres.
static __device__ Decision decide64(const TravParams& T, double dsq, double s1, double s2)
{
    Decision D;
    D.act = ACT_DROP; D.k = -1; D.r = 0.f; D.logr = 0.f;
    double rsq = dsq;
    if (T.metric == ARC) {
        double L = sqrt(dsq);
        double th = 2. * asin(L / 2.);
        rsq = th * th;
    }
    const double s1ps2 = s1 + s2;
    if (rsq < T.minsepsq && s1ps2 < T.minsep && rsq < (T.minsep - s1ps2) * (T.minsep - s1ps2))
        return D;
    if (rsq >= T.maxsepsq && rsq >= (T.maxsep + s1ps2) * (T.maxsep + s1ps2)) return D;
    int k = -1;
    double r = 0., logr = 0.;
    bool single = false;
    if (s1ps2 == 0.) {
        single = true;
    } else {
        double s1ps2sq = s1ps2 * s1ps2;
        if (s1ps2sq > T.asq * rsq) single = false;
        else if (s1ps2sq <= T.bsq * rsq) single = true;
        else if (s1ps2sq > 0.25 * (T.binsize + T.b) * (T.binsize + T.b) * rsq) single = false;
        else {
            logr = 0.5 * log(rsq);
            double kk = (logr - T.logminsep) / T.binsize;
            int ik = int(kk);
            double frackk = kk - ik;
            double f = fmin(frackk, 1. - frackk);
            double t4 = f * T.binsize + T.b;
            double t5 = frackk * T.binsize + T.b - s1ps2sq / rsq;
            if (s1ps2sq > t4 * t4 * rsq) single = false;
            else if (s1ps2sq > t5 * t5 * rsq) single = false;
            else { single = true; k = ik; r = sqrt(rsq); }
        }
    }
    if (single) {
        if (!(rsq >= T.minsepsq && rsq < T.maxsepsq)) return D;
        if (k < 0) {
            r = sqrt(rsq);
            logr = log(r);
            k = int((logr - T.logminsep) / T.binsize);
        }
        if (k == T.nbins) --k;
        if (k < 0 || k >= T.nbins) return D;
        D.act = ACT_ACCEPT; D.k = k; D.r = float(r); D.logr = float(logr);
        return D;
    }
    double bsq_eff = rsq * fmin(T.bsq, T.asq);
    bool sw = s2 > s1;
    double big = sw ? s2 : s1, sml = sw ? s1 : s2;
    bool both = !(big > 2. * sml) && (sml * sml > 0.3422 * bsq_eff);
    D.act = both ? ACT_SPLIT12 : (sw ? ACT_SPLIT2 : ACT_SPLIT1);
    return D;
}

// spin-2 rotation conj(r^2)/|r|^2 (calculate_expmsialpha<2>, include/ProjectHelper.h:45-47).
__device__ __forceinline__ void expm2i(float rx, float ry, float& er, float& ei)
{
    float n = rx * rx + ry * ry;
    float inv = n > 0.f ? __fdividef(1.f, n) : 1.f;
    er = (rx * rx - ry * ry) * inv;
    ei = -2.f * rx * ry * inv;
}

__device__ __forceinline__ void cmul(float ar, float ai, float br, float bi, float& cr, float& ci)
{
    cr = ar * br - ai * bi;
    ci = ar * bi + ai * br;
}

// calculate_expmsialpha<s>(r) (include/ProjectHelper.h:33-60) in FP32: exp(-i s alpha) of
// the direction r; 0 for r = 0 and s > 0 (safe_norm).
__device__ __forceinline__ void expmsi(int s, float rx, float ry, float& er, float& ei)
{
    if (s == 2) { expm2i(rx, ry, er, ei); return; }
    if (s == 0) { er = 1.f; ei = 0.f; return; }
    const float n = rx * rx + ry * ry;
    const float inv = n > 0.f ? rsqrtf(n) : 1.f;
    const float ur = rx * inv, ui = -ry * inv;   // conj(r) / |r|
    if (s == 1) { er = ur; ei = ui; return; }
    const float u2r = ur * ur - ui * ui, u2i = 2.f * ur * ui;
    if (s == 3) { cmul(u2r, u2i, ur, ui, er, ei); return; }
    cmul(u2r, u2i, u2r, u2i, er, ei);
}

// The same in FP64 (ThreeD projections).
static __device__ void expmsi64(int s, double rx, double ry, double& er, double& ei)
{
    if (s == 0) { er = 1.; ei = 0.; return; }
    double n = rx * rx + ry * ry;
    if (!(n > 0.)) n = 1.;
    if (s == 2) { er = (rx * rx - ry * ry) / n; ei = -2. * rx * ry / n; return; }
    const double inv = 1. / sqrt(n);
    const double ur = rx * inv, ui = -ry * inv;
    if (s == 1) { er = ur; ei = ui; return; }
    const double u2r = ur * ur - ui * ui, u2i = 2. * ur * ui;
    if (s == 3) { er = u2r * ur - u2i * ui; ei = u2r * ui + u2i * ur; return; }
    er = u2r * u2r - u2i * u2i; ei = 2. * u2r * u2i;
}

// Spin projections for ThreeD coordinates in FP64 (positions normalised first,
// include/ProjectHelper.h:561-584): g2 by the direction at p2 with spin T.s2 and, when
// both1, g1 by the direction at p1 with spin T.s1 (negated for odd spin,
// include/ProjectHelper.h:386-387).
static __device__ void project3d64(const TravParams& T, int i, int j, bool both1, float& g1r,
                            float& g1i, float& g2r, float& g2i)
{
    double x1 = T.x1[i], y1 = T.y1[i], z1 = T.z1[i];
    double x2 = T.x2[j], y2 = T.y2[j], z2 = T.z2[j];
    double n1 = sqrt(x1 * x1 + y1 * y1 + z1 * z1), n2 = sqrt(x2 * x2 + y2 * y2 + z2 * z2);
    if (n1 == 0.) { x1 = 1.; y1 = 0.; z1 = 0.; } else { x1 /= n1; y1 /= n1; z1 /= n1; }
    if (n2 == 0.) { x2 = 1.; y2 = 0.; z2 = 0.; } else { x2 /= n2; y2 /= n2; z2 /= n2; }
    double dsq = (x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2) + (z1 - z2) * (z1 - z2);
    double ca = (z1 - z2) + 0.5 * z2 * dsq, sa = y1 * x2 - x1 * y2;   // direction at p2
    double er, ei;
    expmsi64(T.s2, sa, -ca, er, ei);
    double a = g2r, b = g2i;
    g2r = float(a * er - b * ei); g2i = float(a * ei + b * er);
    if (both1) {
        double cb = (z2 - z1) + 0.5 * z1 * dsq, sb = y2 * x1 - x2 * y1;   // direction at p1
        expmsi64(T.s1, sb, -cb, er, ei);
        if (T.s1 & 1) { er = -er; ei = -ei; }
        a = g1r; b = g1i;
        g1r = float(a * er - b * ei); g1i = float(a * ei + b * er);
    }
}

// The warp's running totals are double-float pairs (hi, lo), about 48 bits: FP32 adds with
// the rounding error kept (TwoSum, Knuth), instead of FP64 adds, whose rate on this GPU is
// 1/64 of FP32.  They become FP64 once per launch.
__device__ __forceinline__ void df_add(float2& a, float x)
{
    const float s = a.x + x;
    const float bp = s - a.x;
    a.y += (a.x - (s - bp)) + (x - bp);
    a.x = s;
}

__device__ __forceinline__ double df_value(float2 a) { return (double)a.x + (double)a.y; }

// wa[q] += fd[q] (as FP64) for q < n, by the lanes of a warp, eight values per lane at a
// time with all loads issued before the stores: a loop of plain += would wait for each
// read-modify-write in turn (the compiler cannot move a load past a store to the same
// array).
__device__ __forceinline__ void warp_add_totals(double* wa, const float2* fd, int n, int lane)
{
    for (int q0 = 0; q0 < n; q0 += 256) {
        double o[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int q = q0 + 32 * u + lane;
            o[u] = q < n ? wa[q] : 0.;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int q = q0 + 32 * u + lane;
            if (q < n) wa[q] = o[u] + df_value(fd[q]);
        }
    }
}

// The values an accepted pair adds (finishProcess and DirectHelper, src/Corr2.cpp:394-566):
// w1 w2, w1 w2 r, w1 w2 logr, n1 n2 and the correlation products.
__device__ __forceinline__ void accept_values(const TravParams& T, const TCell& A, const TCell& B,
                                              int i, int j, float dx, float dy, float dz,
                                              float dsq, float r, float logr, float (&av)[7],
                                              unsigned long long& acc_nn)
{
    const bool flat = (T.coords == FLAT);
    const float ww = A.b.w * B.b.w;
    av[0] = ww;
    av[1] = ww * r;
    av[2] = ww * logr;
    acc_nn = (unsigned long long)__float_as_int(A.c.z) * (unsigned long long)__float_as_int(B.c.z);
    // DirectHelper<0..3>, src/Corr2.cpp:394-474; getWK = w for N, w k for K.
    if (T.k1 == DN && T.k2 == DN) return;
    const float wk1 = T.k1 == DN ? A.b.w : A.c.x;
    if (T.k2 != DG) {
        av[3] = wk1 * (T.k2 == DN ? B.b.w : B.c.x);               // NK, KK
        return;
    }
    const bool both = (T.k1 == DG);
    float g1r = A.c.x, g1i = A.c.y, g2r = B.c.x, g2i = B.c.y;
    if (flat) {
        // ProjectHelper<Flat>::Project: r = p2 - p1 (ProjectHelper.h:108-147).
        float er, ei;
        expmsi(T.s2, -dx, -dy, er, ei);
        cmul(g2r, g2i, er, ei, g2r, g2i);
        if (both) cmul(g1r, g1i, er, ei, g1r, g1i);
    } else if (T.coords == SPHERE) {
        // ProjectHelper<Sphere>::Project, ProjectHelper.h:362-388, with the direction terms
        // written on accurate differences: y1*x2 - x1*y2 = x1*dy - y1*dx,  d = p1 - p2.
        const float x1 = A.a.x, y1 = A.a.y, z1 = A.a.z, z2 = B.a.z;
        const float sinA = x1 * dy - y1 * dx;
        const float cosA = dz + 0.5f * z2 * dsq;
        float e2r, e2i;
        expmsi(T.s2, sinA, -cosA, e2r, e2i);
        cmul(g2r, g2i, e2r, e2i, g2r, g2i);
        if (both) {
            const float cosB = -dz + 0.5f * z1 * dsq;
            float e1r, e1i;
            expmsi(T.s1, -sinA, -cosB, e1r, e1i);
            if (T.s1 & 1) { e1r = -e1r; e1i = -e1i; }
            cmul(g1r, g1i, e1r, e1i, g1r, g1i);
        }
    } else {
        project3d64(T, i, j, both, g1r, g1i, g2r, g2i);
    }
    if (!both) {
        // DirectHelper<2>: times -wk1 for G (the tangential shear), wk1 otherwise.
        const float f = T.s2 == 2 ? -wk1 : wk1;
        av[3] = g2r * f;
        av[4] = g2i * f;
        return;
    }
    // both_complex_prod(g2, g1), ProjectHelper.h:84-101.
    const float rr = g2r * g1r, ri = g2r * g1i, ir = g2i * g1r, ii = g2i * g1i;
    av[3] = rr + ii;   // xip
    av[4] = ri - ir;
    av[5] = rr - ii;   // xim
    av[6] = ri + ir;
}

}  // namespace tc
