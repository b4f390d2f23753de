// tc_oracle.cpp -- CPU oracle for the TreeCorr 2-point hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++ with OpenMP, the reference
// algorithm of TreeCorr (rmjarvis/TreeCorr) for:
//   * the ball-tree build (Field / Cell),
//   * the dual-tree 2-point traversal with the bin_slop accept/split rule,
//   * the per-pair accumulation for NN, KK and GG with Log binning,
// on Flat, ThreeD and Sphere coordinates with the Euclidean and Arc metrics.
// It is the checker for the CUDA path (tests/, __graft_entry__.smoke, bench.py's
// cpu_baseline and --impl reference arm), never part of the product.
//
// Each function cites the reference file:line it follows.  The restatement keeps the
// reference's precision choices (double positions and bin sums; float cell weight,
// size and payload), its summation order inside a cell, and std::partition /
// std::nth_element for the split so that cell membership and order match.
//
// Parity pin: tests/golden/ holds outputs of the reference C++ itself, built from its own
// sources by oracle/Makefile.ref and driven by tests/golden/make_golden.py; the CPU
// tests compare this oracle to those fixtures.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <limits>
#include <set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum { FLAT = 1, THREED = 2, SPHERE = 3 };             // include/Position.h:24
enum { EUCLIDEAN = 1, ARC = 4 };                       // include/Metric.h:29
enum { MIDDLE = 0, MEDIAN = 1, MEAN = 2, RANDOM = 3 }; // include/Cell.h:26
enum { DN = 0, DK = 1, DG = 2 };                       // N, K, G payloads

typedef std::complex<double> cd;

struct Pt {
    double x, y, z;   // position (Sphere: normalised, include/Position.h:235-257)
    double wpos;      // position weight (src/Field.cpp:146-152)
    float w;          // weight (include/Cell.h:93)
    float d1, d2;     // payload: wk (Cell.h:154) or wz (Cell.h:190), w-weighted
    long index;
};

struct Node {
    double x = 0., y = 0., z = 0.;
    float size = 0.f;  // include/Cell.h:346 (float)
    float w = 0.f;
    long n = 0;
    float d1 = 0.f, d2 = 0.f;
    int left = -1, right = -1;  // -1 for leaves
    long start = 0, end = 0;
    // Sums over the cell's leaves used by the multipole ww corrections:
    // calculateSumWSq / calculateSumWZSq / calculateSumAbsWZSq (src/Cell.cpp:138-168).
    double sumwsq = 0.;
    std::complex<double> sumwzsq = 0.;
    double sumabswzsq = 0.;
};

struct Field {
    int dtype, coords;
    int spin;        // complex data (Z, V, G, T, Q): 0, 1, 2, 3, 4
    double minsize, maxsize;
    int sm, brute, mintop, maxtop;
    std::vector<Pt> pts;
    std::vector<Node> nodes;
    std::vector<int> tops;
    double cx, cy, cz, sizesq;   // overall centre and size (src/Field.cpp:198-203)
    bool built;
};

inline double sqr(double x) { return x * x; }

// Position<Sphere>::normalize, include/Position.h:258-263.
inline void normalize3(double& x, double& y, double& z)
{
    double n = std::sqrt(x * x + y * y + z * z);
    if (n == 0.) { x = 1.; y = 0.; z = 0.; }
    else { x /= n; y /= n; z /= n; }
}

inline double coord_of(const Pt& p, int split)
{ return split == 2 ? p.z : split == 1 ? p.y : p.x; }

// BuildCellData, src/Cell.cpp:170-200: wpos-weighted centroid, sum of w.
void build_cell_data(const Field& f, long start, long end, Node& nd)
{
    const std::vector<Pt>& v = f.pts;
    double wp = v[start].wpos;
    double px = v[start].x * wp, py = v[start].y * wp, pz = v[start].z * wp;
    double ww = v[start].w;
    double sumwp = wp;
    for (long i = start + 1; i != end; ++i) {
        wp = v[i].wpos;
        px += v[i].x * wp; py += v[i].y * wp; pz += v[i].z * wp;
        sumwp += wp;
        ww += v[i].w;
    }
    nd.w = float(ww);
    if (sumwp != 0.) {
        px /= sumwp; py /= sumwp; pz /= sumwp;
        if (f.coords == SPHERE) normalize3(px, py, pz);
    } else {
        px = v[start].x; py = v[start].y; pz = v[start].z;
    }
    nd.x = px; nd.y = py; nd.z = pz;
    nd.n = end - start;
}

inline double safe_norm(const cd& z)
{
    double n = std::norm(z);
    return n > 0. ? n : 1.;
}

// calculate_expmsialpha<s>, include/ProjectHelper.h:33-60 (safe_norm 25-31): the spin-s
// rotation exp(-i s alpha) of a direction r.
inline cd expmsialpha(int s, const cd& r)
{
    switch (s) {
      case 0: return cd(1., 0.);
      case 1: return std::conj(r) / std::sqrt(safe_norm(r));
      case 2: return std::conj(r * r) / safe_norm(r);
      case 3: { cd r3 = r * r * r; return std::conj(r3) / std::sqrt(safe_norm(r3)); }
      default: { cd r2 = r * r; return std::conj(r2 * r2) / safe_norm(r2); }
    }
}
inline cd expmsialpha2(const cd& r) { return expmsialpha(2, r); }

// The public data kinds (N, K, G, Z, V, T, Q = 0..6) as (payload kind, spin).
inline int kind_of(int d) { return d <= 1 ? d : DG; }
inline int spin_of(int d)
{
    static const int spin[7] = {0, 0, 2, 0, 1, 3, 4};
    return (d >= 0 && d < 7) ? spin[d] : 0;
}

// finishAverages: SimpleSum (src/Cell.cpp:221-234) for Flat, ParallelTransportSum
// (src/Cell.cpp:276-321) for ThreeD/Sphere; K is a plain double sum (src/Cell.cpp:208-218).
void finish_averages(const Field& f, long start, long end, Node& nd)
{
    const std::vector<Pt>& v = f.pts;
    if (f.dtype == DK) {
        double s = 0.;
        for (long i = start; i < end; ++i) s += v[i].d1;
        nd.d1 = float(s); nd.d2 = 0.f;
    } else if (f.dtype == DG) {
        cd sum(0.);
        if (f.coords == FLAT) {
            for (long i = start; i < end; ++i) sum += cd(v[i].d1, v[i].d2);
        } else {
            // Position<Sphere> cen(center): normalises for ThreeD, copies for Sphere.
            double cx = nd.x, cy = nd.y, cz = nd.z;
            if (f.coords == THREED) normalize3(cx, cy, cz);
            double z1 = nd.z;   // center.getZ() on the un-normalised centre
            for (long i = start; i < end; ++i) {
                double px = v[i].x, py = v[i].y, pz = v[i].z;
                if (f.coords == THREED) normalize3(px, py, pz);
                double z2 = pz;
                double dsq = sqr(cx - px) + sqr(cy - py) + sqr(cz - pz);
                cd wz(v[i].d1, v[i].d2);
                if (dsq < 1.e-12) {
                    sum += wz;
                } else {
                    double cosA = (z1 - z2) + 0.5 * z2 * dsq;
                    double sinA = cy * px - cx * py;
                    double cosB = (z2 - z1) + 0.5 * z1 * dsq;
                    double sinB = sinA;
                    double cosbeta = -cosA * cosB + sinA * sinB;
                    double sinbeta = sinA * cosB + cosA * sinB;
                    sum += wz * expmsialpha(f.spin, cd(cosbeta, sinbeta));
                }
            }
        }
        nd.d1 = float(sum.real()); nd.d2 = float(sum.imag());
    } else {
        nd.d1 = nd.d2 = 0.f;
    }
}

// CalculateSizeSq, src/Cell.cpp:89-100.
double calc_sizesq(const Field& f, const Node& nd, long start, long end)
{
    double s = 0.;
    for (long i = start; i < end; ++i) {
        const Pt& p = f.pts[i];
        double d = sqr(nd.x - p.x) + sqr(nd.y - p.y);
        if (f.coords != FLAT) d += sqr(nd.z - p.z);
        if (d > s) s = d;
    }
    return s;
}

// SplitData + SplitDataCore<Middle/Median/Mean>, src/Cell.cpp:426-554, with
// Bounds::getSplit (include/Bounds.h:65-66, 133-141).
long split_data(Field& f, long start, long end, const Node& nd, int sm)
{
    std::vector<Pt>& v = f.pts;
    double xmin = v[start].x, xmax = xmin, ymin = v[start].y, ymax = ymin;
    double zmin = v[start].z, zmax = zmin;
    for (long i = start + 1; i < end; ++i) {
        xmin = std::min(xmin, v[i].x); xmax = std::max(xmax, v[i].x);
        ymin = std::min(ymin, v[i].y); ymax = std::max(ymax, v[i].y);
        zmin = std::min(zmin, v[i].z); zmax = std::max(zmax, v[i].z);
    }
    int split;
    if (f.coords == FLAT) {
        split = (ymax - ymin) > (xmax - xmin) ? 1 : 0;
    } else {
        double xr = xmax - xmin, yr = ymax - ymin, zr = zmax - zmin;
        split = yr > xr ? (zr > yr ? 2 : 1) : (zr > xr ? 2 : 0);
    }
    long mid;
    if (sm == MEDIAN) {
        mid = (start + end) / 2;
        std::nth_element(v.begin() + start, v.begin() + mid, v.begin() + end,
                         [split](const Pt& a, const Pt& b)
                         { return coord_of(a, split) < coord_of(b, split); });
        return mid;
    }
    double splitvalue;
    if (sm == MIDDLE) {
        splitvalue = split == 2 ? (zmax + zmin) / 2. : split == 1 ? (ymax + ymin) / 2.
                                                                 : (xmax + xmin) / 2.;
    } else {
        splitvalue = split == 2 ? nd.z : split == 1 ? nd.y : nd.x;
    }
    auto it = std::partition(v.begin() + start, v.begin() + end,
                             [split, splitvalue](const Pt& p)
                             { return coord_of(p, split) < splitvalue; });
    mid = it - v.begin();
    if (mid == start || mid == end) return split_data(f, start, end, nd, MEDIAN);
    return mid;
}

// BuildCell, src/Cell.cpp:556-615.  Nodes are stored depth first from `next`.
int build_cell(Field& f, double minsizesq, long start, long end, const Node* data,
               double sizesq, int& next)
{
    int id = next++;
    Node nd;
    if (end - start == 1) {
        const Pt& p = f.pts[start];
        nd.x = p.x; nd.y = p.y; nd.z = p.z; nd.w = p.w; nd.n = 1;
        nd.d1 = p.d1; nd.d2 = p.d2;
        nd.size = 0.f; nd.left = nd.right = -1; nd.start = start; nd.end = end;
        f.nodes[id] = nd;
        return id;
    }
    if (data) {
        nd = *data;
    } else {
        build_cell_data(f, start, end, nd);
        finish_averages(f, start, end, nd);
        sizesq = calc_sizesq(f, nd, start, end);
    }
    nd.start = start; nd.end = end;
    if (sizesq > minsizesq) {
        double size = f.brute ? std::numeric_limits<double>::max() : std::sqrt(sizesq);
        nd.size = float(size);
        long mid = split_data(f, start, end, nd, f.sm);
        nd.left = build_cell(f, minsizesq, start, mid, nullptr, 0., next);
        nd.right = build_cell(f, minsizesq, mid, end, nullptr, 0., next);
    } else {
        nd.size = 0.f;
        nd.left = nd.right = -1;
    }
    f.nodes[id] = nd;
    return id;
}

// The leaf sums of a subtree, bottom up: a leaf (size 0 or one point) contributes
// w^2, wz^2, |wz|^2; a parent is left + right, as the reference's recursion adds them.
void leaf_sums(Field& f, int id)
{
    Node& nd = f.nodes[id];
    if (nd.size == 0.f || nd.n == 1 || nd.left < 0) {
        double w = nd.w;
        std::complex<double> wz(nd.d1, nd.d2);
        nd.sumwsq = w * w;
        nd.sumwzsq = wz * wz;
        nd.sumabswzsq = std::norm(wz);
        return;
    }
    leaf_sums(f, nd.left);
    leaf_sums(f, nd.right);
    const Node& L = f.nodes[nd.left];
    const Node& R = f.nodes[nd.right];
    nd.sumwsq = L.sumwsq + R.sumwsq;
    nd.sumwzsq = L.sumwzsq + R.sumwzsq;
    nd.sumabswzsq = L.sumabswzsq + R.sumabswzsq;
}

struct TopInfo { Node data; double sizesq; long start, end; };

// SetupTopLevelCells, src/Field.cpp:27-81.
void setup_top(Field& f, double maxsizesq, long start, long end, int mintop, int maxtop,
               std::vector<TopInfo>& tops)
{
    Node nd;
    double sizesq;
    if (end - start == 1) {
        const Pt& p = f.pts[start];
        nd.x = p.x; nd.y = p.y; nd.z = p.z; nd.w = p.w; nd.n = 1;
        nd.d1 = p.d1; nd.d2 = p.d2;
        sizesq = 0.;
    } else {
        build_cell_data(f, start, end, nd);
        sizesq = calc_sizesq(f, nd, start, end);
    }
    if (sizesq == 0 || (sizesq <= maxsizesq && mintop <= 0) || maxtop <= 0) {
        if (end - start > 1) finish_averages(f, start, end, nd);
        tops.push_back(TopInfo{nd, sizesq, start, end});
    } else {
        long mid = split_data(f, start, end, nd, f.sm);
        setup_top(f, maxsizesq, start, mid, mintop - 1, maxtop - 1, tops);
        setup_top(f, maxsizesq, mid, end, mintop - 1, maxtop - 1, tops);
    }
}

// Field::DoBuildCells, src/Field.cpp:230-277.
void build_cells(Field& f)
{
    if (f.built) return;
    f.built = true;
    long n = (long)f.pts.size();
    if (n == 0) return;
    double minsizesq = f.minsize * f.minsize;
    double maxsizesq = f.maxsize * f.maxsize;
    std::vector<TopInfo> tops;
    setup_top(f, maxsizesq, 0, n, f.mintop, f.maxtop, tops);
    f.nodes.assign(2 * n, Node());
    f.tops.resize(tops.size());
    long ntop = (long)tops.size();
#pragma omp parallel for schedule(dynamic)
    for (long i = 0; i < ntop; ++i) {
        int next = int(2 * tops[i].start);
        f.tops[i] = build_cell(f, minsizesq, tops[i].start, tops[i].end,
                               (tops[i].end - tops[i].start > 1) ? &tops[i].data : nullptr,
                               tops[i].sizesq, next);
        leaf_sums(f, f.tops[i]);
    }
}

// ---------------------------------------------------------------------------------------
// 2-point traversal (src/Corr2.cpp:146-566, include/BinType.h:40-156, include/Split.h:82-101)

struct Accum {
    int nbins;
    long long accepted = 0;
    std::vector<double> xi0, xi1, xi2, xi3, meanr, meanlogr, weight, npairs;
    explicit Accum(int nb) : nbins(nb), xi0(nb), xi1(nb), xi2(nb), xi3(nb), meanr(nb),
                             meanlogr(nb), weight(nb), npairs(nb) {}
};

struct Params {
    int dtype, coords, metric, quick, nbins;
    int k1, k2, s1, s2;   // payload kind (DN/DK/DG) and spin of the two fields
    double minsep, maxsep, binsize, b, a;
    double logminsep, halfminsep, minsepsq, maxsepsq, bsq, asq;
    // 3-point: 1 when vertex 1 is an N or K field and the pairs G fields (NGG, KGG): G_n
    // without the +-1 buffer, self-pair sums without z^2 (Corr3::getMP2 buffer 0,
    // src/Corr3.cpp:1307-1313); its "shear" (d1, d2) then holds (w1 or w1 k1, 0).
    int vreal = 0;
};

// MetricHelper<Euclidean>::DistSq (include/Metric.h:143-147, 202-207) and
// MetricHelper<Arc>::DistSq for Sphere (include/Metric.h:668-682).
inline double dist_sq(const Params& P, const Node& c1, const Node& c2)
{
    double dx = c1.x - c2.x, dy = c1.y - c2.y;
    if (P.coords == FLAT) return dx * dx + dy * dy;
    double dz = c1.z - c2.z;
    double dsq = dx * dx + dy * dy + dz * dz;
    if (P.metric == ARC) {
        double L = std::sqrt(dsq);
        double theta = 2. * std::asin(L / 2.);
        return theta * theta;
    }
    return dsq;
}

// ProjectHelper<Sphere>::calculate_direction, include/ProjectHelper.h:272-345.
inline cd calc_direction(double x1, double y1, double z1, double x2, double y2, double z2)
{
    double dsq = sqr(x1 - x2) + sqr(y1 - y2) + sqr(z1 - z2);
    double cosA = (z1 - z2) + 0.5 * z2 * dsq;
    double sinA = y1 * x2 - x1 * y2;
    return cd(sinA, -cosA);
}

// The direction term of a spin-s value at c2 (ProjectHelper<C>::Project, one value):
// Flat: r = p2 - p1 (include/ProjectHelper.h:108-114); Sphere: the direction at p2
// (370-376); ThreeD: the same on the normalised positions (561-569).
inline cd project_one(const Params& P, int s, const Node& c1, const Node& c2)
{
    if (P.coords == FLAT) return expmsialpha(s, cd(c2.x - c1.x, c2.y - c1.y));
    double x1 = c1.x, y1 = c1.y, z1 = c1.z, x2 = c2.x, y2 = c2.y, z2 = c2.z;
    if (P.coords == THREED) { normalize3(x1, y1, z1); normalize3(x2, y2, z2); }
    return expmsialpha(s, calc_direction(x1, y1, z1, x2, y2, z2));
}

// Corr2::finishProcess + DirectHelper<0..3>, src/Corr2.cpp:394-566.
void finish_process(const Params& P, const Node& c1, const Node& c2, double r, double logr,
                    int k, Accum& A)
{
    double ww = double(c1.w) * double(c2.w);
    A.weight[k] += ww;
    if (!P.quick) {
        A.npairs[k] += double(c1.n) * double(c2.n);
        A.meanr[k] += ww * r;
        A.meanlogr[k] += ww * logr;
    }
    // getWK: w for N, w k for K (include/ProjectHelper.h:73-79).
    auto wk = [](const Node& c, int kind) { return kind == DN ? double(c.w) : double(c.d1); };
    if (P.k1 == DN && P.k2 == DN) return;
    if (P.k2 != DG) {
        // DirectHelper<1>: NK, KK.
        A.xi0[k] += wk(c1, P.k1) * wk(c2, P.k2);
    } else if (P.k1 != DG) {
        // DirectHelper<2>: the spin-s value at c2 projected to the line of the pair, times
        // -wk1 for G (tangential shear) and wk1 otherwise.
        cd g2(c2.d1, c2.d2);
        g2 *= project_one(P, P.s2, c1, c2);
        g2 *= (P.s2 == 2 ? -1. : 1.) * wk(c1, P.k1);
        A.xi0[k] += g2.real();
        A.xi1[k] += g2.imag();
    } else {
        // DirectHelper<3>: both values projected, then both_complex_prod(g2, g1).
        cd g1(c1.d1, c1.d2), g2(c2.d1, c2.d2);
        if (P.coords == FLAT) {
            // ProjectHelper<Flat>::Project, include/ProjectHelper.h:126-136.
            cd e = expmsialpha(P.s1, cd(c2.x - c1.x, c2.y - c1.y));
            g1 *= e; g2 *= e;
        } else {
            // ProjectHelper<Sphere>::Project(c1,c2,z1,z2), include/ProjectHelper.h:370-388;
            // ThreeD first normalises both positions (include/ProjectHelper.h:570-584).
            double x1 = c1.x, y1 = c1.y, z1 = c1.z, x2 = c2.x, y2 = c2.y, z2 = c2.z;
            if (P.coords == THREED) { normalize3(x1, y1, z1); normalize3(x2, y2, z2); }
            g2 *= expmsialpha(P.s2, calc_direction(x1, y1, z1, x2, y2, z2));
            g1 *= expmsialpha(P.s1, calc_direction(x2, y2, z2, x1, y1, z1));
            if (P.s1 == 1 || P.s1 == 3) g1 = -g1;
        }
        // both_complex_prod(g2, g1), include/ProjectHelper.h:84-101.
        double z1rz2r = g2.real() * g1.real();
        double z1rz2i = g2.real() * g1.imag();
        double z1iz2r = g2.imag() * g1.real();
        double z1iz2i = g2.imag() * g1.imag();
        A.xi2[k] += z1rz2r - z1iz2i;   // xim = g1 g2
        A.xi3[k] += z1rz2i + z1iz2r;
        A.xi0[k] += z1rz2r + z1iz2i;   // xip = g1 conj(g2)
        A.xi1[k] += z1rz2i - z1iz2r;
    }
}

// BaseCorr2::directProcess11, src/Corr2.cpp:476-525.
inline void direct_process(const Params& P, const Node& c1, const Node& c2, double rsq, int k,
                           double r, double logr, Accum& A)
{
    if (k < 0) {
        r = std::sqrt(rsq);
        logr = std::log(r);
        k = int((logr - P.logminsep) / P.binsize);
    }
    if (k == P.nbins) --k;
    if (k < 0 || k >= P.nbins) return;   // Assert() in the reference; never true in range
    ++A.accepted;
    finish_process(P, c1, c2, r, logr, k, A);
}

// BinTypeHelper<Log>::singleBin, include/BinType.h:93-151.
inline bool single_bin(const Params& P, double rsq, double s1ps2, int& ik, double& r,
                       double& logr)
{
    if (s1ps2 == 0.) return true;
    double s1ps2sq = s1ps2 * s1ps2;
    if (s1ps2sq > P.asq * rsq) return false;
    if (s1ps2sq <= P.bsq * rsq) return true;
    if (s1ps2sq > 0.25 * sqr(P.binsize + P.b) * rsq) return false;
    logr = 0.5 * std::log(rsq);
    double kk = (logr - P.logminsep) / P.binsize;
    ik = int(kk);
    double frackk = kk - ik;
    double f = std::min(frackk, 1. - frackk);
    if (s1ps2sq > sqr(f * P.binsize + P.b) * rsq) return false;
    if (s1ps2sq > sqr(frackk * P.binsize + P.b - s1ps2sq / rsq) * rsq) return false;
    r = std::sqrt(rsq);
    return true;
}

// CalcSplitSq, include/Split.h:82-101.
inline void calc_split_sq(bool& split1, bool& split2, double s1, double s2, double bsq)
{
    const double splitfactorsq = 0.3422;
    if (s2 > s1) {
        calc_split_sq(split2, split1, s2, s1, bsq);
    } else if (s1 > 2. * s2) {
        split1 = true;
    } else {
        split1 = true;
        split2 = s2 * s2 > splitfactorsq * bsq;
    }
}

// BaseCorr2::process11, src/Corr2.cpp:308-389 (Log binning, Euclidean/Arc: no rpar).
void process11(const Params& P, const Field& f1, const Field& f2, int i1, int i2, Accum& A)
{
    const Node& c1 = f1.nodes[i1];
    const Node& c2 = f2.nodes[i2];
    if (c1.w == 0.f || c2.w == 0.f) return;
    double s1 = c1.size, s2 = c2.size;
    const double rsq = dist_sq(P, c1, c2);
    const double s1ps2 = s1 + s2;
    // tooSmallDist / tooLargeDist, include/BinType.h:70-82.
    if (rsq < P.minsepsq && s1ps2 < P.minsep && rsq < sqr(P.minsep - s1ps2)) return;
    if (rsq >= P.maxsepsq && rsq >= sqr(P.maxsep + s1ps2)) return;
    int k = -1;
    double r = 0., logr = 0.;
    if (single_bin(P, rsq, s1ps2, k, r, logr)) {
        if (rsq >= P.minsepsq && rsq < P.maxsepsq)
            direct_process(P, c1, c2, rsq, k, r, logr, A);
    } else {
        bool split1 = false, split2 = false;
        double bsq_eff = rsq * std::min(P.bsq, P.asq);
        calc_split_sq(split1, split2, s1, s2, bsq_eff);
        if (split1 && split2) {
            process11(P, f1, f2, c1.left, c2.left, A);
            process11(P, f1, f2, c1.left, c2.right, A);
            process11(P, f1, f2, c1.right, c2.left, A);
            process11(P, f1, f2, c1.right, c2.right, A);
        } else if (split1) {
            process11(P, f1, f2, c1.left, i2, A);
            process11(P, f1, f2, c1.right, i2, A);
        } else {
            process11(P, f1, f2, i1, c2.left, A);
            process11(P, f1, f2, i1, c2.right, A);
        }
    }
}

// BaseCorr2::process2, src/Corr2.cpp:290-306.
void process2(const Params& P, const Field& f, int i, Accum& A)
{
    const Node& c = f.nodes[i];
    if (c.w == 0.f) return;
    if (c.size <= P.halfminsep) return;
    process2(P, f, c.left, A);
    process2(P, f, c.right, A);
    process11(P, f, f, c.left, c.right, A);
}

void add_into(const Accum& A, double* xi0, double* xi1, double* xi2, double* xi3,
              double* meanr, double* meanlogr, double* weight, double* npairs)
{
    for (int k = 0; k < A.nbins; ++k) {
        if (xi0) xi0[k] += A.xi0[k];
        if (xi1) xi1[k] += A.xi1[k];
        if (xi2) xi2[k] += A.xi2[k];
        if (xi3) xi3[k] += A.xi3[k];
        meanr[k] += A.meanr[k];
        meanlogr[k] += A.meanlogr[k];
        weight[k] += A.weight[k];
        npairs[k] += A.npairs[k];
    }
}

// dpair: the two public data kinds as d1 * 16 + d2.
Params make_params(int dpair, int coords, int metric, int quick, double minsep, double maxsep,
                   int nbins, double binsize, double b, double a)
{
    Params P;
    const int d1 = dpair >> 4, d2 = dpair & 15;
    P.dtype = kind_of(d1);
    P.k1 = kind_of(d1); P.k2 = kind_of(d2); P.s1 = spin_of(d1); P.s2 = spin_of(d2);
    P.coords = coords; P.metric = metric; P.quick = quick; P.nbins = nbins;
    P.minsep = minsep; P.maxsep = maxsep; P.binsize = binsize; P.b = b; P.a = a;
    // BaseCorr2 constructor, src/Corr2.cpp:55-80.
    P.logminsep = std::log(minsep);
    P.halfminsep = 0.5 * minsep;
    P.minsepsq = minsep * minsep;
    P.maxsepsq = maxsep * maxsep;
    P.bsq = b * b;
    P.asq = a * a;
    return P;
}


// ---------------------------------------------------------------------------------------
// 3-point multipole algorithm for GGG, LogMultipole auto-correlation
// (BaseCorr3::multipole, src/Corr3.cpp:1124-1175, and the functions it calls).

struct Out3 {
    int nbins, maxn, size;
    std::vector<double> gam[8];          // gam0r, gam0i, gam1r, gam1i, gam2r, gam2i, gam3r, gam3i
    std::vector<double> meand2, meanlogd2, meand3, meanlogd3, weight, weight_im, ntri;
    Out3(int nb, int mn) : nbins(nb), maxn(mn), size(nb * nb * (2 * mn + 1))
    {
        for (auto& g : gam) g.assign(size, 0.);
        meand2.assign(size, 0.); meanlogd2.assign(size, 0.); meand3.assign(size, 0.);
        meanlogd3.assign(size, 0.); weight.assign(size, 0.); weight_im.assign(size, 0.);
        ntri.assign(size, 0.);
    }
    void add(const Out3& o)
    {
        for (int q = 0; q < 8; ++q) for (int i = 0; i < size; ++i) gam[q][i] += o.gam[q][i];
        for (int i = 0; i < size; ++i) {
            meand2[i] += o.meand2[i]; meanlogd2[i] += o.meanlogd2[i];
            meand3[i] += o.meand3[i]; meanlogd3[i] += o.meanlogd3[i];
            weight[i] += o.weight[i]; weight_im[i] += o.weight_im[i]; ntri[i] += o.ntri[i];
        }
    }
};

// MultipoleScratch<GData> with ww = true, buffer = 1 (include/MultipoleScratch.h:36-125,
// 296-383; Corr3::getMP2, src/Corr3.cpp:1307-1313).
struct MPS {
    int nbins, maxn;
    bool real = false;   // the list's cells carry a real payload (N: w, K: w k), not rotated
    std::vector<cd> Wn, Gn, gg0, gg1, gg2;
    std::vector<double> npairs, sumw, sumwr, sumwlogr, sumww, sumwwr, sumwwlogr;
    MPS(int nb, int mn) : nbins(nb), maxn(mn) { clear(); }
    void clear()
    {
        Wn.assign(nbins * (maxn + 1), 0.);
        Gn.assign(nbins * (2 * (maxn + 1) + 1), 0.);
        gg0.assign(nbins, 0.); gg1.assign(nbins, 0.); gg2.assign(nbins, 0.);
        npairs.assign(nbins, 0.); sumw.assign(nbins, 0.); sumwr.assign(nbins, 0.);
        sumwlogr.assign(nbins, 0.); sumww.assign(nbins, 0.); sumwwr.assign(nbins, 0.);
        sumwwlogr.assign(nbins, 0.);
    }
    int widx(int k) const { return k * (maxn + 1); }
    int gidx(int k) const { return (2 * k + 1) * (maxn + 1) + k; }   // index of n = 0
    cd G(int k, int n) const { return Gn[gidx(k) + n]; }
};

// ExpIPhi: Flat (p2-p1)/r (include/ProjectHelper.h:264-266); Sphere: the normalised
// direction of p2 seen from p1 (526-535); ThreeD normalises the positions first (688-697).
inline cd exp_i_phi(const Params& P, const Node& c1, const Node& c2, double r)
{
    if (P.coords == FLAT) return cd(c2.x - c1.x, c2.y - c1.y) / r;
    double x1 = c1.x, y1 = c1.y, z1 = c1.z, x2 = c2.x, y2 = c2.y, z2 = c2.z;
    if (P.coords == THREED) { normalize3(x1, y1, z1); normalize3(x2, y2, z2); }
    cd z = calc_direction(x2, y2, z2, x1, y1, z1);
    double n = std::norm(z);
    if (!(n > 0.)) n = 1.;
    return z / std::sqrt(n);
}

// The spin-2 projection of c2's shear onto the c1-c2 line (ProjectWithSq).
inline cd project2(const Params& P, const Node& c1, const Node& c2)
{
    if (P.coords == FLAT) return expmsialpha2(cd(c2.x - c1.x, c2.y - c1.y));
    double x1 = c1.x, y1 = c1.y, z1 = c1.z, x2 = c2.x, y2 = c2.y, z2 = c2.z;
    if (P.coords == THREED) { normalize3(x1, y1, z1); normalize3(x2, y2, z2); }
    return expmsialpha2(calc_direction(x1, y1, z1, x2, y2, z2));
}

// Corr3::calculateGn + MultipoleScratch<GData>::calculateGn, src/Corr3.cpp:1681-1704,
// 1767-1828.
void calculate_gn(const Params& P, const Node& c1, const Node& c2, double r, double logr,
                  int k, MPS& mp)
{
    double n = double(c2.n), w = c2.w;
    mp.npairs[k] += n;
    mp.sumw[k] += w;
    mp.sumwr[k] += w * r;
    mp.sumwlogr[k] += w * logr;
    double wsq = c2.sumwsq;
    mp.sumww[k] += wsq;
    mp.sumwwr[k] += wsq * r;
    mp.sumwwlogr[k] += wsq * logr;
    cd wg(c2.d1, c2.d2);
    cd z = exp_i_phi(P, c1, c2, r);
    cd e = mp.real ? cd(1., 0.) : project2(P, c1, c2);
    cd wgsq = c2.sumwzsq;
    wg *= e;
    wgsq *= e * e;
    cd abswgsq = c2.sumabswzsq;
    cd zsq = P.vreal ? cd(1., 0.) : z * z;
    mp.gg0[k] += wgsq * std::conj(zsq);
    mp.gg1[k] += wgsq * zsq;
    mp.gg2[k] += abswgsq * std::conj(zsq);
    int iw = mp.widx(k);
    mp.Wn[iw] += w;
    cd t = w;
    for (int m = 1; m <= mp.maxn; ++m) { t *= z; mp.Wn[iw + m] += t; }
    int ig = mp.gidx(k);
    mp.Gn[ig] += wg;
    t = wg;
    for (int m = 1; m <= mp.maxn + 1; ++m) { t *= z; mp.Gn[ig + m] += t; }
    t = wg;
    cd zc = std::conj(z);
    for (int m = 1; m <= mp.maxn + 1; ++m) { t *= zc; mp.Gn[ig - m] += t; }
}

// Corr3::calculateZeta (src/Corr3.cpp:1861-1974) with MultipoleHelper<5>::CalculateZeta
// (src/Corr3.cpp:2585-2843) for the rows k2 in [kstart, mink_zeta).  Every written entry
// (a, b, n) with min(a,b) in that range equals the direct Porth et al. product, which is
// what the reference's unrolled loops compute; the k2 = k3 entries subtract the
// self-pair sums.
void calculate_zeta(const Params& P, const Node& c1, const MPS& mp, int kstart, int mink_zeta,
                    Out3& O)
{
    const int nb = mp.nbins, maxn = mp.maxn, nn = 2 * maxn + 1;
    const double w1 = c1.w;
    const cd wg1(c1.d1, c1.d2);
    auto idx = [&](int a, int b, int n) { return (a * nb + b) * nn + maxn + n; };
    if (!P.quick) {
        double n1 = double(c1.n);
        for (int k2 = kstart; k2 < mink_zeta; ++k2) {
            int i22 = idx(k2, k2, 0);
            O.ntri[i22] += n1 * mp.npairs[k2] * (mp.npairs[k2] - 1);
            O.meand2[i22] += w1 * (mp.sumw[k2] * mp.sumwr[k2] - mp.sumwwr[k2]);
            O.meanlogd2[i22] += w1 * (mp.sumw[k2] * mp.sumwlogr[k2] - mp.sumwwlogr[k2]);
            O.meand3[i22] += w1 * (mp.sumw[k2] * mp.sumwr[k2] - mp.sumwwr[k2]);
            O.meanlogd3[i22] += w1 * (mp.sumw[k2] * mp.sumwlogr[k2] - mp.sumwwlogr[k2]);
            for (int k3 = k2 + 1; k3 < nb; ++k3) {
                int i23 = idx(k2, k3, 0), i32 = idx(k3, k2, 0);
                double nnn = n1 * mp.npairs[k2] * mp.npairs[k3];
                O.ntri[i23] += nnn; O.ntri[i32] += nnn;
                double ww12 = w1 * mp.sumw[k2], ww13 = w1 * mp.sumw[k3];
                O.meand2[i23] += ww13 * mp.sumwr[k2]; O.meand3[i32] += ww13 * mp.sumwr[k2];
                O.meanlogd2[i23] += ww13 * mp.sumwlogr[k2]; O.meanlogd3[i32] += ww13 * mp.sumwlogr[k2];
                O.meand3[i23] += ww12 * mp.sumwr[k3]; O.meand2[i32] += ww12 * mp.sumwr[k3];
                O.meanlogd3[i23] += ww12 * mp.sumwlogr[k3]; O.meanlogd2[i32] += ww12 * mp.sumwlogr[k3];
            }
        }
    }
    // weight (Porth et al. eq. 27): W[a,b,n] = w1 Wn[a,n] conj(Wn[b,n]), Wn[-n] = conj(Wn[n]).
    auto Wn = [&](int k, int n) { return n >= 0 ? mp.Wn[mp.widx(k) + n] : std::conj(mp.Wn[mp.widx(k) - n]); };
    for (int k2 = kstart; k2 < mink_zeta; ++k2) {
        for (int n = -maxn; n <= maxn; ++n)
            O.weight[idx(k2, k2, n)] += w1 * (std::norm(Wn(k2, n)) - mp.sumww[k2]);
        for (int k3 = k2 + 1; k3 < nb; ++k3) {
            for (int n = -maxn; n <= maxn; ++n) {
                cd a = w1 * Wn(k2, n) * std::conj(Wn(k3, n));
                O.weight[idx(k2, k3, n)] += a.real(); O.weight_im[idx(k2, k3, n)] += a.imag();
                cd b = w1 * Wn(k3, n) * std::conj(Wn(k2, n));
                O.weight[idx(k3, k2, n)] += b.real(); O.weight_im[idx(k3, k2, n)] += b.imag();
            }
        }
    }
    // gam0..3 (Porth et al. eqs. 21, 23-25 with the projection already applied to G).  For
    // NGG / KGG (s = 0, wg1 = w1 or w1 k1) g0 and g2 are MultipoleHelper<2>'s gam0 and gam2
    // (src/Corr3.cpp:2216-2317), its zeta0 and zeta1.
    const int s = P.vreal ? 0 : 1;
    auto add_gam = [&](int a, int b, bool diag) {
        for (int n = -maxn; n <= maxn; ++n) {
            cd g0 = wg1 * mp.G(a, n - s) * mp.G(b, -n - s);
            cd g1 = std::conj(wg1) * mp.G(a, n + s) * mp.G(b, -n + s);
            cd g2 = wg1 * mp.G(a, n - s) * std::conj(mp.G(b, n + s));
            cd g3 = wg1 * std::conj(mp.G(a, -n + s)) * mp.G(b, -n - s);
            if (diag) {
                g0 -= wg1 * mp.gg0[a];
                g1 -= std::conj(wg1) * mp.gg1[a];
                g2 -= wg1 * mp.gg2[a];
                g3 -= wg1 * mp.gg2[a];
            }
            int i = idx(a, b, n);
            O.gam[0][i] += g0.real(); O.gam[1][i] += g0.imag();
            O.gam[2][i] += g1.real(); O.gam[3][i] += g1.imag();
            O.gam[4][i] += g2.real(); O.gam[5][i] += g2.imag();
            O.gam[6][i] += g3.real(); O.gam[7][i] += g3.imag();
        }
    };
    for (int k2 = kstart; k2 < mink_zeta; ++k2) {
        add_gam(k2, k2, true);
        for (int k3 = k2 + 1; k3 < nb; ++k3) { add_gam(k2, k3, false); add_gam(k3, k2, false); }
    }
}

inline bool too_small(const Params& P, double rsq, double s1ps2)
{ return rsq < P.minsepsq && s1ps2 < P.minsep && rsq < sqr(P.minsep - s1ps2); }
inline bool too_large(const Params& P, double rsq, double s1ps2)
{ return rsq >= P.maxsepsq && rsq >= sqr(P.maxsep + s1ps2); }

// BaseCorr3::splitC2Cells, src/Corr3.cpp:1323-1372.
void split_c2_cells(const Params& P, const Field& f, const Node& c1,
                    const std::vector<int>& c2list, std::vector<int>& out)
{
    double s1 = c1.size;
    for (int j : c2list) {
        const Node& c2 = f.nodes[j];
        double s2 = c2.size;
        double rsq = dist_sq(P, c1, c2);
        double s1ps2 = s1 + s2;
        if (too_small(P, rsq, s1ps2) || too_large(P, rsq, s1ps2)) continue;
        int k = -1;
        double r = 0., logr = 0.;
        bool split = !single_bin(P, rsq, s1ps2, k, r, logr);
        if (split && s2 > s1) { out.push_back(c2.left); out.push_back(c2.right); }
        else out.push_back(j);
    }
}

// BaseCorr3::splitC2CellsOrCalculateGn, src/Corr3.cpp:1452-1546.
double split_or_gn(const Params& P, const Field& f, const Node& c1,
                   const std::vector<int>& c2list, std::vector<int>& out, bool& anysplit1,
                   MPS& mp, double prev_maxr)
{
    double s1 = c1.size;
    double maxrem = 0.;
    double thresh1 = (1. - P.binsize) * prev_maxr;   // BinTypeHelper<Log>::oneBinLessThan
    for (int j : c2list) {
        const Node& c2 = f.nodes[j];
        double s2 = c2.size;
        double rsq = dist_sq(P, c1, c2);
        double s1ps2 = s1 + s2;
        if (too_small(P, rsq, s1ps2) || too_large(P, rsq, s1ps2)) continue;
        int k = -1;
        double r = std::sqrt(rsq), logr = 0.;
        if (single_bin(P, rsq, s1ps2, k, r, logr)) {
            if (rsq >= P.minsepsq && rsq < P.maxsepsq) {
                if (k < 0) {
                    logr = std::log(r);
                    k = int((logr - P.logminsep) / P.binsize);
                }
                if (k >= P.nbins) k = P.nbins - 1;   // (unguarded in the reference)
                calculate_gn(P, c1, c2, r, logr, k, mp);
            }
            continue;
        }
        double rtot = r + s1ps2;
        maxrem = std::max(rtot, maxrem);
        bool split1 = false, split2 = false;
        calc_split_sq(split1, split2, s1, s2, rsq * std::min(P.bsq, P.asq));
        if (split1 && r + s1ps2 > thresh1) anysplit1 = true;
        if (split2) { out.push_back(c2.left); out.push_back(c2.right); }
        else out.push_back(j);
    }
    return maxrem;
}

// BaseCorr3::multipoleFinish, src/Corr3.cpp:1548-1613.  c1 is a cell of f1, the list holds
// cells of f2 (f2 = f1 for an auto-correlation).
void multipole_finish(const Params& P, const Field& f1, const Field& f2, int i1,
                      const std::vector<int>& c2list, MPS& mp, int mink_zeta, double maxr,
                      Out3& O)
{
    const Node& c1 = f1.nodes[i1];
    bool anysplit1 = false;
    std::vector<int> newlist;
    maxr = split_or_gn(P, f2, c1, c2list, newlist, anysplit1, mp, maxr);
    if (!newlist.empty()) {
        if (maxr < P.maxsep) {
            int k = maxr < P.minsep ? 0 : int((std::log(maxr) - P.logminsep) / P.binsize) + 1;
            if (k < mink_zeta) {
                calculate_zeta(P, c1, mp, k, mink_zeta, O);
                mink_zeta = k;
            }
        }
        if (anysplit1) {
            MPS copy = mp;
            multipole_finish(P, f1, f2, c1.left, newlist, mp, mink_zeta, maxr, O);
            multipole_finish(P, f1, f2, c1.right, newlist, copy, mink_zeta, maxr, O);
        } else {
            multipole_finish(P, f1, f2, i1, newlist, mp, mink_zeta, maxr, O);
        }
    } else {
        calculate_zeta(P, c1, mp, 0, mink_zeta, O);
    }
}

// BaseCorr3::multipoleSplit1, src/Corr3.cpp:1374-1408 (c1 in f1, the list in f2).
void multipole_split1(const Params& P, const Field& f1, const Field& f2, int i1,
                      const std::vector<int>& c2list, MPS& mp, Out3& O)
{
    const Node& c1 = f1.nodes[i1];
    double s1 = c1.size;
    std::vector<int> newlist;
    split_c2_cells(P, f2, c1, c2list, newlist);
    double maxbsq_eff = P.maxsepsq * std::min(P.bsq, P.asq);
    if (double(s1) * double(s1) > maxbsq_eff) {
        multipole_split1(P, f1, f2, c1.left, newlist, mp, O);
        multipole_split1(P, f1, f2, c1.right, newlist, mp, O);
    } else {
        mp.clear();
        multipole_finish(P, f1, f2, i1, newlist, mp, P.nbins, 0., O);
    }
}

// ---------------------------------------------------------------------------------------
// The three-field multipole: vertex 1 from f1, vertex 2 from f2, vertex 3 from f3
// (BaseCorr3::multipole(field1, field2, field3, ordered), src/Corr3.cpp:1239-1305).

// Corr3::calculateZeta(c1, ordered, mp2, mp3, kstart, mink_zeta), src/Corr3.cpp:1976-2087,
// with the multipole products of MultipoleHelper<5> written directly (its #if 0 form,
// 2868-2890): entries (k2, k3) with min(k2, k3) in [kstart, mink_zeta); mp3 goes with k2
// (it holds the d2 distances) and mp2 with k3; ordered = 1 adds the swapped products.
void calculate_zeta3(const Params& P, const Node& c1, int ordered, const MPS& mp2,
                     const MPS& mp3, int kstart, int mink_zeta, Out3& O)
{
    const int nb = mp2.nbins, maxn = mp2.maxn, nn = 2 * maxn + 1;
    const double w1 = c1.w;
    const cd wg1(c1.d1, c1.d2);
    const int s = P.vreal ? 0 : 1;
    const bool swap23 = ordered == 1;
    // The zeta of MultipoleHelper<3>, <4> and <6> (a real vertex with one real and one
    // spin-2 list, a spin-2 vertex with real lists or with one of each; src/Corr3.cpp:
    // 2418-2446, 2536-2572, 3029-3075) is written for ordered = 4 only and has no swapped
    // term; the weights and means still have it.
    const bool swap_g = swap23 && mp2.real == mp3.real && !(mp2.real && !P.vreal);
    auto idx = [&](int a, int b, int n) { return (a * nb + b) * nn + maxn + n; };
    auto Wn = [&](const MPS& m, int k, int n) {
        return n >= 0 ? m.Wn[m.widx(k) + n] : std::conj(m.Wn[m.widx(k) - n]);
    };
    for (int k2 = kstart; k2 < nb; ++k2) {
        const int k3end = k2 < mink_zeta ? nb : mink_zeta;
        for (int k3 = kstart; k3 < k3end; ++k3) {
            if (!P.quick) {
                const double n1 = double(c1.n);
                const int i = idx(k2, k3, 0);
                if (ordered == 4) {
                    O.ntri[i] += n1 * mp3.npairs[k2] * mp2.npairs[k3];
                    const double ww12 = w1 * mp3.sumw[k2], ww13 = w1 * mp2.sumw[k3];
                    O.meand2[i] += ww13 * mp3.sumwr[k2];
                    O.meanlogd2[i] += ww13 * mp3.sumwlogr[k2];
                    O.meand3[i] += ww12 * mp2.sumwr[k3];
                    O.meanlogd3[i] += ww12 * mp2.sumwlogr[k3];
                } else {
                    O.ntri[i] += n1 * (mp2.npairs[k2] * mp3.npairs[k3] +
                                       mp3.npairs[k2] * mp2.npairs[k3]);
                    O.meand2[i] += w1 * (mp2.sumw[k3] * mp3.sumwr[k2] + mp3.sumw[k3] * mp2.sumwr[k2]);
                    O.meanlogd2[i] += w1 * (mp2.sumw[k3] * mp3.sumwlogr[k2] +
                                            mp3.sumw[k3] * mp2.sumwlogr[k2]);
                    O.meand3[i] += w1 * (mp2.sumw[k2] * mp3.sumwr[k3] + mp3.sumw[k2] * mp2.sumwr[k3]);
                    // The reference's second term takes mp3.sumw at k3 (src/Corr3.cpp:2036).
                    O.meanlogd3[i] += w1 * (mp2.sumw[k2] * mp3.sumwlogr[k3] +
                                            mp3.sumw[k3] * mp2.sumwlogr[k3]);
                }
            }
            for (int n = -maxn; n <= maxn; ++n) {
                const int i = idx(k2, k3, n);
                cd ww = w1 * Wn(mp3, k2, n) * std::conj(Wn(mp2, k3, n));
                cd g0 = wg1 * mp3.G(k2, n - s) * mp2.G(k3, -n - s);
                cd g1 = std::conj(wg1) * mp3.G(k2, n + s) * mp2.G(k3, -n + s);
                cd g2 = wg1 * mp3.G(k2, n - s) * std::conj(mp2.G(k3, n + s));
                cd g3 = wg1 * std::conj(mp3.G(k2, -n + s)) * mp2.G(k3, -n - s);
                if (swap23) ww += w1 * Wn(mp2, k2, n) * std::conj(Wn(mp3, k3, n));
                if (swap_g) {
                    g0 += wg1 * mp2.G(k2, n - s) * mp3.G(k3, -n - s);
                    g1 += std::conj(wg1) * mp2.G(k2, n + s) * mp3.G(k3, -n + s);
                    g2 += wg1 * mp2.G(k2, n - s) * std::conj(mp3.G(k3, n + s));
                    g3 += wg1 * std::conj(mp2.G(k2, -n + s)) * mp3.G(k3, -n - s);
                }
                O.weight[i] += ww.real(); O.weight_im[i] += ww.imag();
                O.gam[0][i] += g0.real(); O.gam[1][i] += g0.imag();
                O.gam[2][i] += g1.real(); O.gam[3][i] += g1.imag();
                O.gam[4][i] += g2.real(); O.gam[5][i] += g2.imag();
                O.gam[6][i] += g3.real(); O.gam[7][i] += g3.imag();
            }
        }
    }
}

// BaseCorr3::multipoleFinish with two lists, src/Corr3.cpp:1615-1679.
void multipole_finish3(const Params& P, const Field& f1, const Field& f2, const Field& f3,
                       int i1, const std::vector<int>& l2, const std::vector<int>& l3,
                       MPS& mp2, MPS& mp3, int ordered, int mink_zeta, double maxr2,
                       double maxr3, Out3& O)
{
    const Node& c1 = f1.nodes[i1];
    bool anysplit1 = false;
    std::vector<int> n2, n3;
    maxr2 = split_or_gn(P, f2, c1, l2, n2, anysplit1, mp2, maxr2);
    maxr3 = split_or_gn(P, f3, c1, l3, n3, anysplit1, mp3, maxr3);
    const double maxr = std::max(maxr2, maxr3);
    if (!n2.empty() || !n3.empty()) {
        if (maxr < P.maxsep) {
            int k = maxr < P.minsep ? 0 : int((std::log(maxr) - P.logminsep) / P.binsize) + 1;
            if (k < mink_zeta) {
                calculate_zeta3(P, c1, ordered, mp2, mp3, k, mink_zeta, O);
                mink_zeta = k;
            }
        }
        if (anysplit1) {
            MPS c2 = mp2, c3 = mp3;
            multipole_finish3(P, f1, f2, f3, c1.left, n2, n3, mp2, mp3, ordered, mink_zeta,
                              maxr2, maxr3, O);
            multipole_finish3(P, f1, f2, f3, c1.right, n2, n3, c2, c3, ordered, mink_zeta,
                              maxr2, maxr3, O);
        } else {
            multipole_finish3(P, f1, f2, f3, i1, n2, n3, mp2, mp3, ordered, mink_zeta, maxr2,
                              maxr3, O);
        }
    } else {
        calculate_zeta3(P, c1, ordered, mp2, mp3, 0, mink_zeta, O);
    }
}

// BaseCorr3::multipoleSplit1 with two lists, src/Corr3.cpp:1410-1449.
void multipole_split1_3(const Params& P, const Field& f1, const Field& f2, const Field& f3,
                        int i1, const std::vector<int>& l2, const std::vector<int>& l3,
                        MPS& mp2, MPS& mp3, int ordered, Out3& O)
{
    const Node& c1 = f1.nodes[i1];
    const double s1 = c1.size;
    std::vector<int> n2, n3;
    split_c2_cells(P, f2, c1, l2, n2);
    split_c2_cells(P, f3, c1, l3, n3);
    const double maxbsq_eff = P.maxsepsq * std::min(P.bsq, P.asq);
    if (s1 * s1 > maxbsq_eff) {
        multipole_split1_3(P, f1, f2, f3, c1.left, n2, n3, mp2, mp3, ordered, O);
        multipole_split1_3(P, f1, f2, f3, c1.right, n2, n3, mp2, mp3, ordered, O);
    } else {
        mp2.clear();
        mp3.clear();
        multipole_finish3(P, f1, f2, f3, i1, n2, n3, mp2, mp3, ordered, P.nbins, 0., 0., O);
    }
}

long long g_last_accepted = 0;   // directProcess11 calls of the last process call

// ---------------------------------------------------------------------------------------
// k-means patches (src/KMeans.cpp), on this oracle's tree.  Positions are 3-vectors with
// z = 0 for Flat; Position<C>::normSq of a difference is ((dx dx + dy dy) + dz dz).

struct P3 { double x = 0., y = 0., z = 0.; };

inline double p3_dsq(const P3& a, const P3& b)
{
    const double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return (dx * dx + dy * dy) + dz * dz;
}
inline bool p3_eq(const P3& a, const P3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline P3 node_pos(const Node& nd) { return P3{nd.x, nd.y, nd.z}; }

// urand, src/Cell.cpp:59-80 (the C library's rand(); a non-zero seed reseeds and draws).
bool g_first_urand = true;
double urand(long long seed = 0)
{
    if (seed != 0) { srand((unsigned)seed); g_first_urand = false; }
    else if (g_first_urand) { srand((unsigned)time(nullptr)); g_first_urand = false; }
    double r = rand();
    return r / RAND_MAX;
}

// SelectRandomFrom, src/Corr2.cpp:622-661.
std::vector<long> select_random(long m, long n)
{
    std::vector<long> sel(n);
    if (m > 3 * n) {
        std::set<long> got;
        while ((long)got.size() < n) {
            long j = long(urand() * m);
            if (j == m) j = m - 1;
            if (got.insert(j).second) sel[got.size() - 1] = j;
        }
    } else {
        std::vector<long> all(m);
        for (long i = 0; i < m; ++i) all[i] = i;
        for (long i = 0; i < n; ++i) {
            long j = long(urand() * (m - i)) + i;
            if (j == m) j = m - 1;
            std::swap(all[i], all[j]);
        }
        std::copy(all.begin(), all.begin() + n, sel.begin());
    }
    return sel;
}

// InitializeCentersTree, recursive part, src/KMeans.cpp:28-59.
void km_init_tree_cell(const Field& f, int id, long first, int nc, std::vector<P3>& cen)
{
    const Node& nd = f.nodes[id];
    if (nc == 1) {
        cen[first] = node_pos(nd);
    } else if (nd.left >= 0) {
        int m1 = nc / 2, m2 = nc - m1;
        if (urand() < 0.5) std::swap(m1, m2);
        km_init_tree_cell(f, nd.left, first, m1, cen);
        km_init_tree_cell(f, nd.right, first + m1, m2, cen);
    } else {
        for (int i = 0; i < nc; ++i) {
            const double a = 1. + urand() * 1.e-8;
            P3 v{nd.x * a, nd.y * a, nd.z * a};
            if (f.coords == SPHERE) normalize3(v.x, v.y, v.z);
            cen[first + i] = v;
        }
    }
}

// getLeafNumber, src/Cell.cpp:675-685.
int leaf_number(const Field& f, int id, long m)
{
    while (f.nodes[id].left >= 0) {
        const Node& l = f.nodes[f.nodes[id].left];
        if (m < l.n) id = f.nodes[id].left;
        else { m -= l.n; id = f.nodes[id].right; }
    }
    return id;
}

// InitializeCentersKMPP, recursive part, src/KMeans.cpp:159-218; returns false for the
// reference's LeafAlreadyUsed exception.
bool km_kmpp_cell(const Field& f, int id, const std::vector<P3>& cen, long ncen, P3& out)
{
    const Node& nd = f.nodes[id];
    if (nd.size == 0.f) {
        for (long j = 0; j < ncen; ++j)
            if (p3_eq(node_pos(nd), cen[j])) return false;
        out = node_pos(nd);
        return true;
    }
    const P3 lp = node_pos(f.nodes[nd.left]), rp = node_pos(f.nodes[nd.right]);
    double d1 = p3_dsq(lp, cen[0]), d2 = p3_dsq(rp, cen[0]);
    for (long j = 1; j < ncen; ++j) {
        const double a = p3_dsq(lp, cen[j]), b = p3_dsq(rp, cen[j]);
        if (a < d1) d1 = a;
        if (b < d2) d2 = b;
    }
    if (d1 + d2 == 0.) return false;
    const double u = urand() * (d1 + d2);
    if (u < d1) {
        if (km_kmpp_cell(f, nd.left, cen, ncen, out)) return true;
        return km_kmpp_cell(f, nd.right, cen, ncen, out);
    }
    if (km_kmpp_cell(f, nd.right, cen, ncen, out)) return true;
    return km_kmpp_cell(f, nd.left, cen, ncen, out);
}

// The per-cell actions of FindCellsInPatches (src/KMeans.cpp:318-541).
struct KMAction {
    int mode;                    // 0 update centres, 1 inertia, 2 assign
    const Field* f;
    const std::vector<P3>* cen;
    std::vector<P3> sum;         // UpdateCenters
    std::vector<double> w;
    std::vector<double> inertia; // CalculateInertia
    double sumw = 0.;
    long* patches = nullptr;     // AssignPatches

    void run(int p, int id)
    {
        const Node& nd = f->nodes[id];
        if (mode == 0) {
            const double ww = nd.w;
            sum[p].x += nd.x * ww; sum[p].y += nd.y * ww; sum[p].z += nd.z * ww;
            w[p] += ww;
        } else if (mode == 1) {
            const double ssq = double(nd.size) * double(nd.size);
            const double ww = nd.w;
            inertia[p] += p3_dsq(node_pos(nd), (*cen)[p]) * ww;
            if (ssq > 0.) inertia[p] += 0.75 * ssq * ww;
            sumw += ww;
        } else {
            for (long k = nd.start; k < nd.end; ++k) patches[f->pts[k].index] = p;
        }
    }
};

// FindCellsInPatches, src/KMeans.cpp:543-645 (candidate swaps included).
void km_find(const Field& f, const std::vector<P3>& cen, int id, std::vector<long>& pat,
             long ncand, std::vector<double>& saved, KMAction& act, const std::vector<double>* I)
{
    const Node& nd = f.nodes[id];
    const P3 c = node_pos(nd);
    const double s = nd.size;
    long closest = pat[0];
    double mind = p3_dsq(c, cen[closest]);
    saved[0] = mind;
    if (I) mind += (*I)[closest];
    for (long j = 1; j < ncand; ++j) {
        const long i = pat[j];
        double d = p3_dsq(c, cen[i]);
        saved[j] = d;
        if (I) d += (*I)[i];
        if (d < mind) {
            std::swap(saved[0], saved[j]);
            std::swap(pat[0], pat[j]);
            closest = i;
            mind = d;
        }
    }
    const double min_d = std::sqrt(saved[0]);
    const double thresh = I ? sqr(min_d + s) + (*I)[closest] : sqr(min_d + 2 * s);
    for (long j = ncand - 1; j > 0; --j) {
        double d = saved[j];
        if (I) {
            const double dd = std::sqrt(d);
            d = (s > dd) ? 0. : sqr(dd - s) + (*I)[pat[j]];
        }
        if (d > thresh) {
            --ncand;
            if (j != ncand) std::swap(pat[j], pat[ncand]);
        }
    }
    if (ncand == 1 || s == 0. || nd.left < 0) {
        act.run((int)closest, id);
    } else {
        km_find(f, cen, nd.left, pat, ncand, saved, act, I);
        km_find(f, cen, nd.right, pat, ncand, saved, act, I);
    }
}

void km_find_all(const Field& f, const std::vector<P3>& cen, KMAction& act,
                 const std::vector<double>* I)
{
    const long np = (long)cen.size();
    std::vector<long> pat(np);
    std::vector<double> saved(np);
    for (long i = 0; i < np; ++i) pat[i] = i;
    for (int t : f.tops) km_find(f, cen, t, pat, np, saved, act, I);
}

std::vector<P3> read_centers(const double* c, int npatch, int coords)
{
    const int dim = coords == FLAT ? 2 : 3;
    std::vector<P3> v(npatch);
    for (int p = 0; p < npatch; ++p) {
        v[p] = P3{c[dim * p], c[dim * p + 1], dim == 3 ? c[dim * p + 2] : 0.};
        if (coords == SPHERE) normalize3(v[p].x, v[p].y, v[p].z);
    }
    return v;
}

void write_centers(const std::vector<P3>& v, double* c, int coords)
{
    const int dim = coords == FLAT ? 2 : 3;
    for (size_t p = 0; p < v.size(); ++p) {
        c[dim * p] = v[p].x; c[dim * p + 1] = v[p].y;
        if (dim == 3) c[dim * p + 2] = v[p].z;
    }
}

// QuickAssign / SelectPatch distance, src/KMeans.cpp:911-935 and 970-1006.
inline double qdist(const double* c, int dim, int k, double x, double y, double z)
{
    const double dx = x - c[dim * k], dy = y - c[dim * k + 1];
    double r = dx * dx + dy * dy;
    if (dim == 3) { const double dz = z - c[dim * k + 2]; r += dz * dz; }
    return r;
}

}  // namespace

extern "C" {

long long orc_last_accepted(void) { return g_last_accepted; }

// Field::Field, src/Field.cpp:163-204 (copies the inputs; cells are built lazily).
void* orc_field_build(int dtype, int coords, const double* x, const double* y, const double* z,
                      const double* d1, const double* d2, const double* w, const double* wpos,
                      long n, double minsize, double maxsize, int sm, int brute, int mintop,
                      int maxtop)
{
    Field* f = new Field();
    f->spin = spin_of(dtype);
    dtype = kind_of(dtype);
    f->dtype = dtype; f->coords = coords; f->minsize = minsize; f->maxsize = maxsize;
    f->sm = sm; f->brute = brute; f->mintop = mintop; f->maxtop = maxtop; f->built = false;
    f->pts.resize(n);
    for (long i = 0; i < n; ++i) {
        Pt& p = f->pts[i];
        p.x = x[i]; p.y = y[i]; p.z = (z && coords != FLAT) ? z[i] : 0.;
        if (coords == SPHERE) normalize3(p.x, p.y, p.z);
        p.wpos = wpos ? wpos[i] : w[i];
        p.w = float(w[i]);
        p.index = i;
        if (dtype == DK) { p.d1 = float(w[i] * d1[i]); p.d2 = 0.f; }
        else if (dtype == DG) { p.d1 = float(w[i] * d1[i]); p.d2 = float(w[i] * d2[i]); }
        else { p.d1 = p.d2 = 0.f; }
    }
    f->cx = f->cy = f->cz = 0.; f->sizesq = 0.;
    if (n > 0) {
        Node nd;
        build_cell_data(*f, 0, n, nd);
        f->cx = nd.x; f->cy = nd.y; f->cz = nd.z;
        f->sizesq = calc_sizesq(*f, nd, 0, n);
    }
    return f;
}

void orc_field_free(void* h) { delete static_cast<Field*>(h); }

long orc_field_ntop(void* h)
{
    Field* f = static_cast<Field*>(h);
    build_cells(*f);
    return (long)f->tops.size();
}

void orc_field_center(void* h, double* out4)
{
    Field* f = static_cast<Field*>(h);
    out4[0] = f->cx; out4[1] = f->cy; out4[2] = f->cz; out4[3] = std::sqrt(f->sizesq);
}

// Canonical depth-first dump of the tree (tops in order, then left before right), used to
// compare cell membership and cell data with the CUDA tree build.
long orc_field_dump(void* h, double* xyz, float* size_w_d, long* n_start, int* depth,
                    long cap)
{
    Field* f = static_cast<Field*>(h);
    build_cells(*f);
    long cnt = 0;
    std::vector<std::pair<int, int>> stack;
    for (long t = (long)f->tops.size() - 1; t >= 0; --t) stack.push_back({f->tops[t], 0});
    while (!stack.empty()) {
        auto [id, d] = stack.back();
        stack.pop_back();
        const Node& nd = f->nodes[id];
        if (cnt < cap) {
            xyz[3 * cnt] = nd.x; xyz[3 * cnt + 1] = nd.y; xyz[3 * cnt + 2] = nd.z;
            size_w_d[4 * cnt] = nd.size; size_w_d[4 * cnt + 1] = nd.w;
            size_w_d[4 * cnt + 2] = nd.d1; size_w_d[4 * cnt + 3] = nd.d2;
            n_start[2 * cnt] = nd.n; n_start[2 * cnt + 1] = nd.start;
            depth[cnt] = d;
        }
        ++cnt;
        if (nd.left >= 0) {
            stack.push_back({nd.right, d + 1});
            stack.push_back({nd.left, d + 1});
        }
    }
    return cnt;
}

// Original indices of the points in final tree order (list-leaf membership checks).
void orc_field_order(void* h, long* out)
{
    Field* f = static_cast<Field*>(h);
    build_cells(*f);
    for (size_t i = 0; i < f->pts.size(); ++i) out[i] = f->pts[i].index;
}

// BaseCorr2::process (auto, src/Corr2.cpp:146-205; cross, 207-288) for Log binning.
// Outputs are caller-owned and accumulated into (+=), like the reference.
int orc_corr2_process(int dtype, int metric, int quick, double minsep, double maxsep, int nbins,
                      double binsize, double b, double a, void* h1, void* h2, int nthreads,
                      double* xi0, double* xi1, double* xi2, double* xi3, double* meanr,
                      double* meanlogr, double* weight, double* npairs)
{
    Field* f1 = static_cast<Field*>(h1);
    Field* f2 = h2 ? static_cast<Field*>(h2) : nullptr;
    Params P = make_params(dtype, f1->coords, metric, quick, minsep, maxsep, nbins, binsize,
                           b, a);
    if (f1->pts.empty() || (f2 && f2->pts.empty())) return 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    if (f2) {
        // Early exit when the fields cannot overlap, src/Corr2.cpp:213-231.
        Node a1, a2;
        a1.x = f1->cx; a1.y = f1->cy; a1.z = f1->cz;
        a2.x = f2->cx; a2.y = f2->cy; a2.z = f2->cz;
        double rsq = dist_sq(P, a1, a2);
        double s1ps2 = std::sqrt(f1->sizesq) + std::sqrt(f2->sizesq);
        if ((rsq < P.minsepsq && s1ps2 < P.minsep && rsq < sqr(P.minsep - s1ps2)) ||
            (rsq >= P.maxsepsq && rsq >= sqr(P.maxsep + s1ps2)))
            return 0;
    }
    build_cells(*f1);
    if (f2) build_cells(*f2);
    const long n1 = (long)f1->tops.size();
    const long n2 = f2 ? (long)f2->tops.size() : 0;
    Accum total(nbins);
#pragma omp parallel
    {
        Accum A(nbins);
#pragma omp for schedule(dynamic)
        for (long i = 0; i < n1; ++i) {
            if (!f2) {
                process2(P, *f1, f1->tops[i], A);
                for (long j = i + 1; j < n1; ++j) process11(P, *f1, *f1, f1->tops[i], f1->tops[j], A);
            } else {
                for (long j = 0; j < n2; ++j) process11(P, *f1, *f2, f1->tops[i], f2->tops[j], A);
            }
        }
#pragma omp critical
        {
            for (int k = 0; k < nbins; ++k) {
                total.xi0[k] += A.xi0[k]; total.xi1[k] += A.xi1[k];
                total.xi2[k] += A.xi2[k]; total.xi3[k] += A.xi3[k];
                total.meanr[k] += A.meanr[k]; total.meanlogr[k] += A.meanlogr[k];
                total.weight[k] += A.weight[k]; total.npairs[k] += A.npairs[k];
            }
            total.accepted += A.accepted;
        }
    }
    g_last_accepted = total.accepted;
    add_into(total, xi0, xi1, xi2, xi3, meanr, meanlogr, weight, npairs);
    return 0;
}

// Only a bounded share of the top-level work: top rows [row0, row1) of the auto loop.
// bench.py times this on a stated sample and scales by the sampled share of point pairs.
int orc_corr2_process_rows(int dtype, int metric, int quick, double minsep, double maxsep,
                           int nbins, double binsize, double b, double a, void* h1, long row0,
                           long row1, int nthreads, double* xi0, double* xi1, double* xi2,
                           double* xi3, double* meanr, double* meanlogr, double* weight,
                           double* npairs)
{
    Field* f1 = static_cast<Field*>(h1);
    Params P = make_params(dtype, f1->coords, metric, quick, minsep, maxsep, nbins, binsize,
                           b, a);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    build_cells(*f1);
    const long n1 = (long)f1->tops.size();
    if (row1 > n1) row1 = n1;
    Accum total(nbins);
#pragma omp parallel
    {
        Accum A(nbins);
#pragma omp for schedule(dynamic)
        for (long i = row0; i < row1; ++i) {
            process2(P, *f1, f1->tops[i], A);
            for (long j = i + 1; j < n1; ++j) process11(P, *f1, *f1, f1->tops[i], f1->tops[j], A);
        }
#pragma omp critical
        {
            for (int k = 0; k < nbins; ++k) {
                total.xi0[k] += A.xi0[k]; total.xi1[k] += A.xi1[k];
                total.xi2[k] += A.xi2[k]; total.xi3[k] += A.xi3[k];
                total.meanr[k] += A.meanr[k]; total.meanlogr[k] += A.meanlogr[k];
                total.weight[k] += A.weight[k]; total.npairs[k] += A.npairs[k];
            }
            total.accepted += A.accepted;
        }
    }
    g_last_accepted = total.accepted;
    add_into(total, xi0, xi1, xi2, xi3, meanr, meanlogr, weight, npairs);
    return 0;
}


// BaseCorr3::multipole for GGG with LogMultipole binning: auto (h2 = h1, src/Corr3.cpp:
// 1124-1175) or cross12 (vertex 1 from h1, vertices 2 and 3 from h2, 1177-1237).
// Outputs have nbins*nbins*(2*maxn+1) entries, accumulated (+=) like the reference's.
static int multipole_run(int metric, int quick, double minsep, double maxsep, int nbins,
                         double binsize, double b, double a, int maxn, void* h1, void* h2,
                         int mode, int nthreads, double** gam8, double* meand2,
                         double* meanlogd2, double* meand3, double* meanlogd3, double* weight,
                         double* weight_im, double* ntri)
{
    Field* f1 = static_cast<Field*>(h1);
    Field* f2 = static_cast<Field*>(h2);
    // Vertex 1: a G field, or for NGG / KGG a K field whose k is 1 (N) or k (K), so that
    // its cells' d1 is the real vertex weight (no parallel transport for spin 0).
    // mode 0: GGG; 1: NGG / KGG; 2: GNN / GKK, whose pairs come as a K field whose k is 1
    // (N) or k (K); 3: KKK / NKK / KNN, vertex and pairs such K fields.
    const bool vreal = mode == 1 || mode == 3, pspin0 = mode == 2 || mode == 3;
    const bool v_ok = vreal ? (f1->dtype == DK && f1->spin == 0) : (f1->dtype == DG && f1->spin == 2);
    const bool p_ok = pspin0 ? (f2->dtype == DK && f2->spin == 0) : (f2->dtype == DG && f2->spin == 2);
    if (!v_ok || !p_ok) return 1;
    if (f1->coords != f2->coords) return 2;
    Params P = make_params(DG * 16 + DG, f1->coords, metric, quick, minsep, maxsep, nbins, binsize, b, a);
    P.vreal = vreal ? 1 : 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    if (f1->pts.empty() || f2->pts.empty()) return 0;
    build_cells(*f1);
    if (f2 != f1) build_cells(*f2);
    const long n1 = (long)f1->tops.size();
    Out3 total(nbins, maxn);
#pragma omp parallel
    {
        Out3 O(nbins, maxn);
        MPS mp(nbins, maxn);
        mp.real = pspin0;
#pragma omp for schedule(dynamic)
        for (long i = 0; i < n1; ++i) multipole_split1(P, *f1, *f2, f1->tops[i], f2->tops, mp, O);
#pragma omp critical
        total.add(O);
    }
    for (int q = 0; q < 8; ++q)
        if (gam8[q]) for (int i = 0; i < total.size; ++i) gam8[q][i] += total.gam[q][i];
    for (int i = 0; i < total.size; ++i) {
        meand2[i] += total.meand2[i]; meanlogd2[i] += total.meanlogd2[i];
        meand3[i] += total.meand3[i]; meanlogd3[i] += total.meanlogd3[i];
        weight[i] += total.weight[i]; weight_im[i] += total.weight_im[i];
        ntri[i] += total.ntri[i];
    }
    return 0;
}

int orc_corr3_multipole_auto(int metric, int quick, double minsep, double maxsep, int nbins,
                             double binsize, double b, double a, int maxn, void* h, int nthreads,
                             double** gam8, double* meand2, double* meanlogd2, double* meand3,
                             double* meanlogd3, double* weight, double* weight_im, double* ntri)
{
    return multipole_run(metric, quick, minsep, maxsep, nbins, binsize, b, a, maxn, h, h, 0,
                         nthreads, gam8, meand2, meanlogd2, meand3, meanlogd3, weight,
                         weight_im, ntri);
}

int orc_corr3_multipole_cross12(int metric, int quick, double minsep, double maxsep, int nbins,
                                double binsize, double b, double a, int maxn, void* h1,
                                void* h2, int mode, int nthreads, double** gam8, double* meand2,
                                double* meanlogd2, double* meand3, double* meanlogd3,
                                double* weight, double* weight_im, double* ntri)
{
    return multipole_run(metric, quick, minsep, maxsep, nbins, binsize, b, a, maxn, h1, h2,
                         mode, nthreads, gam8, meand2, meanlogd2, meand3, meanlogd3, weight,
                         weight_im, ntri);
}

// The three-field multipole (vertex 1 from h1, 2 from h2, 3 from h3; ordered 1 or 4); the
// fields and modes as for orc_corr3_multipole_cross12 (h2 and h3 share a kind).
int orc_corr3_multipole_cross3(int metric, int quick, double minsep, double maxsep, int nbins,
                               double binsize, double b, double a, int maxn, void* h1,
                               void* h2, void* h3, int ordered, int mode, int nthreads,
                               double** gam8, double* meand2, double* meanlogd2,
                               double* meand3, double* meanlogd3, double* weight,
                               double* weight_im, double* ntri)
{
    Field* f1 = static_cast<Field*>(h1);
    Field* f2 = static_cast<Field*>(h2);
    Field* f3 = static_cast<Field*>(h3);
    // mode bit 0: vertex 1 a K field whose k is 1 (N) or k (K); bit 1: the vertex-2 field
    // such a K field; bit 2: the vertex-3 field.
    const bool vreal = mode & 1, r2 = (mode >> 1) & 1, r3 = (mode >> 2) & 1;
    const bool v_ok = vreal ? (f1->dtype == DK && f1->spin == 0) : (f1->dtype == DG && f1->spin == 2);
    auto p_ok = [&](const Field* f, bool real) {
        return real ? (f->dtype == DK && f->spin == 0) : (f->dtype == DG && f->spin == 2);
    };
    if (!v_ok || !p_ok(f2, r2) || !p_ok(f3, r3)) return 1;
    if (f1->coords != f2->coords || f1->coords != f3->coords) return 2;
    if (ordered != 1 && ordered != 4) return 3;
    Params P = make_params(DG * 16 + DG, f1->coords, metric, quick, minsep, maxsep, nbins, binsize, b, a);
    P.vreal = vreal ? 1 : 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    if (f1->pts.empty() || f2->pts.empty() || f3->pts.empty()) return 0;
    build_cells(*f1);
    if (f2 != f1) build_cells(*f2);
    if (f3 != f1 && f3 != f2) build_cells(*f3);
    const long n1 = (long)f1->tops.size();
    Out3 total(nbins, maxn);
#pragma omp parallel
    {
        Out3 O(nbins, maxn);
        MPS mp2(nbins, maxn), mp3(nbins, maxn);
        mp2.real = r2;
        mp3.real = r3;
#pragma omp for schedule(dynamic)
        for (long i = 0; i < n1; ++i)
            multipole_split1_3(P, *f1, *f2, *f3, f1->tops[i], f2->tops, f3->tops, mp2, mp3,
                               ordered, O);
#pragma omp critical
        total.add(O);
    }
    for (int q = 0; q < 8; ++q)
        if (gam8[q]) for (int i = 0; i < total.size; ++i) gam8[q][i] += total.gam[q][i];
    for (int i = 0; i < total.size; ++i) {
        meand2[i] += total.meand2[i]; meanlogd2[i] += total.meanlogd2[i];
        meand3[i] += total.meand3[i]; meanlogd3[i] += total.meanlogd3[i];
        weight[i] += total.weight[i]; weight_im[i] += total.weight_im[i];
        ntri[i] += total.ntri[i];
    }
    return 0;
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// KMeansInitTree1 / InitializeCentersTree, src/KMeans.cpp:61-109, 743-751.
int orc_kmeans_init_tree(void* h, double* centers, int npatch, long long seed)
{
    Field& f = *static_cast<Field*>(h);
    build_cells(f);
    std::vector<P3> cen(npatch);
    const long ncells = (long)f.tops.size();
    urand(seed);
    if (ncells > npatch) {
        const std::vector<long> sel = select_random(ncells, npatch);
        for (int i = 0; i < npatch; ++i) cen[i] = node_pos(f.nodes[f.tops[sel[i]]]);
    } else {
        const long n1 = npatch / ncells, k2 = npatch % ncells, k1 = ncells - k2;
        std::vector<long> nv(ncells);
        for (long k = 0; k < ncells; ++k) nv[k] = k < k1 ? n1 : n1 + 1;
        for (long k = ncells; k > 1; --k) {
            long j = int(urand() * k);
            if (j > k - 1) j = k - 1;
            if (j != k - 1) std::swap(nv[j], nv[k - 1]);
        }
        long first = 0;
        for (long k = 0; k < ncells; ++k) {
            km_init_tree_cell(f, f.tops[k], first, (int)nv[k], cen);
            first += nv[k];
        }
    }
    write_centers(cen, centers, f.coords);
    return 0;
}

// KMeansInitRand1 / InitializeCentersRand, src/KMeans.cpp:111-157, 753-761.
int orc_kmeans_init_rand(void* h, double* centers, int npatch, long long seed)
{
    Field& f = *static_cast<Field*>(h);
    build_cells(f);
    long ntot = 0;
    for (int t : f.tops) ntot += f.nodes[t].n;
    urand(seed);
    const std::vector<long> index = select_random(ntot, npatch);
    std::vector<P3> cen(npatch);
    for (int i = 0; i < npatch; ++i) {
        long m = index[i];
        for (int t : f.tops) {
            if (m < f.nodes[t].n) { cen[i] = node_pos(f.nodes[leaf_number(f, t, m)]); break; }
            m -= f.nodes[t].n;
        }
        for (int i1 = 0; i1 < i; ++i1) {
            if (p3_eq(cen[i1], cen[i])) {
                const double a = 1. + urand() * 1.e-8;
                cen[i].x *= a; cen[i].y *= a; cen[i].z *= a;
            }
        }
    }
    write_centers(cen, centers, f.coords);
    return 0;
}

// KMeansInitKMPP1 / InitializeCentersKMPP, src/KMeans.cpp:220-315, 763-771.
int orc_kmeans_init_kmpp(void* h, double* centers, int npatch, long long seed)
{
    Field& f = *static_cast<Field*>(h);
    build_cells(f);
    const long ncells = (long)f.tops.size();
    urand(seed);
    long ntot = 0;
    for (int t : f.tops) ntot += f.nodes[t].n;
    std::vector<long> per(ncells, 0);
    std::vector<P3> cen(npatch);
    long m = long(urand() * ntot);
    for (long k = 0; k < ncells; ++k) {
        const Node& t = f.nodes[f.tops[k]];
        if (m < t.n) { cen[0] = node_pos(f.nodes[leaf_number(f, f.tops[k], m)]); per[k] += 1; break; }
        m -= t.n;
    }
    const double coef = f.coords == THREED ? 0.6 : 0.5;
    std::vector<double> p(ncells);
    for (int i = 1; i < npatch; ++i) {
        double sump = 0.;
        for (long k = 0; k < ncells; ++k) {
            const Node& t = f.nodes[f.tops[k]];
            double d1 = p3_dsq(cen[0], node_pos(t));
            for (int i1 = 1; i1 < i; ++i1) {
                const double d2 = p3_dsq(cen[i1], node_pos(t));
                if (d2 < d1) d1 = d2;
            }
            p[k] = (t.n - per[k]) * (d1 + coef * sqr(double(t.size)));
            sump += p[k];
        }
        double u = urand();
        for (long k = 0; k < ncells; ++k) {
            p[k] /= sump;
            if (u < p[k]) {
                if (!km_kmpp_cell(f, f.tops[k], cen, i, cen[i])) return 1;
                per[k] += 1;
                break;
            }
            u -= p[k];
        }
    }
    write_centers(cen, centers, f.coords);
    return 0;
}

// KMeansRun1, src/KMeans.cpp:773-833.  Returns the iterations run.
int orc_kmeans_run(void* h, double* centers, int npatch, int max_iter, double tol, int alt)
{
    Field& f = *static_cast<Field*>(h);
    build_cells(f);
    std::vector<P3> cen = read_centers(centers, npatch, f.coords);
    const double tolsq = sqr(tol * std::sqrt(f.sizesq)) * npatch;
    std::vector<double> inertia;
    int it = 0;
    for (; it < max_iter; ++it) {
        if (alt) {
            KMAction ci{1, &f, &cen};
            ci.inertia.assign(npatch, 0.);
            km_find_all(f, cen, ci, nullptr);
            const double meanw = ci.sumw / npatch / 3.;
            inertia = ci.inertia;
            for (int i = 0; i < npatch; ++i) inertia[i] /= meanw;
        }
        KMAction up{0, &f, &cen};
        up.sum.assign(npatch, P3{});
        up.w.assign(npatch, 0.);
        km_find_all(f, cen, up, alt ? &inertia : nullptr);
        for (int i = 0; i < npatch; ++i) {
            if (up.w[i] > 0.) {
                up.sum[i].x /= up.w[i]; up.sum[i].y /= up.w[i]; up.sum[i].z /= up.w[i];
                if (f.coords == SPHERE) normalize3(up.sum[i].x, up.sum[i].y, up.sum[i].z);
            }
        }
        double shiftsq = 0.;
        for (int i = 0; i < npatch; ++i) shiftsq += p3_dsq(cen[i], up.sum[i]);
        cen = up.sum;
        if (shiftsq < tolsq) { ++it; break; }
    }
    write_centers(cen, centers, f.coords);
    return it;
}

// KMeansAssign1, src/KMeans.cpp:835-849.
int orc_kmeans_assign(void* h, const double* centers, int npatch, long* patches)
{
    Field& f = *static_cast<Field*>(h);
    build_cells(f);
    std::vector<P3> cen = read_centers(centers, npatch, f.coords);
    KMAction as{2, &f, &cen};
    as.patches = patches;
    km_find_all(f, cen, as, nullptr);
    return 0;
}

// QuickAssign, src/KMeans.cpp:890-942 (z == NULL: the 2-d form).
void orc_quick_assign(const double* centers, int npatch, const double* x, const double* y,
                      const double* z, long n, long* out)
{
    const int dim = z ? 3 : 2;
    for (long i = 0; i < n; ++i) {
        const double zi = z ? z[i] : 0.;
        int kmin = 0;
        double mn = qdist(centers, dim, 0, x[i], y[i], zi);
        for (int k = 1; k < npatch; ++k) {
            const double r = qdist(centers, dim, k, x[i], y[i], zi);
            if (r < mn) { kmin = k; mn = r; }
        }
        out[i] = kmin;
    }
}

// SelectPatch, src/KMeans.cpp:944-1011.
void orc_select_patch(int patch, const double* centers, int npatch, const double* x,
                      const double* y, const double* z, long n, long* use)
{
    const int dim = z ? 3 : 2;
    for (long i = 0; i < n; ++i) {
        const double zi = z ? z[i] : 0.;
        const double pd = qdist(centers, dim, patch, x[i], y[i], zi);
        use[i] = 1;
        for (int q = 0; q < npatch; ++q) {
            if (q == patch) continue;
            if (qdist(centers, dim, q, x[i], y[i], zi) < pd) { use[i] = 0; break; }
        }
    }
}

}  // extern "C"
