// tree_build.cu -- GPU ball-tree build with the reference's cell rules.
//
// The tree is the one TreeCorr builds (src/Field.cpp:27-81 SetupTopLevelCells,
// src/Cell.cpp:556-615 BuildCell, src/Cell.cpp:426-554 SplitData): every cell holds the
// wpos-weighted centroid of its points (normalised on the sphere), the float sum of w,
// the float payload sum (parallel-transported to the centroid on the sphere), and
// size = float(max |centroid - p|); it is split at the centroid coordinate (Mean) or the
// bounding-box middle (Middle) along the axis of largest extent, while size^2 > min_size^2.
// The top-level phase splits regardless of min_size until size <= max_size and min_top
// levels are done, or max_top levels are reached.
//
// GB300 layout: the build is level-synchronous.  Cells with more than SMALL points are
// processed cooperatively by many blocks (fixed chunks of CH points, deterministic two-stage
// FP64 reductions, a stable scatter into the other of two point buffers).  Cells with at
// most SMALL points are finished by one warp each, which builds the whole subtree with warp
// reductions and ballot-based stable partitions, ping-ponging inside its own point range.
// Cell ids are positional, so no allocation counter is needed: an internal cell that
// splits [s,e) at m gets id m-1, a leaf starting at point s gets id (n-1)+s.
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdio>
#include <vector>
#include <algorithm>

#include "tc_internal.cuh"
#include "tc_host.hpp"

namespace tc {

// ---------------------------------------------------------------------------------------
// device helpers

__device__ __forceinline__ double coord3(const Points& P, int i, int axis)
{ return axis == 2 ? P.z[i] : axis == 1 ? P.y[i] : P.x[i]; }

__device__ __forceinline__ void set_err(int* err, int code)
{ atomicCAS(err, 0, code); }

// Position<Sphere>::normalize, include/Position.h:258-263.
__device__ __forceinline__ void normalize3(double& x, double& y, double& z)
{
    double n = sqrt(x * x + y * y + z * z);
    if (n == 0.) { x = 1.; y = 0.; z = 0.; }
    else { x /= n; y /= n; z /= n; }
}

// Bounds::getSplit, include/Bounds.h:65-66 (Flat) and 133-141 (ThreeD/Sphere).
__device__ __forceinline__ int split_axis(int coords, double xr, double yr, double zr)
{
    if (coords == FLAT) return yr > xr ? 1 : 0;
    return yr > xr ? (zr > yr ? 2 : 1) : (zr > xr ? 2 : 0);
}

// One point's contribution to the parallel-transported sum of a spin-s value,
// src/Cell.cpp:276-321.  (cx,cy,cz) is the centre as Position<Sphere> (normalised for
// ThreeD), cz_raw its raw z.
__device__ __forceinline__ void transport_add(int coords, int spin, double cx, double cy,
                                              double cz, double cz_raw, double px, double py,
                                              double pz, double wr, double wi, double& sr,
                                              double& si)
{
    if (spin == 0) { sr += wr; si += wi; return; }   // calculate_expmsialpha<0> = 1
    if (coords == THREED) normalize3(px, py, pz);
    double dsq = (cx - px) * (cx - px) + (cy - py) * (cy - py) + (cz - pz) * (cz - pz);
    if (dsq < 1.e-12) { sr += wr; si += wi; return; }
    double z1 = cz_raw, z2 = pz;
    double cosA = (z1 - z2) + 0.5 * z2 * dsq;
    double sinA = cy * px - cx * py;
    double cosB = (z2 - z1) + 0.5 * z1 * dsq;
    double sinB = sinA;
    double cb = -cosA * cosB + sinA * sinB;
    double sb = sinA * cosB + cosA * sinB;
    // calculate_expmsialpha<s>(cb + i sb), include/ProjectHelper.h:33-60.
    double er, ei;
    if (spin == 2) {
        double nrm = cb * cb + sb * sb;
        if (!(nrm > 0.)) nrm = 1.;
        er = (cb * cb - sb * sb) / nrm;
        ei = -(2. * cb * sb) / nrm;
    } else if (spin == 1) {
        double nrm = cb * cb + sb * sb;
        if (!(nrm > 0.)) nrm = 1.;
        nrm = sqrt(nrm);
        er = cb / nrm;
        ei = -sb / nrm;
    } else if (spin == 3) {
        // r^3, then conj(r^3) / |r^3|.
        const double r2r = cb * cb - sb * sb, r2i = 2. * cb * sb;
        const double r3r = r2r * cb - r2i * sb, r3i = r2r * sb + r2i * cb;
        double nrm = r3r * r3r + r3i * r3i;
        if (!(nrm > 0.)) nrm = 1.;
        nrm = sqrt(nrm);
        er = r3r / nrm;
        ei = -r3i / nrm;
    } else {
        // r^2 squared, then conj(r^4) / |r^2|^2.
        const double r2r = cb * cb - sb * sb, r2i = 2. * cb * sb;
        const double r4r = r2r * r2r - r2i * r2i, r4i = 2. * r2r * r2i;
        double nrm = r2r * r2r + r2i * r2i;
        if (!(nrm > 0.)) nrm = 1.;
        er = r4r / nrm;
        ei = -r4i / nrm;
    }
    sr += wr * er - wi * ei;
    si += wr * ei + wi * er;
}

// Writes a finished cell and links it to its parent.
__device__ __forceinline__ void write_cell(const Cells& C, int id, double x, double y, double z,
                                           float size, float w, float d1, float d2, int n,
                                           int s, int parent, int side)
{
    C.x[id] = x; C.y[id] = y; C.z[id] = z;
    C.size[id] = size; C.w[id] = w; C.d1[id] = d1; C.d2[id] = d2;
    C.n[id] = n; C.start[id] = s;
    C.left[id] = -1; C.right[id] = -1;
    C.parent[id] = parent;
    if (parent >= 0) {
        if (side == 0) C.left[parent] = id;
        else C.right[parent] = id;
    }
}

__device__ __forceinline__ void add_top(int* tops, int* ntop, int id, int s)
{
    int k = atomicAdd(ntop, 1);
    tops[2 * k] = s;
    tops[2 * k + 1] = id;
}

// The decision of SetupTopLevelCells (src/Field.cpp:57-80) followed by BuildCell
// (src/Cell.cpp:595-613).  Returns true to split.  Updates the task's top-phase state.
__device__ __forceinline__ bool decide_split(const BuildParams& P, int& intop, int mintop,
                                             int maxtop, double sizesq, bool& is_top)
{
    is_top = false;
    if (intop) {
        if (sizesq == 0. || (sizesq <= P.maxsizesq && mintop <= 0) || maxtop <= 0) {
            is_top = true;
            intop = 0;
        } else {
            return true;   // top-level phase: split regardless of min_size
        }
    }
    return sizesq > P.minsizesq;
}

__device__ __forceinline__ float cell_size(const BuildParams& P, double sizesq)
{ return P.brute ? __int_as_float(0x7f800000) : float(sqrt(sizesq)); }

// Copies point i of buffer A into slot j of buffer B.
__device__ __forceinline__ void move_point(const Points& A, int i, const Points& B, int j)
{
    B.x[j] = A.x[i]; B.y[j] = A.y[i]; B.z[j] = A.z[i]; B.wp[j] = A.wp[i];
    B.w[j] = A.w[i]; B.d1[j] = A.d1[i]; B.d2[j] = A.d2[i]; B.idx[j] = A.idx[i];
}

// ---------------------------------------------------------------------------------------
// Input preparation: Field::Field copies every point into a CellData (src/Field.cpp:180-196);
// Position<Sphere> normalises (include/Position.h:245), w is stored as float, and the
// payload as float(w*k) or complex<float>(w*g) (include/Cell.h:138-140, 176-178).

__global__ void k_prepare(int n, int coords, int dkind, const double* x, const double* y,
                          const double* z, const double* d1, const double* d2, const double* w,
                          const double* wpos, Points P)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double px = x[i], py = y[i], pz = (z && coords != FLAT) ? z[i] : 0.;
    if (coords == SPHERE) normalize3(px, py, pz);
    double wi = w[i];
    P.x[i] = px; P.y[i] = py; P.z[i] = pz;
    P.wp[i] = wpos ? wpos[i] : wi;
    P.w[i] = float(wi);
    if (dkind == DK) { P.d1[i] = float(wi * d1[i]); P.d2[i] = 0.f; }
    else if (dkind == DG) { P.d1[i] = float(wi * d1[i]); P.d2[i] = float(wi * d2[i]); }
    else { P.d1[i] = 0.f; P.d2[i] = 0.f; }
    P.idx[i] = i;
}

// ---------------------------------------------------------------------------------------
// Deterministic block reductions (warp butterfly, then warps in a fixed order).

template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double t = 0.;
    if (threadIdx.x == 0) {
        for (int k = 0; k < NT / 32; ++k) t += sh[k];
        sh[0] = t;
    }
    __syncthreads();
    return sh[0];
}

template <int NT, bool MAX>
__device__ __forceinline__ double block_ext(double v, double* sh)
{
    for (int o = 16; o > 0; o >>= 1) {
        double u = __shfl_xor_sync(0xffffffffu, v, o);
        v = MAX ? fmax(v, u) : fmin(v, u);
    }
    int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = sh[0];
        for (int k = 1; k < NT / 32; ++k) t = MAX ? fmax(t, sh[k]) : fmin(t, sh[k]);
        sh[0] = t;
    }
    __syncthreads();
    return sh[0];
}

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_min(double v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int warp_isum(int v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---------------------------------------------------------------------------------------
// Cooperative levels (cells with more than SMALL points).

__global__ void __launch_bounds__(CB) k_chunk_pass1(const Chunk* chunks, const BuildTask* tasks,
                                                     Points P0, Points P1, int coords, Part1* out)
{
    __shared__ double sh[CB / 32];
    const Chunk ch = chunks[blockIdx.x];
    const Points& P = tasks[ch.task].buf ? P1 : P0;
    double sx = 0., sy = 0., sz = 0., swp = 0., sw = 0.;
    double xmin = DBL_MAX, ymin = DBL_MAX, zmin = DBL_MAX;
    double xmax = -DBL_MAX, ymax = -DBL_MAX, zmax = -DBL_MAX;
    for (int i = ch.cs + threadIdx.x; i < ch.ce; i += CB) {
        double px = P.x[i], py = P.y[i], pz = P.z[i], wp = P.wp[i];
        sx += px * wp; sy += py * wp; sz += pz * wp; swp += wp; sw += P.w[i];
        xmin = fmin(xmin, px); xmax = fmax(xmax, px);
        ymin = fmin(ymin, py); ymax = fmax(ymax, py);
        zmin = fmin(zmin, pz); zmax = fmax(zmax, pz);
    }
    Part1 r;
    r.sx = block_sum<CB>(sx, sh); r.sy = block_sum<CB>(sy, sh); r.sz = block_sum<CB>(sz, sh);
    r.swp = block_sum<CB>(swp, sh); r.sw = block_sum<CB>(sw, sh);
    r.xmin = block_ext<CB, false>(xmin, sh); r.xmax = block_ext<CB, true>(xmax, sh);
    r.ymin = block_ext<CB, false>(ymin, sh); r.ymax = block_ext<CB, true>(ymax, sh);
    r.zmin = block_ext<CB, false>(zmin, sh); r.zmax = block_ext<CB, true>(zmax, sh);
    if (threadIdx.x == 0) out[blockIdx.x] = r;
    (void)coords;
}

// One warp per cooperative task: centroid, weight, split axis and value.
__global__ void k_task_combine1(int ntask, const BuildTask* tasks, const int* chunk0,
                                const Part1* part, Points P0, Points P1, BuildParams BP,
                                TaskStats* st)
{
    int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (t >= ntask) return;
    int c0 = chunk0[t], c1 = chunk0[t + 1];
    double sx = 0., sy = 0., sz = 0., swp = 0., sw = 0.;
    double xmin = DBL_MAX, ymin = DBL_MAX, zmin = DBL_MAX;
    double xmax = -DBL_MAX, ymax = -DBL_MAX, zmax = -DBL_MAX;
    for (int c = c0 + lane; c < c1; c += 32) {
        const Part1& p = part[c];
        sx += p.sx; sy += p.sy; sz += p.sz; swp += p.swp; sw += p.sw;
        xmin = fmin(xmin, p.xmin); xmax = fmax(xmax, p.xmax);
        ymin = fmin(ymin, p.ymin); ymax = fmax(ymax, p.ymax);
        zmin = fmin(zmin, p.zmin); zmax = fmax(zmax, p.zmax);
    }
    sx = warp_sum(sx); sy = warp_sum(sy); sz = warp_sum(sz); swp = warp_sum(swp); sw = warp_sum(sw);
    xmin = warp_min(xmin); ymin = warp_min(ymin); zmin = warp_min(zmin);
    xmax = warp_max(xmax); ymax = warp_max(ymax); zmax = warp_max(zmax);
    if (lane) return;
    const BuildTask tk = tasks[t];
    const Points& P = tk.buf ? P1 : P0;
    TaskStats s;
    // BuildCellData, src/Cell.cpp:170-200.
    if (swp != 0.) {
        s.cx = sx / swp; s.cy = sy / swp; s.cz = sz / swp;
        if (BP.coords == SPHERE) normalize3(s.cx, s.cy, s.cz);
    } else {
        s.cx = P.x[tk.s]; s.cy = P.y[tk.s]; s.cz = P.z[tk.s];
    }
    s.w = float(sw);
    s.axis = split_axis(BP.coords, xmax - xmin, ymax - ymin, zmax - zmin);
    if (BP.split == MIDDLE) {   // Bounds::getMiddle, include/Bounds.h:67-68
        s.splitval = s.axis == 2 ? (zmax + zmin) / 2. : s.axis == 1 ? (ymax + ymin) / 2.
                                                                     : (xmax + xmin) / 2.;
    } else {                    // Mean: the centroid, src/Cell.cpp:481-495
        s.splitval = s.axis == 2 ? s.cz : s.axis == 1 ? s.cy : s.cx;
    }
    // Remember whether all points share the split coordinate (needed by the fallback).
    double lo = s.axis == 2 ? zmin : s.axis == 1 ? ymin : xmin;
    double hi = s.axis == 2 ? zmax : s.axis == 1 ? ymax : xmax;
    s.allsame = (lo == hi) ? 1 : 0;
    s.mid = -1;
    s.copy = 0;
    s.byindex = 0;
    st[t] = s;
}

__global__ void __launch_bounds__(CB) k_chunk_pass2(const Chunk* chunks, const BuildTask* tasks,
                                                     const TaskStats* st, Points P0, Points P1,
                                                     int coords, int dkind, int spin, Part2* out)
{
    __shared__ double sh[CB / 32];
    __shared__ int shi[CB / 32];
    const Chunk ch = chunks[blockIdx.x];
    const TaskStats s = st[ch.task];
    const Points& P = tasks[ch.task].buf ? P1 : P0;
    double cx = s.cx, cy = s.cy, cz = s.cz;
    double tcx = cx, tcy = cy, tcz = cz;
    if (coords == THREED) normalize3(tcx, tcy, tcz);
    double sizesq = 0., pr = 0., pi = 0.;
    int nleft = 0;
    for (int i = ch.cs + threadIdx.x; i < ch.ce; i += CB) {
        double px = P.x[i], py = P.y[i], pz = P.z[i];
        double d = (cx - px) * (cx - px) + (cy - py) * (cy - py);
        if (coords != FLAT) d += (cz - pz) * (cz - pz);
        sizesq = fmax(sizesq, d);
        double c = s.axis == 2 ? pz : s.axis == 1 ? py : px;
        nleft += (c < s.splitval) ? 1 : 0;
        if (dkind == DK) {
            pr += P.d1[i];
        } else if (dkind == DG) {
            if (coords == FLAT) { pr += P.d1[i]; pi += P.d2[i]; }
            else transport_add(coords, spin, tcx, tcy, tcz, cz, px, py, pz, P.d1[i], P.d2[i], pr, pi);
        }
    }
    Part2 r;
    r.sizesq = block_ext<CB, true>(sizesq, sh);
    r.pr = block_sum<CB>(pr, sh);
    r.pi = block_sum<CB>(pi, sh);
    for (int o = 16; o > 0; o >>= 1) nleft += __shfl_xor_sync(0xffffffffu, nleft, o);
    if ((threadIdx.x & 31) == 0) shi[threadIdx.x >> 5] = nleft;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int k = 0; k < CB / 32; ++k) t += shi[k];
        r.nleft = t;
        r.pad = 0;
        out[blockIdx.x] = r;
    }
}

// One thread per cooperative task: finish the cell, decide, emit children, and set the
// scatter offsets of its chunks.
__global__ void k_task_combine2(int ntask, BuildTask* tasks, const int* chunk0, Chunk* chunks,
                                const Part2* part, TaskStats* st, BuildParams BP, Cells C,
                                int* tops, int* ntop, BuildTask* big_out, int* nbig_out,
                                BuildTask* small_out, int* nsmall_out, int* err)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntask) return;
    BuildTask tk = tasks[t];
    TaskStats s = st[t];
    int c0 = chunk0[t], c1 = chunk0[t + 1];
    double sizesq = 0., pr = 0., pi = 0.;
    int nleft = 0;
    for (int c = c0; c < c1; ++c) {
        sizesq = fmax(sizesq, part[c].sizesq);
        pr += part[c].pr; pi += part[c].pi;
        nleft += part[c].nleft;
    }
    const int n = tk.e - tk.s;
    bool is_top;
    int intop = tk.intop;
    bool split = decide_split(BP, intop, tk.mintop, tk.maxtop, sizesq, is_top);
    int mid = tk.s + nleft;
    int byindex = 0;
    if (split && (nleft == 0 || nleft == n)) {
        // SplitData falls back to Median when the mean puts everything on one side
        // (src/Cell.cpp:526-551).  On a cooperative level this is only done when every
        // point shares the split coordinate, where any order is a valid nth_element.
        if (s.allsame) { mid = (tk.s + tk.e) / 2; byindex = 1; }
        else { set_err(err, DEV_DEGENERATE_SPLIT); split = false; }
    }
    float d1 = float(pr), d2 = float(pi);
    if (BP.dkind == DN) { d1 = 0.f; d2 = 0.f; }
    if (BP.dkind == DK) d2 = 0.f;
    int id = split ? mid - 1 : (BP.n - 1) + tk.s;
    write_cell(C, id, s.cx, s.cy, s.cz, split ? cell_size(BP, sizesq) : 0.f, s.w, d1, d2, n,
               tk.s, tk.parent, tk.side);
    if (is_top) add_top(tops, ntop, id, tk.s);
    s.mid = split ? mid : -1;
    s.copy = (!split && tk.buf == 1) ? 1 : 0;
    s.byindex = byindex;
    st[t] = s;
    // Chunk offsets for the stable scatter.
    if (split) {
        int loff = 0, roff = 0;
        for (int c = c0; c < c1; ++c) {
            chunks[c].leftoff = loff;
            chunks[c].rightoff = roff;
            int cs = chunks[c].cs, ce = chunks[c].ce;
            int nl = byindex ? max(0, min(ce, mid) - cs) : part[c].nleft;
            loff += nl;
            roff += (ce - cs) - nl;
        }
        BuildTask L = tk, R = tk;
        L.e = mid; R.s = mid;
        L.parent = R.parent = id;
        L.side = 0; R.side = 1;
        L.intop = R.intop = intop;
        L.mintop = R.mintop = tk.mintop - 1;
        L.maxtop = R.maxtop = tk.maxtop - 1;
        L.buf = R.buf = tk.buf ^ 1;
        BuildTask* kids[2] = {&L, &R};
        for (int k = 0; k < 2; ++k) {
            BuildTask& c = *kids[k];
            if (c.e - c.s > SMALL && BP.split != MEDIAN) big_out[atomicAdd(nbig_out, 1)] = c;
            else small_out[atomicAdd(nsmall_out, 1)] = c;
        }
    }
}

// Stable partition of each split chunk into the other buffer (or a copy of a leaf's
// points into buffer 0).
__global__ void __launch_bounds__(CB) k_chunk_scatter(const Chunk* chunks, const BuildTask* tasks,
                                                       const TaskStats* st, Points P0, Points P1)
{
    __shared__ int wsum[2][CB / 32];
    const Chunk ch = chunks[blockIdx.x];
    const BuildTask tk = tasks[ch.task];
    const TaskStats s = st[ch.task];
    const Points& A = tk.buf ? P1 : P0;
    const Points& B = tk.buf ? P0 : P1;
    if (s.mid < 0) {
        if (s.copy) for (int i = ch.cs + threadIdx.x; i < ch.ce; i += CB) move_point(A, i, P0, i);
        return;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const bool by_index = s.byindex != 0;
    int lbase = tk.s + ch.leftoff;
    int rbase = s.mid + ch.rightoff;
    for (int base = ch.cs; base < ch.ce; base += CB) {
        int i = base + threadIdx.x;
        bool valid = i < ch.ce;
        bool left = false;
        if (valid) {
            if (by_index) left = i < s.mid;
            else {
                double c = s.axis == 2 ? A.z[i] : s.axis == 1 ? A.y[i] : A.x[i];
                left = c < s.splitval;
            }
        }
        unsigned bl = __ballot_sync(0xffffffffu, valid && left);
        unsigned br = __ballot_sync(0xffffffffu, valid && !left);
        unsigned lt = (1u << lane) - 1u;
        if (lane == 0) { wsum[0][wid] = __popc(bl); wsum[1][wid] = __popc(br); }
        __syncthreads();
        int lpre = 0, rpre = 0, ltot = 0, rtot = 0;
        for (int k = 0; k < CB / 32; ++k) {
            if (k < wid) { lpre += wsum[0][k]; rpre += wsum[1][k]; }
            ltot += wsum[0][k]; rtot += wsum[1][k];
        }
        if (valid) {
            int dst = left ? lbase + lpre + __popc(bl & lt) : rbase + rpre + __popc(br & lt);
            move_point(A, i, B, dst);
        }
        lbase += ltot;
        rbase += rtot;
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------
// Warp-finished subtrees (cells with at most SMALL points, or every cell for Median).

__device__ __forceinline__ int pack_meta(int side, int intop, int buf, int mintop, int maxtop)
{
    mintop = max(-2000, min(2000, mintop)) + 2048;
    maxtop = max(-2000, min(2000, maxtop)) + 2048;
    return side | (intop << 1) | (buf << 2) | (mintop << 8) | (maxtop << 20);
}

// Cells of at most THREAD_T points are finished by one thread: the steps of the warp loop
// below (src/Cell.cpp:170-200, 520-615) with the sums taken in point order.  Small cells
// are ~94% of a subtree's cells, and a warp spends the same reductions on a 2-point cell
// as on a 2048-point one.
constexpr int THREAD_T = 32;

__device__ void subtree_by_thread(WTask root, Points P0, Points P1, const BuildParams& BP,
                                  const Cells& C, int* tops, int* ntop, int* err)
{
    WTask stk[THREAD_T + 1];
    int sp = 0;
    stk[sp++] = root;
    while (sp > 0) {
        const WTask w = stk[--sp];
        const int s = w.s, e = w.e, n = e - s;
        const int side = w.meta & 1, buf = (w.meta >> 2) & 1;
        int intop = (w.meta >> 1) & 1;
        const int mintop = ((w.meta >> 8) & 0xfff) - 2048;
        const int maxtop = ((w.meta >> 20) & 0xfff) - 2048;
        const Points& A = buf ? P1 : P0;
        const Points& B = buf ? P0 : P1;
        if (n == 1) {
            const int id = (BP.n - 1) + s;
            write_cell(C, id, A.x[s], A.y[s], A.z[s], 0.f, A.w[s], A.d1[s], A.d2[s], 1, s,
                       w.parent, side);
            if (intop) add_top(tops, ntop, id, s);
            if (buf) move_point(A, s, P0, s);
            continue;
        }
        double sx = 0., sy = 0., sz = 0., swp = 0., sw = 0.;
        double xmin = DBL_MAX, ymin = DBL_MAX, zmin = DBL_MAX;
        double xmax = -DBL_MAX, ymax = -DBL_MAX, zmax = -DBL_MAX;
        for (int i = s; i < e; ++i) {
            const double px = A.x[i], py = A.y[i], pz = A.z[i], wp = A.wp[i];
            sx += px * wp; sy += py * wp; sz += pz * wp; swp += wp; sw += A.w[i];
            xmin = fmin(xmin, px); xmax = fmax(xmax, px);
            ymin = fmin(ymin, py); ymax = fmax(ymax, py);
            zmin = fmin(zmin, pz); zmax = fmax(zmax, pz);
        }
        double cx, cy, cz;
        if (swp != 0.) {
            cx = sx / swp; cy = sy / swp; cz = sz / swp;
            if (BP.coords == SPHERE) normalize3(cx, cy, cz);
        } else {
            cx = A.x[s]; cy = A.y[s]; cz = A.z[s];
        }
        const int axis = split_axis(BP.coords, xmax - xmin, ymax - ymin, zmax - zmin);
        double splitval;
        if (BP.split == MIDDLE)
            splitval = axis == 2 ? (zmax + zmin) / 2. : axis == 1 ? (ymax + ymin) / 2.
                                                                   : (xmax + xmin) / 2.;
        else
            splitval = axis == 2 ? cz : axis == 1 ? cy : cx;
        double tcx = cx, tcy = cy, tcz = cz;
        if (BP.coords == THREED) normalize3(tcx, tcy, tcz);
        double sizesq = 0., pr = 0., pi = 0.;
        int nleft = 0;
        for (int i = s; i < e; ++i) {
            const double px = A.x[i], py = A.y[i], pz = A.z[i];
            double d = (cx - px) * (cx - px) + (cy - py) * (cy - py);
            if (BP.coords != FLAT) d += (cz - pz) * (cz - pz);
            sizesq = fmax(sizesq, d);
            const double c = axis == 2 ? pz : axis == 1 ? py : px;
            nleft += (c < splitval) ? 1 : 0;
            if (BP.dkind == DK) pr += A.d1[i];
            else if (BP.dkind == DG) {
                if (BP.coords == FLAT) { pr += A.d1[i]; pi += A.d2[i]; }
                else transport_add(BP.coords, BP.spin, tcx, tcy, tcz, cz, px, py, pz, A.d1[i],
                                   A.d2[i], pr, pi);
            }
        }
        bool is_top;
        const bool split = decide_split(BP, intop, mintop, maxtop, sizesq, is_top);
        bool use_rank = (BP.split == MEDIAN);
        int mid = s + nleft;
        if (split && !use_rank && (nleft == 0 || nleft == n)) use_rank = true;
        if (split && use_rank) mid = (s + e) / 2;   // SplitDataCore<Median>, src/Cell.cpp:464-479
        float d1 = float(pr), d2 = float(pi);
        if (BP.dkind == DN) { d1 = 0.f; d2 = 0.f; }
        if (BP.dkind == DK) d2 = 0.f;
        const int id = split ? mid - 1 : (BP.n - 1) + s;
        write_cell(C, id, cx, cy, cz, split ? cell_size(BP, sizesq) : 0.f, float(sw), d1, d2, n,
                   s, w.parent, side);
        if (is_top) add_top(tops, ntop, id, s);
        if (!split) {
            if (buf) for (int i = s; i < e; ++i) move_point(A, i, P0, i);
            continue;
        }
        // Stable partition into the other buffer.
        int lo = s, hi = mid;
        for (int i = s; i < e; ++i) {
            const double c = axis == 2 ? A.z[i] : axis == 1 ? A.y[i] : A.x[i];
            bool left;
            if (!use_rank) {
                left = c < splitval;
            } else {
                int rank = 0;
                for (int j = s; j < e; ++j) {
                    const double cj = axis == 2 ? A.z[j] : axis == 1 ? A.y[j] : A.x[j];
                    rank += (cj < c || (cj == c && j < i)) ? 1 : 0;
                }
                left = rank < (mid - s);
            }
            move_point(A, i, B, left ? lo++ : hi++);
        }
        if (sp + 2 > THREAD_T + 1) { set_err(err, DEV_TASK_OVERFLOW); return; }
        const int nb = buf ^ 1;
        stk[sp++] = WTask{mid, e, id, pack_meta(1, intop, nb, mintop - 1, maxtop - 1)};
        stk[sp++] = WTask{s, mid, id, pack_meta(0, intop, nb, mintop - 1, maxtop - 1)};
    }
}

__global__ void k_small_subtree(int ntask, const BuildTask* tasks, Points P0, Points P1,
                                BuildParams BP, Cells C, int* tops, int* ntop, WTask* wstack,
                                int* err)
{
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= ntask) return;
    const BuildTask root = tasks[t];
    WTask* stk = wstack + root.s;          // this task owns [root.s, root.e) of the stack
    // Cells of at most THREAD_T points wait here until each lane can take one.
    __shared__ WTask deferred[4][32];
    WTask* dq = deferred[(threadIdx.x >> 5) & 3];
    int ndq = 0;
    int sp = 0;
    if (lane == 0) {
        WTask w0 = {root.s, root.e, root.parent,
                    pack_meta(root.side, root.intop, root.buf, root.mintop, root.maxtop)};
        stk[0] = w0;
    }
    sp = 1;
    __syncwarp();
    while (sp > 0 || ndq > 0) {
        if (sp == 0 || ndq == 32) {
            __syncwarp();
            if (lane < ndq) subtree_by_thread(dq[lane], P0, P1, BP, C, tops, ntop, err);
            ndq = 0;
            __syncwarp();
            continue;
        }
        --sp;
        WTask w = stk[sp];
        __syncwarp();
        if (w.e - w.s <= THREAD_T) {
            if (lane == 0) dq[ndq] = w;
            ++ndq;
            continue;
        }
        const int s = w.s, e = w.e, n = e - s;
        const int side = w.meta & 1, buf = (w.meta >> 2) & 1;
        int intop = (w.meta >> 1) & 1;
        const int mintop = ((w.meta >> 8) & 0xfff) - 2048;
        const int maxtop = ((w.meta >> 20) & 0xfff) - 2048;
        const Points& A = buf ? P1 : P0;
        const Points& B = buf ? P0 : P1;
        if (n == 1) {
            // Single point: a leaf holding the point's own data (src/Cell.cpp:564-575).
            if (lane == 0) {
                int id = (BP.n - 1) + s;
                write_cell(C, id, A.x[s], A.y[s], A.z[s], 0.f, A.w[s], A.d1[s], A.d2[s], 1, s,
                           w.parent, side);
                if (intop) add_top(tops, ntop, id, s);
                if (buf) move_point(A, s, P0, s);
            }
            __syncwarp();
            continue;
        }
        // Pass 1: centroid, weight, bounds (src/Cell.cpp:170-200, 520-525).
        double sx = 0., sy = 0., sz = 0., swp = 0., sw = 0.;
        double xmin = DBL_MAX, ymin = DBL_MAX, zmin = DBL_MAX;
        double xmax = -DBL_MAX, ymax = -DBL_MAX, zmax = -DBL_MAX;
        for (int i = s + lane; i < e; i += 32) {
            double px = A.x[i], py = A.y[i], pz = A.z[i], wp = A.wp[i];
            sx += px * wp; sy += py * wp; sz += pz * wp; swp += wp; sw += A.w[i];
            xmin = fmin(xmin, px); xmax = fmax(xmax, px);
            ymin = fmin(ymin, py); ymax = fmax(ymax, py);
            zmin = fmin(zmin, pz); zmax = fmax(zmax, pz);
        }
        sx = warp_sum(sx); sy = warp_sum(sy); sz = warp_sum(sz); swp = warp_sum(swp);
        sw = warp_sum(sw);
        xmin = warp_min(xmin); ymin = warp_min(ymin); zmin = warp_min(zmin);
        xmax = warp_max(xmax); ymax = warp_max(ymax); zmax = warp_max(zmax);
        double cx, cy, cz;
        if (swp != 0.) {
            cx = sx / swp; cy = sy / swp; cz = sz / swp;
            if (BP.coords == SPHERE) normalize3(cx, cy, cz);
        } else {
            cx = A.x[s]; cy = A.y[s]; cz = A.z[s];
        }
        const int axis = split_axis(BP.coords, xmax - xmin, ymax - ymin, zmax - zmin);
        double splitval;
        if (BP.split == MIDDLE)
            splitval = axis == 2 ? (zmax + zmin) / 2. : axis == 1 ? (ymax + ymin) / 2.
                                                                   : (xmax + xmin) / 2.;
        else
            splitval = axis == 2 ? cz : axis == 1 ? cy : cx;
        // Pass 2: size, payload, left count.
        double tcx = cx, tcy = cy, tcz = cz;
        if (BP.coords == THREED) normalize3(tcx, tcy, tcz);
        double sizesq = 0., pr = 0., pi = 0.;
        int nleft = 0;
        for (int i = s + lane; i < e; i += 32) {
            double px = A.x[i], py = A.y[i], pz = A.z[i];
            double d = (cx - px) * (cx - px) + (cy - py) * (cy - py);
            if (BP.coords != FLAT) d += (cz - pz) * (cz - pz);
            sizesq = fmax(sizesq, d);
            double c = axis == 2 ? pz : axis == 1 ? py : px;
            nleft += (c < splitval) ? 1 : 0;
            if (BP.dkind == DK) pr += A.d1[i];
            else if (BP.dkind == DG) {
                if (BP.coords == FLAT) { pr += A.d1[i]; pi += A.d2[i]; }
                else transport_add(BP.coords, BP.spin, tcx, tcy, tcz, cz, px, py, pz, A.d1[i],
                                   A.d2[i], pr, pi);
            }
        }
        sizesq = warp_max(sizesq); pr = warp_sum(pr); pi = warp_sum(pi);
        nleft = warp_isum(nleft);
        bool is_top;
        bool split = decide_split(BP, intop, mintop, maxtop, sizesq, is_top);
        bool use_rank = (BP.split == MEDIAN);
        int mid = s + nleft;
        if (split && !use_rank && (nleft == 0 || nleft == n)) use_rank = true;
        if (split && use_rank) mid = (s + e) / 2;   // SplitDataCore<Median>, src/Cell.cpp:464-479
        float d1 = float(pr), d2 = float(pi);
        if (BP.dkind == DN) { d1 = 0.f; d2 = 0.f; }
        if (BP.dkind == DK) d2 = 0.f;
        const int id = split ? mid - 1 : (BP.n - 1) + s;
        if (lane == 0) {
            write_cell(C, id, cx, cy, cz, split ? cell_size(BP, sizesq) : 0.f, float(sw), d1, d2,
                       n, s, w.parent, side);
            if (is_top) add_top(tops, ntop, id, s);
        }
        if (!split) {
            if (buf) for (int i = s + lane; i < e; i += 32) move_point(A, i, P0, i);
            __syncwarp();
            continue;
        }
        // Stable partition into the other buffer.
        int lbase = s, rbase = mid;
        const unsigned lt = (1u << lane) - 1u;
        for (int base = s; base < e; base += 32) {
            int i = base + lane;
            bool valid = i < e;
            bool left = false;
            if (valid) {
                double c = axis == 2 ? A.z[i] : axis == 1 ? A.y[i] : A.x[i];
                if (!use_rank) {
                    left = c < splitval;
                } else {
                    // Rank of point i by (coordinate, position): the mid-s smallest go left.
                    int rank = 0;
                    for (int j = s; j < e; ++j) {
                        double cj = axis == 2 ? A.z[j] : axis == 1 ? A.y[j] : A.x[j];
                        rank += (cj < c || (cj == c && j < i)) ? 1 : 0;
                    }
                    left = rank < (mid - s);
                }
            }
            unsigned bl = __ballot_sync(0xffffffffu, valid && left);
            unsigned br = __ballot_sync(0xffffffffu, valid && !left);
            if (valid) {
                int dst = left ? lbase + __popc(bl & lt) : rbase + __popc(br & lt);
                move_point(A, i, B, dst);
            }
            lbase += __popc(bl);
            rbase += __popc(br);
        }
        __syncwarp();
        // Push right then left (left is processed first).
        if (lane == 0) {
            int nb = buf ^ 1;
            WTask R = {mid, e, id, pack_meta(1, intop, nb, mintop - 1, maxtop - 1)};
            WTask L = {s, mid, id, pack_meta(0, intop, nb, mintop - 1, maxtop - 1)};
            if (sp + 2 > root.e - root.s) set_err(err, DEV_TASK_OVERFLOW);
            else { stk[sp] = R; stk[sp + 1] = L; }
        }
        sp += 2;
        if (sp > root.e - root.s) break;
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------------
// Structural check of the finished tree: every internal cell has two children that split
// its point range exactly.  This guarantees that the traversal (which only descends into
// children) terminates; the traversal is not launched on a tree that fails it.

__global__ void k_validate_tree(int ncap, Cells C, const int* tops, int ntop, int* err)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ntop) {
        int t = tops[i];
        if (t < 0 || t >= ncap) set_err(err, DEV_BAD_CHILD);
    }
    if (i >= ncap) return;
    int L = C.left[i], R = C.right[i];
    if (L < 0 && R < 0) return;
    if (L < 0 || R < 0 || L >= ncap || R >= ncap || L == i || R == i) {
        set_err(err, DEV_BAD_CHILD);
        return;
    }
    int n = C.n[i], nl = C.n[L], nr = C.n[R];
    if (nl < 1 || nr < 1 || nl + nr != n || C.start[L] != C.start[i] ||
        C.start[R] != C.start[i] + nl)
        set_err(err, DEV_BAD_CHILD);
}

void launch_validate_tree(int ncap, const Cells& C, const int* tops, int ntop, int* err,
                          cudaStream_t st)
{
    int m = ncap > ntop ? ncap : ntop;
    if (m <= 0) return;
    count_launch(); k_validate_tree<<<(m + 255) / 256, 256, 0, st>>>(ncap, C, tops, ntop, err);
}

// ---------------------------------------------------------------------------------------
// Host orchestration.

int scratch_ensure_level(BuildScratch& S, int nt, int nc)
{
    if (nt > S.cap_tasks) {
        int cap = std::max(nt, 2 * S.cap_tasks);
        dfree(S.tasks); dfree(S.chunk0); dfree(S.stats); dfree(S.big_next);
        TC_TRY(dalloc(&S.tasks, cap));
        TC_TRY(dalloc(&S.chunk0, cap + 1));
        TC_TRY(dalloc(&S.stats, cap));
        TC_TRY(dalloc(&S.big_next, 2 * (size_t)cap + 2));
        S.cap_tasks = cap;
    }
    if (nc > S.cap_chunks) {
        int cap = std::max(nc, 2 * S.cap_chunks);
        dfree(S.chunks); dfree(S.part1); dfree(S.part2);
        TC_TRY(dalloc(&S.chunks, cap));
        TC_TRY(dalloc(&S.part1, cap));
        TC_TRY(dalloc(&S.part2, cap));
        S.cap_chunks = cap;
    }
    return 0;
}

int build_tree(const BuildParams& BP, Points bufs[2], Cells C, int* d_tops, int* d_ntop,
               BuildScratch& S, cudaStream_t st, std::vector<int>& tops_out, int* d_err,
               int mintop, int maxtop)
{
    const int n = BP.n;
    std::vector<BuildTask> big;
    BuildTask root;
    root.s = 0; root.e = n; root.parent = -1; root.side = 0;
    root.mintop = mintop; root.maxtop = maxtop; root.intop = 1; root.buf = 0;
    std::vector<BuildTask> small_host;
    int nsmall = 0;
    TC_CU(cudaMemsetAsync(d_ntop, 0, sizeof(int), st));
    TC_CU(cudaMemsetAsync(S.counters, 0, 2 * sizeof(int), st));
    if (n > SMALL && BP.split != MEDIAN) big.push_back(root);
    else {
        TC_CU(cudaMemcpyAsync(S.small, &root, sizeof(BuildTask), cudaMemcpyHostToDevice, st));
        nsmall = 1;
        TC_CU(cudaMemcpyAsync(S.counters + 1, &nsmall, sizeof(int), cudaMemcpyHostToDevice, st));
    }
    while (!big.empty()) {
        int nt = (int)big.size();
        std::vector<int> c0(nt + 1);
        std::vector<Chunk> chunks;
        for (int t = 0; t < nt; ++t) {
            c0[t] = (int)chunks.size();
            for (int cs = big[t].s; cs < big[t].e; cs += CH) {
                Chunk c; c.task = t; c.cs = cs; c.ce = std::min(cs + CH, big[t].e);
                c.leftoff = c.rightoff = 0;
                chunks.push_back(c);
            }
        }
        c0[nt] = (int)chunks.size();
        int nc = (int)chunks.size();
        TC_TRY(scratch_ensure_level(S, nt, nc));
        TC_CU(cudaMemcpyAsync(S.tasks, big.data(), nt * sizeof(BuildTask), cudaMemcpyHostToDevice, st));
        TC_CU(cudaMemcpyAsync(S.chunk0, c0.data(), (nt + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
        TC_CU(cudaMemcpyAsync(S.chunks, chunks.data(), nc * sizeof(Chunk), cudaMemcpyHostToDevice, st));
        TC_CU(cudaMemsetAsync(S.counters, 0, sizeof(int), st));   // next big count
        count_launch(); k_chunk_pass1<<<nc, CB, 0, st>>>(S.chunks, S.tasks, bufs[0], bufs[1], BP.coords, S.part1);
        count_launch(); k_task_combine1<<<(nt * 32 + 255) / 256, 256, 0, st>>>(nt, S.tasks, S.chunk0, S.part1,
                                                                bufs[0], bufs[1], BP, S.stats);
        count_launch(); k_chunk_pass2<<<nc, CB, 0, st>>>(S.chunks, S.tasks, S.stats, bufs[0], bufs[1], BP.coords,
                                         BP.dkind, BP.spin, S.part2);
        count_launch(); k_task_combine2<<<(nt + 127) / 128, 128, 0, st>>>(nt, S.tasks, S.chunk0, S.chunks, S.part2,
                                                          S.stats, BP, C, d_tops, d_ntop, S.big_next,
                                                          S.counters, S.small + 0, S.counters + 1,
                                                          d_err);
        count_launch(); k_chunk_scatter<<<nc, CB, 0, st>>>(S.chunks, S.tasks, S.stats, bufs[0], bufs[1]);
        TC_CU(cudaGetLastError());
        int cnt[2];
        TC_CU(cudaMemcpyAsync(cnt, S.counters, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
        TC_CU(cudaStreamSynchronize(st));
        big.resize(cnt[0]);
        if (cnt[0] > 0)
            TC_CU(cudaMemcpy(big.data(), S.big_next, cnt[0] * sizeof(BuildTask), cudaMemcpyDeviceToHost));
        nsmall = cnt[1];
    }
    if (nsmall > 0) {
        int threads = 128;
        long long blocks = ((long long)nsmall * 32 + threads - 1) / threads;
        count_launch(); k_small_subtree<<<(unsigned)blocks, threads, 0, st>>>(nsmall, S.small, bufs[0], bufs[1],
                                                              BP, C, d_tops, d_ntop, S.wstack, d_err);
        TC_CU(cudaGetLastError());
    }
    int ntop = 0;
    TC_CU(cudaMemcpyAsync(&ntop, d_ntop, sizeof(int), cudaMemcpyDeviceToHost, st));
    TC_CU(cudaStreamSynchronize(st));
    std::vector<int> pairs(2 * (size_t)ntop);
    if (ntop > 0)
        TC_CU(cudaMemcpy(pairs.data(), d_tops, 2 * sizeof(int) * ntop, cudaMemcpyDeviceToHost));
    // Tops in the reference's depth-first order = increasing first point (left before right).
    std::vector<std::pair<int, int>> v(ntop);
    for (int k = 0; k < ntop; ++k) v[k] = {pairs[2 * k], pairs[2 * k + 1]};
    std::sort(v.begin(), v.end());
    tops_out.resize(ntop);
    for (int k = 0; k < ntop; ++k) tops_out[k] = v[k].second;
    return 0;
}

void launch_prepare(int n, int coords, int dkind, const double* x, const double* y,
                    const double* z, const double* d1, const double* d2, const double* w,
                    const double* wpos, Points P, cudaStream_t st)
{
    if (n <= 0) return;
    count_launch(); k_prepare<<<(n + 255) / 256, 256, 0, st>>>(n, coords, dkind, x, y, z, d1, d2, w, wpos, P);
}

// Overall centre and size of the catalog (Field::Field, src/Field.cpp:198-203):
// one deterministic cooperative task over [0,n).
int field_center(const BuildParams& BP, Points P, BuildScratch& S, cudaStream_t st,
                 double out[4])
{
    const int n = BP.n;
    BuildTask root;
    root.s = 0; root.e = n; root.parent = -1; root.side = 0;
    root.mintop = 0; root.maxtop = 0; root.intop = 0; root.buf = 0;
    std::vector<int> c0(2);
    std::vector<Chunk> chunks;
    for (int cs = 0; cs < n; cs += CH) {
        Chunk c; c.task = 0; c.cs = cs; c.ce = std::min(cs + CH, n); c.leftoff = c.rightoff = 0;
        chunks.push_back(c);
    }
    c0[0] = 0; c0[1] = (int)chunks.size();
    int nc = (int)chunks.size();
    TC_TRY(scratch_ensure_level(S, 1, nc));
    Points Pn = P;
    TC_CU(cudaMemcpyAsync(S.tasks, &root, sizeof(BuildTask), cudaMemcpyHostToDevice, st));
    TC_CU(cudaMemcpyAsync(S.chunk0, c0.data(), 2 * sizeof(int), cudaMemcpyHostToDevice, st));
    TC_CU(cudaMemcpyAsync(S.chunks, chunks.data(), nc * sizeof(Chunk), cudaMemcpyHostToDevice, st));
    BuildParams B2 = BP;
    B2.split = MEAN;
    count_launch(); k_chunk_pass1<<<nc, CB, 0, st>>>(S.chunks, S.tasks, Pn, Pn, BP.coords, S.part1);
    count_launch(); k_task_combine1<<<1, 32, 0, st>>>(1, S.tasks, S.chunk0, S.part1, Pn, Pn, B2, S.stats);
    count_launch(); k_chunk_pass2<<<nc, CB, 0, st>>>(S.chunks, S.tasks, S.stats, Pn, Pn, BP.coords, DN, 0, S.part2);
    TC_CU(cudaGetLastError());
    std::vector<Part2> p2(nc);
    TaskStats ts;
    TC_CU(cudaMemcpyAsync(p2.data(), S.part2, nc * sizeof(Part2), cudaMemcpyDeviceToHost, st));
    TC_CU(cudaMemcpyAsync(&ts, S.stats, sizeof(TaskStats), cudaMemcpyDeviceToHost, st));
    TC_CU(cudaStreamSynchronize(st));
    double sizesq = 0.;
    for (int c = 0; c < nc; ++c) sizesq = std::max(sizesq, p2[c].sizesq);
    out[0] = ts.cx; out[1] = ts.cy; out[2] = ts.cz; out[3] = sizesq;
    return 0;
}

}  // namespace tc
