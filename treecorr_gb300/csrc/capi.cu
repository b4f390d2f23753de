// capi.cu -- the C ABI (include/tcgpu.h): fields, corr objects, process calls.
//
// Objects mirror the reference's native classes: a tc_field is Field<D,C>
// (include/Field.h:88-106) holding its catalog on the device and building its tree lazily;
// a tc_corr2 is Corr2<D1,D2> (include/Corr2.h:139-223) aliasing caller-owned output arrays
// and adding into them.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include "../../include/tcgpu.h"
#include "tc_internal.cuh"
#include "tc_host.hpp"
#include "traverse2pt.hpp"
#include "multipole.hpp"
#include "learned.hpp"
#include "kmeans.hpp"
#include "catalog.hpp"

namespace tc {

static thread_local std::string g_last_error;
void set_last_error(const std::string& msg) { g_last_error = msg; }

static std::atomic<long long> g_launches{0};
// Fixed-order 2-point expansion (bitwise repeatable sums); tc_set_deterministic.
static std::atomic<int> g_deterministic{1};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static cudaStream_t g_stream = nullptr;
static int stream_get(cudaStream_t* s)
{
    if (!g_stream) TC_CU(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking));
    *s = g_stream;
    return 0;
}

static const char* dev_err_msg(int code)
{
    switch (code) {
      case DEV_STACK_OVERFLOW: return "traversal stack overflow";
      case DEV_SPILL_OVERFLOW: return "traversal spill list overflow";
      case DEV_DEGENERATE_SPLIT:
          return "mean split put every point of a large cell on one side although the points "
                 "differ along the split axis (degenerate weights)";
      case DEV_BAD_CHILD: return "traversal asked to split a leaf cell (inconsistent tree)";
      case DEV_TASK_OVERFLOW: return "tree build task stack overflow";
      case DEV_COPY_TIMEOUT:
          return "an asynchronous copy of tile leaves into shared memory did not complete within "
                 "its wait limit";
      default: return "unknown device error";
    }
}

}  // namespace tc

using namespace tc;

struct tc_field {
    int dkind = 0, coords = 0, split = 0, brute = 0, mintop = 0, maxtop = 0;
    int64_t n = 0;
    double minsize = 0., maxsize = 0.;
    bool built = false;
    Points buf[2] = {};
    Cells cells = {};
    TCell* tcells = nullptr;
    int* d_tops_raw = nullptr;   // (start, id) pairs written by the build
    int* d_ntop = nullptr;
    int* d_tops = nullptr;       // ordered top ids
    std::vector<int> tops;
    double center[4] = {0., 0., 0., 0.};   // x, y, z, size^2
    BuildScratch S;
    int* d_err = nullptr;
    float build_ms = 0.f;
    double* leafsums = nullptr;  // 4 per cell, built on first multipole use
    float4* leafsums_f = nullptr;  // the same as floats
    int km_iters = 0;            // iterations of the last k-means run
};

struct tc_corr3 {
    int dv = TC_GDATA;           // data kind of vertex 1
    int dk = TC_GDATA;           // data kind of vertex 2
    int dk3 = TC_GDATA;          // data kind of vertex 3
    int bin_type = 0, nbins = 0, maxn = 0;
    double minsep = 0., maxsep = 0., binsize = 0., b = 0., a = 0.;
    double* zeta[8] = {nullptr};
    double *meand2 = nullptr, *meanlogd2 = nullptr, *meand3 = nullptr, *meanlogd3 = nullptr;
    double *weight = nullptr, *weight_im = nullptr, *ntri = nullptr;
    MPScratch X;
    double ms = 0.;
};

struct tc_corr2 {
    int d1 = 0, d2 = 0, bin_type = 0, nbins = 0;
    double minsep = 0., maxsep = 0., binsize = 0., b = 0., a = 0.;
    double *xi0 = nullptr, *xi1 = nullptr, *xi2 = nullptr, *xi3 = nullptr;
    double *meanr = nullptr, *meanlogr = nullptr, *weight = nullptr, *npairs = nullptr;
    tc_stats stats = {};
    // Traversal scratch, grown on demand.
    int nwarps_alloc = 0, nq_alloc = 0;
    double* wacc = nullptr;
    unsigned long long* wnp = nullptr;
    double* tot = nullptr;
    unsigned long long* totnp = nullptr;
    unsigned long long* ctl = nullptr;   // root_next, nout, counters[3]
    int* idle = nullptr;
    int* d_err = nullptr;
    std::vector<int2*> lev;              // per-level item buffers of the expansion
    std::vector<long long> levcap;
    ExpandSched* sched = nullptr;        // device-side schedule of the expansion
    // Learned opening criterion (mode 2) or sampling of its training pairs (mode 1).
    int mode = 0;
    MLPPacked* mlp = nullptr;
    float mlp_thr = 0.f, cand_factor = 4.f;
    int2* samples = nullptr;
    long long sample_cap = 0;
    unsigned sample_mod = 1;
    // Leaf-pair tiles of the exact mode: the tile list, its control words and the bin edges.
    int2* tiles = nullptr;
    long long tile_cap = 0;
    unsigned long long* tctl = nullptr;
    float* tedge = nullptr;              // [2][nbins+1]: 1/edge^2, log(edge)
    std::vector<cudaEvent_t> kev;        // per-launch events of an expansion batch
    // Tuning (tc_corr2_set_tuning / tc_corr2_autotune): tile leaf size and items per
    // expansion launch, 0 = the defaults.  root_limit / no_output: the autotuner's sample
    // runs (only the first root_limit top-level pairs, results not added to the outputs).
    int tile_leaf = 0;
    long long chunk = 0;
    long long root_limit = 0;
    bool no_output = false;
    // Fixed-order expansion regions (tc_set_deterministic): per warp, 4 children and 1 tile
    // per item it takes at most; counts [2][nwarps].
    int2* det_out = nullptr;
    int2* det_tout = nullptr;
    int* det_cnt = nullptr;
    long long det_out_cap = 0, det_tout_cap = 0;
    int det_cnt_cap = 0;
    unsigned long long* wctr = nullptr;  // per-warp counter slots [warps][8]
    int wctr_cap = 0;
    ~tc_corr2() { for (auto e : kev) cudaEventDestroy(e); }
};

namespace {
// Patches: the combined cell records of all patch fields (children ids rebased, patch id in
// d.y) with their FP64 centres.
__global__ void k_rebase_cells(TCell* t, long long n, int base, int patch)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    TCell c = t[i];
    const int L = __float_as_int(c.c.w), R = __float_as_int(c.d.x);
    c.c.w = __int_as_float(L >= 0 ? L + base : L);
    c.d.x = __int_as_float(R >= 0 ? R + base : R);
    c.d.y = __int_as_float(patch);
    t[i] = c;
}

// Jackknife rows (corr2base.py:1787-1823 pair weights, 1333-1352 _sum, 1274-1294 _finalize):
// row l sums the patch pairs' arrays with weight w(l, i, j) and divides by the weight.
// res: [npair][8][nb] (weight, meanr, meanlogr, xi0..xi3, npairs); stat: the xi indices
// that make the data vector (GG: xi0, xi2 = xip, xim; KK: xi0).
__global__ void k_jackknife_rows(const double* res, const int* pi, const int* pj, int npair,
                                 int nb, int cpw, double wmatch, int nstat, int s0, int s1,
                                 double* v, double* wrow)
{
    const int l = blockIdx.x;
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
        double wsum = 0., x0 = 0., x1 = 0.;
        for (int p = 0; p < npair; ++p) {
            const int i = pi[p], j = pj[p];
            double w;
            if (cpw == 0) w = (i != l && j != l) ? 1. : 0.;                  // simple
            else if (i == l && j == l) w = 0.;
            else if (i == l || j == l) w = cpw == 1 ? 0.5 : wmatch;        // mean / match
            else w = 1.;
            if (w == 0.) continue;
            const double* r = res + (size_t)p * 8 * nb;
            wsum += w * r[t];
            x0 += w * r[(3 + s0) * nb + t];
            if (nstat > 1) x1 += w * r[(3 + s1) * nb + t];
        }
        v[(size_t)l * nstat * nb + t] = wsum != 0. ? x0 / wsum : 0.;
        if (nstat > 1) v[(size_t)l * nstat * nb + nb + t] = wsum != 0. ? x1 / wsum : 0.;
        if (t == 0) wrow[l] = 0.;
    }
}

// C = (1 - 1/n) sum_l (v_l - mean)(v_l - mean)^T (_cov_jackknife, corr2base.py:2432-2445).
__global__ void k_jackknife_cov(const double* v, int nrow, int nv, double* cov)
{
    const int a = blockIdx.x, b = threadIdx.x + blockIdx.y * blockDim.x;
    if (b >= nv) return;
    double ma = 0., mb = 0.;
    for (int l = 0; l < nrow; ++l) { ma += v[(size_t)l * nv + a]; mb += v[(size_t)l * nv + b]; }
    ma /= nrow; mb /= nrow;
    double c = 0.;
    for (int l = 0; l < nrow; ++l) c += (v[(size_t)l * nv + a] - ma) * (v[(size_t)l * nv + b] - mb);
    cov[(size_t)a * nv + b] = (1. - 1. / nrow) * c;
}
}  // namespace

namespace {

void free_points(Points& P)
{
    dfree(P.x); dfree(P.y); dfree(P.z); dfree(P.wp); dfree(P.w); dfree(P.d1); dfree(P.d2);
    dfree(P.idx);
}

int alloc_points(Points& P, int64_t n)
{
    TC_TRY(dalloc(&P.x, n)); TC_TRY(dalloc(&P.y, n)); TC_TRY(dalloc(&P.z, n));
    TC_TRY(dalloc(&P.wp, n)); TC_TRY(dalloc(&P.w, n)); TC_TRY(dalloc(&P.d1, n));
    TC_TRY(dalloc(&P.d2, n)); TC_TRY(dalloc(&P.idx, n));
    return 0;
}

void free_cells(Cells& C)
{
    dfree(C.x); dfree(C.y); dfree(C.z); dfree(C.size); dfree(C.w); dfree(C.d1); dfree(C.d2);
    dfree(C.n); dfree(C.start); dfree(C.left); dfree(C.right); dfree(C.parent);
}

int alloc_cells(Cells& C, int64_t m)
{
    TC_TRY(dalloc(&C.x, m)); TC_TRY(dalloc(&C.y, m)); TC_TRY(dalloc(&C.z, m));
    TC_TRY(dalloc(&C.size, m)); TC_TRY(dalloc(&C.w, m)); TC_TRY(dalloc(&C.d1, m));
    TC_TRY(dalloc(&C.d2, m)); TC_TRY(dalloc(&C.n, m)); TC_TRY(dalloc(&C.start, m));
    TC_TRY(dalloc(&C.left, m)); TC_TRY(dalloc(&C.right, m)); TC_TRY(dalloc(&C.parent, m));
    return 0;
}

void free_scratch(BuildScratch& S)
{
    dfree(S.tasks); dfree(S.chunk0); dfree(S.chunks); dfree(S.part1); dfree(S.part2);
    dfree(S.stats); dfree(S.big_next); dfree(S.small); dfree(S.counters); dfree(S.wstack);
    S.cap_tasks = S.cap_chunks = 0;
}

void field_release(tc_field* f)
{
    free_points(f->buf[0]); free_points(f->buf[1]); free_cells(f->cells);
    dfree(f->tcells); dfree(f->d_tops_raw); dfree(f->d_ntop); dfree(f->d_tops);
    free_scratch(f->S); dfree(f->d_err); dfree(f->leafsums); dfree(f->leafsums_f);
}

int check_dev_err(int* d_err, cudaStream_t st)
{
    int e = 0;
    TC_CU(cudaMemcpyAsync(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    TC_CU(cudaStreamSynchronize(st));
    if (e) {
        set_last_error(std::string("device error: ") + dev_err_msg(e));
        TC_CU(cudaMemsetAsync(d_err, 0, sizeof(int), st));
        return TC_ERR_DEVICE;
    }
    return 0;
}

// BaseField::BuildCells (src/Field.cpp:206-277) on the device.
int field_build(tc_field* f)
{
    if (f->built) return 0;
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    const int64_t n = f->n;
    if (n == 0) { f->built = true; return 0; }
    const int64_t ncap = 2 * n - 1;
    TC_TRY(alloc_cells(f->cells, ncap));
    TC_TRY(dalloc(&f->tcells, ncap));
    TC_TRY(dalloc(&f->d_tops_raw, 2 * n));
    TC_TRY(dalloc(&f->d_ntop, 1));
    TC_TRY(dalloc(&f->S.small, n));
    TC_TRY(dalloc(&f->S.wstack, n));
    TC_TRY(dalloc(&f->S.counters, 2));
    TC_TRY(alloc_points(f->buf[1], n));
    // Unused ids (inside list leaves) keep harmless contents: no children, no points.
    TC_CU(cudaMemsetAsync(f->cells.left, 0xff, ncap * sizeof(int), st));
    TC_CU(cudaMemsetAsync(f->cells.right, 0xff, ncap * sizeof(int), st));
    TC_CU(cudaMemsetAsync(f->cells.parent, 0xff, ncap * sizeof(int), st));
    TC_CU(cudaMemsetAsync(f->cells.n, 0, ncap * sizeof(int), st));
    TC_CU(cudaMemsetAsync(f->cells.w, 0, ncap * sizeof(float), st));
    TC_CU(cudaMemsetAsync(f->cells.size, 0, ncap * sizeof(float), st));
    cudaEvent_t e0, e1;
    TC_CU(cudaEventCreate(&e0));
    TC_CU(cudaEventCreate(&e1));
    TC_CU(cudaEventRecord(e0, st));
    BuildParams BP;
    BP.coords = f->coords; BP.dkind = kind_of(f->dkind); BP.spin = spin_of(f->dkind);
    BP.split = f->split; BP.brute = f->brute;
    BP.minsizesq = f->minsize * f->minsize;
    BP.maxsizesq = f->maxsize * f->maxsize;
    BP.n = (int)n;
    TC_TRY(build_tree(BP, f->buf, f->cells, f->d_tops_raw, f->d_ntop, f->S, st, f->tops, f->d_err,
                      f->mintop, f->maxtop));
    launch_pack_cells((int)ncap, f->cells, f->tcells, st);
    TC_CU(cudaGetLastError());
    TC_TRY(dalloc(&f->d_tops, f->tops.size()));
    TC_CU(cudaMemcpyAsync(f->d_tops, f->tops.data(), f->tops.size() * sizeof(int),
                          cudaMemcpyHostToDevice, st));
    launch_validate_tree((int)ncap, f->cells, f->d_tops, (int)f->tops.size(), f->d_err, st);
    TC_CU(cudaGetLastError());
    TC_CU(cudaEventRecord(e1, st));
    TC_CU(cudaEventSynchronize(e1));
    TC_CU(cudaEventElapsedTime(&f->build_ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    TC_TRY(check_dev_err(f->d_err, st));
    // The second point buffer and the build scratch are no longer needed.
    free_points(f->buf[1]);
    free_scratch(f->S);
    f->built = true;
    return 0;
}

int field_create_impl(int dkind, int coords, const double* x, const double* y, const double* z,
                      const double* d1, const double* d2, const double* w, const double* wpos,
                      int64_t n, double min_size, double max_size, int split_method, int brute,
                      int min_top, int max_top, bool on_device, tc_field** out)
{
    if (!out) { set_last_error("out is NULL"); return TC_ERR_ARG; }
    *out = nullptr;
    if (n < 0 || n > (int64_t)std::numeric_limits<int>::max() / 2) {
        set_last_error("n out of range for the GPU path (0 <= n < 2^30)");
        return TC_ERR_ARG;
    }
    if (dkind < TC_NDATA || dkind > TC_QDATA) { set_last_error("bad data kind"); return TC_ERR_ARG; }
    if (coords != TC_FLAT && coords != TC_THREED && coords != TC_SPHERE) {
        set_last_error("bad coords"); return TC_ERR_ARG;
    }
    if (split_method == TC_RANDOM) {
        set_last_error("split_method='random' is not on the GPU path");
        return TC_ERR_UNSUPPORTED;
    }
    if (split_method < TC_MIDDLE || split_method > TC_RANDOM) {
        set_last_error("bad split_method"); return TC_ERR_ARG;
    }
    if (n > 0 && (!x || !y || !w || (coords != TC_FLAT && !z) || (dkind >= TC_KDATA && !d1) ||
                  (kind_of(dkind) == DG && !d2))) {
        set_last_error("missing input array"); return TC_ERR_ARG;
    }
    tc_field* f = new tc_field();
    f->dkind = dkind; f->coords = coords; f->split = split_method; f->brute = brute ? 1 : 0;
    f->mintop = min_top; f->maxtop = max_top; f->n = n;
    f->minsize = min_size; f->maxsize = max_size;
    cudaStream_t st;
    int rc = stream_get(&st);
    if (rc) { delete f; return rc; }
    auto fail = [&](int code) { field_release(f); delete f; return code; };
    if ((rc = dalloc(&f->d_err, 1))) return fail(rc);
    if (cudaMemsetAsync(f->d_err, 0, sizeof(int), st) != cudaSuccess) {
        set_last_error("cudaMemsetAsync failed"); return fail(TC_ERR_CUDA);
    }
    if (n > 0) {
        if ((rc = alloc_points(f->buf[0], n))) return fail(rc);
        const double* src[7] = {x, y, (coords != TC_FLAT) ? z : nullptr, d1, d2, w, wpos};
        const double* dsrc[7] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
        double* staging = nullptr;
        if (!on_device) {
            // Page-locked host arrays (cudaHostAlloc / cudaHostRegister) are read by the
            // preparation kernel in place, over the host link; the others are copied to a
            // device staging buffer first.  Either way the catalog is copied before this call
            // returns (field_center below waits for the stream), as the reference copies it.
            bool pinned[7] = {false, false, false, false, false, false, false};
            int cnt = 0;
            for (int k = 0; k < 7; ++k) {
                if (!src[k]) continue;
                cudaPointerAttributes at;
                if (cudaPointerGetAttributes(&at, src[k]) == cudaSuccess &&
                    at.type == cudaMemoryTypeHost && at.devicePointer != nullptr) {
                    pinned[k] = true;
                    dsrc[k] = static_cast<const double*>(at.devicePointer);
                } else {
                    cudaGetLastError();
                    ++cnt;
                }
            }
            if (cnt > 0 && (rc = dalloc(&staging, (size_t)cnt * n))) return fail(rc);
            int slot = 0;
            for (int k = 0; k < 7; ++k) {
                if (!src[k] || pinned[k]) continue;
                double* dst = staging + (size_t)slot * n;
                if (cudaMemcpyAsync(dst, src[k], n * sizeof(double), cudaMemcpyHostToDevice, st) !=
                    cudaSuccess) {
                    dfree(staging);
                    set_last_error("host to device copy failed");
                    return fail(TC_ERR_CUDA);
                }
                dsrc[k] = dst;
                ++slot;
            }
        } else {
            for (int k = 0; k < 7; ++k) dsrc[k] = src[k];
        }
        launch_prepare((int)n, coords, kind_of(dkind), dsrc[0], dsrc[1], dsrc[2], dsrc[3], dsrc[4],
                       dsrc[5], dsrc[6], f->buf[0], st);
        BuildParams BP;
        BP.coords = coords; BP.dkind = kind_of(dkind); BP.spin = spin_of(dkind);
        BP.split = split_method; BP.brute = f->brute;
        BP.minsizesq = 0.; BP.maxsizesq = 0.; BP.n = (int)n;
        rc = field_center(BP, f->buf[0], f->S, st, f->center);
        cudaStreamSynchronize(st);   // the caller's arrays are no longer read after this
        dfree(staging);
        if (rc) return fail(rc);
        if (cudaGetLastError() != cudaSuccess) {
            set_last_error("field preparation kernel failed");
            return fail(TC_ERR_CUDA);
        }
    }
    *out = f;
    return TC_OK;
}

double sqr(double x) { return x * x; }

// Accumulators of the level-by-level expansion (per-warp FP64 bins, totals, control words).
int expand_scratch(tc_corr2* c, int nwarps, int nq)
{
    if (nwarps > c->nwarps_alloc || nq > c->nq_alloc || !c->ctl) {
        dfree(c->wacc); dfree(c->wnp); dfree(c->tot); dfree(c->totnp); dfree(c->ctl);
        dfree(c->d_err);
        TC_TRY(dalloc(&c->wacc, (size_t)nwarps * nq * c->nbins));
        TC_TRY(dalloc(&c->wnp, (size_t)nwarps * c->nbins));
        TC_TRY(dalloc(&c->tot, (size_t)nq * c->nbins));
        TC_TRY(dalloc(&c->totnp, (size_t)c->nbins));
        TC_TRY(dalloc(&c->ctl, 8));
        TC_TRY(dalloc(&c->d_err, 1));
        c->nwarps_alloc = nwarps;
        c->nq_alloc = nq;
    }
    return 0;
}

// The expansion's level buffers (up to 1 GB each, ~31 of them at 10M points) come from the
// device's stream-ordered memory pool, which keeps freed memory for the next corr instead of
// returning it to the driver: a new corr per step then costs no cudaMalloc / cudaFree of
// tens of GB (freeing them through the driver took 25 ms per 10M-point correlation).
int pool_alloc_int2(int2** p, size_t count, cudaStream_t st)
{
    static bool configured[64] = {false};
    int dev = 0;
    TC_CU(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && !configured[dev]) {
        cudaMemPool_t pool;
        TC_CU(cudaDeviceGetDefaultMemPool(&pool, dev));
        unsigned long long thr = ~0ULL;   // keep freed blocks in the pool
        TC_CU(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
        configured[dev] = true;
    }
    *p = nullptr;
    const cudaError_t e = cudaMallocAsync((void**)p, std::max<size_t>(count, 1) * sizeof(int2), st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        set_last_error(std::string("cudaMallocAsync of ") + std::to_string(count * sizeof(int2)) +
                       " bytes failed: " + cudaGetErrorString(e));
        return TC_ERR_NOMEM;
    }
    return 0;
}

void pool_free(int2*& p, cudaStream_t st)
{
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
}

// Makes level L's item buffer hold at least `need` items, keeping its first `keep` items.
int level_reserve(tc_corr2* c, int L, long long keep, long long need, cudaStream_t st)
{
    while ((int)c->lev.size() <= L) { c->lev.push_back(nullptr); c->levcap.push_back(0); }
    if (c->levcap[L] >= need) return 0;
    long long cap = std::max(need, 2 * c->levcap[L]);
    int2* p = nullptr;
    TC_TRY(pool_alloc_int2(&p, (size_t)cap, st));
    if (keep > 0)
        TC_CU(cudaMemcpyAsync(p, c->lev[L], sizeof(int2) * (size_t)keep, cudaMemcpyDeviceToDevice, st));
    TC_CU(cudaStreamSynchronize(st));
    pool_free(c->lev[L], st);
    c->lev[L] = p;
    c->levcap[L] = cap;
    return 0;
}



// MetricHelper<M>::DistSq on two host positions (include/Metric.h:143-147, 202-207, 668-682).
double host_dist_sq(int coords, int metric, const double* p1, const double* p2)
{
    double dx = p1[0] - p2[0], dy = p1[1] - p2[1];
    if (coords == TC_FLAT) return dx * dx + dy * dy;
    double dz = p1[2] - p2[2];
    double dsq = dx * dx + dy * dy + dz * dz;
    if (metric == TC_ARC) {
        double th = 2. * std::asin(std::sqrt(dsq) / 2.);
        return th * th;
    }
    return dsq;
}

int check_metric(int coords, int metric)
{
    if (metric == TC_EUCLIDEAN) return 0;
    if (metric == TC_ARC && coords == TC_SPHERE) return 0;
    set_last_error("metric/coords combination is not on the GPU path (Euclidean on any "
                   "coords, Arc on spherical coords)");
    return TC_ERR_UNSUPPORTED;
}

// Number of xi arrays of Corr2<D1,D2> (XiData, include/Corr2.h:225-330): none for NN, one
// for NK/KK, two (real, imaginary) for N or K with a complex kind, four for XX.
int xi_count(int d1, int d2)
{
    if (d1 == TC_NDATA && d2 == TC_NDATA) return 0;
    if (kind_of(d2) != DG) return 1;
    if (kind_of(d1) != DG) return 2;
    return 4;
}

// Adds bin k of the reduced xi sums (quantities 3.. of tot, nb bins each) into the outputs.
void add_xi(tc_corr2* c, const double* tot, int nb, int k)
{
    double* xi[4] = {c->xi0, c->xi1, c->xi2, c->xi3};
    const int nxi = xi_count(c->d1, c->d2);
    for (int q = 0; q < nxi; ++q)
        if (xi[q]) xi[q][k] += tot[(3 + q) * nb + k];
}

// The binning constants of a traversal (BaseCorr2 constructor, src/Corr2.cpp:55-80), in
// FP64 and FP32.
void trav_setup(const tc_corr2* c, TravParams& T, int coords, int metric, int quick, int nq)
{
    std::memset(&T, 0, sizeof(T));
    T.coords = coords; T.metric = metric; T.quick = quick ? 1 : 0;
    T.k1 = kind_of(c->d1); T.k2 = kind_of(c->d2); T.s1 = spin_of(c->d1); T.s2 = spin_of(c->d2);
    T.nbins = c->nbins; T.nqf = nq;
    T.minsep = c->minsep; T.maxsep = c->maxsep; T.binsize = c->binsize; T.b = c->b; T.a = c->a;
    T.logminsep = std::log(c->minsep); T.halfminsep = 0.5 * c->minsep;
    T.minsepsq = c->minsep * c->minsep; T.maxsepsq = c->maxsep * c->maxsep;
    T.bsq = c->b * c->b; T.asq = c->a * c->a;
    T.fminsep = (float)T.minsep; T.fmaxsep = (float)T.maxsep; T.fbinsize = (float)T.binsize;
    T.fb = (float)T.b; T.fminsepsq = (float)T.minsepsq; T.fmaxsepsq = (float)T.maxsepsq;
    T.fbsq = (float)T.bsq; T.fasq = (float)std::min(T.asq, 1e30);
    T.fbb = (float)(0.25 * sqr(T.binsize + T.b));
    T.fmineff = (float)std::min(T.bsq, T.asq);
    T.finvminsepsq = (float)(1. / T.minsepsq);
    T.finvbinsize = (float)(1. / T.binsize);
    T.flogminsep = (float)T.logminsep;
}

// Runs the breadth-first expansion of T to completion (device-side schedule, batches of
// launches, more level buffers on demand).  *derr: the device error word afterwards.
// Items per expansion launch: up to 32M, less for small catalogs (level buffers hold 4
// chunks each: 1 GB per level at the largest size).
long long expand_chunk(long long npoints)
{
    long long CH = 1LL << 16;
    while (CH < (1LL << 25) && CH < 2 * npoints) CH <<= 1;
    return CH;
}

int expand_run(tc_corr2* c, const TravParams& T, int blocks, long long npoints, cudaStream_t st,
               int* derr_out, long long* launches_out)
{
    // The schedule lives on the device: batches of (schedule, expand) launches run without
    // host round trips; the host only adds level buffers when the expansion gets deeper.
    // Chunk size: up to 32M items per launch, less for small catalogs (level buffers hold
    // 4 chunks each: 1 GB per level at the largest size).  Large launches amortise the
    // per-launch work of every warp (bin set-up, the flush of its totals, the fixed-order
    // join, the launch tail): on a 10M-point catalog at bin_slop 0.1, 4M-item chunks took
    // 19% longer than 16M, and 32M took 6% less (2197 launches instead of 4328).
    // The patch batch (mode 3) keeps chunks of at most 16M items: its warps' bins follow the
    // patch pair they work on, and a larger chunk mixes more pairs into one warp's items
    // (2.14 s per 150-patch step at 32M, 1.87 s at 16M).
    long long CH = c->chunk > 0 ? c->chunk : expand_chunk(npoints);
    if (T.mode == 3 && c->chunk == 0 && CH > (1LL << 24)) CH = 1LL << 24;
    if (!c->sched) TC_TRY(dalloc(&c->sched, 1));
    ExpandSched hs;
    std::memset(&hs, 0, sizeof(hs));
    hs.cnt[0] = T.ngen + T.nin;
    hs.cap = 4 * CH;
    hs.chunk_max = CH;
    hs.out_level = -1;
    int nlev = 32;
    for (int l = 1; l < nlev; ++l) {
        TC_TRY(level_reserve(c, l, 0, hs.cap, st));
        hs.lev[l] = c->lev[l];
    }
    hs.nlev = nlev;
    TC_CU(cudaMemcpyAsync(c->sched, &hs, sizeof(hs), cudaMemcpyHostToDevice, st));
    int derr = 0;
    long long launches = 0;
    // Device time of the expansion and tile kernels, from events around every launch.
    constexpr int BATCH = 64;
    if (c->kev.empty()) {
        c->kev.resize(3 * BATCH);
        for (auto& e : c->kev) TC_CU(cudaEventCreate(&e));
    }
    double expand_ms = 0., tiles_ms = 0.;
    for (int batch = 0;; ++batch) {
        TC_TRY(launch_expand_batch(T, blocks, c->sched, BATCH, st, c->kev.data()));
        int flags[3];
        TC_CU(cudaMemcpyAsync(flags, &c->sched->done, 3 * sizeof(int), cudaMemcpyDeviceToHost, st));
        TC_CU(cudaMemcpyAsync(&derr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
        TC_CU(cudaStreamSynchronize(st));
        for (int it = 0; it < BATCH; ++it) {
            float a = 0.f, b = 0.f;
            TC_CU(cudaEventElapsedTime(&a, c->kev[3 * it], c->kev[3 * it + 1]));
            TC_CU(cudaEventElapsedTime(&b, c->kev[3 * it + 1], c->kev[3 * it + 2]));
            expand_ms += a;
            tiles_ms += b;
        }
        if (derr) break;
        if (flags[1]) {   // need_levels: the expansion reached the last allocated level
            if (nlev >= EXP_MAXLEV) {
                set_last_error("the dual-tree expansion is deeper than 512 levels");
                return TC_ERR_DEVICE;
            }
            int nl2 = std::min(EXP_MAXLEV, 2 * nlev);
            for (int l = nlev; l < nl2; ++l) {
                TC_TRY(level_reserve(c, l, 0, hs.cap, st));
                hs.lev[l] = c->lev[l];
            }
            TC_CU(cudaMemcpyAsync(&c->sched->lev[nlev], &hs.lev[nlev],
                                  sizeof(int2*) * (nl2 - nlev), cudaMemcpyHostToDevice, st));
            const int zero = 0;
            TC_CU(cudaMemcpyAsync(&c->sched->nlev, &nl2, sizeof(int), cudaMemcpyHostToDevice, st));
            TC_CU(cudaMemcpyAsync(&c->sched->need_levels, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
            nlev = nl2;
            continue;
        }
        if (flags[0]) break;
        if (batch > 1000000) {
            set_last_error("traversal did not finish within 10^6 batches");
            return TC_ERR_DEVICE;
        }
    }
    TC_CU(cudaMemcpyAsync(&launches, &c->sched->launches, sizeof(long long), cudaMemcpyDeviceToHost, st));
    TC_CU(cudaStreamSynchronize(st));
    *derr_out = derr;
    *launches_out = launches;
    c->stats.expand_ms = expand_ms;
    c->stats.tiles_ms = tiles_ms;
    return TC_OK;
}

// BaseCorr2::process for one or two fields.
int corr_process(tc_corr2* c, tc_field* f1, tc_field* f2, int quick, int metric)
{
    if (!c || !f1) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    if (c->d1 != f1->dkind || (f2 ? c->d2 != f2->dkind : c->d2 != f1->dkind)) {
        set_last_error("field data kind does not match the correlation"); return TC_ERR_ARG;
    }
    if (f2 && f2->coords != f1->coords) {
        set_last_error("fields have different coords"); return TC_ERR_ARG;
    }
    TC_TRY(check_metric(f1->coords, metric));
    c->stats = tc_stats();
    if (f1->n == 0 || (f2 && f2->n == 0)) return TC_OK;
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    if (f2) {
        // Early exit when the fields cannot overlap, src/Corr2.cpp:213-231.
        double rsq = host_dist_sq(f1->coords, metric, f1->center, f2->center);
        double s1ps2 = std::sqrt(f1->center[3]) + std::sqrt(f2->center[3]);
        double minsepsq = c->minsep * c->minsep, maxsepsq = c->maxsep * c->maxsep;
        if ((rsq < minsepsq && s1ps2 < c->minsep && rsq < sqr(c->minsep - s1ps2)) ||
            (rsq >= maxsepsq && rsq >= sqr(c->maxsep + s1ps2)))
            return TC_OK;
    }
    TC_TRY(field_build(f1));
    if (f2) TC_TRY(field_build(f2));
    c->stats.build_ms = f1->build_ms + (f2 ? f2->build_ms : 0.f);

    const int nb = c->nbins;
    const int nq = 3 + xi_count(c->d1, c->d2);
    TravParams T;
    trav_setup(c, T, f1->coords, metric, quick, nq);
    T.autoc = f2 ? 0 : 1;
    tc_field* g = f2 ? f2 : f1;
    T.c1 = f1->tcells; T.c2 = g->tcells;
    T.x1 = f1->cells.x; T.y1 = f1->cells.y; T.z1 = f1->cells.z;
    T.x2 = g->cells.x; T.y2 = g->cells.y; T.z2 = g->cells.z;
    T.tops1 = f1->d_tops; T.tops2 = g->d_tops;
    T.ntop1 = (long long)f1->tops.size(); T.ntop2 = (long long)g->tops.size();
    T.ngen = f2 ? T.ntop1 * T.ntop2 : T.ntop1 * (T.ntop1 + 1) / 2;
    if (c->root_limit > 0 && c->root_limit < T.ngen) T.ngen = c->root_limit;
    if (T.minsep <= 0. || T.binsize <= 0. || nb <= 0) {
        set_last_error("Log binning needs min_sep > 0, bin_size > 0, nbins > 0");
        return TC_ERR_ARG;
    }

    // Breadth-first expansion by levels: each launch takes a chunk of the deepest non-empty
    // level (level 0 = the top-level pairs, generated on the fly) and appends the children to
    // the next level, so memory stays bounded by (depth x 4 chunk) items.
    // The learned criterion's candidates are pairs the rule splits with s <= cand_factor b r:
    // with b = 0 there are none, and the plain traversal (with its tiles) is the same result.
    const int mode = (c->mode == 2 && c->b == 0.) ? 0 : c->mode;
    T.mode = mode;
    T.cand_f2 = (float)(sqr(c->cand_factor * c->b));
    T.mlp_thr = c->mlp_thr;
    T.finvlogrange = (float)(1. / std::log(c->maxsep / c->minsep));
    T.mlp = c->mlp;
    T.samples = c->samples; T.sample_cap = c->sample_cap; T.sample_mod = c->sample_mod;
    int blocks = 0, nwarps = 0;
    TC_TRY(expand_grid(nq, nb, &blocks, &nwarps, mode));
    // Exact mode: every pair the reference accepts is a pair of leaves (angle_slop 0, or two
    // brute fields), so the leaf pairs below small cell pairs go through k_tiles.
    // TCGPU_TILES=0 turns the tiles off (the traversal then walks down to the leaves).
    bool tiles = mode == 0 && (c->a == 0. || (f1->brute && g->brute));
    if (const char* ev = std::getenv("TCGPU_TILES")) tiles = tiles && std::atoi(ev) != 0;
    int tblocks = 0, twarps = 0;
    if (tiles) {
        T.tile_leaf = c->tile_leaf > 0 ? c->tile_leaf : TILE_LEAF;   // (tiles_grid picks the
                                                                     // kernel from T's classes)
        TC_TRY(tiles_grid(T, &tblocks, &twarps));
        const long long cap = c->chunk > 0 ? c->chunk : expand_chunk(f1->n + (f2 ? f2->n : 0));
        if (c->tile_cap < cap) {
            dfree(c->tiles);
            c->tiles = nullptr;
            c->tile_cap = 0;
            TC_TRY(dalloc(&c->tiles, (size_t)cap));
            c->tile_cap = cap;
        }
        if (!c->tctl) TC_TRY(dalloc(&c->tctl, 8));
        if (!c->tedge) TC_TRY(dalloc(&c->tedge, 2 * (size_t)(nb + 1)));
        std::vector<float> te(2 * (size_t)(nb + 1));
        for (int k = 0; k <= nb; ++k) {
            const double le = std::log(c->minsep) + k * c->binsize;   // log of edge k
            te[k] = (float)std::exp(-2. * le);
            te[nb + 1 + k] = (float)le;
        }
        TC_CU(cudaMemcpyAsync(c->tedge, te.data(), te.size() * sizeof(float),
                              cudaMemcpyHostToDevice, st));
        TC_CU(cudaMemsetAsync(c->tctl, 0, 8 * sizeof(unsigned long long), st));
        T.tile_leaf = c->tile_leaf > 0 ? c->tile_leaf : TILE_LEAF;
        T.leaf_base1 = (int)(f1->n - 1);
        T.leaf_base2 = (int)(g->n - 1);
        T.tiles = c->tiles;
        T.tctl = c->tctl;
        T.tile_cap = c->tile_cap;
        T.tile_blocks = tblocks;
        T.tile_wbase = nwarps;
        T.tile_edge = c->tedge;
        T.tile_ledge = c->tedge + nb + 1;
    }
    if (g_deterministic.load() && (mode == 0 || mode == 2)) {
        // Fixed-order expansion: every warp's children and tiles go to regions of its own,
        // joined in warp order after each launch (k_compact).
        const long long CH = c->chunk > 0 ? c->chunk : expand_chunk(f1->n + (f2 ? f2->n : 0));
        const long long ipw = det_items_per_warp(CH, nwarps);
        const long long need_out = 4 * ipw * nwarps, need_t = tiles ? ipw * nwarps : 0;
        if (c->det_out_cap < need_out) {
            dfree(c->det_out); c->det_out = nullptr; c->det_out_cap = 0;
            TC_TRY(dalloc(&c->det_out, (size_t)need_out));
            c->det_out_cap = need_out;
        }
        if (c->det_tout_cap < need_t) {
            dfree(c->det_tout); c->det_tout = nullptr; c->det_tout_cap = 0;
            TC_TRY(dalloc(&c->det_tout, (size_t)need_t));
            c->det_tout_cap = need_t;
        }
        if (c->det_cnt_cap < 2 * nwarps) {
            dfree(c->det_cnt); c->det_cnt = nullptr; c->det_cnt_cap = 0;
            TC_TRY(dalloc(&c->det_cnt, (size_t)2 * nwarps));
            c->det_cnt_cap = 2 * nwarps;
        }
        T.det = 1;
        T.det_nw = nwarps;
        T.det_out = c->det_out;
        T.det_tout = c->det_tout;
        T.det_cnt = c->det_cnt;
        T.det_ccap = 4 * ipw;
        T.det_tcap = ipw;
    }
    TC_TRY(expand_scratch(c, nwarps + twarps, nq));
    T.nsamples = c->ctl + 6;   // ctl exists from here on
    if ((c->mode == 1 && (!c->samples || c->sample_cap <= 0)) || (c->mode == 2 && !c->mlp)) {
        set_last_error("learned-criterion buffers missing");
        return TC_ERR_ARG;
    }
    T.nwarps = nwarps;
    T.wacc = c->wacc; T.wnp = c->wnp; T.err = c->d_err;
    T.counters = c->ctl + 2;
    T.in_tasks = nullptr; T.nin = 0;
    if (!c->wctr || c->wctr_cap < nwarps + twarps) {
        dfree(c->wctr);
        c->wctr_cap = 0;
        TC_TRY(dalloc(&c->wctr, (size_t)(nwarps + twarps) * 8));
        c->wctr_cap = nwarps + twarps;
    }
    T.wctr = c->wctr;
    TC_CU(cudaMemsetAsync(c->wctr, 0, sizeof(unsigned long long) * 8 * (size_t)(nwarps + twarps), st));
    TC_CU(cudaMemsetAsync(c->wacc, 0, sizeof(double) * (size_t)(nwarps + twarps) * nq * nb, st));
    TC_CU(cudaMemsetAsync(c->wnp, 0, sizeof(unsigned long long) * (size_t)(nwarps + twarps) * nb, st));
    TC_CU(cudaMemsetAsync(c->ctl, 0, 8 * sizeof(unsigned long long), st));
    TC_CU(cudaMemsetAsync(c->d_err, 0, sizeof(int), st));
    cudaEvent_t e0, e1;
    TC_CU(cudaEventCreate(&e0));
    TC_CU(cudaEventCreate(&e1));
    TC_CU(cudaEventRecord(e0, st));
    int derr = 0;
    long long launches = 0;
    {
        const int rc = expand_run(c, T, blocks, f1->n + (f2 ? f2->n : 0), st, &derr, &launches);
        if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
    }
    const long long launches_done = launches;
    if (derr) {
        set_last_error(std::string("device error: ") + dev_err_msg(derr));
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        return TC_ERR_DEVICE;
    }
    TC_TRY(launch_reduce(nwarps + twarps, nq, nb, c->wacc, c->wnp, c->tot, c->totnp, st));
    TC_CU(cudaEventRecord(e1, st));
    std::vector<double> tot((size_t)nq * nb);
    std::vector<unsigned long long> totnp(nb);
    // The per-warp counter slots, summed in warp order.
    std::vector<unsigned long long> wc((size_t)(nwarps + twarps) * 8);
    TC_CU(cudaMemcpyAsync(wc.data(), c->wctr, wc.size() * sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, st));
    TC_CU(cudaMemcpyAsync(tot.data(), c->tot, tot.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    TC_CU(cudaMemcpyAsync(totnp.data(), c->totnp, nb * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    TC_CU(cudaStreamSynchronize(st));
    unsigned long long cntr[4] = {0, 0, 0, 0}, tcnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (size_t w = 0; w < (size_t)(nwarps + twarps); ++w) {
        for (int q = 0; q < 4; ++q) cntr[q] += wc[w * 8 + q];
        for (int q = 4; q < 7; ++q) tcnt[q - 2] += wc[w * 8 + q];   // tiles, pairs, FP64
    }
    float ms = 0.f;
    TC_CU(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    c->stats.cell_pairs = (int64_t)cntr[0];
    c->stats.accepted = (int64_t)cntr[1];
    c->stats.escalated = (int64_t)cntr[2];
    c->stats.learned = (int64_t)cntr[3];
    c->stats.launches = launches_done;
    c->stats.traverse_ms = ms;
    c->stats.tiles = tiles ? (int64_t)tcnt[2] : 0;
    c->stats.tile_pairs = (int64_t)tcnt[3];
    c->stats.tile_escalated = (int64_t)tcnt[4];
    // Corr2::finishProcess adds into the caller's arrays (src/Corr2.cpp:527-566).
    for (int k = 0; k < nb && !c->no_output; ++k) {
        c->weight[k] += tot[k];
        if (!quick) {
            c->meanr[k] += tot[nb + k];
            c->meanlogr[k] += tot[2 * nb + k];
            c->npairs[k] += (double)totnp[k];
        }
        add_xi(c, tot.data(), nb, k);
    }
    return TC_OK;
}

// The auto-correlation of an already built field with the fixed traversal scratch: no
// device or host allocation.  It runs the per-warp depth-first traversal kernel (k_traverse,
// which no other path launches) with the same decision and accumulation code as k_expand,
// the warp count capped at NOALLOC_MAXW and the bins at NOALLOC_MAXNB.  Only the exact
// bin_slop criterion runs here: a corr set up for the learned criterion or for sampling its
// training pairs is refused.
int corr_process_auto_noalloc(tc_corr2* c, tc_field* f, int quick, int metric)
{
    if (!c || !f) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    if (c->d1 != f->dkind || c->d2 != f->dkind) {
        set_last_error("field data kind does not match the correlation"); return TC_ERR_ARG;
    }
    if (c->mode != 0) {
        set_last_error("the allocation-free call runs the bin_slop criterion only; this corr "
                       "has the learned criterion or pair sampling set (use "
                       "tc_corr2_process_auto)");
        return TC_ERR_ARG;
    }
    TC_TRY(check_metric(f->coords, metric));
    if (c->nbins > NOALLOC_MAXNB) {
        set_last_error("nbins exceeds the fixed scratch of the allocation-free call (at most 64)");
        return TC_ERR_ARG;
    }
    if (f->n > 0 && !f->built) {
        set_last_error("the field's tree is not built; call tc_field_ntop() first (building "
                       "allocates device memory)");
        return TC_ERR_ARG;
    }
    c->stats = tc_stats();
    if (f->n == 0) return TC_OK;
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    void* base = nullptr;
    TC_TRY(noalloc_scratch(&base));
    unsigned char* B = static_cast<unsigned char*>(base);

    const int nb = c->nbins;
    const int nq = 3 + xi_count(c->d1, c->d2);
    TravParams T;
    trav_setup(c, T, f->coords, metric, quick, nq);
    T.autoc = 1;
    T.c1 = f->tcells; T.c2 = f->tcells;
    T.x1 = f->cells.x; T.y1 = f->cells.y; T.z1 = f->cells.z;
    T.x2 = f->cells.x; T.y2 = f->cells.y; T.z2 = f->cells.z;
    T.tops1 = f->d_tops; T.tops2 = f->d_tops;
    T.ntop1 = (long long)f->tops.size(); T.ntop2 = T.ntop1;
    T.ngen = T.ntop1 * (T.ntop1 + 1) / 2;

    int blocks = 0, nwarps = 0;
    TC_TRY(traverse_grid(nq, nb, &blocks, &nwarps));
    const int wpb = nwarps / blocks;
    if (nwarps > NOALLOC_MAXW) { blocks = NOALLOC_MAXW / wpb; nwarps = blocks * wpb; }
    int2* spill[2] = {reinterpret_cast<int2*>(B + NOALLOC_OFF_SPILL0),
                      reinterpret_cast<int2*>(B + NOALLOC_OFF_SPILL1)};
    double* wacc = reinterpret_cast<double*>(B + NOALLOC_OFF_WACC);
    unsigned long long* wnp = reinterpret_cast<unsigned long long*>(B + NOALLOC_OFF_WNP);
    double* tot = reinterpret_cast<double*>(B + NOALLOC_OFF_TOT);
    unsigned long long* totnp = reinterpret_cast<unsigned long long*>(B + NOALLOC_OFF_TOTNP);
    unsigned long long* ctl = reinterpret_cast<unsigned long long*>(B + NOALLOC_OFF_CTL);
    T.stacks = reinterpret_cast<int2*>(B + NOALLOC_OFF_STACKS);
    T.stack_cap = NOALLOC_SCAP;
    T.nwarps = nwarps;
    T.wacc = wacc; T.wnp = wnp;
    T.idle = reinterpret_cast<int*>(B + NOALLOC_OFF_IDLE);
    T.err = reinterpret_cast<int*>(B + NOALLOC_OFF_ERR);
    T.root_next = ctl; T.nout = ctl + 1; T.counters = ctl + 2;
    T.out_cap = NOALLOC_SPILL;
    // Test hook: a shorter spill list (TCGPU_NOALLOC_SPILL_CAP items) makes the overflow path
    // reachable on test-size catalogs.
    if (const char* e = std::getenv("TCGPU_NOALLOC_SPILL_CAP")) {
        const long long v = std::atoll(e);
        if (v >= 0 && v < T.out_cap) T.out_cap = v;
    }
    // The array keeps the previous call's contents: clear what must start at zero.
    TC_CU(cudaMemsetAsync(wacc, 0, sizeof(double) * (size_t)nwarps * nq * nb, st));
    TC_CU(cudaMemsetAsync(wnp, 0, sizeof(unsigned long long) * (size_t)nwarps * nb, st));
    TC_CU(cudaMemsetAsync(ctl, 0, 8 * sizeof(unsigned long long), st));
    TC_CU(cudaMemsetAsync(T.err, 0, sizeof(int), st));
    int cur = 0, launches = 0, derr = 0;
    long long nin = 0;
    T.in_tasks = nullptr;
    while (true) {
        T.nin = nin;
        T.out_tasks = spill[cur ^ 1];
        TC_CU(cudaMemsetAsync(ctl, 0, 2 * sizeof(unsigned long long), st));
        TC_CU(cudaMemsetAsync(T.idle, 0, sizeof(int), st));
        TC_TRY(launch_traverse(T, blocks, st));
        ++launches;
        unsigned long long nout = 0;
        TC_CU(cudaMemcpyAsync(&nout, ctl + 1, sizeof(nout), cudaMemcpyDeviceToHost, st));
        TC_CU(cudaMemcpyAsync(&derr, T.err, sizeof(int), cudaMemcpyDeviceToHost, st));
        TC_CU(cudaStreamSynchronize(st));
        if (derr || nout == 0) break;
        if (launches >= 100000) {
            set_last_error("traversal did not finish within 100000 relaunches");
            return TC_ERR_DEVICE;
        }
        T.ngen = 0;
        T.in_tasks = spill[cur ^ 1];
        nin = (long long)nout;
        cur ^= 1;
    }
    if (derr == DEV_SPILL_OVERFLOW || derr == DEV_STACK_OVERFLOW) {
        set_last_error("the traversal needs more work-list space than the fixed scratch of the "
                       "allocation-free call holds; use tc_corr2_process_auto");
        return TC_ERR_DEVICE;
    }
    if (derr) {
        set_last_error(std::string("device error: ") + dev_err_msg(derr));
        return TC_ERR_DEVICE;
    }
    TC_TRY(launch_reduce(nwarps, nq, nb, wacc, wnp, tot, totnp, st));
    double h_tot[NOALLOC_NQ * NOALLOC_MAXNB];
    unsigned long long h_np[NOALLOC_MAXNB];
    unsigned long long cnt[3];
    TC_CU(cudaMemcpyAsync(h_tot, tot, sizeof(double) * (size_t)nq * nb, cudaMemcpyDeviceToHost, st));
    TC_CU(cudaMemcpyAsync(h_np, totnp, sizeof(unsigned long long) * (size_t)nb,
                          cudaMemcpyDeviceToHost, st));
    TC_CU(cudaMemcpyAsync(cnt, ctl + 2, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    TC_CU(cudaStreamSynchronize(st));
    c->stats.cell_pairs = (int64_t)cnt[0];
    c->stats.accepted = (int64_t)cnt[1];
    c->stats.escalated = (int64_t)cnt[2];
    c->stats.launches = launches;
    c->stats.build_ms = f->build_ms;   // the field's earlier build; traverse_ms stays 0
    for (int k = 0; k < nb; ++k) {
        c->weight[k] += h_tot[k];
        if (!quick) {
            c->meanr[k] += h_tot[nb + k];
            c->meanlogr[k] += h_tot[2 * nb + k];
            c->npairs[k] += (double)h_np[k];
        }
        add_xi(c, h_tot, nb, k);
    }
    return TC_OK;
}

// The cells of two fields in one id space: field 2's cells follow field 1's, with their
// child ids shifted, so that the multipole kernels walk vertex 1 in field 1 and the pair
// lists in field 2 without knowing there are two trees.
struct JoinedCells {
    Cells cells = {};
    double* ls = nullptr;
    float4* lsf = nullptr;
    TCell* tc = nullptr;
    int* tops2 = nullptr;
    ~JoinedCells()
    {
        dfree(cells.x); dfree(cells.y); dfree(cells.z); dfree(cells.size); dfree(cells.w);
        dfree(cells.d1); dfree(cells.d2); dfree(cells.n); dfree(cells.left);
        dfree(cells.right); dfree(ls); dfree(lsf); dfree(tc); dfree(tops2);
    }
};

__global__ void k_shift_ids(int* a, long long n, int base)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && a[i] >= 0) a[i] += base;
}

// nf fields (2 or 3) side by side; J.tops2 lists the top cells of fields 1..nf-1 (the pair
// lists' starting cells), with their joined ids.
int join_cells(tc_field* const* fs, int nf, JoinedCells& J, cudaStream_t st)
{
    size_t cnt[3], base[3], n = 0, ntops = 0;
    for (int i = 0; i < nf; ++i) {
        cnt[i] = 2 * (size_t)fs[i]->n - 1;
        base[i] = n;
        n += cnt[i];
        if (i > 0) ntops += fs[i]->tops.size();
    }
    TC_TRY(dalloc(&J.cells.x, n)); TC_TRY(dalloc(&J.cells.y, n)); TC_TRY(dalloc(&J.cells.z, n));
    TC_TRY(dalloc(&J.cells.size, n)); TC_TRY(dalloc(&J.cells.w, n));
    TC_TRY(dalloc(&J.cells.d1, n)); TC_TRY(dalloc(&J.cells.d2, n));
    TC_TRY(dalloc(&J.cells.n, n)); TC_TRY(dalloc(&J.cells.left, n));
    TC_TRY(dalloc(&J.cells.right, n));
    TC_TRY(dalloc(&J.ls, 4 * n)); TC_TRY(dalloc(&J.lsf, n)); TC_TRY(dalloc(&J.tc, n));
    TC_TRY(dalloc(&J.tops2, ntops));
    auto cp = [&](auto* dst, const auto* src, size_t per, int i) -> int {
        TC_CU(cudaMemcpyAsync(dst + per * base[i], src, sizeof(*dst) * per * cnt[i],
                              cudaMemcpyDeviceToDevice, st));
        return 0;
    };
    size_t toff = 0;
    for (int i = 0; i < nf; ++i) {
        const Cells& A = fs[i]->cells;
        TC_TRY(cp(J.cells.x, A.x, 1, i)); TC_TRY(cp(J.cells.y, A.y, 1, i));
        TC_TRY(cp(J.cells.z, A.z, 1, i)); TC_TRY(cp(J.cells.size, A.size, 1, i));
        TC_TRY(cp(J.cells.w, A.w, 1, i)); TC_TRY(cp(J.cells.d1, A.d1, 1, i));
        TC_TRY(cp(J.cells.d2, A.d2, 1, i)); TC_TRY(cp(J.cells.n, A.n, 1, i));
        TC_TRY(cp(J.cells.left, A.left, 1, i)); TC_TRY(cp(J.cells.right, A.right, 1, i));
        TC_TRY(cp(J.ls, fs[i]->leafsums, 4, i)); TC_TRY(cp(J.lsf, fs[i]->leafsums_f, 1, i));
        TC_TRY(cp(J.tc, fs[i]->tcells, 1, i));
        if (i == 0) continue;
        const size_t nt = fs[i]->tops.size();
        TC_CU(cudaMemcpyAsync(J.tops2 + toff, fs[i]->d_tops, sizeof(int) * nt,
                              cudaMemcpyDeviceToDevice, st));
        const unsigned g = (unsigned)((cnt[i] + 255) / 256), gt = (unsigned)((nt + 255) / 256);
        const int bi = (int)base[i];
        count_launch(); k_shift_ids<<<g, 256, 0, st>>>(J.cells.left + base[i], (long long)cnt[i], bi);
        count_launch(); k_shift_ids<<<g, 256, 0, st>>>(J.cells.right + base[i], (long long)cnt[i], bi);
        count_launch(); k_rebase_cells<<<g, 256, 0, st>>>(J.tc + base[i], (long long)cnt[i], bi, 0);
        count_launch(); k_shift_ids<<<gt, 256, 0, st>>>(J.tops2 + toff, (long long)nt, bi);
        toff += nt;
    }
    TC_CU(cudaGetLastError());
    return 0;
}

int ensure_leaf_sums(tc_field* f, cudaStream_t st)
{
    if (f->leafsums) return 0;
    const int64_t ncap = 2 * f->n - 1;
    TC_TRY(dalloc(&f->leafsums, 4 * (size_t)ncap));
    TC_TRY(dalloc(&f->leafsums_f, (size_t)ncap));
    TC_TRY(launch_leaf_sums((int)ncap, f->cells, f->leafsums, f->leafsums_f, st));
    return 0;
}

// TripleTraits<D1,D2,D3>::algo (src/Corr3.cpp:1835-1860) for N, K and G vertices.
int c3_algo(const tc_corr3* c)
{
    const bool r2 = c->dk != TC_GDATA, r3 = c->dk3 != TC_GDATA;
    if (c->dv != TC_GDATA) {
        if (c->dv == TC_NDATA && c->dk == TC_NDATA && c->dk3 == TC_NDATA) return 0;
        return r2 && r3 ? 1 : (!r2 && !r3 ? 2 : 3);
    }
    return r2 && r3 ? 4 : (!r2 && !r3 ? 5 : 6);
}

// Zeta arrays written per algorithm (ZetaData<0..4>, include/Corr3.h:581-720).
int c3_nzeta(int algo)
{
    static const int nz[7] = {0, 2, 4, 2, 2, 8, 4};
    return nz[algo];
}

// BaseCorr3::multipole with LogMultipole binning: the auto-correlation (f2 == f1, f3 null,
// src/Corr3.cpp:1124-1175), cross12 (vertex 1 from f1, vertices 2 and 3 from f2,
// 1177-1237), or the three-field cross (vertex 1 from f1, vertex 2 from f2, vertex 3 from
// f3, with ordered 1 or 4, 1239-1305).
int corr3_run(tc_corr3* c, tc_field* f1, tc_field* f2, tc_field* f3, int ordered, int quick,
              int metric)
{
    if (!c || !f1 || !f2) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    if (f1->dkind != c->dv || f2->dkind != c->dk || (f3 ? f3->dkind != c->dk3 : c->dk3 != c->dk)) {
        static const char L[] = "NKGZVTQ";
        const char cls[4] = {L[c->dv], L[c->dk], L[c->dk3], 0};
        set_last_error(std::string(cls) + ": the fields have the wrong data kind for the vertices" +
                       (f3 || c->dk3 == c->dk ? "" : " (this class needs processCross21 or "
                                                     "processCross)"));
        return TC_ERR_ARG;
    }
    if (f1->coords != f2->coords || (f3 && f3->coords != f1->coords)) {
        set_last_error("the fields have different coordinate systems");
        return TC_ERR_ARG;
    }
    TC_TRY(check_metric(f1->coords, metric));
    if (f1->n == 0 || f2->n == 0 || (f3 && f3->n == 0)) return TC_OK;
    const bool three = f3 != nullptr;
    if (three && 2 * c->nbins > MP_MAXNB) {
        set_last_error("the three-field GPU multipole needs nbins <= 64");
        return TC_ERR_UNSUPPORTED;
    }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    tc_field* fs[3] = {f1, f2, f3};
    const int nf = three ? 3 : 2;
    for (int i = 0; i < nf; ++i) {
        TC_TRY(field_build(fs[i]));
        TC_TRY(ensure_leaf_sums(fs[i], st));
    }
    const bool cross = three || f2 != f1;
    JoinedCells J;
    if (cross) TC_TRY(join_cells(fs, nf, J, st));
    int64_t ncap = 0;
    for (int i = 0; i < (cross ? nf : 1); ++i) ncap += 2 * fs[i]->n - 1;
    const Cells& CC = cross ? J.cells : f1->cells;
    if (ncap >= (int64_t)INT32_MAX) {
        set_last_error("too many cells for 32-bit cell ids");
        return TC_ERR_UNSUPPORTED;
    }
    MPParams P;
    std::memset(&P, 0, sizeof(P));
    P.coords = f1->coords; P.metric = metric; P.quick = quick ? 1 : 0;
    P.nbins = c->nbins; P.maxn = c->maxn;
    P.minsep = c->minsep; P.maxsep = c->maxsep; P.binsize = c->binsize; P.b = c->b; P.a = c->a;
    // BaseCorr3 constructor, src/Corr3.cpp:107-115.
    P.logminsep = std::log(c->minsep);
    P.minsepsq = c->minsep * c->minsep; P.maxsepsq = c->maxsep * c->maxsep;
    P.bsq = c->b * c->b; P.asq = c->a * c->a;
    P.maxbsq_eff = P.maxsepsq * std::min(P.bsq, P.asq);
    P.f_minsepsq = (float)P.minsepsq; P.f_minsep = (float)P.minsep; P.f_maxsepsq = (float)P.maxsepsq; P.f_maxsep = (float)P.maxsep;
    P.f_asq = (float)P.asq; P.f_bsq = (float)P.bsq;
    P.f_q25 = (float)(0.25 * (P.binsize + P.b) * (P.binsize + P.b));
    P.f_logminsep = (float)P.logminsep; P.f_binsize = (float)P.binsize; P.f_b = (float)P.b;
    P.f_minba = (float)std::min(P.bsq, P.asq);
    P.x = CC.x; P.y = CC.y; P.z = CC.z;
    P.size = CC.size; P.w = CC.w; P.d1 = CC.d1; P.d2 = CC.d2;
    P.n = CC.n; P.left = CC.left; P.right = CC.right;
    P.ls = cross ? J.ls : f1->leafsums;
    P.lsf = cross ? J.lsf : f1->leafsums_f;
    P.tc = cross ? J.tc : f1->tcells;
    P.tops = f1->d_tops; P.ntop = (int)f1->tops.size();
    P.tops2 = cross ? J.tops2 : f1->d_tops;
    P.ntop2 = (int)(f2->tops.size() + (three ? f3->tops.size() : 0));
    // Distance bins; a three-field cross keeps vertex 3's pairs in bins [nb, 2 nb) of the
    // scratch and the records.
    const int nb = c->nbins, nbv = three ? 2 * nb : nb;
    P.nbins = nbv;
    P.nbd = nb;
    P.three = three ? 1 : 0;
    P.base3 = three ? (int)((2 * f1->n - 1) + (2 * f2->n - 1)) : 0;
    P.typo32 = three && ordered == 1 ? 1 : 0;
    // Every class runs GGG's contraction (MultipoleHelper<5>) on the right payloads: a real
    // vertex (N: w1, K: w1 k1, getWK) takes G_n at n instead of n -+ 1 and self-pair sums
    // without z^2 (vreal; the scratch has no spin-2 buffer, src/Corr3.cpp:1307-1313); a real
    // pair list (N: w, K: w k) is not rotated (a pspin0 bit).  Then, with the algorithm
    // numbers of TripleTraits (1835-1860):
    //   1 (KKK, NKK, NNK, ...; 2108-2214): gam0 = wk1 K_a[n] K_b[-n] is zeta;
    //   2 (NGG, KGG; 2216-2405): gam0 and gam2 are zeta0 and zeta1;
    //   3 (NNG, KGK, ...; 2408-2458): gam0 is zeta;  4 (GNN, GKK; 2462-2580): gam0 is zeta;
    //   6 (GNG, GGK, ...; 3018-3082): gam0 and gam1 are zeta0 and zeta1.
    // A K field carries its real payload already; an N field's cells get it in the joined
    // copy (a class with an N and another kind always has several fields).
    const bool nnn = c->dv == TC_NDATA && c->dk == TC_NDATA && c->dk3 == TC_NDATA;
    const bool vreal = c->dv != TC_GDATA && !nnn;
    const bool l2r = c->dk != TC_GDATA && !nnn, l3r = c->dk3 != TC_GDATA && !nnn;
    const int algo = c3_algo(c);
    if (cross && (vreal || l2r || l3r)) {
        const size_t n1c = 2 * (size_t)f1->n - 1;
        const size_t n2c = three ? 2 * (size_t)f2->n - 1 : (size_t)ncap - n1c;
        if (vreal) {
            if (c->dv == TC_NDATA)
                TC_CU(cudaMemcpyAsync(J.cells.d1, J.cells.w, sizeof(float) * n1c,
                                      cudaMemcpyDeviceToDevice, st));
            TC_CU(cudaMemsetAsync(J.cells.d2, 0, sizeof(float) * n1c, st));
        }
        struct { bool real; int is_n; size_t lo, len; } lists[2] = {
            {l2r, c->dk == TC_NDATA, n1c, n2c},
            {three && l3r, c->dk3 == TC_NDATA, n1c + n2c, (size_t)ncap - n1c - n2c}};
        for (const auto& L : lists)
            if (L.real && L.len > 0)
                TC_TRY(launch_scalar_pairs((int)L.len, L.is_n ? 1 : 0, J.tc + L.lo,
                                           J.cells.d1 + L.lo, J.cells.d2 + L.lo,
                                           J.ls + 4 * L.lo, J.lsf + L.lo, st));
    }
    P.vreal = vreal ? 1 : 0;
    P.pspin0 = (l2r ? 1 : 0) | (three && l3r ? 2 : 0);
    P.ncells = (int)ncap;
    const int nn = 2 * c->maxn + 1;
    const size_t Z = (size_t)nb * nb * nn, Zv = (size_t)nbv * nbv * nn;
    std::vector<double> h(15 * Zv);
    cudaEvent_t e0, e1;
    TC_CU(cudaEventCreate(&e0));
    TC_CU(cudaEventCreate(&e1));
    TC_CU(cudaEventRecord(e0, st));
    int rc = run_multipole(P, c->X, P.ntop, st, h.data());
    TC_CU(cudaEventRecord(e1, st));
    TC_CU(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    c->ms += ms;   // summed over the multipoles of one process call (reset by the caller)
    if (rc) return rc == 3 ? TC_ERR_UNSUPPORTED : (rc == 5 ? TC_ERR_NOMEM : TC_ERR_DEVICE);
    if (three) {
        // calculateZeta(c1, ordered, mp2, mp3, ...), src/Corr3.cpp:1976-2087: entry (k2, k3)
        // is the vertex-3 x vertex-2 block (mp3 at k2, mp2 at k3); ordered = 1 adds the
        // vertex-2 x vertex-3 block (cats 2 and 3 swapped).
        // The zeta of algorithms 3, 4 and 6 (MultipoleHelper<3>, <4>, <6>) is written for
        // ordered = 4 only: it has no swapped term, while their weights and means do.
        const bool gx = algo == 3 || algo == 4 || algo == 6;
        std::vector<double> hz(15 * Z);
        for (int q = 0; q < 15; ++q)
            for (int k2 = 0; k2 < nb; ++k2)
                for (int k3 = 0; k3 < nb; ++k3)
                    for (int n = 0; n < nn; ++n) {
                        const size_t i32 = ((size_t)(k2 + nb) * nbv + k3) * nn + n;
                        const size_t i23 = ((size_t)k2 * nbv + k3 + nb) * nn + n;
                        double v = h[q * Zv + i32];
                        if (ordered == 1 && !(gx && q < 8)) v += h[q * Zv + i23];
                        hz[q * Z + ((size_t)k2 * nb + k3) * nn + n] = v;
                    }
        h.swap(hz);
    }
    // Corr3 adds into the caller's arrays (calculateZeta, src/Corr3.cpp:1861-1974): GGG all
    // of gam0..3; NGG / KGG gam0 and gam2 as their zeta0 (gam0) and zeta1 (gam1); the real
    // classes gam0 as zeta (real, imaginary); NNN nothing.
    const int zmap[8] = {0, 1, 2, 3, 4, 5, 6, 7}, xgmap[4] = {0, 1, 4, 5};
    const int nz = c3_nzeta(algo);
    for (int q = 0; q < nz; ++q) {
        const int src = algo == 2 ? xgmap[q] : zmap[q];
        if (c->zeta[q]) for (size_t i = 0; i < Z; ++i) c->zeta[q][i] += h[src * Z + i];
    }
    double* dst[7] = {c->meand2, c->meanlogd2, c->meand3, c->meanlogd3, c->weight, c->weight_im,
                      c->ntri};
    for (int q = 0; q < 7; ++q) {
        if (quick && (q < 4 || q == 6)) continue;
        if (dst[q]) for (size_t i = 0; i < Z; ++i) dst[q][i] += h[(8 + q) * Z + i];
    }
    return TC_OK;
}

// Canonical depth-first dump of the tree (host walk over device-copied cells).
int64_t field_dump(tc_field* f, double* xyz, float* swd, int64_t* ns, int32_t* depth, int64_t cap)
{
    int rc = field_build(f);
    if (rc) return -rc;
    if (f->n == 0) return 0;
    const int64_t m = 2 * f->n - 1;
    std::vector<double> X(m), Y(m), Z(m);
    std::vector<float> S(m), W(m), D1(m), D2(m);
    std::vector<int> N(m), ST(m), L(m), R(m);
    auto cp = [&](void* dst, const void* src, size_t bytes) {
        return cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost) == cudaSuccess;
    };
    bool ok = cp(X.data(), f->cells.x, m * 8) && cp(Y.data(), f->cells.y, m * 8) &&
              cp(Z.data(), f->cells.z, m * 8) && cp(S.data(), f->cells.size, m * 4) &&
              cp(W.data(), f->cells.w, m * 4) && cp(D1.data(), f->cells.d1, m * 4) &&
              cp(D2.data(), f->cells.d2, m * 4) && cp(N.data(), f->cells.n, m * 4) &&
              cp(ST.data(), f->cells.start, m * 4) && cp(L.data(), f->cells.left, m * 4) &&
              cp(R.data(), f->cells.right, m * 4);
    if (!ok) { set_last_error("device to host copy failed"); return -TC_ERR_CUDA; }
    int64_t cnt = 0;
    std::vector<std::pair<int, int>> stack;
    for (int t = (int)f->tops.size() - 1; t >= 0; --t) stack.push_back({f->tops[t], 0});
    while (!stack.empty()) {
        auto [id, d] = stack.back();
        stack.pop_back();
        if (cnt < cap) {
            xyz[3 * cnt] = X[id]; xyz[3 * cnt + 1] = Y[id]; xyz[3 * cnt + 2] = Z[id];
            swd[4 * cnt] = S[id]; swd[4 * cnt + 1] = W[id];
            swd[4 * cnt + 2] = D1[id]; swd[4 * cnt + 3] = D2[id];
            ns[2 * cnt] = N[id]; ns[2 * cnt + 1] = ST[id];
            depth[cnt] = d;
        }
        ++cnt;
        if (L[id] >= 0) {
            stack.push_back({R[id], d + 1});
            stack.push_back({L[id], d + 1});
        }
    }
    return cnt;
}

}  // namespace

extern "C" {

int tc_field_create(int dkind, int coords, const double* x, const double* y, const double* z,
                    const double* d1, const double* d2, const double* w, const double* wpos,
                    int64_t n, double min_size, double max_size, int split_method, int64_t seed,
                    int brute, int min_top, int max_top, tc_field** out)
{
    km_seed(seed);   // BaseField seeds the random stream (src/Field.cpp:160)
    return field_create_impl(dkind, coords, x, y, z, d1, d2, w, wpos, n, min_size, max_size,
                             split_method, brute, min_top, max_top, false, out);
}

int tc_field_create_device(int dkind, int coords, const double* x, const double* y,
                           const double* z, const double* d1, const double* d2, const double* w,
                           const double* wpos, int64_t n, double min_size, double max_size,
                           int split_method, int64_t seed, int brute, int min_top, int max_top,
                           tc_field** out)
{
    km_seed(seed);
    return field_create_impl(dkind, coords, x, y, z, d1, d2, w, wpos, n, min_size, max_size,
                             split_method, brute, min_top, max_top, true, out);
}

void tc_field_free(tc_field* f)
{
    if (!f) return;
    field_release(f);
    delete f;
}

int64_t tc_field_nobj(const tc_field* f) { return f ? f->n : 0; }

double tc_field_size(const tc_field* f) { return f ? std::sqrt(f->center[3]) : 0.; }

int64_t tc_field_ntop(tc_field* f)
{
    if (!f) { set_last_error("NULL field"); return -TC_ERR_ARG; }
    int rc = field_build(f);
    if (rc) return -rc;
    return (int64_t)f->tops.size();
}

int tc_field_center(const tc_field* f, double* xyz3)
{
    if (!f || !xyz3) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    xyz3[0] = f->center[0]; xyz3[1] = f->center[1]; xyz3[2] = f->center[2];
    return TC_OK;
}

int64_t tc_field_dump(tc_field* f, double* xyz, float* size_w_d, int64_t* n_start,
                      int32_t* depth, int64_t cap)
{
    if (!f) { set_last_error("NULL field"); return -TC_ERR_ARG; }
    return field_dump(f, xyz, size_w_d, n_start, depth, cap);
}

}  // extern "C"

namespace {

// The built field as the k-means code sees it.
int km_view(tc_field* f, KMField& F)
{
    if (!f) { set_last_error("NULL field"); return TC_ERR_ARG; }
    TC_TRY(field_build(f));
    F.coords = f->coords;
    F.n = f->n;
    F.ncap = f->n > 0 ? (int)(2 * f->n - 1) : 0;
    F.cells = f->cells;
    F.d_tops = f->d_tops;
    F.ntop = (int)f->tops.size();
    F.idx = f->buf[0].idx;
    F.size = std::sqrt(f->center[3]);
    return 0;
}

}  // namespace

extern "C" {

int tc_kmeans_init_tree(tc_field* f, double* centers, int npatch, int64_t seed)
{
    KMField F;
    TC_TRY(km_view(f, F));
    if (!centers) { set_last_error("centers is NULL"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    return kmeans_init_tree(F, centers, npatch, (long long)seed, st);
}

int tc_kmeans_init_rand(tc_field* f, double* centers, int npatch, int64_t seed)
{
    KMField F;
    TC_TRY(km_view(f, F));
    if (!centers) { set_last_error("centers is NULL"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    return kmeans_init_rand(F, centers, npatch, (long long)seed, st);
}

int tc_kmeans_init_kmpp(tc_field* f, double* centers, int npatch, int64_t seed)
{
    KMField F;
    TC_TRY(km_view(f, F));
    if (!centers) { set_last_error("centers is NULL"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    return kmeans_init_kmpp(F, centers, npatch, (long long)seed, st);
}

int tc_kmeans_run(tc_field* f, double* centers, int npatch, int max_iter, double tol, int alt)
{
    KMField F;
    TC_TRY(km_view(f, F));
    if (!centers) { set_last_error("centers is NULL"); return TC_ERR_ARG; }
    if (max_iter < 0) { set_last_error("max_iter must be >= 0"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    int iters = 0;
    const int rc = kmeans_run(F, centers, npatch, max_iter, tol, alt != 0, st, &iters);
    f->km_iters = iters;
    return rc;
}

int tc_kmeans_assign(tc_field* f, const double* centers, int npatch, int64_t* patches, int64_t n)
{
    KMField F;
    TC_TRY(km_view(f, F));
    if (!centers || !patches) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    if (n != f->n) { set_last_error("patches must have one entry per point of the field"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    return kmeans_assign(F, centers, npatch, patches, st);
}

int tc_kmeans_iterations(const tc_field* f) { return f ? f->km_iters : 0; }

int tc_quick_assign(const double* centers, int npatch, const double* x, const double* y,
                    const double* z, int64_t n, int64_t* patches)
{
    if (!centers || (n > 0 && (!x || !y || !patches))) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    return quick_assign(centers, npatch, x, y, z, n, patches, false, st);
}

int tc_select_patch(int patch, const double* centers, int npatch, const double* x,
                    const double* y, const double* z, int64_t n, int64_t* use)
{
    if (!centers || (n > 0 && (!x || !y || !use))) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    return select_patch(patch, centers, npatch, x, y, z, n, use, false, st);
}

int tc_quick_assign_device(const double* centers, int npatch, const double* x, const double* y,
                           const double* z, int64_t n, int64_t* patches)
{
    if (!centers || (n > 0 && (!x || !y || !patches))) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    return quick_assign(centers, npatch, x, y, z, n, patches, true, st);
}

int tc_select_patch_device(int patch, const double* centers, int npatch, const double* x,
                           const double* y, const double* z, int64_t n, int64_t* use)
{
    if (!centers || (n > 0 && (!x || !y || !use))) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    return select_patch(patch, centers, npatch, x, y, z, n, use, true, st);
}

int tc_corr2_create(int d1, int d2, int bin_type, double minsep, double maxsep, int nbins,
                    double binsize, double b, double a, double minrpar, double maxrpar,
                    double xp, double yp, double zp, double* xi0, double* xi1, double* xi2,
                    double* xi3, double* meanr, double* meanlogr, double* weight,
                    double* npairs, tc_corr2** out)
{
    if (!out) { set_last_error("out is NULL"); return TC_ERR_ARG; }
    *out = nullptr;
    if (bin_type != TC_LOG) {
        set_last_error("only Log binning is on the GPU path");
        return TC_ERR_UNSUPPORTED;
    }
    const double big = std::numeric_limits<double>::max();
    if (!(minrpar <= -big) || !(maxrpar >= big) || xp != 0. || yp != 0. || zp != 0.) {
        set_last_error("min_rpar/max_rpar/period are not on the GPU path");
        return TC_ERR_UNSUPPORTED;
    }
    if (nbins <= 0 || !(minsep > 0.) || !(maxsep > minsep) || !(binsize > 0.) || b < 0. || a < 0.) {
        set_last_error("invalid binning");
        return TC_ERR_ARG;
    }
    // The classes of src/Corr2.cpp:1204-1232: NN, NK, KK and, for every complex kind X,
    // NX, KX and XX.
    if (d1 < TC_NDATA || d1 > TC_QDATA || d2 < TC_NDATA || d2 > TC_QDATA ||
        !(d1 == d2 || (d1 <= TC_KDATA && d2 > d1))) {
        set_last_error("no correlation class for these data kinds");
        return TC_ERR_ARG;
    }
    const int nxi = xi_count(d1, d2);
    if (!meanr || !meanlogr || !weight || !npairs || (nxi >= 1 && !xi0) ||
        (nxi >= 2 && !xi1) || (nxi >= 4 && (!xi2 || !xi3))) {
        set_last_error("missing output array");
        return TC_ERR_ARG;
    }
    tc_corr2* c = new tc_corr2();
    c->d1 = d1; c->d2 = d2; c->bin_type = bin_type; c->nbins = nbins;
    c->minsep = minsep; c->maxsep = maxsep; c->binsize = binsize; c->b = b; c->a = a;
    c->xi0 = xi0; c->xi1 = xi1; c->xi2 = xi2; c->xi3 = xi3;
    c->meanr = meanr; c->meanlogr = meanlogr; c->weight = weight; c->npairs = npairs;
    *out = c;
    return TC_OK;
}

void tc_corr2_free(tc_corr2* c)
{
    if (!c) return;
    dfree(c->wacc); dfree(c->wnp);
    dfree(c->tot); dfree(c->totnp); dfree(c->ctl); dfree(c->idle); dfree(c->d_err);
    {
        cudaStream_t st = nullptr;
        if (stream_get(&st) == 0)
            for (auto& p : c->lev) pool_free(p, st);
    }
    dfree(c->sched);
    dfree(c->mlp); dfree(c->samples);
    dfree(c->tiles); dfree(c->tctl); dfree(c->tedge);
    dfree(c->det_out); dfree(c->det_tout); dfree(c->det_cnt); dfree(c->wctr);
    delete c;
}

// ---- GenerateXYZ (src/KMeans.cpp:1013-1050) ------------------------------------------
namespace {
__global__ void k_generate_xyz(double* x, double* y, double* z, const double* ra,
                               const double* dec, const double* r, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double sr, cr, sd, cd;
    sincos(ra[i], &sr, &cr);
    sincos(dec[i], &sd, &cd);
    double xi = cd * cr, yi = cd * sr, zi = sd;
    if (r) { const double ri = r[i]; xi *= ri; yi *= ri; zi *= ri; }
    x[i] = xi; y[i] = yi; z[i] = zi;
}
}  // namespace

int tc_generate_xyz_device(double* x, double* y, double* z, const double* ra, const double* dec,
                           const double* r, int64_t n)
{
    if (n < 0 || (n > 0 && (!x || !y || !z || !ra || !dec))) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    if (n == 0) return TC_OK;
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    count_launch();
    k_generate_xyz<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, y, z, ra, dec, r, n);
    TC_CU(cudaGetLastError());
    TC_CU(cudaStreamSynchronize(st));
    return TC_OK;
}

int tc_generate_xyz(double* x, double* y, double* z, const double* ra, const double* dec,
                    const double* r, int64_t n)
{
    if (n < 0 || (n > 0 && (!x || !y || !z || !ra || !dec))) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    if (n == 0) return TC_OK;
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    double* d = nullptr;
    const int nin = r ? 3 : 2;
    TC_TRY(dalloc(&d, (size_t)n * (3 + nin)));
    double *dx = d, *dy = d + n, *dz = d + 2 * n, *dra = d + 3 * n, *ddec = d + 4 * n;
    double* dr = r ? d + 5 * n : nullptr;
    int rc = TC_OK;
    if (cudaMemcpyAsync(dra, ra, sizeof(double) * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(ddec, dec, sizeof(double) * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        (r && cudaMemcpyAsync(dr, r, sizeof(double) * n, cudaMemcpyHostToDevice, st) != cudaSuccess)) {
        set_last_error("host to device copy failed"); rc = TC_ERR_CUDA;
    }
    if (rc == TC_OK) rc = tc_generate_xyz_device(dx, dy, dz, dra, ddec, dr, n);
    if (rc == TC_OK &&
        (cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
         cudaMemcpyAsync(y, dy, sizeof(double) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
         cudaMemcpyAsync(z, dz, sizeof(double) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
         cudaStreamSynchronize(st) != cudaSuccess)) {
        set_last_error("device to host copy failed"); rc = TC_ERR_CUDA;
    }
    dfree(d);
    return rc;
}

// ---- Catalog ingestion (treecorr/catalog.py:1343-1487; catalog.cu) -----------------------
int tc_catalog_finish_device(int64_t n, int ncols, double* const* cols, double* w, double* wpos,
                             const int64_t* flag, int64_t ignore_flag, int w_given,
                             int keep_zero_weight, tc_catalog_info* info)
{
    if (!info) { set_last_error("NULL info"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    return catalog_finish_device(n, ncols, cols, w, wpos, flag, ignore_flag, w_given,
                                 keep_zero_weight, st, info);
}

int tc_catalog_finish(int64_t n, int ncols, double* const* cols, double* w, double* wpos,
                      const int64_t* flag, int64_t ignore_flag, int w_given,
                      int keep_zero_weight, tc_catalog_info* info)
{
    if (!info || n < 0 || ncols < 0 || ncols > TC_CAT_MAXCOLS || (ncols > 0 && !cols) ||
        (n > 0 && !w)) {
        set_last_error("catalog: bad arguments (n >= 0, 0 <= ncols <= TC_CAT_MAXCOLS, w needed)");
        return TC_ERR_ARG;
    }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    const int nd = ncols + 1 + (wpos ? 1 : 0);
    double* d = nullptr;
    int64_t* dflag = nullptr;
    TC_TRY(dalloc(&d, (size_t)std::max<int64_t>(n, 1) * nd));
    if (flag) {
        const int rc = dalloc(&dflag, (size_t)std::max<int64_t>(n, 1));
        if (rc) { dfree(d); return rc; }
    }
    std::vector<double*> host(cols, cols + ncols), dev(nd);
    host.push_back(w);
    if (wpos) host.push_back(wpos);
    for (int c = 0; c < nd; ++c) dev[c] = d + (size_t)c * std::max<int64_t>(n, 1);
    int rc = TC_OK;
    cudaError_t e = cudaSuccess;
    for (int c = 0; c < nd && e == cudaSuccess && n > 0; ++c) {
        if (c == ncols && !w_given) continue;   // filled on the device
        if (!host[c]) { set_last_error("catalog: NULL column"); rc = TC_ERR_ARG; break; }
        e = cudaMemcpyAsync(dev[c], host[c], sizeof(double) * n, cudaMemcpyHostToDevice, st);
    }
    if (rc == TC_OK && e == cudaSuccess && flag && n > 0)
        e = cudaMemcpyAsync(dflag, flag, sizeof(int64_t) * n, cudaMemcpyHostToDevice, st);
    if (rc == TC_OK && e != cudaSuccess) {
        set_last_error(std::string("host to device copy: ") + cudaGetErrorString(e));
        rc = TC_ERR_CUDA;
    }
    if (rc == TC_OK)
        rc = catalog_finish_device(n, ncols, dev.data(), dev[ncols], wpos ? dev[ncols + 1] : nullptr,
                                   flag ? dflag : nullptr, ignore_flag, w_given, keep_zero_weight,
                                   st, info);
    if (rc == TC_OK && n > 0) {
        for (int c = 0; c < nd && e == cudaSuccess; ++c)
            if (info->nkeep > 0)
                e = cudaMemcpyAsync(host[c], dev[c], sizeof(double) * info->nkeep,
                                    cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_last_error(std::string("device to host copy: ") + cudaGetErrorString(e));
            rc = TC_ERR_CUDA;
        }
    }
    dfree(d);
    dfree(dflag);
    return rc;
}

int tc_catalog_center_size_device(int64_t n, const double* x, const double* y, const double* z,
                                  double* out)
{
    if (!out) { set_last_error("NULL out"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    return catalog_center_size_device(n, x, y, z, st, out);
}

int tc_catalog_center_size(int64_t n, const double* x, const double* y, const double* z,
                           double* out)
{
    if (!out || n <= 0 || !x || !y) { set_last_error("catalog centre: n > 0 and x, y needed"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    const int nc = z ? 3 : 2;
    double* d = nullptr;
    TC_TRY(dalloc(&d, (size_t)n * nc));
    const double* src[3] = {x, y, z};
    cudaError_t e = cudaSuccess;
    for (int c = 0; c < nc && e == cudaSuccess; ++c)
        e = cudaMemcpyAsync(d + (size_t)c * n, src[c], sizeof(double) * n, cudaMemcpyHostToDevice, st);
    int rc = TC_OK;
    if (e != cudaSuccess) {
        set_last_error(std::string("host to device copy: ") + cudaGetErrorString(e));
        rc = TC_ERR_CUDA;
    } else {
        rc = catalog_center_size_device(n, d, d + n, z ? d + 2 * n : nullptr, st, out);
    }
    dfree(d);
    return rc;
}

// ---- Patches ----------------------------------------------------------------------------
// All patch-pair correlations of one set of patch fields in one expansion (the per-pair
// loop of corr2base.py:929-950 / _process_all_auto): pairs (i, j), i <= j, whose fields
// can overlap; each gets its own arrays.
int tc_corr2_process_patches(tc_corr2* c, tc_field* const* fields, int npatch, int metric,
                             int quick, int max_pairs, int32_t* pair_i, int32_t* pair_j,
                             double* results, int* npairs_out)
{
    if (!c || !fields || npatch < 1 || !pair_i || !pair_j || !results || !npairs_out) {
        set_last_error("NULL argument"); return TC_ERR_ARG;
    }
    *npairs_out = 0;
    c->stats = tc_stats();
    const int coords = fields[0]->coords;
    for (int i = 0; i < npatch; ++i) {
        if (!fields[i] || fields[i]->dkind != c->d1 || c->d2 != c->d1 ||
            fields[i]->coords != coords) {
            set_last_error("patch fields must exist and match the corr's data kind and coords");
            return TC_ERR_ARG;
        }
    }
    TC_TRY(check_metric(coords, metric));
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    long long npoints = 0;
    for (int i = 0; i < npatch; ++i) {
        if (fields[i]->n == 0) continue;
        TC_TRY(field_build(fields[i]));
        npoints += fields[i]->n;
        c->stats.build_ms += fields[i]->build_ms;
    }
    // The pairs, as the reference chooses them (triviallyZero, src/Corr2.cpp:1107-1128).
    const double minsepsq = c->minsep * c->minsep, maxsepsq = c->maxsep * c->maxsep;
    std::vector<int> P1, P2;
    std::vector<int> pidx((size_t)npatch * npatch, -1);
    for (int i = 0; i < npatch; ++i) {
        if (fields[i]->n == 0) continue;
        for (int j = i; j < npatch; ++j) {
            if (fields[j]->n == 0) continue;
            if (i != j) {
                const double rsq = host_dist_sq(coords, metric, fields[i]->center, fields[j]->center);
                const double s = std::sqrt(fields[i]->center[3]) + std::sqrt(fields[j]->center[3]);
                if ((rsq < minsepsq && s < c->minsep && rsq < sqr(c->minsep - s)) ||
                    (rsq >= maxsepsq && rsq >= sqr(c->maxsep + s)))
                    continue;
            }
            pidx[(size_t)i * npatch + j] = pidx[(size_t)j * npatch + i] = (int)P1.size();
            P1.push_back(i); P2.push_back(j);
        }
    }
    const int npair = (int)P1.size();
    if (npair > max_pairs) { set_last_error("more patch pairs than max_pairs"); return TC_ERR_ARG; }
    const int nb = c->nbins;
    const int nq = 3 + xi_count(c->d1, c->d2);
    for (int p = 0; p < npair; ++p) { pair_i[p] = P1[p]; pair_j[p] = P2[p]; }
    std::fill(results, results + (size_t)npair * 8 * nb, 0.);
    *npairs_out = npair;
    if (npair == 0) return TC_OK;
    // Combined cells and roots.
    std::vector<long long> base(npatch, 0);
    long long ncells = 0;
    for (int i = 0; i < npatch; ++i) { base[i] = ncells; if (fields[i]->n) ncells += 2 * fields[i]->n - 1; }
    TCell* tc = nullptr;
    double* xyz = nullptr;
    int* d_pidx = nullptr;
    double* pacc = nullptr;
    unsigned long long* pnp = nullptr;
    long long* d_roff = nullptr;
    int2* d_pairs = nullptr;
    int* d_top = nullptr;
    int* d_topoff = nullptr;
    int rc = TC_OK;
    // Root tables: the top-level items are generated on the device from them.
    std::vector<int> htop, htopoff(npatch + 1, 0);
    for (int i = 0; i < npatch; ++i) {
        htopoff[i] = (int)htop.size();
        if (fields[i]->n)
            for (int t : fields[i]->tops) htop.push_back((int)(t + base[i]));
    }
    htopoff[npatch] = (int)htop.size();
    std::vector<long long> hroff(npair + 1, 0);
    std::vector<int2> hpairs(npair);
    for (int p = 0; p < npair; ++p) {
        const long long ni = htopoff[P1[p] + 1] - htopoff[P1[p]];
        const long long nj = htopoff[P2[p] + 1] - htopoff[P2[p]];
        hroff[p + 1] = hroff[p] + (P1[p] == P2[p] ? ni * (ni + 1) / 2 : ni * nj);
        hpairs[p] = make_int2(P1[p], P2[p]);
    }
    do {
        if (ncells > 2147483647LL) { set_last_error("too many cells for one patch expansion"); rc = TC_ERR_ARG; break; }
        if ((rc = dalloc(&tc, (size_t)ncells))) break;
        if ((rc = dalloc(&xyz, (size_t)ncells * 3))) break;
        if ((rc = dalloc(&d_roff, hroff.size()))) break;
        if ((rc = dalloc(&d_pairs, hpairs.size()))) break;
        if ((rc = dalloc(&d_top, std::max<size_t>(htop.size(), 1)))) break;
        if ((rc = dalloc(&d_topoff, htopoff.size()))) break;
        if ((rc = dalloc(&d_pidx, pidx.size()))) break;
        if ((rc = dalloc(&pacc, (size_t)npair * nq * nb))) break;
        if ((rc = dalloc(&pnp, (size_t)npair * nb))) break;
        for (int i = 0; i < npatch && !rc; ++i) {
            const long long n = fields[i]->n ? 2 * fields[i]->n - 1 : 0;
            if (!n) continue;
            if (cudaMemcpyAsync(tc + base[i], fields[i]->tcells, sizeof(TCell) * n, cudaMemcpyDeviceToDevice, st) ||
                cudaMemcpyAsync(xyz + base[i], fields[i]->cells.x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st) ||
                cudaMemcpyAsync(xyz + ncells + base[i], fields[i]->cells.y, sizeof(double) * n, cudaMemcpyDeviceToDevice, st) ||
                cudaMemcpyAsync(xyz + 2 * ncells + base[i], fields[i]->cells.z, sizeof(double) * n, cudaMemcpyDeviceToDevice, st)) {
                set_last_error("cell copy failed"); rc = TC_ERR_CUDA; break;
            }
            count_launch();
            k_rebase_cells<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(tc + base[i], n, (int)base[i], i);
        }
        if (rc) break;
        if (cudaMemcpyAsync(d_roff, hroff.data(), sizeof(long long) * hroff.size(), cudaMemcpyHostToDevice, st) ||
            cudaMemcpyAsync(d_pairs, hpairs.data(), sizeof(int2) * hpairs.size(), cudaMemcpyHostToDevice, st) ||
            cudaMemcpyAsync(d_top, htop.data(), sizeof(int) * htop.size(), cudaMemcpyHostToDevice, st) ||
            cudaMemcpyAsync(d_topoff, htopoff.data(), sizeof(int) * htopoff.size(), cudaMemcpyHostToDevice, st) ||
            cudaMemcpyAsync(d_pidx, pidx.data(), sizeof(int) * pidx.size(), cudaMemcpyHostToDevice, st) ||
            cudaMemsetAsync(pacc, 0, sizeof(double) * (size_t)npair * nq * nb, st) ||
            cudaMemsetAsync(pnp, 0, sizeof(unsigned long long) * (size_t)npair * nb, st)) {
            set_last_error("patch setup copy failed"); rc = TC_ERR_CUDA; break;
        }
        TravParams T;
        trav_setup(c, T, coords, metric, quick, nq);
        T.c1 = tc; T.c2 = tc;
        T.x1 = xyz; T.y1 = xyz + ncells; T.z1 = xyz + 2 * ncells;
        T.x2 = T.x1; T.y2 = T.y1; T.z2 = T.z1;
        T.ngen = hroff[npair]; T.in_tasks = nullptr; T.nin = 0;
        T.mode = 3; T.npatch = npatch; T.pair_index = d_pidx; T.pacc = pacc; T.pnp = pnp;
        T.npair = npair; T.proot_off = d_roff; T.ppairs = d_pairs; T.ptop = d_top;
        T.ptop_off = d_topoff;
        int blocks = 0, nwarps = 0;
        if ((rc = expand_grid(nq, nb, &blocks, &nwarps, 3))) break;
        if ((rc = expand_scratch(c, nwarps, nq))) break;
        T.nwarps = nwarps; T.err = c->d_err; T.counters = c->ctl + 2;
        cudaMemsetAsync(c->ctl, 0, 8 * sizeof(unsigned long long), st);
        cudaMemsetAsync(c->d_err, 0, sizeof(int), st);
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0); cudaEventCreate(&e1);
        cudaEventRecord(e0, st);
        int derr = 0;
        long long launches = 0;
        rc = expand_run(c, T, blocks, npoints, st, &derr, &launches);
        cudaEventRecord(e1, st);
        if (!rc && derr) { set_last_error(std::string("device error: ") + dev_err_msg(derr)); rc = TC_ERR_DEVICE; }
        std::vector<double> hacc;
        std::vector<unsigned long long> hnp;
        unsigned long long cntr[4] = {0, 0, 0, 0};
        if (!rc) {
            hacc.resize((size_t)npair * nq * nb);
            hnp.resize((size_t)npair * nb);
            if (cudaMemcpyAsync(hacc.data(), pacc, sizeof(double) * hacc.size(), cudaMemcpyDeviceToHost, st) ||
                cudaMemcpyAsync(hnp.data(), pnp, sizeof(unsigned long long) * hnp.size(), cudaMemcpyDeviceToHost, st) ||
                cudaMemcpyAsync(cntr, c->ctl + 2, sizeof(cntr), cudaMemcpyDeviceToHost, st) ||
                cudaStreamSynchronize(st)) { set_last_error("result copy failed"); rc = TC_ERR_CUDA; }
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        if (rc) break;
        // results[p] = weight, meanr, meanlogr, xi0..xi3, npairs (each nb doubles).
        for (int p = 0; p < npair; ++p) {
            double* r = results + (size_t)p * 8 * nb;
            const double* a = hacc.data() + (size_t)p * nq * nb;
            for (int k = 0; k < nb; ++k) {
                r[k] = a[k];
                if (!quick) { r[nb + k] = a[nb + k]; r[2 * nb + k] = a[2 * nb + k]; }
                for (int q = 3; q < nq; ++q) r[q * nb + k] = a[q * nb + k];
                if (!quick) r[7 * nb + k] = (double)hnp[(size_t)p * nb + k];
            }
        }
        c->stats.cell_pairs = (int64_t)cntr[0];
        c->stats.accepted = (int64_t)cntr[1];
        c->stats.escalated = (int64_t)cntr[2];
        c->stats.launches = launches;
        c->stats.traverse_ms = ms;
    } while (0);
    dfree(tc); dfree(xyz); dfree(d_pidx); dfree(pacc); dfree(pnp);
    dfree(d_roff); dfree(d_pairs); dfree(d_top); dfree(d_topoff);
    return rc;
}

// Jackknife data vectors and covariance on the device (see k_jackknife_rows).
int tc_jackknife_cov(const double* results, const int32_t* pair_i, const int32_t* pair_j,
                     int npair, int npatch, int nbins, int dkind, int cross_patch_weight,
                     double* v_out, double* cov_out)
{
    if (!results || !pair_i || !pair_j || !v_out || !cov_out || npair < 1 || npatch < 2 || nbins < 1) {
        set_last_error("bad argument"); return TC_ERR_ARG;
    }
    if (dkind != TC_GDATA && dkind != TC_KDATA) { set_last_error("jackknife rows for GG and KK only"); return TC_ERR_UNSUPPORTED; }
    if (cross_patch_weight < 0 || cross_patch_weight > 2) { set_last_error("cross_patch_weight: 0 simple, 1 mean, 2 match"); return TC_ERR_ARG; }
    const int nstat = dkind == TC_GDATA ? 2 : 1;
    const int nv = nstat * nbins;
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    double *dres = nullptr, *dv = nullptr, *dw = nullptr, *dc = nullptr;
    int* dpi = nullptr;
    int rc = TC_OK;
    do {
        if ((rc = dalloc(&dres, (size_t)npair * 8 * nbins))) break;
        if ((rc = dalloc(&dpi, (size_t)2 * npair))) break;
        if ((rc = dalloc(&dv, (size_t)npatch * nv))) break;
        if ((rc = dalloc(&dw, (size_t)npatch))) break;
        if ((rc = dalloc(&dc, (size_t)nv * nv))) break;
        if (cudaMemcpyAsync(dres, results, sizeof(double) * npair * 8 * nbins, cudaMemcpyHostToDevice, st) ||
            cudaMemcpyAsync(dpi, pair_i, sizeof(int) * npair, cudaMemcpyHostToDevice, st) ||
            cudaMemcpyAsync(dpi + npair, pair_j, sizeof(int) * npair, cudaMemcpyHostToDevice, st)) {
            set_last_error("copy failed"); rc = TC_ERR_CUDA; break;
        }
        // 'match' weight, Mohammad and Percival (2022) eq. 27 as in corr2base.py:1812.
        const double wmatch = 1. - (double)npatch / (2. + std::sqrt(2.) * (npatch - 1));
        count_launch();
        k_jackknife_rows<<<npatch, 128, 0, st>>>(dres, dpi, dpi + npair, npair, nbins,
                                                 cross_patch_weight, wmatch, nstat, 0, 2, dv, dw);
        count_launch();
        k_jackknife_cov<<<dim3(nv, (nv + 127) / 128), 128, 0, st>>>(dv, npatch, nv, dc);
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(v_out, dv, sizeof(double) * npatch * nv, cudaMemcpyDeviceToHost, st) ||
            cudaMemcpyAsync(cov_out, dc, sizeof(double) * nv * nv, cudaMemcpyDeviceToHost, st) ||
            cudaStreamSynchronize(st)) { set_last_error("jackknife kernels failed"); rc = TC_ERR_CUDA; }
    } while (0);
    dfree(dres); dfree(dpi); dfree(dv); dfree(dw); dfree(dc);
    return rc;
}

int tc_tcgen05_selftest(const float* a, const float* b, float* c, int n, int k)
{
    if (!a || !b || !c) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    const int rc = tcgen05_selftest(a, b, c, n, k, st);
    return rc == 0 ? TC_OK : (rc == 1 ? TC_ERR_ARG : (rc == 4 ? TC_ERR_DEVICE : TC_ERR_CUDA));
}

int tc_mlp_nparam(void) { return MLP_NPARAM; }

int tc_corr2_set_learned(tc_corr2* c, const float* params, double threshold, double cand_factor)
{
    if (!c) { set_last_error("NULL corr"); return TC_ERR_ARG; }
    if (!params) { c->mode = 0; return TC_OK; }
    if (!(cand_factor >= 1.)) { set_last_error("cand_factor must be >= 1"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    TC_TRY(mlp_pack(params, &c->mlp, st));
    c->mlp_thr = (float)threshold;
    c->cand_factor = (float)cand_factor;
    c->mode = 2;
    return TC_OK;
}

int tc_learn_collect(tc_corr2* c, tc_field* f, int metric, int sample_mod, int64_t max_samples,
                     int64_t max_point_pairs, float* feat_out, float* target_out, int64_t* n_out)
{
    if (!c || !f || !feat_out || !target_out || !n_out) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    if (sample_mod < 1 || max_samples < 1) { set_last_error("sample_mod and max_samples must be >= 1"); return TC_ERR_ARG; }
    *n_out = 0;
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    if (c->sample_cap < max_samples) {
        dfree(c->samples);
        c->sample_cap = 0;
        TC_TRY(dalloc(&c->samples, (size_t)max_samples));
        c->sample_cap = max_samples;
    }
    const int old_mode = c->mode;
    c->mode = 1;
    c->sample_mod = (unsigned)sample_mod;
    const long long cap_keep = c->sample_cap;
    c->sample_cap = max_samples;
    int rc = corr_process(c, f, nullptr, 0, metric);
    c->sample_cap = cap_keep;
    c->mode = old_mode;
    if (rc) return rc;
    unsigned long long ns = 0;
    TC_CU(cudaMemcpy(&ns, c->ctl + 6, sizeof(ns), cudaMemcpyDeviceToHost));
    const long long n = std::min<long long>((long long)ns, max_samples);
    if (n == 0) return TC_OK;
    float *dfeat = nullptr, *dtar = nullptr;
    TC_TRY(dalloc(&dfeat, (size_t)n * MLP_IN));
    if (dalloc(&dtar, (size_t)n)) { dfree(dfeat); return TC_ERR_NOMEM; }
    LabelParams L;
    std::memset(&L, 0, sizeof(L));
    L.coords = f->coords; L.metric = metric; L.nbins = c->nbins;
    L.minsepsq = c->minsep * c->minsep; L.maxsepsq = c->maxsep * c->maxsep;
    L.logminsep = std::log(c->minsep); L.binsize = c->binsize;
    L.finvminsepsq = (float)(1. / L.minsepsq); L.finvbinsize = (float)(1. / c->binsize);
    L.finvlogrange = (float)(1. / std::log(c->maxsep / c->minsep)); L.fbinsize = (float)c->binsize;
    L.max_point_pairs = max_point_pairs;
    L.c1 = f->tcells; L.c2 = f->tcells;
    L.start1 = f->cells.start; L.start2 = f->cells.start;
    L.x1 = f->buf[0].x; L.y1 = f->buf[0].y; L.z1 = f->buf[0].z;
    L.x2 = f->buf[0].x; L.y2 = f->buf[0].y; L.z2 = f->buf[0].z;
    L.w1 = f->buf[0].w; L.w2 = f->buf[0].w;
    rc = launch_label(L, c->samples, n, dfeat, dtar, st);
    if (!rc) {
        cudaMemcpyAsync(feat_out, dfeat, sizeof(float) * n * MLP_IN, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(target_out, dtar, sizeof(float) * n, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) { set_last_error("labelling failed"); rc = TC_ERR_CUDA; }
    }
    dfree(dfeat); dfree(dtar);
    if (rc) return rc == 5 ? TC_ERR_NOMEM : (rc == 2 ? TC_ERR_CUDA : rc);
    *n_out = n;
    return TC_OK;
}

int tc_mlp_grad(const float* params, const float* x, const float* y, int64_t n, float* grad,
                float* loss)
{
    if (!params || !x || !y || !grad || !loss || n < 1) { set_last_error("bad argument"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    return mlp_grad_host(params, x, y, n, grad, loss, st) ? TC_ERR_CUDA : TC_OK;
}

int tc_mlp_infer(const float* params, const float* x, int64_t n, float* y)
{
    if (!params || !x || !y || n < 1) { set_last_error("bad argument"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    return mlp_infer_host(params, x, n, y, st) ? TC_ERR_CUDA : TC_OK;
}

int tc_mlp_train(float* params, const float* x, const float* y, int64_t n, int steps, int batch,
                 float lr, unsigned seed, float* loss_out)
{
    if (!params || !x || !y || n < 1 || steps < 0 || batch < 1) { set_last_error("bad argument"); return TC_ERR_ARG; }
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    return mlp_train_host(params, x, y, n, steps, batch, lr, seed, loss_out, st) ? TC_ERR_CUDA : TC_OK;
}

int tc_corr2_set_tuning(tc_corr2* c, int tile_leaf, int64_t chunk)
{
    if (!c) { set_last_error("NULL corr"); return TC_ERR_ARG; }
    if (tile_leaf != 0 && (tile_leaf < 8 || tile_leaf > 64)) {
        set_last_error("tile_leaf must be 0 (default) or 8..64"); return TC_ERR_ARG;
    }
    if (chunk != 0 && (chunk < (1 << 16) || chunk > (1LL << 26))) {
        set_last_error("chunk must be 0 (default) or 2^16..2^26 work items"); return TC_ERR_ARG;
    }
    c->tile_leaf = tile_leaf;
    c->chunk = chunk;
    return TC_OK;
}

namespace {
// The autotuner's choices per configuration (classes, coordinates, metric, binning, slops,
// brute fields and catalog sizes to a factor of 2), for the life of the process.
struct TuneKey {
    int d1, d2, coords, metric, nbins, brute, lg1, lg2;
    double minsep, maxsep, b, a;
    bool operator<(const TuneKey& o) const
    {
        return std::tie(d1, d2, coords, metric, nbins, brute, lg1, lg2, minsep, maxsep, b, a) <
               std::tie(o.d1, o.d2, o.coords, o.metric, o.nbins, o.brute, o.lg1, o.lg2,
                        o.minsep, o.maxsep, o.b, o.a);
    }
};
std::map<TuneKey, std::pair<int, long long>> g_tuned;
std::mutex g_tune_mu;
int ilog2(long long n) { int l = 0; while (n > 1) { n >>= 1; ++l; } return l; }
}  // namespace

// Times the correlation of f1 (and f2) on its first `frac` of top-level pairs for tile leaf
// sizes 24..64 (exact mode) and then for expansion chunks of 1/2, 1/4 and 1/8 of the default
// (down to 2^21 items): a coordinate search on event-timed device time.  Keeps the fastest
// in c and in a per-process cache, and leaves the caller's outputs untouched.
int tc_corr2_autotune(tc_corr2* c, tc_field* f1, tc_field* f2, int metric, double frac,
                      int* tile_leaf_out, int64_t* chunk_out, double* ms_out)
{
    if (!c || !f1) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    if (!(frac > 0. && frac <= 1.)) { set_last_error("frac must be in (0, 1]"); return TC_ERR_ARG; }
    if (c->mode != 0) { set_last_error("autotune runs the bin_slop criterion only"); return TC_ERR_ARG; }
    TuneKey key{c->d1, c->d2, f1->coords, metric, c->nbins, f1->brute + 2 * (f2 ? f2->brute : 0),
                ilog2(f1->n + 1), f2 ? ilog2(f2->n + 1) : -1, c->minsep, c->maxsep, c->b, c->a};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            c->tile_leaf = it->second.first;
            c->chunk = it->second.second;
            if (tile_leaf_out) *tile_leaf_out = c->tile_leaf;
            if (chunk_out) *chunk_out = c->chunk;
            if (ms_out) *ms_out = 0.;
            return TC_OK;
        }
    }
    TC_TRY(field_build(f1));
    if (f2) TC_TRY(field_build(f2));
    const long long ntop1 = (long long)f1->tops.size();
    const long long ngen = f2 ? ntop1 * (long long)f2->tops.size() : ntop1 * (ntop1 + 1) / 2;
    const bool exact = c->a == 0. || (f1->brute && (f2 ? f2->brute : f1->brute));
    const long long npoints = f1->n + (f2 ? f2->n : 0);
    const long long ch0 = expand_chunk(npoints);
    c->root_limit = std::max<long long>(1, (long long)(frac * (double)ngen));
    c->no_output = true;
    auto trial = [&](int leaf, long long ch, double* ms) {
        c->tile_leaf = leaf;
        c->chunk = ch;
        const int rc = corr_process(c, f1, f2, 0, metric);
        *ms = c->stats.traverse_ms;
        return rc;
    };
    int best_leaf = 0;
    long long best_ch = 0;
    double best = 0., ms = 0.;
    int rc = trial(exact ? TILE_LEAF : 0, ch0, &ms);   // allocations, first launches
    if (!rc) rc = trial(exact ? TILE_LEAF : 0, ch0, &best);
    best_leaf = exact ? TILE_LEAF : 0;
    best_ch = ch0;
    if (!rc && exact) {
        for (int leaf = 24; leaf <= 64 && !rc; leaf += 8) {
            if (leaf == TILE_LEAF) continue;
            rc = trial(leaf, ch0, &ms);
            if (!rc && ms < best) { best = ms; best_leaf = leaf; }
        }
    }
    for (long long ch = ch0 >> 1; ch >= std::max<long long>(1LL << 21, ch0 >> 3) && !rc; ch >>= 1) {
        rc = trial(best_leaf, ch, &ms);
        if (!rc && ms < best) { best = ms; best_ch = ch; }
    }
    c->root_limit = 0;
    c->no_output = false;
    c->stats = tc_stats();
    if (rc) { c->tile_leaf = 0; c->chunk = 0; return rc; }
    c->tile_leaf = best_leaf;
    c->chunk = best_ch == ch0 ? 0 : best_ch;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tuned[key] = {c->tile_leaf, c->chunk};
    }
    if (tile_leaf_out) *tile_leaf_out = c->tile_leaf;
    if (chunk_out) *chunk_out = c->chunk;
    if (ms_out) *ms_out = best;
    return TC_OK;
}

int tc_corr2_process_auto(tc_corr2* c, tc_field* f, int dots, int quick, int metric)
{
    (void)dots;
    if (!f) { set_last_error("NULL field"); return TC_ERR_ARG; }
    return corr_process(c, f, nullptr, quick, metric);
}

int tc_corr2_process_cross(tc_corr2* c, tc_field* f1, tc_field* f2, int dots, int quick,
                           int metric)
{
    (void)dots;
    if (!f1 || !f2) { set_last_error("NULL field"); return TC_ERR_ARG; }
    return corr_process(c, f1, f2, quick, metric);
}

int tc_corr2_process_auto_noalloc(tc_corr2* c, tc_field* f, int quick, int metric)
{
    return corr_process_auto_noalloc(c, f, quick, metric);
}

int tc_corr2_trivially_zero(tc_corr2* c, int metric, int coords, double x1, double y1,
                            double z1, double s1, double x2, double y2, double z2, double s2,
                            int* out)
{
    if (!c || !out) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    TC_TRY(check_metric(coords, metric));
    // BaseCorr2::triviallyZero, src/Corr2.cpp:590-601; Position<Sphere> normalises.
    double p1[3] = {x1, y1, coords == TC_FLAT ? 0. : z1};
    double p2[3] = {x2, y2, coords == TC_FLAT ? 0. : z2};
    if (coords == TC_SPHERE) {
        for (double* p : {p1, p2}) {
            double nn = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
            if (nn == 0.) { p[0] = 1.; p[1] = 0.; p[2] = 0.; }
            else { p[0] /= nn; p[1] /= nn; p[2] /= nn; }
        }
    }
    double rsq = host_dist_sq(coords, metric, p1, p2);
    double s1ps2 = s1 + s2;
    double maxsepsq = c->maxsep * c->maxsep;
    *out = (rsq >= maxsepsq && rsq >= sqr(c->maxsep + s1ps2)) ? 1 : 0;
    return TC_OK;
}

int tc_corr2_stats(const tc_corr2* c, tc_stats* out)
{
    if (!c || !out) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    *out = c->stats;
    return TC_OK;
}

int tc_corr3_create(int d1, int d2, int d3, int bin_type, double minsep, double maxsep,
                    int nbins, double binsize, double b, double a, double minu, double maxu,
                    int nubins, double ubinsize, double bu, double minv, double maxv,
                    int nvbins, double vbinsize, double bv, double minrpar, double maxrpar,
                    double xp, double yp, double zp, double* zeta0, double* zeta1,
                    double* zeta2, double* zeta3, double* zeta4, double* zeta5, double* zeta6,
                    double* zeta7, double* meand1, double* meanlogd1, double* meand2,
                    double* meanlogd2, double* meand3, double* meanlogd3, double* meanu,
                    double* meanv, double* weight, double* weight_im, double* ntri,
                    tc_corr3** out)
{
    (void)minu; (void)maxu; (void)ubinsize; (void)bu; (void)minv; (void)maxv; (void)nvbins;
    (void)vbinsize; (void)bv; (void)meand1; (void)meanlogd1; (void)meanu; (void)meanv;
    if (!out) { set_last_error("out is NULL"); return TC_ERR_ARG; }
    *out = nullptr;
    // The 21 classes of WrapCorr3 (src/Corr3.cpp:4233-4262): N, K or G at each vertex, not
    // all three different.
    auto nkg = [](int d) { return d == TC_NDATA || d == TC_KDATA || d == TC_GDATA; };
    if (!nkg(d1) || !nkg(d2) || !nkg(d3) || (d1 != d2 && d2 != d3 && d1 != d3)) {
        set_last_error("the GPU 3-point path has the N, K and G classes of the reference "
                       "(GGG, NNN, KKK, NKK, NNG, GKG, ...)");
        return TC_ERR_UNSUPPORTED;
    }
    if (bin_type != TC_LOGMULTIPOLE) {
        set_last_error("only LogMultipole binning is on the GPU 3-point path");
        return TC_ERR_UNSUPPORTED;
    }
    const double big = std::numeric_limits<double>::max();
    if (!(minrpar <= -big) || !(maxrpar >= big) || xp != 0. || yp != 0. || zp != 0.) {
        set_last_error("min_rpar/max_rpar/period are not on the GPU path");
        return TC_ERR_UNSUPPORTED;
    }
    if (nbins <= 0 || nubins < 0 || !(minsep > 0.) || !(maxsep > minsep) || !(binsize > 0.)) {
        set_last_error("invalid binning");
        return TC_ERR_ARG;
    }
    tc_corr3 probe;
    probe.dv = d1; probe.dk = d2; probe.dk3 = d3;
    const int nz = c3_nzeta(c3_algo(&probe));
    double* z[8] = {zeta0, zeta1, zeta2, zeta3, zeta4, zeta5, zeta6, zeta7};
    bool have = true;
    for (int q = 0; q < nz; ++q) have = have && z[q];
    if (!have || !meand2 || !meanlogd2 || !meand3 || !meanlogd3 || !weight || !weight_im ||
        !ntri) {
        set_last_error("missing output array");
        return TC_ERR_ARG;
    }
    tc_corr3* c = new tc_corr3();
    c->dv = d1;
    c->dk = d2;
    c->dk3 = d3;
    c->bin_type = bin_type; c->nbins = nbins; c->maxn = nubins;
    c->minsep = minsep; c->maxsep = maxsep; c->binsize = binsize; c->b = b; c->a = a;
    for (int q = 0; q < 8; ++q) c->zeta[q] = q < nz ? z[q] : nullptr;
    c->meand2 = meand2; c->meanlogd2 = meanlogd2; c->meand3 = meand3; c->meanlogd3 = meanlogd3;
    c->weight = weight; c->weight_im = weight_im; c->ntri = ntri;
    *out = c;
    return TC_OK;
}

void tc_corr3_free(tc_corr3* c)
{
    if (!c) return;
    free_mp_scratch(c->X);
    delete c;
}

int tc_corr3_process_auto(tc_corr3* c, tc_field* f, int dots, int quick, int metric)
{
    (void)dots;
    if (c) c->ms = 0.;
    return corr3_run(c, f, f, nullptr, 1, quick, metric);
}

int tc_corr3_process_cross12(tc_corr3* c, tc_field* f1, tc_field* f2, int ordered, int dots,
                             int quick, int metric)
{
    (void)dots;
    if (c) c->ms = 0.;
    // ProcessCross12c, src/Corr3.cpp:3730-3768.
    if (ordered == 0) TC_TRY(corr3_run(c, f2, f1, f2, 1, quick, metric));
    else if (ordered != 1) { set_last_error("ordered must be 0 or 1"); return TC_ERR_ARG; }
    return corr3_run(c, f1, f2, nullptr, 1, quick, metric);
}

int tc_corr3_process_cross21(tc_corr3* c, tc_field* f1, tc_field* f2, int ordered, int dots,
                             int quick, int metric)
{
    (void)dots;
    if (c) c->ms = 0.;
    // ProcessCross21c, src/Corr3.cpp:3831-3868.
    if (ordered == 0) {
        TC_TRY(corr3_run(c, f2, f1, f1, 1, quick, metric));
        TC_TRY(corr3_run(c, f1, f2, f1, 1, quick, metric));
        return corr3_run(c, f1, f1, f2, 1, quick, metric);
    }
    if (ordered == 3) return corr3_run(c, f1, f1, f2, 4, quick, metric);
    set_last_error("ordered must be 0 or 3");
    return TC_ERR_ARG;
}

int tc_corr3_process_cross(tc_corr3* c, tc_field* f1, tc_field* f2, tc_field* f3, int ordered,
                           int dots, int quick, int metric)
{
    (void)dots;
    if (c) c->ms = 0.;
    if (!f3) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    // ProcessCrossc, src/Corr3.cpp:3938-3976.
    switch (ordered) {
      case 0:
        TC_TRY(corr3_run(c, f2, f1, f3, 1, quick, metric));
        TC_TRY(corr3_run(c, f3, f1, f2, 1, quick, metric));
        return corr3_run(c, f1, f2, f3, 1, quick, metric);
      case 1: return corr3_run(c, f1, f2, f3, 1, quick, metric);
      case 2:
        TC_TRY(corr3_run(c, f1, f2, f3, 4, quick, metric));
        return corr3_run(c, f3, f2, f1, 4, quick, metric);
      case 3:
        TC_TRY(corr3_run(c, f1, f2, f3, 4, quick, metric));
        return corr3_run(c, f2, f1, f3, 4, quick, metric);
      case 4: return corr3_run(c, f1, f2, f3, 4, quick, metric);
      default: set_last_error("ordered must be 0 .. 4"); return TC_ERR_ARG;
    }
}

double tc_corr3_last_ms(const tc_corr3* c) { return c ? c->ms : 0.; }

int tc_corr3_stats(const tc_corr3* c, int64_t out[3])
{
    if (!c || !out) { set_last_error("NULL argument"); return TC_ERR_ARG; }
    out[0] = c->X.records - c->X.overflow;
    out[1] = c->X.overflow;
    out[2] = c->X.waves;
    return TC_OK;
}

int tc_set_omp_threads(int num_threads) { (void)num_threads; return 1; }
int tc_get_omp_threads(void) { return 1; }

int tc_trim_memory(void)
{
    int dev = 0;
    TC_CU(cudaGetDevice(&dev));
    cudaStream_t st;
    TC_TRY(stream_get(&st));
    TC_CU(cudaStreamSynchronize(st));
    cudaMemPool_t pool;
    TC_CU(cudaDeviceGetDefaultMemPool(&pool, dev));
    TC_CU(cudaMemPoolTrimTo(pool, 0));
    return TC_OK;
}

int tc_set_deterministic(int on)
{
    const int prev = g_deterministic.load();
    g_deterministic.store(on ? 1 : 0);
    return prev;
}
int tc_get_deterministic(void) { return g_deterministic.load(); }

const char* tc_last_error(void) { return g_last_error.c_str(); }

long long tc_launch_count(void) { return g_launches.load(); }

void* tc_stream(void)
{
    cudaStream_t s = nullptr;
    if (stream_get(&s)) return nullptr;
    return (void*)s;
}

}  // extern "C"
