// catalog.cu -- catalog ingestion on device columns.
//
// The column work of TreeCorr's Catalog._finish_input (treecorr/catalog.py:1343-1487) for a
// catalog whose columns already live in GPU memory, so that a pipeline can go from raw
// columns to a field without a host round trip:
//   * flag -> weight (1393-1404): w = 0 and wpos = 0 where (flag & ignore_flag) != 0, with
//     ignore_flag = ~ok_flag unless given;
//   * checkForNaN (1406-1425, 1684-1704) on every column in the caller's order, then w, then
//     wpos: a NaN row gets w = 0 and the NaN becomes 0; counts per column;
//   * wpos == 0 -> w = 0 (1433-1450), counting the rows whose w was not 0 (the reference's
//     "invalid" case, which it logs and then fixes the same way);
//   * sumw (1452-1462): the sum of w when the weights are non-trivial (w given, flags, or a
//     NaN / zero wpos that created a weight column), else the row count; sumw == 0 is an
//     error;
//   * the removal of rows with wpos == 0 (or w == 0 without wpos) unless keep_zero_weight
//     (1464-1468, Catalog.select): a stable compaction of every column in place.
// GenerateXYZ (1609-1622) is the separate tc_generate_xyz_device; the catalog's centre and
// size (_get_center_size, 1330-1341: the unweighted mean position and the largest distance
// from it, which triviallyZero uses to skip far patch pairs) is catalog_center_size_device.
//
// k_cat_mark does the per-row rules, one thread per row, with integer atomic counts (rare:
// NaNs and zero wpos) and per-block partial sums of w (a fixed shuffle tree), keep counts
// and non-zero counts; k_cat_total (one block) adds the block partials in a fixed order and
// turns the keep counts into block offsets; k_cat_scatter moves one column's kept rows to
// their ranks (warp ballots), into a scratch column copied back.  Every sum is formed in a
// fixed order, so the results repeat bit for bit; sumw differs from numpy's pairwise sum
// only in rounding (~1e-16 relative).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "tc_host.hpp"
#include "catalog.hpp"

namespace tc {

namespace {

constexpr int CAT_TPB = 256;               // threads per block (rows per block)
constexpr int CAT_WPB = CAT_TPB / 32;
constexpr int CAT_TOT = 1024;              // threads of the single-block total

struct CatCols {
    double* p[TC_CAT_MAXCOLS];
};

// counts: [0, ncols) NaNs per column, ncols: w NaNs, ncols + 1: wpos NaNs, ncols + 2: rows
// with wpos == 0, ncols + 3: of those, rows whose w was not 0.
__global__ void __launch_bounds__(CAT_TPB) k_cat_mark(int64_t n, int ncols,
                                                 const __grid_constant__ CatCols C, double* w,
                                                 double* wpos, const int64_t* flag,
                                                 int64_t ignore, int w_given,
                                                 unsigned long long* counts, double* bsum,
                                                 int* bkeep, int* bnz, unsigned char* keep)
{
    __shared__ double ws[CAT_WPB];
    const int64_t i = (int64_t)blockIdx.x * CAT_TPB + threadIdx.x;
    double wi = 0.;
    bool kp = false, nz = false;
    if (i < n) {
        wi = w_given ? w[i] : 1.0;
        double p = wpos ? wpos[i] : 0.;
        if (flag && (flag[i] & ignore) != 0) {
            wi = 0.;
            p = 0.;
        }
        for (int c = 0; c < ncols; ++c) {
            const double v = C.p[c][i];
            if (v != v) {
                wi = 0.;
                C.p[c][i] = 0.;
                atomicAdd(&counts[c], 1ull);
            }
        }
        if (wi != wi) {
            wi = 0.;
            atomicAdd(&counts[ncols], 1ull);
        }
        if (wpos) {
            if (p != p) {
                wi = 0.;
                p = 0.;
                atomicAdd(&counts[ncols + 1], 1ull);
            }
            if (p == 0.) {
                atomicAdd(&counts[ncols + 2], 1ull);
                if (wi != 0.) atomicAdd(&counts[ncols + 3], 1ull);
                wi = 0.;
            }
            wpos[i] = p;
        }
        w[i] = wi;
        kp = (wpos ? p : wi) != 0.;
        nz = wi != 0.;
        keep[i] = kp ? 1 : 0;
    }
    double s = wi;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    const int nk = __syncthreads_count(kp);
    const int nzc = __syncthreads_count(nz);
    if (threadIdx.x == 0) {
        double t = 0.;
        for (int q = 0; q < CAT_WPB; ++q) t += ws[q];
        bsum[blockIdx.x] = t;
        bkeep[blockIdx.x] = nk;
        bnz[blockIdx.x] = nzc;
    }
}

// One block: tot[0] = sum of the block sums, itot[0] = kept rows, itot[1] = non-zero rows,
// boff[b] = kept rows before block b.  Thread t takes a contiguous run of blocks.
__global__ void __launch_bounds__(CAT_TOT) k_cat_total(int nblk, const double* bsum, const int* bkeep,
                                                  const int* bnz, int64_t* boff, double* tot,
                                                  long long* itot)
{
    __shared__ double ds[CAT_TOT];
    __shared__ long long ks[CAT_TOT], zs[CAT_TOT];
    const int t = threadIdx.x;
    const int per = (nblk + CAT_TOT - 1) / CAT_TOT;
    const int b0 = t * per, b1 = min(nblk, b0 + per);
    double s = 0.;
    long long k = 0, z = 0;
    for (int b = b0; b < b1; ++b) { s += bsum[b]; k += bkeep[b]; z += bnz[b]; }
    ds[t] = s; ks[t] = k; zs[t] = z;
    __syncthreads();
    if (t == 0) {
        double S = 0.;
        long long K = 0, Z = 0;
        for (int q = 0; q < CAT_TOT; ++q) {
            S += ds[q];
            const long long kq = ks[q];
            ks[q] = K;          // exclusive prefix of the kept rows per thread run
            K += kq;
            Z += zs[q];
        }
        tot[0] = S;
        itot[0] = K;
        itot[1] = Z;
    }
    __syncthreads();
    long long off = ks[t];
    for (int b = b0; b < b1; ++b) { boff[b] = off; off += bkeep[b]; }
}

// The kept rows of one column at their ranks: dst[boff[block] + rank in block] = src[i].
__global__ void __launch_bounds__(CAT_TPB) k_cat_scatter(int64_t n, const double* src, double* dst,
                                                    const unsigned char* keep,
                                                    const int64_t* boff)
{
    __shared__ int woff[CAT_WPB];
    const int64_t i = (int64_t)blockIdx.x * CAT_TPB + threadIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const bool kp = i < n && keep[i] != 0;
    const unsigned m = __ballot_sync(0xffffffffu, kp);
    if (lane == 0) woff[wid] = __popc(m);
    __syncthreads();
    int before = 0;
    for (int q = 0; q < wid; ++q) before += woff[q];
    if (kp) dst[boff[blockIdx.x] + before + __popc(m & ((1u << lane) - 1u))] = src[i];
}

// Catalog._get_center_size (treecorr/catalog.py:1330-1341): block sums of x, y, z for the
// unweighted mean, then the largest squared distance from it.
__global__ void __launch_bounds__(CAT_TPB) k_cat_sums(int64_t n, const double* x, const double* y,
                                                      const double* z, double* bsum)
{
    __shared__ double ws[3][CAT_WPB];
    const int64_t i = (int64_t)blockIdx.x * CAT_TPB + threadIdx.x;
    double v[3] = {0., 0., 0.};
    if (i < n) { v[0] = x[i]; v[1] = y[i]; v[2] = z ? z[i] : 0.; }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
        if ((threadIdx.x & 31) == 0) ws[c][threadIdx.x >> 5] = v[c];
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.;
        for (int q = 0; q < CAT_WPB; ++q) t += ws[threadIdx.x][q];
        bsum[(size_t)blockIdx.x * 3 + threadIdx.x] = t;
    }
}

// One block: the means from the block sums (fixed order), into cs[0..2].
__global__ void __launch_bounds__(CAT_TOT) k_cat_mean(int nblk, int64_t n, const double* bsum,
                                                      double* cs)
{
    __shared__ double ds[3][CAT_TOT];
    const int t = threadIdx.x;
    const int per = (nblk + CAT_TOT - 1) / CAT_TOT;
    const int b0 = t * per, b1 = min(nblk, b0 + per);
    double s0 = 0., s1 = 0., s2 = 0.;
    for (int b = b0; b < b1; ++b) { s0 += bsum[3 * b]; s1 += bsum[3 * b + 1]; s2 += bsum[3 * b + 2]; }
    ds[0][t] = s0; ds[1][t] = s1; ds[2][t] = s2;
    __syncthreads();
    if (t < 3) {
        double S = 0.;
        for (int q = 0; q < CAT_TOT; ++q) S += ds[t][q];
        cs[t] = S / (double)n;
    }
}

// The largest squared distance from the mean (an order-free maximum, as non-negative
// doubles compared through their bit patterns).
__global__ void __launch_bounds__(CAT_TPB) k_cat_maxd(int64_t n, const double* x, const double* y,
                                                      const double* z, const double* cs,
                                                      unsigned long long* dmax)
{
    const int64_t i = (int64_t)blockIdx.x * CAT_TPB + threadIdx.x;
    double d = 0.;
    if (i < n) {
        const double dx = x[i] - cs[0], dy = y[i] - cs[1];
        d = dx * dx + dy * dy;
        if (z) { const double dz = z[i] - cs[2]; d += dz * dz; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d = fmax(d, __shfl_xor_sync(0xffffffffu, d, o));
    if ((threadIdx.x & 31) == 0) atomicMax(dmax, (unsigned long long)__double_as_longlong(d));
}

}  // namespace

int catalog_center_size_device(int64_t n, const double* x, const double* y, const double* z,
                               cudaStream_t st, double out[4])
{
    out[0] = out[1] = out[2] = out[3] = 0.;
    if (n <= 0 || !x || !y) { set_last_error("catalog centre: n > 0 and x, y needed"); return TC_ERR_ARG; }
    const int64_t nblk64 = (n + CAT_TPB - 1) / CAT_TPB;
    if (nblk64 > (int64_t)0x7fffffff) { set_last_error("catalog: too many rows"); return TC_ERR_ARG; }
    const int nblk = (int)nblk64;
    double* bsum = nullptr;
    double* cs = nullptr;
    unsigned long long* dmax = nullptr;
    int rc = 0;
    if ((rc = dalloc(&bsum, (size_t)nblk * 3)) || (rc = dalloc(&cs, 3)) || (rc = dalloc(&dmax, 1))) {
        dfree(bsum); dfree(cs); dfree(dmax);
        return rc;
    }
    double hc[3] = {0., 0., 0.};
    unsigned long long hm = 0;
    cudaError_t e = cudaMemsetAsync(dmax, 0, sizeof(unsigned long long), st);
    if (e == cudaSuccess) {
        count_launch();
        k_cat_sums<<<nblk, CAT_TPB, 0, st>>>(n, x, y, z, bsum);
        count_launch();
        k_cat_mean<<<1, CAT_TOT, 0, st>>>(nblk, n, bsum, cs);
        count_launch();
        k_cat_maxd<<<nblk, CAT_TPB, 0, st>>>(n, x, y, z, cs, dmax);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc, cs, 3 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hm, dmax, sizeof(hm), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dfree(bsum); dfree(cs); dfree(dmax);
    if (e != cudaSuccess) {
        set_last_error(std::string("catalog centre: ") + cudaGetErrorString(e));
        return TC_ERR_CUDA;
    }
    out[0] = hc[0]; out[1] = hc[1]; out[2] = z ? hc[2] : 0.;
    double dm;
    std::memcpy(&dm, &hm, sizeof(dm));
    out[3] = std::sqrt(dm);
    return TC_OK;
}

int catalog_finish_device(int64_t n, int ncols, double* const* cols, double* w, double* wpos,
                          const int64_t* flag, int64_t ignore_flag, int w_given,
                          int keep_zero_weight, cudaStream_t st, tc_catalog_info* out)
{
    *out = tc_catalog_info();
    if (n < 0 || ncols < 0 || ncols > TC_CAT_MAXCOLS || (ncols > 0 && !cols) || (n > 0 && !w)) {
        set_last_error("catalog: bad arguments (n >= 0, 0 <= ncols <= TC_CAT_MAXCOLS, w needed)");
        return TC_ERR_ARG;
    }
    CatCols C{};
    for (int c = 0; c < ncols; ++c) {
        if (n > 0 && !cols[c]) { set_last_error("catalog: NULL column"); return TC_ERR_ARG; }
        C.p[c] = cols[c];
    }
    if (n == 0) {
        out->nontrivial_w = (w_given || flag) ? 1 : 0;
        if (out->nontrivial_w) { set_last_error("Catalog has invalid sumw == 0"); return TC_ERR_ARG; }
        return TC_OK;
    }
    const int64_t nblk64 = (n + CAT_TPB - 1) / CAT_TPB;
    if (nblk64 > (int64_t)0x7fffffff) { set_last_error("catalog: too many rows"); return TC_ERR_ARG; }
    const int nblk = (int)nblk64;
    const int nc = ncols + 4;
    unsigned long long* counts = nullptr;
    double* bsum = nullptr;
    int* bkeep = nullptr;
    int* bnz = nullptr;
    int64_t* boff = nullptr;
    unsigned char* keep = nullptr;
    double* tot = nullptr;
    long long* itot = nullptr;
    double* tmp = nullptr;
    int rc = 0;
    auto cleanup = [&]() {
        dfree(counts); dfree(bsum); dfree(bkeep); dfree(bnz); dfree(boff); dfree(keep);
        dfree(tot); dfree(itot); dfree(tmp);
    };
    if ((rc = dalloc(&counts, nc)) || (rc = dalloc(&bsum, nblk)) || (rc = dalloc(&bkeep, nblk)) ||
        (rc = dalloc(&bnz, nblk)) || (rc = dalloc(&boff, nblk)) || (rc = dalloc(&keep, n)) ||
        (rc = dalloc(&tot, 1)) || (rc = dalloc(&itot, 2))) {
        cleanup();
        return rc;
    }
    std::vector<unsigned long long> hc(nc);
    double hs = 0.;
    long long hi[2] = {0, 0};
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(unsigned long long) * nc, st);
    if (e == cudaSuccess) {
        count_launch();
        k_cat_mark<<<nblk, CAT_TPB, 0, st>>>(n, ncols, C, w, wpos, flag, ignore_flag, w_given, counts,
                                        bsum, bkeep, bnz, keep);
        count_launch();
        k_cat_total<<<1, CAT_TOT, 0, st>>>(nblk, bsum, bkeep, bnz, boff, tot, itot);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc.data(), counts, sizeof(unsigned long long) * nc, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, tot, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hi, itot, 2 * sizeof(long long), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_last_error(std::string("catalog ingestion: ") + cudaGetErrorString(e));
        cleanup();
        return TC_ERR_CUDA;
    }
    long long nans = 0;
    for (int c = 0; c < ncols + 2; ++c) {
        out->nan_counts[c] = (int64_t)hc[c];
        nans += (long long)hc[c];
    }
    out->wpos_zero = (int64_t)hc[ncols + 2];
    out->wpos_conflicts = (int64_t)hc[ncols + 3];
    const bool nontrivial = w_given || flag || nans > 0 || (wpos && out->wpos_zero > 0);
    out->nontrivial_w = nontrivial ? 1 : 0;
    out->sumw = nontrivial ? hs : (double)n;
    out->nobj = nontrivial ? (int64_t)hi[1] : n;
    out->nkeep = n;
    if (nontrivial && out->sumw == 0.) {
        set_last_error("Catalog has invalid sumw == 0");
        cleanup();
        return TC_ERR_ARG;
    }
    const int64_t nkeep = (int64_t)hi[0];
    if (nontrivial && !keep_zero_weight && nkeep < n) {
        if ((rc = dalloc(&tmp, n))) { cleanup(); return rc; }
        std::vector<double*> all(cols, cols + ncols);
        all.push_back(w);
        if (wpos) all.push_back(wpos);
        for (double* col : all) {
            count_launch();
            k_cat_scatter<<<nblk, CAT_TPB, 0, st>>>(n, col, tmp, keep, boff);
            e = cudaGetLastError();
            if (e == cudaSuccess && nkeep > 0)
                e = cudaMemcpyAsync(col, tmp, sizeof(double) * nkeep, cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) break;
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            set_last_error(std::string("catalog compaction: ") + cudaGetErrorString(e));
            cleanup();
            return TC_ERR_CUDA;
        }
        out->nkeep = nkeep;
    }
    cleanup();
    return TC_OK;
}

}  // namespace tc
