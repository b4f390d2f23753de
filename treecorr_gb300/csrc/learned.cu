// learned.cu -- training and evaluation kernels of the learned opening criterion, and the
// labels of its training pairs.  No reference counterpart (see learned.cuh).
//
//   * k_learn_label: for cell pairs the bin_slop rule splits (sampled by the traversal),
//     the exact contribution is recomputed point pair by point pair and compared with the
//     accepted one: target = log10(leak + 1e-5), leak = the weight fraction of the point
//     pairs whose bin differs from the bin of the cells' separation (out of range counts
//     as a different bin).  One warp per pair.
//   * k_mlp_grad: forward and backward of the 5-64-64-1 ReLU network for a mean squared
//     error, FP32, 64 samples per block; the block's weight gradients are formed from the
//     staged activations in shared memory and added with one atomic per parameter.
//   * k_mlp_adam: Adam step.
//   * k_mlp_pack: FP32 master parameters -> FP16 mma fragments (MLPPacked).
//   * k_mlp_infer: the traversal's warp evaluation over a batch (to test it).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "tc_internal.cuh"
#include "tc_host.hpp"
#include "learned.cuh"
#include "learned.hpp"

namespace tc {

// ---------------------------------------------------------------------------------------
// Packing.

__global__ void k_mlp_pack(const float* P, MLPPacked* W)
{
    const float* W1 = P;
    const float* W2 = P + MLP_OFF_W2;
    for (int idx = threadIdx.x; idx < 8 * 32; idx += blockDim.x) {
        const int nt = idx >> 5, lane = idx & 31, g = lane >> 2, t = lane & 3;
        const int n = nt * 8 + g, k0 = 2 * t, k1 = 2 * t + 1;
        W->w1f[nt][lane] = pack_half2(k0 < MLP_IN ? W1[n * MLP_IN + k0] : 0.f,
                                      k1 < MLP_IN ? W1[n * MLP_IN + k1] : 0.f);
    }
    for (int idx = threadIdx.x; idx < 4 * 8 * 32; idx += blockDim.x) {
        const int kt = idx >> 8, nt = (idx >> 5) & 7, lane = idx & 31, g = lane >> 2, t = lane & 3;
        const int n = nt * 8 + g, k = kt * 16 + 2 * t;
        W->w2f[kt][nt][lane] = make_uint2(pack_half2(W2[n * MLP_H + k], W2[n * MLP_H + k + 1]),
                                          pack_half2(W2[n * MLP_H + k + 8], W2[n * MLP_H + k + 9]));
    }
    for (int i = threadIdx.x; i < MLP_H; i += blockDim.x) {
        W->b1[i] = P[MLP_OFF_B1 + i];
        W->b2[i] = P[MLP_OFF_B2 + i];
        W->w3[i] = P[MLP_OFF_W3 + i];
    }
    if (threadIdx.x == 0) { W->b3 = P[MLP_OFF_B3]; W->pad[0] = W->pad[1] = W->pad[2] = 0.f; }
}

// ---------------------------------------------------------------------------------------
// Training.

static constexpr int GB = 64;   // samples per gradient block

__global__ void __launch_bounds__(GB) k_mlp_grad(const float* P, const float* X, const float* Y,
                                                 const int* idx, long long off, long long bsz,
                                                 float inv_count, float* grad, float* loss)
{
    extern __shared__ float gs[];
    float* sW2 = gs;                           // 64 x 64
    float* sW1 = sW2 + MLP_H * MLP_H;          // 64 x 5
    float* sb1 = sW1 + MLP_H * MLP_IN;
    float* sb2 = sb1 + MLP_H;
    float* sw3 = sb2 + MLP_H;
    float* h1s = sw3 + MLP_H;                  // [GB][64] activations and deltas
    float* h2s = h1s + GB * MLP_H;
    float* d2s = h2s + GB * MLP_H;
    float* d1s = d2s + GB * MLP_H;
    float* xs = d1s + GB * MLP_H;              // [GB][5]
    float* dys = xs + GB * MLP_IN;             // [GB]
    const int tid = threadIdx.x;
    for (int q = tid; q < MLP_H * MLP_H; q += GB) sW2[q] = P[MLP_OFF_W2 + q];
    for (int q = tid; q < MLP_H * MLP_IN; q += GB) sW1[q] = P[q];
    for (int q = tid; q < MLP_H; q += GB) {
        sb1[q] = P[MLP_OFF_B1 + q]; sb2[q] = P[MLP_OFF_B2 + q]; sw3[q] = P[MLP_OFF_W3 + q];
    }
    __syncthreads();
    const long long s = off + (long long)blockIdx.x * GB + tid;
    const bool valid = s < off + bsz;
    float x[MLP_IN];
    float t = 0.f;
    if (valid) {
        const long long r = idx ? idx[s] : s;
#pragma unroll
        for (int k = 0; k < MLP_IN; ++k) x[k] = X[r * MLP_IN + k];
        t = Y[r];
    } else {
#pragma unroll
        for (int k = 0; k < MLP_IN; ++k) x[k] = 0.f;
    }
    float* h1 = h1s + tid * MLP_H;
    float* h2 = h2s + tid * MLP_H;
    float* d2 = d2s + tid * MLP_H;
    float* d1 = d1s + tid * MLP_H;
    for (int i = 0; i < MLP_H; ++i) {
        float a = sb1[i];
#pragma unroll
        for (int k = 0; k < MLP_IN; ++k) a += sW1[i * MLP_IN + k] * x[k];
        h1[i] = fmaxf(a, 0.f);
    }
    float y = P[MLP_OFF_B3];
    for (int j = 0; j < MLP_H; ++j) {
        float a = sb2[j];
        for (int i = 0; i < MLP_H; ++i) a += sW2[j * MLP_H + i] * h1[i];
        h2[j] = fmaxf(a, 0.f);
        y += sw3[j] * h2[j];
    }
    const float e = valid ? (y - t) : 0.f;
    const float dy = 2.f * e * inv_count;
    for (int j = 0; j < MLP_H; ++j) d2[j] = h2[j] > 0.f ? dy * sw3[j] : 0.f;
    for (int i = 0; i < MLP_H; ++i) {
        float a = 0.f;
        for (int j = 0; j < MLP_H; ++j) a += sW2[j * MLP_H + i] * d2[j];
        d1[i] = h1[i] > 0.f ? a : 0.f;
    }
#pragma unroll
    for (int k = 0; k < MLP_IN; ++k) xs[tid * MLP_IN + k] = x[k];
    dys[tid] = dy;
    // Loss: block sum of e^2 / count.
    float l = e * e * inv_count;
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((tid & 31) == 0) atomicAdd(loss, l);
    __syncthreads();
    // Weight gradients of the block: sums over its samples.
    for (int q = tid; q < MLP_H * MLP_H; q += GB) {
        const int j = q / MLP_H, i = q % MLP_H;
        float a = 0.f;
        for (int u = 0; u < GB; ++u) a += d2s[u * MLP_H + j] * h1s[u * MLP_H + i];
        atomicAdd(&grad[MLP_OFF_W2 + q], a);
    }
    for (int q = tid; q < MLP_H * MLP_IN; q += GB) {
        const int i = q / MLP_IN, k = q % MLP_IN;
        float a = 0.f;
        for (int u = 0; u < GB; ++u) a += d1s[u * MLP_H + i] * xs[u * MLP_IN + k];
        atomicAdd(&grad[q], a);
    }
    for (int q = tid; q < MLP_H; q += GB) {
        float a1 = 0.f, a2 = 0.f, a3 = 0.f;
        for (int u = 0; u < GB; ++u) {
            a1 += d1s[u * MLP_H + q];
            a2 += d2s[u * MLP_H + q];
            a3 += dys[u] * h2s[u * MLP_H + q];
        }
        atomicAdd(&grad[MLP_OFF_B1 + q], a1);
        atomicAdd(&grad[MLP_OFF_B2 + q], a2);
        atomicAdd(&grad[MLP_OFF_W3 + q], a3);
    }
    if (tid == 0) {
        float a = 0.f;
        for (int u = 0; u < GB; ++u) a += dys[u];
        atomicAdd(&grad[MLP_OFF_B3], a);
    }
}

static size_t mlp_grad_smem()
{
    return sizeof(float) * ((size_t)MLP_H * MLP_H + MLP_H * MLP_IN + 3 * MLP_H +
                            4 * (size_t)GB * MLP_H + GB * MLP_IN + GB);
}

__global__ void k_mlp_adam(float* P, const float* grad, float* m, float* v, int n, float lr,
                           float beta1, float beta2, float eps, float bc1, float bc2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = grad[i];
    const float mi = beta1 * m[i] + (1.f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    P[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// ---------------------------------------------------------------------------------------
// Evaluation of the traversal's warp function over a batch (tests and threshold tuning).

__global__ void k_mlp_infer(const MLPPacked* Wg, const float* X, long long n, float* Y)
{
    __shared__ MLPPacked W;
    __shared__ __align__(16) __half sx[4][32 * 8];
    __shared__ float sy[4][32];
    for (int q = threadIdx.x; q < (int)(sizeof(MLPPacked) / 4); q += blockDim.x)
        reinterpret_cast<uint32_t*>(&W)[q] = reinterpret_cast<const uint32_t*>(Wg)[q];
    __syncthreads();
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long base = ((long long)blockIdx.x * 4 + wib) * 32;
    if (base >= n) return;                 // whole warps only: base is warp-uniform
    const long long s = base + lane;
    float x[MLP_IN];
#pragma unroll
    for (int k = 0; k < MLP_IN; ++k) x[k] = s < n ? X[s * MLP_IN + k] : 0.f;
    const float y = mlp_warp_eval(W, x, sx[wib], sy[wib]);
    if (s < n) Y[s] = y;
}

// ---------------------------------------------------------------------------------------
// Labels of sampled cell pairs.

__global__ void k_learn_label(LabelParams L, const int2* pairs, long long npairs, float* feat,
                              float* target)
{
    const int lane = threadIdx.x & 31;
    const long long p = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (p >= npairs) return;
    const int2 pr = pairs[p];
    const TCell A = L.c1[pr.x], B = L.c2[pr.y];
    const bool flat = L.coords == FLAT, arc = L.metric == ARC;
    // The cell pair's separation and features, as the traversal computes them.
    const float dx = (A.a.x - B.a.x) + (A.b.x - B.b.x);
    const float dy = (A.a.y - B.a.y) + (A.b.y - B.b.y);
    const float dz = flat ? 0.f : (A.a.z - B.a.z) + (A.b.z - B.b.z);
    const float dsq = dx * dx + dy * dy + dz * dz;
    float rsq = dsq;
    if (arc) { const float th = arc_from_chord_sq(dsq); rsq = th * th; }
    const float lr = 0.5f * logf(rsq * L.finvminsepsq);
    const int kc = (int)(lr * L.finvbinsize);
    const int n1 = __float_as_int(A.c.z), n2 = __float_as_int(B.c.z);
    const int st1 = L.start1[pr.x], st2 = L.start2[pr.y];
    bool ok = (long long)n1 * n2 <= L.max_point_pairs && kc >= 0 && kc < L.nbins;
    // Exact contribution: every point pair's bin.
    double wtot = 0., wleak = 0.;
    if (ok) {
        for (int a = 0; a < n1; ++a) {
            const int ia = st1 + a;
            const double xa = L.x1[ia], ya = L.y1[ia], za = flat ? 0. : L.z1[ia];
            const float wa = L.w1[ia];
            for (int b = lane; b < n2; b += 32) {
                const int ib = st2 + b;
                const double ex = xa - L.x2[ib], ey = ya - L.y2[ib], ez = flat ? 0. : za - L.z2[ib];
                double q = ex * ex + ey * ey + ez * ez;
                if (arc) { const double th = 2. * asin(0.5 * sqrt(q)); q = th * th; }
                const float wab = wa * L.w2[ib];
                int kb = -1;
                if (q >= L.minsepsq && q < L.maxsepsq) {
                    kb = (int)((0.5 * log(q) - L.logminsep) / L.binsize);
                    if (kb >= L.nbins) kb = L.nbins - 1;
                }
                wtot += wab;
                if (kb != kc) wleak += wab;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        wtot += __shfl_xor_sync(0xffffffffu, wtot, o);
        wleak += __shfl_xor_sync(0xffffffffu, wleak, o);
    }
    if (lane == 0) {
        float x[MLP_IN];
        mlp_features(A.a.w, B.a.w, sqrtf(rsq), lr, L.finvbinsize, L.finvlogrange, L.fbinsize, x);
#pragma unroll
        for (int k = 0; k < MLP_IN; ++k) feat[p * MLP_IN + k] = x[k];
        target[p] = (ok && wtot > 0.) ? (float)log10(wleak / wtot + 1e-5) : NAN;
    }
}

// ---------------------------------------------------------------------------------------
// Host.

int mlp_pack(const float* h_params, MLPPacked** d_out, cudaStream_t st)
{
    float* d = nullptr;
    TC_TRY(dalloc(&d, (size_t)MLP_NPARAM));
    if (!*d_out) TC_TRY(dalloc(d_out, 1));
    TC_CU(cudaMemcpyAsync(d, h_params, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice, st));
    count_launch();
    k_mlp_pack<<<1, 256, 0, st>>>(d, *d_out);
    TC_CU(cudaGetLastError());
    TC_CU(cudaStreamSynchronize(st));
    dfree(d);
    return 0;
}

int launch_label(const LabelParams& L, const int2* pairs, long long n, float* feat, float* target,
                 cudaStream_t st)
{
    if (n <= 0) return 0;
    count_launch();
    k_learn_label<<<(unsigned)((n * 32 + 127) / 128), 128, 0, st>>>(L, pairs, n, feat, target);
    TC_CU(cudaGetLastError());
    return 0;
}

static int grad_pass(const float* dP, const float* dX, const float* dY, const int* didx,
                     long long off, long long bsz, float* dgrad, float* dloss, cudaStream_t st)
{
    const size_t sm = mlp_grad_smem();
    static bool attr = false;
    if (!attr) {
        TC_CU(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        attr = true;
    }
    count_launch();
    k_mlp_grad<<<(unsigned)((bsz + GB - 1) / GB), GB, sm, st>>>(dP, dX, dY, didx, off, bsz,
                                                               1.f / (float)bsz, dgrad, dloss);
    TC_CU(cudaGetLastError());
    return 0;
}

int mlp_grad_host(const float* P, const float* X, const float* Y, long long n, float* grad,
                  float* loss, cudaStream_t st)
{
    float *dP = nullptr, *dX = nullptr, *dY = nullptr, *dg = nullptr, *dl = nullptr;
    int rc = 0;
    do {
        if ((rc = dalloc(&dP, (size_t)MLP_NPARAM))) break;
        if ((rc = dalloc(&dX, (size_t)n * MLP_IN))) break;
        if ((rc = dalloc(&dY, (size_t)n))) break;
        if ((rc = dalloc(&dg, (size_t)MLP_NPARAM))) break;
        if ((rc = dalloc(&dl, 1))) break;
        cudaMemcpyAsync(dP, P, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dX, X, sizeof(float) * n * MLP_IN, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dY, Y, sizeof(float) * n, cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(dg, 0, sizeof(float) * MLP_NPARAM, st);
        cudaMemsetAsync(dl, 0, sizeof(float), st);
        if ((rc = grad_pass(dP, dX, dY, nullptr, 0, n, dg, dl, st))) break;
        cudaMemcpyAsync(grad, dg, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(loss, dl, sizeof(float), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) { set_last_error("mlp gradient failed"); rc = 2; }
    } while (0);
    dfree(dP); dfree(dX); dfree(dY); dfree(dg); dfree(dl);
    return rc;
}

int mlp_infer_host(const float* P, const float* X, long long n, float* Y, cudaStream_t st)
{
    MLPPacked* W = nullptr;
    float *dX = nullptr, *dY = nullptr;
    int rc = 0;
    do {
        if ((rc = mlp_pack(P, &W, st))) break;
        if ((rc = dalloc(&dX, (size_t)std::max(n, 1LL) * MLP_IN))) break;
        if ((rc = dalloc(&dY, (size_t)std::max(n, 1LL)))) break;
        cudaMemcpyAsync(dX, X, sizeof(float) * n * MLP_IN, cudaMemcpyHostToDevice, st);
        count_launch();
        k_mlp_infer<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(W, dX, n, dY);
        if (cudaGetLastError() != cudaSuccess) { set_last_error("mlp inference launch failed"); rc = 2; break; }
        cudaMemcpyAsync(Y, dY, sizeof(float) * n, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) { set_last_error("mlp inference failed"); rc = 2; }
    } while (0);
    dfree(W); dfree(dX); dfree(dY);
    return rc;
}

int mlp_train_host(float* P, const float* X, const float* Y, long long n, int steps, int batch,
                   float lr, unsigned seed, float* loss_out, cudaStream_t st)
{
    float *dP = nullptr, *dX = nullptr, *dY = nullptr, *dg = nullptr, *dl = nullptr;
    float *dm = nullptr, *dv = nullptr;
    int* didx = nullptr;
    int rc = 0;
    const long long bsz = std::min<long long>(std::max(batch, GB), n);
    std::vector<int> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    std::mt19937 rng(seed);
    do {
        if ((rc = dalloc(&dP, (size_t)MLP_NPARAM))) break;
        if ((rc = dalloc(&dm, (size_t)MLP_NPARAM))) break;
        if ((rc = dalloc(&dv, (size_t)MLP_NPARAM))) break;
        if ((rc = dalloc(&dg, (size_t)MLP_NPARAM))) break;
        if ((rc = dalloc(&dl, (size_t)std::max(steps, 1)))) break;
        if ((rc = dalloc(&dX, (size_t)n * MLP_IN))) break;
        if ((rc = dalloc(&dY, (size_t)n))) break;
        if ((rc = dalloc(&didx, (size_t)n))) break;
        cudaMemcpyAsync(dP, P, sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dX, X, sizeof(float) * n * MLP_IN, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dY, Y, sizeof(float) * n, cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(dm, 0, sizeof(float) * MLP_NPARAM, st);
        cudaMemsetAsync(dv, 0, sizeof(float) * MLP_NPARAM, st);
        cudaMemsetAsync(dl, 0, sizeof(float) * std::max(steps, 1), st);
        long long pos = n;   // position in the current permutation
        const float b1 = 0.9f, b2 = 0.999f;
        for (int it = 0; it < steps && !rc; ++it) {
            if (pos + bsz > n) {   // new epoch: reshuffle
                std::shuffle(perm.begin(), perm.end(), rng);
                cudaMemcpyAsync(didx, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
                if (cudaStreamSynchronize(st) != cudaSuccess) { rc = 2; break; }
                pos = 0;
            }
            cudaMemsetAsync(dg, 0, sizeof(float) * MLP_NPARAM, st);
            if ((rc = grad_pass(dP, dX, dY, didx, pos, bsz, dg, dl + it, st))) break;
            pos += bsz;
            const float bc1 = 1.f - std::pow(b1, (float)(it + 1)), bc2 = 1.f - std::pow(b2, (float)(it + 1));
            count_launch();
            k_mlp_adam<<<(MLP_NPARAM + 255) / 256, 256, 0, st>>>(dP, dg, dm, dv, MLP_NPARAM, lr, b1, b2,
                                                              1e-8f, bc1, bc2);
            if (cudaGetLastError() != cudaSuccess) { set_last_error("adam launch failed"); rc = 2; }
        }
        if (rc) break;
        cudaMemcpyAsync(P, dP, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, st);
        if (loss_out) cudaMemcpyAsync(loss_out, dl, sizeof(float) * steps, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) { set_last_error("mlp training failed"); rc = 2; }
    } while (0);
    dfree(dP); dfree(dm); dfree(dv); dfree(dg); dfree(dl); dfree(dX); dfree(dY); dfree(didx);
    return rc;
}

}  // namespace tc
