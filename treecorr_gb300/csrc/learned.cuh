// learned.cuh -- the learned opening criterion: a 5-64-64-1 MLP evaluated by one warp for
// its 32 lanes' cell pairs inside the traversal (FP16 weights and activations, FP32
// accumulation, mma.sync m16n8k16), and the features it reads.
//
// No reference counterpart: TreeCorr decides with the bin_slop rule alone
// (BinTypeHelper<Log>::singleBin, include/BinType.h:93-151).  The learned criterion only
// revisits pairs that rule would split; the rule stays the fallback for everything else.
#pragma once

#include <cuda_fp16.h>
#include <cstdint>

namespace tc {

static constexpr int MLP_IN = 5, MLP_H = 64;
// FP32 master parameters, in this order: W1[64][5], b1[64], W2[64][64], b2[64], w3[64], b3.
static constexpr int MLP_NPARAM = MLP_H * MLP_IN + MLP_H + MLP_H * MLP_H + MLP_H + MLP_H + 1;
static constexpr int MLP_OFF_B1 = MLP_H * MLP_IN;
static constexpr int MLP_OFF_W2 = MLP_OFF_B1 + MLP_H;
static constexpr int MLP_OFF_B2 = MLP_OFF_W2 + MLP_H * MLP_H;
static constexpr int MLP_OFF_W3 = MLP_OFF_B2 + MLP_H;
static constexpr int MLP_OFF_B3 = MLP_OFF_W3 + MLP_H;

// Weights packed in mma fragment order (built once on the device from the FP32 master):
//   w1f[nt][lane]        layer-1 B fragment (k = input 2t, 2t+1; n = nt*8 + g), 8 x 32 u32
//   w2f[kt][nt][lane]    layer-2 B fragments (two u32 per lane), 4 x 8 x 32 uint2
//   b1, b2, w3 (FP32), b3
struct MLPPacked {
    uint32_t w1f[8][32];
    uint2 w2f[4][8][32];
    float b1[MLP_H], b2[MLP_H], w3[MLP_H];
    float b3;
    float pad[3];
};

// Features of a cell pair (sizes s1, s2, separation r on the metric's scale): the larger
// and smaller size over the bin width at r (r * bin_size), the distance of log(r) to the
// nearest bin edge in units of the bin size, the position of log(r) in the binned range,
// and the bin size.
__device__ __forceinline__ void mlp_features(float s1, float s2, float r, float logr_minsep,
                                             float inv_binsize, float inv_logrange,
                                             float binsize, float (&x)[MLP_IN])
{
    const float sb = fmaxf(s1, s2), ss = fminf(s1, s2);
    const float wbin = fmaxf(r * binsize, 1e-30f);
    const float kk = logr_minsep * inv_binsize;
    const float fr = kk - floorf(kk);
    x[0] = sb / wbin;
    x[1] = ss / wbin;
    x[2] = fminf(fr, 1.f - fr);
    x[3] = logr_minsep * inv_logrange;
    x[4] = binsize;
}

__device__ __forceinline__ uint32_t pack_half2(float a, float b)
{
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

__device__ __forceinline__ void mma16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// The MLP for the 32 lanes of a warp: lane l's features x give its output, returned to
// lane l.  sx: 32 x 8 halves of warp-private shared memory; sy: 32 floats.  All 32 lanes
// must call it (the mma instructions are warp-collective).
__device__ __forceinline__ float mlp_warp_eval(const MLPPacked& W, const float (&x)[MLP_IN],
                                               __half* sx, float* sy)
{
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int c = 0; c < 8; ++c) sx[lane * 8 + c] = __float2half(c < MLP_IN ? x[c] : 0.f);
    __syncwarp();
    // Layer-1 A fragments (rows = samples of m-tile mt, cols = inputs 0..15; cols >= 8 are 0).
    uint32_t xa[2][2];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        const __half* r0 = sx + (mt * 16 + g) * 8 + 2 * t;
        const __half* r1 = sx + (mt * 16 + g + 8) * 8 + 2 * t;
        xa[mt][0] = *reinterpret_cast<const uint32_t*>(r0);
        xa[mt][1] = *reinterpret_cast<const uint32_t*>(r1);
    }
    // Layer 1 -> relu -> FP16 A fragments of layer 2 (k-tile kt = n-tiles 2kt, 2kt+1).
    uint32_t ha[2][4][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float bl = W.b1[nt * 8 + 2 * t], bh = W.b1[nt * 8 + 2 * t + 1];
        const uint32_t b0 = W.w1f[nt][lane];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            float d[4] = {bl, bh, bl, bh};
            mma16816(d, xa[mt][0], xa[mt][1], 0u, 0u, b0, 0u);
            const uint32_t lo = pack_half2(fmaxf(d[0], 0.f), fmaxf(d[1], 0.f));
            const uint32_t hi = pack_half2(fmaxf(d[2], 0.f), fmaxf(d[3], 0.f));
            ha[mt][nt >> 1][(nt & 1) * 2 + 0] = lo;
            ha[mt][nt >> 1][(nt & 1) * 2 + 1] = hi;
        }
    }
    // Layer 2 -> relu -> dot with w3 (FP32).
    float y0[2] = {0.f, 0.f}, y1[2] = {0.f, 0.f};   // rows g and g+8 of each m-tile
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float bl = W.b2[nt * 8 + 2 * t], bh = W.b2[nt * 8 + 2 * t + 1];
        const float wl = W.w3[nt * 8 + 2 * t], wh = W.w3[nt * 8 + 2 * t + 1];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            float d[4] = {bl, bh, bl, bh};
#pragma unroll
            for (int kt = 0; kt < 4; ++kt) {
                const uint2 b = W.w2f[kt][nt][lane];
                mma16816(d, ha[mt][kt][0], ha[mt][kt][1], ha[mt][kt][2], ha[mt][kt][3], b.x, b.y);
            }
            y0[mt] += fmaxf(d[0], 0.f) * wl + fmaxf(d[1], 0.f) * wh;
            y1[mt] += fmaxf(d[2], 0.f) * wl + fmaxf(d[3], 0.f) * wh;
        }
    }
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        y0[mt] += __shfl_xor_sync(0xffffffffu, y0[mt], 1);
        y0[mt] += __shfl_xor_sync(0xffffffffu, y0[mt], 2);
        y1[mt] += __shfl_xor_sync(0xffffffffu, y1[mt], 1);
        y1[mt] += __shfl_xor_sync(0xffffffffu, y1[mt], 2);
        if (t == 0) {
            sy[mt * 16 + g] = y0[mt] + W.b3;
            sy[mt * 16 + g + 8] = y1[mt] + W.b3;
        }
    }
    __syncwarp();
    const float y = sy[lane];
    __syncwarp();
    return y;
}

}  // namespace tc
