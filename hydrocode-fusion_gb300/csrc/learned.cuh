// learned.cuh -- learned starting pressure for the exact Riemann solver.
//
// A 6 -> 64 -> 64 -> 1 ReLU MLP predicts y = log(p*/pbar) of a Riemann problem
// from scale-free features; the FP32 form starts its Newton iteration at
// p = pbar * exp(y) instead of the reference's half-linearised intersection
// (riemann_solver_exact_Ben.c:86-93), then polishes with Newton and falls
// back to the FP64 reference iteration when the polish does not converge.
//
//   features (pbar = sqrt(pL pR)):
//     x0 = +lr/4.6, x1 = -lr/4.6   lr = log(rhoL/rhoR)/2
//     x2 = +lp/4.6, x3 = -lp/4.6   lp = log(pL/pR)/2
//     x4 = asinh((uR-uL)/cL)/4, x5 = asinh((uR-uL)/cR)/4
//
// Inference is warp-cooperative on the tensor cores: each lane brings the
// features of its own interface, the warp runs two 16-row M tiles of
// mma.sync.m16n8k16 (BF16 inputs and weights, FP32 accumulation); the output
// fragment of one layer is already the input fragment of the next (bias and
// ReLU applied in registers), so no shared-memory round trip is needed.  A
// 64x64 layer is far too small for tcgen05/TMEM to pay off inside the flux
// kernel.  Weights live in shared memory pre-swizzled in fragment order.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/hydro_gb300.h"

namespace hydro {

constexpr int MLP_IN = 6, MLP_H = 64;
constexpr int MLP_NPARAM = MLP_H * MLP_IN + MLP_H + MLP_H * MLP_H + MLP_H + MLP_H + 1;  // 4673
static_assert(MLP_NPARAM == HYDRO_MLP_NPARAM, "parameter count of the C ABI");
// offsets in the flat FP32 parameter vector
constexpr int MLP_W1 = 0, MLP_B1 = MLP_W1 + MLP_H * MLP_IN, MLP_W2 = MLP_B1 + MLP_H,
              MLP_B2 = MLP_W2 + MLP_H * MLP_H, MLP_W3 = MLP_B2 + MLP_H, MLP_B3 = MLP_W3 + MLP_H;
// fragment buffer (uint32 words): layer 1 [8 ntile][32 lane][2], layer 2 [4 kc][8 nt][32][2], layer 3 [4 kc][32][2]
constexpr int MLP_F1 = 0, MLP_F2 = MLP_F1 + 8 * 32 * 2, MLP_F3 = MLP_F2 + 4 * 8 * 32 * 2, MLP_NFRAG = MLP_F3 + 4 * 32 * 2;
constexpr float MLP_LSCALE = 1.0f / 4.6f, MLP_USCALE = 0.25f;

__device__ __host__ inline float mlp_asinh(float v)
{
    float a = fabsf(v);
    float r = logf(a + sqrtf(a * a + 1.0f));
    return v < 0.f ? -r : r;
}

// Features of a Riemann problem; returns pbar.
__device__ __host__ inline float mlp_features(float rL, float uL, float pL, float cL, float rR, float uR, float pR,
                                              float cR, float x[6])
{
    float lr = 0.5f * logf(rL / rR), lp = 0.5f * logf(pL / pR);
    float du = uR - uL;
    x[0] = lr * MLP_LSCALE;
    x[1] = -lr * MLP_LSCALE;
    x[2] = lp * MLP_LSCALE;
    x[3] = -lp * MLP_LSCALE;
    x[4] = mlp_asinh(du / cL) * MLP_USCALE;
    x[5] = mlp_asinh(du / cR) * MLP_USCALE;
    return sqrtf(pL * pR);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma16816(float d[4], const uint32_t a[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Builds the fragment-ordered BF16 weights from the FP32 parameter vector.
// B[k][n] = W[n][k] (y = W x); lane (g = lane/4, t = lane%4) of n-tile nt,
// k-chunk kc holds {W[nt*8+g][kc*16+2t], [..+1]} and {[..+8], [..+9]}.
static __global__ void k_mlp_pack(const float* __restrict__ prm, uint32_t* __restrict__ frag)
{
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= 8 * 32 + 4 * 8 * 32 + 4 * 32)
        return;
    auto w = [&](int layer, int n, int k) -> float {
        if (layer == 1)
            return (k < MLP_IN) ? prm[MLP_W1 + n * MLP_IN + k] : 0.f;
        if (layer == 2)
            return prm[MLP_W2 + n * MLP_H + k];
        return (n == 0) ? prm[MLP_W3 + k] : 0.f;
    };
    int layer, kc, nt, lane;
    uint32_t* dst;
    if (tid < 8 * 32) {
        layer = 1; kc = 0; nt = tid / 32; lane = tid % 32;
        dst = frag + MLP_F1 + (nt * 32 + lane) * 2;
    } else if (tid < 8 * 32 + 4 * 8 * 32) {
        int r = tid - 8 * 32;
        layer = 2; kc = r / (8 * 32); nt = (r / 32) % 8; lane = r % 32;
        dst = frag + MLP_F2 + ((kc * 8 + nt) * 32 + lane) * 2;
    } else {
        int r = tid - 8 * 32 - 4 * 8 * 32;
        layer = 3; kc = r / 32; nt = 0; lane = r % 32;
        dst = frag + MLP_F3 + (kc * 32 + lane) * 2;
    }
    const int g = lane >> 2, t = lane & 3, n = nt * 8 + g, k0 = kc * 16 + 2 * t;
    dst[0] = pack_bf16(w(layer, n, k0), w(layer, n, k0 + 1));
    dst[1] = pack_bf16(w(layer, n, k0 + 8), w(layer, n, k0 + 9));
}

// Shared-memory image of the network used by the kernels.
struct MlpShared {
    uint32_t frag[MLP_NFRAG];
    float b1[MLP_H], b2[MLP_H], b3;
};

__device__ __forceinline__ void mlp_load_shared(MlpShared& S, const uint32_t* __restrict__ frag,
                                                const float* __restrict__ prm, int tid, int nthreads)
{
    for (int q = tid; q < MLP_NFRAG; q += nthreads)
        S.frag[q] = frag[q];
    for (int q = tid; q < MLP_H; q += nthreads) {
        S.b1[q] = prm[MLP_B1 + q];
        S.b2[q] = prm[MLP_B2 + q];
    }
    if (tid == 0)
        S.b3 = prm[MLP_B3];
}

// The shared-memory image of the network built once in global memory, for
// kernels that read it through L1 instead of staging it (one block).
static __global__ void k_mlp_image(const uint32_t* __restrict__ frag, const float* __restrict__ prm,
                                   MlpShared* __restrict__ img)
{
    mlp_load_shared(*img, frag, prm, threadIdx.x, blockDim.x);
}

__device__ __forceinline__ float relu(float v) { return v > 0.f ? v : 0.f; }

// Warp-cooperative forward pass: all 32 lanes call it with their own features
// (garbage is fine for lanes that do not need the result); returns this lane's
// output.  rows (warp-uniform): only lanes below it need a result; with 16 or
// fewer the second 16-row tile of the mma is skipped (its rows are independent
// of the first's, so the results of lanes 0-15 do not change).
__device__ __forceinline__ float warp_mlp(const float x[6], const MlpShared& S, int rows = 32)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float mine = 0.f;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        if (mt == 1 && rows <= 16)
            break;
        // layer-1 A fragment: rows g and g+8 of this M tile, columns 2t and 2t+1 (6 and 7 are padding)
        const int s0 = mt * 16 + g, s1 = s0 + 8;
        float f0[6], f1[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            f0[k] = __shfl_sync(FULL, x[k], s0);
            f1[k] = __shfl_sync(FULL, x[k], s1);
        }
        float a0 = (t == 0) ? f0[0] : (t == 1) ? f0[2] : (t == 2) ? f0[4] : 0.f;
        float a1 = (t == 0) ? f0[1] : (t == 1) ? f0[3] : (t == 2) ? f0[5] : 0.f;
        float a2 = (t == 0) ? f1[0] : (t == 1) ? f1[2] : (t == 2) ? f1[4] : 0.f;
        float a3 = (t == 0) ? f1[1] : (t == 1) ? f1[3] : (t == 2) ? f1[5] : 0.f;
        const uint32_t A1[4] = {pack_bf16(a0, a1), pack_bf16(a2, a3), 0u, 0u};
        // layer 1 -> layer-2 A fragments
        uint32_t A2[4][4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int nt = 2 * q + h;
                float c[4] = {0.f, 0.f, 0.f, 0.f};
                mma16816(c, A1, S.frag[MLP_F1 + (nt * 32 + lane) * 2], S.frag[MLP_F1 + (nt * 32 + lane) * 2 + 1]);
                const float bb0 = S.b1[nt * 8 + 2 * t], bb1 = S.b1[nt * 8 + 2 * t + 1];
                A2[q][2 * h] = pack_bf16(relu(c[0] + bb0), relu(c[1] + bb1));
                A2[q][2 * h + 1] = pack_bf16(relu(c[2] + bb0), relu(c[3] + bb1));
            }
        }
        // layer 2 -> layer-3 A fragments, two n-tiles (one k-chunk of layer 3) at a time
        uint32_t A3[4][4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int nt = 2 * q + h;
                float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int kc = 0; kc < 4; ++kc) {
                    const int o = MLP_F2 + ((kc * 8 + nt) * 32 + lane) * 2;
                    mma16816(c, A2[kc], S.frag[o], S.frag[o + 1]);
                }
                const float bb0 = S.b2[nt * 8 + 2 * t], bb1 = S.b2[nt * 8 + 2 * t + 1];
                A3[q][2 * h] = pack_bf16(relu(c[0] + bb0), relu(c[1] + bb1));
                A3[q][2 * h + 1] = pack_bf16(relu(c[2] + bb0), relu(c[3] + bb1));
            }
        }
        // layer 3 (n-tile 0, column 0 meaningful)
        float o3[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kc = 0; kc < 4; ++kc)
            mma16816(o3, A3[kc], S.frag[MLP_F3 + (kc * 32 + lane) * 2], S.frag[MLP_F3 + (kc * 32 + lane) * 2 + 1]);
        // row r of this tile sits in lane 4*(r%8): o3[0] for r < 8, o3[2] for r >= 8
        const int src = 4 * (lane & 7);
        const float v0 = __shfl_sync(FULL, o3[0], src);
        const float v2 = __shfl_sync(FULL, o3[2], src);
        if ((lane >> 4) == mt)
            mine = (((lane & 15) < 8) ? v0 : v2) + S.b3;
    }
    return mine;
}

// The same forward pass out of line, for the step kernels: its fragment
// registers then do not add to the register pressure of the whole tile code
// (the network runs on a small fraction of the faces).  All 32 lanes call it.
static __device__ __noinline__ float warp_mlp_outline(float x0, float x1, float x2, float x3, float x4, float x5,
                                                      const MlpShared* S, int rows)
{
    const float x[6] = {x0, x1, x2, x3, x4, x5};
    return warp_mlp(x, *S, rows);
}

}  // namespace hydro
