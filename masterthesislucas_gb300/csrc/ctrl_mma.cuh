// The controller network on the tensor cores, one warp per 32 rows: BF16
// mma.sync m16n8k16 with FP32 accumulation, each layer's accumulator
// fragments re-packed in registers as the next layer's A operand (bias and
// ReLU in FP32, inputs and hidden activations rounded to BF16).  Fragment
// layouts (PTX ISA, mma.m16n8k16 with .bf16): g = lane / 4, q = lane % 4;
// A regs {row g, cols 2q..2q+1}, {row g+8, same}, {row g, cols 8+2q..},
// {row g+8, cols 8+2q..}; B regs {k 2q..2q+1, col g}, {k 8+2q.., col g};
// C {row g, cols 2q, 2q+1}, {row g+8, cols 2q, 2q+1}.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace tc {
namespace ctrl {

constexpr int kW1S = 24;  // padded row length (bf16) of W1 [64][16]: conflict-free fragment loads
constexpr int kW2S = 72;  // padded row length of W2 [64][64] and W3 [8][64]
constexpr int kXS = 24;   // padded row of the per-warp feature tile [32][16]
constexpr int kWarps = 4;
constexpr uint8_t kOpen = 0xFF;

struct Smem {
    __nv_bfloat16 w1[TC_MLP_HIDDEN * kW1S];
    __nv_bfloat16 w2[TC_MLP_HIDDEN * kW2S];
    __nv_bfloat16 w3[8 * kW2S];
    float b1[TC_MLP_HIDDEN], b2[TC_MLP_HIDDEN], b3[8];
    float mean[TC_MLP_IN], istd[TC_MLP_IN];
    __nv_bfloat16 x[kWarps][32 * kXS];
    float y[kWarps][32 * 8];
};

__device__ inline uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x (low half) = lo
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ inline uint32_t lds32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ inline void mma16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// weights (FP32 values already representable in BF16), biases and the
// input normalisation into shared memory
__device__ inline void load_weights(Smem& S, const float* __restrict__ w, const float* __restrict__ mean,
                                    const float* __restrict__ stdv)
{
    constexpr int NI = TC_MLP_IN, NH = TC_MLP_HIDDEN, NO = TC_MLP_OUT;
    const float* W2 = w + NH * NI + NH;
    const float* B2 = W2 + NH * NH;
    const float* W3 = B2 + NH;
    const float* B3 = W3 + NO * NH;
    for (int i = threadIdx.x; i < NH * NI; i += blockDim.x) S.w1[(i / NI) * kW1S + i % NI] = __float2bfloat16(w[i]);
    for (int i = threadIdx.x; i < NH * NH; i += blockDim.x) S.w2[(i / NH) * kW2S + i % NH] = __float2bfloat16(W2[i]);
    for (int i = threadIdx.x; i < 8 * NH; i += blockDim.x)
        S.w3[(i / NH) * kW2S + i % NH] = __float2bfloat16(i < NO * NH ? W3[i] : 0.f);
    for (int i = threadIdx.x; i < NH; i += blockDim.x) {
        S.b1[i] = w[NH * NI + i];
        S.b2[i] = B2[i];
    }
    for (int i = threadIdx.x; i < 8; i += blockDim.x) S.b3[i] = i < NO ? B3[i] : 0.f;
    for (int i = threadIdx.x; i < NI; i += blockDim.x) {
        S.mean[i] = mean[i];
        S.istd[i] = 1.0f / stdv[i];
    }
}

// The MLP on the 32 rows of the warp (row = lane); all lanes must call it.
// Returns this lane's 5 outputs in y.
__device__ inline void warp_mlp(Smem& S, int wid, int lane, const float* f, bool use, float* y)
{
    __nv_bfloat16* X = S.x[wid];
    float* Y = S.y[wid];
#pragma unroll
    for (int k = 0; k < TC_MLP_IN; k += 2) {
        const float x0 = use ? (f[k] - S.mean[k]) * S.istd[k] : 0.f;
        const float x1 = use ? (f[k + 1] - S.mean[k + 1]) * S.istd[k + 1] : 0.f;
        *reinterpret_cast<uint32_t*>(X + lane * kXS + k) = pack_bf16(x0, x1);
    }
    __syncwarp();
    const int g = lane >> 2, q = lane & 3;
#pragma unroll 1
    for (int t = 0; t < 2; t++) {
        const int r0 = 16 * t + g, r1 = r0 + 8;
        const uint32_t a0 = lds32(X + r0 * kXS + 2 * q), a1 = lds32(X + r1 * kXS + 2 * q);
        const uint32_t a2 = lds32(X + r0 * kXS + 8 + 2 * q), a3 = lds32(X + r1 * kXS + 8 + 2 * q);
        uint32_t A[4][4];
        {
            float h[8][4];
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                h[nt][0] = h[nt][2] = S.b1[nt * 8 + 2 * q];
                h[nt][1] = h[nt][3] = S.b1[nt * 8 + 2 * q + 1];
                const __nv_bfloat16* wr = S.w1 + (nt * 8 + g) * kW1S;
                mma16816(h[nt], a0, a1, a2, a3, lds32(wr + 2 * q), lds32(wr + 8 + 2 * q));
            }
#pragma unroll
            for (int kt = 0; kt < 4; kt++) {
                A[kt][0] = pack_bf16(fmaxf(h[2 * kt][0], 0.f), fmaxf(h[2 * kt][1], 0.f));
                A[kt][1] = pack_bf16(fmaxf(h[2 * kt][2], 0.f), fmaxf(h[2 * kt][3], 0.f));
                A[kt][2] = pack_bf16(fmaxf(h[2 * kt + 1][0], 0.f), fmaxf(h[2 * kt + 1][1], 0.f));
                A[kt][3] = pack_bf16(fmaxf(h[2 * kt + 1][2], 0.f), fmaxf(h[2 * kt + 1][3], 0.f));
            }
        }
        {
            float h[8][4];
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                h[nt][0] = h[nt][2] = S.b2[nt * 8 + 2 * q];
                h[nt][1] = h[nt][3] = S.b2[nt * 8 + 2 * q + 1];
                const __nv_bfloat16* wr = S.w2 + (nt * 8 + g) * kW2S;
#pragma unroll
                for (int kt = 0; kt < 4; kt++)
                    mma16816(h[nt], A[kt][0], A[kt][1], A[kt][2], A[kt][3], lds32(wr + kt * 16 + 2 * q),
                             lds32(wr + kt * 16 + 8 + 2 * q));
            }
#pragma unroll
            for (int kt = 0; kt < 4; kt++) {
                A[kt][0] = pack_bf16(fmaxf(h[2 * kt][0], 0.f), fmaxf(h[2 * kt][1], 0.f));
                A[kt][1] = pack_bf16(fmaxf(h[2 * kt][2], 0.f), fmaxf(h[2 * kt][3], 0.f));
                A[kt][2] = pack_bf16(fmaxf(h[2 * kt + 1][0], 0.f), fmaxf(h[2 * kt + 1][1], 0.f));
                A[kt][3] = pack_bf16(fmaxf(h[2 * kt + 1][2], 0.f), fmaxf(h[2 * kt + 1][3], 0.f));
            }
        }
        float o[4];
        o[0] = o[2] = S.b3[2 * q];
        o[1] = o[3] = S.b3[2 * q + 1];
        const __nv_bfloat16* wr = S.w3 + g * kW2S;
#pragma unroll
        for (int kt = 0; kt < 4; kt++)
            mma16816(o, A[kt][0], A[kt][1], A[kt][2], A[kt][3], lds32(wr + kt * 16 + 2 * q),
                     lds32(wr + kt * 16 + 8 + 2 * q));
        Y[r0 * 8 + 2 * q] = o[0];
        Y[r0 * 8 + 2 * q + 1] = o[1];
        Y[r1 * 8 + 2 * q] = o[2];
        Y[r1 * 8 + 2 * q + 1] = o[3];
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < TC_MLP_OUT; k++) y[k] = Y[lane * 8 + k];
    __syncwarp();
}

}  // namespace ctrl

}  // namespace tc
