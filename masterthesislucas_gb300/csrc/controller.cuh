// Features of a node pair for the expansion-order controller (shared by the
// error sampler and the list builder, so training and inference see the same
// numbers).  Inputs are scaled to the level's cell size h: R = (COM_A -
// COM_B)/h, multipoles mu_a = sum (r/h)^a / a! about each COM (total-order
// layout, order >= 8), COM offsets from the ideal cell centres in units of h.
//
// The per-node part (node_features, 8 floats) is computed once per node; a
// pair's 16 features combine two of them with the pair geometry.
#pragma once

#include "common.cuh"

namespace tc {

constexpr int kNodeFeat = 8;

__device__ inline float mp_norm(const float* mu, int k)
{
    // sqrt(sum_{|a|=k} mu_a^2) / M0
    float s = 0.f;
    const int base = k * (k + 1) / 2;
    for (int b = 0; b <= k; b++) s += mu[base + b] * mu[base + b];
    return sqrtf(s) / fmaxf(mu[0], 1e-30f);
}

// nf: spread, log2 M0, |COM offset|, log10 norms at orders 2, 4, 6, 8, 0
__device__ inline void node_features(const float* mu, float cx, float cy, float* nf)
{
    const float m0 = fmaxf(mu[0], 1e-30f);
    // mu_(2,0) and mu_(0,2) sit at linear indices 3 and 5
    nf[0] = sqrtf(fmaxf(2.f * (mu[3] + mu[5]) / m0, 0.f));
    nf[1] = log2f(m0);
    nf[2] = sqrtf(cx * cx + cy * cy);
    nf[3] = log10f(mp_norm(mu, 2) + 1e-12f);
    nf[4] = log10f(mp_norm(mu, 4) + 1e-12f);
    nf[5] = log10f(mp_norm(mu, 6) + 1e-12f);
    nf[6] = log10f(mp_norm(mu, 8) + 1e-12f);
    nf[7] = 0.f;
}

__device__ inline void pair_features_nf(float Rx, float Ry, const float* nfA, const float* nfB, float c_over_h2,
                                        int level, float* f)
{
    const float r = sqrtf(Rx * Rx + Ry * Ry);
    const float rr = fmaxf(r, 1e-6f);
    f[0] = log2f(rr);
    f[1] = fminf(fabsf(Rx), fabsf(Ry)) / rr;
    f[2] = nfA[0];
    f[3] = nfB[0];
    f[4] = (nfA[0] + nfB[0]) / rr;
    f[5] = nfA[1];
    f[6] = nfB[1];
    f[7] = nfA[2];
    f[8] = nfB[2];
    f[9] = nfB[3];
    f[10] = nfB[4];
    f[11] = nfB[5];
    f[12] = nfB[6];
    f[13] = nfA[4];
    f[14] = log2f(fmaxf(c_over_h2, 1e-30f));
    f[15] = (float)level / 16.0f;
}

__device__ inline void pair_features(float Rx, float Ry, const float* muA, const float* muB, float cAx, float cAy,
                                     float cBx, float cBy, float c_over_h2, int level, float* f)
{
    float a[kNodeFeat], b[kNodeFeat];
    node_features(muA, cAx, cAy, a);
    node_features(muB, cBx, cBy, b);
    pair_features_nf(Rx, Ry, a, b, c_over_h2, level, f);
}

}  // namespace tc
