// Cartesian Taylor expansion helpers of the order-p FMM (total-order
// coefficient layout, scaled kernel derivatives, monomials, M2M/L2L shifts),
// shared by the solver and the order controller's error sampler.
#pragma once

#include "common.cuh"

namespace tc {

__host__ __device__ constexpr int ncoef(int p) { return (p + 1) * (p + 2) / 2; }
__host__ __device__ constexpr int cidx(int a, int b) { return (a + b) * (a + b + 1) / 2 + b; }
// coefficient arrays are padded to 16 bytes per node for vector loads
__host__ __device__ constexpr int kstride(int p) { return (ncoef(p) + 3) & ~3; }
// total degree of the coefficient with linear index i
__host__ __device__ constexpr int cdeg(int i)
{
    int k = 0;
    while ((k + 1) * (k + 2) / 2 <= i) k++;
    return k;
}

struct PotParams {
    float nu;    // phi = pref * u^-nu
    float c;     // u = r^2 + c (before scaling)
    float kappa; // pair term t = kappa * phi
    int kind;    // TC_KERNEL_*
    // expansions about the centre of mass have no dipole; about the cell centre
    // (TC_CENTRE_BOX) the M2L includes it
    int dipole = 0;
};

// scaled derivatives D_g, |g| <= P, at scaled offset (x, y) for a level of size h
template <int P>
__device__ inline void derivs(float x, float y, float h, const PotParams& pp, float* D)
{
    const float c = pp.c / (h * h);
    const float u = x * x + y * y + c;
    const float iu = __fdividef(1.0f, u);
    // pref * h^-2nu * u^-nu (scaled potential)
    if (pp.kind == TC_KERNEL_GRAVITY)
        D[0] = rsqrtf(u) / h;
    else
        D[0] = -0.5f * iu / (h * h);
    const float nu2 = 2.0f * pp.nu;
#pragma unroll
    for (int k = 1; k <= P; k++) {
#pragma unroll
        for (int b = 0; b <= k; b++) {
            const int a = k - b;
            float t;
            if (a >= 1) {
                t = (nu2 + 2.0f * (a - 1)) * x * D[cidx(a - 1, b)];
                if (b >= 1) t += 2.0f * b * y * D[cidx(a, b - 1)];
                if (a >= 2) t += (nu2 * (a - 1) + (float)((a - 1) * (a - 2))) * D[cidx(a - 2, b)];
                if (b >= 2) t += (float)(b * (b - 1)) * D[cidx(a, b - 2)];
            } else {
                t = (nu2 + 2.0f * (b - 1)) * y * D[cidx(0, b - 1)];
                if (b >= 2) t += (nu2 * (b - 1) + (float)((b - 1) * (b - 2))) * D[cidx(0, b - 2)];
            }
            D[cidx(a, b)] = -t * iu;
        }
    }
}

// monomials w_g = d^g / g! for |g| <= Q
template <int Q>
__device__ inline void monomials(float dx, float dy, float* w)
{
    w[0] = 1.0f;
#pragma unroll
    for (int k = 1; k <= Q; k++) {
#pragma unroll
        for (int b = 0; b <= k; b++) {
            const int a = k - b;
            if (a >= 1)
                w[cidx(a, b)] = w[cidx(a - 1, b)] * dx * (1.0f / a);
            else
                w[cidx(a, b)] = w[cidx(a, b - 1)] * dy * (1.0f / b);
        }
    }
}

// acc_a += sum_{b <= a} in_b * w_(a-b)       (M2M: mu(parent) from mu(child))
template <int P>
__device__ inline void shift_up(const float* in, const float* w, float* acc)
{
#pragma unroll
    for (int ka = 0; ka <= P; ka++)
#pragma unroll
        for (int ba = 0; ba <= ka; ba++) {
            const int aa = ka - ba;
            float s = 0.f;
#pragma unroll
            for (int kb = 0; kb <= ka; kb++)
#pragma unroll
                for (int bb = 0; bb <= kb; bb++) {
                    const int ab = kb - bb;
                    if (ab <= aa && bb <= ba) s += in[cidx(ab, bb)] * w[cidx(aa - ab, ba - bb)];
                }
            acc[cidx(aa, ba)] += s;
        }
}

// acc_b += sum_{g >= b} in_g * w_(g-b)       (L2L: local at d from local at 0)
template <int P>
__device__ inline void shift_down(const float* in, const float* w, float* acc)
{
#pragma unroll
    for (int kb = 0; kb <= P; kb++)
#pragma unroll
        for (int bb = 0; bb <= kb; bb++) {
            const int ab = kb - bb;
            float s = 0.f;
#pragma unroll
            for (int kg = kb; kg <= P; kg++)
#pragma unroll
                for (int bg = 0; bg <= kg; bg++) {
                    const int ag = kg - bg;
                    if (ag >= ab && bg >= bb) s += in[cidx(ag, bg)] * w[cidx(ag - ab, bg - bb)];
                }
            acc[cidx(ab, bb)] += s;
        }
}

}  // namespace tc
