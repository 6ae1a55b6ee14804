// Radial interaction kernels shared by the tree code and the direct sums.
// A kernel gives, for s = |R|^2, the radial factors of the force
// F(R) = R g(s): D1 = g, D2 = 2 g', D3 = 4 g'' (the derivative terms of the
// reference's TSNE_FMM_SYM_MORTON_*_Kernel, nBodySolverFMM_SYM_MORTON.h:622-636)
// and the scalar pair term t(s) summed into the solver's total.
#pragma once

#include "common.cuh"

namespace tc {

template <typename real>
__device__ inline real rcp(real x);
template <>
__device__ inline float rcp<float>(float x) { return __fdividef(1.0f, x); }
template <>
__device__ inline double rcp<double>(double x) { return 1.0 / x; }
template <typename real>
__device__ inline real rsq(real x);
template <>
__device__ inline float rsq<float>(float x) { return rsqrtf(x); }
template <>
__device__ inline double rsq<double>(double x) { return 1.0 / sqrt(x); }

// Single-instruction approximations of the PTX ISA (rcp.approx.ftz.f32,
// rsqrt.approx.ftz.f32: relative error below 2^-23 and 2^-22.9) for the
// P2P inner loops, where every instruction of the pair is on the critical
// issue path.
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Packed FP32 pairs (fma/add/sub/mul.rn.ftz.f32x2, sm_100 and later): two
// sources' coordinates in one 64-bit register, one instruction for both.
__device__ __forceinline__ unsigned long long f2_pack(float a, float b)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(unsigned long long v, float& a, float& b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b, unsigned long long c)
{
    unsigned long long d;
    asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ unsigned long long f2_add(unsigned long long a, unsigned long long b)
{
    unsigned long long d;
    asm("add.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b)
{
    unsigned long long d;
    asm("sub.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b)
{
    unsigned long long d;
    asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// Student-t kernel of the t-SNE repulsion: F(R) = R (1+r^2)^-2, pair term (1+r^2)^-1
template <typename real>
struct KTsne {
    __device__ inline void far(real s, real& D1, real& D2, real& D3, real& t) const
    {
        real inv = rcp<real>(real(1) + s);
        real i2 = inv * inv;
        D1 = i2;
        D2 = real(-4) * i2 * inv;
        D3 = real(24) * i2 * i2;
        t = inv;
    }
    __device__ inline void near(real s, real& D1, real& t) const
    {
        real fd = rcp<real>(real(1) + s);
        D1 = fd * fd;
        t = fd;
    }
    // near() of s = Rx^2 + Ry^2 with the constant folded into the FMA chain
    __device__ __forceinline__ void near_xy(float Rx, float Ry, float& D1, float& t) const
    {
        const float fd = rcp_approx(fmaf(Ry, Ry, fmaf(Rx, Rx, 1.0f)));
        D1 = fd * fd;
        t = fd;
    }
    // near_xy of two sources at once (packed): D1 = sign * a, t = sign * tt
    static constexpr float kSign = 1.0f;
    __device__ __forceinline__ void near_xy2(unsigned long long Rx, unsigned long long Ry, unsigned long long& a,
                                             unsigned long long& tt) const
    {
        float u0, u1;
        f2_unpack(f2_fma(Ry, Ry, f2_fma(Rx, Rx, f2_pack(1.0f, 1.0f))), u0, u1);
        tt = f2_pack(rcp_approx(u0), rcp_approx(u1));
        a = f2_mul(tt, tt);
    }
};

// 2D Plummer-softened gravity: F(R) = -R (r^2+eps^2)^-3/2, pair term -(r^2+eps^2)^-1/2
template <typename real>
struct KGrav {
    real eps2;
    __device__ inline void far(real s, real& D1, real& D2, real& D3, real& t) const
    {
        real u = s + eps2;
        real iu = rcp<real>(u);
        real isq = rsq<real>(u);
        real g = -isq * iu;
        D1 = g;
        D2 = real(-3) * g * iu;
        D3 = real(-5) * D2 * iu;
        t = -isq;
    }
    __device__ inline void near(real s, real& D1, real& t) const
    {
        real isq = rsq<real>(s + eps2);
        D1 = -isq * isq * isq;
        t = -isq;
    }
    __device__ __forceinline__ void near_xy(float Rx, float Ry, float& D1, float& t) const
    {
        const float isq = rsqrt_approx(fmaf(Ry, Ry, fmaf(Rx, Rx, (float)eps2)));
        D1 = -(isq * isq) * isq;
        t = -isq;
    }
    // near_xy of two sources at once (packed): D1 = sign * a, t = sign * tt
    static constexpr float kSign = -1.0f;
    __device__ __forceinline__ void near_xy2(unsigned long long Rx, unsigned long long Ry, unsigned long long& a,
                                             unsigned long long& tt) const
    {
        const float e = (float)eps2;
        float u0, u1;
        f2_unpack(f2_fma(Ry, Ry, f2_fma(Rx, Rx, f2_pack(e, e))), u0, u1);
        tt = f2_pack(rsqrt_approx(u0), rsqrt_approx(u1));
        a = f2_mul(f2_mul(tt, tt), tt);
    }
};


}  // namespace tc
