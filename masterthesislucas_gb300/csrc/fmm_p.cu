// Order-p symmetric Morton FMM: the reference's Cartesian Taylor scheme
// (src/nbodysolvers/cpu/nBodySolverFMM_SYM_MORTON.h:622-836 truncates at total
// order 3: multipole M0 + M2, local C1..C3) generalised to total order p.
//
// Expansions are about each node's centre of mass, with the reference's
// dual-tree MAC and lists (lists.cu).  Non-accepted leaf pairs interact by
// direct P2P (no point-node stage: at order p an M2P costs as much as a
// leaf-sized P2P).  Every quantity is scaled by the cell size h_l of its level
// so that FP32 covers orders up to 16 on deep trees:
//   mu_a  = sum_i m_i (r_i / h)^a / a!                      multipole
//   D_g   = h^|g| d^g phi(R)                                kernel derivatives
//   L_b   = sum_a (-1)^|a| mu_a D_(a+b),  |a| + |b| <= p     local (M2L)
// with phi the radial potential whose gradient is the force (t-SNE:
// -1/(2(1+r^2)); gravity: (r^2+eps^2)^-1/2).  The derivatives come from the
// recurrence u D_k = -[(2nu + 2n_i) x_i D_(k-e_i) + 2 n_j x_j D_(k-e_j)
// + (2nu n_i + n_i(n_i-1)) D_(k-2e_i) + n_j(n_j-1) D_(k-2e_j)] for
// phi = u^-nu, u = r^2 + c, n = k - e_i, obtained by differentiating
// u grad(phi) = -2 nu R phi.
#include <type_traits>

#include "expansion.cuh"
#include "kernels.cuh"
#include "m2l_tc.cuh"
#include "state.cuh"

namespace tc {
namespace {

// ------------------------------------------------------------------ P2M
// mu_a = sum (r/h)^a / a! about the COM.  Leaves of up to kLeafSmall
// particles take one thread each (monomials built degree by degree, two rows
// live); the larger leaves, listed by the leaf build, one warp each.

template <int P>
__global__ void __launch_bounds__(128) k_p2m_small(int dep, float h, const uint32_t* __restrict__ count,
                                                   const uint32_t* __restrict__ first,
                                                   const float* __restrict__ comrel, const float* __restrict__ prel,
                                                   float* __restrict__ mu, const uint32_t* __restrict__ act, const uint32_t* __restrict__ act_pos)
{
    constexpr int K = ncoef(P);
    const uint32_t li = level_index(dep);
    const int64_t nl = (int64_t)1 << (2 * dep);
    const float ih = 1.0f / h;
    const uint32_t k1 = act_pos[li + nl];
    for (uint32_t k = act_pos[li] + blockIdx.x * blockDim.x + threadIdx.x; k < k1; k += gridDim.x * blockDim.x) {
        const int64_t node = act[k];
        const uint32_t c = count[node];
        if (c == 0 || c > kLeafSmall) continue;
        const uint32_t f = first[node];
        const float cx = comrel[2 * node], cy = comrel[2 * node + 1];
        float acc[K];
#pragma unroll
        for (int k = 0; k < K; k++) acc[k] = 0.f;
        for (uint32_t q = 0; q < c; q++) {
            const float dx = (prel[2 * (f + q)] - cx) * ih, dy = (prel[2 * (f + q) + 1] - cy) * ih;
            float row[P + 1];
            row[0] = 1.0f;
            acc[0] += 1.0f;
#pragma unroll
            for (int k = 1; k <= P; k++) {
                // degree k from degree k-1: w_(a,b) = w_(a-1,b) dx / a, w_(0,k) = w_(0,k-1) dy / k
                const float last = row[k - 1];
#pragma unroll
                for (int b = 0; b < k; b++) row[b] = row[b] * dx * (1.0f / (k - b));
                row[k] = last * dy * (1.0f / k);
#pragma unroll
                for (int b = 0; b <= k; b++) acc[cidx(k - b, b)] += row[b];
            }
        }
        float4* o4 = reinterpret_cast<float4*>(mu + node * kstride(P));
#pragma unroll
        for (int c4 = 0; c4 < kstride(P) / 4; c4++)
            o4[c4] = make_float4(4 * c4 < K ? acc[4 * c4] : 0.f, 4 * c4 + 1 < K ? acc[4 * c4 + 1] : 0.f,
                                 4 * c4 + 2 < K ? acc[4 * c4 + 2] : 0.f, 4 * c4 + 3 < K ? acc[4 * c4 + 3] : 0.f);
    }
}

template <int P>
__global__ void __launch_bounds__(128) k_p2m(int dep, float h, const uint32_t* __restrict__ count,
                                             const uint32_t* __restrict__ first, const float* __restrict__ comrel,
                                             const float* __restrict__ prel, const uint32_t* __restrict__ big,
                                             float* __restrict__ mu)
{
    constexpr int K = ncoef(P);
    const int lane = threadIdx.x & 31;
    const uint32_t li = level_index(dep);
    const int64_t nbig = big[0];
    const float ih = 1.0f / h;
    const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); w < nbig; w += wstride) {
        const int64_t node = li + big[1 + w];
        const uint32_t c = count[node];
        const uint32_t f = first[node];
        const float cx = comrel[2 * node], cy = comrel[2 * node + 1];
        float acc[K];
#pragma unroll
        for (int k = 0; k < K; k++) acc[k] = 0.f;
        for (uint32_t q = lane; q < c; q += 32) {
            float w[K];
            monomials<P>((prel[2 * (f + q)] - cx) * ih, (prel[2 * (f + q) + 1] - cy) * ih, w);
#pragma unroll
            for (int k = 0; k < K; k++) acc[k] += w[k];
        }
#pragma unroll
        for (int k = 0; k < K; k++) {
            const float v = warp_sum(acc[k]);
            if (lane == 0) mu[node * kstride(P) + k] = v;
        }
    }
}

// the K coefficients of one node (stride KS, a multiple of 4) through 16-byte
// accesses
template <int K, int KS>
__device__ __forceinline__ void load_coefs(const float* __restrict__ src, float* dst)
{
    const float4* s4 = reinterpret_cast<const float4*>(src);
#pragma unroll
    for (int c = 0; c < KS / 4; c++) {
        const float4 v = s4[c];
        if (4 * c < K) dst[4 * c] = v.x;
        if (4 * c + 1 < K) dst[4 * c + 1] = v.y;
        if (4 * c + 2 < K) dst[4 * c + 2] = v.z;
        if (4 * c + 3 < K) dst[4 * c + 3] = v.w;
    }
}

template <int K, int KS>
__device__ __forceinline__ void store_coefs(float* __restrict__ dst, const float* src)
{
    float4* o4 = reinterpret_cast<float4*>(dst);
#pragma unroll
    for (int c = 0; c < KS / 4; c++)
        o4[c] = make_float4(4 * c < K ? src[4 * c] : 0.f, 4 * c + 1 < K ? src[4 * c + 1] : 0.f,
                            4 * c + 2 < K ? src[4 * c + 2] : 0.f, 4 * c + 3 < K ? src[4 * c + 3] : 0.f);
}

// coefficient k of degree d scaled by 2^-d (a child-scale multipole at the
// parent's scale, or a parent-scale local expansion at the child's)
template <int K>
__device__ __forceinline__ void halve_by_degree(float* c)
{
#pragma unroll
    for (int k = 0; k < K; k++) c[k] *= 1.0f / (float)(1 << cdeg(k));
}

// levels of up to this many cells (4^8) shift their children with four lanes per node
constexpr int64_t kM2mQuadLevelNodes = (int64_t)1 << 16;

// ------------------------------------------------------------------ M2M
// one thread per node of level l: shift the children's multipoles (child
// scale h/2) to the node's COM at scale h
template <int P>
__global__ void __launch_bounds__(128) k_m2m(int l, float hl, const uint32_t* __restrict__ count,
                                             const float* __restrict__ comrel, float* __restrict__ mu, const uint32_t* __restrict__ act, const uint32_t* __restrict__ act_pos)
{
    constexpr int K = ncoef(P);
    const uint32_t li = level_index(l), lc = level_index(l + 1);
    const int64_t nl = (int64_t)1 << (2 * l);
    const float ih = 1.0f / hl;
    const uint32_t k1 = act_pos[li + nl];
    for (uint32_t k = act_pos[li] + blockIdx.x * blockDim.x + threadIdx.x; k < k1; k += gridDim.x * blockDim.x) {
        const int64_t node = act[k];
        const int64_t i = node - li;
        const float px = comrel[2 * node], py = comrel[2 * node + 1];
        float acc[K];
#pragma unroll
        for (int k = 0; k < K; k++) acc[k] = 0.f;
        for (int j = 0; j < 4; j++) {
            const int64_t ch = lc + 4 * i + j;
            if (count[ch] == 0) continue;
            // child COM - parent COM: child cell centre sits at (+-1/4, +-1/4) h of the parent's
            const float ox = ((j & 1) ? 0.25f : -0.25f) * hl, oy = ((j & 2) ? 0.25f : -0.25f) * hl;
            const float dx = (ox + comrel[2 * ch] - px) * ih, dy = (oy + comrel[2 * ch + 1] - py) * ih;
            float in[K], w[K];
            load_coefs<K, kstride(P)>(mu + ch * kstride(P), in);
            halve_by_degree<K>(in);  // child scale -> parent scale
            monomials<P>(dx, dy, w);
            shift_up<P>(in, w, acc);
        }
        store_coefs<K, kstride(P)>(mu + node * kstride(P), acc);
    }
}

// ------------------------------------------------------------------ shifts at orders >= 10
// Streaming shifts: one thread per node, the shift's monomials and the
// accumulators in registers, the input expansion read coefficient by
// coefficient (no third register array).
// input degree KA and up, one degree per instantiation (a single nest over
// all degrees exceeds the unroller's limit at order 12)
template <int P, int KA>
__device__ __forceinline__ void m2m_deg(const float* __restrict__ in, const float* w, float* acc)
{
    if constexpr (KA <= P) {
        constexpr float sc = 1.0f / (float)(1 << KA);  // child -> parent scale
#pragma unroll
        for (int ba = 0; ba <= KA; ba++) {
            const float v = __ldg(in + cidx(KA - ba, ba)) * sc;
#pragma unroll
            for (int kg = 0; kg + KA <= P; kg++)
#pragma unroll
                for (int bg = 0; bg <= kg; bg++) acc[cidx(KA - ba + kg - bg, ba + bg)] += v * w[cidx(kg - bg, bg)];
        }
        m2m_deg<P, KA + 1>(in, w, acc);
    }
}

template <int P>
__device__ __forceinline__ void m2m_child(float dx, float dy, const float* __restrict__ in, float* acc)
{
    float w[ncoef(P)];
    monomials<P>(dx, dy, w);
    m2m_deg<P, 0>(in, w, acc);
}

template <int P>
__global__ void __launch_bounds__(128) k_m2m_stream(int l, float hl, const uint32_t* __restrict__ count,
                                                    const float* __restrict__ comrel, float* __restrict__ mu, const uint32_t* __restrict__ act, const uint32_t* __restrict__ act_pos)
{
    constexpr int K = ncoef(P), KS = kstride(P);
    const uint32_t li = level_index(l), lc = level_index(l + 1);
    const int64_t nl = (int64_t)1 << (2 * l);
    const float ih = 1.0f / hl;
    const uint32_t k1 = act_pos[li + nl];
    for (uint32_t k = act_pos[li] + blockIdx.x * blockDim.x + threadIdx.x; k < k1; k += gridDim.x * blockDim.x) {
        const int64_t node = act[k];
        const int64_t i = node - li;
        const float px = comrel[2 * node], py = comrel[2 * node + 1];
        float acc[K];
#pragma unroll
        for (int k = 0; k < K; k++) acc[k] = 0.f;
#pragma unroll 1
        for (int j = 0; j < 4; j++) {
            const int64_t ch = lc + 4 * i + j;
            if (count[ch] == 0) continue;
            // child COM - parent COM: child cell centre sits at (+-1/4, +-1/4) h of the parent's
            const float ox = (j & 1) ? 0.25f : -0.25f, oy = (j & 2) ? 0.25f : -0.25f;
            m2m_child<P>(ox + (comrel[2 * ch] - px) * ih, oy + (comrel[2 * ch + 1] - py) * ih, mu + ch * KS, acc);
        }
        float4* o4 = reinterpret_cast<float4*>(mu + node * KS);
#pragma unroll
        for (int c = 0; c < KS / 4; c++)
            o4[c] = make_float4(4 * c < K ? acc[4 * c] : 0.f, 4 * c + 1 < K ? acc[4 * c + 1] : 0.f,
                                4 * c + 2 < K ? acc[4 * c + 2] : 0.f, 4 * c + 3 < K ? acc[4 * c + 3] : 0.f);
    }
}

// coarse levels: four lanes per node, one per child, summed by two butterfly
// steps (the fine levels keep one thread per node and its children in turn)
template <int P>
__global__ void __launch_bounds__(128) k_m2m_quad(int l, float hl, const uint32_t* __restrict__ count,
                                                  const float* __restrict__ comrel, float* __restrict__ mu,
                                                  const uint32_t* __restrict__ act, const uint32_t* __restrict__ act_pos)
{
    constexpr int K = ncoef(P), KS = kstride(P);
    const uint32_t li = level_index(l), lc = level_index(l + 1);
    const int64_t nl = (int64_t)1 << (2 * l);
    const float ih = 1.0f / hl;
    const int j = threadIdx.x & 3;
    const uint32_t k0 = act_pos[li], k1 = act_pos[li + nl];
    const uint32_t nodes_per_pass = gridDim.x * (blockDim.x >> 2);
    for (uint32_t base = k0; base < k1; base += nodes_per_pass) {
        const uint32_t k = base + blockIdx.x * (blockDim.x >> 2) + (threadIdx.x >> 2);
        const bool valid = k < k1;
        float acc[K];
#pragma unroll
        for (int c = 0; c < K; c++) acc[c] = 0.f;
        int64_t node = 0;
        if (valid) {
            node = act[k];
            const int64_t i = node - li;
            const int64_t ch = lc + 4 * i + j;
            if (count[ch] != 0) {
                const float px = comrel[2 * node], py = comrel[2 * node + 1];
                const float ox = (j & 1) ? 0.25f : -0.25f, oy = (j & 2) ? 0.25f : -0.25f;
                const float dx = ox + (comrel[2 * ch] - px) * ih, dy = oy + (comrel[2 * ch + 1] - py) * ih;
                if constexpr (P >= 10) {
                    m2m_child<P>(dx, dy, mu + ch * KS, acc);
                } else {
                    float in[K], w[K];
                    load_coefs<K, KS>(mu + ch * KS, in);
                    halve_by_degree<K>(in);  // child scale -> parent scale
                    monomials<P>(dx, dy, w);
                    shift_up<P>(in, w, acc);
                }
            }
        }
#pragma unroll
        for (int c = 0; c < K; c++) {
            acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 1);
            acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 2);
        }
        if (valid && j == 0) store_coefs<K, KS>(mu + node * KS, acc);
    }
}

template <int P>
__global__ void __launch_bounds__(128) k_l2l_stream(int l, float hl, const uint32_t* __restrict__ count,
                                                    const float* __restrict__ comrel, float* __restrict__ loc, const uint32_t* __restrict__ act, const uint32_t* __restrict__ act_pos)
{
    constexpr int K = ncoef(P), KS = kstride(P);
    const uint32_t li = level_index(l), lp = level_index(l - 1);
    const int64_t nl = (int64_t)1 << (2 * l);
    const float ih = 1.0f / hl;
    const uint32_t k1 = act_pos[li + nl];
    for (uint32_t k = act_pos[li] + blockIdx.x * blockDim.x + threadIdx.x; k < k1; k += gridDim.x * blockDim.x) {
        const int64_t node = act[k];
        const int64_t i = node - li;
        const int64_t par = lp + (i >> 2);
        const int j = (int)(i & 3);
        const float ox = ((j & 1) ? 0.5f : -0.5f), oy = ((j & 2) ? 0.5f : -0.5f);
        const float ddx = ox + (comrel[2 * node] - comrel[2 * par]) * ih;
        const float ddy = oy + (comrel[2 * node + 1] - comrel[2 * par + 1]) * ih;
        float w[K], acc[K];
        monomials<P>(ddx, ddy, w);
        const float4* a4 = reinterpret_cast<const float4*>(loc + node * KS);
#pragma unroll
        for (int c = 0; c < KS / 4; c++) {
            const float4 v = a4[c];
            if (4 * c < K) acc[4 * c] = v.x;
            if (4 * c + 1 < K) acc[4 * c + 1] = v.y;
            if (4 * c + 2 < K) acc[4 * c + 2] = v.z;
            if (4 * c + 3 < K) acc[4 * c + 3] = v.w;
        }
        const float* in = loc + par * KS;
#pragma unroll
        for (int kg = 0; kg <= P; kg++) {
            const float sc = 1.0f / (float)(1 << kg);  // parent scale 2h -> h
#pragma unroll
            for (int bg = 0; bg <= kg; bg++) {
                const int ag = kg - bg;
                const float v = in[cidx(ag, bg)] * sc;
#pragma unroll
                for (int ab = 0; ab <= ag; ab++)
#pragma unroll
                    for (int bb = 0; bb <= bg; bb++) acc[cidx(ab, bb)] += v * w[cidx(ag - ab, bg - bb)];
            }
        }
        float4* o4 = reinterpret_cast<float4*>(loc + node * KS);
#pragma unroll
        for (int c = 0; c < KS / 4; c++)
            o4[c] = make_float4(4 * c < K ? acc[4 * c] : 0.f, 4 * c + 1 < K ? acc[4 * c + 1] : 0.f,
                                4 * c + 2 < K ? acc[4 * c + 2] : 0.f, 4 * c + 3 < K ? acc[4 * c + 3] : 0.f);
    }
}

// ------------------------------------------------------------------ M2L
// L_b += sum_a (-1)^|a| mu_a D_(a+b) at order P for one source (multipoles
// stored with stride KSS); L holds at least ncoef(P) coefficients.
template <int P, int KSS>
__device__ __forceinline__ void m2l_acc(float Rx, float Ry, float hl, const PotParams& pp, const float* __restrict__ m,
                                        float* L)
{
    constexpr int K = ncoef(P);
    constexpr int KS = kstride(P);
    static_assert(KS <= KSS, "storage order below the launch order");
    float D[K];
    derivs<P>(Rx, Ry, hl, pp, D);
    const float4* m4 = reinterpret_cast<const float4*>(m);
    float dip[2] = {0.f, 0.f};
#pragma unroll
    for (int c = 0; c < KS / 4; c++) {
        const float4 q = __ldg(m4 + c);
        const float mv[4] = {q.x, q.y, q.z, q.w};
        if (c == 0) {
            dip[0] = q.y;
            dip[1] = q.z;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int ia = 4 * c + j;
            if (ia >= K) continue;
            const int ka = cdeg(ia), ba = ia - ka * (ka + 1) / 2;
            if (ka == 1) continue;  // the dipole vanishes about the COM (added below about the cell centre)
            const float ma = (ka & 1) ? -mv[j] : mv[j];
#pragma unroll
            for (int kb = 0; kb + ka <= P; kb++)
#pragma unroll
                for (int bb = 0; bb <= kb; bb++) L[cidx(kb - bb, bb)] += ma * D[cidx(ka - ba + kb - bb, ba + bb)];
        }
    }
    if (pp.dipole) {
        // a = (1, 0) and (0, 1): sign (-1)^1
#pragma unroll
        for (int kb = 0; kb + 1 <= P; kb++)
#pragma unroll
            for (int bb = 0; bb <= kb; bb++) {
                const int ab = kb - bb;
                L[cidx(ab, bb)] -= dip[0] * D[cidx(ab + 1, bb)] + dip[1] * D[cidx(ab, bb + 1)];
            }
    }
}

// the far-field pair sum of node A, kappa * sum_b L_b mu_b(A), from its M2L sum alone
template <int K, int KS>
__device__ __forceinline__ double m2l_pairsum(int64_t na, bool any, float kappa, const float* L,
                                              const float* __restrict__ mu)
{
    if (!any) return 0.0;
    const float* m = mu + na * KS;
    float zs = 0.f;
#pragma unroll
    for (int k = 0; k < K; k++) zs += L[k] * m[k];
    return (double)kappa * (double)zs;
}

template <int K, int KS>
__device__ __forceinline__ void m2l_write(int64_t na, double z, const float* L, float* __restrict__ loc,
                                          double* __restrict__ zpart)
{
    zpart[na] = z;
    float4* o4 = reinterpret_cast<float4*>(loc + na * KS);
#pragma unroll
    for (int c = 0; c < KS / 4; c++)
        o4[c] = make_float4(4 * c < K ? L[4 * c] : 0.f, 4 * c + 1 < K ? L[4 * c + 1] : 0.f,
                            4 * c + 2 < K ? L[4 * c + 2] : 0.f, 4 * c + 3 < K ? L[4 * c + 3] : 0.f);
}

// the node's local expansion and its far-field pair sum
template <int K, int KS>
__device__ __forceinline__ void m2l_store(int64_t na, bool any, float kappa, const float* L,
                                          const float* __restrict__ mu, float* __restrict__ loc,
                                          double* __restrict__ zpart)
{
    m2l_write<K, KS>(na, m2l_pairsum<K, KS>(na, any, kappa, L, mu), L, loc, zpart);
}

// L2L into node (level l) from its parent's final local expansion: the same
// arithmetic as k_l2l, with the node's own sum acc still in registers
template <int P>
__device__ __forceinline__ void l2l_into(int64_t node, int l, float ih, const float* __restrict__ comrel,
                                         const float* __restrict__ loc, float* acc)
{
    constexpr int K = ncoef(P);
    const uint32_t li = level_index(l), lp = level_index(l - 1);
    const int64_t i = node - li;
    const int64_t par = lp + (i >> 2);
    const int j = (int)(i & 3);
    const float ox = ((j & 1) ? 0.5f : -0.5f), oy = ((j & 2) ? 0.5f : -0.5f);
    const float ddx = ox + (comrel[2 * node] - comrel[2 * par]) * ih;
    const float ddy = oy + (comrel[2 * node + 1] - comrel[2 * par + 1]) * ih;
    float in[K], w[K];
    load_coefs<K, kstride(P)>(loc + par * kstride(P), in);
    halve_by_degree<K>(in);  // parent scale 2h -> child scale h
    monomials<P>(ddx, ddy, w);
    shift_down<P>(in, w, acc);
}

// one thread per sink node A of level l: L(A) = sum over nn(A) of M2L; with
// L2L, plus the parent's final local expansion shifted to A (the level's L2L
// fused in: A's sum is not written and read back), held to the unfused form's
// registers so the M2L loop keeps its resident warps
#ifndef TC_M2L_FUSED_MIN_BLOCKS
#define TC_M2L_FUSED_MIN_BLOCKS 4  // resident blocks per SM of the order-8 fused M2L + L2L
#endif
template <int P, bool L2L = false>
__global__ void __launch_bounds__(128, L2L ? (P >= 8 ? TC_M2L_FUSED_MIN_BLOCKS : P >= 6 ? 5 : 7) : 1) k_m2l_p(int l, float hl, PotParams pp, const uint32_t* __restrict__ nn_ptr,
                                               const uint32_t* __restrict__ nn_idx, const uint32_t* __restrict__ count,
                                               const float* __restrict__ comrel, const float* __restrict__ mu,
                                               float* __restrict__ loc, double* __restrict__ zpart, const uint32_t* __restrict__ act, const uint32_t* __restrict__ act_pos)
{
    constexpr int K = ncoef(P), KS = kstride(P);
    const uint32_t li = level_index(l);
    const int64_t nl = (int64_t)1 << (2 * l);
    const float ih = 1.0f / hl;
    const float2* comrel2 = reinterpret_cast<const float2*>(comrel);
    const uint32_t k1 = act_pos[li + nl];  // empty nodes are never read
    for (uint32_t k = act_pos[li] + blockIdx.x * blockDim.x + threadIdx.x; k < k1; k += gridDim.x * blockDim.x) {
        const int64_t na = act[k];
        const int64_t a = na - li;
        const uint32_t b0 = nn_ptr[a], b1 = nn_ptr[a + 1];
        float L[K];
#pragma unroll
        for (int k = 0; k < K; k++) L[k] = 0.f;
        const int iax = (int)compact16((uint32_t)a), iay = (int)compact16((uint32_t)a >> 1);
        const float2 ca = comrel2[na];
        // the next entry's index and COM are loaded one iteration ahead, so
        // the dependent index -> COM loads overlap the current M2L
        uint32_t bn = b0 < b1 ? nn_idx[b0] : 0u;
        float2 cn = comrel2[li + bn];
        for (uint32_t e = b0; e < b1; e++) {
            const uint32_t b = bn;
            const float2 cb = cn;
            if (e + 1 < b1) {
                bn = nn_idx[e + 1];
                cn = comrel2[li + bn];
            }
            const int64_t nb = li + b;
            const float Rx = (float)(iax - (int)compact16(b)) + (ca.x - cb.x) * ih;
            const float Ry = (float)(iay - (int)compact16(b >> 1)) + (ca.y - cb.y) * ih;
            m2l_acc<P, KS>(Rx, Ry, hl, pp, mu + nb * KS, L);
        }
        if constexpr (L2L) {
            const double z = m2l_pairsum<K, KS>(na, b0 != b1, pp.kappa, L, mu);
            l2l_into<P>(na, l, ih, comrel, loc, L);
            m2l_write<K, KS>(na, z, L, loc, zpart);
        } else {
            m2l_store<K, KS>(na, b0 != b1, pp.kappa, L, mu, loc, zpart);
        }
    }
}

// The coarse levels hold few sink nodes, so one thread per node leaves the GPU
// idle behind each node's serial list: one warp per node instead, the lanes
// taking the list's entries in turn (entry e to lane e mod 32) into their own
// accumulators, then a fixed butterfly sum over the lanes.
template <int P>
__global__ void __launch_bounds__(128) k_m2l_warp(int l, float hl, PotParams pp, const uint32_t* __restrict__ nn_ptr,
                                                  const uint32_t* __restrict__ nn_idx, const float* __restrict__ comrel,
                                                  const float* __restrict__ mu, float* __restrict__ loc,
                                                  double* __restrict__ zpart, const uint32_t* __restrict__ act,
                                                  const uint32_t* __restrict__ act_pos)
{
    constexpr int K = ncoef(P), KS = kstride(P);
    const uint32_t li = level_index(l);
    const int64_t nl = (int64_t)1 << (2 * l);
    const float ih = 1.0f / hl;
    const float2* comrel2 = reinterpret_cast<const float2*>(comrel);
    const int lane = threadIdx.x & 31;
    const uint32_t k1 = act_pos[li + nl];
    const uint32_t wstride = gridDim.x * (blockDim.x >> 5);
    for (uint32_t k = act_pos[li] + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < k1; k += wstride) {
        const int64_t na = act[k];
        const int64_t a = na - li;
        const uint32_t b0 = nn_ptr[a], b1 = nn_ptr[a + 1];
        float L[K];
#pragma unroll
        for (int c = 0; c < K; c++) L[c] = 0.f;
        const int iax = (int)compact16((uint32_t)a), iay = (int)compact16((uint32_t)a >> 1);
        const float2 ca = comrel2[na];
        for (uint32_t e = b0 + lane; e < b1; e += 32) {
            const uint32_t b = nn_idx[e];
            const int64_t nb = li + b;
            const float2 cb = comrel2[nb];
            const float Rx = (float)(iax - (int)compact16(b)) + (ca.x - cb.x) * ih;
            const float Ry = (float)(iay - (int)compact16(b >> 1)) + (ca.y - cb.y) * ih;
            m2l_acc<P, KS>(Rx, Ry, hl, pp, mu + nb * KS, L);
        }
#pragma unroll
        for (int c = 0; c < K; c++)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) L[c] += __shfl_xor_sync(0xffffffffu, L[c], o);
        if (lane == 0) m2l_store<K, KS>(na, b0 != b1, pp.kappa, L, mu, loc, zpart);
    }
}

// Per-pair orders (the learned controller, or the bounding-radius rule): a
// node's accepted entries come sorted by order bucket (orders 4, 6, 8, 10,
// 12) over expansions stored at order PST.  The launch with OLO == 0 writes
// the node's local expansion (zeros above PACC); a launch with OLO > 0 adds.
// The learned controller (PST 12) takes two launches per level: buckets
// 4..8 with an order-8 accumulator (half the registers, twice the resident
// warps), then 10 and 12 with an order-12 one.  (A lower-order contribution
// has no coefficients above its order, so the pair sum over the stored
// coefficients equals the sum of the per-order sums.)
template <int PST, int PACC, int OLO, int OHI>
__global__ void __launch_bounds__(128) k_m2l_mixed(int l, float hl, PotParams pp, const uint32_t* __restrict__ nn_ptr,
                                                   const uint32_t* __restrict__ nn_idx,
                                                   const uint8_t* __restrict__ ord,
                                                   const uint32_t* __restrict__ count,
                                                   const float* __restrict__ comrel, const float* __restrict__ mu,
                                                   float* __restrict__ loc, double* __restrict__ zpart, const uint32_t* __restrict__ act, const uint32_t* __restrict__ act_pos)
{
    constexpr int K = ncoef(PACC), KS = kstride(PST);
    constexpr bool first = OLO == 0;
    const uint32_t li = level_index(l);
    const int64_t nl = (int64_t)1 << (2 * l);
    const float ih = 1.0f / hl;
    const float2* comrel2 = reinterpret_cast<const float2*>(comrel);
    const uint32_t k1 = act_pos[li + nl];
    for (uint32_t k = act_pos[li] + blockIdx.x * blockDim.x + threadIdx.x; k < k1; k += gridDim.x * blockDim.x) {
        const int64_t na = act[k];
        const int64_t a = na - li;
        const uint32_t p0 = nn_ptr[a], b1 = nn_ptr[a + 1];
        uint32_t e = p0;
        while (e < b1 && ord[e] < OLO) e++;
        const uint32_t b0 = e;
        float L[K];
#pragma unroll
        for (int k = 0; k < K; k++) L[k] = 0.f;
        const int iax = (int)compact16((uint32_t)a), iay = (int)compact16((uint32_t)a >> 1);
        const float2 ca = comrel2[na];
        // next entry's order, index and COM one iteration ahead
        uint8_t on = e < b1 ? ord[e] : 0xff;
        uint32_t bn = e < b1 ? nn_idx[e] : 0u;
        float2 cn = comrel2[li + bn];
        auto bucket = [&](auto order_tag, int o) {
            constexpr int PO = decltype(order_tag)::value;
            for (; e < b1 && on == o; e++) {
                const uint32_t b = bn;
                const float2 cb = cn;
                on = 0xff;
                if (e + 1 < b1) {
                    on = ord[e + 1];
                    bn = nn_idx[e + 1];
                    cn = comrel2[li + bn];
                }
                const int64_t nb = li + b;
                const float Rx = (float)(iax - (int)compact16(b)) + (ca.x - cb.x) * ih;
                const float Ry = (float)(iay - (int)compact16(b >> 1)) + (ca.y - cb.y) * ih;
                if constexpr (PO <= PACC) m2l_acc<PO, KS>(Rx, Ry, hl, pp, mu + nb * KS, L);
            }
        };
        if constexpr (OLO <= 0 && 0 <= OHI) bucket(std::integral_constant<int, 4>{}, 0);
        if constexpr (OLO <= 1 && 1 <= OHI) bucket(std::integral_constant<int, 6>{}, 1);
        if constexpr (OLO <= 2 && 2 <= OHI) bucket(std::integral_constant<int, 8>{}, 2);
        if constexpr (OLO <= 3 && 3 <= OHI) bucket(std::integral_constant<int, 10>{}, 3);
        if constexpr (OLO <= 4 && 4 <= OHI) bucket(std::integral_constant<int, 12>{}, 4);
        const bool any = e != b0;
        if (first) {
            m2l_store<K, KS>(na, any, pp.kappa, L, mu, loc, zpart);
        } else if (any) {
            const float* m = mu + na * KS;
            float zs = 0.f;
#pragma unroll
            for (int k = 0; k < K; k++) zs += L[k] * m[k];
            zpart[na] += (double)pp.kappa * (double)zs;
            float4* o4 = reinterpret_cast<float4*>(loc + na * KS);
#pragma unroll
            for (int c = 0; c < KS / 4; c++) {
                float4 v = o4[c];
                v.x += 4 * c < K ? L[4 * c] : 0.f;
                v.y += 4 * c + 1 < K ? L[4 * c + 1] : 0.f;
                v.z += 4 * c + 2 < K ? L[4 * c + 2] : 0.f;
                v.w += 4 * c + 3 < K ? L[4 * c + 3] : 0.f;
                o4[c] = v;
            }
        }
    }
}

// the same on the coarse levels: a warp per sink node, lanes taking the
// entries in turn whatever their bucket (each entry evaluated at its own
// order), then a butterfly sum
template <int PST, int PACC, int OLO, int OHI>
__global__ void __launch_bounds__(128) k_m2l_mixed_warp(int l, float hl, PotParams pp,
                                                        const uint32_t* __restrict__ nn_ptr,
                                                        const uint32_t* __restrict__ nn_idx,
                                                        const uint8_t* __restrict__ ord,
                                                        const float* __restrict__ comrel, const float* __restrict__ mu,
                                                        float* __restrict__ loc, double* __restrict__ zpart,
                                                        const uint32_t* __restrict__ act,
                                                        const uint32_t* __restrict__ act_pos)
{
    constexpr int K = ncoef(PACC), KS = kstride(PST);
    constexpr bool first = OLO == 0;
    const uint32_t li = level_index(l);
    const int64_t nl = (int64_t)1 << (2 * l);
    const float ih = 1.0f / hl;
    const float2* comrel2 = reinterpret_cast<const float2*>(comrel);
    const int lane = threadIdx.x & 31;
    const uint32_t k1 = act_pos[li + nl];
    const uint32_t wstride = gridDim.x * (blockDim.x >> 5);
    for (uint32_t k = act_pos[li] + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < k1; k += wstride) {
        const int64_t na = act[k];
        const int64_t a = na - li;
        const uint32_t p0 = nn_ptr[a], b1 = nn_ptr[a + 1];
        float L[K];
#pragma unroll
        for (int c = 0; c < K; c++) L[c] = 0.f;
        const int iax = (int)compact16((uint32_t)a), iay = (int)compact16((uint32_t)a >> 1);
        const float2 ca = comrel2[na];
        bool mine = false;
        for (uint32_t e = p0 + lane; e < b1; e += 32) {
            const int o = ord[e];
            if (o < OLO || o > OHI) continue;
            mine = true;
            const uint32_t b = nn_idx[e];
            const int64_t nb = li + b;
            const float2 cb = comrel2[nb];
            const float Rx = (float)(iax - (int)compact16(b)) + (ca.x - cb.x) * ih;
            const float Ry = (float)(iay - (int)compact16(b >> 1)) + (ca.y - cb.y) * ih;
            if constexpr (OLO <= 0 && 0 <= OHI && 4 <= PACC) if (o == 0) m2l_acc<4, KS>(Rx, Ry, hl, pp, mu + nb * KS, L);
            if constexpr (OLO <= 1 && 1 <= OHI && 6 <= PACC) if (o == 1) m2l_acc<6, KS>(Rx, Ry, hl, pp, mu + nb * KS, L);
            if constexpr (OLO <= 2 && 2 <= OHI && 8 <= PACC) if (o == 2) m2l_acc<8, KS>(Rx, Ry, hl, pp, mu + nb * KS, L);
            if constexpr (OLO <= 3 && 3 <= OHI && 10 <= PACC) if (o == 3) m2l_acc<10, KS>(Rx, Ry, hl, pp, mu + nb * KS, L);
            if constexpr (OLO <= 4 && 4 <= OHI && 12 <= PACC) if (o == 4) m2l_acc<12, KS>(Rx, Ry, hl, pp, mu + nb * KS, L);
        }
        const bool any = __any_sync(0xffffffffu, mine);
#pragma unroll
        for (int c = 0; c < K; c++)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) L[c] += __shfl_xor_sync(0xffffffffu, L[c], o);
        if (lane != 0) continue;
        if (first) {
            m2l_store<K, KS>(na, any, pp.kappa, L, mu, loc, zpart);
        } else if (any) {
            const float* m = mu + na * KS;
            float zs = 0.f;
#pragma unroll
            for (int c = 0; c < K; c++) zs += L[c] * m[c];
            zpart[na] += (double)pp.kappa * (double)zs;
            float4* o4 = reinterpret_cast<float4*>(loc + na * KS);
#pragma unroll
            for (int c = 0; c < KS / 4; c++) {
                float4 v = o4[c];
                v.x += 4 * c < K ? L[4 * c] : 0.f;
                v.y += 4 * c + 1 < K ? L[4 * c + 1] : 0.f;
                v.z += 4 * c + 2 < K ? L[4 * c + 2] : 0.f;
                v.w += 4 * c + 3 < K ? L[4 * c + 3] : 0.f;
                o4[c] = v;
            }
        }
    }
}

// ------------------------------------------------------------------ L2L
// one thread per node of level l >= 1: L_fin = L_own + shift(L_fin(parent))
template <int P>
__global__ void __launch_bounds__(128) k_l2l(int l, float hl, const uint32_t* __restrict__ count,
                                             const float* __restrict__ comrel, float* __restrict__ loc, const uint32_t* __restrict__ act, const uint32_t* __restrict__ act_pos)
{
    constexpr int K = ncoef(P);
    const uint32_t li = level_index(l), lp = level_index(l - 1);
    const int64_t nl = (int64_t)1 << (2 * l);
    const float ih = 1.0f / hl;
    const uint32_t k1 = act_pos[li + nl];
    for (uint32_t k = act_pos[li] + blockIdx.x * blockDim.x + threadIdx.x; k < k1; k += gridDim.x * blockDim.x) {
        const int64_t node = act[k];
        const int64_t i = node - li;
        const int64_t par = lp + (i >> 2);
        const int j = (int)(i & 3);
        // node COM - parent COM in units of the node's cell size h: the child
        // cell centre sits (+-1/2, +-1/2) h from the parent's
        const float ox = ((j & 1) ? 0.5f : -0.5f), oy = ((j & 2) ? 0.5f : -0.5f);
        const float ddx = ox + (comrel[2 * node] - comrel[2 * par]) * ih;
        const float ddy = oy + (comrel[2 * node + 1] - comrel[2 * par + 1]) * ih;
        float in[K], w[K], acc[K];
        load_coefs<K, kstride(P)>(loc + par * kstride(P), in);
        halve_by_degree<K>(in);  // parent scale 2h -> child scale h
        load_coefs<K, kstride(P)>(loc + node * kstride(P), acc);
        monomials<P>(ddx, ddy, w);
        shift_down<P>(in, w, acc);
        store_coefs<K, kstride(P)>(loc + node * kstride(P), acc);
    }
}

// levels of up to this many cells (4^8) take a warp per sink node in the M2L
// (measured: at level 9 of a 4M-particle tree the thread-per-node form is
// already faster)
constexpr int64_t kM2lWarpLevelNodes = (int64_t)1 << 16;

// ------------------------------------------------------------------ near field
constexpr int kNearWarps = 4;

// sinks per block item: leaves of more than 32 particles are split into
// items of this many sinks, a block (a warp per 32 sinks) each
constexpr uint32_t kBlockSinks = 32u * kNearWarps;

// per leaf: warp items (a leaf of 1..32 particles) and block items (a larger
// leaf, one per kBlockSinks of its particles)
__global__ void k_chunks(int dep, const uint32_t* __restrict__ count, uint32_t* __restrict__ nwarp,
                         uint32_t* __restrict__ nblock)
{
    const uint32_t li = level_index(dep);
    const int64_t nl = (int64_t)1 << (2 * dep);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nl; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t c = count[li + i];
        nwarp[i] = c >= 1u && c <= 32u ? 1u : 0u;
        nblock[i] = c > 32u ? (c + kBlockSinks - 1u) / kBlockSinks : 0u;
    }
}

// item -> leaf for both kinds, from the exclusive scans of their counts (items
// of one leaf are consecutive), and the number of pair-sum words the near
// field writes (warp items first, then block items); cap bounds every map
__global__ void k_chunk_leaf(int dep, const uint32_t* __restrict__ wptr, const uint32_t* __restrict__ bptr,
                             uint32_t* __restrict__ witem, uint32_t* __restrict__ bitem, uint32_t cap,
                             uint32_t* __restrict__ nz)
{
    const int64_t nl = (int64_t)1 << (2 * dep);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nl; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t w1 = min(wptr[i + 1], cap), b1 = min(bptr[i + 1], cap);
        for (uint32_t c = wptr[i]; c < w1; c++) witem[c] = (uint32_t)i;
        for (uint32_t c = bptr[i]; c < b1; c++) bitem[c] = (uint32_t)i;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *nz = min(min(wptr[nl], cap) + min(bptr[nl], cap), cap);
}

// Sources staged per warp (a block item stages kNearWarps times as many), in
// the sink leaf's frame.  The whole near list of a sink leaf is usually a few
// hundred particles, so one or two fills (256 measured 0.4 % slower per step; 768,
// whose 24 KB per block leaves room for one block fewer per SM, 1.6 % slower).
#ifndef TC_NEAR_BUF
#define TC_NEAR_BUF 512
#endif
constexpr int kNearBuf = TC_NEAR_BUF;
// Padding source: far enough that its force factor underflows to zero and its
// pair term (~1e-18 gravity, ~1e-36 t-SNE) is absorbed by any real sum.
constexpr float kFarAway = 1.0e18f;

// One sink (px, py) against its share of the staged sources: g lanes share a
// sink, lane r of the group takes 16-byte slots r, r + g, r + 2g, ... (two
// sources each, stored (x0, x1, y0, y1) so that each pair of coordinates is
// one packed FP32x2 operand; consecutive lanes read consecutive slots, so the
// group's loads are conflict-free and the groups' identical loads
// broadcast).  Both sources of a slot go through each instruction together
// (fma/add/sub/mul.f32x2), halving the instructions per pair; the two
// partial sums per accumulator are added at the end.  n4 is a multiple of 4g,
// so every lane runs the same number of trips.
template <typename KN>
__device__ __forceinline__ void p2p_staged(const KN& ker, const float4* __restrict__ s4, uint32_t n4, uint32_t r,
                                           uint32_t g, float px, float py, float& gx, float& gy, float& zs)
{
    const unsigned long long px2 = f2_pack(px, px), py2 = f2_pack(py, py);
    unsigned long long ax = 0ull, ay = 0ull, az = 0ull;  // packed +0.0f, +0.0f
    for (uint32_t j = r; j < n4; j += 4 * g) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const float4 t4 = s4[j + u * g];
            const unsigned long long Rx = f2_sub(px2, f2_pack(t4.x, t4.y));
            const unsigned long long Ry = f2_sub(py2, f2_pack(t4.z, t4.w));
            unsigned long long a, tt;
            ker.near_xy2(Rx, Ry, a, tt);
            ax = f2_fma(a, Rx, ax);
            ay = f2_fma(a, Ry, ay);
            az = f2_add(az, tt);
        }
    }
    float a0, a1;
    f2_unpack(ax, a0, a1);
    gx += KN::kSign * (a0 + a1);
    f2_unpack(ay, a0, a1);
    gy += KN::kSign * (a0 + a1);
    f2_unpack(az, a0, a1);
    zs += KN::kSign * (a0 + a1);
}

// Direct P2P of a leaf S's sinks with every particle of near(S); each sink's
// FP32 force goes to nearf (sorted order).  It reads nothing the far field
// writes, so it runs on a stream of its own beside the far field.
// * The near list is read 32 entries at a time, one per lane (index, first
//   particle, count, frame offset), and broadcast by shuffles.
// * Its particles are staged into shared memory shifted into S's
//   cell-relative frame (x_T + (cell_T - cell_S) h), so the inner loop is one
//   unrolled pass over a flat array, padded with far-away sources.
// * A warp's m sinks get g = 2^floor(log2(32/m)) lanes each, which split the
//   sources; their partial forces are summed by shuffles.
// One item routine serves both kinds of work item: a warp item (a leaf of up
// to 32 particles, a warp staging into its own buffer) and a block item (up
// to kBlockSinks sinks of a larger leaf: the block's warps stage the list once
// into the block's buffer, each warp a different run of 32 positions, and
// each computes its own 32 sinks against it; a warp past the leaf's end only
// stages).  Every count that steers the staging is the same in all the
// item's warps (they read the same entries), so the block's barriers are
// reached uniformly.  Returns the warp's pair sum.
template <bool kBlk, typename KN>
__device__ __forceinline__ float near_item(const KN& ker, int dep, float h, const uint32_t* __restrict__ count,
                                           const uint32_t* __restrict__ first, const uint32_t* __restrict__ near_ptr,
                                           const uint32_t* __restrict__ near_idx, const float2* __restrict__ prel2,
                                           uint32_t n, float2* __restrict__ nearf, int64_t si, uint32_t c0,
                                           uint32_t m, float* buf, uint32_t cap, uint32_t& n_pp)
{
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t run0 = kBlk ? 32u * w : 0u, rstep = kBlk ? 32u * kNearWarps : 32u;
    auto sync = [&]() {
        if constexpr (kBlk)
            __syncthreads();
        else
            __syncwarp();
    };
    const float4* buf4 = reinterpret_cast<const float4*>(buf);
    auto stage = [&](uint32_t q, float x, float y) {
        buf[(q >> 1) * 4 + (q & 1)] = x;
        buf[(q >> 1) * 4 + 2 + (q & 1)] = y;
    };
    const uint32_t li = level_index(dep);
    const int64_t S = li + si;
    const uint32_t fS = first[S];
    uint32_t g = 32u, r = lane, sk = 0u;
    if (m > 0u) {
        const uint32_t lg = 5u - (32u - __clz(m - 1u));  // log2 g, g * m <= 32
        g = 1u << lg;
        r = lane & (g - 1u);
        sk = lane >> lg;
    }
    const bool act = sk < m;
    const uint32_t s = fS + c0 + (act ? sk : 0u);
    const int isx = (int)compact16((uint32_t)si), isy = (int)compact16((uint32_t)si >> 1);
    const float2 p2 = act ? prel2[s] : make_float2(0.f, 0.f);
    const float px = p2.x, py = p2.y;
    float gx = 0.f, gy = 0.f, zs = 0.f;
    uint32_t fill = 0, staged = 0;
    bool has_self = false;
    const uint32_t e0 = near_ptr[si], e1 = near_ptr[si + 1];
    for (uint32_t eb = e0; eb < e1; eb += 32) {
        const uint32_t nt = min(32u, e1 - eb);
        uint32_t mf = 0, mc = 0;
        float mox = 0.f, moy = 0.f;
        if (lane < nt) {
            const uint32_t ti = near_idx[eb + lane];
            mf = first[li + ti];
            mc = count[li + ti];
            mox = (float)((int)compact16(ti) - isx) * h;
            moy = (float)((int)compact16(ti >> 1) - isy) * h;
            has_self |= ti == (uint32_t)si;
        }
        // the batch's particles as one flat range [0, tot): position q
        // belongs to entry t with ex_t <= q < ex_t + c_t (exclusive
        // prefix ex over the lanes).  Every entry is a non-empty leaf, so
        // the entries' first positions are distinct and t is the number
        // of entries starting at or before q, minus one
        uint32_t inc = mc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= (uint32_t)o) inc += v;
        }
        const uint32_t ex = inc - mc, tot = __shfl_sync(0xffffffffu, inc, 31);
        for (uint32_t q0 = 0; q0 < tot;) {
            if (fill == cap) {
                // evaluate the staged sources (cap is a multiple of 8g)
                sync();
                if (act) p2p_staged(ker, buf4, cap / 2, r, g, px, py, gx, gy, zs);
                sync();
                staged += fill;
                fill = 0;
            }
            const uint32_t take = min(tot - q0, cap - fill);
            for (uint32_t b0 = run0; b0 < take; b0 += rstep) {
                const uint32_t base = q0 + b0, q = base + lane;
                // entries starting before this run of 32 positions, and a bit per entry starting in it
                const uint32_t before = __popc(__ballot_sync(0xffffffffu, lane < nt && ex < base));
                const uint32_t d = ex - base;  // < 32 only for an entry starting in the run
                const uint32_t bits = __reduce_or_sync(0xffffffffu, (lane < nt && d < 32u) ? 1u << d : 0u);
                // in [0, nt): entry 0 starts at position 0
                const uint32_t t = before + __popc(bits & (0xffffffffu >> (31u - lane))) - 1u;
                const uint32_t fT = __shfl_sync(0xffffffffu, mf, t), eT = __shfl_sync(0xffffffffu, ex, t);
                const float ox = __shfl_sync(0xffffffffu, mox, t), oy = __shfl_sync(0xffffffffu, moy, t);
                if (b0 + lane < take) {
                    // the particle index stays below n even for a list that broke the non-empty rule
                    const uint32_t src = fT + (q - eT);
                    const float2 t2 = src < n ? prel2[src] : make_float2(kFarAway, kFarAway);
                    stage(fill + b0 + lane, t2.x + ox, t2.y + oy);
                }
            }
            fill += take;
            q0 += take;
        }
    }
    if (fill > 0) {
        // padded with far-away sources to a multiple of 8g (block items: of 8 * 32, every warp's g)
        const uint32_t pad = kBlk ? 256u : 8u * g;
        const uint32_t n8 = (fill + pad - 1u) / pad * pad;
        for (uint32_t q = fill + (kBlk ? threadIdx.x : lane); q < n8; q += kBlk ? 32u * kNearWarps : 32u)
            stage(q, kFarAway, kFarAway);
        sync();
        if (act) p2p_staged(ker, buf4, ((fill + 8u * g - 1u) / (8u * g) * (8u * g)) / 2, r, g, px, py, gx, gy, zs);
        sync();
        staged += fill;
    }
    has_self = __any_sync(0xffffffffu, has_self);
    // the g lanes of a sink hold partial forces: sum them into lane r = 0
    for (uint32_t o = g >> 1; o > 0; o >>= 1) {
        gx += __shfl_xor_sync(0xffffffffu, gx, o);
        gy += __shfl_xor_sync(0xffffffffu, gy, o);
    }
    if (act && r == 0) {
        n_pp += staged;
        if (has_self) {
            // the staged sources included the sink itself: R = 0 adds no
            // force but adds the kernel's pair term at r = 0, removed here
            float D1, t0;
            ker.near_xy(0.0f, 0.0f, D1, t0);
            zs -= t0;
            n_pp--;
        }
        nearf[s] = make_float2(gx, gy);
    }
    // the warp's pair sum: FP32 over the lanes (each lane's partial is an FP32 sum already)
    return warp_sum(act ? zs : 0.0f);
}

// Block items first (each block takes whole items), then warp items (each
// warp its own); per item one FP64 pair-sum word in zwork: warp items at
// [0, nw), block items after them.
template <typename KN>
#ifndef TC_NEAR_MIN_WARPS
#define TC_NEAR_MIN_WARPS 40  // resident warps per SM the near field's registers are held to (48: no spills)
#endif
__global__ void __launch_bounds__(32 * kNearWarps, TC_NEAR_MIN_WARPS / kNearWarps)
    k_near_p(KN ker, int dep, float h, const uint32_t* __restrict__ count, const uint32_t* __restrict__ first,
             const uint32_t* __restrict__ near_ptr, const uint32_t* __restrict__ near_idx,
             const uint32_t* __restrict__ wptr, const uint32_t* __restrict__ witem,
             const uint32_t* __restrict__ bptr, const uint32_t* __restrict__ bitem, uint32_t cap,
             const float* __restrict__ prel, uint32_t n, float2* __restrict__ nearf, double* __restrict__ zwork,
             unsigned long long* __restrict__ counters)
{
    // staged sources, two per 16-byte slot as (x0, x1, y0, y1): the whole
    // array for a block item, a quarter per warp for warp items
    __shared__ __align__(16) float s_src[kNearWarps * 2 * kNearBuf];
    __shared__ float s_z[kNearWarps];
    uint32_t n_pp = 0;
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const float2* prel2 = reinterpret_cast<const float2*>(prel);
    const uint32_t li = level_index(dep);
    const int64_t nl = (int64_t)1 << (2 * dep);
    const uint32_t nw = min(wptr[nl], cap), nb = min(bptr[nl], cap);
    for (uint32_t bi = blockIdx.x; bi < nb; bi += gridDim.x) {
        const int64_t si = bitem[bi];
        const uint32_t cS = count[li + si];
        const uint32_t c0 = (bi - bptr[si]) * kBlockSinks + 32u * w;
        const uint32_t m = cS > c0 ? min(32u, cS - c0) : 0u;
        const float z = near_item<true>(ker, dep, h, count, first, near_ptr, near_idx, prel2, n, nearf, si, c0, m,
                                        s_src, (uint32_t)(kNearWarps * kNearBuf), n_pp);
        if (lane == 0) s_z[w] = z;
        __syncthreads();
        if (threadIdx.x == 0 && nw + bi < cap) {
            float zb = 0.f;
#pragma unroll
            for (int i = 0; i < kNearWarps; i++) zb += s_z[i];
            zwork[nw + bi] = (double)zb;
        }
        __syncthreads();
    }
    const int64_t wstride = (int64_t)gridDim.x * kNearWarps;
    for (int64_t wi = blockIdx.x * (int64_t)kNearWarps + w; wi < nw; wi += wstride) {
        const int64_t si = witem[wi];
        const uint32_t cS = count[li + si];  // 1..32
        const float z = near_item<false>(ker, dep, h, count, first, near_ptr, near_idx, prel2, n, nearf, si, 0u, cS,
                                         s_src + w * 2 * kNearBuf, (uint32_t)kNearBuf, n_pp);
        if (lane == 0) zwork[wi] = (double)z;
    }
    const unsigned long long a = warp_sum((unsigned long long)n_pp);
    if (lane == 0 && a) atomicAdd(counters + 0, a);
}

// L2P of the final local expansion of each particle's leaf plus the particle's
// near-field force, written (or added) in FP64:
//   F_x = (1/h) sum_{a+b<P} L_{a+1,b} w_{a,b},  F_y = (1/h) sum L_{a,b+1} w_{a,b},
// w_{a,b} = dx^a/a! dy^b/b!.  One thread per particle in sorted order; the
// leaf comes from the particle's sorted Morton code.  The leaf's coefficients
// are read in storage order, 16 bytes at a time (a warp's particles lie in a
// few leaves, so each read is a few L1 lines), and each goes to the x and y
// sums it belongs to.  (Staging a tile's leaves in shared memory costs more:
// a leaf holds about ten particles, so the per-leaf copy is as long as the
// evaluation.)
template <int P>
__global__ void __launch_bounds__(128) k_l2p_p(int dep, float h, int64_t n, const uint32_t* __restrict__ codes,
                                             const float* __restrict__ comrel, const float* __restrict__ loc,
                                             const float* __restrict__ prel, const float2* __restrict__ nearf,
                                             const uint32_t* __restrict__ perm, double* __restrict__ grad,
                                             int accumulate, int scatter, int vec16)
{
    constexpr int K = ncoef(P), KS = kstride(P), KW = ncoef(P - 1);
    const uint32_t li = level_index(dep);
    const int shift = 32 - 2 * dep;
    const float ih = 1.0f / h;
    const float2* prel2 = reinterpret_cast<const float2*>(prel);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t S = li + (dep ? (codes[k] >> shift) : 0u);
        const float2 p2 = prel2[k];
        const float2 f = nearf[k];
        const uint32_t pm = scatter ? perm[k] : 0u;
        float wv[KW];
        monomials<P - 1>((p2.x - comrel[2 * S]) * ih, (p2.y - comrel[2 * S + 1]) * ih, wv);
        const float4* L4 = reinterpret_cast<const float4*>(loc + S * KS);
        float lx = 0.f, ly = 0.f;
#pragma unroll
        for (int c = 0; c < KS / 4; c++) {
            const float4 q = L4[c];
            const float qv[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int i = 4 * c + j;
                if (i >= K) continue;
                const int d = cdeg(i), bb = i - d * (d + 1) / 2, aa = d - bb;  // coefficient (aa, bb)
                if (aa >= 1) lx = fmaf(qv[j], wv[cidx(aa - 1, bb)], lx);
                if (bb >= 1) ly = fmaf(qv[j], wv[cidx(aa, bb - 1)], ly);
            }
        }
        const int64_t o = scatter ? (int64_t)pm : k;
        double ox2 = f64_of_f32(lx * ih + f.x), oy2 = f64_of_f32(ly * ih + f.y);
        if (vec16) {
            // one 16-byte access per particle (the scattered order makes each its own transaction)
            double2* g2 = reinterpret_cast<double2*>(grad) + o;
            if (accumulate) {
                const double2 a = *g2;
                ox2 += a.x;
                oy2 += a.y;
            }
            *g2 = make_double2(ox2, oy2);
        } else {
            if (accumulate) {
                ox2 += grad[2 * o];
                oy2 += grad[2 * o + 1];
            }
            grad[2 * o] = ox2;
            grad[2 * o + 1] = oy2;
        }
    }
}

__global__ void k_sum_z2(const double* __restrict__ a, int64_t na, const double* __restrict__ c,
                         const uint32_t* __restrict__ nc, double* __restrict__ out)
{
    __shared__ double ws[32];
    double s = 0.0;
    const int64_t ncv = *nc;
    for (int64_t i = threadIdx.x; i < na; i += blockDim.x) s += a[i];
    for (int64_t i = threadIdx.x; i < ncv; i += blockDim.x) s += c[i];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) *out = *out + v;
    }
}

// M2L of every level on the tensor cores (box-centred expansions): the level's
// operators, the BF16 hi/lo multipole rows, then one persistent launch per
// level writing loc and zpart as the SIMT M2L does
template <int Q>
int m2l_tensor(Handle& h, const PotParams& pp)
{
    using S = tcm::Shape<Q>;
    cudaStream_t s = h.stream;
    const int dep = h.depth;
    if (h.centre != TC_CENTRE_BOX) {
        tc_set_error("tensor-core M2L: needs box-centred expansions (tc_set_expansion_centre)");
        return TC_ERR_STATE;
    }
    if (h.adapt || h.ctrl_on) {
        tc_set_error("tensor-core M2L: fixed order only (no per-pair orders or controller)");
        return TC_ERR_STATE;
    }
    const int R = tcm::offset_radius(h.mac == TC_MAC_BMAX, h.cfg.theta);
    if (R > tcm::kMaxR) {
        tc_set_error("tensor-core M2L: theta %g reaches offsets beyond %d cells", h.cfg.theta, tcm::kMaxR);
        return TC_ERR_INVALID;
    }
    const int W = 2 * R + 1;
    const size_t ops_level = (size_t)W * W * 2 * S::OPB;
    int rc;
    if ((rc = ensure(h.tc_ops, ops_level * (dep + 1))) ||
        (rc = ensure(h.tc_mubf, (size_t)h.nnodes * 2 * S::ROWB)))
        return rc;
    static bool attr_set = false;
    if (!attr_set) {
        TC_CUDA_TRY(cudaFuncSetAttribute(tcm::k_m2l_tc<Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM));
        attr_set = true;
    }
    uint32_t* status = P<uint32_t>(h.err) + 6;
    TC_CUDA_TRY(cudaMemsetAsync(status, 0, 4, s));
    const uint32_t* act = P<uint32_t>(h.act);
    const uint32_t* act_pos = P<uint32_t>(h.act_pos);
    const float* comrel = P<float>(h.comrel);
    float* mu = P<float>(h.mu);
    float* loc = P<float>(h.loc);
    double* zp = P<double>(h.zpart);
    const uint32_t* count = P<uint32_t>(h.count);
    const uint32_t* ptr = P<uint32_t>(h.ptr_pool);
    const uint32_t* idx = P<uint32_t>(h.idx_pool);
    // levels with few parents keep the SIMT kernels: a tile's offsets run one after another, so a level
    // needs tiles for every SM before the tensor cores pay
    int lmin = dep + 1;
    for (int l = dep; l >= 2 && ((int64_t)1 << (2 * (l - 1))) >= (int64_t)tcm::kRows * sm_count(); l--) lmin = l;
    if (h.m2l_tc_all) lmin = 1;
    if (lmin <= dep) {
        tcm::k_mu_split<Q><<<grid_for((int64_t)h.nnodes * S::KC, 256), 256, 0, s>>>(
            h.nnodes, level_index(lmin), mu, act, act_pos, P<uint8_t>(h.tc_mubf));
        h.launches++;
    }
    for (int l = 1; l <= dep; l++) {
        const float hl = (float)(h.L / (double)(1u << l));
        const int64_t nl = (int64_t)1 << (2 * l);
        if (l < lmin) {
            if (nl <= kM2lWarpLevelNodes)
                k_m2l_warp<Q><<<grid_for(nl * 32, 128), 128, 0, s>>>(l, hl, pp, ptr + h.lists.nn_ptr_off[l],
                                                                   idx + h.lists.nn_idx_off[l], comrel, mu, loc,
                                                                   zp, act, act_pos);
            else
                k_m2l_p<Q><<<grid_for(nl, 128), 128, 0, s>>>(l, hl, pp, ptr + h.lists.nn_ptr_off[l],
                                                             idx + h.lists.nn_idx_off[l], count, comrel, mu, loc,
                                                             zp, act, act_pos);
            h.launches++;
            continue;
        }
        uint8_t* ops = P<uint8_t>(h.tc_ops) + ops_level * l;
        tcm::k_m2l_tc_ops<Q><<<W * W, 128, 0, s>>>(hl, pp, R, ops);
        const int64_t tiles = 4 * ((nl / 4 + tcm::kRows - 1) / tcm::kRows);
        const int grid = (int)(tiles < sm_count() ? tiles : sm_count());
        tcm::k_m2l_tc<Q><<<grid, 128, S::SMEM, s>>>(l, R, ptr + h.lists.nn_ptr_off[l], idx + h.lists.nn_idx_off[l],
                                                     count, mu, P<uint8_t>(h.tc_mubf), ops, pp.kappa, loc, zp,
                                                     act, act_pos, status);
        h.launches += 2;
    }
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

template <int ORD, typename KN>
int solve_p(Handle& h, KN ker, const PotParams& pp, double* d_grad, int accumulate, int scatter, double* d_total)
{
    constexpr int K = ncoef(ORD);
    cudaStream_t s = h.stream;
    const int dep = h.depth;
    const int64_t nn = h.nnodes;
    const int64_t nleaf = (int64_t)1 << (2 * dep);
    const int64_t wmax = h.n / 32 + (h.n < nleaf ? h.n : nleaf) + 1;
    int rc;
    if ((rc = ensure(h.mu, nn * kstride(ORD) * 4)) || (rc = ensure(h.loc, nn * kstride(ORD) * 4)) ||
        (rc = ensure(h.zpart, nn * 8 + 64)) ||
        (rc = ensure(h.counters, 64)) || (rc = ensure(h.zwork, wmax * 8)) || (rc = ensure(h.nearf, h.n * 8)) ||
        (rc = ensure_near_stream(h)) || (rc = record(h, 4)))
        return rc;
    TC_CUDA_TRY(cudaMemsetAsync(h.counters.p, 0, 64, s));
    h.stage_split = true;
    // the near field (P2P) reads only the tree and its lists: it runs on a second stream from here, beside
    // the far field, and the L2P after both joins the two
    cudaStream_t sn = s;
    if (h.near_overlap) {
        sn = h.near_stream;
        TC_CUDA_TRY(cudaEventRecord(h.ev_fork, s));
        TC_CUDA_TRY(cudaStreamWaitEvent(sn, h.ev_fork, 0));
    }
    const uint32_t* count_n = P<uint32_t>(h.count);
    if ((rc = record_on(h, 8, sn))) return rc;
    if (!h.items_ready) {
        // the work-item tables, unless the update built them beside its list build
        const cudaStream_t main = h.stream;
        h.stream = sn;
        rc = near_items(h);
        h.stream = main;
        if (rc) return rc;
    }
    const uint32_t* wptr = P<uint32_t>(h.chunk);
    const uint32_t* bptr = wptr + (nleaf + 1);
    const uint32_t* nz = bptr + (nleaf + 1);  // pair-sum words the near field writes
    const uint32_t* witem = P<uint32_t>(h.chunk_leaf);
    const uint32_t* bitem = witem + wmax;
    {
        const int64_t wblk = (wmax + kNearWarps - 1) / kNearWarps;
        const uint32_t* ptr_n = P<uint32_t>(h.ptr_pool);
        const uint32_t* idx_n = P<uint32_t>(h.idx_pool);
        k_near_p<KN><<<(unsigned)(wblk < sm_count() * 256 ? wblk : sm_count() * 256), 32 * kNearWarps, 0, sn>>>(
            ker, dep, (float)(h.L / (double)(1u << dep)), count_n, P<uint32_t>(h.first),
            ptr_n + h.lists.near_ptr_off[dep], idx_n + h.lists.near_idx_off[dep], wptr, witem, bptr, bitem,
            (uint32_t)wmax, P<float>(h.prel), (uint32_t)h.n, P<float2>(h.nearf), P<double>(h.zwork),
            P<unsigned long long>(h.counters));
    }
    if ((rc = record_on(h, 9, sn))) return rc;
    if (h.near_overlap) TC_CUDA_TRY(cudaEventRecord(h.ev_join, sn));
    // the far field: beside the near field it runs on a stream of higher priority, so that its chain of
    // dependent launches takes SMs first as near-field blocks retire (the handle's stream points there
    // until the join; the guard restores it on every exit)
    const cudaStream_t s_call = s;
    struct StreamSwap {
        Handle& hh;
        cudaStream_t saved;
        ~StreamSwap() { hh.stream = saved; }
    } swap{h, h.stream};
    if (h.near_overlap) {
        TC_CUDA_TRY(cudaStreamWaitEvent(h.far_stream, h.ev_fork, 0));
        h.stream = h.far_stream;
        s = h.far_stream;
    }
    if ((rc = record(h, 11))) return rc;  // the far field starts
    float* mu = P<float>(h.mu);
    float* loc = P<float>(h.loc);
    double* zp = P<double>(h.zpart);
    const float* comrel = P<float>(h.comrel);
    const uint32_t* count = P<uint32_t>(h.count);
    auto hl = [&](int l) { return (float)(h.L / (double)(1u << l)); };
    if (h.mu_stride != kstride(ORD)) {
        tc_set_error("order-p solve: multipoles of another order (update the tree first)");
        return TC_ERR_STATE;
    }
    const uint32_t* ptr = P<uint32_t>(h.ptr_pool);
    const uint32_t* idx = P<uint32_t>(h.idx_pool);
    // fixed order below 10: the fine levels' L2L runs inside their M2L launch (after the coarse levels' L2L)
    bool per_pair = false;
    if constexpr (ORD == 12) per_pair = h.ctrl_on || h.adapt;
    else if constexpr (ORD >= 6) per_pair = h.adapt;
    const bool tc_m2l = h.m2l_tc;
    const bool fuse = ORD < 10 && !per_pair && !tc_m2l;
    // a captured step's update ran the coarse levels (and the clearing) beside its list build
    const bool coarse_done = h.coarse_ready && fuse;
    if (!coarse_done) {
        TC_CUDA_TRY(cudaMemsetAsync(loc, 0, kstride(ORD) * 4, s));
        TC_CUDA_TRY(cudaMemsetAsync(zp, 0, nn * 8, s));
    }
    int nfused = 0;
    if (tc_m2l) {
        if ((rc = m2l_tensor<ORD>(h, pp))) return rc;
    }
    for (int l = 1; l <= dep && !tc_m2l; l++) {
        const int64_t nl = (int64_t)1 << (2 * l);
        if (fuse && nl > kM2lWarpLevelNodes) continue;
        if (coarse_done && nl <= kM2lWarpLevelNodes) continue;
        const uint32_t* np_ = ptr + h.lists.nn_ptr_off[l];
        const uint32_t* ni_ = idx + h.lists.nn_idx_off[l];
        bool mixed = false;
        const uint8_t* od = P<uint8_t>(h.ord_pool) + h.lists.nn_idx_off[l];
        const uint32_t* act = P<uint32_t>(h.act);
        const uint32_t* act_pos = P<uint32_t>(h.act_pos);
        const bool coarse = nl <= kM2lWarpLevelNodes;
        if constexpr (ORD == 12) {
            if (h.ctrl_on || h.adapt) {
                if (coarse) {
                    k_m2l_mixed_warp<12, 8, 0, 2><<<grid_for(nl * 32, 128), 128, 0, s>>>(
                        l, hl(l), pp, np_, ni_, od, comrel, mu, loc, zp, act, act_pos);
                    k_m2l_mixed_warp<12, 12, 3, 4><<<grid_for(nl * 32, 128), 128, 0, s>>>(
                        l, hl(l), pp, np_, ni_, od, comrel, mu, loc, zp, act, act_pos);
                } else {
                    k_m2l_mixed<12, 8, 0, 2><<<grid_for(nl, 128), 128, 0, s>>>(l, hl(l), pp, np_, ni_, od, count,
                                                                               comrel, mu, loc, zp, act, act_pos);
                    k_m2l_mixed<12, 12, 3, 4><<<grid_for(nl, 128), 128, 0, s>>>(l, hl(l), pp, np_, ni_, od, count,
                                                                                comrel, mu, loc, zp, act, act_pos);
                }
                h.launches++;
                mixed = true;
            }
        } else if constexpr (ORD >= 6) {
            if (h.adapt) {
                constexpr int OB = (ORD - 4) / 2;  // the bucket of order ORD
                if (coarse)
                    k_m2l_mixed_warp<ORD, ORD, 0, OB><<<grid_for(nl * 32, 128), 128, 0, s>>>(
                        l, hl(l), pp, np_, ni_, od, comrel, mu, loc, zp, act, act_pos);
                else
                    k_m2l_mixed<ORD, ORD, 0, OB><<<grid_for(nl, 128), 128, 0, s>>>(l, hl(l), pp, np_, ni_, od, count,
                                                                                  comrel, mu, loc, zp, act, act_pos);
                mixed = true;
            }
        }
        if (!mixed) {
            if (nl <= kM2lWarpLevelNodes)
                k_m2l_warp<ORD><<<grid_for(nl * 32, 128), 128, 0, s>>>(l, hl(l), pp, np_, ni_, comrel, mu, loc, zp,
                                                                       act, act_pos);
            else
                k_m2l_p<ORD><<<grid_for(nl, 128), 128, 0, s>>>(l, hl(l), pp, np_, ni_, count, comrel, mu, loc, zp,
                                                               act, act_pos);
        }
    }
    for (int l = 1; l <= dep; l++) {
        const int64_t nl = (int64_t)1 << (2 * l);
        if (coarse_done && nl <= kM2lWarpLevelNodes) continue;
        if constexpr (ORD < 10) {
            if (fuse && nl > kM2lWarpLevelNodes) {
                k_m2l_p<ORD, true><<<grid_for(nl, 128), 128, 0, s>>>(
                    l, hl(l), pp, ptr + h.lists.nn_ptr_off[l], idx + h.lists.nn_idx_off[l], count, comrel, mu, loc,
                    zp, P<uint32_t>(h.act), P<uint32_t>(h.act_pos));
                nfused++;
                continue;
            }
        }
        if constexpr (ORD >= 10)
            k_l2l_stream<ORD><<<grid_for(nl, 128), 128, 0, s>>>(l, hl(l), count, comrel, loc, P<uint32_t>(h.act), P<uint32_t>(h.act_pos));
        else
            k_l2l<ORD><<<grid_for(nl, 128), 128, 0, s>>>(l, hl(l), count, comrel, loc, P<uint32_t>(h.act), P<uint32_t>(h.act_pos));
    }
    // the far field's pair-sum parts, one word per node, summed on its stream while the near field runs
    const int64_t nsum = sum_tmp_doubles();
    if ((rc = ensure(h.sumtmp, (2 * nsum + 1) * 8))) return rc;
    double* zfar = P<double>(h.sumtmp) + 2 * nsum;
    if ((rc = sum_f64(zp, nn, nullptr, nullptr, zfar, 0, P<double>(h.sumtmp), s))) return rc;
    if ((rc = record(h, 5))) return rc;
    if (h.near_overlap) {
        TC_CUDA_TRY(cudaEventRecord(h.ev_far, s));
        h.stream = swap.saved;
        s = s_call;
        TC_CUDA_TRY(cudaStreamWaitEvent(s, h.ev_far, 0));
        TC_CUDA_TRY(cudaStreamWaitEvent(s, h.ev_join, 0));
    }
    if (h.wait_grad) {
        // the caller's gradient, copied in on the copy stream behind the far and near fields, is added to
        // from here on
        TC_CUDA_TRY(cudaStreamWaitEvent(s, h.ev_grad, 0));
        h.wait_grad = false;
    }
    if ((rc = record(h, 10))) return rc;
    k_l2p_p<ORD><<<grid_for(h.n, 128, sm_count() * 12), 128, 0, s>>>(dep, hl(dep), h.n, P<uint32_t>(h.codes), comrel, loc,
                                                     P<float>(h.prel), P<float2>(h.nearf), P<uint32_t>(h.perm),
                                                     d_grad, accumulate, scatter,
                                                     (reinterpret_cast<uintptr_t>(d_grad) & 15) == 0);
    if ((rc = record(h, 6))) return rc;
    // the pair sum: the far field's total plus the near field's per-item words
    if ((rc = sum_f64(zfar, 1, P<double>(h.zwork), nz, d_total, 1, P<double>(h.sumtmp) + nsum, s))) return rc;
    // far field (an M2L and an L2L launch per level, one fused launch per fine level), the near field, the
    // L2P and two two-kernel sums; the item tables and a captured update's coarse levels count themselves
    h.launches += 2 * dep - nfused + 6 - (coarse_done ? 2 * kFarCoarseLevel : 0);
    TC_CUDA_TRY(cudaGetLastError());
    if (tc_m2l) {
        // the tensor-core M2L's status word (list offsets beyond its operators, a bounded wait that gave up)
        TC_CUDA_TRY(cudaMemcpyAsync(h.h_words + 48, P<uint32_t>(h.err) + 6, 4, cudaMemcpyDeviceToHost, s));
        if (!h.nosync) {
            TC_CUDA_TRY(cudaStreamSynchronize(s));
            if (h.h_words[48]) {
                tc_set_error("tensor-core M2L: %s", (h.h_words[48] & tcm::kErrTimeout)
                                                          ? "a bounded device wait gave up"
                                                          : "a list offset beyond the operator table");
                return (h.h_words[48] & tcm::kErrTimeout) ? TC_ERR_TIMEOUT : TC_ERR_INVALID;
            }
        }
    }
    return record(h, 7);
}

template <int ORD>
int multipoles_p(Handle& h)
{
    cudaStream_t s = h.stream;
    const int dep = h.depth;
    const int64_t nn = h.nnodes;
    const int64_t nleaf = (int64_t)1 << (2 * dep);
    int rc;
    if ((rc = ensure(h.mu, nn * kstride(ORD) * 4))) return rc;
    float* mu = P<float>(h.mu);
    const float* comrel = P<float>(h.comrel);
    const uint32_t* count = P<uint32_t>(h.count);
    auto hl = [&](int l) { return (float)(h.L / (double)(1u << l)); };
    k_p2m_small<ORD><<<grid_for(nleaf, 128), 128, 0, s>>>(dep, hl(dep), count, P<uint32_t>(h.first), comrel,
                                                         P<float>(h.prel), mu, P<uint32_t>(h.act), P<uint32_t>(h.act_pos));
    k_p2m<ORD><<<grid_for((h.n / (kLeafSmall + 1) + 1) * 32, 128), 128, 0, s>>>(
        dep, hl(dep), count, P<uint32_t>(h.first), comrel, P<float>(h.prel), P<uint32_t>(h.bigleaf), mu);
    for (int l = dep - 1; l >= 0; l--) {
        const int64_t nl = (int64_t)1 << (2 * l);
        if (nl <= kM2mQuadLevelNodes)
            k_m2m_quad<ORD><<<grid_for(nl * 4, 128), 128, 0, s>>>(l, hl(l), count, comrel, mu, P<uint32_t>(h.act),
                                                                  P<uint32_t>(h.act_pos));
        else if constexpr (ORD >= 10)
            k_m2m_stream<ORD><<<grid_for(nl, 128), 128, 0, s>>>(l, hl(l), count, comrel, mu, P<uint32_t>(h.act), P<uint32_t>(h.act_pos));
        else
            k_m2m<ORD><<<grid_for(nl, 128), 128, 0, s>>>(l, hl(l), count, comrel, mu, P<uint32_t>(h.act), P<uint32_t>(h.act_pos));
    }
    h.launches += 2 + dep;
    h.mu_stride = kstride(ORD);
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

// the kernel's parameters for the expansion kernels
PotParams make_pp(const Handle& h)
{
    PotParams pp;
    pp.kind = h.cfg.kernel;
    pp.dipole = h.centre == TC_CENTRE_BOX;
    if (h.cfg.kernel == TC_KERNEL_GRAVITY) {
        pp.nu = 0.5f;
        pp.c = (float)(h.cfg.softening * h.cfg.softening);
        pp.kappa = -1.0f;
    } else {
        pp.nu = 1.0f;
        pp.c = 1.0f;
        pp.kappa = -2.0f;
    }
    return pp;
}

template <int P>
int dispatch_kernel(Handle& h, double* d_grad, int accumulate, int scatter, double* d_total)
{
    const PotParams pp = make_pp(h);
    if (h.cfg.kernel == TC_KERNEL_GRAVITY)
        return solve_p<P>(h, KGrav<float>{pp.c}, pp, d_grad, accumulate, scatter, d_total);
    return solve_p<P>(h, KTsne<float>{}, pp, d_grad, accumulate, scatter, d_total);
}

// The fused fixed-order path's coarse levels: the local expansions zeroed
// (root) and the pair-sum parts cleared, M2L of levels 1..kFarCoarseLevel (a
// warp per sink node), then their L2L in order.  The solve continues from
// level kFarCoarseLevel + 1.  Returns 1, queueing nothing, when an earlier
// solve has not sized the buffers for this tree and order (nothing may be
// allocated here: the call runs inside a captured update).
template <int ORD>
int far_coarse_p(Handle& h, const PotParams& pp)
{
    cudaStream_t s = h.stream;
    if (h.mu_stride != kstride(ORD) || h.loc.bytes < (size_t)h.nnodes * kstride(ORD) * 4 ||
        h.zpart.bytes < (size_t)h.nnodes * 8)
        return 1;
    const int dep = h.depth;
    const int lc = dep < kFarCoarseLevel ? dep : kFarCoarseLevel;
    float* mu = P<float>(h.mu);
    float* loc = P<float>(h.loc);
    double* zp = P<double>(h.zpart);
    const float* comrel = P<float>(h.comrel);
    const uint32_t* count = P<uint32_t>(h.count);
    const uint32_t* ptr = P<uint32_t>(h.ptr_pool);
    const uint32_t* idx = P<uint32_t>(h.idx_pool);
    const uint32_t* act = P<uint32_t>(h.act);
    const uint32_t* act_pos = P<uint32_t>(h.act_pos);
    auto hl = [&](int l) { return (float)(h.L / (double)(1u << l)); };
    TC_CUDA_TRY(cudaMemsetAsync(loc, 0, kstride(ORD) * 4, s));
    TC_CUDA_TRY(cudaMemsetAsync(zp, 0, h.nnodes * 8, s));
    for (int l = 1; l <= lc; l++) {
        const int64_t nl = (int64_t)1 << (2 * l);
        k_m2l_warp<ORD><<<grid_for(nl * 32, 128), 128, 0, s>>>(l, hl(l), pp, ptr + h.lists.nn_ptr_off[l],
                                                               idx + h.lists.nn_idx_off[l], comrel, mu, loc, zp, act,
                                                               act_pos);
    }
    for (int l = 1; l <= lc; l++) {
        const int64_t nl = (int64_t)1 << (2 * l);
        k_l2l<ORD><<<grid_for(nl, 128), 128, 0, s>>>(l, hl(l), count, comrel, loc, act, act_pos);
    }
    h.launches += 2 * lc;
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

}  // namespace

// Each expansion order's kernels live in their own object: the build compiles
// this file once per order with TC_FMM_ORDER set (in parallel) and once without
// it for the order switch below.
template <int P>
int multipoles_order(Handle& h);
template <int P>
int solve_order(Handle& h, double* d_grad, double* d_total, int accumulate, int scatter);
template <int P>
int far_coarse_order(Handle& h);

#ifdef TC_FMM_ORDER
template <int P>
int multipoles_order(Handle& h)
{
    return multipoles_p<P>(h);
}

template <int P>
int solve_order(Handle& h, double* d_grad, double* d_total, int accumulate, int scatter)
{
    return dispatch_kernel<P>(h, d_grad, accumulate, scatter, d_total);
}

template <int P>
int far_coarse_order(Handle& h)
{
    if constexpr (P < 10)
        return far_coarse_p<P>(h, make_pp(h));
    else
        return TC_ERR_STATE;
}

template int multipoles_order<TC_FMM_ORDER>(Handle& h);
template int far_coarse_order<TC_FMM_ORDER>(Handle& h);
template int solve_order<TC_FMM_ORDER>(Handle& h, double* d_grad, double* d_total, int accumulate, int scatter);
#else
int near_items(Handle& h)
{
    cudaStream_t s = h.stream;
    const int dep = h.depth;
    const int64_t nleaf = (int64_t)1 << (2 * dep);
    const int64_t wmax = h.n / 32 + (h.n < nleaf ? h.n : nleaf) + 1;
    int rc;
    if ((rc = ensure(h.chunk, (2 * (nleaf + 1) + 1) * 4)) || (rc = ensure(h.chunk_leaf, 2 * wmax * 4)) ||
        (rc = ensure(h.items_cnt, 2 * nleaf * 4 + 64)) || (rc = ensure(h.items_tmp, 2 * scan_tmp_words(nleaf) * 4)))
        return rc;
    uint32_t* nwarp = P<uint32_t>(h.items_cnt);
    uint32_t* nblock = nwarp + nleaf;
    uint32_t* wptr = P<uint32_t>(h.chunk);
    uint32_t* bptr = wptr + (nleaf + 1);
    uint32_t* nz = bptr + (nleaf + 1);
    uint32_t* witem = P<uint32_t>(h.chunk_leaf);
    k_chunks<<<grid_for(nleaf, 256), 256, 0, s>>>(dep, P<uint32_t>(h.count), nwarp, nblock);
    if ((rc = exclusive_scan2_u32(nwarp, wptr, nblock, bptr, nleaf, P<uint32_t>(h.items_tmp), s))) return rc;
    k_chunk_leaf<<<grid_for(nleaf, 256), 256, 0, s>>>(dep, wptr, bptr, witem, witem + wmax, (uint32_t)wmax, nz);
    h.launches += 2 + (nleaf <= 2048 ? 1 : 3);
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

bool far_coarse_applies(const Handle& h)
{
    const int o = h.cfg.order;
    return (o == 3 || o == 4 || o == 6 || o == 8) && !h.adapt && !h.ctrl_on && !h.m2l_tc &&
           h.depth > kFarCoarseLevel;
}

int build_far_coarse(Handle& h)
{
    switch (h.cfg.order) {
    case 3: return far_coarse_order<3>(h);
    case 4: return far_coarse_order<4>(h);
    case 6: return far_coarse_order<6>(h);
    case 8: return far_coarse_order<8>(h);
    default:
        tc_set_error("coarse far field: fixed orders 3, 4, 6, 8 only");
        return TC_ERR_INVALID;
    }
}

int build_multipoles(Handle& h)
{
    switch (h.cfg.order) {
    case 3: return multipoles_order<3>(h);
    case 4: return multipoles_order<4>(h);
    case 6: return multipoles_order<6>(h);
    case 8: return multipoles_order<8>(h);
    case 10: return multipoles_order<10>(h);
    case 12: return multipoles_order<12>(h);
    default:
        tc_set_error("unsupported expansion order %d (3, 4, 6, 8, 10, 12)", h.cfg.order);
        return TC_ERR_INVALID;
    }
}

int solve_fmm_order(Handle& h, double* d_grad, double* d_total, int accumulate, int scatter)
{
    switch (h.cfg.order) {
    case 3: return solve_order<3>(h, d_grad, d_total, accumulate, scatter);
    case 4: return solve_order<4>(h, d_grad, d_total, accumulate, scatter);
    case 6: return solve_order<6>(h, d_grad, d_total, accumulate, scatter);
    case 8: return solve_order<8>(h, d_grad, d_total, accumulate, scatter);
    case 10: return solve_order<10>(h, d_grad, d_total, accumulate, scatter);
    case 12: return solve_order<12>(h, d_grad, d_total, accumulate, scatter);
    default:
        tc_set_error("unsupported expansion order %d (3, 4, 6, 8, 10, 12)", h.cfg.order);
        return TC_ERR_INVALID;
    }
}
#endif

}  // namespace tc
