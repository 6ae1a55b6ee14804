// Tensor-core M2L for box-centred order-p expansions (TC_CENTRE_BOX), on the
// 5th-generation tensor cores (tcgen05, accumulators in tensor memory).
//
// The reference's M2L (TSNE_FMM_SYM_MORTON_NN_Kernel,
// src/nbodysolvers/cpu/nBodySolverFMM_SYM_MORTON.h:622-723) translates a
// node's multipole into the local expansion of a well-separated node through
// the kernel's derivatives at their separation.  With expansions about cell
// centres every same-level pair is an integer multiple o of the cell size h
// apart, so the order-p translation
//     L_b += sum_a (-1)^|a| mu_a D_(a+b)(o h),    |a| + |b| <= p,
// is one K x K matrix T_o (K = (p+1)(p+2)/2) per level and offset.  A CTA
// takes 128 sink nodes of a level (one child slot of 128 consecutive non-empty
// parents) and, for every offset
// o in the union of their interaction lists, multiplies the 128 x K block of
// source multipoles at that offset (a zero row where a sink has no source
// there) by T_o, accumulating all offsets of the tile in tensor memory:
//     D[sink][b] += sum_a A_o[sink][a] T_o[b][a].
// Precision: BF16 operands with a hi/lo split, x = x_hi + x_lo with
// x_hi = bf16(x) and x_lo = bf16(x - x_hi), and three products
// A_hi T_hi + A_hi T_lo + A_lo T_hi accumulated in FP32 (about 16 significant
// bits per product, against the FP32 SIMT kernels' 24).
//
// Data movement: the operators of a level are built once per solve
// (k_m2l_tc_ops, hi and lo tiles in the MMA's shared-memory layout) and each
// is brought into shared memory by one bulk copy (cp.async.bulk, completing on
// an mbarrier); the multipole rows are pre-split into bf16 hi/lo rows
// (k_mu_split) and gathered by 16-byte cp.async copies.  A ring of kStages
// buffers lets the copies of later offsets run while the MMAs of earlier ones
// execute.  Shared-memory operands use the no-swizzle K-major layout: 8-row x
// 16-byte core matrices, rows of a core matrix 16 bytes apart, core matrices
// 128 bytes apart along M/N (stride byte offset) and R/8 * 128 bytes apart
// along K (leading byte offset).
//
// Every wait on an mbarrier is bounded (about one second); a CTA that gives up
// records a status bit, waits (bounded) for the copies and MMAs it issued,
// frees its tensor memory and returns.
#pragma once

#include <cuda_bf16.h>

#include "expansion.cuh"

namespace tc {
namespace tcm {
// internal linkage: every order's object of fmm_p.cu includes these kernels
namespace {

constexpr int kRows = 128;                   // sinks per tile (the MMA's M)
constexpr int kChunk = 32;                   // union offsets per refill of a row's source table
constexpr int kMaxR = 15;                    // offsets with |o|_inf <= kMaxR
constexpr int kMaxW = 2 * kMaxR + 1;
constexpr int kMaxOff = kMaxW * kMaxW;       // 961
constexpr int kBitWords = (kMaxOff + 31) / 32;
constexpr uint32_t kNoSrc = 0xFFFFFFFFu;
// status bits written to the error word
constexpr uint32_t kErrOffset = 1u;   // a list entry beyond the operator table's offsets
constexpr uint32_t kErrTimeout = 2u;  // a bounded wait gave up

template <int P>
struct Shape {
    static constexpr int K = ncoef(P);
    static constexpr int KP = (K + 15) / 16 * 16;   // K and N padded to the BF16 MMA's K step (16)
    static constexpr int KC = KP / 8;               // 16-byte chunks of a row
    static constexpr int OPB = KP * KP * 2;         // one BF16 operator (hi or lo)
    static constexpr int ROWB = KP * 2;             // one BF16 multipole row (hi or lo)
    static constexpr int AB = kRows * KP * 2;       // one A operand (hi or lo)
    static constexpr int STAGE = 2 * AB + 2 * OPB;  // A_hi A_lo B_hi B_lo
    static constexpr int kStages = STAGE <= 36 * 1024 ? 5 : (STAGE <= 60 * 1024 ? 3 : 2);
    static constexpr int kAhead = kStages >= 4 ? kStages - 2 : 1;  // steps whose copies run ahead of the MMAs
    static constexpr int TCOLS = KP <= 32 ? 32 : (KP <= 64 ? 64 : 128);
    // shared memory: stages, row-source table, offset list, bit words, prefix, barriers, tmem slot, flags
    static constexpr int OFF_ROWSRC = kStages * STAGE;
    static constexpr int OFF_ULIST = OFF_ROWSRC + kChunk * kRows * 4;
    static constexpr int OFF_BITS = OFF_ULIST + ((kMaxOff * 2 + 15) / 16) * 16;
    static constexpr int OFF_WPRE = OFF_BITS + 32 * 4;
    static constexpr int OFF_BARS = OFF_WPRE + 32 * 4;
    static constexpr int OFF_MISC = OFF_BARS + 2 * kStages * 8;
    static constexpr int SMEM = OFF_MISC + 16 + 1024;  // + alignment slack
};

// byte offset of element (row, k) of a BF16 K-major operand with R rows
__host__ __device__ constexpr int cano(int row, int k, int R)
{
    return ((k >> 3) * (R >> 3) + (row >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t start, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((start >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N and M
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ uint64_t now_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// waits for the phase with the given parity to complete; false after about a second
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    const uint64_t t0 = now_ns();
    for (uint32_t it = 0;; it++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((it & 63u) == 63u && now_ns() - t0 > 1000000000ull) return false;
    }
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void cp16(uint32_t dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

template <int N>
__device__ __forceinline__ void cp_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's tensor-memory lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// the largest |o|_inf of a list entry of a box-centred handle: a pair opened
// at the parent level is at most r_max / (theta h_parent) parent cells apart
// (r_max the largest radius sum the criterion allows there), and its children
// at most twice that plus one cell
inline int offset_radius(bool bmax, double theta)
{
    const double parent = bmax ? 1.4142135623730951 / theta : 2.0 / theta;
    return (int)std::floor(2.0 * parent + 1e-9) + 1;
}

// ------------------------------------------------------------------ operators
// T_o[b][a] = (-1)^|a| D_(a+b)(o), |a| + |b| <= P, as BF16 hi and lo tiles in
// the B operand's layout (rows b, K index a), for every offset |o|_inf <= R;
// one block per offset
template <int P>
__global__ void __launch_bounds__(128) k_m2l_tc_ops(float hl, PotParams pp, int R, uint8_t* __restrict__ ops)
{
    using S = Shape<P>;
    constexpr int K = S::K, KP = S::KP;
    __shared__ float D[K];
    const int W = 2 * R + 1;
    const int oid = blockIdx.x;
    const int ox = oid / W - R, oy = oid % W - R;
    if (threadIdx.x == 0) {
        float d[K];
        if (ox == 0 && oy == 0) {
            for (int k = 0; k < K; k++) d[k] = 0.f;  // never used: a node does not translate to itself
        } else {
            derivs<P>((float)ox, (float)oy, hl, pp, d);
        }
        for (int k = 0; k < K; k++) D[k] = d[k];
    }
    __syncthreads();
    uint8_t* hi = ops + (size_t)oid * 2 * S::OPB;
    uint8_t* lo = hi + S::OPB;
    for (int e = threadIdx.x; e < KP * KP; e += blockDim.x) {
        const int b = e / KP, a = e % KP;
        float v = 0.f;
        if (a < K && b < K) {
            const int ka = cdeg(a), kb = cdeg(b);
            if (ka + kb <= P) {
                const int ay = a - ka * (ka + 1) / 2, ax = ka - ay;
                const int by = b - kb * (kb + 1) / 2, bx = kb - by;
                v = D[cidx(ax + bx, ay + by)];
                if (ka & 1) v = -v;
            }
        }
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
        *reinterpret_cast<__nv_bfloat16*>(hi + cano(b, a, KP)) = h;
        *reinterpret_cast<__nv_bfloat16*>(lo + cano(b, a, KP)) = l;
    }
}

// multipoles of the non-empty nodes from first_node on as BF16 hi and lo rows
// (KP entries each, zero-padded), at the node's position in the non-empty
// list; one thread per 8 coefficients (a 16-byte chunk of each row)
template <int P>
__global__ void k_mu_split(int64_t nn, uint32_t first_node, const float* __restrict__ mu,
                           const uint32_t* __restrict__ act, const uint32_t* __restrict__ act_pos,
                           uint8_t* __restrict__ mu_bf)
{
    using S = Shape<P>;
    constexpr int K = S::K, KC = S::KC, KS = kstride(P);
    const uint32_t k0 = act_pos[first_node], k1 = act_pos[nn];
    const int64_t items = (int64_t)(k1 - k0) * KC;
    for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < items;
         it += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t k = k0 + (uint32_t)(it / KC);
        const int c = (int)(it % KC);
        const float* m = mu + (int64_t)act[k] * KS;
        uint32_t hw[4], lw[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int i0 = 8 * c + 2 * j, i1 = i0 + 1;
            const float v0 = i0 < K ? m[i0] : 0.f, v1 = i1 < K ? m[i1] : 0.f;
            const __nv_bfloat16 h0 = __float2bfloat16_rn(v0), h1 = __float2bfloat16_rn(v1);
            const __nv_bfloat16 l0 = __float2bfloat16_rn(v0 - __bfloat162float(h0));
            const __nv_bfloat16 l1 = __float2bfloat16_rn(v1 - __bfloat162float(h1));
            hw[j] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
            lw[j] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
        }
        uint8_t* row = mu_bf + (size_t)k * 2 * S::ROWB;
        *reinterpret_cast<uint4*>(row + 16 * c) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *reinterpret_cast<uint4*>(row + S::ROWB + 16 * c) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
    }
}

// ------------------------------------------------------------------ M2L
// Persistent: each CTA walks tiles of level l.  Tile t holds child slot
// j = t % 4 of 128 consecutive non-empty parents (level l - 1) in Morton
// order: row r is child j of parent r when that child is non-empty.  Sinks in
// the same slot of their parent have the same candidate offsets (the children
// of the parent's near list), so a tile's union of offsets stays small.
// Writes loc (the node's M2L sum, as the SIMT M2L does) and its far-field
// pair sum zpart.
template <int P>
__global__ void __launch_bounds__(128, 1)
    k_m2l_tc(int l, int R, const uint32_t* __restrict__ nn_ptr, const uint32_t* __restrict__ nn_idx,
             const uint32_t* __restrict__ count, const float* __restrict__ mu, const uint8_t* __restrict__ mu_bf,
             const uint8_t* __restrict__ ops,
             float kappa, float* __restrict__ loc, double* __restrict__ zpart, const uint32_t* __restrict__ act,
             const uint32_t* __restrict__ act_pos, uint32_t* __restrict__ err)
{
    using S = Shape<P>;
    constexpr int K = S::K, KP = S::KP, KC = S::KC, KS = kstride(P);
    constexpr int NS = S::kStages, LA = S::kAhead;
    constexpr uint32_t IDESC = idesc_bf16(kRows, KP);
    constexpr uint32_t LBO_A = (kRows / 8) * 128, LBO_B = (KP / 8) * 128, SBO = 128;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint32_t* rowsrc = reinterpret_cast<uint32_t*>(smem + S::OFF_ROWSRC);
    uint16_t* ulist = reinterpret_cast<uint16_t*>(smem + S::OFF_ULIST);
    uint32_t* bits = reinterpret_cast<uint32_t*>(smem + S::OFF_BITS);
    uint32_t* wpre = reinterpret_cast<uint32_t*>(smem + S::OFF_WPRE);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S::OFF_BARS);  // [0, NS) operators, [NS, 2NS) MMAs
    uint32_t* misc = reinterpret_cast<uint32_t*>(smem + S::OFF_MISC);  // [0] tmem base, [1] union size, [2] abort
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t li = level_index(l), lp = level_index(l - 1);
    const uint32_t k0 = act_pos[lp], k1 = act_pos[li];  // the non-empty parents
    const uint32_t ntiles = 4u * ((k1 - k0 + kRows - 1) / kRows);
    if (blockIdx.x >= ntiles) return;  // uniform: the whole CTA leaves before any allocation
    const int W = 2 * R + 1, nwords = (W * W + 31) / 32;
    auto stage_a = [&](int s, int lohalf) { return smem + s * S::STAGE + lohalf * S::AB; };
    auto stage_b = [&](int s, int lohalf) { return smem + s * S::STAGE + 2 * S::AB + lohalf * S::OPB; };
    if (tid == 0) {
        for (int s = 0; s < 2 * NS; s++) mbar_init(saddr(bars + s), 1);
        misc[2] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(misc)),
                     "r"(S::TCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // every stage's A rows start zero; a row is rewritten only when its sink has a source at the step's offset
    for (int i = tid; i < NS * 2 * S::AB / 16; i += blockDim.x) {
        const int s = i / (2 * S::AB / 16), r = i % (2 * S::AB / 16);
        reinterpret_cast<uint4*>(stage_a(s, 0))[r] = make_uint4(0u, 0u, 0u, 0u);
    }
    uint32_t dirty = 0;  // bit s: this thread's row of stage s holds data
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = misc[0];
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    uint32_t step = 0;  // steps issued by this CTA so far (stage = step % NS, phase = step / NS)
    bool abort = false;

    for (uint32_t tile = blockIdx.x; tile < ntiles && !abort; tile += gridDim.x) {
        const uint32_t kk = k0 + (tile >> 2) * kRows + tid;
        const uint32_t a = kk < k1 ? 4u * (act[kk] - lp) + (tile & 3u) : 0u;  // level-local child index
        const int64_t na = (int64_t)li + a;
        const bool row_ok = kk < k1 && count[na] != 0;
        const uint32_t e0 = row_ok ? nn_ptr[a] : 0u, e1 = row_ok ? nn_ptr[a + 1] : 0u;
        const int iax = (int)compact16(a), iay = (int)compact16(a >> 1);
        auto offset_of = [&](uint32_t b, int& oid) {
            const int ox = iax - (int)compact16(b), oy = iay - (int)compact16(b >> 1);
            if (ox < -R || ox > R || oy < -R || oy > R) return false;
            oid = (ox + R) * W + (oy + R);
            return true;
        };
        // 1. the union of the tile's offsets, as a bit set and an ordered list
        if (tid < 32) bits[tid] = 0;
        __syncthreads();
        for (uint32_t e = e0; e < e1; e++) {
            int oid;
            if (offset_of(nn_idx[e], oid))
                atomicOr(&bits[oid >> 5], 1u << (oid & 31));
            else
                atomicOr(err, kErrOffset);
        }
        __syncthreads();
        if (tid < 32) {
            const uint32_t v = tid < nwords ? (uint32_t)__popc(bits[tid]) : 0u;
            uint32_t inc = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
                if (tid >= o) inc += t;
            }
            wpre[tid] = inc - v;
            if (tid == 31) misc[1] = inc;
            uint32_t wb = tid < nwords ? bits[tid] : 0u, r = inc - v;
            while (wb) {
                const int bt = __ffs(wb) - 1;
                ulist[r++] = (uint16_t)(tid * 32 + bt);
                wb &= wb - 1u;
            }
        }
        __syncthreads();
        const uint32_t U = misc[1];
        auto union_index = [&](int oid) {
            const uint32_t w = bits[oid >> 5];
            return wpre[oid >> 5] + (uint32_t)__popc(w & ((1u << (oid & 31)) - 1u));
        };
        // this thread's sources at the union offsets [c * kChunk, (c + 1) * kChunk), as their positions in the
        // non-empty list (the rows of the BF16 copy)
        auto refill = [&](uint32_t c) {
#pragma unroll 8
            for (int j = 0; j < kChunk; j++) rowsrc[j * kRows + tid] = kNoSrc;
            for (uint32_t e = e0; e < e1; e++) {
                const uint32_t b = nn_idx[e];
                int oid;
                if (!offset_of(b, oid)) continue;
                const uint32_t u = union_index(oid);
                // the source's row in the BF16 copy, looked up once per chunk rather than once per step
                if (u >= c * kChunk && u < (c + 1) * kChunk) rowsrc[(u - c * kChunk) * kRows + tid] = act_pos[li + b];
            }
        };
        // copies of union offset u into stage (step0 + u) % NS
        const uint32_t step0 = step;
        auto issue_copies = [&](uint32_t u) {
            const uint32_t g = step0 + u;
            const int s = (int)(g % NS);
            if (u % kChunk == 0) refill(u / kChunk);
            if (g >= (uint32_t)NS && !mbar_wait(saddr(bars + NS + s), ((g / NS) - 1) & 1)) {
                atomicOr(err, kErrTimeout);
                misc[2] = 1;
            }
            if (tid == 0) {
                const uint32_t tb = saddr(bars + s);
                mbar_expect_tx(tb, 2 * S::OPB);
                bulk_g2s(saddr(stage_b(s, 0)), ops + (size_t)ulist[u] * 2 * S::OPB, 2 * S::OPB, tb);
            }
            const uint32_t src = rowsrc[(u % kChunk) * kRows + tid];
            const uint32_t ahi = saddr(stage_a(s, 0)), alo = saddr(stage_a(s, 1));
            if (src != kNoSrc) {
                const uint8_t* g8 = mu_bf + (size_t)src * 2 * S::ROWB;
#pragma unroll
                for (int c = 0; c < KC; c++) {
                    cp16(ahi + cano(tid, 8 * c, kRows), g8 + 16 * c);
                    cp16(alo + cano(tid, 8 * c, kRows), g8 + S::ROWB + 16 * c);
                }
                dirty |= 1u << s;
            } else if (dirty & (1u << s)) {
#pragma unroll
                for (int c = 0; c < KC; c++) {
                    *reinterpret_cast<uint4*>(stage_a(s, 0) + cano(tid, 8 * c, kRows)) = make_uint4(0u, 0u, 0u, 0u);
                    *reinterpret_cast<uint4*>(stage_a(s, 1) + cano(tid, 8 * c, kRows)) = make_uint4(0u, 0u, 0u, 0u);
                }
                dirty &= ~(1u << s);
            }
            cp_commit();
        };
        // 2. the offsets of the union, copies running LA steps ahead of the MMAs
        // LA groups in flight from the start (empty ones past the union's end)
        for (uint32_t u = 0; u < (uint32_t)LA; u++) {
            if (u < U)
                issue_copies(u);
            else
                cp_commit();
        }
        for (uint32_t u = 0; u < U; u++) {
            if (u + LA < U)
                issue_copies(u + LA);
            else
                cp_commit();  // an empty group keeps the count of groups in flight at LA
            cp_wait<LA>();
            fence_async_smem();
            __syncthreads();
            if (misc[2]) {
                abort = true;
                break;
            }
            const uint32_t g = step0 + u;
            const int s = (int)(g % NS);
            if (tid == 0) {
                if (!mbar_wait(saddr(bars + s), (g / NS) & 1)) {
                    atomicOr(err, kErrTimeout);
                    misc[2] = 1;
                } else {
                    tc_fence_after();
                    const uint32_t ahi = saddr(stage_a(s, 0)), alo = saddr(stage_a(s, 1));
                    const uint32_t bhi = saddr(stage_b(s, 0)), blo = saddr(stage_b(s, 1));
#pragma unroll
                    for (int j = 0; j < KP / 16; j++)
                        mma_bf16(tmem, sdesc(ahi + j * 2 * LBO_A, LBO_A, SBO), sdesc(bhi + j * 2 * LBO_B, LBO_B, SBO),
                                 IDESC, (u > 0 || j > 0) ? 1u : 0u);
#pragma unroll
                    for (int j = 0; j < KP / 16; j++)
                        mma_bf16(tmem, sdesc(ahi + j * 2 * LBO_A, LBO_A, SBO), sdesc(blo + j * 2 * LBO_B, LBO_B, SBO),
                                 IDESC, 1u);
#pragma unroll
                    for (int j = 0; j < KP / 16; j++)
                        mma_bf16(tmem, sdesc(alo + j * 2 * LBO_A, LBO_A, SBO), sdesc(bhi + j * 2 * LBO_B, LBO_B, SBO),
                                 IDESC, 1u);
                    mma_commit(saddr(bars + NS + s));
                }
            }
        }
        step = step0 + U;
        cp_wait<0>();
        __syncthreads();
        if (misc[2]) abort = true;
        if (abort) break;
        // 3. epilogue: the tile's sums from tensor memory (lane = row = thread)
        float L[KP];
        if (U > 0) {
            const uint32_t g = step - 1;
            if (!mbar_wait(saddr(bars + NS + (int)(g % NS)), (g / NS) & 1)) {
                atomicOr(err, kErrTimeout);
                misc[2] = 1;
            }
            tc_fence_after();
#pragma unroll
            for (int c = 0; c < KP / 16; c++) tmem_ld16(trow + 16 * c, L + 16 * c);
        } else {
#pragma unroll
            for (int k = 0; k < KP; k++) L[k] = 0.f;
        }
        if (row_ok) {
            const bool any = e1 > e0;
            float zs = 0.f;
            const float* m = mu + na * KS;
#pragma unroll
            for (int k = 0; k < K; k++) {
                if (!any) L[k] = 0.f;
                zs += L[k] * m[k];
            }
            zpart[na] = any ? (double)kappa * (double)zs : 0.0;
            float4* o4 = reinterpret_cast<float4*>(loc + na * KS);
#pragma unroll
            for (int c = 0; c < KS / 4; c++)
                o4[c] = make_float4(4 * c < K ? L[4 * c] : 0.f, 4 * c + 1 < K ? L[4 * c + 1] : 0.f,
                                    4 * c + 2 < K ? L[4 * c + 2] : 0.f, 4 * c + 3 < K ? L[4 * c + 3] : 0.f);
        }
        // the next tile's first MMA overwrites the accumulator: every lane has read it
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (misc[2]) abort = true;
    }
    // in-flight work of an aborted CTA: bounded waits on what it issued, then the tensor memory is freed
    if (abort) {
        cp_wait<0>();
        for (uint32_t g = (step >= (uint32_t)NS ? step - NS : 0); g < step; g++) {
            mbar_wait(saddr(bars + (int)(g % NS)), (g / NS) & 1);
            mbar_wait(saddr(bars + NS + (int)(g % NS)), (g / NS) & 1);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(S::TCOLS) : "memory");
}

}  // namespace
}  // namespace tcm
}  // namespace tc
