// Shared device helpers for the GB300 tree-code library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/treecode.h"

#define TC_CUDA_TRY(expr)                                   \
    do {                                                    \
        cudaError_t _e = (expr);                            \
        if (_e != cudaSuccess) return tc_cuda_fail(_e, #expr); \
    } while (0)

int tc_cuda_fail(cudaError_t e, const char* what);
void tc_set_error(const char* fmt, ...);

namespace tc {

// multiprocessors of the current device (cudaDevAttrMultiProcessorCount, looked
// up once per device; 152 on GB300): grids are sized in multiples of it
int sm_count();
// leaves above this many particles take a warp (leaf moments, P2M) in the order-p path
constexpr uint32_t kLeafSmall = 32;

__host__ __device__ inline uint32_t spread16(uint32_t x)
{
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

__host__ __device__ inline uint32_t compact16(uint32_t x)
{
    x &= 0x55555555u;
    x = (x | (x >> 1)) & 0x33333333u;
    x = (x | (x >> 2)) & 0x0F0F0F0Fu;
    x = (x | (x >> 4)) & 0x00FF00FFu;
    x = (x | (x >> 8)) & 0x0000FFFFu;
    return x;
}

// first node of level l in the level-dense layout: (4^l - 1) / 3
__host__ __device__ inline uint32_t level_index(int l) { return (uint32_t)((((uint64_t)1 << (2 * l)) - 1) / 3); }

// x widened to a double with integer operations (exact, as the IEEE formats
// relate): the FP32 -> FP64 conversion instruction shares GB300's narrow FP64
// pipe.  Normal numbers rebias the exponent (+896) and move the fraction up 29
// bits; subnormals are normalised; zeros, infinities and NaNs keep their form.
__device__ __forceinline__ double f64_of_f32(float x)
{
    const uint32_t b = __float_as_uint(x);
    const uint32_t sign = b & 0x80000000u, e = (b >> 23) & 0xFFu, m = b & 0x7FFFFFu;
    unsigned long long r;
    if (e == 0u) {
        if (m == 0u) {
            r = 0ull;
        } else {
            const uint32_t t = 31u - (uint32_t)__clz(m);  // value m * 2^-149 = 2^(t - 149) * (m / 2^t)
            r = ((unsigned long long)(t + 874u) << 52) | ((unsigned long long)(m ^ (1u << t)) << (52u - t));
        }
    } else {
        r = ((unsigned long long)(e == 0xFFu ? 0x7FFu : e + 896u) << 52) | ((unsigned long long)m << 29);
    }
    return __longlong_as_double((long long)(r | ((unsigned long long)sign << 32)));
}

template <typename T>
__device__ inline T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// exclusive scan of one value per thread across the block; returns the block total
__device__ inline uint32_t block_exclusive_scan(uint32_t v, uint32_t& total)
{
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t blk_total;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    if (warp == 0) {
        uint32_t t = lane < nw ? warp_tot[lane] : 0u;
        uint32_t s = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) warp_tot[lane] = s - t;
        if (lane == nw - 1) blk_total = s;
    }
    __syncthreads();
    total = blk_total;
    uint32_t r = warp_tot[warp] + x - v;
    __syncthreads();
    return r;
}


inline int grid_for(int64_t n, int block, int cap = sm_count() * 32)
{
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

// ---------------------------------------------------------------- scan
// Exclusive scan of n u32 values; out must hold n+1 entries and receives the
// total in out[n].  tmp must hold scan_tmp_words(n) u32.
int64_t scan_tmp_words(int64_t n);
int exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* tmp, cudaStream_t s);
// the same for two arrays of length n in one set of launches, every output
// clamped to cap0 / cap1; tmp must hold 2 * scan_tmp_words(n) u32
int exclusive_scan2_u32(const uint32_t* in0, uint32_t* out0, const uint32_t* in1, uint32_t* out1, int64_t n,
                        uint32_t* tmp, cudaStream_t s, uint32_t cap0 = UINT32_MAX, uint32_t cap1 = UINT32_MAX);

// Deterministic FP64 sum of a[0..na) followed by c[0..*nc) (nc a device
// pointer, may be NULL) into *out (+= when accumulate).  tmp holds
// sum_tmp_doubles() doubles.
int64_t sum_tmp_doubles();
int sum_f64(const double* a, int64_t na, const double* c, const uint32_t* nc, double* out, int accumulate,
            double* tmp, cudaStream_t s);

// Exact bounding box of n device points (x, y doubles) as four order-preserving
// 64-bit keys (min x, min y, max x, max y) in d_keys4; NaN/inf sets *d_err.
int bbox_keys(const double* d_pos, int64_t n, double* d_keys4, uint32_t* d_err, cudaStream_t s);
__host__ __device__ inline double bbox_unkey(unsigned long long k)
{
    unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    union {
        unsigned long long i;
        double d;
    } c;
    c.i = u;
    return c.d;
}

// ---------------------------------------------------------------- sort
// Stable LSD radix sort of 32-bit keys by bits lo_bit..31 (passes of 8 bits)
// with 32-bit values; the result lands in keys/vals, alt_* are scratch of n
// entries each.  With an odd number of passes the input keys must be in
// alt_keys instead of keys.  The values are the input positions (iota).
int64_t radix_tmp_words(int64_t n);
int radix_sort_u32(uint32_t* keys, uint32_t* vals, uint32_t* alt_keys, uint32_t* alt_vals, int64_t n,
                   uint32_t* tmp, cudaStream_t s, int* launches, int lo_bit = 0);

}  // namespace tc
