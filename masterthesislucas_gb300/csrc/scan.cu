// Device-wide exclusive prefix sum of u32 (reduce -> scan partials -> scan).
#include "common.cuh"

namespace tc {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanChunk = kScanThreads * kScanItems;

__global__ void k_scan_reduce(const uint32_t* __restrict__ in, int64_t n, uint32_t* __restrict__ partial)
{
    int64_t base = (int64_t)blockIdx.x * kScanChunk;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        int64_t k = base + (int64_t)i * kScanThreads + threadIdx.x;
        if (k < n) s += in[k];
    }
    s = warp_sum(s);
    __shared__ uint32_t ws[kScanThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kScanThreads / 32; w++) t += ws[w];
        partial[blockIdx.x] = t;
    }
}

__global__ void k_scan_partials(uint32_t* partial, int64_t nb)
{
    uint32_t carry = 0;
    for (int64_t base = 0; base < nb; base += blockDim.x) {
        int64_t k = base + threadIdx.x;
        uint32_t v = k < nb ? partial[k] : 0u;
        uint32_t tot;
        uint32_t ex = block_exclusive_scan(v, tot);
        if (k < nb) partial[k] = carry + ex;
        carry += tot;
    }
}

// A chunk moves between global and shared memory in coalesced rows (row i,
// thread t: item i * kScanThreads + t) and each thread scans its own
// kScanItems consecutive items from shared memory; the padded index keeps
// both access patterns free of bank conflicts.
__device__ __forceinline__ int chunk_slot(int x) { return x + (x >> 5); }
constexpr int kChunkWords = kScanChunk + kScanChunk / 32;

__device__ __forceinline__ void load_chunk(const uint32_t* __restrict__ in, int64_t base, int64_t n, uint32_t* sm,
                                           uint32_t (&v)[kScanItems])
{
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        const int x = i * kScanThreads + threadIdx.x;
        sm[chunk_slot(x)] = base + x < n ? in[base + x] : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kScanItems; i++) v[i] = sm[chunk_slot(threadIdx.x * kScanItems + i)];
}

// v holds this thread's exclusive results; sm still holds the inputs, so the block syncs before overwriting
__device__ __forceinline__ void store_chunk(uint32_t* __restrict__ out, int64_t base, int64_t n, uint32_t* sm,
                                            const uint32_t (&v)[kScanItems])
{
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kScanItems; i++) sm[chunk_slot(threadIdx.x * kScanItems + i)] = v[i];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        const int x = i * kScanThreads + threadIdx.x;
        if (base + x < n) out[base + x] = sm[chunk_slot(x)];
    }
}

__global__ void k_scan_final(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int64_t n,
                             const uint32_t* __restrict__ partial, int64_t nb)
{
    __shared__ uint32_t sm[kChunkWords];
    const int64_t base = (int64_t)blockIdx.x * kScanChunk;
    uint32_t v[kScanItems];
    load_chunk(in, base, n, sm, v);
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) s += v[i];
    uint32_t tot;
    uint32_t ex = block_exclusive_scan(s, tot) + partial[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        const uint32_t x = v[i];
        v[i] = ex;
        ex += x;
    }
    store_chunk(out, base, n, sm, v);
    if (blockIdx.x == nb - 1 && threadIdx.x == 0) out[n] = partial[blockIdx.x] + tot;
}

// two arrays at once: blockIdx.y selects (in0, out0) or (in1, out1); the
// partials of array y sit at partial + y * nb
__global__ void k_scan_reduce2(const uint32_t* __restrict__ in0, const uint32_t* __restrict__ in1, int64_t n,
                               uint32_t* __restrict__ partial, int64_t nb)
{
    const uint32_t* in = blockIdx.y ? in1 : in0;
    int64_t base = (int64_t)blockIdx.x * kScanChunk;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        int64_t k = base + (int64_t)i * kScanThreads + threadIdx.x;
        if (k < n) s += in[k];
    }
    s = warp_sum(s);
    __shared__ uint32_t ws[kScanThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kScanThreads / 32; w++) t += ws[w];
        partial[blockIdx.y * nb + blockIdx.x] = t;
    }
}

__global__ void k_scan_partials2(uint32_t* partial, int64_t nb)
{
    uint32_t* p = partial + blockIdx.x * nb;
    uint32_t carry = 0;
    for (int64_t base = 0; base < nb; base += blockDim.x) {
        int64_t k = base + threadIdx.x;
        uint32_t v = k < nb ? p[k] : 0u;
        uint32_t tot;
        uint32_t ex = block_exclusive_scan(v, tot);
        if (k < nb) p[k] = carry + ex;
        carry += tot;
    }
}

// partial == nullptr: a single chunk (nb == 1), no carry.  Outputs are
// clamped to cap0 / cap1.
__global__ void k_scan_final2(const uint32_t* __restrict__ in0, uint32_t* __restrict__ out0,
                              const uint32_t* __restrict__ in1, uint32_t* __restrict__ out1, int64_t n,
                              const uint32_t* __restrict__ partial, int64_t nb, uint32_t cap0, uint32_t cap1)
{
    const uint32_t* in = blockIdx.y ? in1 : in0;
    uint32_t* out = blockIdx.y ? out1 : out0;
    const uint32_t cap = blockIdx.y ? cap1 : cap0;
    const uint32_t carry = partial ? partial[blockIdx.y * nb + blockIdx.x] : 0u;
    __shared__ uint32_t sm[kChunkWords];
    const int64_t base = (int64_t)blockIdx.x * kScanChunk;
    uint32_t v[kScanItems];
    load_chunk(in, base, n, sm, v);
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) s += v[i];
    uint32_t tot;
    uint32_t ex = block_exclusive_scan(s, tot) + carry;
#pragma unroll
    for (int i = 0; i < kScanItems; i++) {
        const uint32_t x = v[i];
        v[i] = min(ex, cap);
        ex += x;
    }
    store_chunk(out, base, n, sm, v);
    if (blockIdx.x == nb - 1 && threadIdx.x == 0) out[n] = min(carry + tot, cap);
}

// fixed (8 per SM of a 152-SM GB300) so that the order of the deterministic
// sums does not depend on the device
constexpr int kSumBlocks = 8 * 152;

// stage 1 of sum_f64: block b sums the grid-stride slice b of a[0..na) ++ c[0..*nc)
// (four loads in flight per thread over a, then the rest one at a time)
__global__ void k_sum_partial(const double* __restrict__ a, int64_t na, const double* __restrict__ c,
                              const uint32_t* __restrict__ nc, double* __restrict__ partial)
{
    __shared__ double ws[32];
    const int64_t ncv = nc ? (int64_t)*nc : 0;
    const int64_t tot = na + ncv;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; i + 3 * stride < na; i += 4 * stride) {
        s0 += a[i];
        s1 += a[i + stride];
        s2 += a[i + 2 * stride];
        s3 += a[i + 3 * stride];
    }
    for (; i < tot; i += stride) s0 += i < na ? a[i] : c[i - na];
    double s = (s0 + s1) + (s2 + s3);
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

__global__ void k_sum_final(const double* __restrict__ partial, int np, double* __restrict__ out, int accumulate)
{
    __shared__ double ws[32];
    double s = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += partial[i];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) *out = accumulate ? *out + v : v;
    }
}

}  // namespace

int64_t sum_tmp_doubles() { return kSumBlocks; }

int sum_f64(const double* a, int64_t na, const double* c, const uint32_t* nc, double* out, int accumulate,
            double* tmp, cudaStream_t s)
{
    k_sum_partial<<<kSumBlocks, 256, 0, s>>>(a, na, c, nc, tmp);
    k_sum_final<<<1, 256, 0, s>>>(tmp, kSumBlocks, out, accumulate);
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

int64_t scan_tmp_words(int64_t n) { return (n + kScanChunk - 1) / kScanChunk + 1; }

int exclusive_scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* tmp, cudaStream_t s)
{
    if (n <= 0) {
        TC_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(uint32_t), s));
        return TC_OK;
    }
    int64_t nb = (n + kScanChunk - 1) / kScanChunk;
    if (nb == 1) {
        // one array: blockIdx.y is 0, the second pair is never read
        k_scan_final2<<<dim3(1, 1), kScanThreads, 0, s>>>(in, out, nullptr, nullptr, n, nullptr, 1, UINT32_MAX,
                                                          UINT32_MAX);
        TC_CUDA_TRY(cudaGetLastError());
        return TC_OK;
    }
    k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, tmp);
    k_scan_partials<<<1, 1024, 0, s>>>(tmp, nb);
    k_scan_final<<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, tmp, nb);
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

int exclusive_scan2_u32(const uint32_t* in0, uint32_t* out0, const uint32_t* in1, uint32_t* out1, int64_t n,
                        uint32_t* tmp, cudaStream_t s, uint32_t cap0, uint32_t cap1)
{
    if (n <= 0) {
        TC_CUDA_TRY(cudaMemsetAsync(out0, 0, sizeof(uint32_t), s));
        TC_CUDA_TRY(cudaMemsetAsync(out1, 0, sizeof(uint32_t), s));
        return TC_OK;
    }
    int64_t nb = (n + kScanChunk - 1) / kScanChunk;
    if (nb == 1) {
        k_scan_final2<<<dim3(1, 2), kScanThreads, 0, s>>>(in0, out0, in1, out1, n, nullptr, 1, cap0, cap1);
    } else {
        k_scan_reduce2<<<dim3((unsigned)nb, 2), kScanThreads, 0, s>>>(in0, in1, n, tmp, nb);
        k_scan_partials2<<<2, 1024, 0, s>>>(tmp, nb);
        k_scan_final2<<<dim3((unsigned)nb, 2), kScanThreads, 0, s>>>(in0, out0, in1, out1, n, tmp, nb, cap0, cap1);
    }
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

}  // namespace tc
