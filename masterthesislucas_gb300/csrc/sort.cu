// Stable LSD radix sort of (u32 key, u32 value): 4 passes of 8 bits, each a
// per-tile digit histogram, a device-wide scan of the digit-major histogram
// table, and a stable scatter.  The scatter ranks keys in their input order
// with warp match-any groups against warp-private digit counters, stages the
// tile digit-sorted in shared memory and writes each digit run contiguously.  Stability makes ties between equal
// Morton codes keep input order, which defines the permutation where the
// reference's unstable integer_sort (nBodySolverFMM_SYM_MORTON.h:89) does not.
#include "common.cuh"

namespace tc {
namespace {

constexpr int RT = 256;           // threads per tile
#ifndef TC_SORT_RI
#define TC_SORT_RI 8
#endif
constexpr int RI = TC_SORT_RI;    // keys per thread
constexpr int RTILE = RT * RI;    // keys per tile
constexpr int RADIX = 256;
constexpr int NW = RT / 32;

__global__ void __launch_bounds__(RT) k_radix_hist(const uint32_t* __restrict__ keys, int64_t n, int shift,
                                                   uint32_t* __restrict__ hist, int nblocks)
{
    __shared__ uint32_t h[RADIX];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RTILE;
    uint32_t k[RI];
#pragma unroll
    for (int r = 0; r < RI; r++) {
        const int64_t p = base + (int64_t)r * RT + threadIdx.x;
        k[r] = p < n ? keys[p] : 0u;
    }
#pragma unroll
    for (int r = 0; r < RI; r++)
        if (base + (int64_t)r * RT + threadIdx.x < n) atomicAdd(&h[(k[r] >> shift) & 255u], 1u);
    __syncthreads();
    hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(RT) k_radix_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                      uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                      int64_t n, int shift, const uint32_t* __restrict__ offs,
                                                      int nblocks, int iota_vals)
{
    __shared__ uint32_t s_keys[RTILE];
    __shared__ uint32_t s_vals[RTILE];
    __shared__ uint32_t s_wh[NW][RADIX];  // per warp: digit counts, then the warp's offset within the digit
    __shared__ uint32_t s_start[RADIX];
    __shared__ uint32_t s_gofs[RADIX];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t lt_mask = (1u << lane) - 1u;
    for (int i = tid; i < NW * RADIX; i += RT) (&s_wh[0][0])[i] = 0;
    __syncthreads();
    // this block's global start of each digit, fetched while the tile is ranked
    const uint32_t goff = offs[(int64_t)tid * nblocks + blockIdx.x];
    uint32_t key[RI], val[RI], rank[RI], dig[RI];
    const int64_t base = (int64_t)blockIdx.x * RTILE + (int64_t)warp * (32 * RI);
    uint32_t* wh = s_wh[warp];
    // warp w ranks the tile's w-th run of RT * RI / NW consecutive keys, 32 at a time, against its own counters:
    // warps cover the tile in input order, so (warp, row, lane) order is input order and the sort is stable.
    // All of the warp's loads first (independent, in flight together), then the ranking.
#pragma unroll
    for (int r = 0; r < RI; r++) {
        const int64_t p = base + r * 32 + lane;
        const bool valid = p < n;
        key[r] = valid ? kin[p] : 0u;
        val[r] = valid ? (iota_vals ? (uint32_t)p : vin[p]) : 0u;
    }
#pragma unroll
    for (int r = 0; r < RI; r++) {
        const uint32_t d = base + r * 32 + lane < n ? ((key[r] >> shift) & 255u) : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t before = d < 256u ? wh[d] : 0u;
        __syncwarp();
        if (d < 256u && lane == (uint32_t)(__ffs(peers) - 1)) wh[d] = before + __popc(peers);
        __syncwarp();
        rank[r] = before + __popc(peers & lt_mask);
        dig[r] = d;
    }
    __syncthreads();
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < NW; w++) {
        const uint32_t c = s_wh[w][tid];
        s_wh[w][tid] = run;
        run += c;
    }
    uint32_t tot;
    const uint32_t st = block_exclusive_scan(run, tot);
    s_start[tid] = st;
    s_gofs[tid] = goff - st;  // global position of tile slot j of digit d: s_gofs[d] + j (mod 2^32)
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RI; r++) {
        if (dig[r] < 256u) {
            const uint32_t idx = s_start[dig[r]] + wh[dig[r]] + rank[r];
            s_keys[idx] = key[r];
            s_vals[idx] = val[r];
        }
    }
    __syncthreads();
    const int64_t rem = n - (int64_t)blockIdx.x * RTILE;
    const int cnt = rem < RTILE ? (int)rem : RTILE;
#pragma unroll
    for (int r = 0; r < RI; r++) {
        const int j = r * RT + tid;
        if (j < cnt) {
            const uint32_t k = s_keys[j];
            const uint32_t o = s_gofs[(k >> shift) & 255u] + (uint32_t)j;
            kout[o] = k;
            vout[o] = s_vals[j];
        }
    }
}

}  // namespace

int64_t radix_tmp_words(int64_t n)
{
    int64_t nb = (n + RTILE - 1) / RTILE;
    int64_t h = nb * RADIX;
    return 2 * (h + 1) + scan_tmp_words(h) + 8;
}

int radix_sort_u32(uint32_t* keys, uint32_t* vals, uint32_t* alt_keys, uint32_t* alt_vals, int64_t n,
                   uint32_t* tmp, cudaStream_t s, int* launches, int lo_bit)
{
    if (n <= 0) return TC_OK;
    const int nb = (int)((n + RTILE - 1) / RTILE);
    const int64_t h = (int64_t)nb * RADIX;
    uint32_t* hist = tmp;
    uint32_t* offs = tmp + (h + 1);
    uint32_t* stmp = offs + (h + 1);
    const int npass = (32 - lo_bit + 7) / 8;
    // an odd number of passes starts from the alternate buffers (the keys are
    // there), so that the result always lands in keys / vals
    uint32_t *ki = keys, *vi = vals, *ko = alt_keys, *vo = alt_vals;
    if (npass & 1) {
        ki = alt_keys;
        vi = alt_vals;
        ko = keys;
        vo = vals;
    }
    for (int pass = 0; pass < npass; pass++) {
        const int shift = lo_bit + 8 * pass;
        k_radix_hist<<<nb, RT, 0, s>>>(ki, n, shift, hist, nb);
        int rc = exclusive_scan_u32(hist, offs, h, stmp, s);
        if (rc) return rc;
        k_radix_scatter<<<nb, RT, 0, s>>>(ki, vi, ko, vo, n, shift, offs, nb, pass == 0);
        if (launches) *launches += 2 + (h <= 2048 ? 1 : 3);  // histogram, scatter, scan
        uint32_t* t = ki; ki = ko; ko = t;
        t = vi; vi = vo; vo = t;
    }
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

}  // namespace tc
