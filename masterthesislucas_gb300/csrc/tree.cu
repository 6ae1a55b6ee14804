// Tree construction, bit-exact to NBodySolverFMM_SYM_MORTON::updateTree
// (src/nbodysolvers/cpu/nBodySolverFMM_SYM_MORTON.h:79-95):
//   createMortonCode (:538-561)  -> k_morton_fast + k_morton_exact (FP32
//                                   where its floor provably agrees, else FP64)
//   integer_sort (:89)           -> radix_sort_u32   (stable on input order)
//   createLeafNodes (:328-379)   -> k_gather_bounds + k_leaf_moments
//   bottomUpNodeConstruction (:381-470) -> k_bottom_up, one launch per level
// Leaf moments are summed sequentially in sorted order by one thread per
// leaf and internal nodes combine children in the reference's j = 3..0 order,
// so COM, M0 and M2 come out bit-identical to the reference's FP64 values.
// The order-p path (FP32 only) builds its records in tree_p.cu instead.
// Alongside the FP64 node record the kernels write the compute copies in
// cell-relative coordinates (COM minus the ideal cell centre), which keep
// FP32 differences accurate to a fraction of the cell size.
#include <cmath>

#include "state.cuh"

namespace tc {
namespace {

// one coordinate of createMortonCode (:545-549): (uint32)clamp(((p - min)/L) * 65536, 0, 65535).
// FP64 division runs at 1/64 of the FP32 rate on GB300, so the quotient is
// first formed as (p - min) * (65536/L), within 2 ulp of the exact product;
// only when that lands within 1e-9 of an integer can the floor differ from
// the reference's, and then the reference's own division decides.
__device__ inline uint32_t morton_coord(double p, double nm, double L, double s65536)
{
    const double a = p + nm;
    double v = a * s65536;
    const double f = v - floor(v);
    if (f < 1e-9 || f > 1.0 - 1e-9) v = (a / (L)) * 65536.0;
    v = (v < 0.0) ? 0.0 : v;             // glm::max(v, 0)
    v = (65535.0 < v) ? 65535.0 : v;     // glm::min(v, 65535)
    return (uint32_t)v;
}

// IEEE double as an integer with the same order (for box tests on the integer pipe)
__device__ inline long long dorder(double v)
{
    const long long b = __double_as_longlong(v);
    return b >= 0 ? b : (long long)(0x8000000000000000ull - (unsigned long long)b);
}

// v rounded to the nearest float (ties to even) with integer operations: the
// FP64 -> FP32 conversion instruction shares GB300's narrow FP64 pipe.
// Results below the smallest normal float flush to a signed zero.
__device__ inline float f32_rn(double v)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7FFull);
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    if (e == 0x7FF) return m ? __uint_as_float(0x7FC00000u) : __uint_as_float(sign | 0x7F800000u);
    const int ef = e - 1023 + 127;
    if (ef <= 0) return __uint_as_float(sign);
    if (ef >= 255) return __uint_as_float(sign | 0x7F800000u);
    unsigned long long r = m >> 29;
    const unsigned long long rem = m & ((1ull << 29) - 1ull);
    if (rem > (1ull << 28) || (rem == (1ull << 28) && (r & 1ull))) r++;
    // a mantissa carry (r = 2^23) moves into the exponent, as rounding does
    const uint32_t bits = ((uint32_t)ef << 23) + (uint32_t)r;
    return __uint_as_float(sign | (bits < 0x7F800000u ? bits : 0x7F800000u));
}

// createMortonCode's quantisation, fast form.  FP64 runs at 1/64 of the FP32
// rate on GB300, so the quotient ((p - min) / L) * 65536 is first formed in
// FP32 from the FP64 difference: fl32(fl32(p - min) * fl32(65536 / L)) is
// within 3 * 2^-24 relative (<= 0.012 absolute below 65536) of the
// reference's FP64 value, so its floor is the reference's whenever its
// fraction lies in [1/64, 63/64).  Points with a coordinate closer than that
// to a cell edge are queued, and k_morton_exact recomputes them with the
// reference's FP64 arithmetic.  Each block queues into its own region of
// morton_region(n, grid) entries (shared-memory counter, no global atomics).
// The box test compares the doubles' order-preserving integer images.
constexpr int kMortonThreads = 256;

__host__ __device__ inline int64_t morton_region(int64_t n, int64_t grid)
{
    const int64_t per = grid * kMortonThreads;
    return ((n + per - 1) / per) * kMortonThreads;
}

__global__ void __launch_bounds__(kMortonThreads)
    k_morton_fast(const double2* __restrict__ pos, int64_t n, double minx, double miny, double maxx, double maxy,
                  float s65536, uint32_t* __restrict__ codes, uint32_t* __restrict__ err,
                  uint32_t* __restrict__ queue, uint32_t* __restrict__ qcount)
{
    __shared__ uint32_t s_count;
    if (threadIdx.x == 0) s_count = 0;
    __syncthreads();
    uint32_t* region = queue + (int64_t)blockIdx.x * morton_region(n, gridDim.x);
    const long long kx0 = dorder(minx), kx1 = dorder(maxx), ky0 = dorder(miny), ky1 = dorder(maxy);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 p = pos[i];
        const long long kx = dorder(p.x), ky = dorder(p.y);
        // NaN images lie outside every finite box
        if (!(kx >= kx0 && kx <= kx1 && ky >= ky0 && ky <= ky1)) atomicOr(err, 1u);
        const float vx = f32_rn(p.x - minx) * s65536, vy = f32_rn(p.y - miny) * s65536;
        bool exact = false;
        uint32_t q[2];
        const float v2[2] = {vx, vy};
#pragma unroll
        for (int c = 0; c < 2; c++) {
            const float v = v2[c];
            if (v >= 65535.0f + 1.0f / 64.0f) {
                q[c] = 65535u;  // the reference's clamp whatever the last bits
            } else {
                const float f = v - floorf(v);
                exact |= !(f >= 1.0f / 64.0f && f < 63.0f / 64.0f);
                q[c] = v > 0.0f ? (uint32_t)v : 0u;
            }
        }
        if (exact)
            region[atomicAdd(&s_count, 1u)] = (uint32_t)i;
        else
            codes[i] = (spread16(q[1]) << 1) | spread16(q[0]);
    }
    __syncthreads();
    if (threadIdx.x == 0) qcount[blockIdx.x] = s_count;
}

// the queued points of k_morton_fast, in the reference's FP64 arithmetic: block
// b of the same grid takes region b
__global__ void __launch_bounds__(kMortonThreads)
    k_morton_exact(const double2* __restrict__ pos, int64_t n, double minx, double miny, double L,
                   const uint32_t* __restrict__ queue, const uint32_t* __restrict__ qcount,
                   uint32_t* __restrict__ codes)
{
    const double nmx = -minx, nmy = -miny;
    const double s65536 = 65536.0 / L;
    const uint32_t* region = queue + (int64_t)blockIdx.x * morton_region(n, gridDim.x);
    const uint32_t nq = qcount[blockIdx.x];
    for (uint32_t k = threadIdx.x; k < nq; k += blockDim.x) {
        const uint32_t i = region[k];
        const double2 p = pos[i];
        codes[i] = (spread16(morton_coord(p.y, nmy, L, s65536)) << 1) | spread16(morton_coord(p.x, nmx, L, s65536));
    }
}

template <typename real>
__global__ void k_gather_bounds(const uint32_t* __restrict__ codes, const uint32_t* __restrict__ perm,
                                const double2* __restrict__ pos_in, int64_t n, int depth, double minx, double miny,
                                double h, double2* __restrict__ pos64, real* __restrict__ prel,
                                uint32_t* __restrict__ first, uint32_t* __restrict__ endp)
{
    const int shift = 32 - 2 * depth;
    const uint32_t li = level_index(depth);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t leaf = depth ? (codes[k] >> shift) : 0u;
        double2 p = pos_in[perm[k]];
        pos64[k] = p;
        uint32_t ix = compact16(leaf), iy = compact16(leaf >> 1);
        double cx = minx + ((double)ix + 0.5) * h;
        double cy = miny + ((double)iy + 0.5) * h;
        prel[2 * k] = (real)(p.x - cx);
        prel[2 * k + 1] = (real)(p.y - cy);
        if (k == 0 || (depth ? (codes[k - 1] >> shift) : 0u) != leaf) first[li + leaf] = (uint32_t)k;
        if (k == n - 1 || (depth ? (codes[k + 1] >> shift) : 0u) != leaf) endp[li + leaf] = (uint32_t)(k + 1);
    }
}

// cell centres relative to the box corner, (i + 0.5) h for i < 2^depth
__global__ void k_cell_offsets(int w, double h, double* __restrict__ off)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w; i += gridDim.x * blockDim.x)
        off[i] = ((double)i + 0.5) * h;
}

// k_gather_bounds for FP32 compute copies: p - centre as (p - min) - (i + 0.5) h
// from the offset table (two FP64 additions per coordinate; the difference is
// the FP64 one to within its last bits, far below FP32 resolution)
__global__ void k_gather_bounds_f32(const uint32_t* __restrict__ codes, const uint32_t* __restrict__ perm,
                                    const double2* __restrict__ pos_in, int64_t n, int depth, double minx,
                                    double miny, const double* __restrict__ off, double2* __restrict__ pos64,
                                    float2* __restrict__ prel, uint32_t* __restrict__ first,
                                    uint32_t* __restrict__ endp)
{
    const int shift = 32 - 2 * depth;
    const uint32_t li = level_index(depth);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t leaf = depth ? (codes[k] >> shift) : 0u;
        const double2 p = pos_in[perm[k]];
        pos64[k] = p;
        const uint32_t ix = compact16(leaf), iy = compact16(leaf >> 1);
        prel[k] = make_float2(f32_rn((p.x - minx) - off[ix]), f32_rn((p.y - miny) - off[iy]));
        if (k == 0 || (depth ? (codes[k - 1] >> shift) : 0u) != leaf) first[li + leaf] = (uint32_t)k;
        if (k == n - 1 || (depth ? (codes[k + 1] >> shift) : 0u) != leaf) endp[li + leaf] = (uint32_t)(k + 1);
    }
}

template <typename real>
__device__ inline void write_compute(int64_t node, double comx, double comy, double m0, double m2xx, double m2xy,
                                     double m2yy, double cx, double cy, real* comrel, real* m0r, real* m2t)
{
    comrel[2 * node] = (real)(comx - cx);
    comrel[2 * node + 1] = (real)(comy - cy);
    m0r[node] = (real)m0;
    double inv = m0 > 0.0 ? 1.0 / m0 : 0.0;
    m2t[3 * node] = (real)(inv * m2xx);
    m2t[3 * node + 1] = (real)(inv * m2xy);
    m2t[3 * node + 2] = (real)(inv * m2yy);
}

// createLeafNodes, second loop (:355-377) plus the first-occupant box (:343-350)
template <typename real>
__global__ void k_leaf_moments(const double2* __restrict__ pos64, int depth, double minx, double miny, double h,
                               uint32_t* __restrict__ count, const uint32_t* __restrict__ first,
                               double2* __restrict__ com64, double* __restrict__ m0, double* __restrict__ m2,
                               double2* __restrict__ bbc, double* __restrict__ bblen, real* __restrict__ comrel,
                               real* __restrict__ m0r, real* __restrict__ m2t)
{
    const uint32_t li = level_index(depth);
    const int64_t nl = (int64_t)1 << (2 * depth);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nl; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t node = li + i;
        uint32_t f = first[node];
        uint32_t c = count[node] - f;  // count holds the end index here
        count[node] = c;
        uint32_t ix = compact16((uint32_t)i), iy = compact16((uint32_t)i >> 1);
        double cx = minx + ((double)ix + 0.5) * h;
        double cy = miny + ((double)iy + 0.5) * h;
        if (c == 0) {
            com64[node] = make_double2(0.0, 0.0);
            m0[node] = 0.0;
            m2[3 * node] = m2[3 * node + 1] = m2[3 * node + 2] = 0.0;
            bbc[node] = make_double2(0.0, 0.0);
            bblen[node] = 0.0;
            write_compute<real>(node, cx, cy, 0.0, 0.0, 0.0, 0.0, cx, cy, comrel, m0r, m2t);
            continue;
        }
        double sx = 0.0, sy = 0.0;
        for (uint32_t p = f; p < f + c; p++) {
            double2 q = pos64[p];
            sx += q.x;
            sy += q.y;
        }
        double M0 = (double)c;
        sx /= M0;
        sy /= M0;
        double a = 0.0, b = 0.0, d = 0.0;
        for (uint32_t p = f; p < f + c; p++) {
            double2 q = pos64[p];
            double rx = q.x - sx, ry = q.y - sy;
            a += rx * rx;
            b += rx * ry;
            d += ry * ry;
        }
        com64[node] = make_double2(sx, sy);
        m0[node] = M0;
        m2[3 * node] = a;
        m2[3 * node + 1] = b;
        m2[3 * node + 2] = d;
        // BBcentre = minPos + h * g + 0.5 * h (:345)
        bbc[node] = make_double2(minx + h * (double)ix + 0.5 * h, miny + h * (double)iy + 0.5 * h);
        bblen[node] = h;
        write_compute<real>(node, sx, sy, M0, a, b, d, cx, cy, comrel, m0r, m2t);
    }
}

// bottomUpNodeConstruction (:381-470) for one level l
template <typename real>
__global__ void k_bottom_up(int l, double minx, double miny, double hl, uint32_t* __restrict__ count,
                            uint32_t* __restrict__ first, double2* __restrict__ com64, double* __restrict__ m0,
                            double* __restrict__ m2, double2* __restrict__ bbc, double* __restrict__ bblen,
                            real* __restrict__ comrel, real* __restrict__ m0r, real* __restrict__ m2t)
{
    const uint32_t li = level_index(l), lc = level_index(l + 1);
    const int64_t nl = (int64_t)1 << (2 * l);
    const double offx[4] = {0.5, -0.5, 0.5, -0.5};
    const double offy[4] = {0.5, 0.5, -0.5, -0.5};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nl; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t node = li + i;
        const int64_t fc = lc + 4 * i;
        uint32_t cnt = 0, fp = 0;
        double cx = 0.0, cy = 0.0, M0 = 0.0, bx = 0.0, by = 0.0, len = 0.0;
        for (int j = 3; j >= 0; j--) {
            const int64_t ch = fc + j;
            uint32_t cc = count[ch];
            if (cc == 0) continue;
            double clen = bblen[ch];
            double2 cb = bbc[ch];
            bx = offx[j] * clen + cb.x;
            by = offy[j] * clen + cb.y;
            len = 2.0 * clen;
            fp = first[ch];
            cnt += cc;
            double cm = m0[ch];
            double2 cc2 = com64[ch];
            cx += cm * cc2.x;
            cy += cm * cc2.y;
            M0 += cm;
        }
        uint32_t ix = compact16((uint32_t)i), iy = compact16((uint32_t)i >> 1);
        double ccx = minx + ((double)ix + 0.5) * hl;
        double ccy = miny + ((double)iy + 0.5) * hl;
        count[node] = cnt;
        first[node] = fp;
        if (cnt == 0) {
            com64[node] = make_double2(0.0, 0.0);
            m0[node] = 0.0;
            m2[3 * node] = m2[3 * node + 1] = m2[3 * node + 2] = 0.0;
            bbc[node] = make_double2(0.0, 0.0);
            bblen[node] = 0.0;
            write_compute<real>(node, ccx, ccy, 0.0, 0.0, 0.0, 0.0, ccx, ccy, comrel, m0r, m2t);
            continue;
        }
        cx /= M0;
        cy /= M0;
        double a = 0.0, b = 0.0, d = 0.0;
        for (int j = 0; j < 4; j++) {
            const int64_t ch = fc + j;
            double cm = m0[ch];
            if (cm == 0.0) continue;
            double2 cc2 = com64[ch];
            double rx = cc2.x - cx, ry = cc2.y - cy;
            a += rx * rx;
            b += rx * ry;
            d += ry * ry;
            a += m2[3 * ch];
            b += m2[3 * ch + 1];
            d += m2[3 * ch + 2];
        }
        com64[node] = make_double2(cx, cy);
        m0[node] = M0;
        m2[3 * node] = a;
        m2[3 * node + 1] = b;
        m2[3 * node + 2] = d;
        bbc[node] = make_double2(bx, by);
        bblen[node] = len;
        write_compute<real>(node, cx, cy, M0, a, b, d, ccx, ccy, comrel, m0r, m2t);
    }
}

}  // namespace

// ---------------------------------------------------------------- active nodes
// The order-p passes over a level (M2M, M2L, L2L, P2M, lists) visit only its
// non-empty nodes: on clustered inputs most cells of the deep levels are empty
// (about 9 of 10 leaves at depth 11 for two 4M-particle disks), and a thread
// per cell would leave most lanes idle.
__global__ void k_act_flag(const uint32_t* __restrict__ count, int64_t nn, uint32_t* __restrict__ flag)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= nn; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = i < nn && count[i] != 0;
}

__global__ void k_act_scatter(const uint32_t* __restrict__ count, int64_t nn, const uint32_t* __restrict__ pos,
                              uint32_t* __restrict__ act)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn; i += (int64_t)gridDim.x * blockDim.x)
        if (count[i] != 0) act[pos[i]] = (uint32_t)i;
}

int build_active(Handle& h)
{
    cudaStream_t s = h.stream;
    const int64_t nn = h.nnodes;
    int rc;
    if ((rc = ensure(h.act, (nn + 1) * 4)) || (rc = ensure(h.act_pos, (nn + 2) * 4)) ||
        (rc = ensure(h.tmp, scan_tmp_words(nn + 1) * 4)))
        return rc;
    uint32_t* act = P<uint32_t>(h.act);
    uint32_t* pos = P<uint32_t>(h.act_pos);
    k_act_flag<<<grid_for(nn + 1, 256), 256, 0, s>>>(P<uint32_t>(h.count), nn, act);
    if ((rc = exclusive_scan_u32(act, pos, nn + 1, P<uint32_t>(h.tmp), s))) return rc;
    k_act_scatter<<<grid_for(nn, 256), 256, 0, s>>>(P<uint32_t>(h.count), nn, pos, act);
    h.launches += 2;
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

int build_tree(Handle& h, const double* d_pos, int64_t n, double minx, double miny, double maxx, double maxy)
{
    cudaStream_t s = h.stream;
    const double nmx = -minx, nmy = -miny;
    const double ax = maxx + nmx, ay = maxy + nmy;
    const double L = (ax < ay) ? ay : ax;  // compMax(maxPos - minPos) (:84-85)
    if (!(L > 0.0) || !std::isfinite(L)) {
        tc_set_error("bounding box must have a positive finite extent (got %g)", L);
        return TC_ERR_INVALID;
    }
    int depth = h.cfg.depth;
    if (depth < 0) {
        uint32_t d = 0;
        tc_get_depth(h.cfg.max_children, n, &d);
        depth = (int)d;
    }
    if (depth > 15) {
        tc_set_error("tree depth %d exceeds the 15 levels that 32-bit Morton codes resolve", depth);
        return TC_ERR_INVALID;
    }
    int64_t nn = 0;
    tc_node_count((uint32_t)depth, &nn);
    h.depth = depth;
    h.n = n;
    h.nnodes = nn;
    h.minx = minx;
    h.miny = miny;
    h.L = L;
    h.tree_ready = false;
    const bool f64 = h.cfg.precision == TC_PREC_FP64;
    const size_t rs = f64 ? 8 : 4;
    int rc = 0;
    if ((rc = ensure(h.codes, n * 4)) || (rc = ensure(h.perm, n * 4)) || (rc = ensure(h.alt_keys, n * 4)) ||
        (rc = ensure(h.alt_vals, n * 4)) || (rc = ensure(h.pos64, n * 16)) || (rc = ensure(h.prel, n * 2 * rs)) ||
        (rc = ensure(h.count, nn * 4)) || (rc = ensure(h.first, nn * 4)) || (rc = ensure(h.com64, nn * 16)) ||
        (rc = ensure(h.m0, nn * 8)) || (rc = ensure(h.m2, nn * 24)) || (rc = ensure(h.bbc, nn * 16)) ||
        (rc = ensure(h.bblen, nn * 8)) || (rc = ensure(h.comrel, nn * 2 * rs)) || (rc = ensure(h.m0r, nn * rs)) ||
        (rc = ensure(h.m2t, nn * 3 * rs)) || (rc = ensure(h.tmp, radix_tmp_words(n) * 4)) ||
        (rc = ensure(h.err, 64)))
        return rc;

    if ((rc = record(h, 0))) return rc;
    TC_CUDA_TRY(cudaMemsetAsync(h.err.p, 0, sizeof(uint32_t), s));
    // order p in FP32: the physics-mode moments of tree_p.cu.  Codes, permutation and topology are the
    // reference's on every path: FP64 Morton quantisation and a sort over all 32 code bits, whose tie
    // order (stable) fixes the in-leaf order the reference's unstable sort leaves undefined.
    const bool physics = h.cfg.order && !f64;
    // codes by the FP32 fast path; points near a cell edge queued per block for the FP64 path
    const int mgrid = grid_for(n, kMortonThreads);
    if ((rc = ensure(h.mqueue, (size_t)(mgrid * morton_region(n, mgrid) + mgrid) * 4))) return rc;
    uint32_t* mq = P<uint32_t>(h.mqueue);
    uint32_t* mcount = mq + mgrid * morton_region(n, mgrid);
    k_morton_fast<<<mgrid, kMortonThreads, 0, s>>>((const double2*)d_pos, n, minx, miny, maxx, maxy,
                                                   (float)(65536.0 / L), P<uint32_t>(h.codes), P<uint32_t>(h.err), mq,
                                                   mcount);
    k_morton_exact<<<mgrid, kMortonThreads, 0, s>>>((const double2*)d_pos, n, minx, miny, L, mq, mcount,
                                                    P<uint32_t>(h.codes));
    h.launches += 2;
    TC_CUDA_TRY(cudaGetLastError());
    rc = radix_sort_u32(P<uint32_t>(h.codes), P<uint32_t>(h.perm), P<uint32_t>(h.alt_keys), P<uint32_t>(h.alt_vals), n,
                        P<uint32_t>(h.tmp), s, &h.launches, 0);
    if (rc || (rc = record(h, 1))) return rc;
    const uint32_t li = level_index(depth);
    const int64_t nleaf = (int64_t)1 << (2 * depth);
    TC_CUDA_TRY(cudaMemsetAsync(P<uint32_t>(h.count) + li, 0, nleaf * 4, s));
    TC_CUDA_TRY(cudaMemsetAsync(P<uint32_t>(h.first) + li, 0, nleaf * 4, s));
    const double hleaf = L / (double)(1u << depth);
    if (f64) {
        k_gather_bounds<double><<<grid_for(n, 256), 256, 0, s>>>(P<uint32_t>(h.codes), P<uint32_t>(h.perm),
                                                                 (const double2*)d_pos, n, depth, minx, miny, hleaf,
                                                                 P<double2>(h.pos64), P<double>(h.prel),
                                                                 P<uint32_t>(h.first), P<uint32_t>(h.count));
        k_leaf_moments<double><<<grid_for(nleaf, 128), 128, 0, s>>>(
            P<double2>(h.pos64), depth, minx, miny, hleaf, P<uint32_t>(h.count), P<uint32_t>(h.first),
            P<double2>(h.com64), P<double>(h.m0), P<double>(h.m2), P<double2>(h.bbc), P<double>(h.bblen),
            P<double>(h.comrel), P<double>(h.m0r), P<double>(h.m2t));
    } else {
        const int w = 1 << depth;
        if ((rc = ensure(h.celloff, (size_t)w * 8))) return rc;
        k_cell_offsets<<<grid_for(w, 256), 256, 0, s>>>(w, hleaf, P<double>(h.celloff));
        k_gather_bounds_f32<<<grid_for(n, 256), 256, 0, s>>>(P<uint32_t>(h.codes), P<uint32_t>(h.perm),
                                                             (const double2*)d_pos, n, depth, minx, miny,
                                                             P<double>(h.celloff), P<double2>(h.pos64),
                                                             P<float2>(h.prel), P<uint32_t>(h.first),
                                                             P<uint32_t>(h.count));
        h.launches++;
        if (physics) {
            if ((rc = build_records_p(h, hleaf))) return rc;
        } else {
            k_leaf_moments<float><<<grid_for(nleaf, 128), 128, 0, s>>>(
                P<double2>(h.pos64), depth, minx, miny, hleaf, P<uint32_t>(h.count), P<uint32_t>(h.first),
                P<double2>(h.com64), P<double>(h.m0), P<double>(h.m2), P<double2>(h.bbc), P<double>(h.bblen),
                P<float>(h.comrel), P<float>(h.m0r), P<float>(h.m2t));
        }
    }
    h.launches += physics ? 1 : 2;
    for (int l = depth - 1; l >= 0 && !physics; l--) {
        const double hl = L / (double)(1u << l);
        const int64_t nl = (int64_t)1 << (2 * l);
        if (f64)
            k_bottom_up<double><<<grid_for(nl, 128), 128, 0, s>>>(
                l, minx, miny, hl, P<uint32_t>(h.count), P<uint32_t>(h.first), P<double2>(h.com64), P<double>(h.m0),
                P<double>(h.m2), P<double2>(h.bbc), P<double>(h.bblen), P<double>(h.comrel), P<double>(h.m0r),
                P<double>(h.m2t));
        else
            k_bottom_up<float><<<grid_for(nl, 128), 128, 0, s>>>(
                l, minx, miny, hl, P<uint32_t>(h.count), P<uint32_t>(h.first), P<double2>(h.com64), P<double>(h.m0),
                P<double>(h.m2), P<double2>(h.bbc), P<double>(h.bblen), P<float>(h.comrel), P<float>(h.m0r),
                P<float>(h.m2t));
        h.launches++;
    }
    TC_CUDA_TRY(cudaGetLastError());
    if (h.cfg.order && (rc = build_active(h))) return rc;
    // order-p multipoles belong to the tree: the list builder's controller reads them
    if (h.cfg.order && !h.split_mu && (rc = build_multipoles(h))) return rc;
    if ((rc = record(h, 2))) return rc;
    h.tree_ready = true;
    return TC_OK;
}

}  // namespace tc
