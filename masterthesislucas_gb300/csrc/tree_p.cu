// Tree records for the order-p path ("physics mode"): the same level-dense
// quadtree as NBodySolverFMM_SYM_MORTON::updateTree
// (src/nbodysolvers/cpu/nBodySolverFMM_SYM_MORTON.h:79-95, 328-470).  Codes,
// permutation and topology come from the bit-exact k_morton + 32-bit sort of
// tree.cu, so counts, first particles, child links and the FP64 boxes
// (BBcentre, BBlength, rounded in the reference's operation order) are the
// reference's.  The moments are built without the FP64 arithmetic the
// reference-order path needs for bit parity -- FP64 runs at 1/64 of the FP32
// rate on GB300, and the order-p solve reads only cell-relative FP32 data:
// * leaf centres of mass and second moments are FP32 sums of the particles'
//   cell-relative coordinates (written by the gather in FP64 arithmetic);
// * internal nodes combine their children's relative centres of mass shifted
//   by the exact child-centre offsets (+-h/4), mass-weighted (the physical
//   parallel-axis second moment, not the reference's quirk).
// The FP64 records (com64 = cell centre + relative COM, m0, m2, bbc, bblen)
// are written for non-empty nodes only; readers test count first.
#include "state.cuh"

namespace tc {
namespace {

__device__ inline double2 cell_centre(int64_t i, double minx, double miny, double h)
{
    const uint32_t ix = compact16((uint32_t)i), iy = compact16((uint32_t)i >> 1);
    return make_double2(minx + ((double)ix + 0.5) * h, miny + ((double)iy + 0.5) * h);
}

// createLeafNodes' box (:343-345): BBcentre = (minPos + h * g) + 0.5 * h, with
// round-to-nearest operations the compiler does not contract into FMAs
__device__ inline double2 leaf_box(int64_t i, double minx, double miny, double h)
{
    const uint32_t ix = compact16((uint32_t)i), iy = compact16((uint32_t)i >> 1);
    const double hh = __dmul_rn(0.5, h);
    return make_double2(__dadd_rn(__dadd_rn(minx, __dmul_rn(h, (double)ix)), hh),
                        __dadd_rn(__dadd_rn(miny, __dmul_rn(h, (double)iy)), hh));
}

// the node record from its relative COM and second moment (about the COM);
// centre is the compute frame's cell centre, box the reference's BBcentre
__device__ inline void write_node(int64_t node, double2 centre, double2 box, double h, uint32_t c, float rx,
                                  float ry, float a, float b, float d, float br, double2* com64, double* m0,
                                  double* m2, double2* bbc, double* bblen, float* comrel, float* m0r, float* m2t,
                                  float* bmax)
{
    bmax[node] = br;
    const float ic = 1.0f / (float)c;
    com64[node] = make_double2(centre.x + (double)rx, centre.y + (double)ry);
    m0[node] = (double)c;
    m2[3 * node] = (double)a;
    m2[3 * node + 1] = (double)b;
    m2[3 * node + 2] = (double)d;
    bbc[node] = box;
    bblen[node] = h;
    comrel[2 * node] = rx;
    comrel[2 * node + 1] = ry;
    m0r[node] = (float)c;
    m2t[3 * node] = a * ic;
    m2t[3 * node + 1] = b * ic;
    m2t[3 * node + 2] = d * ic;
}

// leaves of up to kLeafSmall particles, one thread each; larger leaves are
// listed for k_leaf_big_p.  count holds the end index on entry.
__global__ void k_leaf_small_p(int depth, double minx, double miny, double h, uint32_t* __restrict__ count,
                               const uint32_t* __restrict__ first, const float2* __restrict__ prel,
                               double2* __restrict__ com64, double* __restrict__ m0, double* __restrict__ m2,
                               double2* __restrict__ bbc, double* __restrict__ bblen, float* __restrict__ comrel,
                               float* __restrict__ m0r, float* __restrict__ m2t, uint32_t* __restrict__ big,
                               float* __restrict__ bmax, int box)
{
    const uint32_t li = level_index(depth);
    const int64_t nl = (int64_t)1 << (2 * depth);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nl; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t node = li + i;
        const uint32_t e = count[node];
        if (e == 0) continue;  // empty (first and count were zeroed)
        const uint32_t f = first[node];
        const uint32_t c = e - f;
        count[node] = c;
        if (c > kLeafSmall) {
            big[1 + atomicAdd(big, 1u)] = (uint32_t)i;
            continue;
        }
        float sx = 0.f, sy = 0.f;
        for (uint32_t p = f; p < e; p++) {
            const float2 q = prel[p];
            sx += q.x;
            sy += q.y;
        }
        const float ic = 1.0f / (float)c;
        sx *= ic;
        sy *= ic;
        float a = 0.f, b = 0.f, d = 0.f, r2 = 0.f, c2 = 0.f;
        for (uint32_t p = f; p < e; p++) {
            const float2 q = prel[p];
            const float rx = q.x - sx, ry = q.y - sy;
            a = fmaf(rx, rx, a);
            b = fmaf(rx, ry, b);
            d = fmaf(ry, ry, d);
            r2 = fmaxf(r2, fmaf(rx, rx, ry * ry));
            c2 = fmaxf(c2, fmaf(q.x, q.x, q.y * q.y));
        }
        write_node(node, cell_centre(i, minx, miny, h), leaf_box(i, minx, miny, h), h, c, box ? 0.f : sx,
                   box ? 0.f : sy, a, b, d, sqrtf(box ? c2 : r2), com64, m0, m2, bbc, bblen, comrel, m0r, m2t, bmax);
    }
}

__global__ void k_leaf_big_p(int depth, double minx, double miny, double h, const uint32_t* __restrict__ count,
                             const uint32_t* __restrict__ first, const float2* __restrict__ prel,
                             double2* __restrict__ com64, double* __restrict__ m0, double* __restrict__ m2,
                             double2* __restrict__ bbc, double* __restrict__ bblen, float* __restrict__ comrel,
                             float* __restrict__ m0r, float* __restrict__ m2t, const uint32_t* __restrict__ big,
                             float* __restrict__ bmax, int box)
{
    const int lane = threadIdx.x & 31;
    const uint32_t li = level_index(depth);
    const int64_t nbig = big[0];
    const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); w < nbig; w += wstride) {
        const int64_t i = big[1 + w];
        const int64_t node = li + i;
        const uint32_t c = count[node], f = first[node];
        float sx = 0.f, sy = 0.f;
        for (uint32_t p = f + lane; p < f + c; p += 32) {
            const float2 q = prel[p];
            sx += q.x;
            sy += q.y;
        }
        const float ic = 1.0f / (float)c;
        sx = warp_sum(sx) * ic;
        sy = warp_sum(sy) * ic;
        float a = 0.f, b = 0.f, d = 0.f, r2 = 0.f, c2 = 0.f;
        for (uint32_t p = f + lane; p < f + c; p += 32) {
            const float2 q = prel[p];
            const float rx = q.x - sx, ry = q.y - sy;
            a = fmaf(rx, rx, a);
            b = fmaf(rx, ry, b);
            d = fmaf(ry, ry, d);
            r2 = fmaxf(r2, fmaf(rx, rx, ry * ry));
            c2 = fmaxf(c2, fmaf(q.x, q.x, q.y * q.y));
        }
        a = warp_sum(a);
        b = warp_sum(b);
        d = warp_sum(d);
        for (int o = 16; o > 0; o >>= 1) {
            r2 = fmaxf(r2, __shfl_xor_sync(0xffffffffu, r2, o));
            c2 = fmaxf(c2, __shfl_xor_sync(0xffffffffu, c2, o));
        }
        if (lane == 0)
            write_node(node, cell_centre(i, minx, miny, h), leaf_box(i, minx, miny, h), h, c, box ? 0.f : sx,
                       box ? 0.f : sy, a, b, d, sqrtf(box ? c2 : r2), com64, m0, m2, bbc, bblen, comrel, m0r, m2t,
                       bmax);
    }
}

// node i of level l from level l + 1: counts, first particle (lowest
// non-empty child), mass-weighted COM and second moment in the node's
// cell-relative frame (child centre = node centre + (+-h/4, +-h/4), bit 0 of
// the child slot is x)
__device__ __forceinline__ void bottom_up_node(int l, int64_t i, double minx, double miny, double hl,
                                               uint32_t* __restrict__ count, uint32_t* __restrict__ first,
                                               double2* __restrict__ com64, double* __restrict__ m0,
                                               double* __restrict__ m2, double2* __restrict__ bbc,
                                               double* __restrict__ bblen, float* __restrict__ comrel,
                                               float* __restrict__ m0r, float* __restrict__ m2t,
                                               float* __restrict__ bmax, int box)
{
    const uint32_t li = level_index(l), lc = level_index(l + 1);
    const float q = (float)(0.25 * hl);
    const float2* cr2 = reinterpret_cast<const float2*>(comrel);
    const int64_t node = li + i;
    const int64_t fc = lc + 4 * i;
    const uint32_t c4[4] = {count[fc], count[fc + 1], count[fc + 2], count[fc + 3]};
    const uint32_t cnt = c4[0] + c4[1] + c4[2] + c4[3];
    if (cnt == 0) {
        count[node] = 0;
        first[node] = 0;
        return;
    }
    uint32_t fp = 0;
    float sx = 0.f, sy = 0.f;
    float2 g[4];
    double2 bbox = make_double2(0.0, 0.0);
#pragma unroll
    for (int j = 3; j >= 0; j--) {
        g[j] = make_float2(0.f, 0.f);
        if (c4[j] == 0) continue;
        fp = first[fc + j];
        // bottomUpNodeConstruction's box (:381-470): offset[j] * L_child + BBcentre_child, the lowest
        // non-empty child last (bit 0 of the child slot is x)
        const double cl = bblen[fc + j];
        const double2 cb = bbc[fc + j];
        bbox = make_double2(__dadd_rn(__dmul_rn((j & 1) ? -0.5 : 0.5, cl), cb.x),
                           __dadd_rn(__dmul_rn((j & 2) ? -0.5 : 0.5, cl), cb.y));
        const float2 r = cr2[fc + j];
        g[j] = make_float2(r.x + ((j & 1) ? q : -q), r.y + ((j & 2) ? q : -q));
        sx = fmaf((float)c4[j], g[j].x, sx);
        sy = fmaf((float)c4[j], g[j].y, sy);
    }
    const float ic = 1.0f / (float)cnt;
    sx *= ic;
    sy *= ic;
    // box-centred expansions: the node's frame is its cell centre, and bmax bounds its particles'
    // distance from there
    if (box) sx = sy = 0.f;
    float a = 0.f, b = 0.f, d = 0.f, br = 0.f;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        if (c4[j] == 0) continue;
        const float w = (float)c4[j];
        const float rx = g[j].x - sx, ry = g[j].y - sy;
        a += w * (m2t[3 * (fc + j)] + rx * rx);
        b += w * (m2t[3 * (fc + j) + 1] + rx * ry);
        d += w * (m2t[3 * (fc + j) + 2] + ry * ry);
        // every particle of child j lies within bmax_j of the child's COM
        br = fmaxf(br, sqrtf(fmaf(rx, rx, ry * ry)) + bmax[fc + j]);
    }
    count[node] = cnt;
    first[node] = fp;
    write_node(node, cell_centre(i, minx, miny, hl), bbox, hl, cnt, sx, sy, a, b, d, br, com64, m0, m2, bbc, bblen,
               comrel, m0r, m2t, bmax);
}

// level l from level l + 1, a thread per node
__global__ void k_bottom_up_p(int l, double minx, double miny, double hl, uint32_t* __restrict__ count,
                              uint32_t* __restrict__ first, double2* __restrict__ com64, double* __restrict__ m0,
                              double* __restrict__ m2, double2* __restrict__ bbc, double* __restrict__ bblen,
                              float* __restrict__ comrel, float* __restrict__ m0r, float* __restrict__ m2t,
                              float* __restrict__ bmax, int box)
{
    const int64_t nl = (int64_t)1 << (2 * l);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nl; i += (int64_t)gridDim.x * blockDim.x)
        bottom_up_node(l, i, minx, miny, hl, count, first, com64, m0, m2, bbc, bblen, comrel, m0r, m2t, bmax, box);
}

// levels l0 .. 0 in one block (the coarse levels, a few thousand nodes at
// most: per-level launches would cost more than their work), a barrier
// between levels; hl0 is level l0's cell size
constexpr int kBottomUpCoarseLevel = 6;
__global__ void __launch_bounds__(1024) k_bottom_up_coarse(int l0, double minx, double miny, double hl0,
                                                           uint32_t* __restrict__ count, uint32_t* __restrict__ first,
                                                           double2* __restrict__ com64, double* __restrict__ m0,
                                                           double* __restrict__ m2, double2* __restrict__ bbc,
                                                           double* __restrict__ bblen, float* __restrict__ comrel,
                                                           float* __restrict__ m0r, float* __restrict__ m2t,
                                                           float* __restrict__ bmax, int box)
{
    double hl = hl0;
    for (int l = l0; l >= 0; l--) {
        const int64_t nl = (int64_t)1 << (2 * l);
        for (int64_t i = threadIdx.x; i < nl; i += blockDim.x)
            bottom_up_node(l, i, minx, miny, hl, count, first, com64, m0, m2, bbc, bblen, comrel, m0r, m2t, bmax,
                           box);
        __syncthreads();
        hl *= 2.0;
    }
}

}  // namespace

int build_records_p(Handle& h, double hleaf)
{
    cudaStream_t s = h.stream;
    const int depth = h.depth;
    const int64_t nleaf = (int64_t)1 << (2 * depth);
    const int64_t maxbig = h.n / (kLeafSmall + 1) + 1;
    const int box = h.centre == TC_CENTRE_BOX;
    int rc;
    if ((rc = ensure(h.bigleaf, (maxbig + 1) * 4)) || (rc = ensure(h.bmax, h.nnodes * 4))) return rc;
    TC_CUDA_TRY(cudaMemsetAsync(h.bigleaf.p, 0, 4, s));
    k_leaf_small_p<<<grid_for(nleaf, 128), 128, 0, s>>>(
        depth, h.minx, h.miny, hleaf, P<uint32_t>(h.count), P<uint32_t>(h.first), P<float2>(h.prel),
        P<double2>(h.com64), P<double>(h.m0), P<double>(h.m2), P<double2>(h.bbc), P<double>(h.bblen),
        P<float>(h.comrel), P<float>(h.m0r), P<float>(h.m2t), P<uint32_t>(h.bigleaf), P<float>(h.bmax), box);
    k_leaf_big_p<<<grid_for(maxbig * 32, 128), 128, 0, s>>>(
        depth, h.minx, h.miny, hleaf, P<uint32_t>(h.count), P<uint32_t>(h.first), P<float2>(h.prel),
        P<double2>(h.com64), P<double>(h.m0), P<double>(h.m2), P<double2>(h.bbc), P<double>(h.bblen),
        P<float>(h.comrel), P<float>(h.m0r), P<float>(h.m2t), P<uint32_t>(h.bigleaf), P<float>(h.bmax), box);
    h.launches += 2;
    for (int l = depth - 1; l > kBottomUpCoarseLevel; l--) {
        const double hl = h.L / (double)(1u << l);
        const int64_t nl = (int64_t)1 << (2 * l);
        k_bottom_up_p<<<grid_for(nl, 128), 128, 0, s>>>(l, h.minx, h.miny, hl, P<uint32_t>(h.count),
                                                        P<uint32_t>(h.first), P<double2>(h.com64), P<double>(h.m0),
                                                        P<double>(h.m2), P<double2>(h.bbc), P<double>(h.bblen),
                                                        P<float>(h.comrel), P<float>(h.m0r), P<float>(h.m2t),
                                                        P<float>(h.bmax), box);
        h.launches++;
    }
    if (depth > 0) {
        const int l0 = depth - 1 < kBottomUpCoarseLevel ? depth - 1 : kBottomUpCoarseLevel;
        k_bottom_up_coarse<<<1, 1024, 0, s>>>(l0, h.minx, h.miny, h.L / (double)(1u << l0), P<uint32_t>(h.count),
                                              P<uint32_t>(h.first), P<double2>(h.com64), P<double>(h.m0),
                                              P<double>(h.m2), P<double2>(h.bbc), P<double>(h.bblen),
                                              P<float>(h.comrel), P<float>(h.m0r), P<float>(h.m2t), P<float>(h.bmax),
                                              box);
        h.launches++;
    }
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

}  // namespace tc
