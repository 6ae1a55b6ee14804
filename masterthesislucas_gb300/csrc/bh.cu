// Barnes-Hut on the GPU with the reference's own tree: NBodySolverBH + QuadTree
// (src/nbodysolvers/cpu/nBodySolverBH.h:33-116, src/trees/cpu/quadtree.h:29-172).
//
// Tree (level-synchronous, device):
//   root box [lo, lo + D + 1e-4]^2 (D = largest extent, quadtree.h:29-53); a
//   node with more than maxChildren occupants splits at mid = lo + (hi.x-lo.x)/2
//   on both axes (:104-107) into HH, HL, LH, LL (:109-134), each child keeping
//   its parent's occupant order.  Per level: classify the points of splitting
//   nodes, four scans give each point its slot in the stable quadrant
//   partition of its node, children are appended in HH, HL, LH, LL order.
// Masses and COMs (quadtree.h:137-172) are rebuilt bottom-up with the
// reference's types: float totalMass, FP64 COM, and the child COM seen by the
// parent through std::pair<float, glm::vec2>, i.e. rounded to float.
// Traversal (nBodySolverBH.h:56-89): one thread per point, depth-first in the
// children order with the MAC l/|x - com| < theta; a node with at most one
// child is treated as a leaf (PP over all its occupants).  In FP64 the
// result is the reference's, bit for bit (same operations, same order).
//
// The multipole variant (NBodySolverBHMP + QuadTreeMultiPole,
// src/nbodysolvers/cpu/nBodySolverBHMP.h:17-135,
// src/trees/cpu/quadtreemultipole.h:31-289) uses the same tree with FP64
// masses and COMs and a quadrupole sum_c [M_c (dc dc^T) + Q_c]; an accepted
// node contributes the FMM kernels' C1 (monopole + quadrupole).
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "kernels.cuh"
#include "state.cuh"

namespace tc {
namespace {

struct Quad {
    double x, y, z, w;  // xx, xy, yx, yy
};

struct BHNodes {
    double2* lo;
    double2* hi;
    uint32_t* start;
    uint32_t* count;
    uint32_t* first_child;  // index of the first child, valid when nchild > 0
    uint32_t* nchild;
    float* mass;
    double2* com;   // full-precision COM (the node's own member)
    float2* comf;   // the COM its parent sees (float)
    double* m64;    // multipole variant: FP64 mass
    Quad* quad;     // multipole variant: quadrupole
};

// QuadTreeMultiPole::createTree's moments for one level (children done)
__global__ void k_bhmp_moments(uint32_t lvl_begin, uint32_t lvl_end, BHNodes t, const double2* __restrict__ pos,
                               const uint32_t* __restrict__ order)
{
    for (uint32_t k = lvl_begin + blockIdx.x * blockDim.x + threadIdx.x; k < lvl_end; k += gridDim.x * blockDim.x) {
        double m = 0.0, cx = 0.0, cy = 0.0;
        Quad q = {0.0, 0.0, 0.0, 0.0};
        if (t.nchild[k] == 0) {
            for (uint32_t i = t.start[k]; i < t.start[k] + t.count[k]; i++) {
                const double2 p = pos[order[i]];
                m += 1.0;
                cx += 1.0 * p.x;
                cy += 1.0 * p.y;
            }
            cx /= m;
            cy /= m;
            for (uint32_t i = t.start[k]; i < t.start[k] + t.count[k]; i++) {
                const double2 p = pos[order[i]];
                const double rx = p.x - cx, ry = p.y - cy;
                q.x += rx * rx;
                q.y += rx * ry;
                q.z += ry * rx;
                q.w += ry * ry;
            }
        } else {
            const uint32_t f = t.first_child[k], e = f + t.nchild[k];
            for (uint32_t c = f; c < e; c++) {
                const double mc = t.m64[c];
                const double2 cc = t.com[c];
                m += mc;
                cx += mc * cc.x;
                cy += mc * cc.y;
            }
            cx /= m;
            cy /= m;
            for (uint32_t c = f; c < e; c++) {
                const double mc = t.m64[c];
                const double2 cc = t.com[c];
                const double rx = cc.x - cx, ry = cc.y - cy;
                const Quad qc = t.quad[c];
                q.x += mc * (rx * rx);
                q.y += mc * (rx * ry);
                q.z += mc * (ry * rx);
                q.w += mc * (ry * ry);
                q.x += qc.x;
                q.y += qc.y;
                q.z += qc.z;
                q.w += qc.w;
            }
        }
        t.m64[k] = m;
        t.com[k] = make_double2(cx, cy);
        t.quad[k] = q;
    }
}

// C1 of a source of mass m and quadrupole Q at offset R (the FMM kernels' far
// field, nBodySolverBHMP.h:111-126)
template <typename real>
__device__ inline void bh_far_c1(real Rx, real Ry, real m, Quad Q, real D1, real D2, real D3, real& ox, real& oy)
{
    const double inv = 1.0 / (double)m;
    const real Txx = (real)(inv * Q.x), Txy = (real)(inv * Q.y), Tyx = (real)(inv * Q.z), Tyy = (real)(inv * Q.w);
    const real S1 = Txx + Tyy;
    const real S2 = (Rx * Rx * Txx) + (Rx * Ry * Txy) + (Ry * Rx * Tyx) + (Ry * Ry * Tyy);
    const real S3x = Rx * Txx + Ry * Txy;
    const real S3y = Rx * Tyx + Ry * Tyy;
    const real base = D1 + real(0.5) * S1 * D2 + real(0.5) * S2 * D3;
    ox = m * (Rx * base + S3x * D2);
    oy = m * (Ry * base + S3y * D2);
}

__global__ void k_bh_root(const double* __restrict__ keys, uint32_t n, BHNodes t)
{
    // keys: order-preserving images of min x, min y, max x, max y
    const unsigned long long* k = reinterpret_cast<const unsigned long long*>(keys);
    const double lx = bbox_unkey(k[0]), ly = bbox_unkey(k[1]);
    const double hx = bbox_unkey(k[2]), hy = bbox_unkey(k[3]);
    const double ax = hx - lx, ay = hy - ly;
    const double ld = (ax < ay) ? ay : ax;  // std::max(a, b)
    t.lo[0] = make_double2(lx, ly);
    t.hi[0] = make_double2(lx + ld + 0.0001, ly + ld + 0.0001);
    t.start[0] = 0;
    t.count[0] = n;
    t.nchild[0] = 0;
    t.first_child[0] = 0;
}

__device__ inline int quadrant(double x, double y, double2 lo, double2 hi)
{
    const double l = (hi.x - lo.x) / 2.0;
    const double mx = lo.x + l, my = lo.y + l;
    if (x >= mx && y >= my) return 0;  // HH
    if (x >= mx && y < my) return 1;   // HL
    if (x < mx && y >= my) return 2;   // LH
    return 3;                          // LL
}

// points of splitting nodes of this level: quadrant indicators
__global__ void k_bh_classify(const double2* __restrict__ pos, const uint32_t* __restrict__ order,
                              const uint32_t* __restrict__ node_of, uint32_t n, uint32_t lvl_begin, uint32_t lvl_end,
                              BHNodes t, int maxc, uint32_t* __restrict__ ind /* 4 x n */, uint8_t* __restrict__ q)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t nd = node_of[i];
        int qq = 4;
        if (nd >= lvl_begin && nd < lvl_end && t.count[nd] > (uint32_t)maxc) {
            const double2 p = pos[order[i]];
            qq = quadrant(p.x, p.y, t.lo[nd], t.hi[nd]);
        }
        q[i] = (uint8_t)qq;
        for (int k = 0; k < 4; k++) ind[(size_t)k * n + i] = (qq == k);
    }
}

// per splitting node of the level: number of non-empty children (for the child scan)
__global__ void k_bh_nchild(uint32_t lvl_begin, uint32_t lvl_end, BHNodes t, int maxc,
                            const uint32_t* __restrict__ pre /* 4 x (n+1) */, uint32_t n, uint32_t* __restrict__ nc)
{
    for (uint32_t k = lvl_begin + blockIdx.x * blockDim.x + threadIdx.x; k < lvl_end; k += gridDim.x * blockDim.x) {
        uint32_t c = 0;
        if (t.count[k] > (uint32_t)maxc) {
            const uint32_t s = t.start[k], e = s + t.count[k];
            for (int qd = 0; qd < 4; qd++) c += (pre[(size_t)qd * (n + 1) + e] - pre[(size_t)qd * (n + 1) + s]) > 0;
        }
        nc[k - lvl_begin] = c;
    }
}

// create the children of the splitting nodes (appended at child_base + offset)
__global__ void k_bh_children(uint32_t lvl_begin, uint32_t lvl_end, BHNodes t, int maxc,
                              const uint32_t* __restrict__ pre, uint32_t n, const uint32_t* __restrict__ coff,
                              uint32_t child_base)
{
    for (uint32_t k = lvl_begin + blockIdx.x * blockDim.x + threadIdx.x; k < lvl_end; k += gridDim.x * blockDim.x) {
        if (t.count[k] <= (uint32_t)maxc) {
            t.nchild[k] = 0;
            continue;
        }
        const uint32_t s = t.start[k], e = s + t.count[k];
        const double2 lo = t.lo[k], hi = t.hi[k];
        const double l = (hi.x - lo.x) / 2.0;
        const double mx = lo.x + l, my = lo.y + l;
        const double2 clo[4] = {make_double2(mx, my), make_double2(mx, lo.y), make_double2(lo.x, my), lo};
        const double2 chi[4] = {hi, make_double2(hi.x, my), make_double2(mx, hi.y), make_double2(mx, my)};
        uint32_t c = child_base + coff[k - lvl_begin];
        t.first_child[k] = c;
        uint32_t nc = 0, off = s;
        for (int qd = 0; qd < 4; qd++) {
            const uint32_t cnt = pre[(size_t)qd * (n + 1) + e] - pre[(size_t)qd * (n + 1) + s];
            if (cnt == 0) continue;
            t.lo[c] = clo[qd];
            t.hi[c] = chi[qd];
            t.start[c] = off;
            t.count[c] = cnt;
            t.nchild[c] = 0;
            t.first_child[c] = 0;
            off += cnt;
            c++;
            nc++;
        }
        t.nchild[k] = nc;
    }
}

// stable partition of each splitting node's occupants by quadrant
__global__ void k_bh_scatter(const uint32_t* __restrict__ order, const uint32_t* __restrict__ node_of,
                             const uint8_t* __restrict__ q, uint32_t n, BHNodes t,
                             const uint32_t* __restrict__ pre, uint32_t* __restrict__ order2,
                             uint32_t* __restrict__ node_of2)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int qq = q[i];
        const uint32_t nd = node_of[i];
        if (qq == 4) {
            order2[i] = order[i];
            node_of2[i] = nd;
            continue;
        }
        const uint32_t s = t.start[nd], e = s + t.count[nd];
        uint32_t dst = s, child = t.first_child[nd];
        for (int k = 0; k < qq; k++) {
            const uint32_t cnt = pre[(size_t)k * (n + 1) + e] - pre[(size_t)k * (n + 1) + s];
            dst += cnt;
            child += cnt > 0;
        }
        dst += pre[(size_t)qq * (n + 1) + i] - pre[(size_t)qq * (n + 1) + s];
        order2[dst] = order[i];
        node_of2[dst] = child;
    }
}

// createTree's mass/COM for the nodes of one level (children already done)
__global__ void k_bh_mass(uint32_t lvl_begin, uint32_t lvl_end, BHNodes t, const double2* __restrict__ pos,
                          const uint32_t* __restrict__ order)
{
    for (uint32_t k = lvl_begin + blockIdx.x * blockDim.x + threadIdx.x; k < lvl_end; k += gridDim.x * blockDim.x) {
        float tm = 0.0f;
        double cx = 0.0, cy = 0.0;
        if (t.nchild[k] == 0) {
            for (uint32_t i = t.start[k]; i < t.start[k] + t.count[k]; i++) {
                tm = (float)((double)tm + 1.0);
                const double2 p = pos[order[i]];
                cx += 1.0 * p.x;
                cy += 1.0 * p.y;
            }
        } else {
            for (uint32_t c = t.first_child[k]; c < t.first_child[k] + t.nchild[k]; c++) {
                const double m = (double)t.mass[c];
                tm = (float)((double)tm + m);
                const float2 cc = t.comf[c];
                cx += m * (double)cc.x;
                cy += m * (double)cc.y;
            }
        }
        cx /= (double)tm;
        cy /= (double)tm;
        t.mass[k] = tm;
        t.com[k] = make_double2(cx, cy);
        t.comf[k] = make_float2((float)cx, (float)cy);
    }
}

constexpr int kBHStack = 128;

// traverseBH (nBodySolverBH.h:56-89) per point, depth first in children order
template <typename real, typename K, bool MP>
__global__ void __launch_bounds__(128) k_bh_traverse(K ker, const double2* __restrict__ pos, uint32_t n, BHNodes t,
                                                     const uint32_t* __restrict__ order, double theta,
                                                     double* __restrict__ grad, double* __restrict__ zrow,
                                                     uint32_t* __restrict__ err)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const double2 x = pos[p];
        real gx = 0, gy = 0, z = 0;
        uint32_t stack[kBHStack];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const uint32_t nd = stack[--sp];
            const double l = t.hi[nd].x - t.lo[nd].x;
            const double2 c = t.com[nd];
            const double dx = x.x - c.x, dy = x.y - c.y;
            const double len = sqrt(dx * dx + dy * dy);
            if (l / len < theta) {
                if constexpr (MP) {
                    const real tm = (real)t.m64[nd];
                    real D1, D2, D3, tt;
                    ker.far((real)(dx * dx + dy * dy), D1, D2, D3, tt);
                    real cx1, cy1;
                    bh_far_c1<real>((real)dx, (real)dy, tm, t.quad[nd], D1, D2, D3, cx1, cy1);
                    z += tm * tt;
                    gx += cx1;
                    gy += cy1;
                } else {
                    const real tm = (real)t.mass[nd];
                    real D1, tt;
                    ker.near((real)(dx * dx + dy * dy), D1, tt);
                    z += tm * tt;
                    gx += tm * D1 * (real)dx;
                    gy += tm * D1 * (real)dy;
                }
            } else if (t.nchild[nd] <= 1) {
                for (uint32_t i = t.start[nd]; i < t.start[nd] + t.count[nd]; i++) {
                    const uint32_t o = order[i];
                    if (o == p) continue;
                    const double2 q = pos[o];
                    const double ex = x.x - q.x, ey = x.y - q.y;
                    real D1, tt;
                    ker.near((real)(ex * ex + ey * ey), D1, tt);
                    z += tt;
                    gx += D1 * (real)ex;
                    gy += D1 * (real)ey;
                }
            } else {
                const uint32_t f = t.first_child[nd], nc = t.nchild[nd];
                if (sp + (int)nc > kBHStack) {
                    atomicOr(err, 2u);  // stack exhausted: report, stop this point
                    break;
                }
                for (int c = (int)nc - 1; c >= 0; c--) stack[sp++] = f + (uint32_t)c;
            }
        }
        grad[2 * p] = (double)gx;
        grad[2 * p + 1] = (double)gy;
        zrow[p] = (double)z;
    }
}

// Scratch of one call, carved from a per-device workspace that persists
// between calls and only grows (calls on one device are serialised by its
// mutex), so that repeated solves allocate nothing after the first.
struct BHWork {
    std::mutex mu;
    Buf slot[32];
    cudaEvent_t done = nullptr;  // recorded after each call's last use of the workspace
    bool recorded = false;
};

// records the workspace's completion event on every exit of a call
struct WorkRelease {
    BHWork& w;
    cudaStream_t s;
    ~WorkRelease()
    {
        if (w.done && cudaEventRecord(w.done, s) == cudaSuccess) w.recorded = true;
    }
};

__global__ void k_bh_iota(uint32_t* __restrict__ order, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) order[i] = i;
}

BHWork& bh_work(int dev)
{
    static std::mutex m;
    static std::map<int, std::unique_ptr<BHWork>> w;
    std::lock_guard<std::mutex> g(m);
    auto& p = w[dev];
    if (!p) p.reset(new BHWork());
    return *p;
}

struct DevBuf {
    void* p = nullptr;
};

thread_local BHWork* g_work = nullptr;
thread_local int g_slot = 0;

template <typename T>
int dalloc(DevBuf& b, size_t count)
{
    if (!g_work || g_slot >= 32) {
        tc_set_error("bh: workspace slots exhausted");
        return TC_ERR_STATE;
    }
    Buf& w = g_work->slot[g_slot++];
    int rc = ensure(w, count * sizeof(T) + 16);
    if (rc) return rc;
    b.p = w.p;
    return TC_OK;
}

}  // namespace



}  // namespace tc

using namespace tc;

namespace tc {
namespace {

int bh_solve_impl(int kernel, double softening, int max_children, double theta, int precision,
                  const double* d_pos_xy, int64_t n64, double* d_grad_xy, double* d_total, void* stream, bool mp)
{
    if (!d_pos_xy || !d_grad_xy || n64 <= 0 || n64 > (1 << 30) || max_children <= 0 || !(theta > 0.0) ||
        (kernel != TC_KERNEL_TSNE && kernel != TC_KERNEL_GRAVITY)) {
        tc_set_error("tc_bh_solve_device: invalid arguments");
        return TC_ERR_INVALID;
    }
    const uint32_t n = (uint32_t)n64;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = TC_OK;
    int dev = 0;
    TC_CUDA_TRY(cudaGetDevice(&dev));
    BHWork& work = bh_work(dev);
    std::lock_guard<std::mutex> work_lock(work.mu);
    if (!work.done) TC_CUDA_TRY(cudaEventCreateWithFlags(&work.done, cudaEventDisableTiming));
    // the previous call's kernels (possibly on another stream) finish first
    if (work.recorded) TC_CUDA_TRY(cudaStreamWaitEvent(s, work.done, 0));
    WorkRelease release_on_exit{work, s};
    g_work = &work;
    g_slot = 0;
    // node capacity (splits past it are refused, not written)
    const size_t cap = (size_t)4 * n + 64;
    DevBuf b_lo, b_hi, b_start, b_count, b_fc, b_nc, b_mass, b_com, b_comf, b_order, b_order2, b_nodeof, b_nodeof2,
        b_q, b_ind, b_pre, b_nck, b_coff, b_tmp, b_bbox, b_zrow, b_err;
    if ((rc = dalloc<double2>(b_lo, cap)) || (rc = dalloc<double2>(b_hi, cap)) || (rc = dalloc<uint32_t>(b_start, cap)) ||
        (rc = dalloc<uint32_t>(b_count, cap)) || (rc = dalloc<uint32_t>(b_fc, cap)) ||
        (rc = dalloc<uint32_t>(b_nc, cap)) || (rc = dalloc<float>(b_mass, cap)) || (rc = dalloc<double2>(b_com, cap)) ||
        (rc = dalloc<float2>(b_comf, cap)) || (rc = dalloc<uint32_t>(b_order, n)) ||
        (rc = dalloc<uint32_t>(b_order2, n)) || (rc = dalloc<uint32_t>(b_nodeof, n)) ||
        (rc = dalloc<uint32_t>(b_nodeof2, n)) || (rc = dalloc<uint8_t>(b_q, n)) ||
        (rc = dalloc<uint32_t>(b_ind, (size_t)4 * n)) || (rc = dalloc<uint32_t>(b_pre, (size_t)4 * (n + 1))) ||
        (rc = dalloc<uint32_t>(b_nck, cap)) || (rc = dalloc<uint32_t>(b_coff, cap + 1)) ||
        (rc = dalloc<uint32_t>(b_tmp, (size_t)scan_tmp_words((int64_t)cap + n) + 16)) ||
        (rc = dalloc<double>(b_bbox, 4)) || (rc = dalloc<double>(b_zrow, n)) || (rc = dalloc<uint32_t>(b_err, 4)))
        return rc;
    DevBuf b_m64, b_quad;
    if (mp && ((rc = dalloc<double>(b_m64, cap)) || (rc = dalloc<Quad>(b_quad, cap)))) return rc;
    BHNodes t{(double2*)b_lo.p, (double2*)b_hi.p, (uint32_t*)b_start.p, (uint32_t*)b_count.p, (uint32_t*)b_fc.p,
              (uint32_t*)b_nc.p, (float*)b_mass.p, (double2*)b_com.p, (float2*)b_comf.p, (double*)b_m64.p,
              (Quad*)b_quad.p};
    uint32_t* order = (uint32_t*)b_order.p;
    uint32_t* order2 = (uint32_t*)b_order2.p;
    uint32_t* node_of = (uint32_t*)b_nodeof.p;
    uint32_t* node_of2 = (uint32_t*)b_nodeof2.p;
    uint32_t* ind = (uint32_t*)b_ind.p;
    uint32_t* pre = (uint32_t*)b_pre.p;
    TC_CUDA_TRY(cudaMemsetAsync(b_err.p, 0, 16, s));
    if ((rc = bbox_keys(d_pos_xy, n64, (double*)b_bbox.p, (uint32_t*)b_err.p, s))) return rc;
    TC_CUDA_TRY(cudaMemsetAsync(node_of, 0, (size_t)n * 4, s));
    k_bh_iota<<<grid_for(n, 256), 256, 0, s>>>(order, n);
    k_bh_root<<<1, 1, 0, s>>>((const double*)b_bbox.p, n, t);
    std::vector<uint32_t> level_begin = {0}, level_end = {1};
    uint32_t total_nodes = 1;
    const int grid = grid_for(n, 256);
    for (int lvl = 0; lvl < 64; lvl++) {
        const uint32_t lb = level_begin.back(), le = level_end.back();
        k_bh_classify<<<grid, 256, 0, s>>>((const double2*)d_pos_xy, order, node_of, n, lb, le, t, max_children, ind,
                                           (uint8_t*)b_q.p);
        for (int k = 0; k < 4; k++)
            if ((rc = exclusive_scan_u32(ind + (size_t)k * n, pre + (size_t)k * (n + 1), n, (uint32_t*)b_tmp.p, s)))
                return rc;
        k_bh_nchild<<<grid_for(le - lb, 256), 256, 0, s>>>(lb, le, t, max_children, pre, n, (uint32_t*)b_nck.p);
        if ((rc = exclusive_scan_u32((uint32_t*)b_nck.p, (uint32_t*)b_coff.p, le - lb, (uint32_t*)b_tmp.p, s))) return rc;
        uint32_t nnew = 0;
        TC_CUDA_TRY(cudaMemcpyAsync(&nnew, (uint32_t*)b_coff.p + (le - lb), 4, cudaMemcpyDeviceToHost, s));
        TC_CUDA_TRY(cudaStreamSynchronize(s));
        if (total_nodes + nnew > cap) {
            tc_set_error("tc_bh_solve_device: node capacity exceeded (coincident points?)");
            return TC_ERR_INVALID;
        }
        k_bh_children<<<grid_for(le - lb, 256), 256, 0, s>>>(lb, le, t, max_children, pre, n, (uint32_t*)b_coff.p,
                                                            total_nodes);
        if (nnew == 0) break;
        k_bh_scatter<<<grid, 256, 0, s>>>(order, node_of, (const uint8_t*)b_q.p, n, t, pre, order2, node_of2);
        std::swap(order, order2);
        std::swap(node_of, node_of2);
        level_begin.push_back(total_nodes);
        total_nodes += nnew;
        level_end.push_back(total_nodes);
        if (lvl == 63) {
            tc_set_error("tc_bh_solve_device: tree deeper than 64 levels (coincident points?)");
            return TC_ERR_INVALID;
        }
    }
    for (int l = (int)level_begin.size() - 1; l >= 0; l--) {
        if (mp)
            k_bhmp_moments<<<grid_for(level_end[l] - level_begin[l], 128), 128, 0, s>>>(
                level_begin[l], level_end[l], t, (const double2*)d_pos_xy, order);
        else
            k_bh_mass<<<grid_for(level_end[l] - level_begin[l], 128), 128, 0, s>>>(level_begin[l], level_end[l], t,
                                                                                   (const double2*)d_pos_xy, order);
    }
    const double e2 = softening * softening;
    const double2* P2 = (const double2*)d_pos_xy;
    double* zr = (double*)b_zrow.p;
    uint32_t* er = (uint32_t*)b_err.p;
    const int gt = grid_for(n, 128);
    if (precision == TC_PREC_FP64) {
        if (kernel == TC_KERNEL_GRAVITY) {
            if (mp)
                k_bh_traverse<double, KGrav<double>, true>
                    <<<gt, 128, 0, s>>>(KGrav<double>{e2}, P2, n, t, order, theta, d_grad_xy, zr, er);
            else
                k_bh_traverse<double, KGrav<double>, false>
                    <<<gt, 128, 0, s>>>(KGrav<double>{e2}, P2, n, t, order, theta, d_grad_xy, zr, er);
        } else {
            if (mp)
                k_bh_traverse<double, KTsne<double>, true>
                    <<<gt, 128, 0, s>>>(KTsne<double>{}, P2, n, t, order, theta, d_grad_xy, zr, er);
            else
                k_bh_traverse<double, KTsne<double>, false>
                    <<<gt, 128, 0, s>>>(KTsne<double>{}, P2, n, t, order, theta, d_grad_xy, zr, er);
        }
    } else {
        if (kernel == TC_KERNEL_GRAVITY) {
            if (mp)
                k_bh_traverse<float, KGrav<float>, true>
                    <<<gt, 128, 0, s>>>(KGrav<float>{(float)e2}, P2, n, t, order, theta, d_grad_xy, zr, er);
            else
                k_bh_traverse<float, KGrav<float>, false>
                    <<<gt, 128, 0, s>>>(KGrav<float>{(float)e2}, P2, n, t, order, theta, d_grad_xy, zr, er);
        } else {
            if (mp)
                k_bh_traverse<float, KTsne<float>, true>
                    <<<gt, 128, 0, s>>>(KTsne<float>{}, P2, n, t, order, theta, d_grad_xy, zr, er);
            else
                k_bh_traverse<float, KTsne<float>, false>
                    <<<gt, 128, 0, s>>>(KTsne<float>{}, P2, n, t, order, theta, d_grad_xy, zr, er);
        }
    }
    DevBuf b_sum;
    if ((rc = dalloc<double>(b_sum, sum_tmp_doubles()))) return rc;
    if (d_total && (rc = sum_f64((const double*)b_zrow.p, n, nullptr, nullptr, d_total, 0, (double*)b_sum.p, s)))
        return rc;
    uint32_t herr = 0;
    TC_CUDA_TRY(cudaMemcpyAsync(&herr, b_err.p, 4, cudaMemcpyDeviceToHost, s));
    TC_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr) {
        tc_set_error("tc_bh_solve_device: traversal stack exhausted");
        return TC_ERR_INVALID;
    }
    return TC_OK;
}

}  // namespace
}  // namespace tc

extern "C" int tc_bh_solve_device(int kernel, double softening, int max_children, double theta, int precision,
                                  const double* d_pos_xy, int64_t n64, double* d_grad_xy, double* d_total,
                                  void* stream)
{
    return bh_solve_impl(kernel, softening, max_children, theta, precision, d_pos_xy, n64, d_grad_xy, d_total, stream,
                         false);
}

extern "C" int tc_bhmp_solve_device(int kernel, double softening, int max_children, double theta, int precision,
                                    const double* d_pos_xy, int64_t n64, double* d_grad_xy, double* d_total,
                                    void* stream)
{
    return bh_solve_impl(kernel, softening, max_children, theta, precision, d_pos_xy, n64, d_grad_xy, d_total, stream,
                         true);
}

struct OwnBuf {
    void* p = nullptr;
    ~OwnBuf() { if (p) cudaFree(p); }
};

static int bh_solve_host(int kernel, double softening, int max_children, double theta, int precision,
                         const double* pos_xy, int64_t n, double* grad_xy, double* total, bool mp)
{
    if (!pos_xy || !grad_xy || n <= 0) {
        tc_set_error("tc_bh_solve: invalid arguments");
        return TC_ERR_INVALID;
    }
    cudaStream_t s;
    TC_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    OwnBuf dp, dg, dt;
    int rc = TC_OK;
    cudaError_t e = cudaMalloc(&dp.p, (size_t)n * 16);
    if (e == cudaSuccess) e = cudaMalloc(&dg.p, (size_t)n * 16);
    if (e == cudaSuccess) e = cudaMalloc(&dt.p, 8);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dp.p, pos_xy, (size_t)n * 16, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        rc = tc::bh_solve_impl(kernel, softening, max_children, theta, precision, (const double*)dp.p, n,
                               (double*)dg.p, (double*)dt.p, s, mp);
        if (rc == TC_OK) e = cudaMemcpyAsync(grad_xy, dg.p, (size_t)n * 16, cudaMemcpyDeviceToHost, s);
        if (rc == TC_OK && e == cudaSuccess && total) e = cudaMemcpyAsync(total, dt.p, 8, cudaMemcpyDeviceToHost, s);
    }
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (rc) return rc;
    if (e != cudaSuccess) return tc_cuda_fail(e, "tc_bh_solve");
    if (e2 != cudaSuccess) return tc_cuda_fail(e2, "tc_bh_solve sync");
    return TC_OK;
}

extern "C" int tc_bh_solve(int kernel, double softening, int max_children, double theta, int precision,
                           const double* pos_xy, int64_t n, double* grad_xy, double* total)
{
    return bh_solve_host(kernel, softening, max_children, theta, precision, pos_xy, n, grad_xy, total, false);
}

extern "C" int tc_bhmp_solve(int kernel, double softening, int max_children, double theta, int precision,
                             const double* pos_xy, int64_t n, double* grad_xy, double* total)
{
    return bh_solve_host(kernel, softening, max_children, theta, precision, pos_xy, n, grad_xy, total, true);
}
