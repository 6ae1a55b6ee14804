// The t-SNE gradient step around the force call, device resident:
//   TSNE::updateRepulsive  (src/nBodyInstances/tsne.h:287-301)  g = (4/Z) * repulsion, un-permuted by ID
//   TSNE::updateAttractive (tsne.h:356-381)  g_i += exag * sum_j P_ij q_ij (y_j - y_i), CSR rows
//   TSNE::updatePoints     (tsne.h:179-206)  y' = y + lr g + momentum (y - y_prev)
// The repulsion comes from the tree code with its output scattered straight
// to ID order; the attractive term, the 4/Z scale and the momentum update are
// one fused kernel (one warp per CSR row) that reads Z from device memory.
// Z is summed in FP64; the attractive products run in FP32 on FP64
// differences of the FP64 embedding.
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "state.cuh"

namespace tc {
namespace {

template <typename real>
__device__ inline real rcp1(real x);
template <>
__device__ inline float rcp1<float>(float x) { return __fdividef(1.0f, x); }
template <>
__device__ inline double rcp1<double>(double x) { return 1.0 / x; }

// real: precision of the attractive products (FP32 product path, FP64 parity path)
template <typename real, typename vreal>
__global__ void k_tsne_attr_update(int64_t n, const uint32_t* __restrict__ row_ptr, const uint32_t* __restrict__ col,
                                   const vreal* __restrict__ val, const double2* __restrict__ y,
                                   const double2* __restrict__ y_prev, const double* __restrict__ grad_rep,
                                   const double* __restrict__ z, const double* __restrict__ prm,
                                   const double* __restrict__ lrp, double2* __restrict__ y_next,
                                   double* __restrict__ grad_out)
{
    const int lane = threadIdx.x & 31;
    const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
    const double scale = 4.0 / *z;
    // exaggeration and momentum (prm[0], prm[2]) and the learning rate: device-resident so that a
    // captured step replays with new values
    const double exag = prm[0], mom = prm[2], lr = *lrp;
    for (int64_t i = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += wstride) {
        const double2 yi = y[i];
        const uint32_t e0 = row_ptr[i], e1 = row_ptr[i + 1];
        real ax = 0, ay = 0;
        for (uint32_t e = e0 + lane; e < e1; e += 32) {
            const double2 yj = y[col[e]];
            const real dx = (real)(yj.x - yi.x), dy = (real)(yj.y - yi.y);
            const real q = rcp1<real>(real(1) + (dx * dx + dy * dy));
            const real w = (real)val[e] * q;
            ax += w * dx;
            ay += w * dy;
        }
        ax = warp_sum(ax);
        ay = warp_sum(ay);
        if (lane == 0) {
            const double gx = grad_rep[2 * i] * scale + exag * (double)ax;
            const double gy = grad_rep[2 * i + 1] * scale + exag * (double)ay;
            const double2 yp = y_prev[i];
            y_next[i] = make_double2(yi.x + lr * gx + mom * (yi.x - yp.x), yi.y + lr * gy + mom * (yi.y - yp.y));
            grad_out[2 * i] = gx;
            grad_out[2 * i + 1] = gy;
        }
    }
}

}  // namespace

int device_bbox(Handle& h, const double* d_pos, int64_t n, double mn[2], double mx[2]);

}  // namespace tc

using namespace tc;

struct tc_tsne {
    tc_handle* solver = nullptr;
    Handle* hs = nullptr;
    int64_t n = 0;
    int64_t nnz = 0;
    Buf y[3];       // rotating: current, previous, next
    int cur = 0, prev = 1, next = 2;
    Buf row_ptr, col, val, grad_rep, grad, z, prm;
    double* h_prm = nullptr;  // pinned staging of {exag, lr, momentum}
    double last_z = 0.0;
    int launches = 0;
    // repulsion by the particle-mesh solver instead of the tree (cell_size > 0)
    double pm_cell = 0.0;
};

namespace tc {
namespace {

// One t-SNE step enqueued on the solver's stream, without rotating the
// embedding buffers; prm points at {exag, -, momentum} and lrp at the
// learning rate, on the device.  box: the tree's bounding box (min x, min y,
// max x, max y), or NULL for the embedding's exact extent (a host round trip).
int tsne_enqueue(tc_tsne* t, const double* prm, const double* lrp, const double* box)
{
    Handle& h = *t->hs;
    const double* y = P<double>(t->y[t->cur]);
    int rc, launches = 0;
    if (t->pm_cell > 0.0) {
        // the reference's TSNE with nBodySelect "PM" (tsne.h:116: 4 nodes, cell_size, 4 boxes)
        if ((rc = pm_solve_device(4, t->pm_cell, 4, y, t->n, P<double>(t->grad_rep), P<double>(t->z), h.stream)))
            return rc;
        launches = 40;
    } else {
        rc = box ? tc_update_tree_device(t->solver, y, t->n, box, box + 2)
                 : tc_update_tree_device(t->solver, y, t->n, nullptr, nullptr);
        if (rc) return rc;
        launches = h.launches;
        TC_CUDA_TRY(cudaMemsetAsync(t->z.p, 0, 8, h.stream));
        rc = tc_solve_device(t->solver, P<double>(t->grad_rep), P<double>(t->z), 0, 1);
        if (rc) return rc;
        launches += h.launches;
    }
    if (h.cfg.precision == TC_PREC_FP64)
        k_tsne_attr_update<double, double><<<grid_for(t->n * 32, 256, sm_count() * 32), 256, 0, h.stream>>>(
            t->n, P<uint32_t>(t->row_ptr), P<uint32_t>(t->col), P<double>(t->val), P<double2>(t->y[t->cur]),
            P<double2>(t->y[t->prev]), P<double>(t->grad_rep), P<double>(t->z), prm, lrp, P<double2>(t->y[t->next]),
            P<double>(t->grad));
    else
        k_tsne_attr_update<float, float><<<grid_for(t->n * 32, 256, sm_count() * 32), 256, 0, h.stream>>>(
            t->n, P<uint32_t>(t->row_ptr), P<uint32_t>(t->col), P<float>(t->val), P<double2>(t->y[t->cur]),
            P<double2>(t->y[t->prev]), P<double>(t->grad_rep), P<double>(t->z), prm, lrp, P<double2>(t->y[t->next]),
            P<double>(t->grad));
    TC_CUDA_TRY(cudaGetLastError());
    t->launches = launches + 1;
    return TC_OK;
}

void tsne_rotate(tc_tsne* t)
{
    const int c = t->cur, p = t->prev, nx = t->next;
    t->prev = c;
    t->cur = nx;
    t->next = p;
}

}  // namespace
}  // namespace tc


extern "C" {

int tc_tsne_create(const tc_config* cfg, int64_t n, const uint32_t* row_ptr, const uint32_t* col, const double* val,
                   const double* y0, tc_tsne** out)
{
    if (!cfg || !row_ptr || !col || !val || !y0 || !out || n <= 1) {
        tc_set_error("tc_tsne_create: invalid arguments");
        return TC_ERR_INVALID;
    }
    *out = nullptr;
    tc_config c = *cfg;
    c.kernel = TC_KERNEL_TSNE;
    tc_tsne* t = new tc_tsne();
    int rc = tc_create(&c, &t->solver);
    if (rc) {
        delete t;
        return rc;
    }
    t->hs = &t->solver->h;
    Handle& h = *t->hs;
    t->n = n;
    t->nnz = row_ptr[n];
    for (int64_t i = 0; i < n; i++)
        if (row_ptr[i + 1] < row_ptr[i]) rc = TC_ERR_INVALID;
    for (int64_t e = 0; e < t->nnz && rc == TC_OK; e++)
        if (col[e] >= (uint64_t)n || !std::isfinite(val[e])) rc = TC_ERR_INVALID;
    if (rc) {
        tc_set_error("tc_tsne_create: malformed CSR affinity matrix");
        tc_destroy(t->solver);
        delete t;
        return rc;
    }
    // FP32 affinities on the product path, FP64 in the parity precision
    const bool f64 = c.precision == TC_PREC_FP64;
    const size_t vbytes = f64 ? 8 : 4;
    std::vector<float> vf(f64 ? 0 : t->nnz);
    for (int64_t e = 0; e < (int64_t)vf.size(); e++) vf[e] = (float)val[e];
    const void* vsrc = f64 ? (const void*)val : (const void*)vf.data();
    for (int k = 0; k < 3 && rc == TC_OK; k++) rc = ensure(t->y[k], (size_t)n * 16);
    if (!rc) rc = ensure(t->row_ptr, (size_t)(n + 1) * 4);
    if (!rc) rc = ensure(t->col, (size_t)t->nnz * 4 + 16);
    if (!rc) rc = ensure(t->val, (size_t)t->nnz * vbytes + 16);
    if (!rc) rc = ensure(t->grad_rep, (size_t)n * 16);
    if (!rc) rc = ensure(t->grad, (size_t)n * 16);
    if (!rc) rc = ensure(t->z, 64);
    if (!rc) rc = ensure(t->prm, 64);
    if (!rc && cudaMallocHost(&t->h_prm, 64) != cudaSuccess) rc = TC_ERR_NOMEM;
    cudaError_t e = cudaSuccess;
    if (!rc) e = cudaMemcpyAsync(t->row_ptr.p, row_ptr, (n + 1) * 4, cudaMemcpyHostToDevice, h.stream);
    if (!rc && e == cudaSuccess && t->nnz) e = cudaMemcpyAsync(t->col.p, col, t->nnz * 4, cudaMemcpyHostToDevice, h.stream);
    if (!rc && e == cudaSuccess && t->nnz)
        e = cudaMemcpyAsync(t->val.p, vsrc, t->nnz * vbytes, cudaMemcpyHostToDevice, h.stream);
    if (!rc && e == cudaSuccess) e = cudaMemcpyAsync(t->y[0].p, y0, n * 16, cudaMemcpyHostToDevice, h.stream);
    if (!rc && e == cudaSuccess) e = cudaMemcpyAsync(t->y[1].p, y0, n * 16, cudaMemcpyHostToDevice, h.stream);
    if (!rc && e == cudaSuccess) e = cudaStreamSynchronize(h.stream);
    if (!rc && e != cudaSuccess) rc = tc_cuda_fail(e, "tc_tsne_create upload");
    if (rc) {
        for (Buf& b : t->y) release(b);
        release(t->row_ptr), release(t->col), release(t->val), release(t->grad_rep), release(t->grad), release(t->z);
        release(t->prm);
        if (t->h_prm) cudaFreeHost(t->h_prm);
        tc_destroy(t->solver);
        delete t;
        return rc;
    }
    *out = t;
    return TC_OK;
}

int tc_tsne_destroy(tc_tsne* t)
{
    if (!t) return TC_OK;
    cudaSetDevice(t->hs->cfg.device);
    cudaStreamSynchronize(t->hs->stream);
    for (Buf& b : t->y) release(b);
    release(t->row_ptr), release(t->col), release(t->val), release(t->grad_rep), release(t->grad), release(t->z);
    release(t->prm);
    if (t->h_prm) cudaFreeHost(t->h_prm);
    tc_destroy(t->solver);
    delete t;
    return TC_OK;
}

int tc_tsne_set_theta(tc_tsne* t, double theta) { return t ? tc_set_theta(t->solver, theta) : TC_ERR_INVALID; }

int tc_tsne_set_repulsion(tc_tsne* t, int method, double cell_size)
{
    if (!t || (method != TC_REPULSION_TREE && method != TC_REPULSION_PM) ||
        (method == TC_REPULSION_PM && !(cell_size > 0.0))) {
        tc_set_error("tc_tsne_set_repulsion: invalid arguments");
        return TC_ERR_INVALID;
    }
    t->pm_cell = method == TC_REPULSION_PM ? cell_size : 0.0;
    return TC_OK;
}

int tc_tsne_set_depth(tc_tsne* t, int depth)
{
    if (!t || depth < 0 || depth > 15) return TC_ERR_INVALID;
    t->hs->cfg.depth = depth;
    t->hs->tree_ready = false;  // the next step builds the tree (and exact lists) at this depth
    return TC_OK;
}

// One iteration of TSNE_buffers::timeStep (src/nBodyInstances/tsne_buffers.h:125-168):
// tree on the current embedding, repulsion + Z, attractive term, momentum step.
// exag_code is the code's factor (16 early / 4 late in the reference).
int tc_tsne_step(tc_tsne* t, double exag_code, double momentum, double lr, double* z_out)
{
    if (!t) return TC_ERR_INVALID;
    Handle& h = *t->hs;
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));  // the pinned staging buffer is reused
    t->h_prm[0] = exag_code;
    t->h_prm[1] = lr;
    t->h_prm[2] = momentum;
    TC_CUDA_TRY(cudaMemcpyAsync(t->prm.p, t->h_prm, 24, cudaMemcpyHostToDevice, h.stream));
    int rc = tsne_enqueue(t, P<double>(t->prm), P<double>(t->prm) + 1, nullptr);
    if (rc) return rc;
    tsne_rotate(t);
    if (z_out) {
        TC_CUDA_TRY(cudaMemcpyAsync(h.h_total, t->z.p, 8, cudaMemcpyDeviceToHost, h.stream));
        TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
        *z_out = h.h_total[0];
    }
    return TC_OK;
}

int tc_tsne_get(tc_tsne* t, double* y, double* y_prev, double* grad)
{
    if (!t) return TC_ERR_INVALID;
    Handle& h = *t->hs;
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    if (y) TC_CUDA_TRY(cudaMemcpyAsync(y, t->y[t->cur].p, t->n * 16, cudaMemcpyDeviceToHost, h.stream));
    if (y_prev) TC_CUDA_TRY(cudaMemcpyAsync(y_prev, t->y[t->prev].p, t->n * 16, cudaMemcpyDeviceToHost, h.stream));
    if (grad) TC_CUDA_TRY(cudaMemcpyAsync(grad, t->grad.p, t->n * 16, cudaMemcpyDeviceToHost, h.stream));
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    return TC_OK;
}

int tc_tsne_last_launch_count(tc_tsne* t) { return t ? t->launches : 0; }

}  // extern "C"

// ---------------------------------------------------------------- batches
// Many independent embeddings advance in lockstep, one CUDA graph launch per
// step.  Each system's whole step (tree, lists, FMM, attractive term, update)
// is captured as its own graph with no host round trip inside: the tree is
// built over a fixed square box, the lists use the capacities of the last
// exact build, and the step parameters are read from device memory.  The
// batch graph holds the systems' graphs as independent child nodes.  After
// each launch the host checks every system's flags (a point outside its box,
// a list over capacity); such a system's step is recomputed uncaptured
// (exact lists, a new box when it left the old one; same inputs, since the
// step writes a separate output buffer), and only that system's graphs are
// captured again and swapped into the batch graphs.  The box is the
// embedding's extent enlarged by `margin` plus the distance the fastest
// point would travel in kLookahead steps at its last displacement, so that
// a growing embedding keeps its box for many steps.  The embedding buffers
// rotate over three phases: three graphs per system and three batch graphs.
constexpr double kLookahead = 16.0;

struct tc_tsne_batch {
    std::vector<tc_tsne*> sys;
    std::vector<std::array<double, 4>> box;
    std::vector<std::array<cudaGraph_t, 3>> g;
    std::array<std::vector<cudaGraphNode_t>, 3> node;
    double margin = 0.5;
    int device = 0;
    cudaStream_t s0 = nullptr;
    cudaGraphExec_t exec[3] = {nullptr, nullptr, nullptr};
    // the graphs exec[k] was instantiated from: node[k] belongs to root[k], and an in-place update of one
    // system's child node needs that graph alive
    cudaGraph_t root[3] = {nullptr, nullptr, nullptr};
    Buf prm, ext;
    double* h_prm = nullptr;
    uint64_t* h_ext = nullptr;
    bool warm = false;
    bool capture = true;
    double lr_per_point = -1.0;
    int64_t launches = 0, captures = 0, redos = 0;
    int64_t us_graph = 0, us_restep = 0;  // host time in graph launches and in re-steps (+ re-captures)
};

namespace tc {
namespace {

// the largest per-axis displacement |y - y_prev| (non-negative doubles order
// like their bit patterns)
__global__ void k_step_extent(const double2* __restrict__ y, const double2* __restrict__ yp, int64_t n,
                              unsigned long long* __restrict__ out)
{
    double mx = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 a = y[i], b = yp[i];
        mx = fmax(mx, fmax(fabs(a.x - b.x), fabs(a.y - b.y)));
    }
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, 16));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, 8));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, 4));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
    if ((threadIdx.x & 31) == 0 && mx == mx) atomicMax(out, (unsigned long long)__double_as_longlong(mx));
}

void set_phase(tc_tsne* t, int k)
{
    t->cur = k;
    t->prev = (k + 1) % 3;
    t->next = (k + 2) % 3;
}

int batch_box(tc_tsne_batch* b, size_t i)
{
    tc_tsne* t = b->sys[i];
    Handle& h = *t->hs;
    double mn[2], mx[2];
    int rc = device_bbox(h, P<double>(t->y[t->cur]), t->n, mn, mx);
    if (rc) return rc;
    TC_CUDA_TRY(cudaMemsetAsync(b->ext.p, 0, 8, h.stream));
    k_step_extent<<<grid_for(t->n, 256, sm_count() * 4), 256, 0, h.stream>>>(
        P<double2>(t->y[t->cur]), P<double2>(t->y[t->prev]), t->n, P<unsigned long long>(b->ext));
    TC_CUDA_TRY(cudaMemcpyAsync(b->h_ext, b->ext.p, 8, cudaMemcpyDeviceToHost, h.stream));
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    double step;
    std::memcpy(&step, b->h_ext, 8);
    const double cx = 0.5 * (mn[0] + mx[0]), cy = 0.5 * (mn[1] + mx[1]);
    double e = 0.5 * (mx[0] - mn[0] > mx[1] - mn[1] ? mx[0] - mn[0] : mx[1] - mn[1]);
    e = e * (1.0 + b->margin) + kLookahead * step + 1e-12 * (1.0 + std::fabs(cx) + std::fabs(cy));
    b->box[i] = {cx - e, cy - e, cx + e, cy + e};
    return TC_OK;
}

// An uncaptured step of system i over its box (refreshed first when asked,
// and whenever a point lies outside it), exact lists on overflow; synchronised.
int batch_plain_step(tc_tsne_batch* b, size_t i, bool refresh)
{
    tc_tsne* t = b->sys[i];
    int rc;
    if (refresh && (rc = batch_box(b, i))) return rc;
    // the step parameters live on the batch stream
    TC_CUDA_TRY(cudaStreamSynchronize(b->s0));
    t->hs->nosync = false;
    rc = tsne_enqueue(t, P<double>(b->prm), P<double>(t->prm) + 1, b->box[i].data());
    if (rc == TC_ERR_INVALID && !refresh) {  // left the box: a new box, the same step again
        if ((rc = batch_box(b, i))) return rc;
        rc = tsne_enqueue(t, P<double>(b->prm), P<double>(t->prm) + 1, b->box[i].data());
    }
    if (rc) return rc;
    TC_CUDA_TRY(cudaStreamSynchronize(t->hs->stream));
    return TC_OK;
}

// the three phase graphs of system i (no allocation may happen inside a capture)
int capture_system(tc_tsne_batch* b, size_t i)
{
    tc_tsne* t = b->sys[i];
    Handle& h = *t->hs;
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    int rc = prepare_nosync(h);
    if (rc) return rc;
    const int c0 = t->cur, p0 = t->prev, n0 = t->next;
    for (int k = 0; k < 3 && rc == TC_OK; k++) {
        set_phase(t, k);
        cudaError_t eb = cudaStreamBeginCapture(h.stream, cudaStreamCaptureModeThreadLocal);
        if (eb != cudaSuccess) {
            rc = tc_cuda_fail(eb, "cudaStreamBeginCapture");
            break;
        }
        h.nosync = true;
        rc = tsne_enqueue(t, P<double>(b->prm), P<double>(t->prm) + 1, b->box[i].data());
        h.nosync = false;
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(h.stream, &g);
        if (rc || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            if (!rc) rc = tc_cuda_fail(e, "cudaStreamEndCapture");
            break;
        }
        if (b->g[i][k]) cudaGraphDestroy(b->g[i][k]);
        b->g[i][k] = g;
        b->captures++;
    }
    t->cur = c0, t->prev = p0, t->next = n0;
    return rc;
}

int build_exec(tc_tsne_batch* b, int k)
{
    if (b->exec[k]) {
        cudaGraphExecDestroy(b->exec[k]);
        b->exec[k] = nullptr;
    }
    if (b->root[k]) {
        cudaGraphDestroy(b->root[k]);
        b->root[k] = nullptr;
    }
    cudaGraph_t root = nullptr;
    TC_CUDA_TRY(cudaGraphCreate(&root, 0));
    b->node[k].assign(b->sys.size(), nullptr);
    cudaError_t e = cudaSuccess;
    for (size_t i = 0; i < b->sys.size() && e == cudaSuccess; i++)
        e = cudaGraphAddChildGraphNode(&b->node[k][i], root, nullptr, 0, b->g[i][k]);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec[k], root, cudaGraphInstantiateFlagUseNodePriority);
    if (e != cudaSuccess) {
        cudaGraphDestroy(root);
        b->exec[k] = nullptr;
        b->node[k].assign(b->sys.size(), nullptr);
        return tc_cuda_fail(e, "batch graph");
    }
    // kept: a re-captured system is swapped in through its node (cudaGraphExecChildGraphNodeSetParams)
    b->root[k] = root;
    return TC_OK;
}

void drop_all(tc_tsne_batch* b)
{
    for (int k = 0; k < 3; k++) {
        if (b->exec[k]) {
            cudaGraphExecDestroy(b->exec[k]);
            b->exec[k] = nullptr;
        }
        if (b->root[k]) {
            cudaGraphDestroy(b->root[k]);
            b->root[k] = nullptr;
        }
    }
    for (auto& gs : b->g)
        for (cudaGraph_t& g : gs)
            if (g) {
                cudaGraphDestroy(g);
                g = nullptr;
            }
}

}  // namespace
}  // namespace tc

extern "C" {

int tc_tsne_batch_create(tc_tsne* const* systems, int count, double margin, tc_tsne_batch** out)
{
    if (!systems || count <= 0 || !out || !(margin >= 0.0)) {
        tc_set_error("tc_tsne_batch_create: invalid arguments");
        return TC_ERR_INVALID;
    }
    *out = nullptr;
    const int dev = systems[0] ? systems[0]->hs->cfg.device : 0;
    for (int i = 0; i < count; i++) {
        const tc_tsne* t = systems[i];
        if (!t || t->hs->cfg.device != dev || t->hs->cfg.order == 0 || t->hs->cfg.precision != TC_PREC_FP32 ||
            t->cur != systems[0]->cur || t->pm_cell > 0.0) {
            tc_set_error("tc_tsne_batch_create: systems must be FP32 order-p tree solvers on one device, in step");
            return TC_ERR_INVALID;
        }
    }
    TC_CUDA_TRY(cudaSetDevice(dev));
    tc_tsne_batch* b = new tc_tsne_batch();
    b->sys.assign(systems, systems + count);
    b->box.resize(count);
    b->g.assign(count, {nullptr, nullptr, nullptr});
    b->margin = margin;
    b->device = dev;
    // list regions twice the last exact totals: while the embeddings grow, a region that
    // overflows costs an uncaptured re-step and a re-capture of that system
    for (tc_tsne* t : b->sys) t->hs->cap_slack = 1.0;
    // one graph holds all the systems, which already run side by side: each system's near field stays on its
    // own stream after its far field (its fork/join branches and priorities measured slower in the batch)
    for (tc_tsne* t : b->sys) t->hs->near_overlap = false;
    cudaError_t e = cudaStreamCreateWithFlags(&b->s0, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_prm, 64);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_ext, 64);
    int rc = e == cudaSuccess ? ensure(b->prm, 64) : tc_cuda_fail(e, "tc_tsne_batch_create");
    if (!rc) rc = ensure(b->ext, 64);
    if (rc) {
        tc_tsne_batch_destroy(b);
        return rc;
    }
    *out = b;
    return TC_OK;
}

int tc_tsne_batch_destroy(tc_tsne_batch* b)
{
    if (!b) return TC_OK;
    cudaSetDevice(b->device);
    if (b->s0) cudaStreamSynchronize(b->s0);
    drop_all(b);
    if (b->s0) cudaStreamDestroy(b->s0);
    release(b->prm);
    release(b->ext);
    if (b->h_prm) cudaFreeHost(b->h_prm);
    if (b->h_ext) cudaFreeHost(b->h_ext);
    delete b;
    return TC_OK;
}

int tc_tsne_batch_step(tc_tsne_batch* b, double exag_code, double momentum, double lr_per_point)
{
    if (!b) return TC_ERR_INVALID;
    TC_CUDA_TRY(cudaSetDevice(b->device));
    TC_CUDA_TRY(cudaStreamSynchronize(b->s0));  // the pinned staging buffer is reused
    b->h_prm[0] = exag_code;
    b->h_prm[1] = 0.0;
    b->h_prm[2] = momentum;
    TC_CUDA_TRY(cudaMemcpyAsync(b->prm.p, b->h_prm, 24, cudaMemcpyHostToDevice, b->s0));
    if (lr_per_point != b->lr_per_point) {
        // each system's learning rate lr_per_point * n (the reference's N/15 at 1/15)
        for (tc_tsne* t : b->sys) {
            TC_CUDA_TRY(cudaStreamSynchronize(t->hs->stream));
            t->h_prm[1] = lr_per_point * (double)t->n;
            TC_CUDA_TRY(cudaMemcpyAsync(P<double>(t->prm) + 1, t->h_prm + 1, 8, cudaMemcpyHostToDevice, b->s0));
        }
        b->lr_per_point = lr_per_point;
    }
    int rc;
    if (!b->warm || !b->capture) {
        // uncaptured steps: the first one (exact boxes and lists size every
        // buffer), or all of them when capture is off
        for (size_t i = 0; i < b->sys.size(); i++)
            if ((rc = batch_plain_step(b, i, !b->warm))) return rc;
        b->warm = true;
    } else {
        const int phase = b->sys[0]->cur;
        if (!b->exec[0]) {
            for (size_t i = 0; i < b->sys.size(); i++)
                if ((rc = capture_system(b, i))) return rc;
            for (int k = 0; k < 3; k++)
                if ((rc = build_exec(b, k))) return rc;
        }
        const auto t0 = std::chrono::steady_clock::now();
        TC_CUDA_TRY(cudaGraphLaunch(b->exec[phase], b->s0));
        TC_CUDA_TRY(cudaStreamSynchronize(b->s0));
        const auto t1 = std::chrono::steady_clock::now();
        b->us_graph += std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();
        b->launches++;
        for (size_t i = 0; i < b->sys.size(); i++) {
            const int st = tc_async_status(b->sys[i]->solver);
            if (!st) continue;
            if ((rc = batch_plain_step(b, i, (st & 1) != 0))) return rc;
            b->redos++;
            // this system's graphs again (new box or capacities), swapped into the batch graphs
            if ((rc = capture_system(b, i))) return rc;
            for (int k = 0; k < 3; k++)
                if (cudaGraphExecChildGraphNodeSetParams(b->exec[k], b->node[k][i], b->g[i][k]) != cudaSuccess) {
                    cudaGetLastError();
                    if ((rc = build_exec(b, k))) return rc;
                }
        }
        b->us_restep += std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - t1)
                            .count();
    }
    for (tc_tsne* t : b->sys) tsne_rotate(t);
    return TC_OK;
}

int tc_tsne_batch_set_capture(tc_tsne_batch* b, int enable)
{
    if (!b) return TC_ERR_INVALID;
    b->capture = enable != 0;
    if (!b->capture) drop_all(b);
    return TC_OK;
}

int tc_tsne_batch_stats(tc_tsne_batch* b, int64_t* out)
{
    if (!b || !out) return TC_ERR_INVALID;
    int64_t np = 0, kern = 0;
    for (tc_tsne* t : b->sys) {
        np += t->n;
        kern += t->launches;
    }
    size_t nodes = 0;
    for (auto& gs : b->g)
        if (gs[0]) {
            size_t c = 0;
            cudaGraphGetNodes(gs[0], nullptr, &c);
            nodes += c;
        }
    out[0] = b->launches;
    out[1] = b->captures;
    out[2] = b->redos;
    out[3] = (int64_t)nodes;
    out[4] = np;
    out[5] = kern;
    out[6] = b->us_graph;
    out[7] = b->us_restep;
    return TC_OK;
}

}  // extern "C"
