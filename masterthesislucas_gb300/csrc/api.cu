// C ABI of libtreecode.so (declared in include/treecode.h): handle lifetime,
// host <-> device staging, and the update/solve entry points that stand in
// for NBodySolver::updateTree / solveNbody (src/nbodysolvers/cpu/nBodySolver.h:17-18).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <functional>
#include <new>
#include <vector>

#include "state.cuh"

static thread_local char g_err[512] = "";

void tc_set_error(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int tc_cuda_fail(cudaError_t e, const char* what)
{
    tc_set_error("CUDA error %s (%s) in %s", cudaGetErrorName(e), cudaGetErrorString(e), what);
    return e == cudaErrorMemoryAllocation ? TC_ERR_NOMEM : TC_ERR_CUDA;
}

namespace tc {

int sm_count()
{
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (cache[dev] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
        cache[dev] = v;
    }
    return cache[dev];
}

int ensure(Buf& b, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    if (b.bytes >= bytes) return TC_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
        b.p = nullptr;
        return tc_cuda_fail(e, "cudaMalloc");
    }
    b.bytes = bytes;
    return TC_OK;
}

void release(Buf& b)
{
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
}

int record_on(Handle& h, int i, cudaStream_t s)
{
    if (h.nosync) return TC_OK;  // stage timing events stay out of captured graphs
    if (!h.ev_ready) {
        for (auto& e : h.ev) TC_CUDA_TRY(cudaEventCreate(&e));
        h.ev_ready = true;
    }
    if (i == 4) h.stage_split = false;
    TC_CUDA_TRY(cudaEventRecord(h.ev[i], s));
    return TC_OK;
}

int record(Handle& h, int i) { return record_on(h, i, h.stream); }

int ensure_near_stream(Handle& h)
{
    if (h.near_stream) return TC_OK;
    int least = 0, greatest = 0;
    TC_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    TC_CUDA_TRY(cudaStreamCreateWithPriority(&h.near_stream, cudaStreamNonBlocking, least));
    TC_CUDA_TRY(cudaStreamCreateWithPriority(&h.far_stream, cudaStreamNonBlocking, greatest));
    TC_CUDA_TRY(cudaEventCreateWithFlags(&h.ev_fork, cudaEventDisableTiming));
    TC_CUDA_TRY(cudaEventCreateWithFlags(&h.ev_join, cudaEventDisableTiming));
    TC_CUDA_TRY(cudaEventCreateWithFlags(&h.ev_far, cudaEventDisableTiming));
    TC_CUDA_TRY(cudaEventCreateWithFlags(&h.ev_mu, cudaEventDisableTiming));
    TC_CUDA_TRY(cudaEventCreateWithFlags(&h.ev_lists, cudaEventDisableTiming));
    return TC_OK;
}

namespace {

__global__ void k_bbox(const double2* __restrict__ pos, int64_t n, double* __restrict__ out, uint32_t* err)
{
    double mnx = INFINITY, mny = INFINITY, mxx = -INFINITY, mxy = -INFINITY;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 p = pos[i];
        if (!(isfinite(p.x) && isfinite(p.y))) atomicOr(err, 1u);
        mnx = fmin(mnx, p.x);
        mny = fmin(mny, p.y);
        mxx = fmax(mxx, p.x);
        mxy = fmax(mxy, p.y);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mnx = fmin(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
        mny = fmin(mny, __shfl_xor_sync(0xffffffffu, mny, o));
        mxx = fmax(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
        mxy = fmax(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
    }
    __shared__ double s[4][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        s[0][w] = mnx;
        s[1][w] = mny;
        s[2][w] = mxx;
        s[3][w] = mxy;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); k++) {
            mnx = fmin(mnx, s[0][k]);
            mny = fmin(mny, s[1][k]);
            mxx = fmax(mxx, s[2][k]);
            mxy = fmax(mxy, s[3][k]);
        }
        // min/max are exact and order-independent: atomics on the ordered
        // integer image of the doubles are deterministic
        auto key = [](double v) {
            unsigned long long u = (unsigned long long)__double_as_longlong(v);
            return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
        };
        unsigned long long* o = reinterpret_cast<unsigned long long*>(out);
        atomicMin(o + 0, key(mnx));
        atomicMin(o + 1, key(mny));
        atomicMax(o + 2, key(mxx));
        atomicMax(o + 3, key(mxy));
    }
}

__global__ void k_bbox_init(double* out)
{
    unsigned long long* o = reinterpret_cast<unsigned long long*>(out);
    o[0] = o[1] = 0xFFFFFFFFFFFFFFFFull;
    o[2] = o[3] = 0ull;
}

inline double unkey(unsigned long long k)
{
    unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    double d;
    std::memcpy(&d, &u, 8);
    return d;
}

// the caller's point IDs follow the points through the sort: out[k] = in[perm[k]]
__global__ void k_gather_ids(const int32_t* __restrict__ in, const uint32_t* __restrict__ perm, int64_t n,
                             int32_t* __restrict__ out)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        out[k] = in[perm[k]];
}

// refreshes the compute copy of the positions after tc_solve received new ones
template <typename real>
__global__ void k_prel(const double2* __restrict__ pos64, const uint32_t* __restrict__ codes, int64_t n, int depth,
                       double minx, double miny, double h, real* __restrict__ prel)
{
    const int shift = 32 - 2 * depth;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t leaf = depth ? (codes[k] >> shift) : 0u;
        double cx = minx + ((double)compact16(leaf) + 0.5) * h;
        double cy = miny + ((double)compact16(leaf >> 1) + 0.5) * h;
        double2 p = pos64[k];
        prel[2 * k] = (real)(p.x - cx);
        prel[2 * k + 1] = (real)(p.y - cy);
    }
}

}  // namespace

int bbox_keys(const double* d_pos, int64_t n, double* d_keys4, uint32_t* d_err, cudaStream_t s)
{
    k_bbox_init<<<1, 1, 0, s>>>(d_keys4);
    k_bbox<<<grid_for(n, 256, sm_count() * 4), 256, 0, s>>>((const double2*)d_pos, n, d_keys4, d_err);
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

int device_bbox(Handle& h, const double* d_pos, int64_t n, double mn[2], double mx[2])
{
    int rc;
    if ((rc = ensure(h.err, 64)) || (rc = ensure(h.dtotal, 64))) return rc;
    double* o = P<double>(h.dtotal) + 2;
    TC_CUDA_TRY(cudaMemsetAsync(h.err.p, 0, 4, h.stream));
    k_bbox_init<<<1, 1, 0, h.stream>>>(o);
    k_bbox<<<grid_for(n, 256, sm_count() * 4), 256, 0, h.stream>>>((const double2*)d_pos, n, o, P<uint32_t>(h.err));
    h.launches += 2;
    TC_CUDA_TRY(cudaMemcpyAsync(h.h_words, o, 32, cudaMemcpyDeviceToHost, h.stream));
    TC_CUDA_TRY(cudaMemcpyAsync(h.h_words + 8, h.err.p, 4, cudaMemcpyDeviceToHost, h.stream));
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    if (h.h_words[8]) {
        tc_set_error("positions contain NaN or infinity");
        return TC_ERR_INVALID;
    }
    unsigned long long k[4];
    std::memcpy(k, h.h_words, 32);
    mn[0] = unkey(k[0]);
    mn[1] = unkey(k[1]);
    mx[0] = unkey(k[2]);
    mx[1] = unkey(k[3]);
    return TC_OK;
}

int refresh_positions(Handle& h)
{
    const double hl = h.L / (double)(1u << h.depth);
    if (h.cfg.precision == TC_PREC_FP64)
        k_prel<double><<<grid_for(h.n, 256), 256, 0, h.stream>>>(P<double2>(h.pos64), P<uint32_t>(h.codes), h.n,
                                                                h.depth, h.minx, h.miny, hl, P<double>(h.prel));
    else
        k_prel<float><<<grid_for(h.n, 256), 256, 0, h.stream>>>(P<double2>(h.pos64), P<uint32_t>(h.codes), h.n,
                                                               h.depth, h.minx, h.miny, hl, P<float>(h.prel));
    h.launches++;
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

int dump_final_locals(Handle& h, std::vector<double>& out);

}  // namespace tc

using namespace tc;


extern "C" {

const char* tc_last_error(void) { return g_err; }

int tc_config_init(tc_config* cfg)
{
    if (!cfg) return TC_ERR_INVALID;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->kernel = TC_KERNEL_TSNE;
    cfg->max_children = 16;
    cfg->depth = -1;
    cfg->theta = 0.5;
    cfg->softening = 1e-3;
    cfg->precision = TC_PREC_FP32;
    cfg->device = 0;
    cfg->stream = nullptr;
    cfg->order = 0;
    return TC_OK;
}

int tc_get_depth(int max_children, int64_t n, uint32_t* depth)
{
    if (!depth || max_children <= 0 || n < 0) {
        tc_set_error("tc_get_depth: invalid arguments");
        return TC_ERR_INVALID;
    }
    // N / max_children is an integer division in the reference
    const double circle_area = 3.141592653589793238462643383279502884 / 4.0;
    int64_t q = (int64_t)(int)n / max_children;
    if (q < 1) {
        *depth = 0;
        return TC_OK;
    }
    double d = std::log((1.0 / circle_area) * (double)q) / std::log(4.0);
    double c = std::ceil(d);
    *depth = c < 0 ? 0u : (uint32_t)c;
    return TC_OK;
}

int tc_node_count(uint32_t depth, int64_t* count)
{
    if (!count || depth > 20) return TC_ERR_INVALID;
    int64_t t = 0, s = 1;
    for (uint32_t l = 0; l <= depth; l++) {
        t += s;
        s *= 4;
    }
    *count = t;
    return TC_OK;
}

int tc_create(const tc_config* cfg, tc_handle** out)
{
    if (!cfg || !out) {
        tc_set_error("tc_create: null argument");
        return TC_ERR_INVALID;
    }
    *out = nullptr;
    if (!(cfg->theta > 0.0) || cfg->max_children <= 0 || (cfg->kernel != TC_KERNEL_TSNE && cfg->kernel != TC_KERNEL_GRAVITY) ||
        (cfg->precision != TC_PREC_FP32 && cfg->precision != TC_PREC_FP64) || cfg->depth > 15 ||
        cfg->order < 0 || cfg->order > 16 || (cfg->order > 0 && cfg->precision != TC_PREC_FP32) ||
        !(cfg->softening >= 0.0) || (cfg->kernel == TC_KERNEL_GRAVITY && !(cfg->softening > 0.0))) {
        tc_set_error("tc_create: invalid configuration");
        return TC_ERR_INVALID;
    }
    TC_CUDA_TRY(cudaSetDevice(cfg->device));
    tc_handle* t = new (std::nothrow) tc_handle();
    if (!t) return TC_ERR_NOMEM;
    t->h.cfg = *cfg;
    if (cfg->stream) {
        t->h.stream = (cudaStream_t)cfg->stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&t->h.stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete t;
            return tc_cuda_fail(e, "cudaStreamCreate");
        }
        t->h.own_stream = true;
    }
    cudaError_t e = cudaMallocHost(&t->h.h_total, 64);
    if (e == cudaSuccess) e = cudaMallocHost(&t->h.h_words, 64 * 4);
    if (e != cudaSuccess) {
        tc_destroy(t);
        return tc_cuda_fail(e, "cudaMallocHost");
    }
    // status words the asynchronous paths report through (tc_async_status): none raised yet
    std::memset(t->h.h_words, 0, 64 * 4);
    std::memset(t->h.h_total, 0, 64);
    *out = t;
    return TC_OK;
}

int tc_destroy(tc_handle* t)
{
    if (!t) return TC_OK;
    Handle& h = t->h;
    cudaSetDevice(h.cfg.device);
    if (h.stream) cudaStreamSynchronize(h.stream);
    if (h.near_stream) cudaStreamSynchronize(h.near_stream);
    if (h.far_stream) cudaStreamSynchronize(h.far_stream);
    if (h.copy_stream) cudaStreamSynchronize(h.copy_stream);
    Buf* bufs[] = {&h.codes, &h.perm, &h.alt_keys, &h.alt_vals, &h.pos_in, &h.pos64, &h.prel, &h.grad_acc,
                   &h.count, &h.first, &h.com64, &h.m0, &h.m2, &h.bbc, &h.bblen, &h.comrel, &h.m0r, &h.m2t,
                   &h.loc, &h.locfin, &h.mu, &h.chunk, &h.zwork, &h.zloc, &h.counters, &h.ptr_pool, &h.idx_pool, &h.cnt_tmp, &h.lstat, &h.ord_pool, &h.nfeat, &h.dec, &h.bigleaf, &h.chunk_leaf, &h.act, &h.act_pos, &h.bmax, &h.celloff, &h.mqueue, &h.nearf, &h.items_cnt, &h.items_tmp, &h.tc_ops, &h.tc_mubf, &h.diagpart, &h.ctrl_w, &h.tmp, &h.err, &h.zpart, &h.dtotal, &h.sumtmp,
                   &h.host_stage, &h.ids_dev};
    for (Buf* b : bufs) release(*b);
    if (h.step_graph) cudaGraphExecDestroy(h.step_graph);
    if (h.h_total) cudaFreeHost(h.h_total);
    if (h.h_words) cudaFreeHost(h.h_words);
    if (h.copy_stream) {
        cudaStreamSynchronize(h.copy_stream);
        cudaStreamDestroy(h.copy_stream);
    }
    if (h.near_stream) cudaStreamDestroy(h.near_stream);
    if (h.far_stream) cudaStreamDestroy(h.far_stream);
    if (h.ev_far) cudaEventDestroy(h.ev_far);
    if (h.ev_mu) cudaEventDestroy(h.ev_mu);
    if (h.ev_lists) cudaEventDestroy(h.ev_lists);
    if (h.ev_ready)
        for (auto& e : h.ev) cudaEventDestroy(e);
    if (h.ev_fork) cudaEventDestroy(h.ev_fork);
    if (h.ev_join) cudaEventDestroy(h.ev_join);
    if (h.ev_tree) cudaEventDestroy(h.ev_tree);
    if (h.ev_grad) cudaEventDestroy(h.ev_grad);
    if (h.own_stream && h.stream) cudaStreamDestroy(h.stream);
    delete t;
    return TC_OK;
}

int tc_set_theta(tc_handle* t, double theta)
{
    if (!t || !(theta > 0.0)) return TC_ERR_INVALID;
    t->h.cfg.theta = theta;
    // the lists depend on theta: a new update_tree is needed before solving
    t->h.tree_ready = false;
    return TC_OK;
}

static int ensure_copy_stream(Handle& h)
{
    if (h.copy_stream) return TC_OK;
    TC_CUDA_TRY(cudaStreamCreateWithFlags(&h.copy_stream, cudaStreamNonBlocking));
    TC_CUDA_TRY(cudaEventCreateWithFlags(&h.ev_tree, cudaEventDisableTiming));
    TC_CUDA_TRY(cudaEventCreateWithFlags(&h.ev_grad, cudaEventDisableTiming));
    return TC_OK;
}

// after_tree (may be null) is called once the sorted records are enqueued, before the interaction lists
// are built (the list build waits on the host for the list sizes)
static int update_common(Handle& h, const double* d_pos, int64_t n, const double* mn, const double* mx,
                         const std::function<int()>& after_tree)
{
    if (n <= 0 || n > (int64_t)0x7FFFFFFF) {
        tc_set_error("n must be in [1, 2^31)");
        return TC_ERR_INVALID;
    }
    if (!std::isfinite(mn[0]) || !std::isfinite(mn[1]) || !std::isfinite(mx[0]) || !std::isfinite(mx[1])) {
        tc_set_error("bounding box is not finite");
        return TC_ERR_INVALID;
    }
    // order-p multipoles without the learned controller (whose list build reads them): built on a side
    // stream beside the interaction lists, which need only the tree, and joined before the update returns
    // (streams are never created inside a capture: a captured update follows an ordinary one).  The near
    // field's work-item tables follow them there; in a captured step (whose list build has no host round
    // trip that could redo the lists) so do the far field's coarse levels, once their lists are built.
    const bool split = h.cfg.order && !h.ctrl_on && h.near_overlap && (h.near_stream || !h.nosync);
    const bool coarse = split && h.nosync && far_coarse_applies(h);
    h.items_ready = false;
    h.coarse_ready = false;
    h.split_mu = split;
    int rc = split ? ensure_near_stream(h) : TC_OK;
    if (!rc) rc = build_tree(h, d_pos, n, mn[0], mn[1], mx[0], mx[1]);
    h.split_mu = false;
    bool forked = false;
    const cudaStream_t main = h.stream;
    if (!rc && split) {
        TC_CUDA_TRY(cudaEventRecord(h.ev_fork, h.stream));
        TC_CUDA_TRY(cudaStreamWaitEvent(h.near_stream, h.ev_fork, 0));
        forked = true;
        h.stream = h.near_stream;
        rc = build_multipoles(h);
        if (!rc) rc = near_items(h);
        h.stream = main;
        h.items_ready = rc == TC_OK;
    }
    if (!rc && (rc = after_tree()) == TC_OK) {
        // beside the side stream's work the list build (the update's critical path) runs on the
        // high-priority stream, forked from and joined back to the handle's stream
#ifndef TC_LISTS_PRIORITY
#define TC_LISTS_PRIORITY 1
#endif
        const bool hp = TC_LISTS_PRIORITY && forked && h.far_stream;
        if (hp) {
            TC_CUDA_TRY(cudaEventRecord(h.ev_fork, main));
            TC_CUDA_TRY(cudaStreamWaitEvent(h.far_stream, h.ev_fork, 0));
            h.stream = h.far_stream;
        }
        h.lists_event_level = coarse ? kFarCoarseLevel : -1;
        rc = build_lists(h);  // synchronises the stream (list sizes), except in no-sync mode
        h.lists_event_level = -1;
        h.stream = main;
        if (hp) {
            cudaError_t e = cudaEventRecord(h.ev_far, h.far_stream);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(main, h.ev_far, 0);
            if (!rc && e != cudaSuccess) rc = tc_cuda_fail(e, "list-build join");
        }
    }
    if (!rc && coarse) {
        TC_CUDA_TRY(cudaStreamWaitEvent(h.near_stream, h.ev_lists, 0));
        h.stream = h.near_stream;
        const int rcc = build_far_coarse(h);  // 1: skipped, the solve runs the coarse levels itself
        h.stream = main;
        h.coarse_ready = rcc == TC_OK;
        if (rcc < 0) rc = rcc;
    }
    if (forked) {
        cudaError_t e = cudaEventRecord(h.ev_mu, h.near_stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(h.stream, h.ev_mu, 0);
        if (!rc && e != cudaSuccess) rc = tc_cuda_fail(e, "side-stream join");
    }
    if (rc) return rc;
    TC_CUDA_TRY(cudaMemcpyAsync(h.h_words + 8, h.err.p, 4, cudaMemcpyDeviceToHost, h.stream));
    if (h.nosync) return TC_OK;  // the caller reads the flags after its own synchronisation
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    if (h.h_words[8]) {
        h.tree_ready = false;
        tc_set_error("a position is NaN or lies outside the bounding box");
        return TC_ERR_INVALID;
    }
    return TC_OK;
}

int tc_update_tree(tc_handle* t, double* pos_xy, int32_t* ids, int64_t n, const double min_xy[2],
                   const double max_xy[2])
{
    if (!t || !pos_xy || !min_xy || !max_xy) {
        tc_set_error("tc_update_tree: null argument");
        return TC_ERR_INVALID;
    }
    Handle& h = t->h;
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    h.launches = 0;
    int rc;
    if ((rc = ensure(h.pos_in, (size_t)n * 16)) || (rc = ensure_copy_stream(h))) return rc;
    if (ids && (rc = ensure(h.ids_dev, (size_t)n * 8))) return rc;
    cudaStream_t c = h.copy_stream;
    int32_t* ids_in = ids ? P<int32_t>(h.ids_dev) : nullptr;
    TC_CUDA_TRY(cudaMemcpyAsync(h.pos_in.p, pos_xy, (size_t)n * 16, cudaMemcpyHostToDevice, h.stream));
    if (ids) TC_CUDA_TRY(cudaMemcpyAsync(ids_in, ids, (size_t)n * 4, cudaMemcpyHostToDevice, c));
    // the sorted positions and IDs travel back to the caller on the copy stream while the interaction
    // lists are built: the reference's updateTree returns its points reordered
    auto back = [&]() -> int {
        TC_CUDA_TRY(cudaEventRecord(h.ev_tree, h.stream));
        TC_CUDA_TRY(cudaStreamWaitEvent(c, h.ev_tree, 0));
        TC_CUDA_TRY(cudaMemcpyAsync(pos_xy, h.pos64.p, (size_t)n * 16, cudaMemcpyDeviceToHost, c));
        if (ids) {
            // the records' IDs move with them on the device: no host gather
            int32_t* ids_out = ids_in + n;
            k_gather_ids<<<grid_for(n, 256), 256, 0, c>>>(ids_in, P<uint32_t>(h.perm), n, ids_out);
            TC_CUDA_TRY(cudaGetLastError());
            h.launches++;
            TC_CUDA_TRY(cudaMemcpyAsync(ids, ids_out, (size_t)n * 4, cudaMemcpyDeviceToHost, c));
        }
        return TC_OK;
    };
    rc = update_common(h, P<double>(h.pos_in), n, min_xy, max_xy, back);
    // the copy stream's work is finished before returning, on every path
    const cudaError_t ec = cudaStreamSynchronize(c);
    if (rc) return rc;
    if (ec != cudaSuccess) return tc_cuda_fail(ec, "tc_update_tree");
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    return TC_OK;
}

int tc_update_tree_device(tc_handle* t, const double* d_pos_xy, int64_t n, const double* min_xy,
                          const double* max_xy)
{
    if (!t || !d_pos_xy || (!min_xy) != (!max_xy)) {
        tc_set_error("tc_update_tree_device: invalid arguments");
        return TC_ERR_INVALID;
    }
    Handle& h = t->h;
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    h.launches = 0;
    double mn[2], mx[2];
    if (min_xy) {
        mn[0] = min_xy[0];
        mn[1] = min_xy[1];
        mx[0] = max_xy[0];
        mx[1] = max_xy[1];
    } else {
        int rc = device_bbox(h, d_pos_xy, n, mn, mx);
        if (rc) return rc;
    }
    return update_common(h, d_pos_xy, n, mn, mx, []() { return TC_OK; });
}

int tc_solve_device(tc_handle* t, double* d_grad_xy, double* d_total, int accumulate, int scatter)
{
    if (!t || !d_grad_xy || !d_total) return TC_ERR_INVALID;
    Handle& h = t->h;
    if (!h.tree_ready) {
        tc_set_error("tc_solve: no tree (call tc_update_tree first)");
        return TC_ERR_STATE;
    }
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    h.launches = 0;
    return h.cfg.order ? solve_fmm_order(h, d_grad_xy, d_total, accumulate, scatter)
                       : solve_fmm(h, d_grad_xy, d_total, accumulate, scatter);
}

int tc_solve(tc_handle* t, double* total, const double* pos_xy, double* grad_xy, int64_t n)
{
    if (!t || !total || !grad_xy) {
        tc_set_error("tc_solve: null argument");
        return TC_ERR_INVALID;
    }
    Handle& h = t->h;
    if (!h.tree_ready) {
        tc_set_error("tc_solve: no tree (call tc_update_tree first)");
        return TC_ERR_STATE;
    }
    if (n != h.n) {
        tc_set_error("tc_solve: n (%lld) differs from the tree's (%lld)", (long long)n, (long long)h.n);
        return TC_ERR_INVALID;
    }
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    h.launches = 0;
    int rc;
    if ((rc = ensure(h.grad_acc, (size_t)n * 16)) || (rc = ensure(h.dtotal, 64)) || (rc = ensure_copy_stream(h)))
        return rc;
    // the forces add to the caller's (applyForces accumulates into derivative): the sum is taken on the
    // device, result + grad_xy[i] in one FP64 add per component, and copied straight back.  The caller's
    // gradient comes in on the copy stream; the order-p solve waits for it only before its near-field
    // kernel (the first to touch it), so the copy overlaps the far field
    TC_CUDA_TRY(cudaMemcpyAsync(h.grad_acc.p, grad_xy, (size_t)n * 16, cudaMemcpyHostToDevice, h.copy_stream));
    TC_CUDA_TRY(cudaEventRecord(h.ev_grad, h.copy_stream));
    if (pos_xy) {
        TC_CUDA_TRY(cudaMemcpyAsync(h.pos64.p, pos_xy, (size_t)n * 16, cudaMemcpyHostToDevice, h.stream));
        if ((rc = refresh_positions(h))) return rc;
    }
    TC_CUDA_TRY(cudaMemsetAsync(h.dtotal.p, 0, 8, h.stream));
    if (h.cfg.order) {
        h.wait_grad = true;
        rc = solve_fmm_order(h, P<double>(h.grad_acc), P<double>(h.dtotal), 1, 0);
        if (h.wait_grad) {  // a path that never reached the near field still orders the copy before returning
            h.wait_grad = false;
            if (!rc) TC_CUDA_TRY(cudaStreamWaitEvent(h.stream, h.ev_grad, 0));
        }
    } else {
        TC_CUDA_TRY(cudaStreamWaitEvent(h.stream, h.ev_grad, 0));
        rc = solve_fmm(h, P<double>(h.grad_acc), P<double>(h.dtotal), 1, 0);
    }
    if (rc) {
        cudaStreamSynchronize(h.copy_stream);
        return rc;
    }
    TC_CUDA_TRY(cudaMemcpyAsync(grad_xy, h.grad_acc.p, (size_t)n * 16, cudaMemcpyDeviceToHost, h.stream));
    TC_CUDA_TRY(cudaMemcpyAsync(h.h_total, h.dtotal.p, 8, cudaMemcpyDeviceToHost, h.stream));
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    *total += h.h_total[0];
    return TC_OK;
}

int tc_get_tree(tc_handle* t, uint32_t* codes, int32_t* perm, double* pos_sorted, double* nodes)
{
    if (!t) return TC_ERR_INVALID;
    Handle& h = t->h;
    if (h.depth < 0 || h.n == 0) return TC_ERR_STATE;
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    cudaStream_t s = h.stream;
    const int64_t n = h.n, nn = h.nnodes;
    if (codes) TC_CUDA_TRY(cudaMemcpyAsync(codes, h.codes.p, n * 4, cudaMemcpyDeviceToHost, s));
    if (perm) TC_CUDA_TRY(cudaMemcpyAsync(perm, h.perm.p, n * 4, cudaMemcpyDeviceToHost, s));
    if (pos_sorted) TC_CUDA_TRY(cudaMemcpyAsync(pos_sorted, h.pos64.p, n * 16, cudaMemcpyDeviceToHost, s));
    if (nodes) {
        std::vector<uint32_t> cnt(nn), fst(nn);
        std::vector<double> com(2 * nn), m0(nn), m2(3 * nn), bbc(2 * nn), len(nn);
        TC_CUDA_TRY(cudaMemcpyAsync(cnt.data(), h.count.p, nn * 4, cudaMemcpyDeviceToHost, s));
        TC_CUDA_TRY(cudaMemcpyAsync(fst.data(), h.first.p, nn * 4, cudaMemcpyDeviceToHost, s));
        TC_CUDA_TRY(cudaMemcpyAsync(com.data(), h.com64.p, nn * 16, cudaMemcpyDeviceToHost, s));
        TC_CUDA_TRY(cudaMemcpyAsync(m0.data(), h.m0.p, nn * 8, cudaMemcpyDeviceToHost, s));
        TC_CUDA_TRY(cudaMemcpyAsync(m2.data(), h.m2.p, nn * 24, cudaMemcpyDeviceToHost, s));
        TC_CUDA_TRY(cudaMemcpyAsync(bbc.data(), h.bbc.p, nn * 16, cudaMemcpyDeviceToHost, s));
        TC_CUDA_TRY(cudaMemcpyAsync(len.data(), h.bblen.p, nn * 8, cudaMemcpyDeviceToHost, s));
        std::vector<double> fin;
        int rc = dump_final_locals(h, fin);
        if (rc) return rc;
        TC_CUDA_TRY(cudaStreamSynchronize(s));
        for (int64_t k = 0; k < nn; k++) {
            double* o = nodes + k * 27;
            if (cnt[k] == 0) {
                // an empty node is the reference's default-constructed record; the order-p path leaves
                // the device records of empty nodes unwritten
                for (int j = 0; j < 27; j++) o[j] = 0.0;
                continue;
            }
            int l = 0;
            while (l < h.depth && (int64_t)level_index(l + 1) <= k) l++;
            const int64_t i = k - level_index(l);
            o[0] = bbc[2 * k];
            o[1] = bbc[2 * k + 1];
            o[2] = len[k];
            o[3] = (cnt[k] != 0 && l < h.depth) ? (double)(level_index(l + 1) + 4 * i) : 0.0;
            o[4] = fst[k];
            o[5] = cnt[k];
            o[6] = com[2 * k];
            o[7] = com[2 * k + 1];
            o[8] = m0[k];
            o[9] = m2[3 * k];
            o[10] = m2[3 * k + 1];
            o[11] = m2[3 * k + 1];
            o[12] = m2[3 * k + 2];
            const double* c = fin.empty() ? nullptr : fin.data() + 9 * k;
            double C[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            if (c && cnt[k] != 0)
                for (int j = 0; j < 9; j++) C[j] = c[j];
            o[13] = C[L_C1X];
            o[14] = C[L_C1Y];
            o[15] = C[L_C2XX];
            o[16] = C[L_C2XY];
            o[17] = C[L_C2XY];
            o[18] = C[L_C2YY];
            // C3 in i*4 + j*2 + k order: xxx xxy xyx xyy yxx yxy yyx yyy
            o[19] = C[L_C3XXX];
            o[20] = C[L_C3XXY];
            o[21] = C[L_C3XXY];
            o[22] = C[L_C3XYY];
            o[23] = C[L_C3XXY];
            o[24] = C[L_C3XYY];
            o[25] = C[L_C3XYY];
            o[26] = C[L_C3YYY];
        }
    } else {
        TC_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return TC_OK;
}

int tc_get_list_stats(tc_handle* t, uint32_t* nn_pairs, uint32_t* near_pairs)
{
    if (!t || t->h.depth < 0) return TC_ERR_STATE;
    for (int l = 0; l <= t->h.depth; l++) {
        if (nn_pairs) nn_pairs[l] = t->h.lists.nn_total.size() > (size_t)l ? t->h.lists.nn_total[l] : 0;
        if (near_pairs) near_pairs[l] = t->h.lists.near_total.size() > (size_t)l ? t->h.lists.near_total[l] : 0;
    }
    return TC_OK;
}

int tc_get_node_boxes(tc_handle* t, int level, double* boxes, int64_t cap, int64_t* count)
{
    if (!t || !count) return TC_ERR_INVALID;
    Handle& h = t->h;
    if (h.depth < 0) return TC_ERR_STATE;
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    const int64_t nn = h.nnodes;
    std::vector<uint32_t> cnt(nn);
    std::vector<double> bbc(2 * nn), len(nn);
    TC_CUDA_TRY(cudaMemcpyAsync(cnt.data(), h.count.p, nn * 4, cudaMemcpyDeviceToHost, h.stream));
    TC_CUDA_TRY(cudaMemcpyAsync(bbc.data(), h.bbc.p, nn * 16, cudaMemcpyDeviceToHost, h.stream));
    TC_CUDA_TRY(cudaMemcpyAsync(len.data(), h.bblen.p, nn * 8, cudaMemcpyDeviceToHost, h.stream));
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    int64_t c = 0;
    for (int l = 0; l <= h.depth; l++) {
        if (level >= 0 && l != level) continue;
        for (int64_t k = level_index(l); k < (int64_t)level_index(l + 1); k++) {
            if (cnt[k] == 0) continue;
            if (boxes && c < cap) {
                boxes[3 * c] = bbc[2 * k];
                boxes[3 * c + 1] = bbc[2 * k + 1];
                boxes[3 * c + 2] = len[k];
            }
            c++;
        }
    }
    *count = c;
    return TC_OK;
}

int tc_last_launch_count(tc_handle* t) { return t ? t->h.launches : 0; }

int tc_get_stage_times(tc_handle* t, double* ms)
{
    if (!t || !ms) return TC_ERR_INVALID;
    Handle& h = t->h;
    if (!h.ev_ready) return TC_ERR_STATE;
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    if (h.near_stream) TC_CUDA_TRY(cudaStreamSynchronize(h.near_stream));
    if (h.far_stream) TC_CUDA_TRY(cudaStreamSynchronize(h.far_stream));
    // stage k spans events (a, b); a < 0: the stage does not exist on this path
    const int split_a[TC_NSTAGES] = {0, 1, 2, 11, 8, 10, 6}, split_b[TC_NSTAGES] = {1, 2, 3, 5, 9, 6, 7};
    const int plain_a[TC_NSTAGES] = {0, 1, 2, 4, 5, -1, 6}, plain_b[TC_NSTAGES] = {1, 2, 3, 5, 6, -1, 7};
    const int* a = h.stage_split ? split_a : plain_a;
    const int* b = h.stage_split ? split_b : plain_b;
    for (int k = 0; k < TC_NSTAGES; k++) {
        float f = 0.f;
        cudaError_t e = a[k] < 0 ? cudaSuccess : cudaEventElapsedTime(&f, h.ev[a[k]], h.ev[b[k]]);
        ms[k] = e == cudaSuccess ? (double)f : -1.0;
    }
    cudaGetLastError();
    return TC_OK;
}

int tc_get_counters(tc_handle* t, uint64_t* counts)
{
    if (!t || !counts) return TC_ERR_INVALID;
    Handle& h = t->h;
    if (!h.counters.p) return TC_ERR_STATE;
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    TC_CUDA_TRY(cudaMemcpyAsync(counts, h.counters.p, 3 * 8, cudaMemcpyDeviceToHost, h.stream));
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    uint64_t m2l = 0;
    for (size_t l = 0; l < h.lists.nn_total.size(); l++) m2l += h.lists.nn_total[l];
    counts[3] = m2l;
    return TC_OK;
}

}  // extern "C"

extern "C" int tc_async_status(tc_handle* t)
{
    if (!t) return TC_ERR_INVALID;
    const Handle& h = t->h;
    return (h.h_words[8] ? 1 : 0) | (h.h_words[40] ? 2 : 0) | (h.h_words[48] ? 4 : 0);
}

extern "C" int tc_set_variant(tc_handle* t, int variant)
{
    if (!t || (variant != TC_VARIANT_SYM && variant != TC_VARIANT_MORTON)) {
        tc_set_error("tc_set_variant: unknown variant");
        return TC_ERR_INVALID;
    }
    if (variant == TC_VARIANT_MORTON && t->h.cfg.order != 0) {
        tc_set_error("tc_set_variant: the non-symmetric solver runs at the reference's expansion order (order 0)");
        return TC_ERR_INVALID;
    }
    t->h.variant = variant;
    t->h.tree_ready = false;  // the interaction lists depend on the MAC
    return TC_OK;
}

extern "C" int tc_set_leaf_p2p(tc_handle* t, int max_pairs)
{
    if (!t || max_pairs < 0) return TC_ERR_INVALID;
    if (max_pairs > 0 && t->h.cfg.order == 0) {
        tc_set_error("tc_set_leaf_p2p: needs an order-p handle (the reference order keeps its interaction set)");
        return TC_ERR_INVALID;
    }
    t->h.p2p_cut = (uint32_t)max_pairs;
    t->h.tree_ready = false;
    return TC_OK;
}

extern "C" int tc_set_adaptive_order(tc_handle* t, double slack)
{
    if (!t || std::isnan(slack)) return TC_ERR_INVALID;
    Handle& h = t->h;
    const bool enable = slack > 0.0;
    if (enable && (h.mac != TC_MAC_BMAX || h.cfg.order < 6 || (h.cfg.order & 1))) {
        tc_set_error("tc_set_adaptive_order: needs TC_MAC_BMAX and order 6, 8, 10 or 12");
        return TC_ERR_INVALID;
    }
    h.adapt = enable;
    h.adapt_slack = enable ? slack : 0.0;
    h.tree_ready = false;
    return TC_OK;
}

extern "C" int tc_set_expansion_centre(tc_handle* t, int centre)
{
    if (!t || (centre != TC_CENTRE_COM && centre != TC_CENTRE_BOX)) {
        tc_set_error("tc_set_expansion_centre: unknown centre");
        return TC_ERR_INVALID;
    }
    if (centre == TC_CENTRE_BOX && (t->h.cfg.order == 0 || t->h.cfg.precision != TC_PREC_FP32)) {
        tc_set_error("tc_set_expansion_centre: box-centred expansions need an order-p FP32 handle");
        return TC_ERR_INVALID;
    }
    t->h.centre = centre;
    if (centre != TC_CENTRE_BOX) t->h.m2l_tc = false;
    t->h.tree_ready = false;
    return TC_OK;
}

extern "C" int tc_set_m2l_engine(tc_handle* t, int engine)
{
    if (!t || (engine != TC_M2L_SIMT && engine != TC_M2L_TENSOR && engine != TC_M2L_TENSOR_ALL)) {
        tc_set_error("tc_set_m2l_engine: unknown engine");
        return TC_ERR_INVALID;
    }
    if (engine != TC_M2L_SIMT && t->h.centre != TC_CENTRE_BOX) {
        tc_set_error("tc_set_m2l_engine: the tensor-core M2L needs box-centred expansions (set them first)");
        return TC_ERR_INVALID;
    }
    t->h.m2l_tc = engine != TC_M2L_SIMT;
    t->h.m2l_tc_all = engine == TC_M2L_TENSOR_ALL;
    return TC_OK;
}

extern "C" int tc_set_near_overlap(tc_handle* t, int on)
{
    if (!t) return TC_ERR_INVALID;
    t->h.near_overlap = on != 0;
    return TC_OK;
}

extern "C" int tc_set_mac(tc_handle* t, int mac)
{
    if (!t || (mac != TC_MAC_CELL && mac != TC_MAC_BMAX)) {
        tc_set_error("tc_set_mac: unknown criterion");
        return TC_ERR_INVALID;
    }
    if (mac == TC_MAC_BMAX && t->h.cfg.order == 0) {
        tc_set_error("tc_set_mac: the bounding-radius criterion needs an order-p handle");
        return TC_ERR_INVALID;
    }
    t->h.mac = mac;
    if (mac != TC_MAC_BMAX) t->h.adapt = false;
    t->h.tree_ready = false;  // the interaction lists depend on the MAC
    return TC_OK;
}

extern "C" int tc_step_capture(tc_handle* t, const double* d_pos_xy, int64_t n, const double* box, double* d_grad_xy,
                               double* d_total, int scatter)
{
    if (!t || !d_pos_xy || !box || !d_grad_xy || !d_total) {
        tc_set_error("tc_step_capture: null argument");
        return TC_ERR_INVALID;
    }
    Handle& h = t->h;
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    if (!h.tree_ready || h.n != n) {
        tc_set_error("tc_step_capture: needs a synchronous update of the same n first (it sizes the lists)");
        return TC_ERR_STATE;
    }
    // one ordinary solve sizes the solver's buffers; then nothing may allocate
    int rc = tc_solve_device(t, d_grad_xy, d_total, 0, scatter);
    if (rc) return rc;
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    if ((rc = prepare_nosync(h))) return rc;
    if (h.step_graph) {
        cudaGraphExecDestroy(h.step_graph);
        h.step_graph = nullptr;
    }
    TC_CUDA_TRY(cudaStreamBeginCapture(h.stream, cudaStreamCaptureModeThreadLocal));
    h.nosync = true;
    rc = tc_update_tree_device(t, d_pos_xy, n, box, box + 2);
    int launches = h.launches;
    if (!rc) {
        const cudaError_t e = cudaMemsetAsync(d_total, 0, 8, h.stream);
        rc = e == cudaSuccess ? tc_solve_device(t, d_grad_xy, d_total, 0, scatter) : tc_cuda_fail(e, "memset");
        launches += h.launches;
    }
    h.nosync = false;
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(h.stream, &g);
    if (rc || ee != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return rc ? rc : tc_cuda_fail(ee, "cudaStreamEndCapture");
    }
    // kernel nodes keep their capture stream's priority (the far field above the near field)
    const cudaError_t ei = cudaGraphInstantiate(&h.step_graph, g, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        h.step_graph = nullptr;
        return tc_cuda_fail(ei, "cudaGraphInstantiate");
    }
    h.graph_launches = launches;
    return TC_OK;
}

extern "C" int tc_step_launch(tc_handle* t)
{
    if (!t) return TC_ERR_INVALID;
    Handle& h = t->h;
    if (!h.step_graph) {
        tc_set_error("tc_step_launch: no captured step");
        return TC_ERR_STATE;
    }
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    TC_CUDA_TRY(cudaGraphLaunch(h.step_graph, h.stream));
    h.launches = h.graph_launches;
    return TC_OK;
}
