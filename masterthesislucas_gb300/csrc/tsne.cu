// The t-SNE gradient step around the force call, device resident:
//   TSNE::updateRepulsive  (src/nBodyInstances/tsne.h:287-301)  g = (4/Z) * repulsion, un-permuted by ID
//   TSNE::updateAttractive (tsne.h:356-381)  g_i += exag * sum_j P_ij q_ij (y_j - y_i), CSR rows
//   TSNE::updatePoints     (tsne.h:179-206)  y' = y + lr g + momentum (y - y_prev)
// The repulsion comes from the tree code with its output scattered straight
// to ID order; the attractive term, the 4/Z scale and the momentum update are
// one fused kernel (one warp per CSR row) that reads Z from device memory.
// Z is summed in FP64; the attractive products run in FP32 on FP64
// differences of the FP64 embedding.
#include <cmath>
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
                                   const double* __restrict__ z, double exag, double lr, double mom,
                                   double2* __restrict__ y_next, double* __restrict__ grad_out)
{
    const int lane = threadIdx.x & 31;
    const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
    const double scale = 4.0 / *z;
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
    Buf row_ptr, col, val, grad_rep, grad, z;
    double last_z = 0.0;
    int launches = 0;
};


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
    tc_destroy(t->solver);
    delete t;
    return TC_OK;
}

int tc_tsne_set_theta(tc_tsne* t, double theta) { return t ? tc_set_theta(t->solver, theta) : TC_ERR_INVALID; }

// One iteration of TSNE_buffers::timeStep (src/nBodyInstances/tsne_buffers.h:125-168):
// tree on the current embedding, repulsion + Z, attractive term, momentum step.
// exag_code is the code's factor (16 early / 4 late in the reference).
int tc_tsne_step(tc_tsne* t, double exag_code, double momentum, double lr, double* z_out)
{
    if (!t) return TC_ERR_INVALID;
    Handle& h = *t->hs;
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    const double* y = P<double>(t->y[t->cur]);
    int rc = tc_update_tree_device(t->solver, y, t->n, nullptr, nullptr);
    if (rc) return rc;
    int launches = h.launches;
    TC_CUDA_TRY(cudaMemsetAsync(t->z.p, 0, 8, h.stream));
    rc = tc_solve_device(t->solver, P<double>(t->grad_rep), P<double>(t->z), 0, 1);
    if (rc) return rc;
    launches += h.launches;
    if (h.cfg.precision == TC_PREC_FP64)
        k_tsne_attr_update<double, double><<<grid_for(t->n * 32, 256, kSMs * 32), 256, 0, h.stream>>>(
            t->n, P<uint32_t>(t->row_ptr), P<uint32_t>(t->col), P<double>(t->val), P<double2>(t->y[t->cur]),
            P<double2>(t->y[t->prev]), P<double>(t->grad_rep), P<double>(t->z), exag_code, lr, momentum,
            P<double2>(t->y[t->next]), P<double>(t->grad));
    else
        k_tsne_attr_update<float, float><<<grid_for(t->n * 32, 256, kSMs * 32), 256, 0, h.stream>>>(
            t->n, P<uint32_t>(t->row_ptr), P<uint32_t>(t->col), P<float>(t->val), P<double2>(t->y[t->cur]),
            P<double2>(t->y[t->prev]), P<double>(t->grad_rep), P<double>(t->z), exag_code, lr, momentum,
            P<double2>(t->y[t->next]), P<double>(t->grad));
    TC_CUDA_TRY(cudaGetLastError());
    t->launches = launches + 1;
    int c = t->cur, p = t->prev, nx = t->next;
    t->prev = c;
    t->cur = nx;
    t->next = p;
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
