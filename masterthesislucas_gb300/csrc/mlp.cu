// The expansion-order controller's network: a 3-layer MLP 16 -> 64 -> 64 -> 5
// (ReLU hidden layers), BF16 weights with FP32 accumulation, trained on the
// GPU by hand-written forward/backward and Adam kernels.
//
// Master parameters are FP32; every forward pass (training and inference)
// uses them rounded to BF16 (round-to-nearest-even), and the gradient with
// respect to the rounded weights updates the FP32 master copy.  Inputs are
// normalised by per-feature mean/std stored with the network.  Training
// batches are drawn by a counter-based hash, so a training run is a pure
// function of (data, seed, hyper-parameters).
//
// Layout of the parameter vector (TC_MLP_NPARAM floats):
//   W1[64][16] b1[64] W2[64][64] b2[64] W3[5][64] b3[5]
#include <cmath>
#include <vector>

#include "ctrl_mma.cuh"
#include "state.cuh"

namespace tc {
namespace {

constexpr int NI = TC_MLP_IN, NH = TC_MLP_HIDDEN, NO = TC_MLP_OUT;
constexpr int OW1 = 0, OB1 = OW1 + NH * NI, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH, OB3 = OW3 + NO * NH;
constexpr int NP = OB3 + NO;
static_assert(NP == TC_MLP_NPARAM, "parameter layout");
constexpr int TB = 64;  // samples per training block

__device__ __host__ inline float round_bf16(float x)
{
    // round to nearest even on the upper 16 bits (finite inputs)
    union {
        float f;
        uint32_t u;
    } v;
    v.f = x;
    const uint32_t lsb = (v.u >> 16) & 1u;
    v.u = (v.u + 0x7FFFu + lsb) & 0xFFFF0000u;
    return v.f;
}

__device__ inline uint64_t mix64(uint64_t x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

// forward of one sample with weights in shared memory (already BF16-rounded)
__device__ inline void forward_one(const float* w, const float* x, float* h1, float* h2, float* y)
{
    for (int i = 0; i < NH; i++) {
        float s = w[OB1 + i];
#pragma unroll
        for (int k = 0; k < NI; k++) s += w[OW1 + i * NI + k] * x[k];
        h1[i] = fmaxf(s, 0.f);
    }
    for (int i = 0; i < NH; i++) {
        float s = w[OB2 + i];
#pragma unroll 8
        for (int j = 0; j < NH; j++) s += w[OW2 + i * NH + j] * h1[j];
        h2[i] = fmaxf(s, 0.f);
    }
    for (int o = 0; o < NO; o++) {
        float s = w[OB3 + o];
#pragma unroll 8
        for (int j = 0; j < NH; j++) s += w[OW3 + o * NH + j] * h2[j];
        y[o] = s;
    }
}

__global__ void k_round_params(const float* __restrict__ master, float* __restrict__ rounded)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NP; i += gridDim.x * blockDim.x)
        rounded[i] = round_bf16(master[i]);
}

// one block of TB samples: forward, backward and the block's gradient partial
__global__ void __launch_bounds__(TB) k_mlp_grad(const float* __restrict__ wr, const float* __restrict__ X,
                                                 const float* __restrict__ T, const float* __restrict__ mean,
                                                 const float* __restrict__ stdv, int64_t n, int batch,
                                                 uint64_t seed, uint64_t step, int sample_random,
                                                 float* __restrict__ gpart, float* __restrict__ lpart)
{
    extern __shared__ float sm[];
    float* w = sm;                       // NP
    float* xs = w + NP;                  // TB x (NI+1)
    float* h1s = xs + TB * (NI + 1);     // TB x (NH+1)
    float* h2s = h1s + TB * (NH + 1);
    float* d1s = h2s + TB * (NH + 1);
    float* d2s = d1s + TB * (NH + 1);
    float* dys = d2s + TB * (NH + 1);    // TB x NO
    float* red = dys + TB * NO;          // TB
    const int t = threadIdx.x;
    for (int i = t; i < NP; i += TB) w[i] = wr[i];
    const int bi = blockIdx.x * TB + t;  // position in the batch
    const bool act = bi < batch;
    int64_t si = 0;
    if (act) {
        si = sample_random ? (int64_t)(mix64(seed * 0x9E3779B97F4A7C15ull + step * 1315423911ull + (uint64_t)bi) %
                                       (uint64_t)n)
                           : (int64_t)bi;
    }
    float x[NI];
    for (int k = 0; k < NI; k++) x[k] = act ? (X[si * NI + k] - mean[k]) / stdv[k] : 0.f;
    __syncthreads();
    float* h1 = h1s + t * (NH + 1);
    float* h2 = h2s + t * (NH + 1);
    float y[NO];
    forward_one(w, x, h1, h2, y);
    float loss = 0.f;
    float* dy = dys + t * NO;
    for (int o = 0; o < NO; o++) {
        const float e = act ? (y[o] - T[si * NO + o]) : 0.f;
        loss += e * e;
        dy[o] = act ? 2.f * e / (float)(batch * NO) : 0.f;
    }
    // backward through the layers (this sample)
    float* d2 = d2s + t * (NH + 1);
    float* d1 = d1s + t * (NH + 1);
    for (int j = 0; j < NH; j++) {
        float s = 0.f;
        for (int o = 0; o < NO; o++) s += w[OW3 + o * NH + j] * dy[o];
        d2[j] = h2[j] > 0.f ? s : 0.f;
    }
    for (int j = 0; j < NH; j++) {
        float s = 0.f;
#pragma unroll 8
        for (int i = 0; i < NH; i++) s += w[OW2 + i * NH + j] * d2[i];
        d1[j] = h1[j] > 0.f ? s : 0.f;
    }
    for (int k = 0; k < NI; k++) xs[t * (NI + 1) + k] = x[k];
    red[t] = loss;
    __syncthreads();
    // weight gradients of the block: each thread owns a strided set of entries
    float* g = gpart + (int64_t)blockIdx.x * NP;
    for (int e = t; e < NP; e += TB) {
        float s = 0.f;
        if (e < OB1) {
            const int i = (e - OW1) / NI, k = (e - OW1) % NI;
            for (int q = 0; q < TB; q++) s += d1s[q * (NH + 1) + i] * xs[q * (NI + 1) + k];
        } else if (e < OW2) {
            const int i = e - OB1;
            for (int q = 0; q < TB; q++) s += d1s[q * (NH + 1) + i];
        } else if (e < OB2) {
            const int i = (e - OW2) / NH, j = (e - OW2) % NH;
            for (int q = 0; q < TB; q++) s += d2s[q * (NH + 1) + i] * h1s[q * (NH + 1) + j];
        } else if (e < OW3) {
            const int i = e - OB2;
            for (int q = 0; q < TB; q++) s += d2s[q * (NH + 1) + i];
        } else if (e < OB3) {
            const int o = (e - OW3) / NH, j = (e - OW3) % NH;
            for (int q = 0; q < TB; q++) s += dys[q * NO + o] * h2s[q * (NH + 1) + j];
        } else {
            const int o = e - OB3;
            for (int q = 0; q < TB; q++) s += dys[q * NO + o];
        }
        g[e] = s;
    }
    if (t == 0) {
        float l = 0.f;
        for (int q = 0; q < TB; q++) l += red[q];
        lpart[blockIdx.x] = l;
    }
}

__global__ void k_grad_sum(const float* __restrict__ gpart, int nblk, const float* __restrict__ lpart,
                           float* __restrict__ grad, float* __restrict__ loss)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < NP; e += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nblk; b++) s += gpart[(int64_t)b * NP + e];
        grad[e] = s;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        float l = 0.f;
        for (int b = 0; b < nblk; b++) l += lpart[b];
        *loss = l;
    }
}

__global__ void k_adam(float* __restrict__ master, float* __restrict__ m1, float* __restrict__ m2,
                       const float* __restrict__ grad, float lr, float b1, float b2, float eps, float bc1, float bc2,
                       float* __restrict__ rounded)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NP; i += gridDim.x * blockDim.x) {
        const float g = grad[i];
        const float a = b1 * m1[i] + (1.f - b1) * g;
        const float b = b2 * m2[i] + (1.f - b2) * g * g;
        m1[i] = a;
        m2[i] = b;
        const float p = master[i] - lr * (a / bc1) / (sqrtf(b / bc2) + eps);
        master[i] = p;
        rounded[i] = round_bf16(p);
    }
}

__global__ void __launch_bounds__(128) k_mlp_forward(const float* __restrict__ wr, const float* __restrict__ X,
                                                     const float* __restrict__ mean, const float* __restrict__ stdv,
                                                     int64_t n, float* __restrict__ Y)
{
    __shared__ float w[NP];
    for (int i = threadIdx.x; i < NP; i += blockDim.x) w[i] = wr[i];
    __syncthreads();
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        float x[NI], h1[NH], h2[NH], y[NO];
        for (int k = 0; k < NI; k++) x[k] = (X[s * NI + k] - mean[k]) / stdv[k];
        forward_one(w, x, h1, h2, y);
        for (int o = 0; o < NO; o++) Y[s * NO + o] = y[o];
    }
}

// the list builder's tensor-core forward (BF16 inputs and activations), for tests
__global__ void __launch_bounds__(32 * ctrl::kWarps) k_mlp_forward_tc(const float* __restrict__ wr,
                                                                     const float* __restrict__ mean,
                                                                     const float* __restrict__ stdv,
                                                                     const float* __restrict__ X, int64_t n,
                                                                     float* __restrict__ Y)
{
    __shared__ __align__(16) ctrl::Smem S;
    ctrl::load_weights(S, wr, mean, stdv);
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t nwarps = (int64_t)gridDim.x * ctrl::kWarps;
    for (int64_t base = ((int64_t)blockIdx.x * ctrl::kWarps + wid) * 32; base < n; base += nwarps * 32) {
        const int64_t r = base + lane;
        float f[NI], y[NO];
        const bool use = r < n;
        for (int k = 0; k < NI; k++) f[k] = use ? X[r * NI + k] : 0.f;
        ctrl::warp_mlp(S, wid, lane, f, use, y);
        if (use)
            for (int k = 0; k < NO; k++) Y[r * NO + k] = y[k];
    }
}

}  // namespace
}  // namespace tc

using namespace tc;

struct tc_mlp {
    Buf master, rounded, m1, m2, grad, gpart, lpart, loss, mean, stdv;
    int64_t step = 0;
    cudaStream_t stream = nullptr;
};

static size_t grad_smem() { return sizeof(float) * (NP + TB * (NI + 1) + 4 * TB * (NH + 1) + TB * NO + TB); }

extern "C" {

int tc_mlp_create(uint64_t seed, tc_mlp** out)
{
    if (!out) return TC_ERR_INVALID;
    tc_mlp* m = new tc_mlp();
    int rc = 0;
    if ((rc = ensure(m->master, NP * 4)) || (rc = ensure(m->rounded, NP * 4)) || (rc = ensure(m->m1, NP * 4)) ||
        (rc = ensure(m->m2, NP * 4)) || (rc = ensure(m->grad, NP * 4)) || (rc = ensure(m->loss, 64)) ||
        (rc = ensure(m->mean, NI * 4)) || (rc = ensure(m->stdv, NI * 4))) {
        delete m;
        return rc;
    }
    // He-style uniform initialisation from a seeded LCG (deterministic)
    std::vector<float> p(NP, 0.f);
    uint64_t s = seed * 6364136223846793005ull + 1442695040888963407ull;
    auto uni = [&]() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return (float)((s >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
    };
    for (int i = 0; i < NH * NI; i++) p[OW1 + i] = uni() * std::sqrt(6.f / NI);
    for (int i = 0; i < NH * NH; i++) p[OW2 + i] = uni() * std::sqrt(6.f / NH);
    for (int i = 0; i < NO * NH; i++) p[OW3 + i] = uni() * std::sqrt(3.f / NH);
    std::vector<float> one(NI, 1.f), zero(NI, 0.f);
    cudaError_t e = cudaMemcpy(m->master.p, p.data(), NP * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(m->m1.p, 0, NP * 4);
    if (e == cudaSuccess) e = cudaMemset(m->m2.p, 0, NP * 4);
    if (e == cudaSuccess) e = cudaMemcpy(m->mean.p, zero.data(), NI * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(m->stdv.p, one.data(), NI * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        delete m;
        return tc_cuda_fail(e, "tc_mlp_create");
    }
    k_round_params<<<grid_for(NP, 256), 256>>>(P<float>(m->master), P<float>(m->rounded));
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        delete m;
        return tc_cuda_fail(e, "tc_mlp_create round");
    }
    *out = m;
    return TC_OK;
}

int tc_mlp_destroy(tc_mlp* m)
{
    if (!m) return TC_OK;
    Buf* bufs[] = {&m->master, &m->rounded, &m->m1, &m->m2, &m->grad, &m->gpart, &m->lpart,
                   &m->loss, &m->mean, &m->stdv};
    for (Buf* b : bufs) release(*b);
    delete m;
    return TC_OK;
}

int tc_mlp_set_normalization(tc_mlp* m, const float* mean, const float* stdv)
{
    if (!m || !mean || !stdv) return TC_ERR_INVALID;
    for (int k = 0; k < NI; k++)
        if (!(stdv[k] > 0.f) || !std::isfinite(mean[k])) return TC_ERR_INVALID;
    TC_CUDA_TRY(cudaMemcpy(m->mean.p, mean, NI * 4, cudaMemcpyHostToDevice));
    TC_CUDA_TRY(cudaMemcpy(m->stdv.p, stdv, NI * 4, cudaMemcpyHostToDevice));
    return TC_OK;
}

int tc_mlp_get_params(tc_mlp* m, float* params, float* mean, float* stdv)
{
    if (!m) return TC_ERR_INVALID;
    if (params) TC_CUDA_TRY(cudaMemcpy(params, m->master.p, NP * 4, cudaMemcpyDeviceToHost));
    if (mean) TC_CUDA_TRY(cudaMemcpy(mean, m->mean.p, NI * 4, cudaMemcpyDeviceToHost));
    if (stdv) TC_CUDA_TRY(cudaMemcpy(stdv, m->stdv.p, NI * 4, cudaMemcpyDeviceToHost));
    return TC_OK;
}

int tc_mlp_set_params(tc_mlp* m, const float* params)
{
    if (!m || !params) return TC_ERR_INVALID;
    TC_CUDA_TRY(cudaMemcpy(m->master.p, params, NP * 4, cudaMemcpyHostToDevice));
    k_round_params<<<grid_for(NP, 256), 256>>>(P<float>(m->master), P<float>(m->rounded));
    TC_CUDA_TRY(cudaDeviceSynchronize());
    return TC_OK;
}

int tc_mlp_forward_tc(tc_mlp* m, const float* d_x, int64_t n, float* d_y)
{
    if (!m || !d_x || !d_y || n <= 0) return TC_ERR_INVALID;
    const int64_t blocks = (n + 32 * ctrl::kWarps - 1) / (32 * ctrl::kWarps);
    k_mlp_forward_tc<<<(unsigned)(blocks < sm_count() * 16 ? blocks : sm_count() * 16), 32 * ctrl::kWarps>>>(
        P<float>(m->rounded), P<float>(m->mean), P<float>(m->stdv), d_x, n, d_y);
    TC_CUDA_TRY(cudaGetLastError());
    TC_CUDA_TRY(cudaDeviceSynchronize());
    return TC_OK;
}

int tc_set_controller(tc_handle* t, tc_mlp* m, double tau)
{
    if (!t) return TC_ERR_INVALID;
    Handle& h = t->h;
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    if (!m) {  // back to the MAC
        h.ctrl_on = false;
        h.tree_ready = false;
        return TC_OK;
    }
    if (!(tau > 0.0) || !(tau < 1.0)) {
        tc_set_error("tc_set_controller: tau must lie in (0, 1)");
        return TC_ERR_INVALID;
    }
    if (h.cfg.order != 12 || h.cfg.precision != TC_PREC_FP32) {
        tc_set_error("tc_set_controller: needs an FP32 order-12 handle");
        return TC_ERR_INVALID;
    }
    int rc;
    if ((rc = ensure(h.ctrl_w, (NP + 2 * NI) * 4 + 64))) return rc;
    TC_CUDA_TRY(cudaMemcpyAsync(h.ctrl_w.p, m->rounded.p, NP * 4, cudaMemcpyDeviceToDevice, h.stream));
    TC_CUDA_TRY(cudaMemcpyAsync(P<float>(h.ctrl_w) + NP, m->mean.p, NI * 4, cudaMemcpyDeviceToDevice, h.stream));
    TC_CUDA_TRY(cudaMemcpyAsync(P<float>(h.ctrl_w) + NP + NI, m->stdv.p, NI * 4, cudaMemcpyDeviceToDevice, h.stream));
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    h.ctrl_on = true;
    h.ctrl_log_tau = (float)std::log10(tau);
    h.ctrl_c = h.cfg.kernel == TC_KERNEL_GRAVITY ? h.cfg.softening * h.cfg.softening : 1.0;
    // the lists (and their capacities) change with the acceptance rule
    h.tree_ready = false;
    h.lists.caps_depth = -1;
    return TC_OK;
}

static int grad_pass(tc_mlp* m, const float* d_x, const float* d_t, int64_t n, int batch, uint64_t seed,
                     int sample_random)
{
    const int nblk = (batch + TB - 1) / TB;
    int rc;
    if ((rc = ensure(m->gpart, (size_t)nblk * NP * 4)) || (rc = ensure(m->lpart, (size_t)nblk * 4 + 16))) return rc;
    static bool attr = false;
    if (!attr) {
        TC_CUDA_TRY(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)grad_smem()));
        attr = true;
    }
    k_mlp_grad<<<nblk, TB, grad_smem()>>>(P<float>(m->rounded), d_x, d_t, P<float>(m->mean), P<float>(m->stdv), n,
                                          batch, seed, (uint64_t)m->step, sample_random, P<float>(m->gpart),
                                          P<float>(m->lpart));
    k_grad_sum<<<grid_for(NP, 256), 256>>>(P<float>(m->gpart), nblk, P<float>(m->lpart), P<float>(m->grad),
                                          P<float>(m->loss));
    TC_CUDA_TRY(cudaGetLastError());
    return TC_OK;
}

int tc_mlp_gradient(tc_mlp* m, const float* d_x, const float* d_t, int64_t n, float* grad, float* loss)
{
    if (!m || !d_x || !d_t || n <= 0 || n > (1 << 20)) return TC_ERR_INVALID;
    int rc = grad_pass(m, d_x, d_t, n, (int)n, 0, 0);
    if (rc) return rc;
    TC_CUDA_TRY(cudaDeviceSynchronize());
    if (grad) TC_CUDA_TRY(cudaMemcpy(grad, m->grad.p, NP * 4, cudaMemcpyDeviceToHost));
    if (loss) TC_CUDA_TRY(cudaMemcpy(loss, m->loss.p, 4, cudaMemcpyDeviceToHost));
    return TC_OK;
}

int tc_mlp_train(tc_mlp* m, const float* d_x, const float* d_t, int64_t n, int steps, int batch, float lr,
                 uint64_t seed, float* last_loss)
{
    if (!m || !d_x || !d_t || n <= 0 || steps <= 0 || batch <= 0 || batch > (1 << 20) || !(lr > 0.f))
        return TC_ERR_INVALID;
    const float b1 = 0.9f, b2 = 0.999f;
    for (int s = 0; s < steps; s++) {
        int rc = grad_pass(m, d_x, d_t, n, batch, seed, 1);
        if (rc) return rc;
        m->step++;
        const float bc1 = 1.f - std::pow(b1, (float)m->step), bc2 = 1.f - std::pow(b2, (float)m->step);
        k_adam<<<grid_for(NP, 256), 256>>>(P<float>(m->master), P<float>(m->m1), P<float>(m->m2), P<float>(m->grad),
                                          lr, b1, b2, 1e-8f, bc1, bc2, P<float>(m->rounded));
    }
    TC_CUDA_TRY(cudaGetLastError());
    TC_CUDA_TRY(cudaDeviceSynchronize());
    if (last_loss) TC_CUDA_TRY(cudaMemcpy(last_loss, m->loss.p, 4, cudaMemcpyDeviceToHost));
    return TC_OK;
}

int tc_mlp_forward(tc_mlp* m, const float* d_x, int64_t n, float* d_y)
{
    if (!m || !d_x || !d_y || n <= 0) return TC_ERR_INVALID;
    k_mlp_forward<<<grid_for(n, 128, sm_count() * 8), 128>>>(P<float>(m->rounded), d_x, P<float>(m->mean),
                                                       P<float>(m->stdv), n, d_y);
    TC_CUDA_TRY(cudaGetLastError());
    TC_CUDA_TRY(cudaDeviceSynchronize());
    return TC_OK;
}

}  // extern "C"
