// Training data for the expansion-order controller: for sampled node pairs
// (A sink, B source) of a built tree, the pair's features and the relative
// error of its order-p far field (M2L at order p, evaluated exactly at A's
// particles, i.e. the L2L/L2P chain of the FMM) against the direct sum over
// B's particles, for p in {4, 6, 8, 10, 12}.  The method measures its own
// errors; the features are the ones the controller sees at list-build time.
//
// Feature vector (all lengths in units of the level's cell size h):
//   0 log2|R|          1 min(|Rx|,|Ry|)/|R|    2 spread of A   3 spread of B
//   4 (spread A + spread B)/|R|                5 log2 M0(A)    6 log2 M0(B)
//   7 |COM(A) - centre(A)|                     8 |COM(B) - centre(B)|
//   9..12 log10 of B's normalised multipole norms at orders 2, 4, 6, 8
//   13 log10 of A's order-4 norm   14 log2(c/h^2) (kernel scale)   15 level/16
// (spread = sqrt(2 (mu20 + mu02) / M0), the RMS particle distance.)
#include <cmath>

#include "controller.cuh"
#include "expansion.cuh"
#include "kernels.cuh"
#include "state.cuh"

namespace tc {
namespace {

constexpr int PMAX = 12;
constexpr int KMAX = ncoef(PMAX);
constexpr int KSMAX = kstride(PMAX);
constexpr int SB = 64;  // threads per sampled pair
constexpr int SA_MAX = 64;
__constant__ int c_orders[TC_MLP_OUT] = {4, 6, 8, 10, 12};

template <typename KN>
__global__ void __launch_bounds__(SB) k_pair_errors(KN ker, PotParams pp, int dep, const int* __restrict__ pairs,
                                                    int64_t np,
                                                    const uint32_t* __restrict__ count,
                                                    const uint32_t* __restrict__ first, const double2* __restrict__ com64,
                                                    const float* __restrict__ comrel, const float* __restrict__ mu,
                                                    const double2* __restrict__ pos64, const float* __restrict__ hlev,
                                                    float* __restrict__ feat, float* __restrict__ err)
{
    __shared__ float sD[KMAX];
    __shared__ float sL[TC_MLP_OUT][KMAX];
    __shared__ float2 sb[SB];
    __shared__ float red[SB][TC_MLP_OUT + 1];
    const int t = threadIdx.x;
    for (int64_t s = blockIdx.x; s < np; s += gridDim.x) {
        const int l = pairs[3 * s], a = pairs[3 * s + 1], b = pairs[3 * s + 2];
        const bool valid = l >= 1 && l <= dep && a >= 0 && b >= 0 && a < (1 << (2 * l)) && b < (1 << (2 * l)) &&
                           count[level_index(l) + a] != 0 && count[level_index(l) + b] != 0;
        if (!valid) {  // refused input: no reads through the pair's indices
            if (t < TC_MLP_IN) feat[s * TC_MLP_IN + t] = 0.f;
            if (t < TC_MLP_OUT) err[s * TC_MLP_OUT + t] = 0.f;
            continue;
        }
        const int64_t A = level_index(l) + a, B = level_index(l) + b;
        const float h = hlev[l];
        const double2 cA = com64[A], cB = com64[B];
        const float Rx = (float)((cA.x - cB.x) / h), Ry = (float)((cA.y - cB.y) / h);
        if (t == 0) {
            derivs<PMAX>(Rx, Ry, h, pp, sD);
            pair_features(Rx, Ry, mu + A * KSMAX, mu + B * KSMAX, comrel[2 * A] / h, comrel[2 * A + 1] / h,
                          comrel[2 * B] / h, comrel[2 * B + 1] / h, pp.c / (h * h), l, feat + s * TC_MLP_IN);
        }
        __syncthreads();
        // order-p local expansions of A from B (scaled)
        const float* mB = mu + B * KSMAX;
        for (int beta = t; beta < KMAX; beta += SB) {
            const int kb = cdeg(beta), bb = beta - kb * (kb + 1) / 2, ab = kb - bb;
            for (int o = 0; o < TC_MLP_OUT; o++) {
                const int p = c_orders[o];
                float acc = 0.f;
                if (kb <= p) {
                    for (int ka = 0; ka + kb <= p; ka++) {
                        if (ka == 1) continue;
                        for (int ba = 0; ba <= ka; ba++) {
                            const float m = mB[cidx(ka - ba, ba)];
                            acc += ((ka & 1) ? -m : m) * sD[cidx(ka - ba + ab, ba + bb)];
                        }
                    }
                }
                sL[o][beta] = acc;
            }
        }
        __syncthreads();
        // sink particles: up to SA_MAX of A, evenly spaced
        const uint32_t cA_n = count[A], fA = first[A], cB_n = count[B], fB = first[B];
        const uint32_t sa = cA_n < SA_MAX ? cA_n : SA_MAX;
        const bool act = (uint32_t)t < sa;
        float dx = 0.f, dy = 0.f;
        if (act) {
            const double2 x = pos64[fA + (uint32_t)(((uint64_t)t * cA_n) / sa)];
            dx = (float)((x.x - cA.x) / h);
            dy = (float)((x.y - cA.y) / h);
        }
        float fx = 0.f, fy = 0.f;
        for (uint32_t q0 = 0; q0 < cB_n; q0 += SB) {
            __syncthreads();
            if (q0 + t < cB_n) {
                const double2 y = pos64[fB + q0 + t];
                sb[t] = make_float2((float)((y.x - cA.x) / h), (float)((y.y - cA.y) / h));
            }
            __syncthreads();
            const uint32_t m = min((uint32_t)SB, cB_n - q0);
            if (act)
                for (uint32_t j = 0; j < m; j++) {
                    const float rx = (dx - sb[j].x) * h, ry = (dy - sb[j].y) * h;
                    float D1, tt;
                    ker.near(rx * rx + ry * ry, D1, tt);
                    fx += D1 * rx;
                    fy += D1 * ry;
                }
        }
        // the order-p approximations at the same particle
        float e2[TC_MLP_OUT];
        if (act) {
            float w[ncoef(PMAX - 1)];
            monomials<PMAX - 1>(dx, dy, w);
            for (int o = 0; o < TC_MLP_OUT; o++) {
                const int p = c_orders[o];
                float gx = 0.f, gy = 0.f;
                for (int k = 0; k < p; k++)
                    for (int bq = 0; bq <= k; bq++) {
                        const int aq = k - bq;
                        gx += sL[o][cidx(aq + 1, bq)] * w[cidx(aq, bq)];
                        gy += sL[o][cidx(aq, bq + 1)] * w[cidx(aq, bq)];
                    }
                gx /= h;
                gy /= h;
                e2[o] = (gx - fx) * (gx - fx) + (gy - fy) * (gy - fy);
            }
        } else {
            for (int o = 0; o < TC_MLP_OUT; o++) e2[o] = 0.f;
        }
        for (int o = 0; o < TC_MLP_OUT; o++) red[t][o] = e2[o];
        red[t][TC_MLP_OUT] = act ? fx * fx + fy * fy : 0.f;
        __syncthreads();
        if (t == 0) {
            float ref = 0.f;
            for (int q = 0; q < SB; q++) ref += red[q][TC_MLP_OUT];
            for (int o = 0; o < TC_MLP_OUT; o++) {
                float e = 0.f;
                for (int q = 0; q < SB; q++) e += red[q][o];
                const float rel = ref > 0.f ? sqrtf(e / ref) : 1.f;
                err[s * TC_MLP_OUT + o] = log10f(fmaxf(rel, 1e-8f));
            }
        }
        __syncthreads();
    }
}

}  // namespace
}  // namespace tc

using namespace tc;

extern "C" int tc_get_list(tc_handle* t, int level, int kind, uint32_t* ptr, uint32_t* idx, int64_t* total)
{
    if (!t || kind < 0 || kind > 2) return TC_ERR_INVALID;
    Handle& h = t->h;
    if (!h.tree_ready || level < 0 || level > h.depth) return TC_ERR_STATE;
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    const Lists& L = h.lists;
    const int64_t nl = (int64_t)1 << (2 * level);
    const int64_t tot = kind == 1 ? L.near_total[level] : L.nn_total[level];
    if (total) *total = tot;
    if (kind == 2) {  // order buckets of the accepted pairs (one byte each)
        if (!h.ctrl_on) {
            tc_set_error("tc_get_list: no controller on this handle");
            return TC_ERR_STATE;
        }
        if (idx && tot)
            TC_CUDA_TRY(cudaMemcpyAsync(idx, P<uint8_t>(h.ord_pool) + L.nn_idx_off[level], tot,
                                        cudaMemcpyDeviceToHost, h.stream));
        TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
        return TC_OK;
    }
    const uint32_t* dptr = P<uint32_t>(h.ptr_pool) + (kind ? L.near_ptr_off[level] : L.nn_ptr_off[level]);
    const uint32_t* didx = P<uint32_t>(h.idx_pool) + (kind ? L.near_idx_off[level] : L.nn_idx_off[level]);
    if (ptr) TC_CUDA_TRY(cudaMemcpyAsync(ptr, dptr, (nl + 1) * 4, cudaMemcpyDeviceToHost, h.stream));
    if (idx && tot) TC_CUDA_TRY(cudaMemcpyAsync(idx, didx, tot * 4, cudaMemcpyDeviceToHost, h.stream));
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    return TC_OK;
}

extern "C" int tc_lc_pair_errors(tc_handle* t, const int32_t* d_pairs, int64_t n, float* d_feat, float* d_err)
{
    if (!t || !d_pairs || !d_feat || !d_err || n <= 0) return TC_ERR_INVALID;
    Handle& h = t->h;
    if (!h.tree_ready || h.cfg.order != 12 || !h.mu.p) {
        tc_set_error("tc_lc_pair_errors: needs a solved order-12 handle");
        return TC_ERR_STATE;
    }
    TC_CUDA_TRY(cudaSetDevice(h.cfg.device));
    float hl[16];
    for (int l = 0; l < 16; l++) hl[l] = (float)(h.L / (double)(1u << l));
    Buf dh;
    int rc = ensure(dh, sizeof(hl));
    if (rc) return rc;
    TC_CUDA_TRY(cudaMemcpyAsync(dh.p, hl, sizeof(hl), cudaMemcpyHostToDevice, h.stream));
    PotParams pp;
    pp.kind = h.cfg.kernel;
    const int grid = (int)(n < sm_count() * 16 ? n : sm_count() * 16);
    if (h.cfg.kernel == TC_KERNEL_GRAVITY) {
        pp.nu = 0.5f;
        pp.c = (float)(h.cfg.softening * h.cfg.softening);
        pp.kappa = -1.f;
        k_pair_errors<<<grid, SB, 0, h.stream>>>(KGrav<float>{pp.c}, pp, h.depth, d_pairs, n, P<uint32_t>(h.count),
                                                 P<uint32_t>(h.first), P<double2>(h.com64), P<float>(h.comrel),
                                                 P<float>(h.mu), P<double2>(h.pos64), P<float>(dh), d_feat, d_err);
    } else {
        pp.nu = 1.f;
        pp.c = 1.f;
        pp.kappa = -2.f;
        k_pair_errors<<<grid, SB, 0, h.stream>>>(KTsne<float>{}, pp, h.depth, d_pairs, n, P<uint32_t>(h.count),
                                                 P<uint32_t>(h.first), P<double2>(h.com64), P<float>(h.comrel),
                                                 P<float>(h.mu), P<double2>(h.pos64), P<float>(dh), d_feat, d_err);
    }
    TC_CUDA_TRY(cudaGetLastError());
    TC_CUDA_TRY(cudaStreamSynchronize(h.stream));
    release(dh);
    return TC_OK;
}
