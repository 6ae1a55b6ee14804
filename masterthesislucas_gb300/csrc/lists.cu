// Interaction lists: the recursion of traverse_SYM_NN
// (src/nbodysolvers/cpu/nBodySolverFMM_SYM_MORTON.h:154-270) turned into a
// level-synchronous, per-sink-node construction.
//
// The reference walks unordered node pairs (A, B) of the same level from
// (root, root).  A pair is accepted for the symmetric M2L when
// |com_A - com_B|^2 > ((L_A + L_B) / theta)^2; otherwise, above the leaf level,
// every pair of non-empty children is visited (j >= i when A == B); at the
// leaf level a non-accepted pair becomes a point-level interaction.
//
// Here each node A stores the partners of every visited pair it belongs to,
// in both directions, split into
//   nn(A)   - partners accepted by the MAC (M2L sources for A),
//   near(A) - partners not accepted (refined at the next level; at the leaf
//             level they are the P2P / PN partners, including A itself).
// Since near(child) and nn(child) are drawn from the non-empty children of
// near(parent), the lists hold exactly the reference's visited pairs.  The
// MAC is evaluated in FP64 from the bit-exact COMs, so the decisions are the
// reference's decisions.
#include "state.cuh"

namespace tc {
namespace {

__device__ inline bool mac_accept(double2 a, double2 b, double len, double inv_theta)
{
    double dx = a.x - b.x, dy = a.y - b.y;
    double dist = dx * dx + dy * dy;
    double thr = (len + len) * inv_theta;
    return dist > thr * thr;
}

// The same decision, decided in FP32 from cell-relative COMs whenever the FP32
// squared distance is farther than a relative 1e-5 from the threshold (the
// FP32 distance is accurate to ~1e-7 relative for the offsets that occur);
// inside that band the exact FP64 test decides.  FP64 throughput on GB300 is
// 1/64 of FP32, and the band holds a vanishing fraction of candidates.
template <typename real>
__device__ inline bool mac_accept_fast(int dix, int diy, real hl, real thr2, const real* cra, const real* crb,
                                       double2 a, double2 b, double len, double inv_theta)
{
    if (sizeof(real) == 4) {
        const real dx = (real)dix * hl + (cra[0] - crb[0]);
        const real dy = (real)diy * hl + (cra[1] - crb[1]);
        const real d2 = dx * dx + dy * dy;
        if (d2 > thr2 * (real)(1.0 + 1e-5)) return true;
        if (d2 < thr2 * (real)(1.0 - 1e-5)) return false;
    }
    return mac_accept(a, b, len, inv_theta);
}

// one thread per node of level l; fill == 0 counts, fill == 1 writes
template <typename real>
__global__ void k_lists(int l, double inv_theta, real hl, const uint32_t* __restrict__ count,
                        const double2* __restrict__ com64, const real* __restrict__ comrel,
                        const double* __restrict__ bblen, const uint32_t* __restrict__ pnear_ptr,
                        const uint32_t* __restrict__ pnear_idx, uint32_t pcap, uint32_t* __restrict__ nn_cnt,
                        uint32_t* __restrict__ near_cnt, const uint32_t* __restrict__ nn_ptr,
                        uint32_t* __restrict__ nn_idx, uint32_t nn_cap, const uint32_t* __restrict__ near_ptr,
                        uint32_t* __restrict__ near_idx, uint32_t near_cap, uint32_t* __restrict__ ovf, int fill)
{
    const uint32_t np = l ? (1u << (2 * (l - 1))) : 0u;
    const uint32_t li = level_index(l);
    const int64_t nl = (int64_t)1 << (2 * l);
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < nl; a += (int64_t)gridDim.x * blockDim.x) {
        uint32_t nn = 0, nr = 0;
        if (count[li + a] != 0) {
            if (l == 0) {
                nr = 1;
                if (fill) {
                    if (near_ptr[a] < near_cap) near_idx[near_ptr[a]] = 0;
                    else atomicOr(ovf, 1u);
                }
            } else {
                const double2 ca = com64[li + a];
                const double len = bblen[li + a];
                const real thr = (real)((len + len) * inv_theta);
                const real thr2 = thr * thr;
                const int iax = (int)compact16((uint32_t)a), iay = (int)compact16((uint32_t)a >> 1);
                const real cra[2] = {comrel[2 * (li + a)], comrel[2 * (li + a) + 1]};
                const uint32_t p = (uint32_t)(a >> 2);
                const uint32_t nb = fill ? nn_ptr[a] : 0, rb = fill ? near_ptr[a] : 0;
                const uint32_t pe1 = pnear_ptr[p + 1] < pcap ? pnear_ptr[p + 1] : pcap;
                for (uint32_t e = pnear_ptr[p]; e < pe1; e++) {
                    const uint32_t bp = pnear_idx[e];
                    if (bp >= np) continue;  // only after an overflowed parent level
                    for (uint32_t j = 0; j < 4; j++) {
                        const uint32_t b = 4 * bp + j;
                        if (count[li + b] == 0) continue;
                        if (mac_accept_fast<real>(iax - (int)compact16(b), iay - (int)compact16(b >> 1), hl, thr2, cra,
                                                  comrel + 2 * (li + b), ca, com64[li + b], len, inv_theta)) {
                            if (fill) {
                                if (nb + nn < nn_cap) nn_idx[nb + nn] = b;
                                else atomicOr(ovf, 1u);
                            }
                            nn++;
                        } else {
                            if (fill) {
                                if (rb + nr < near_cap) near_idx[rb + nr] = b;
                                else atomicOr(ovf, 1u);
                            }
                            nr++;
                        }
                    }
                }
            }
        }
        if (!fill) {
            nn_cnt[a] = nn;
            near_cnt[a] = nr;
        }
    }
}

// per-level list totals (last entries of the CSR pointer arrays)
__global__ void k_list_totals(const uint32_t* __restrict__ ptr, const int64_t* __restrict__ offs, int nlev,
                              uint32_t* __restrict__ out)
{
    for (int k = threadIdx.x; k < 2 * nlev; k += blockDim.x) {
        const int l = k >> 1;
        out[k] = ptr[offs[k] + ((int64_t)1 << (2 * l))];
    }
}

}  // namespace

int build_lists(Handle& h)
{
    cudaStream_t s = h.stream;
    const int depth = h.depth;
    Lists& L = h.lists;
    L.nn_total.assign(depth + 1, 0);
    L.near_total.assign(depth + 1, 0);
    L.nn_ptr_off.assign(depth + 1, 0);
    L.near_ptr_off.assign(depth + 1, 0);
    L.nn_idx_off.assign(depth + 1, 0);
    L.near_idx_off.assign(depth + 1, 0);
    // pointer pool: two (4^l + 1)-word CSR pointer arrays per level
    int64_t ptr_words = 0;
    for (int l = 0; l <= depth; l++) {
        int64_t nl = (int64_t)1 << (2 * l);
        L.nn_ptr_off[l] = ptr_words;
        ptr_words += nl + 1;
        L.near_ptr_off[l] = ptr_words;
        ptr_words += nl + 1;
    }
    const int64_t nleaf = (int64_t)1 << (2 * depth);
    int rc;
    if ((rc = ensure(h.ptr_pool, ptr_words * 4)) || (rc = ensure(h.cnt_tmp, 2 * nleaf * 4 + 64)) ||
        (rc = ensure(h.tmp, (radix_tmp_words(h.n) > scan_tmp_words(nleaf) ? radix_tmp_words(h.n)
                                                                           : scan_tmp_words(nleaf)) * 4)))
        return rc;
    uint32_t* ptr = P<uint32_t>(h.ptr_pool);
    uint32_t* nn_cnt = P<uint32_t>(h.cnt_tmp);
    uint32_t* near_cnt = nn_cnt + nleaf;
    const double inv_theta = 1.0 / h.cfg.theta;
    uint32_t* ovf_flag = P<uint32_t>(h.err) + 1;
    auto launch = [&](int l, const uint32_t* pnp, const uint32_t* pni, uint32_t pcap, uint32_t* nnc, uint32_t* nrc,
                      const uint32_t* nnp, uint32_t* nni, uint32_t nncap, const uint32_t* nrp, uint32_t* nri,
                      uint32_t nrcap, int fill) {
        const int64_t nl = (int64_t)1 << (2 * l);
        const double hl = h.L / (double)(1u << l);
        if (h.cfg.precision == TC_PREC_FP64)
            k_lists<double><<<grid_for(nl, 128), 128, 0, s>>>(l, inv_theta, hl, P<uint32_t>(h.count),
                                                             P<double2>(h.com64), P<double>(h.comrel),
                                                             P<double>(h.bblen), pnp, pni, pcap, nnc, nrc, nnp, nni,
                                                             nncap, nrp, nri, nrcap, ovf_flag, fill);
        else
            k_lists<float><<<grid_for(nl, 128), 128, 0, s>>>(l, inv_theta, (float)hl, P<uint32_t>(h.count),
                                                            P<double2>(h.com64), P<float>(h.comrel),
                                                            P<double>(h.bblen), pnp, pni, pcap, nnc, nrc, nnp, nni,
                                                            nncap, nrp, nri, nrcap, ovf_flag, fill);
    };
    uint32_t* ovf = P<uint32_t>(h.err) + 1;
    TC_CUDA_TRY(cudaMemsetAsync(ovf, 0, 4, s));
    // Fast mode: per-level regions sized from the last exact totals (x1.25),
    // no host round trip between levels; one synchronisation at the end
    // verifies that no level overflowed, else the exact mode reruns.
    const bool fast = L.caps_depth == depth && (int64_t)L.nn_cap.size() == depth + 1;
    if (fast) {
        int64_t words = 0;
        for (int l = 0; l <= depth; l++) {
            L.nn_idx_off[l] = words;
            words += L.nn_cap[l];
            L.near_idx_off[l] = words;
            words += L.near_cap[l];
        }
        if ((rc = ensure(h.idx_pool, (size_t)words * 4 + 64))) return rc;
        for (int l = 0; l <= depth; l++) {
            const int64_t nl = (int64_t)1 << (2 * l);
            const uint32_t* pnp = l ? ptr + L.near_ptr_off[l - 1] : nullptr;
            const uint32_t* pni = l ? P<uint32_t>(h.idx_pool) + L.near_idx_off[l - 1] : nullptr;
            const uint32_t pcap = l ? L.near_cap[l - 1] : 0u;
            launch(l, pnp, pni, pcap, nn_cnt, near_cnt, nullptr, nullptr, 0, nullptr, nullptr, 0, 0);
            uint32_t* nnp = ptr + L.nn_ptr_off[l];
            uint32_t* nrp = ptr + L.near_ptr_off[l];
            if ((rc = exclusive_scan_u32(nn_cnt, nnp, nl, P<uint32_t>(h.tmp), s))) return rc;
            if ((rc = exclusive_scan_u32(near_cnt, nrp, nl, P<uint32_t>(h.tmp), s))) return rc;
            launch(l, pnp, pni, pcap, nullptr, nullptr, nnp, P<uint32_t>(h.idx_pool) + L.nn_idx_off[l], L.nn_cap[l],
                   nrp, P<uint32_t>(h.idx_pool) + L.near_idx_off[l], L.near_cap[l], 1);
            h.launches += 8;
        }
        // totals of every level plus the overflow flag, in one round trip
        std::vector<int64_t> offs(2 * (depth + 1));
        for (int l = 0; l <= depth; l++) {
            offs[2 * l] = L.nn_ptr_off[l];
            offs[2 * l + 1] = L.near_ptr_off[l];
        }
        if ((rc = ensure(h.lstat, offs.size() * 8 + 4 * 64))) return rc;
        TC_CUDA_TRY(cudaMemcpyAsync(h.lstat.p, offs.data(), offs.size() * 8, cudaMemcpyHostToDevice, s));
        uint32_t* dtot = (uint32_t*)((char*)h.lstat.p + offs.size() * 8);
        k_list_totals<<<1, 64, 0, s>>>(ptr, P<int64_t>(h.lstat), depth + 1, dtot);
        h.launches++;
        TC_CUDA_TRY(cudaMemcpyAsync(h.h_words, dtot, 4 * 2 * (depth + 1), cudaMemcpyDeviceToHost, s));
        TC_CUDA_TRY(cudaMemcpyAsync(h.h_words + 40, ovf, 4, cudaMemcpyDeviceToHost, s));
        TC_CUDA_TRY(cudaStreamSynchronize(s));
        bool over = h.h_words[40] != 0;
        for (int l = 0; l <= depth; l++) {
            L.nn_total[l] = h.h_words[2 * l];
            L.near_total[l] = h.h_words[2 * l + 1];
            over = over || L.nn_total[l] > L.nn_cap[l] || L.near_total[l] > L.near_cap[l];
        }
        if (!over) {
            TC_CUDA_TRY(cudaGetLastError());
            return record(h, 3);
        }
        TC_CUDA_TRY(cudaMemsetAsync(ovf, 0, 4, s));
    }
    // exact mode: the host reads each level's totals before the next level
    // (the first call, and after a fast-mode overflow)
    int64_t idx_words = 0;
    for (int l = 0; l <= depth; l++) {
        const int64_t nl = (int64_t)1 << (2 * l);
        const uint32_t* pnp = l ? ptr + L.near_ptr_off[l - 1] : nullptr;
        const uint32_t* pni = l ? P<uint32_t>(h.idx_pool) + L.near_idx_off[l - 1] : nullptr;
        const uint32_t pcap = l ? L.near_total[l - 1] : 0u;
        launch(l, pnp, pni, pcap, nn_cnt, near_cnt, nullptr, nullptr, 0, nullptr, nullptr, 0, 0);
        uint32_t* nnp = ptr + L.nn_ptr_off[l];
        uint32_t* nrp = ptr + L.near_ptr_off[l];
        if ((rc = exclusive_scan_u32(nn_cnt, nnp, nl, P<uint32_t>(h.tmp), s))) return rc;
        if ((rc = exclusive_scan_u32(near_cnt, nrp, nl, P<uint32_t>(h.tmp), s))) return rc;
        TC_CUDA_TRY(cudaMemcpyAsync(h.h_words, nnp + nl, 4, cudaMemcpyDeviceToHost, s));
        TC_CUDA_TRY(cudaMemcpyAsync(h.h_words + 1, nrp + nl, 4, cudaMemcpyDeviceToHost, s));
        TC_CUDA_TRY(cudaStreamSynchronize(s));
        L.nn_total[l] = h.h_words[0];
        L.near_total[l] = h.h_words[1];
        L.nn_idx_off[l] = idx_words;
        idx_words += L.nn_total[l];
        L.near_idx_off[l] = idx_words;
        idx_words += L.near_total[l];
        // grow the pool keeping the earlier levels (needed as parents)
        if ((size_t)idx_words * 4 > h.idx_pool.bytes) {
            Buf nb;
            if ((rc = ensure(nb, (size_t)(idx_words * 4 * 3 / 2 + 1024)))) return rc;
            if (h.idx_pool.p && L.nn_idx_off[l] > 0)
                TC_CUDA_TRY(cudaMemcpyAsync(nb.p, h.idx_pool.p, L.nn_idx_off[l] * 4, cudaMemcpyDeviceToDevice, s));
            TC_CUDA_TRY(cudaStreamSynchronize(s));
            release(h.idx_pool);
            h.idx_pool = nb;
        }
        pni = l ? P<uint32_t>(h.idx_pool) + L.near_idx_off[l - 1] : nullptr;
        launch(l, pnp, pni, pcap, nullptr, nullptr, nnp, P<uint32_t>(h.idx_pool) + L.nn_idx_off[l], L.nn_total[l],
               nrp, P<uint32_t>(h.idx_pool) + L.near_idx_off[l], L.near_total[l], 1);
        h.launches += 8;
    }
    // capacities for the next calls
    L.nn_cap.resize(depth + 1);
    L.near_cap.resize(depth + 1);
    for (int l = 0; l <= depth; l++) {
        L.nn_cap[l] = (uint32_t)(L.nn_total[l] + L.nn_total[l] / 4 + 256);
        L.near_cap[l] = (uint32_t)(L.near_total[l] + L.near_total[l] / 4 + 256);
    }
    L.caps_depth = depth;
    TC_CUDA_TRY(cudaGetLastError());
    return record(h, 3);
}

}  // namespace tc
