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
// near(parent), the lists hold exactly the reference's visited pairs.  At the
// reference's expansion order the MAC is decided as the reference decides it
// (FP64 from the bit-exact COMs wherever FP32 is not conclusive).  Order-p
// handles build physics-mode trees (FP32 records) and may open by the nodes'
// bounding radii instead of their cell sizes, send cheap accepted leaf pairs
// to P2P, or give accepted pairs their own expansion order; the structure of
// the lists is the same.
#include <cmath>

#include "controller.cuh"
#include "ctrl_mma.cuh"
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

// the non-symmetric solver's MAC (nBodySolverFMM_MORTON.h:150-153):
// (L_A + L_B) / |com_A - com_B| < theta, in the reference's operation order
__device__ inline bool mac_accept_m(double2 a, double2 b, double len, double theta)
{
    double dx = a.x - b.x, dy = a.y - b.y;
    double dist = sqrt(dx * dx + dy * dy);
    return (len + len) / dist < theta;
}

// The same decision, decided in FP32 from cell-relative COMs whenever the FP32
// squared distance is farther than a relative 1e-5 from the threshold (the
// FP32 distance is accurate to ~1e-7 relative for the offsets that occur);
// inside that band the exact FP64 test decides.  FP64 throughput on GB300 is
// 1/64 of FP32, and the band holds a vanishing fraction of candidates.
template <typename real>
__device__ inline bool mac_accept_fast(int dix, int diy, real hl, real thr2, const real* cra, const real* crb,
                                       double2 a, double2 b, double len, double inv_theta, double theta, int variant)
{
    if (sizeof(real) == 4) {
        const real dx = (real)dix * hl + (cra[0] - crb[0]);
        const real dy = (real)diy * hl + (cra[1] - crb[1]);
        const real d2 = dx * dx + dy * dy;
        if (d2 > thr2 * (real)(1.0 + 1e-5)) return true;
        if (d2 < thr2 * (real)(1.0 - 1e-5)) return false;
    }
    return variant ? mac_accept_m(a, b, len, theta) : mac_accept(a, b, len, inv_theta);
}

// levels of up to this many cells (4^TC_LISTS_WARP_LEVEL) build their lists with a warp per node
#ifndef TC_LISTS_WARP_LEVEL
#define TC_LISTS_WARP_LEVEL 8
#endif
constexpr int64_t kListsWarpLevelNodes = (int64_t)1 << (2 * TC_LISTS_WARP_LEVEL);

// Squared-ratio thresholds of the per-pair order rule: an accepted pair with
// (b_A + b_B)^2 <= t[o] |dcom|^2 takes order bucket o (orders 4, 6, 8, 10, 12);
// t[o] = (slack theta^(p + 1))^(2 / (q_o + 1)) below the handle's order p,
// and unbounded at p.
struct OrderRule {
    float t[5];
};

// one thread per node of level l; fill == 0 counts, fill == 1 writes.  With
// nn_ord (per-pair orders) the fill pass writes a node's accepted entries
// grouped by order bucket, ascending, and the bucket of each in nn_ord.
template <typename real>
__global__ void k_lists(int l, double inv_theta, double theta, int variant, real hl, const uint32_t* __restrict__ count,
                        const double2* __restrict__ com64, const real* __restrict__ comrel,
                        const double* __restrict__ bblen, const uint32_t* __restrict__ pnear_ptr,
                        const uint32_t* __restrict__ pnear_idx, uint32_t pcap, uint32_t* __restrict__ nn_cnt,
                        uint32_t* __restrict__ near_cnt, const uint32_t* __restrict__ nn_ptr,
                        uint32_t* __restrict__ nn_idx, uint32_t nn_cap, const uint32_t* __restrict__ near_ptr,
                        uint32_t* __restrict__ near_idx, uint32_t near_cap, uint32_t* __restrict__ ovf, int fill,
                        const uint32_t* __restrict__ act, const uint32_t* __restrict__ act_pos,
                        const float* __restrict__ bmax, float theta2, uint8_t* __restrict__ nn_ord, OrderRule rule,
                        uint8_t* __restrict__ dec, uint32_t p2p_cut)
{
    const uint32_t np = l ? (1u << (2 * (l - 1))) : 0u;
    const uint32_t li = level_index(l);
    const int64_t nl = (int64_t)1 << (2 * l);
    // with an active-node list only the non-empty nodes are visited (the
    // caller zeroes the counts of the others)
    const int64_t k0 = act ? (int64_t)act_pos[li] : 0, k1 = act ? (int64_t)act_pos[li + nl] : nl;
    for (int64_t k = k0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < k1; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = act ? (int64_t)act[k] - li : k;
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
                const float ba = bmax ? bmax[li + a] : 0.f;
                const uint32_t p = (uint32_t)(a >> 2);
                const uint32_t pe0 = pnear_ptr[p], pe1 = pnear_ptr[p + 1] < pcap ? pnear_ptr[p + 1] : pcap;
                // p2p_cut (leaf level only; 0 off): an accepted pair of leaves with at most p2p_cut
                // particle pairs goes to the near list, where direct P2P is cheaper than an M2L
                const uint32_t ca_n = p2p_cut ? count[li + a] : 0u;
                auto direct_cheaper = [&](uint32_t b) { return p2p_cut && ca_n * count[li + b] <= p2p_cut; };
                // every non-empty candidate: f(b, accepted, order bucket)
                auto visit = [&](auto&& f) {
                    for (uint32_t e = pe0; e < pe1; e++) {
                        const uint32_t bp = pnear_idx[e];
                        if (bp >= np) continue;  // only after an overflowed parent level
                        for (uint32_t j = 0; j < 4; j++) {
                            const uint32_t b = 4 * bp + j;
                            if (count[li + b] == 0) continue;
                            bool acc;
                            int o = 0;
                            if (bmax) {
                                // bounding-radius MAC in the cell-relative FP32 frame:
                                // theta^2 |com_A - com_B|^2 > (b_A + b_B)^2
                                const float dx = (float)(iax - (int)compact16(b)) * (float)hl +
                                                 ((float)cra[0] - (float)comrel[2 * (li + b)]);
                                const float dy = (float)(iay - (int)compact16(b >> 1)) * (float)hl +
                                                 ((float)cra[1] - (float)comrel[2 * (li + b) + 1]);
                                const float rb = ba + bmax[li + b], rb2 = rb * rb, d2 = fmaf(dx, dx, dy * dy);
                                acc = theta2 * d2 > rb2;
                                if (nn_ord && acc)
                                    while (o < 4 && rb2 > rule.t[o] * d2) o++;
                            } else {
                                acc = mac_accept_fast<real>(iax - (int)compact16(b), iay - (int)compact16(b >> 1), hl,
                                                            thr2, cra, comrel + 2 * (li + b), ca, com64[li + b], len,
                                                            inv_theta, theta, variant);
                            }
                            if (acc && direct_cheaper(b)) acc = false;
                            f(b, acc, o);
                        }
                    }
                };
                if (!fill && dec && !nn_ord) {
                    // count pass that keeps its decisions: per parent near entry e and
                    // sibling slot a & 3, bits 0-3 accepted child j, bits 4-7 non-empty child j
                    for (uint32_t e = pe0; e < pe1; e++) {
                        const uint32_t bp = pnear_idx[e];
                        uint32_t bits = 0;
                        if (bp < np) {
                            for (uint32_t j = 0; j < 4; j++) {
                                const uint32_t b = 4 * bp + j;
                                if (count[li + b] == 0) continue;
                                bool acc;
                                if (bmax) {
                                    const float dx = (float)(iax - (int)compact16(b)) * (float)hl +
                                                     ((float)cra[0] - (float)comrel[2 * (li + b)]);
                                    const float dy = (float)(iay - (int)compact16(b >> 1)) * (float)hl +
                                                     ((float)cra[1] - (float)comrel[2 * (li + b) + 1]);
                                    const float rb = ba + bmax[li + b];
                                    acc = theta2 * fmaf(dx, dx, dy * dy) > rb * rb;
                                } else {
                                    acc = mac_accept_fast<real>(iax - (int)compact16(b), iay - (int)compact16(b >> 1),
                                                                hl, thr2, cra, comrel + 2 * (li + b), ca, com64[li + b],
                                                                len, inv_theta, theta, variant);
                                }
                                if (acc && direct_cheaper(b)) acc = false;
                                bits |= (acc ? 1u : 0u) << j | 16u << j;
                                if (acc) nn++;
                                else nr++;
                            }
                        }
                        dec[4u * e + (uint32_t)(a & 3)] = (uint8_t)bits;
                    }
                } else if (fill && dec && !nn_ord) {
                    // fill pass from the count pass's decisions
                    uint32_t pos = nn_ptr[a];
                    const uint32_t rb0 = near_ptr[a];
                    for (uint32_t e = pe0; e < pe1; e++) {
                        const uint32_t bits = dec[4u * e + (uint32_t)(a & 3)];
                        if (bits == 0) continue;
                        const uint32_t bp = pnear_idx[e];
                        for (uint32_t j = 0; j < 4; j++) {
                            if (!(bits & (16u << j))) continue;
                            const uint32_t b = 4 * bp + j;
                            if (bits & (1u << j)) {
                                if (pos < nn_cap) nn_idx[pos] = b;
                                else atomicOr(ovf, 1u);
                                pos++;
                            } else {
                                if (rb0 + nr < near_cap) near_idx[rb0 + nr] = b;
                                else atomicOr(ovf, 1u);
                                nr++;
                            }
                        }
                    }
                } else if (!fill) {
                    visit([&](uint32_t, bool acc, int) {
                        if (acc) nn++;
                        else nr++;
                    });
                } else {
                    uint32_t start[5] = {nn_ptr[a], 0, 0, 0, 0};
                    if (nn_ord) {
                        uint32_t cnt[5] = {0, 0, 0, 0, 0};
                        visit([&](uint32_t, bool acc, int o) {
                            if (acc) cnt[o]++;
                        });
#pragma unroll
                        for (int o = 1; o < 5; o++) start[o] = start[o - 1] + cnt[o - 1];
                    }
                    const uint32_t rb0 = near_ptr[a];
                    visit([&](uint32_t b, bool acc, int o) {
                        if (acc) {
                            const uint32_t pos = start[o]++;
                            if (pos < nn_cap) {
                                nn_idx[pos] = b;
                                if (nn_ord) nn_ord[pos] = (uint8_t)o;
                            } else {
                                atomicOr(ovf, 1u);
                            }
                        } else {
                            if (rb0 + nr < near_cap) near_idx[rb0 + nr] = b;
                            else atomicOr(ovf, 1u);
                            nr++;
                        }
                    });
                }
            }
        }
        if (!fill) {
            nn_cnt[a] = nn;
            near_cnt[a] = nr;
        }
    }
}

// Coarse levels (few sink nodes, long candidate lists per node): one warp per
// non-empty node, the lanes taking the candidates (parent near entry e, child
// j) in order 32 at a time; ballots count them and place each accepted /
// opened entry at its rank, so the lists equal the one-thread form's entry for
// entry.  FP32 order-p path without per-pair orders; l >= 1.
__global__ void __launch_bounds__(128) k_lists_warp(int l, double inv_theta, double theta, int variant, float hl,
                                                    const uint32_t* __restrict__ count,
                                                    const double2* __restrict__ com64, const float* __restrict__ comrel,
                                                    const double* __restrict__ bblen,
                                                    const uint32_t* __restrict__ pnear_ptr,
                                                    const uint32_t* __restrict__ pnear_idx, uint32_t pcap,
                                                    uint32_t* __restrict__ nn_cnt, uint32_t* __restrict__ near_cnt,
                                                    const uint32_t* __restrict__ nn_ptr, uint32_t* __restrict__ nn_idx,
                                                    uint32_t nn_cap, const uint32_t* __restrict__ near_ptr,
                                                    uint32_t* __restrict__ near_idx, uint32_t near_cap,
                                                    uint32_t* __restrict__ ovf, int fill,
                                                    const uint32_t* __restrict__ act,
                                                    const uint32_t* __restrict__ act_pos,
                                                    const float* __restrict__ bmax, float theta2, uint32_t p2p_cut)
{
    const uint32_t np = 1u << (2 * (l - 1));
    const uint32_t li = level_index(l);
    const int64_t nl = (int64_t)1 << (2 * l);
    const int lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t k1 = act_pos[li + nl];
    const uint32_t wstride = gridDim.x * (blockDim.x >> 5);
    for (uint32_t k = act_pos[li] + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < k1; k += wstride) {
        const int64_t a = (int64_t)act[k] - li;
        const double2 ca = com64[li + a];
        const double len = bblen[li + a];
        const float thr = (float)((len + len) * inv_theta);
        const float thr2 = thr * thr;
        const int iax = (int)compact16((uint32_t)a), iay = (int)compact16((uint32_t)a >> 1);
        const float cra[2] = {comrel[2 * (li + a)], comrel[2 * (li + a) + 1]};
        const float ba = bmax ? bmax[li + a] : 0.f;
        const uint32_t ca_n = p2p_cut ? count[li + a] : 0u;
        const uint32_t p = (uint32_t)(a >> 2);
        const uint32_t pe0 = pnear_ptr[p], pe1 = pnear_ptr[p + 1] < pcap ? pnear_ptr[p + 1] : pcap;
        const uint32_t ncand = 4u * (pe1 > pe0 ? pe1 - pe0 : 0u);
        uint32_t nn = 0, nr = 0;
        const uint32_t nb0 = fill ? nn_ptr[a] : 0u, rb0 = fill ? near_ptr[a] : 0u;
        for (uint32_t c0 = 0; c0 < ncand; c0 += 32) {
            const uint32_t c = c0 + lane;
            bool valid = false, acc = false;
            uint32_t b = 0;
            if (c < ncand) {
                const uint32_t bp = pnear_idx[pe0 + (c >> 2)];
                b = 4 * bp + (c & 3);
                if (bp < np && count[li + b] != 0) {
                    valid = true;
                    if (bmax) {
                        const float dx = (float)(iax - (int)compact16(b)) * hl + (cra[0] - comrel[2 * (li + b)]);
                        const float dy = (float)(iay - (int)compact16(b >> 1)) * hl + (cra[1] - comrel[2 * (li + b) + 1]);
                        const float rb = ba + bmax[li + b];
                        acc = theta2 * fmaf(dx, dx, dy * dy) > rb * rb;
                    } else {
                        acc = mac_accept_fast<float>(iax - (int)compact16(b), iay - (int)compact16(b >> 1), hl, thr2,
                                                     cra, comrel + 2 * (li + b), ca, com64[li + b], len, inv_theta,
                                                     theta, variant);
                    }
                    if (acc && p2p_cut && ca_n * count[li + b] <= p2p_cut) acc = false;
                }
            }
            const uint32_t m_acc = __ballot_sync(0xffffffffu, valid && acc);
            const uint32_t m_rej = __ballot_sync(0xffffffffu, valid && !acc);
            if (fill && valid) {
                if (acc) {
                    const uint32_t pos = nb0 + nn + __popc(m_acc & lt);
                    if (pos < nn_cap) nn_idx[pos] = b;
                    else atomicOr(ovf, 1u);
                } else {
                    const uint32_t pos = rb0 + nr + __popc(m_rej & lt);
                    if (pos < near_cap) near_idx[pos] = b;
                    else atomicOr(ovf, 1u);
                }
            }
            nn += __popc(m_acc);
            nr += __popc(m_rej);
        }
        if (!fill && lane == 0) {
            nn_cnt[a] = nn;
            near_cnt[a] = nr;
        }
    }
}

// ---------------------------------------------------------------- controller
// The learned order controller replaces the MAC: every candidate pair (the
// non-empty children of a near pair of the parent level) is given to the MLP,
// which predicts log10 of the pair's relative far-field error at orders
// 4, 6, 8, 10, 12; the pair is accepted at the lowest order whose prediction
// is below log10(tau), and opened (near list) when none is.  Self pairs and
// pairs whose RMS spreads overlap ((s_A + s_B)/|R| >= 0.9) are opened without
// evaluating the network.
//
// The network runs on the tensor cores (ctrl_mma.cuh), one warp per 32
// candidates.  The count pass stores each candidate's decision (one byte per
// (parent near entry, child slot, sibling)); the fill pass only reads them.

// per-node features for the controller (all levels; empty nodes skipped)
__global__ void k_node_feat(int depth, double L, const uint32_t* __restrict__ count, const float* __restrict__ comrel,
                            const float* __restrict__ mu, int mu_stride, float4* __restrict__ nfeat, int64_t nnodes,
                            const uint32_t* __restrict__ act, const uint32_t* __restrict__ act_pos)
{
    const int64_t k1 = act_pos[nnodes];
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < k1; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = act[k];
        int l = 0;
        while (l < depth && i >= (int64_t)level_index(l + 1)) l++;
        const float ih = (float)((double)(1u << l) / L);
        float nf[kNodeFeat];
        node_features(mu + i * (int64_t)mu_stride, comrel[2 * i] * ih, comrel[2 * i + 1] * ih, nf);
        nfeat[2 * i] = make_float4(nf[0], nf[1], nf[2], nf[3]);
        nfeat[2 * i + 1] = make_float4(nf[4], nf[5], nf[6], nf[7]);
    }
}

// Count pass: one lane per node of level l >= 1 (warps of 32 consecutive
// nodes); lanes step through their candidates together and the warp runs the
// network whenever one of its lanes needs it.  dec[16 e + 4 j + (a & 3)] holds
// the decision for child j of parent near entry e: order bucket or kOpen.
__global__ void __launch_bounds__(32 * ctrl::kWarps) k_lists_ctrl_count(
    int l, float hl, float c_over_h2, const uint32_t* __restrict__ count, const float* __restrict__ comrel,
    const float4* __restrict__ nfeat, const uint32_t* __restrict__ pnear_ptr, const uint32_t* __restrict__ pnear_idx,
    uint32_t pcap, uint32_t* __restrict__ nn_cnt, uint32_t* __restrict__ near_cnt, uint8_t* __restrict__ dec,
    const float* __restrict__ wctrl, float log_tau, const uint32_t* __restrict__ act,
    const uint32_t* __restrict__ act_pos)
{
    __shared__ __align__(16) ctrl::Smem S;
    ctrl::load_weights(S, wctrl, wctrl + TC_MLP_NPARAM, wctrl + TC_MLP_NPARAM + TC_MLP_IN);
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t np = 1u << (2 * (l - 1));
    const uint32_t li = level_index(l);
    const int64_t nl = (int64_t)1 << (2 * l);
    const float ih = 1.0f / hl;
    const int64_t nwarps = (int64_t)gridDim.x * ctrl::kWarps;
    // lanes take consecutive non-empty nodes of the level (the counts of the
    // empty ones are zeroed by the caller)
    const int64_t k0 = act_pos[li], k1 = act_pos[li + nl];
    for (int64_t base = k0 + ((int64_t)blockIdx.x * ctrl::kWarps + wid) * 32; base < k1; base += nwarps * 32) {
        const bool valid = base + lane < k1;
        const int64_t a = valid ? (int64_t)act[base + lane] - li : 0;
        bool active = valid;
        uint32_t e = 0, e1 = 0, j = 0, nn = 0, nr = 0;
        int iax = 0, iay = 0;
        float cax = 0.f, cay = 0.f;
        float nfA[kNodeFeat];
        if (active) {
            const uint32_t p = (uint32_t)(a >> 2);
            e = pnear_ptr[p];
            e1 = pnear_ptr[p + 1] < pcap ? pnear_ptr[p + 1] : pcap;
            iax = (int)compact16((uint32_t)a);
            iay = (int)compact16((uint32_t)a >> 1);
            cax = comrel[2 * (li + a)] * ih;
            cay = comrel[2 * (li + a) + 1] * ih;
            const float4 n0 = nfeat[2 * (li + a)], n1 = nfeat[2 * (li + a) + 1];
            nfA[0] = n0.x, nfA[1] = n0.y, nfA[2] = n0.z, nfA[3] = n0.w;
            nfA[4] = n1.x, nfA[5] = n1.y, nfA[6] = n1.z, nfA[7] = n1.w;
        }
        while (__any_sync(0xffffffffu, active)) {
            // this lane's next non-empty candidate
            bool have = false;
            uint32_t b = 0, slot = 0;
            while (active) {
                if (e >= e1) {
                    active = false;
                    break;
                }
                const uint32_t bp = pnear_idx[e];
                const uint32_t jj = j, ee = e;
                if (++j == 4) {
                    j = 0;
                    e++;
                }
                if (bp >= np) continue;  // only after an overflowed parent level
                b = 4 * bp + jj;
                if (count[li + b] == 0) continue;
                slot = 16u * ee + 4u * jj + (uint32_t)(a & 3);
                have = true;
                break;
            }
            float f[TC_MLP_IN];
            bool use = false;
            if (have && b != (uint32_t)a) {
                const float cbx = comrel[2 * (li + b)] * ih, cby = comrel[2 * (li + b) + 1] * ih;
                const float Rx = (float)(iax - (int)compact16(b)) + (cax - cbx);
                const float Ry = (float)(iay - (int)compact16(b >> 1)) + (cay - cby);
                const float4 n0 = nfeat[2 * (li + b)], n1 = nfeat[2 * (li + b) + 1];
                const float nfB[kNodeFeat] = {n0.x, n0.y, n0.z, n0.w, n1.x, n1.y, n1.z, n1.w};
                pair_features_nf(Rx, Ry, nfA, nfB, c_over_h2, l, f);
                use = f[4] < 0.9f;
            }
            int d = -1;
            if (__any_sync(0xffffffffu, use)) {
                float y[TC_MLP_OUT];
                ctrl::warp_mlp(S, wid, lane, f, use, y);
                if (use)
                    for (int o = TC_MLP_OUT - 1; o >= 0; o--)
                        if (y[o] <= log_tau) d = o;
            }
            if (have) {
                dec[slot] = d >= 0 ? (uint8_t)d : ctrl::kOpen;
                if (d >= 0) nn++;
                else nr++;
            }
        }
        if (valid) {
            nn_cnt[a] = nn;
            near_cnt[a] = nr;
        }
    }
}

// Fill pass: one thread per node; the decisions of the count pass.  Each
// node's accepted entries are written grouped by order bucket (ascending), so
// that the M2L launch of one bucket reads one contiguous range per node.
__global__ void k_lists_ctrl_fill(int l, const uint32_t* __restrict__ count, const uint32_t* __restrict__ pnear_ptr,
                                  const uint32_t* __restrict__ pnear_idx, uint32_t pcap, const uint8_t* __restrict__ dec,
                                  const uint32_t* __restrict__ nn_ptr, uint32_t* __restrict__ nn_idx,
                                  uint8_t* __restrict__ nn_ord, uint32_t nn_cap, const uint32_t* __restrict__ near_ptr,
                                  uint32_t* __restrict__ near_idx, uint32_t near_cap, uint32_t* __restrict__ ovf,
                                  const uint32_t* __restrict__ act, const uint32_t* __restrict__ act_pos)
{
    const uint32_t np = 1u << (2 * (l - 1));
    const uint32_t li = level_index(l);
    const int64_t nl = (int64_t)1 << (2 * l);
    const int64_t k1 = act_pos[li + nl];
    for (int64_t k = act_pos[li] + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < k1;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = (int64_t)act[k] - li;
        const uint32_t p = (uint32_t)(a >> 2);
        const uint32_t pe0 = pnear_ptr[p];
        const uint32_t pe1 = pnear_ptr[p + 1] < pcap ? pnear_ptr[p + 1] : pcap;
        uint32_t start[TC_MLP_OUT] = {0, 0, 0, 0, 0};
        for (uint32_t e = pe0; e < pe1; e++) {
            const uint32_t bp = pnear_idx[e];
            if (bp >= np) continue;
            for (uint32_t j = 0; j < 4; j++) {
                if (count[li + 4 * bp + j] == 0) continue;
                const uint8_t d = dec[16u * e + 4u * j + (uint32_t)(a & 3)];
                if (d < TC_MLP_OUT) start[d]++;
            }
        }
        uint32_t run = nn_ptr[a];
        for (int o = 0; o < TC_MLP_OUT; o++) {
            const uint32_t c = start[o];
            start[o] = run;
            run += c;
        }
        uint32_t nr = near_ptr[a];
        for (uint32_t e = pe0; e < pe1; e++) {
            const uint32_t bp = pnear_idx[e];
            if (bp >= np) continue;
            for (uint32_t j = 0; j < 4; j++) {
                const uint32_t b = 4 * bp + j;
                if (count[li + b] == 0) continue;
                const uint8_t d = dec[16u * e + 4u * j + (uint32_t)(a & 3)];
                if (d < TC_MLP_OUT) {
                    const uint32_t pos = start[d]++;
                    if (pos < nn_cap) {
                        nn_idx[pos] = b;
                        nn_ord[pos] = d;
                    } else {
                        atomicOr(ovf, 1u);
                    }
                } else {
                    if (nr < near_cap) near_idx[nr] = b;
                    else atomicOr(ovf, 1u);
                    nr++;
                }
            }
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

// Sizes the list pools for a fast (capacity-based) build ahead of a stream
// capture, where no allocation may happen.  The pools' contents are not kept.
int prepare_nosync(Handle& h)
{
    const Lists& L = h.lists;
    if (L.caps_depth != h.depth || (int64_t)L.nn_cap.size() != h.depth + 1) {
        tc_set_error("no-sync list build needs the capacities of an earlier build at this depth");
        return TC_ERR_STATE;
    }
    int64_t words = 0;
    for (int l = 0; l <= h.depth; l++) words += (int64_t)L.nn_cap[l] + L.near_cap[l];
    int rc;
    if ((rc = ensure(h.idx_pool, (size_t)words * 4 + 64))) return rc;
    if ((h.adapt || h.ctrl_on) && (rc = ensure(h.ord_pool, h.idx_pool.bytes / 4 + 64))) return rc;
    // per-candidate decisions (controller: 16 bytes per parent near entry; MAC lists: 4), sized for the widest
    // parent level
    uint32_t pmax = 0;
    for (int l = 0; l < h.depth; l++) pmax = L.near_cap[l] > pmax ? L.near_cap[l] : pmax;
    if ((rc = ensure(h.dec, (size_t)pmax * (h.ctrl_on ? 16 : 4) + 64))) return rc;
    return TC_OK;
}

int build_lists(Handle& h)
{
    cudaStream_t s = h.stream;
    const int depth = h.depth;
    Lists& L = h.lists;
    if (!h.nosync || (int64_t)L.nn_total.size() != depth + 1) {
        // a no-sync (captured) build keeps the totals of the last exact or fast build
        L.nn_total.assign(depth + 1, 0);
        L.near_total.assign(depth + 1, 0);
    }
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
        (rc = ensure(h.tmp, (radix_tmp_words(h.n) > 2 * scan_tmp_words(nleaf) ? radix_tmp_words(h.n)
                                                                               : 2 * scan_tmp_words(nleaf)) * 4)))
        return rc;
    uint32_t* ptr = P<uint32_t>(h.ptr_pool);
    uint32_t* nn_cnt = P<uint32_t>(h.cnt_tmp);
    uint32_t* near_cnt = nn_cnt + nleaf;
    // order p (FP32): the tree build listed the non-empty nodes
    const uint32_t* act = h.cfg.order && h.cfg.precision != TC_PREC_FP64 ? P<uint32_t>(h.act) : nullptr;
    const uint32_t* act_pos = act ? P<uint32_t>(h.act_pos) : nullptr;
    const float* bmax = act && h.mac == TC_MAC_BMAX ? P<float>(h.bmax) : nullptr;
    // per-pair orders from the bounding-radius bound (orders 4..12 in steps of 2)
    const bool adapt = bmax && h.adapt;
    OrderRule rule{};
    for (int o = 0; o < 5; o++) {
        const int q = 4 + 2 * o;
        rule.t[o] = q < h.cfg.order
                        ? (float)std::pow(h.adapt_slack * std::pow(h.cfg.theta, h.cfg.order + 1), 2.0 / (q + 1))
                        : 3.0e38f;
    }
    const double inv_theta = 1.0 / h.cfg.theta;
    uint32_t* ovf_flag = P<uint32_t>(h.err) + 1;
    auto launch = [&](int l, const uint32_t* pnp, const uint32_t* pni, uint32_t pcap, uint32_t* nnc, uint32_t* nrc,
                      const uint32_t* nnp, uint32_t* nni, uint32_t nncap, const uint32_t* nrp, uint32_t* nri,
                      uint32_t nrcap, int fill) -> int {
        const int64_t nl = (int64_t)1 << (2 * l);
        const double hl = h.L / (double)(1u << l);
        if (h.ctrl_on && l > 0) {
            if (!fill) {
                int rc2 = ensure(h.dec, (size_t)pcap * 16 + 64);
                if (rc2) return rc2;
                k_lists_ctrl_count<<<grid_for(nl, 32 * ctrl::kWarps, sm_count() * 16), 32 * ctrl::kWarps, 0, s>>>(
                    l, (float)hl, (float)(h.ctrl_c / (hl * hl)), P<uint32_t>(h.count), P<float>(h.comrel),
                    P<float4>(h.nfeat), pnp, pni, pcap, nnc, nrc, P<uint8_t>(h.dec), P<float>(h.ctrl_w),
                    h.ctrl_log_tau, act, act_pos);
            } else {
                // nni points into the index pool; the order of entry i sits at byte i of the order pool
                uint8_t* ordp = P<uint8_t>(h.ord_pool) + (nni - P<uint32_t>(h.idx_pool));
                k_lists_ctrl_fill<<<grid_for(nl, 128), 128, 0, s>>>(l, P<uint32_t>(h.count), pnp, pni, pcap,
                                                                    P<uint8_t>(h.dec), nnp, nni, ordp, nncap, nrp,
                                                                    nri, nrcap, ovf_flag, act, act_pos);
            }
        } else if (h.cfg.precision == TC_PREC_FP64) {
            k_lists<double><<<grid_for(nl, 128), 128, 0, s>>>(l, inv_theta, h.cfg.theta, h.variant, hl,
                                                             P<uint32_t>(h.count),
                                                             P<double2>(h.com64), P<double>(h.comrel),
                                                             P<double>(h.bblen), pnp, pni, pcap, nnc, nrc, nnp, nni,
                                                             nncap, nrp, nri, nrcap, ovf_flag, fill, nullptr, nullptr, nullptr,
                                                             0.f, nullptr, rule, nullptr, 0u);
        } else {
            // the count pass keeps its decisions for the fill pass (one byte per parent near entry and
            // sibling slot)
            if (!fill && l > 0 && !adapt) {
                int rc2 = ensure(h.dec, (size_t)pcap * 4 + 64);
                if (rc2) return rc2;
            }
            if (act && !adapt && l > 0 && nl <= kListsWarpLevelNodes) {
                k_lists_warp<<<grid_for(nl * 32, 128), 128, 0, s>>>(
                    l, inv_theta, h.cfg.theta, h.variant, (float)hl, P<uint32_t>(h.count), P<double2>(h.com64),
                    P<float>(h.comrel), P<double>(h.bblen), pnp, pni, pcap, nnc, nrc, nnp, nni, nncap, nrp, nri, nrcap,
                    ovf_flag, fill, act, act_pos, bmax, (float)(h.cfg.theta * h.cfg.theta),
                    l == depth ? h.p2p_cut : 0u);
                return 0;
            }
            k_lists<float><<<grid_for(nl, 128), 128, 0, s>>>(l, inv_theta, h.cfg.theta, h.variant, (float)hl,
                                                            P<uint32_t>(h.count),
                                                            P<double2>(h.com64), P<float>(h.comrel),
                                                            P<double>(h.bblen), pnp, pni, pcap, nnc, nrc, nnp, nni,
                                                            nncap, nrp, nri, nrcap, ovf_flag, fill, act, act_pos, bmax,
                                                            (float)(h.cfg.theta * h.cfg.theta),
                                                            adapt && fill ? P<uint8_t>(h.ord_pool) +
                                                                                (nni - P<uint32_t>(h.idx_pool))
                                                                          : nullptr,
                                                            rule, l > 0 && !adapt ? P<uint8_t>(h.dec) : nullptr,
                                                            act && l == depth ? h.p2p_cut : 0u);
        }
        return 0;
    };
    if (h.ctrl_on) {
        if (!act) {
            tc_set_error("controller: needs the order-p FP32 tree");
            return TC_ERR_STATE;
        }
        if (h.mu_stride < 45) {  // the features read multipoles up to order 8
            tc_set_error("controller: the handle's multipoles are below order 8");
            return TC_ERR_STATE;
        }
        if ((rc = ensure(h.nfeat, (size_t)h.nnodes * 32))) return rc;
        k_node_feat<<<grid_for(h.nnodes, 256), 256, 0, s>>>(depth, h.L, P<uint32_t>(h.count), P<float>(h.comrel),
                                                             P<float>(h.mu), h.mu_stride, P<float4>(h.nfeat),
                                                             h.nnodes, act, act_pos);
        h.launches++;
    }
    uint32_t* ovf = P<uint32_t>(h.err) + 1;
    TC_CUDA_TRY(cudaMemsetAsync(ovf, 0, 4, s));
    // Fast mode: per-level regions sized from the last exact totals (x1.25),
    // no host round trip between levels; one synchronisation at the end
    // verifies that no level overflowed, else the exact mode reruns.
    const bool fast = L.caps_depth == depth && (int64_t)L.nn_cap.size() == depth + 1;
    if (h.nosync && !fast) {
        tc_set_error("no-sync list build needs the capacities of an earlier build at this depth");
        return TC_ERR_STATE;
    }
    if (fast) {
        int64_t words = 0;
        for (int l = 0; l <= depth; l++) {
            L.nn_idx_off[l] = words;
            words += L.nn_cap[l];
            L.near_idx_off[l] = words;
            words += L.near_cap[l];
        }
        if ((rc = ensure(h.idx_pool, (size_t)words * 4 + 64))) return rc;
        if ((h.ctrl_on || adapt) && (rc = ensure(h.ord_pool, h.idx_pool.bytes / 4 + 64))) return rc;
        for (int l = 0; l <= depth; l++) {
            const int64_t nl = (int64_t)1 << (2 * l);
            const uint32_t* pnp = l ? ptr + L.near_ptr_off[l - 1] : nullptr;
            const uint32_t* pni = l ? P<uint32_t>(h.idx_pool) + L.near_idx_off[l - 1] : nullptr;
            const uint32_t pcap = l ? L.near_cap[l - 1] : 0u;
            if (act) {
                TC_CUDA_TRY(cudaMemsetAsync(nn_cnt, 0, nl * 4, s));
                TC_CUDA_TRY(cudaMemsetAsync(near_cnt, 0, nl * 4, s));
            }
            if ((rc = launch(l, pnp, pni, pcap, nn_cnt, near_cnt, nullptr, nullptr, 0, nullptr, nullptr, 0, 0)))
                return rc;
            uint32_t* nnp = ptr + L.nn_ptr_off[l];
            uint32_t* nrp = ptr + L.near_ptr_off[l];
            // a captured build cannot check capacities before the lists are read: its CSR pointers are
            // clamped to the capacities, so an overflowed level yields truncated lists (and the overflow
            // flag) instead of out-of-range reads
            if ((rc = exclusive_scan2_u32(nn_cnt, nnp, near_cnt, nrp, nl, P<uint32_t>(h.tmp), s,
                                          h.nosync ? L.nn_cap[l] : UINT32_MAX,
                                          h.nosync ? L.near_cap[l] : UINT32_MAX)))
                return rc;
            if ((rc = launch(l, pnp, pni, pcap, nullptr, nullptr, nnp, P<uint32_t>(h.idx_pool) + L.nn_idx_off[l],
                             L.nn_cap[l], nrp, P<uint32_t>(h.idx_pool) + L.near_idx_off[l], L.near_cap[l], 1)))
                return rc;
            h.launches += 2 + (nl <= 2048 ? 1 : 3);  // count, fill, scan
            // the levels so far are final: work that reads only them may start on another stream
            if (l == h.lists_event_level) TC_CUDA_TRY(cudaEventRecord(h.ev_lists, s));
        }
        if (h.nosync) {
            // captured step: the overflow flag lands in pinned memory for the caller to check
            TC_CUDA_TRY(cudaMemcpyAsync(h.h_words + 40, ovf, 4, cudaMemcpyDeviceToHost, s));
            TC_CUDA_TRY(cudaGetLastError());
            return TC_OK;
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
        if (act) {
            TC_CUDA_TRY(cudaMemsetAsync(nn_cnt, 0, nl * 4, s));
            TC_CUDA_TRY(cudaMemsetAsync(near_cnt, 0, nl * 4, s));
        }
        if ((rc = launch(l, pnp, pni, pcap, nn_cnt, near_cnt, nullptr, nullptr, 0, nullptr, nullptr, 0, 0))) return rc;
        uint32_t* nnp = ptr + L.nn_ptr_off[l];
        uint32_t* nrp = ptr + L.near_ptr_off[l];
        if ((rc = exclusive_scan2_u32(nn_cnt, nnp, near_cnt, nrp, nl, P<uint32_t>(h.tmp), s))) return rc;
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
        if ((h.ctrl_on || adapt) && h.ord_pool.bytes < h.idx_pool.bytes / 4 + 64) {
            Buf nb;
            if ((rc = ensure(nb, h.idx_pool.bytes / 4 + 64))) return rc;
            if (h.ord_pool.p && L.nn_idx_off[l] > 0)
                TC_CUDA_TRY(cudaMemcpyAsync(nb.p, h.ord_pool.p, L.nn_idx_off[l], cudaMemcpyDeviceToDevice, s));
            TC_CUDA_TRY(cudaStreamSynchronize(s));
            release(h.ord_pool);
            h.ord_pool = nb;
        }
        pni = l ? P<uint32_t>(h.idx_pool) + L.near_idx_off[l - 1] : nullptr;
        if ((rc = launch(l, pnp, pni, pcap, nullptr, nullptr, nnp, P<uint32_t>(h.idx_pool) + L.nn_idx_off[l],
                         L.nn_total[l], nrp, P<uint32_t>(h.idx_pool) + L.near_idx_off[l], L.near_total[l], 1)))
            return rc;
        h.launches += 2 + (nl <= 2048 ? 1 : 3);  // count, fill, scan
    }
    // capacities for the next calls
    L.nn_cap.resize(depth + 1);
    L.near_cap.resize(depth + 1);
    for (int l = 0; l <= depth; l++) {
        L.nn_cap[l] = (uint32_t)(L.nn_total[l] + (int64_t)(L.nn_total[l] * h.cap_slack) + 256);
        L.near_cap[l] = (uint32_t)(L.near_total[l] + (int64_t)(L.near_total[l] * h.cap_slack) + 256);
    }
    L.caps_depth = depth;
    TC_CUDA_TRY(cudaGetLastError());
    return record(h, 3);
}

}  // namespace tc
