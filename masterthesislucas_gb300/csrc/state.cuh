// Device-resident state of one solver handle (the GB300 counterpart of the
// reference's NodeFMM_MORTON_2D vector plus the particle buffer it sorts).
//
// HBM layout (structure of arrays, everything sized once and reused):
//   particles, Morton order    codes u32, perm u32 (input index = reference ID),
//                              pos64 double2 (bit-exact tree build),
//                              prel real2 (position relative to its leaf's cell
//                              centre, the compute copy for P2P/M2P/L2P)
//   nodes, level-dense         count u32, first u32, com64 double2, m0 double,
//   (levelIndex[l] + i)        m2 double3 (xx, xy, yy), bbc double2, bblen double
//                              comrel real2 (COM - ideal cell centre), m0r real,
//                              m2t real3 (M2 / M0), loc real[9] local expansion
//   interaction lists          per level: NN (accepted M2L partners) and near
//                              (partners to refine / leaf partners), CSR u32
#pragma once

#include <vector>

#include "common.cuh"

namespace tc {

// local expansion layout (9 unique coefficients of C1, C2, C3)
enum { L_C1X = 0, L_C1Y, L_C2XX, L_C2XY, L_C2YY, L_C3XXX, L_C3XXY, L_C3XYY, L_C3YYY, L_NCOEF };

struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
};

struct Lists {
    // per level l (0..depth): CSR over the 4^l nodes of the level (dense index)
    std::vector<uint32_t> nn_total, near_total;  // host copies of the totals
    std::vector<int64_t> nn_ptr_off, near_ptr_off;   // word offsets into ptr pool
    std::vector<int64_t> nn_idx_off, near_idx_off;   // word offsets into idx pool
    std::vector<uint32_t> nn_cap, near_cap;          // region sizes of the fast build
    int caps_depth = -1;
};

struct Handle {
    tc_config cfg;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // host-buffer entry points: copies that overlap the kernels run on copy_stream (created on first use);
    // ev_tree marks the sorted records, ev_grad the caller's gradient on the device, which the order-p solve
    // waits for before its near-field kernel adds to it (wait_grad)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_tree = nullptr, ev_grad = nullptr;
    bool wait_grad = false;
    // order-p solves: the near field on near_stream beside the far field on far_stream (higher priority),
    // both forked by ev_fork and joined by ev_join / ev_far before the L2P; the near field's FP32 forces
    // in nearf (sorted order)
#ifndef TC_NEAR_OVERLAP_DEFAULT
#define TC_NEAR_OVERLAP_DEFAULT 1
#endif
    bool near_overlap = TC_NEAR_OVERLAP_DEFAULT;
    cudaStream_t near_stream = nullptr, far_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_far = nullptr;
    // the update's multipoles on near_stream beside the list build (ev_mu marks them done); build_tree
    // leaves them out while split_mu is set
    bool split_mu = false;
    cudaEvent_t ev_mu = nullptr;
    // also on that side stream: the near field's work-item tables (items_ready; their own scratch, items_cnt
    // and items_tmp, since the list build uses cnt_tmp and tmp meanwhile) and, in a captured step, the far
    // field's coarse levels once their lists are built (coarse_ready; ev_lists marks list level
    // lists_event_level built).  The next update clears both flags.
    bool items_ready = false, coarse_ready = false;
    int lists_event_level = -1;
    cudaEvent_t ev_lists = nullptr;
    Buf items_cnt, items_tmp;
    Buf nearf;
    int depth = -1;
    int64_t n = 0;
    int64_t nnodes = 0;
    double minx = 0, miny = 0, L = 0;
    bool tree_ready = false;
    int launches = 0;   // kernels launched by the last call

    // particles
    Buf codes, perm, alt_keys, alt_vals, pos_in, pos64, prel, grad_acc;
    // nodes
    Buf count, first, com64, m0, m2, bbc, bblen, comrel, m0r, m2t, loc, locfin, chunk, zwork, zloc, mu;
    // lists
    Buf ptr_pool, idx_pool, cnt_tmp, lstat, ord_pool, nfeat, dec;
    // order-p path: leaves above kLeafSmall particles ([0] count, then indices)
    Buf bigleaf;
    Buf chunk_leaf;  // near-field work item -> its leaf (order-p solve)
    // order p: the non-empty nodes of every level in Morton order (act) and the
    // exclusive scan of non-emptiness over all nodes (act_pos); level l owns
    // act[act_pos[li] .. act_pos[li + 4^l])
    Buf act, act_pos;
    // order p: per node, the largest distance of its particles from its COM
    // (an upper bound for internal nodes), FP32
    Buf bmax;
    Buf celloff;  // FP32 gather: leaf cell centres relative to the box corner
    Buf mqueue;   // Morton codes: per-block queues of points for the FP64 path, then the per-block counts
    Buf diagpart;  // leapfrog diagnostics: per-block partial sums
    // learned order controller (order-p mode): weights + normalisation copy
    // no-sync mode (stream capture): no host round trips or stage events; the
    // outside-box and list-overflow flags are copied to pinned h_words[8], [40]
    // reference-order solver: 0 the symmetric FMM_SYM_MORTON, 1 the non-symmetric FMM_MORTON
    int variant = 0;
    int mac = 0;  // TC_MAC_CELL or TC_MAC_BMAX (order p)
    // order p: TC_CENTRE_COM (expansions about each node's centre of mass) or TC_CENTRE_BOX (about its cell
    // centre; comrel is then zero and bmax the particles' distance from the cell centre)
    int centre = 0;
    // order p, box-centred: M2L on the tensor cores (m2l_tc.cuh) instead of the FP32 SIMT kernels
    bool m2l_tc = false;
    bool m2l_tc_all = false;  // every level on the tensor cores (else levels with few parents stay SIMT)
    Buf tc_ops;   // tensor-core M2L: BF16 hi/lo operators per level and offset
    Buf tc_mubf;  // tensor-core M2L: BF16 hi/lo multipole rows per non-empty node
    // order p with TC_MAC_BMAX: per-pair expansion order from the bound
    bool adapt = false;
    double adapt_slack = 0.0;
    // order p: accepted leaf pairs with at most this many particle pairs are evaluated by P2P
    uint32_t p2p_cut = 0;
    bool nosync = false;
    double cap_slack = 0.25;  // fast-mode list capacity: exact total * (1 + slack) + 256
    bool ctrl_on = false;
    float ctrl_log_tau = -4.f;
    double ctrl_c = 0.0;      // kernel constant c of u = r^2 + c
    Buf ctrl_w;
    int mu_stride = 0;        // floats per node of mu (kstride of the solve order)
    Lists lists;
    // scratch
    Buf tmp, err, zpart, dtotal, host_stage, sumtmp;
    Buf ids_dev;  // tc_update_tree: the caller's IDs in, permuted by the sort out
    // stage timing (CUDA events on the handle's stream) and interaction counters
    cudaGraphExec_t step_graph = nullptr;  // a captured update + solve (tc_step_capture)
    int graph_launches = 0;
    cudaEvent_t ev[12] = {};
    bool ev_ready = false;
    bool stage_split = false;  // the last solve recorded the order-p events (8-11)
    Buf counters;  // u64: p2p pairs, m2p, p2l (device)
    double* h_total = nullptr;     // pinned
    uint32_t* h_words = nullptr;   // pinned, 64 words
};

int ensure(Buf& b, size_t bytes);
void release(Buf& b);

// stage boundaries (index into Handle::ev), on the handle's stream unless
// noted: 0 update start, 1 sorted, 2 tree built, 3 lists built, 4 solve
// start, 5 far field done, 6 near field done (order p: L2P done), 7 solve
// done; order-p solves also: 8 / 9 near field start / done (near_stream),
// 10 L2P start, 11 far field start
int record(Handle& h, int i);
int record_on(Handle& h, int i, cudaStream_t s);
// the order-p near and far fields' streams and fork/join events (created on first use, never inside a capture)
int ensure_near_stream(Handle& h);

template <typename T>
inline T* P(const Buf& b) { return reinterpret_cast<T*>(b.p); }

// tree.cu
int build_tree(Handle& h, const double* d_pos, int64_t n, double minx, double miny, double maxx, double maxy);
// lists.cu
int build_lists(Handle& h);
// fmm.cu
int solve_fmm(Handle& h, double* d_grad, double* d_total, int accumulate, int scatter);
// fmm_p.cu (tc_config.order != 0)
int solve_fmm_order(Handle& h, double* d_grad, double* d_total, int accumulate, int scatter);
int build_multipoles(Handle& h);
// the order-p near field's work-item tables on the handle's stream (leaf counts only)
int near_items(Handle& h);
// the order-p far field's coarse levels (M2L and L2L of the levels of at most 4^8 nodes) on the handle's
// stream, for the fused fixed-order path (1, nothing queued, when no earlier solve sized its buffers);
// far_coarse_applies says whether the handle takes that path
bool far_coarse_applies(const Handle& h);
int build_far_coarse(Handle& h);
// the last level far_coarse covers
constexpr int kFarCoarseLevel = 8;
// order-p FP32 tree (tree_p.cu): the node records after the gather of the
// sorted particles
int build_records_p(Handle& h, double hleaf);
// particle-mesh t-SNE repulsion (pm.cu): gradient in input order and Z
int pm_solve_device(int n_interp, double cell_size, int min_intervals, const double* d_pos, int64_t n, double* d_grad,
                    double* d_total, cudaStream_t s);
int prepare_nosync(Handle& h);

}  // namespace tc

// the opaque handle of the C ABI
struct tc_handle {
    tc::Handle h;
};
