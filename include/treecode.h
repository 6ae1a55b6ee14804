/*
 * treecode.h -- C ABI of the GB300 2D tree-code library (libtreecode.so).
 *
 * Drop-in boundary for the per-step force/gradient call of the reference's
 * tree solvers.  The reference interface is the abstract class
 *
 *   template <class T> class NBodySolver {                       // src/nbodysolvers/cpu/nBodySolver.h:9-23
 *     int maxChildren; double theta; double cell_size;
 *     virtual void solveNbody(double& total, std::vector<T>& points) = 0;
 *     virtual void updateTree(std::vector<T>& points, glm::dvec2 minPos, glm::dvec2 maxPos) = 0;
 *     virtual std::vector<VertexPos2Col3> getNodesBufferData(int level) = 0;
 *   };
 *
 * implemented by NBodySolverFMM_SYM_MORTON<TsnePoint2D>
 * (src/nbodysolvers/cpu/nBodySolverFMM_SYM_MORTON.h:29-614).  A handle plays
 * the solver object; positions cross the boundary as interleaved (x, y)
 * doubles and the particle identity (TsnePoint2D::ID) as int32.
 *
 * Conventions: every entry point returns TC_OK (0) or a negative TC_ERR_*
 * status and never aborts; tc_last_error() describes the last failure of the
 * calling thread.  Host pointers are borrowed for the duration of the call;
 * device buffers belong to the handle.  A handle is not thread-safe and runs
 * on one CUDA stream (tc_config.stream, or one it creates).
 */
#ifndef TREECODE_H
#define TREECODE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TC_OK 0
#define TC_ERR_INVALID -1   /* bad argument or input (NaN, point outside box) */
#define TC_ERR_CUDA -2      /* CUDA runtime error                            */
#define TC_ERR_NOMEM -3     /* device allocation failed                      */
#define TC_ERR_STATE -4     /* call out of order (solve before update_tree)  */
#define TC_ERR_TIMEOUT -5   /* a bounded device wait gave up                 */

#define TC_KERNEL_TSNE 0     /* Student-t repulsion (TSNE_FMM_SYM_MORTON_*_Kernel) */
#define TC_KERNEL_GRAVITY 1  /* 2D Plummer-softened gravity                        */

#define TC_PREC_FP32 0  /* expansions and P2P in FP32 (tree build, MACs and Z in FP64) */
#define TC_PREC_FP64 1  /* everything in FP64 (parity diagnostics)                     */

typedef struct tc_handle tc_handle;

typedef struct tc_config {
    int kernel;        /* TC_KERNEL_*                                           */
    int max_children;  /* NBodySolver::maxChildren (leaf size for getDepth)     */
    int depth;         /* tree depth; < 0 selects getDepth(max_children, n)     */
    double theta;      /* NBodySolver::theta, opening criterion                 */
    double softening;  /* gravity softening length eps                          */
    int precision;     /* TC_PREC_*                                             */
    int device;        /* CUDA device ordinal                                   */
    void* stream;      /* cudaStream_t to run on, or NULL for a private stream  */
    int order;         /* 0: the reference's expansion (M0+M2 multipole, C1..C3
                          local, point-node MAC stage); p in {3,4,6,8,10,12}:
                          total-order-p Cartesian expansions about the COM,
                          direct P2P for non-accepted leaf pairs (FP32 only) */
} tc_config;

/* Defaults: t-SNE kernel, leaf 16, automatic depth, theta 0.5, FP32. */
int tc_config_init(tc_config* cfg);

/* Constructor of NBodySolverFMM_SYM_MORTON (nBodySolverFMM_SYM_MORTON.h:49-67). */
int tc_create(const tc_config* cfg, tc_handle** out);
int tc_destroy(tc_handle* h);

/* NBodySolver::theta is a public field the caller changes between iterations
 * (TSNE::setThetaForAll, src/nBodyInstances/tsne.h:245-252).               */
int tc_set_theta(tc_handle* h, double theta);

/* Solver variant at the reference's expansion order (tc_config.order 0):
 * TC_VARIANT_SYM       NBodySolverFMM_SYM_MORTON (the default),
 * TC_VARIANT_MORTON    NBodySolverFMM_MORTON (src/nbodysolvers/cpu/
 *                      nBodySolverFMM_MORTON.h:28-505): ordered (sink,
 *                      source) traversal with the MAC (L_A + L_B)/|dcom| <
 *                      theta, node-node kernels into the sink only, and at
 *                      the leaves M2P (L_T/|x - com_T| < theta) or P2P for
 *                      every sink point (traverseBHMP, :199-232).
 * Takes effect at the next tc_update_tree.                                 */
#define TC_VARIANT_SYM 0
#define TC_VARIANT_MORTON 1
int tc_set_variant(tc_handle* h, int variant);

/* Opening criterion of an order-p handle (no counterpart in the reference):
 * TC_MAC_CELL  the reference's (L_A + L_B)/theta < |com_A - com_B| with L the
 *              cell sizes (the default);
 * TC_MAC_BMAX  (b_A + b_B)/theta < |com_A - com_B| with b the largest
 *              distance of a node's particles from its centre of mass (the
 *              radius the Taylor expansions about the COM converge in), so
 *              nodes whose particles sit near their COM are accepted sooner.
 * Takes effect at the next tc_update_tree.                                 */
#define TC_MAC_CELL 0
#define TC_MAC_BMAX 1
int tc_set_mac(tc_handle* h, int mac);

/* Expansion centre of an order-p FP32 handle (no counterpart in the
 * reference, whose expansions are about each node's centre of mass):
 * TC_CENTRE_COM  multipoles and locals about each node's centre of mass (the
 *                default);
 * TC_CENTRE_BOX  about each node's cell centre.  Every same-level pair is then
 *                an integer multiple of the cell size apart, so the M2L
 *                operator of a pair depends only on its level and grid
 *                offset; TC_MAC_BMAX measures the particles' distance from
 *                the cell centre.
 * Takes effect at the next tc_update_tree.                                 */
#define TC_CENTRE_COM 0
#define TC_CENTRE_BOX 1
int tc_set_expansion_centre(tc_handle* h, int centre);

/* M2L engine of a box-centred order-p handle (no counterpart in the
 * reference, whose M2L is TSNE_FMM_SYM_MORTON_NN_Kernel,
 * nBodySolverFMM_SYM_MORTON.h:622-723, in FP64 on the CPU):
 * TC_M2L_SIMT    FP32 kernels, one sink node per thread or warp (default);
 * TC_M2L_TENSOR  the 5th-generation tensor cores: per level, tiles of 128
 *                sink nodes times the level's per-offset K x K operators in
 *                BF16 with a hi/lo split (three products, FP32 accumulation,
 *                about 16 significant bits).  Fixed order only; opening
 *                angles that reach list offsets beyond 15 cells (theta below
 *                about 0.2 with TC_MAC_BMAX) are rejected at tc_solve.  Its
 *                operators take (depth + 1) * (2R+1)^2 * 4 * K_pad^2 bytes
 *                and its BF16 multipole copy 4 * K_pad bytes per node.
 * Levels whose parents number fewer than 128 per SM keep the SIMT kernels
 * (a tile's offsets run in sequence, so a level needs tiles for every SM);
 * TC_M2L_TENSOR_ALL runs every level on the tensor cores.
 * Needs TC_CENTRE_BOX set first; setting TC_CENTRE_COM returns to SIMT.  */
#define TC_M2L_SIMT 0
#define TC_M2L_TENSOR 1
#define TC_M2L_TENSOR_ALL 2
int tc_set_m2l_engine(tc_handle* h, int engine);

/* Order-p solves run their near field (P2P) on a second, internal stream
 * beside the far field (M2L, L2L): it reads only the tree and its lists.  The
 * L2P, which adds the final local expansions to the near-field forces, waits
 * for both.  on = 0 runs the two in sequence on the handle's stream (the
 * results are identical either way).  Default on; tc_tsne_batch_create
 * turns it off for its systems (their graphs already run side by side).    */
int tc_set_near_overlap(tc_handle* h, int on);

/* Per-pair expansion order on a TC_MAC_BMAX handle of order p in {6, 8, 10,
 * 12} (no counterpart in the reference): an accepted pair with ratio
 * r = (b_A + b_B)/|com_A - com_B| < theta is evaluated at the lowest order
 * q in {4, 6, 8, 10, 12}, q <= p, with r^(q+1) <= slack * theta^(p+1) (slack
 * = 1 keeps every pair's truncation bound at the fixed-order one; smaller
 * values are more conservative); the multipoles and local expansions keep
 * order p.  slack <= 0 returns to order p for every pair.  Takes effect at
 * the next tc_update_tree.                                                 */
int tc_set_adaptive_order(tc_handle* h, double slack);

/* Order-p handles (no counterpart in the reference): at the leaf level an
 * accepted pair of leaves A, B with n_A * n_B <= max_pairs is evaluated by
 * direct P2P instead of an M2L (an order-p M2L costs about as much as 70
 * particle pairs; the direct sum is also exact).  0 (the default) turns it
 * off.  Takes effect at the next tc_update_tree.                           */
int tc_set_leaf_p2p(tc_handle* h, int max_pairs);

/* getDepth (nBodySolverFMM_SYM_MORTON.h:106-115), clamped at 0 for n < leaf. */
int tc_get_depth(int max_children, int64_t n, uint32_t* depth);
/* node count of the level-dense tree, initNodesSize (:117-151).             */
int tc_node_count(uint32_t depth, int64_t* count);

/* updateTree (nBodySolverFMM_SYM_MORTON.h:79-95).  pos_xy (n x 2, host) and
 * ids (n, host, may be NULL) are reordered in place into Morton order, as the
 * reference sorts its particle vector.  min_xy/max_xy are the caller's
 * bounding box (TSNE::updateMinMaxPos); every point must lie inside it.      */
int tc_update_tree(tc_handle* h, double* pos_xy, int32_t* ids, int64_t n, const double min_xy[2],
                   const double max_xy[2]);

/* solveNbody (nBodySolverFMM_SYM_MORTON.h:69-77).  Adds the repulsive force
 * (t-SNE: sum q_ij^2 (y_i - y_j), unnormalised; gravity: acceleration of unit
 * masses) into grad_xy (host, sorted order) and the kernel's pair sum into
 * *total (t-SNE: Z).  pos_xy must be the positions passed to the preceding
 * tc_update_tree, in the order it returned (it may be NULL).              */
int tc_solve(tc_handle* h, double* total, const double* pos_xy, double* grad_xy, int64_t n);

/* Device-resident variants (pointers are device memory on the handle's
 * device).  d_pos_xy is in the caller's order and is not modified; when
 * min_xy is NULL the bounding box is computed on the device.  Results of
 * tc_solve_device are written in Morton order, or scattered back to the
 * caller's order when scatter != 0; accumulate selects += over =.         */
int tc_update_tree_device(tc_handle* h, const double* d_pos_xy, int64_t n, const double* min_xy,
                          const double* max_xy);
int tc_solve_device(tc_handle* h, double* d_grad_xy, double* d_total, int accumulate, int scatter);

/* Reads back the tree of the last update: Morton codes, permutation (input
 * index of each sorted point), sorted positions, and 27 doubles per node in
 * the order BBcentre(2) BBlength firstChildIndex firstParticleIndex
 * particleIndexAmount centreOfMass(2) M0 M2(4) C1(2) C2(4) C3(8), the fields
 * of NodeFMM_MORTON_2D (src/trees/cpu/nodeFMM_MORTON_2D.h:8-25).  The C
 * fields hold the final local expansions of the last solve, after the L2L
 * pass, in the solve's precision.  Any pointer may be NULL.             */
int tc_get_tree(tc_handle* h, uint32_t* codes, int32_t* perm, double* pos_sorted, double* nodes);

/* Interaction-list statistics of the last update: per level the number of
 * accepted node pairs (directed) and near pairs.  Arrays of depth+1.    */
int tc_get_list_stats(tc_handle* h, uint32_t* nn_pairs, uint32_t* near_pairs);

/* getNodesBufferData (nBodySolverFMM_SYM_MORTON.h:97-104): boxes of the
 * non-empty nodes of one level (level < 0: all levels) as (cx, cy, length)
 * triples.  *count receives how many exist; at most cap are written.     */
int tc_get_node_boxes(tc_handle* h, int level, double* boxes, int64_t cap, int64_t* count);

/* Kernels launched by the last update/solve call on this handle. */
int tc_last_launch_count(tc_handle* h);

/* Device time of the stages of the last update + solve, in milliseconds,
 * from CUDA events: [0] Morton codes + radix sort, [1] leaf build + upward
 * pass, [2] interaction lists, [3] far field (M2L, L2L), [4] near field (P2P,
 * M2P, P2L; of an order-p solve, on its own stream and overlapping [3] unless
 * tc_set_near_overlap(h, 0)), [5] L2P of an order-p solve (0 otherwise: the
 * reference-order near field includes it), [6] Z reduction.  Synchronises. */
#define TC_NSTAGES 7
int tc_get_stage_times(tc_handle* h, double* ms);
/* Interaction counts of the last solve: [0] P2P pair evaluations, [1] M2P,
 * [2] P2L, [3] M2L (directed; each unordered reference pair counts twice). */
int tc_get_counters(tc_handle* h, uint64_t* counts);

/* ---------------------------------------------------------------- direct sums
 * NBodySolverNaive::solveNbody (src/nbodysolvers/cpu/nBodySolverNaive.h:53-112)
 * and the GPU naive step cudaTsneNaiveStepRep
 * (src/nbodysolvers/gpu/nBodySolverGpuNaive.cu:50-81): O(N^2) force on the
 * sink rows `rows` (NULL: all n points, then m is ignored) from all n points,
 * written (not accumulated) to grad_rows (m x 2); *total receives the pair
 * sum over those rows.  TC_PREC_FP64 is the error oracle of the tree code.  */
int tc_direct(int kernel, double softening, int precision, const double* pos_xy, int64_t n,
              const int64_t* rows, int64_t m, double* grad_rows, double* total);
int tc_direct_device(int kernel, double softening, int precision, const double* d_pos_xy, int64_t n,
                     const int64_t* d_rows, int64_t m, double* d_grad_rows, double* d_total, void* stream);

/* ---------------------------------------------------------------- affinities
 * The t-SNE P matrix that the reference reads from openTSNE's output
 * (MnistLoader.ipynb cell 14; CSR by TSNE::setupEfficientPmatrix,
 * src/nBodyInstances/tsne.h:462-520), built on the GPU.  All pointers are
 * device memory on the current device; stream may be NULL.
 *
 * tc_knn_device: the k nearest neighbours of each of the n rows of d_x
 * (n x dim FP32, row-major), self excluded, by squared distance summed over
 * the dimensions in order in FP32 (one fused multiply-add per dimension);
 * each row of d_dist / d_idx (n x k) ordered by (distance, index).
 * 1 <= k <= 128, k < n.                                                    */
int tc_knn_device(const float* d_x, int64_t n, int dim, int k, float* d_dist, int32_t* d_idx, void* stream);
/* tc_perplexity_device: per row, the Gaussian precision beta bisected (start
 * 1, doubled until bracketed, at most max_iter steps) until the entropy of
 * p_j = exp(-beta (d_j - d_0)) / s is within tol of log(perplexity); writes
 * p (n x k FP64).  exp and log are the library's own FP64 series.         */
int tc_perplexity_device(const float* d_dist, int64_t n, int k, double perplexity, int max_iter, double tol,
                         double* d_p, void* stream);
/* tc_symmetrize_device: (P + P^T) / (2N) as CSR with rows sorted and columns
 * sorted within each row: d_row_ptr (n + 1), d_col and d_val with capacity
 * 2 n k; *nnz receives the entry count (the call synchronises the stream).
 * Allocates its sort scratch from the stream's memory pool.               */
int tc_symmetrize_device(const int32_t* d_idx, const double* d_p, int64_t n, int k, uint32_t* d_row_ptr,
                         uint32_t* d_col, double* d_val, int64_t* nnz, void* stream);

/* Same result as tc_direct_device, but allocates no device memory at all.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc (a stream under CUDA-graph capture, a host framework that owns
 * all device memory, a loop that must not block in the allocator).  Its
 * partial sums use one static device array of TC_DIRECT_NOALLOC_SCRATCH
 * doubles (4 MiB) that every GPU loading this library keeps until exit.
 * Limits: m <= TC_DIRECT_NOALLOC_SCRATCH / 4 rows (larger m returns
 * TC_ERR_INVALID); d_rows NULL selects rows 0..m-1.  The first call
 * on a device looks up the array's device address (cudaGetSymbolAddress),
 * so make that first call before any stream capture.  All calls share the
 * array: calls that overlap on the GPU race and must be serialised.        */
#define TC_DIRECT_NOALLOC_SCRATCH (1 << 19)
int tc_direct_device_noalloc(int kernel, double softening, int precision, const double* d_pos_xy, int64_t n,
                             const int64_t* d_rows, int64_t m, double* d_grad_rows, double* d_total, void* stream);

/* ---------------------------------------------------------------- Barnes-Hut
 * NBodySolverBH::updateTree + solveNbody with the reference's QuadTree
 * (src/nbodysolvers/cpu/nBodySolverBH.h:33-116, src/trees/cpu/quadtree.h:29-172):
 * same root box, split rule, children order, float masses and monopole MAC
 * l/|x - com| < theta.  Forces (input order) and the pair sum are written,
 * not accumulated.  FP64 reproduces the reference's interaction set and
 * values to rounding; FP32 evaluates the same interactions in FP32.        */
int tc_bh_solve(int kernel, double softening, int max_children, double theta, int precision,
                const double* pos_xy, int64_t n, double* grad_xy, double* total);
int tc_bh_solve_device(int kernel, double softening, int max_children, double theta, int precision,
                       const double* d_pos_xy, int64_t n, double* d_grad_xy, double* d_total, void* stream);
/* NBodySolverBHMP + QuadTreeMultiPole (src/nbodysolvers/cpu/nBodySolverBHMP.h:
 * 17-135, src/trees/cpu/quadtreemultipole.h:31-289): the same tree with FP64
 * masses and a quadrupole per node; accepted nodes contribute monopole +
 * quadrupole (TSNEBHMPPNKernel, :97-126).  Arguments as tc_bh_solve.        */
int tc_bhmp_solve(int kernel, double softening, int max_children, double theta, int precision,
                  const double* pos_xy, int64_t n, double* grad_xy, double* total);
int tc_bhmp_solve_device(int kernel, double softening, int max_children, double theta, int precision,
                         const double* d_pos_xy, int64_t n, double* d_grad_xy, double* d_total, void* stream);

/* ---------------------------------------------------------------- particle mesh
 * NBodySolverPM::solveNbody (src/nbodysolvers/cpu/nBodySolverPM.h:274-305,
 * computeFftGradient :763-1039): the FFT-accelerated interpolation t-SNE
 * repulsion (FIt-SNE) in FP64.  Boxes of side about cell_size (at least
 * min_intervals per dimension) on the square [min, max]^2 of all coordinates
 * (min/max as the reference's single `if / else if` pass finds them),
 * n_interp (1..8) Lagrange nodes per box and dimension; the reference's TSNE
 * passes (4, cell_size, 4) (src/nBodyInstances/tsne.h:116).  grad_xy
 * (input order) is overwritten with the reference's derivative
 * (sum_j q_ij^2 (y_i - y_j)), *total with the pair sum over i != j of q_ij,
 * as the reference overwrites both.  Needs libcufft (loaded at the first
 * call).                                                                    */
int tc_pm_solve(int n_interp, double cell_size, int min_intervals, const double* pos_xy, int64_t n,
                double* grad_xy, double* total);
int tc_pm_solve_device(int n_interp, double cell_size, int min_intervals, const double* d_pos_xy, int64_t n,
                       double* d_grad_xy, double* d_total, void* stream);

/* ---------------------------------------------------------------- N-body time step
 * Kick-drift-kick leapfrog on a gravity handle.  The reference's N-body
 * scenes step kick-then-drift around their solver call (2D, commented out:
 * src/nBodyInstances/gravitysim.h:99-127; 3D: nbodySim.h:215-240); this is
 * the time-centred leapfrog form of that loop with the project's softened
 * 2D kernel and FP64 energy/momentum diagnostics.  Device arrays in
 * input order: positions, velocities and accelerations (n x 2 FP64, G = 1,
 * equal masses `mass`).  init != 0 first computes the acceleration at the
 * current positions (the first call); dt == 0 with init only evaluates.
 * d_diag (device, 4 doubles) receives {kinetic, potential, Px, Py} after the
 * step, summed in FP64 in a fixed order.  Asynchronous on the handle's stream. */
int tc_leapfrog_step(tc_handle* h, double* d_pos_xy, double* d_vel_xy, double* d_acc_xy, int64_t n, double dt,
                     double mass, int init, double* d_diag);

/* ---------------------------------------------------------------- order controller
 * No counterpart in the reference (its expansion order is fixed).  A 3-layer
 * MLP (16 pair features -> 64 -> 64 -> 5, ReLU; BF16 weights, FP32
 * accumulation) predicts log10 of the relative far-field force error of a
 * node pair at orders 4, 6, 8, 10, 12; training and inference run in this
 * library's own kernels.  Parameter layout: W1[64][16] b1[64] W2[64][64]
 * b2[64] W3[5][64] b3[5].  Device pointers: d_x (n x 16), d_t / d_y (n x 5). */
#define TC_MLP_IN 16
#define TC_MLP_HIDDEN 64
#define TC_MLP_OUT 5
#define TC_MLP_NPARAM 5573
typedef struct tc_mlp tc_mlp;
int tc_mlp_create(uint64_t seed, tc_mlp** out);
int tc_mlp_destroy(tc_mlp* m);
int tc_mlp_set_normalization(tc_mlp* m, const float* mean, const float* stdv);
int tc_mlp_get_params(tc_mlp* m, float* params, float* mean, float* stdv);
int tc_mlp_set_params(tc_mlp* m, const float* params);
/* mean-squared-error gradient of the whole set d_x/d_t (n <= 2^20), host out */
int tc_mlp_gradient(tc_mlp* m, const float* d_x, const float* d_t, int64_t n, float* grad, float* loss);
/* Adam on seeded random mini-batches of the set */
int tc_mlp_train(tc_mlp* m, const float* d_x, const float* d_t, int64_t n, int steps, int batch, float lr,
                 uint64_t seed, float* last_loss);
int tc_mlp_forward(tc_mlp* m, const float* d_x, int64_t n, float* d_y);
/* the same network as the list builder evaluates it: tensor-core BF16
 * inputs and hidden activations, FP32 accumulation                         */
int tc_mlp_forward_tc(tc_mlp* m, const float* d_x, int64_t n, float* d_y);

/* Training data from a solved order-12 handle: for node pairs d_pairs (n x 3:
 * level, sink index, source index within the level) the 16 features and
 * log10 of the relative error of the pair's far field at orders 4..12
 * against the direct sum over the source's particles.                    */
int tc_lc_pair_errors(tc_handle* h, const int32_t* d_pairs, int64_t n, float* d_feat, float* d_err);
/* Copy one level's interaction list (kind 0: accepted pairs, 1: near pairs)
 * of the last update: CSR pointers (4^level + 1) and entries (*total).
 * kind 2 (controller handles): the accepted pairs' order buckets 0..4
 * (orders 4, 6, 8, 10, 12), one byte each, into idx.                      */
int tc_get_list(tc_handle* h, int level, int kind, uint32_t* ptr, uint32_t* idx, int64_t* total);
/* Replace the MAC of an FP32 order-12 handle by the controller m: every
 * candidate pair is accepted at the lowest order in {4, 6, 8, 10, 12} whose
 * predicted relative error is <= tau, else opened.  The weights are copied
 * (later training of m does not change the handle); m == NULL switches back
 * to the MAC.  The next update_tree rebuilds the lists.                   */
int tc_set_controller(tc_handle* h, tc_mlp* m, double tau);

/* ---------------------------------------------------------------- t-SNE step
 * The TSNE class around the solver (src/nBodyInstances/tsne.h:42-563),
 * device resident.  P is the symmetric affinity matrix as CSR (rows and
 * columns sorted, as TSNE::setupEfficientPmatrix builds it, tsne.h:462-520);
 * values are stored as FP32.  y0 (n x 2) initialises both the current and the
 * previous embedding (TSNE::generateInitialPoints, tsne.h:522-562).         */
typedef struct tc_tsne tc_tsne;
int tc_tsne_create(const tc_config* cfg, int64_t n, const uint32_t* row_ptr, const uint32_t* col,
                   const double* val, const double* y0, tc_tsne** out);
int tc_tsne_destroy(tc_tsne* t);
int tc_tsne_set_theta(tc_tsne* t, double theta);
/* tree depth of the next steps (0..15); the reference derives it from N */
int tc_tsne_set_depth(tc_tsne* t, int depth);
/* The repulsion of the next steps: the tree solver of the handle's config
 * (TC_REPULSION_TREE, the default) or the particle-mesh solver with the
 * reference's TSNE settings (TC_REPULSION_PM: 4 nodes per box, boxes of side
 * cell_size, at least 4 per dimension; nBodySelect "PM", tsne.h:116, whose
 * cell_size TSNE::setCellSizeForAll changes).  Particle-mesh systems cannot
 * join a batch (their grid is sized on the host every step).              */
#define TC_REPULSION_TREE 0
#define TC_REPULSION_PM 1
int tc_tsne_set_repulsion(tc_tsne* t, int method, double cell_size);
/* One TSNE_buffers::timeStep (tsne_buffers.h:125-168): updateTree on the
 * current embedding, updateRepulsive (tsne.h:287-301), updateAttractive
 * (:356-381) with factor exag_code (the reference uses 16 for the first 250
 * iterations, then 4), updatePoints (:179-206) with the given momentum and
 * learning rate.  *z_out (may be NULL) receives the repulsive normaliser Z. */
int tc_tsne_step(tc_tsne* t, double exag_code, double momentum, double lr, double* z_out);
/* Current embedding, previous embedding and last gradient, in ID order.    */
int tc_tsne_get(tc_tsne* t, double* y, double* y_prev, double* grad);
int tc_tsne_last_launch_count(tc_tsne* t);

/* Batches: many independent embeddings (each its own tc_tsne, FP32, order
 * p > 0, created on one device and stepped only through the batch) advance
 * in lockstep, one CUDA graph launch per step.  Inside the graph every
 * system's tree is built over a fixed square box (its extent enlarged by
 * `margin` plus a look-ahead of its last displacement, refreshed when a
 * point leaves it) with the list capacities of its last exact build; after
 * each launch a system that left its box or overflowed a list is stepped
 * again uncaptured and its graphs are re-captured.  No counterpart in the
 * reference (one embedding per TSNE object).                              */
typedef struct tc_tsne_batch tc_tsne_batch;
int tc_tsne_batch_create(tc_tsne* const* systems, int count, double margin, tc_tsne_batch** out);
int tc_tsne_batch_destroy(tc_tsne_batch* b);
/* exag_code and momentum as tc_tsne_step; each system's learning rate is
 * lr_per_point * its n (the reference's N/15 at 1/15)                      */
int tc_tsne_batch_step(tc_tsne_batch* b, double exag_code, double momentum, double lr_per_point);
/* stats (8 values): {graph launches, captures, uncaptured re-steps, nodes
 * in the systems' phase-0 graphs, particles in the batch, kernels per step,
 * host microseconds in graph launches, host microseconds in re-steps}.     */
int tc_tsne_batch_stats(tc_tsne_batch* b, int64_t* stats);
/* enable == 0: the same steps (same boxes, same refresh rule) enqueued
 * uncaptured, one system after another; for checking the graph path.     */
int tc_tsne_batch_set_capture(tc_tsne_batch* b, int enable);
/* A whole force step (tc_update_tree_device over a fixed box + a fresh pair
 * sum + tc_solve_device) captured once as a CUDA graph on the handle's stream
 * and replayed by tc_step_launch with one launch and no host round trip.  No
 * counterpart in the reference.  The capture needs an earlier synchronous
 * tc_update_tree_device of the same n (its list sizes bound the captured
 * lists) and runs one ordinary solve first.  box: min x, min y, max x, max y
 * (host).  After a replay has been synchronised, tc_async_status(h) != 0
 * means the step is invalid (a point left the box or a list outgrew its
 * capacity): redo it with tc_update_tree_device + tc_solve_device and capture
 * again.  The graph keeps the pointers it was captured with.                */
int tc_step_capture(tc_handle* h, const double* d_pos_xy, int64_t n, const double* box, double* d_grad_xy,
                    double* d_total, int scatter);
int tc_step_launch(tc_handle* h);
/* After the stream of a no-sync (captured) update has been synchronised:
 * bit 0 a position lay outside the box, bit 1 a list level overflowed.    */
int tc_async_status(tc_handle* h);

const char* tc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
