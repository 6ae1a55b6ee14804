/*
 * TEST INFRASTRUCTURE -- NOT PART OF THE PRODUCT.
 *
 * Plain-C restatement of the reference's CPU tree-code path, used only as the
 * checker (tests/, the smoke check, and the CPU-baseline leg of bench.py).
 * Every routine cites the reference file:line it restates.  It is pinned
 * against the reference compiled from its own sources (oracle/Makefile.ref,
 * oracle/ref_harness.cpp) through the golden fixtures in tests/golden/.
 *
 * All arithmetic is FP64 in the reference's operation order; build with
 * -ffp-contract=off so results are identical on x86-64 and aarch64.
 */
#ifndef TREECODE_ORACLE_H
#define TREECODE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_KERNEL_TSNE = 0, ORC_KERNEL_GRAVITY = 1 };

/* NodeFMM_MORTON_2D (src/trees/cpu/nodeFMM_MORTON_2D.h:8-25), flattened.   */
typedef struct {
    double bb_c[2];        /* BBcentre                                     */
    double bb_len;         /* BBlength                                     */
    uint32_t first_child;  /* firstChildIndex (0 = leaf or empty)          */
    uint32_t first_part;   /* firstParticleIndex                           */
    uint32_t count;        /* particleIndexAmount                          */
    uint32_t pad;
    double com[2];         /* centreOfMass                                 */
    double m0;             /* M0                                           */
    double m2[4];          /* M2 (row-major 2x2)                           */
    double c1[2];          /* C1                                           */
    double c2[4];          /* C2 (row-major 2x2)                           */
    double c3[8];          /* C3 (i*4 + j*2 + k)                           */
} orc_node;

/* NBodySolverFMM_SYM_MORTON::getDepth (nBodySolverFMM_SYM_MORTON.h:106-115) */
uint32_t orc_get_depth(int max_children, int64_t n);
/* total node count of the level-dense tree, initNodesSize (:117-151)        */
int64_t orc_node_count(uint32_t depth);

/* createMortonCode + spread16 (:538-561).  pos is n x 2 (x,y).              */
void orc_morton_codes(int64_t n, const double* pos, const double min_xy[2],
                      const double max_xy[2], uint32_t* codes);

/* Stable sort of codes; perm[k] = input index of the k-th sorted point.
 * Stands in for boost integer_sort (:89), whose tie order is undefined.     */
void orc_sort_perm(int64_t n, const uint32_t* codes, int32_t* perm);

/* createLeafNodes + bottomUpNodeConstruction (:328-470) on Morton-sorted
 * positions.  nodes must hold orc_node_count(depth) entries; it is zeroed.  */
void orc_build_tree(uint32_t depth, int64_t n, const double* pos_sorted,
                    const double min_xy[2], const double max_xy[2], orc_node* nodes);

/* solveNbody (:69-77): traverse_SYM_NN (:154-270), traverse_SYM_PN
 * (:272-313), kernels NN/PN/PP (:622-836 for t-SNE; gravity is the project's
 * softened kernel in the same slots), root C2/C3 /= M0, applyForces
 * (:482-536).  grad (n x 2, sorted order) and *total are accumulated.      */
void orc_sym_fmm_solve(int kernel, double eps, uint32_t depth, double theta,
                       int64_t n, const double* pos_sorted, orc_node* nodes,
                       double* grad, double* total);

/* updateTree + solveNbody in one call (what the reference's caller does).
 * Outputs are in the sorted order; ids_sorted[k] = input index.            */
void orc_sym_fmm(int kernel, double eps, int max_children, int depth, double theta,
                 int64_t n, const double* pos, const double min_xy[2], const double max_xy[2],
                 uint32_t* codes_sorted, int32_t* ids_sorted, double* pos_sorted,
                 double* grad_sorted, double* total, orc_node* nodes /* may be NULL */);

/* NBodySolverFMM_MORTON (nBodySolverFMM_MORTON.h), the non-symmetric
 * variant: traverseFMM (:148-197) over ordered (sink, source) pairs with
 * the MAC (L_A + L_B)/|com_A - com_B| < theta, traverseBHMP/BHRMP
 * (:199-268), kernels NN/PN/NP/PP (:513-683; gravity as in the symmetric
 * solver), applyForces (:382-430).  Same tree build; arguments as
 * orc_sym_fmm / orc_sym_fmm_solve.                                         */
void orc_fmm_morton_solve(int kernel, double eps, double theta, const double* pos_sorted, orc_node* nodes,
                          double* grad, double* total);
void orc_fmm_morton(int kernel, double eps, int max_children, int depth, double theta,
                    int64_t n, const double* pos, const double min_xy[2], const double max_xy[2],
                    uint32_t* codes_sorted, int32_t* ids_sorted, double* pos_sorted,
                    double* grad_sorted, double* total, orc_node* nodes /* may be NULL */);

/* NBodySolverNaive::solveNbody + TSNEnaiveKernel (nBodySolverNaive.h:53-141):
 * FP64 O(N^2), input order, nthreads row partitions.  grad is overwritten. */
void orc_naive(int kernel, double eps, int64_t n, const double* pos, double* grad,
               double* total, int nthreads);

/* FP64 direct sum for a subset of sink particles (rows idx[0..m)).          */
void orc_direct_rows(int kernel, double eps, int64_t n, const double* pos, int64_t m,
                     const int64_t* idx, double* grad_rows, int nthreads);

/* NBodySolverBH + QuadTree (nBodySolverBH.h:33-116, quadtree.h:29-172).
 * grad is overwritten (input order), total overwritten.                    */
int orc_bh(int kernel, double eps, int max_children, double theta, int64_t n,
           const double* pos, double* grad, double* total);
/* NBodySolverBHMP + QuadTreeMultiPole (nBodySolverBHMP.h:17-135,
 * quadtreemultipole.h:31-289): Barnes-Hut with FP64 masses and a quadrupole
 * correction (the C1 of the FMM kernels) at accepted nodes.                 */
int orc_bhmp(int kernel, double eps, int max_children, double theta, int64_t n,
             const double* pos, double* grad, double* total);

/* NBodySolverPM::solveNbody (nBodySolverPM.h:274-305, computeFftGradient
 * :763-1039): FFT-accelerated interpolation of the t-SNE repulsion with p
 * Lagrange nodes per box and boxes of side about cell_size (at least
 * min_intervals per dimension).  grad (input order) = the reference's
 * derivative (-dC), *total = the pair sum excluding self pairs.             */
int orc_pm(int p, double cell_size, int min_intervals, int64_t n, const double* pos, double* grad,
           double* total);

/* TSNE::updateAttractive (tsne.h:356-381): grad[i] += exag * sum_j P_ij q_ij (y_j - y_i) */
void orc_tsne_attractive(int64_t n, const uint32_t* row_ptr, const uint32_t* col,
                         const double* val, const double* pos, double exag, double* grad);

/* One full t-SNE iteration as TSNE_buffers::timeStep composes it
 * (tsne.h:272-301 updateDerivative/updateRepulsive, :356-381 updateAttractive,
 * :179-206 updatePoints): y_next = y + lr*g + mom*(y - y_prev).  All arrays
 * are in ID order.  exag_code is the code's factor (16 early, 4 late in the
 * reference).  grad_out receives g, *z_out the repulsive normaliser.        */
void orc_tsne_step(int64_t n, const double* y, const double* y_prev,
                   const uint32_t* row_ptr, const uint32_t* col, const double* val,
                   int max_children, int depth, double theta, double exag_code,
                   double lr, double momentum, double* y_next, double* grad_out, double* z_out);

/* The t-SNE affinity matrix (openTSNE's PerplexityBasedNN restated, see
 * treecode_oracle.c): exact kNN with FP32 squared distances summed over the
 * dimensions in order (fmaf), neighbours ordered by (distance, index), self
 * excluded; dist/idx are n x k.                                             */
void orc_knn(int64_t n, int dim, const float* x, int k, float* dist, int32_t* idx);
/* FP64 exp and log from their series (range reduction by ln 2).            */
double orc_exp(double x);
double orc_log(double x);
/* Per-row bisection of the Gaussian bandwidth to the perplexity; p (n x k)
 * holds the row-normalised conditional probabilities.                     */
void orc_perplexity(int64_t n, int k, const float* dist, double perplexity, int max_iter, double tol, double* p);
/* (P + P^T) / (2N) as CSR with rows and columns sorted (setupEfficientPmatrix
 * layout); row_ptr n + 1, col/val capacity 2nk.  Returns nnz.              */
int64_t orc_symmetrize(int64_t n, int k, const int32_t* idx, const double* p, uint32_t* row_ptr, uint32_t* col,
                       double* val);

#ifdef __cplusplus
}
#endif
#endif
