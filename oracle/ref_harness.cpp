// Test infrastructure only: a C-ABI harness around the reference's own CPU
// tree solvers, compiled straight from the reference sources by
// oracle/Makefile.ref into oracle/_ref/libref_oracle.so.  It is used to pin the
// C restatement (oracle/treecode_oracle.c) and to generate the golden fixtures
// under tests/golden/.  Nothing in the product links it.
//
// Solvers driven (reference paths, relative to the reference project):
//   NBodySolverFMM_SYM_MORTON   src/nbodysolvers/cpu/nBodySolverFMM_SYM_MORTON.h:29-614
//   NBodySolverNaive            src/nbodysolvers/cpu/nBodySolverNaive.h:18-112
//   NBodySolverBH               src/nbodysolvers/cpu/nBodySolverBH.h:14-89
//   NBodySolverFMM_MORTON       src/nbodysolvers/cpu/nBodySolverFMM_MORTON.h:28-505
//   NBodySolverBHMP             src/nbodysolvers/cpu/nBodySolverBHMP.h:17-135
// The t-SNE kernels are the reference's own (TSNE_FMM_SYM_MORTON_*_Kernel,
// TSNEnaiveKernel, TSNEBH*Kernel, TSNEFMM_MORTON*Kernel).  The reference has no
// live gravity kernel; the gravity kernels below are this project's
// 2D Plummer-softened force, written in the reference's kernel slots with the
// same structure as the t-SNE ones (D1 = g, D2 = 2g', D3 = 4g'' of the radial
// factor g(s), s = r^2).
#define INDEX_TRACKER
#define GLM_ENABLE_EXPERIMENTAL
#include <cstdint>
#include <cmath>
#include <chrono>
#include <vector>

#include "nbodysolvers/cpu/nBodySolverFMM_SYM_MORTON.h"
#include "nbodysolvers/cpu/nBodySolverFMM_MORTON.h"
#include "nbodysolvers/cpu/nBodySolverNaive.h"
#include "nbodysolvers/cpu/nBodySolverBH.h"
#include "nbodysolvers/cpu/nBodySolverBHMP.h"

namespace {

double g_eps2 = 1e-6;  // softening^2 used by the gravity kernels

// radial factors of the softened gravity force F(R) = R * g(s), s = |R|^2
inline void grav_derivs(double s, double& D1, double& D2, double& D3, double& t)
{
    double u = s + g_eps2;
    double iu = 1.0 / u;
    double isq = 1.0 / std::sqrt(u);
    double g = -isq * iu;                 // -(u)^-3/2
    D1 = g;
    D2 = -3.0 * g * iu;                   // 2 g'  =  3 u^-5/2
    D3 = -5.0 * D2 * iu;                  // 4 g'' = -15 u^-7/2
    t = -isq;                             // pair potential
}

// C1 of a source node (mass MB0, second moment MB2) seen from offset R
inline void far_c1(const glm::dvec2& R, double MB0, const Fastor::Tensor<double, 2, 2>& MB2,
                   double D1, double D2, double D3, double out[2])
{
    Fastor::Tensor<double, 2, 2> M = (1.0 / MB0) * MB2;
    double s1 = M(0, 0) + M(1, 1);
    double s2 = R.x * R.x * M(0, 0) + R.x * R.y * M(0, 1) + R.y * R.x * M(1, 0) + R.y * R.y * M(1, 1);
    double s30 = R.x * M(0, 0) + R.y * M(0, 1);
    double s31 = R.x * M(1, 0) + R.y * M(1, 1);
    out[0] = MB0 * (R.x * (D1 + 0.5 * s1 * D2 + 0.5 * s2 * D3) + s30 * D2);
    out[1] = MB0 * (R.y * (D1 + 0.5 * s1 * D2 + 0.5 * s2 * D3) + s31 * D2);
}

inline void c2c3(const glm::dvec2& R, double scale, double D1, double D2, double D3,
                 Fastor::Tensor<double, 2, 2>& C2, Fastor::Tensor<double, 2, 2, 2>& C3)
{
    double r[2] = {R.x, R.y};
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
            C2(i, j) = scale * ((i == j ? D1 : 0.0) + r[i] * r[j] * D2);
            for (int k = 0; k < 2; k++) {
                double d = ((i == j) ? r[k] : 0.0) + ((i == k) ? r[j] : 0.0) + ((j == k) ? r[i] : 0.0);
                C3(i, j, k) = scale * (d * D2 + r[i] * r[j] * r[k] * D3);
            }
        }
}

void GRAV_SYM_NN(double& total, NodeFMM_MORTON_2D& A, NodeFMM_MORTON_2D& B)
{
    glm::dvec2 R = A.centreOfMass - B.centreOfMass;
    double D1, D2, D3, t;
    grav_derivs(R.x * R.x + R.y * R.y, D1, D2, D3, t);
    double c1[2];
    Fastor::Tensor<double, 2, 2> C2;
    Fastor::Tensor<double, 2, 2, 2> C3;
    far_c1(R, B.M0, B.M2, D1, D2, D3, c1);
    c2c3(R, A.M0 * B.M0, D1, D2, D3, C2, C3);
    A.C1(0) += c1[0]; A.C1(1) += c1[1];
    A.C2 += C2; A.C3 += C3;
    glm::dvec2 Rm = -R;
    far_c1(Rm, A.M0, A.M2, D1, D2, D3, c1);
    B.C1(0) += c1[0]; B.C1(1) += c1[1];
    B.C2 += C2; B.C3 += -C3;
    total += 2.0 * (A.M0 * B.M0) * t;
}

void GRAV_SYM_PN(double& total, TsnePoint2D& p, NodeFMM_MORTON_2D& B)
{
    glm::dvec2 R = p.position - B.centreOfMass;
    double D1, D2, D3, t;
    grav_derivs(R.x * R.x + R.y * R.y, D1, D2, D3, t);
    double c1[2];
    far_c1(R, B.M0, B.M2, D1, D2, D3, c1);
    p.derivative += glm::dvec2(c1[0], c1[1]);
    glm::dvec2 Rm = -R;
    Fastor::Tensor<double, 2, 2> C2;
    Fastor::Tensor<double, 2, 2, 2> C3;
    c2c3(Rm, B.M0, D1, D2, D3, C2, C3);
    B.C1(0) += Rm.x * D1; B.C1(1) += Rm.y * D1;
    B.C2 += C2; B.C3 += C3;
    total += 2.0 * B.M0 * t;
}

void GRAV_SYM_PP(double& total, TsnePoint2D& a, TsnePoint2D& b)
{
    glm::dvec2 R = a.position - b.position;
    double D1, D2, D3, t;
    grav_derivs(R.x * R.x + R.y * R.y, D1, D2, D3, t);
    a.derivative += D1 * R;
    b.derivative += D1 * (-R);
    total += 2.0 * t;
}

// gravity in the non-symmetric solver's slots (TSNEFMM_MORTON*Kernel layout,
// nBodySolverFMM_MORTON.h:513-683): sink side only, C2/C3 with the source mass
void GRAV_M_NN(double& total, NodeFMM_MORTON_2D& A, NodeFMM_MORTON_2D& B)
{
    glm::dvec2 R = A.centreOfMass - B.centreOfMass;
    double D1, D2, D3, t;
    grav_derivs(R.x * R.x + R.y * R.y, D1, D2, D3, t);
    total += (A.M0 * B.M0) * t;
    double c1[2];
    Fastor::Tensor<double, 2, 2> C2;
    Fastor::Tensor<double, 2, 2, 2> C3;
    far_c1(R, B.M0, B.M2, D1, D2, D3, c1);
    c2c3(R, B.M0, D1, D2, D3, C2, C3);
    A.C1(0) += c1[0]; A.C1(1) += c1[1];
    A.C2 += C2; A.C3 += C3;
}

void GRAV_M_PN(double& total, TsnePoint2D& p, NodeFMM_MORTON_2D& B)
{
    glm::dvec2 R = p.position - B.centreOfMass;
    double D1, D2, D3, t;
    grav_derivs(R.x * R.x + R.y * R.y, D1, D2, D3, t);
    total += B.M0 * t;
    double c1[2];
    far_c1(R, B.M0, B.M2, D1, D2, D3, c1);
    p.derivative += glm::dvec2(c1[0], c1[1]);
}

void GRAV_M_NP(double& total, NodeFMM_MORTON_2D& A, TsnePoint2D& p)
{
    glm::dvec2 R = A.centreOfMass - p.position;
    double D1, D2, D3, t;
    grav_derivs(R.x * R.x + R.y * R.y, D1, D2, D3, t);
    total += A.M0 * t;
    Fastor::Tensor<double, 2, 2> C2;
    Fastor::Tensor<double, 2, 2, 2> C3;
    c2c3(R, 1.0, D1, D2, D3, C2, C3);
    A.C1(0) += R.x * D1; A.C1(1) += R.y * D1;
    A.C2 += C2; A.C3 += C3;
}

void GRAV_M_PP(double& total, TsnePoint2D& a, TsnePoint2D& b)
{
    glm::dvec2 R = a.position - b.position;
    double D1, D2, D3, t;
    grav_derivs(R.x * R.x + R.y * R.y, D1, D2, D3, t);
    total += t;
    a.derivative += D1 * R;
}

// gravity in NBodySolverBHMP's point-node slot: C1 with the node's quadrupole
void GRAV_BHMP_PN(double& total, TsnePoint2D& p, QuadTreeMultiPole<TsnePoint2D>* node)
{
    glm::dvec2 R = p.position - node->centreOfMass;
    double D1, D2, D3, t;
    grav_derivs(R.x * R.x + R.y * R.y, D1, D2, D3, t);
    total += node->totalMass * t;
    double c1[2];
    far_c1(R, node->totalMass, node->quadrupole, D1, D2, D3, c1);
    p.derivative += glm::dvec2(c1[0], c1[1]);
}

void GRAV_NAIVE(double& total, TsnePoint2D& a, TsnePoint2D& b)
{
    glm::dvec2 R = a.position - b.position;
    double D1, D2, D3, t;
    grav_derivs(R.x * R.x + R.y * R.y, D1, D2, D3, t);
    total += t;
    a.derivative += D1 * R;
}

void GRAV_BH_PN(double& total, TsnePoint2D& p, QuadTree<TsnePoint2D>* node)
{
    glm::dvec2 R = p.position - node->centreOfMass;
    double D1, D2, D3, t;
    grav_derivs(R.x * R.x + R.y * R.y, D1, D2, D3, t);
    total += node->totalMass * t;
    p.derivative += node->totalMass * D1 * R;
}

std::vector<TsnePoint2D> make_points(int64_t n, const double* pos)
{
    std::vector<TsnePoint2D> pts(n);
    for (int64_t i = 0; i < n; i++)
        pts[i] = TsnePoint2D(glm::dvec2(pos[2 * i], pos[2 * i + 1]), glm::dvec2(0.0), 0, (int)i, 0u);
    return pts;
}

}  // namespace

#define REF_NODE_STRIDE 27

extern "C" {

int ref_node_stride(void) { return REF_NODE_STRIDE; }

unsigned ref_get_depth(int max_children, int n)
{
    return NBodySolverFMM_SYM_MORTON<TsnePoint2D>::getDepth(max_children, n);
}

// Runs updateTree + solveNbody of NBodySolverFMM_SYM_MORTON (kernel 0 = t-SNE,
// 1 = softened gravity).  Outputs are in the solver's (Morton-sorted) order.
// nodes (optional) receives REF_NODE_STRIDE doubles per node after the solve.
// times (optional) receives {updateTree seconds, solveNbody seconds}.
int ref_sym_fmm(int kernel, double eps, int max_children, int depth, double theta,
                int64_t n, const double* pos_xy, const double* minmax,
                uint32_t* codes, int32_t* ids, double* pos_sorted, double* grad,
                double* total, double* nodes, double* times, int symmetric)
{
    g_eps2 = eps * eps;
    std::vector<TsnePoint2D> pts = make_points(n, pos_xy);
    glm::dvec2 mn(minmax[0], minmax[1]), mx(minmax[2], minmax[3]);
    double tot = 0.0;
    std::vector<NodeFMM_MORTON_2D>* nv = nullptr;
    double t_build = 0.0, t_solve = 0.0;
    NBodySolverFMM_SYM_MORTON<TsnePoint2D>* sym = nullptr;
    NBodySolverFMM_MORTON<TsnePoint2D>* asym = nullptr;
    if (symmetric) {
        if (kernel == 0)
            sym = new NBodySolverFMM_SYM_MORTON<TsnePoint2D>(&TSNE_FMM_SYM_MORTON_NN_Kernel, &TSNE_FMM_SYM_MORTON_PN_Kernel,
                                                             &TSNE_FMM_SYM_MORTON_PP_Kernel, max_children, depth, theta);
        else
            sym = new NBodySolverFMM_SYM_MORTON<TsnePoint2D>(&GRAV_SYM_NN, &GRAV_SYM_PN, &GRAV_SYM_PP, max_children, depth, theta);
        auto t0 = std::chrono::steady_clock::now();
        sym->updateTree(pts, mn, mx);
        auto t1 = std::chrono::steady_clock::now();
        sym->solveNbody(tot, pts);
        auto t2 = std::chrono::steady_clock::now();
        t_build = std::chrono::duration<double>(t1 - t0).count();
        t_solve = std::chrono::duration<double>(t2 - t1).count();
        nv = &sym->nodes;
    } else {
        if (kernel == 0)
            asym = new NBodySolverFMM_MORTON<TsnePoint2D>(&TSNEFMM_MORTONNNKernel, &TSNEFMM_MORTONPNKernel,
                                                           &TSNEFMM_MORTONNPKernel, &TSNEFMM_MORTONPPKernel,
                                                           max_children, depth, theta);
        else
            asym = new NBodySolverFMM_MORTON<TsnePoint2D>(&GRAV_M_NN, &GRAV_M_PN, &GRAV_M_NP, &GRAV_M_PP,
                                                           max_children, depth, theta);
        auto t0 = std::chrono::steady_clock::now();
        asym->updateTree(pts, mn, mx);
        auto t1 = std::chrono::steady_clock::now();
        asym->solveNbody(tot, pts);
        auto t2 = std::chrono::steady_clock::now();
        t_build = std::chrono::duration<double>(t1 - t0).count();
        t_solve = std::chrono::duration<double>(t2 - t1).count();
        nv = &asym->nodes;
    }
    for (int64_t i = 0; i < n; i++) {
        if (codes) codes[i] = pts[i].morton_code;
        if (ids) ids[i] = pts[i].ID;
        if (pos_sorted) { pos_sorted[2 * i] = pts[i].position.x; pos_sorted[2 * i + 1] = pts[i].position.y; }
        if (grad) { grad[2 * i] = pts[i].derivative.x; grad[2 * i + 1] = pts[i].derivative.y; }
    }
    if (total) *total = tot;
    if (times) { times[0] = t_build; times[1] = t_solve; }
    if (nodes) {
        for (size_t k = 0; k < nv->size(); k++) {
            const NodeFMM_MORTON_2D& q = (*nv)[k];
            double* o = nodes + k * REF_NODE_STRIDE;
            o[0] = q.BBcentre.x; o[1] = q.BBcentre.y; o[2] = q.BBlength;
            o[3] = q.firstChildIndex; o[4] = q.firstParticleIndex; o[5] = q.particleIndexAmount;
            o[6] = q.centreOfMass.x; o[7] = q.centreOfMass.y; o[8] = q.M0;
            o[9] = q.M2(0, 0); o[10] = q.M2(0, 1); o[11] = q.M2(1, 0); o[12] = q.M2(1, 1);
            o[13] = q.C1(0); o[14] = q.C1(1);
            o[15] = q.C2(0, 0); o[16] = q.C2(0, 1); o[17] = q.C2(1, 0); o[18] = q.C2(1, 1);
            for (int i = 0; i < 2; i++)
                for (int j = 0; j < 2; j++)
                    for (int k2 = 0; k2 < 2; k2++) o[19 + i * 4 + j * 2 + k2] = q.C3(i, j, k2);
        }
    }
    delete sym;
    delete asym;
    return 0;
}

// NBodySolverNaive (FP64, hardware_concurrency() threads), input order.
int ref_naive(int kernel, double eps, int64_t n, const double* pos_xy, double* grad, double* total)
{
    g_eps2 = eps * eps;
    std::vector<TsnePoint2D> pts = make_points(n, pos_xy);
    NBodySolverNaive<TsnePoint2D> s(kernel == 0 ? &TSNEnaiveKernel : &GRAV_NAIVE);
    double tot = 0.0;
    s.solveNbody(tot, pts);
    for (int64_t i = 0; i < n; i++) { grad[2 * i] = pts[i].derivative.x; grad[2 * i + 1] = pts[i].derivative.y; }
    if (total) *total = tot;
    return 0;
}

// NBodySolverBH (pointer quadtree, monopole), input order.
int ref_bh(int kernel, double eps, int max_children, double theta, int64_t n, const double* pos_xy,
           double* grad, double* total, double* times)
{
    g_eps2 = eps * eps;
    std::vector<TsnePoint2D> pts = make_points(n, pos_xy);
    NBodySolverBH<TsnePoint2D> s(kernel == 0 ? &TSNEBHPNKernel : &GRAV_BH_PN,
                                 kernel == 0 ? &TSNEBHPPKernel : &GRAV_NAIVE, max_children, theta);
    double tot = 0.0;
    auto t0 = std::chrono::steady_clock::now();
    s.updateTree(pts, glm::dvec2(0.0), glm::dvec2(0.0));
    auto t1 = std::chrono::steady_clock::now();
    s.solveNbody(tot, pts);
    auto t2 = std::chrono::steady_clock::now();
    for (int64_t i = 0; i < n; i++) { grad[2 * i] = pts[i].derivative.x; grad[2 * i + 1] = pts[i].derivative.y; }
    if (total) *total = tot;
    if (times) {
        times[0] = std::chrono::duration<double>(t1 - t0).count();
        times[1] = std::chrono::duration<double>(t2 - t1).count();
    }
    return 0;
}

// NBodySolverBHMP (kernel 0 = t-SNE, 1 = softened gravity), input order.
int ref_bhmp(int kernel, double eps, int max_children, double theta, int64_t n, const double* pos_xy,
             double* grad, double* total)
{
    g_eps2 = eps * eps;
    std::vector<TsnePoint2D> pts = make_points(n, pos_xy);
    NBodySolverBHMP<TsnePoint2D> s(kernel == 0 ? &TSNEBHMPPNKernel : &GRAV_BHMP_PN,
                                   kernel == 0 ? &TSNEBHMPPPKernel : &GRAV_NAIVE, max_children, theta);
    double tot = 0.0;
    s.updateTree(pts, glm::dvec2(0.0), glm::dvec2(0.0));
    s.solveNbody(tot, pts);
    for (int64_t i = 0; i < n; i++) { grad[2 * i] = pts[i].derivative.x; grad[2 * i + 1] = pts[i].derivative.y; }
    if (total) *total = tot;
    return 0;
}

}  // extern "C"
