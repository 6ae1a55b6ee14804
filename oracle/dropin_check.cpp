// TEST INFRASTRUCTURE: proves the drop-in boundary.  Compiles the reference's
// own solver headers together with include/gpu_tree_solver.hpp, holds the GPU
// solver through the reference's NBodySolver<TsnePoint2D>* interface exactly as
// TSNE::nBodySolvers does (src/nBodyInstances/tsne.h:104-122), and, when run on
// a machine with a GPU, compares it with NBodySolverFMM_SYM_MORTON on the same
// points.  Built by oracle/Makefile.ref (target dropin) into oracle/_ref/.
#define INDEX_TRACKER
#define GLM_ENABLE_EXPERIMENTAL
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "nbodysolvers/cpu/nBodySolverFMM_SYM_MORTON.h"
#include "gpu_tree_solver.hpp"

int main()
{
    const int n = 20000;
    std::mt19937 gen(216308u);
    std::normal_distribution<double> dist(0.0, 3.0);
    std::vector<TsnePoint2D> a(n), b;
    for (int i = 0; i < n; i++) a[i] = TsnePoint2D(glm::dvec2(dist(gen), dist(gen)), glm::dvec2(0.0), 0, i, 0u);
    b = a;
    glm::dvec2 mn(1e300), mx(-1e300);
    for (auto& p : a) {
        mn = glm::min(mn, p.position);
        mx = glm::max(mx, p.position);
    }
    const unsigned depth = NBodySolverFMM_SYM_MORTON<TsnePoint2D>::getDepth(16, n);
    NBodySolver<TsnePoint2D>* ref = new NBodySolverFMM_SYM_MORTON<TsnePoint2D>(
        &TSNE_FMM_SYM_MORTON_NN_Kernel, &TSNE_FMM_SYM_MORTON_PN_Kernel, &TSNE_FMM_SYM_MORTON_PP_Kernel, 16, depth, 0.5);
    NBodySolver<TsnePoint2D>* gpu = new GpuTreeSolver<TsnePoint2D>(TC_KERNEL_TSNE, 16, (int)depth, 0.5);
    double ta = 0.0, tb = 0.0;
    ref->updateTree(a, mn, mx);
    ref->solveNbody(ta, a);
    gpu->updateTree(b, mn, mx);
    gpu->solveNbody(tb, b);
    double worst = 0.0;
    int order_mismatch = 0;
    for (int i = 0; i < n; i++) {
        if (a[i].ID != b[i].ID) order_mismatch++;
        glm::dvec2 d = a[i].derivative - b[i].derivative;
        worst = std::max(worst, glm::length(d) / glm::length(a[i].derivative));
    }
    std::printf("dropin: order mismatches %d, max rel force diff %.3e, total %.9e vs %.9e\n", order_mismatch, worst, ta, tb);
    delete ref;
    delete gpu;
    return (order_mismatch == 0 && worst < 1e-3 && std::fabs(ta - tb) < 1e-5 * std::fabs(ta)) ? 0 : 1;
}
