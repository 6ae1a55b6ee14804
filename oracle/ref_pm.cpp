// Test infrastructure only: a C-ABI entry around the reference's particle-mesh
// (FFT-interpolation) t-SNE repulsion solver NBodySolverPM
// (src/nbodysolvers/cpu/nBodySolverPM.h:93-1039), compiled from the reference
// sources by oracle/Makefile.ref into oracle/_ref/libref_oracle.so together
// with oracle/fftw_stub.cpp (the four FFTW functions it calls).  Used to pin the
// C restatement (orc_pm in oracle/treecode_oracle.c) and to generate golden
// fixtures.  Nothing in the product links it.
#define INDEX_TRACKER
#define GLM_ENABLE_EXPERIMENTAL
#include <cstdint>
#include <vector>

#include "nbodysolvers/cpu/nBodySolverPM.h"

extern "C" {

// NBodySolverPM::solveNbody on n points (input order): derivative (the
// repulsive gradient, -dC) and the returned pair sum.  n_interp, cell_size and
// min_intervals are the constructor's arguments (tsne.h:116 passes 4,
// cell_size, 4).
int ref_pm(int n_interp, double cell_size, int min_intervals, int64_t n, const double* pos_xy, double* grad,
           double* total)
{
    std::vector<TsnePoint2D> pts(n);
    for (int64_t i = 0; i < n; i++) {
        pts[i].position = glm::dvec2(pos_xy[2 * i], pos_xy[2 * i + 1]);
        pts[i].derivative = glm::dvec2(0.0);
        pts[i].ID = (int)i;
    }
    Eigen::SparseMatrix<double> P((Eigen::Index)n, (Eigen::Index)n);  // the attractive term is not computed here
    NBodySolverPM<TsnePoint2D> s(P, pts, n_interp, cell_size, min_intervals);
    double tot = 0.0;
    s.solveNbody(tot, pts);
    for (int64_t i = 0; i < n; i++) {
        grad[2 * i] = pts[i].derivative.x;
        grad[2 * i + 1] = pts[i].derivative.y;
    }
    if (total) *total = tot;
    return 0;
}

}  // extern "C"
