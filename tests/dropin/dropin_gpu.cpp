// TEST INFRASTRUCTURE: runs the drop-in adaptor GpuTreeSolver<TsnePoint2D>
// through the NBodySolver<TsnePoint2D>* interface the reference's drivers hold
// (TSNE::nBodySolvers), on points read from a file:
//   dropin_gpu <in.bin> <out.bin> <max_children> <theta>
// in.bin: int64 n, then n x (x, y) doubles; out.bin: for the returned (Morton)
// order, n x (ID int32), n x (x, y), n x (dx, dy) doubles, the pair sum, and
// the number of node-box vertices of level -1.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <vector>

#include "nbody_interface.hpp"
#include "gpu_tree_solver.hpp"

int main(int argc, char** argv)
{
    if (argc != 5) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int64_t n = 0;
    if (std::fread(&n, 8, 1, f) != 1 || n <= 0) return 2;
    std::vector<double> xy(2 * n);
    if (std::fread(xy.data(), 8, 2 * n, f) != (size_t)(2 * n)) return 2;
    std::fclose(f);
    std::vector<TsnePoint2D> pts(n);
    glm::dvec2 mn(1e300, 1e300), mx(-1e300, -1e300);
    for (int64_t i = 0; i < n; i++) {
        pts[i].position = glm::dvec2(xy[2 * i], xy[2 * i + 1]);
        pts[i].ID = (int)i;
        mn.x = xy[2 * i] < mn.x ? xy[2 * i] : mn.x;
        mn.y = xy[2 * i + 1] < mn.y ? xy[2 * i + 1] : mn.y;
        mx.x = xy[2 * i] > mx.x ? xy[2 * i] : mx.x;
        mx.y = xy[2 * i + 1] > mx.y ? xy[2 * i + 1] : mx.y;
    }
    const int max_children = std::atoi(argv[3]);
    const double theta = std::atof(argv[4]);
    NBodySolver<TsnePoint2D>* s = new GpuTreeSolver<TsnePoint2D>(TC_KERNEL_TSNE, max_children, -1, theta, 0,
                                                                 1e-3, TC_PREC_FP64);
    double total = 0.0;
    int64_t nverts = 0;
    try {
        s->updateTree(pts, mn, mx);
        s->solveNbody(total, pts);
        nverts = (int64_t)s->getNodesBufferData(-1).size();
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    delete s;
    FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 2;
    for (auto& p : pts) std::fwrite(&p.ID, 4, 1, o);
    for (auto& p : pts) std::fwrite(&p.position, 8, 2, o);
    for (auto& p : pts) std::fwrite(&p.derivative, 8, 2, o);
    std::fwrite(&total, 8, 1, o);
    std::fwrite(&nverts, 8, 1, o);
    std::fclose(o);
    return 0;
}
