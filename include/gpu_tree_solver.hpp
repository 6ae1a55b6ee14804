// gpu_tree_solver.hpp -- drop-in NBodySolver for the reference's t-SNE and
// experiment drivers, backed by libtreecode.so (include/treecode.h).
//
// The reference's drivers hold their solvers as NBodySolver<T>*
// (src/nbodysolvers/cpu/nBodySolver.h:9-23; TSNE::nBodySolvers,
// src/nBodyInstances/tsne.h:104-122).  GpuTreeSolver<T> implements that
// interface for any point type with `glm::dvec2 position, derivative` and
// `int ID` (TsnePoint2D under INDEX_TRACKER, src/particles/tsnePoint2D.h:6-37):
//
//   updateTree(points, minPos, maxPos)  -> tc_update_tree: the vector is
//       reordered into Morton order in place, exactly as
//       NBodySolverFMM_SYM_MORTON::updateTree sorts it (records move whole);
//   solveNbody(total, points)           -> tc_solve: adds the force into
//       points[i].derivative and the pair sum into total;
//   getNodesBufferData(level)           -> tc_get_node_boxes, as line
//       segments in the reference's VertexPos2Col3 layout.
//
// Header-only; include it after the reference's nBodySolver.h and link with
// -ltreecode.  Errors are reported by throwing std::runtime_error (the
// reference's solvers have no error channel; this keeps failures visible).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "treecode.h"

template <typename T>
class GpuTreeSolver : public NBodySolver<T>
{
public:
    // kernel: TC_KERNEL_TSNE / TC_KERNEL_GRAVITY; depth < 0 selects getDepth
    // (max_children, n) like the reference's TSNE constructor (tsne.h:119-122);
    // order 0 is the reference's expansion, p > 0 the order-p expansion.
    GpuTreeSolver(int kernel, int max_children, int depth, double theta, int order = 0, double softening = 1e-3,
                  int precision = TC_PREC_FP32, int device = 0)
    {
        tc_config cfg;
        tc_config_init(&cfg);
        cfg.kernel = kernel;
        cfg.max_children = max_children;
        cfg.depth = depth;
        cfg.theta = theta;
        cfg.order = order;
        cfg.softening = softening;
        cfg.precision = precision;
        cfg.device = device;
        check(tc_create(&cfg, &h_));
        this->maxChildren = max_children;
        this->theta = theta;
        applied_theta_ = theta;
    }

    ~GpuTreeSolver() override { tc_destroy(h_); }

    GpuTreeSolver(const GpuTreeSolver&) = delete;
    GpuTreeSolver& operator=(const GpuTreeSolver&) = delete;

    void updateTree(std::vector<T>& points, glm::dvec2 minPos, glm::dvec2 maxPos) override
    {
        // the reference's drivers change the public theta field between
        // iterations (TSNE::setThetaForAll); pick it up here
        if (this->theta != applied_theta_) {
            check(tc_set_theta(h_, this->theta));
            applied_theta_ = this->theta;
        }
        const int64_t n = (int64_t)points.size();
        pos_.resize(2 * n);
        ids_.resize(n);
        for (int64_t i = 0; i < n; i++) {
            pos_[2 * i] = points[i].position.x;
            pos_[2 * i + 1] = points[i].position.y;
            ids_[i] = (int32_t)i;  // slot in the caller's vector
        }
        const double mn[2] = {minPos.x, minPos.y}, mx[2] = {maxPos.x, maxPos.y};
        check(tc_update_tree(h_, pos_.data(), ids_.data(), n, mn, mx));
        std::vector<T> sorted(points.size());
        for (int64_t k = 0; k < n; k++) sorted[k] = points[ids_[k]];
        points.swap(sorted);
    }

    void solveNbody(double& total, std::vector<T>& points) override
    {
        const int64_t n = (int64_t)points.size();
        grad_.assign(2 * n, 0.0);
        double t = 0.0;
        check(tc_solve(h_, &t, nullptr, grad_.data(), n));
        for (int64_t i = 0; i < n; i++) {
            points[i].derivative.x += grad_[2 * i];
            points[i].derivative.y += grad_[2 * i + 1];
        }
        total += t;
    }

    std::vector<VertexPos2Col3> getNodesBufferData(int level) override
    {
        int64_t count = 0;
        check(tc_get_node_boxes(h_, level, nullptr, 0, &count));
        std::vector<double> boxes(3 * count);
        check(tc_get_node_boxes(h_, level, boxes.data(), count, &count));
        std::vector<VertexPos2Col3> out;
        out.reserve(8 * count);
        const glm::vec3 col(1.0f, 1.0f, 1.0f);
        for (int64_t k = 0; k < count; k++) {
            const float cx = (float)boxes[3 * k], cy = (float)boxes[3 * k + 1], hl = 0.5f * (float)boxes[3 * k + 2];
            const glm::vec2 lo(cx - hl, cy - hl), hi(cx + hl, cy + hl);
            out.push_back(VertexPos2Col3(glm::vec2(lo.x, lo.y), col));
            out.push_back(VertexPos2Col3(glm::vec2(hi.x, lo.y), col));
            out.push_back(VertexPos2Col3(glm::vec2(lo.x, lo.y), col));
            out.push_back(VertexPos2Col3(glm::vec2(lo.x, hi.y), col));
            out.push_back(VertexPos2Col3(glm::vec2(lo.x, hi.y), col));
            out.push_back(VertexPos2Col3(glm::vec2(hi.x, hi.y), col));
            out.push_back(VertexPos2Col3(glm::vec2(hi.x, lo.y), col));
            out.push_back(VertexPos2Col3(glm::vec2(hi.x, hi.y), col));
        }
        return out;
    }

private:
    static void check(int rc)
    {
        if (rc != TC_OK) throw std::runtime_error(std::string("treecode: ") + tc_last_error());
    }

    tc_handle* h_ = nullptr;
    double applied_theta_ = 0.0;
    std::vector<double> pos_, grad_;
    std::vector<int32_t> ids_;
};
