// TEST INFRASTRUCTURE: a minimal stand-in for the reference's solver interface,
// so that include/gpu_tree_solver.hpp can be compiled and run where the
// reference's sources are absent (the GPU machine).  It declares only what the
// adaptor uses, with the reference's names and signatures:
//   NBodySolver<T> with public maxChildren / theta and the virtual
//   updateTree / solveNbody / getNodesBufferData
//   (src/nbodysolvers/cpu/nBodySolver.h:9-23);
//   glm's dvec2 / vec2 / vec3 as plain value types;
//   VertexPos2Col3 (position + colour vertex);
//   a point with position, derivative and ID (src/particles/tsnePoint2D.h).
// The real interface is exercised by oracle/dropin_check.cpp against the
// reference's own headers where they exist.
#pragma once

#include <vector>

namespace glm {
struct dvec2 {
    double x = 0.0, y = 0.0;
    dvec2() = default;
    dvec2(double a, double b) : x(a), y(b) {}
};
struct vec2 {
    float x = 0.f, y = 0.f;
    vec2() = default;
    vec2(float a, float b) : x(a), y(b) {}
};
struct vec3 {
    float x = 0.f, y = 0.f, z = 0.f;
    vec3() = default;
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};
}  // namespace glm

struct VertexPos2Col3 {
    glm::vec2 pos;
    glm::vec3 col;
    VertexPos2Col3(glm::vec2 p, glm::vec3 c) : pos(p), col(c) {}
};

template <typename T>
class NBodySolver
{
public:
    virtual ~NBodySolver() = default;
    virtual void updateTree(std::vector<T>& points, glm::dvec2 minPos, glm::dvec2 maxPos) = 0;
    virtual void solveNbody(double& total, std::vector<T>& points) = 0;
    virtual std::vector<VertexPos2Col3> getNodesBufferData(int level) = 0;
    int maxChildren = 0;
    double theta = 0.0;
};

struct TsnePoint2D {
    glm::dvec2 position, derivative;
    int ID = 0;
};
