// Scene and mesh loading for the command-line driver, in the reference's file formats:
//   scene: {"mesh_path", "dt", "viscosity", "total_time"}  (NavierStokesAssembly::init, include/assembly.h:885-935)
//          plus optional "steps" (exact step count) and "solver" ("fp64" | "mixed")
//   mesh:  {"elements", "nodes", "elementsCount", "velocityNodesCount", "pressureNodesCount", "elementSize",
//           "uDirichlet": [{"nodes", "u", "v"}], "pDirichlet": [{"nodes", "p"}]}   (FemGrid2D::loadJSON, cpp/grid.cpp:9-78)
#pragma once
#include <string>
#include <vector>

namespace nsfhost {

struct Scene {
    std::string meshPath;
    double dt = 0, viscosity = 0, totalTime = 0;
    int steps = -1;                     // -1: the reference rule, int(total_time / dt) - 1 steps
    std::string solver = "fp64";
    int nNodes = 0, nElements = 0, nPressure = 0;
    std::vector<float> xy;
    std::vector<int> elements;
    // Dirichlet data per listed occurrence, in file order, evaluated at the node (variables x, y; and t = 0 when
    // an expression uses t)
    std::vector<int> uNodes, pNodes;
    std::vector<double> gu, gv, gp;
    // the groups' expression strings and, per occurrence, the index of its u, v and p expression (for
    // nsf_sim_set_bc_expressions when the data depend on time)
    std::vector<std::string> expressions;
    std::vector<int> uExpr, vExpr, pExpr;
    bool timeDependent = false;

    int step_count() const;
};

// Throws std::runtime_error with the reference's messages ("Missing required param: dt", ...).
Scene load_scene(const std::string& scenePath);
void load_mesh(const std::string& meshPath, Scene& s);

// out_<timeStep>.json with keys p, timeStep, u, v (the keys exportSolution writes, include/assembly.h:953-978)
void write_solution(const std::string& folder, int timeStep, int nNodes, int nPressure, const double* uv,
                    const double* p);

// Reads an out_<t>.json back (uv = [u | v], p); returns its timeStep.  The reference has no reader for its own
// result files beyond the convergence-order estimate (cpp/main.cpp:53-61); this one resumes a run.
int read_solution(const std::string& path, int nNodes, int nPressure, std::vector<double>& uv,
                  std::vector<double>& p);

}  // namespace nsfhost
