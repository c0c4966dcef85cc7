#include "scene.h"

#include <cstdio>
#include <filesystem>
#include <fstream>
#include <stdexcept>

#include "expression.h"
#include "json.h"

namespace nsfhost {

int Scene::step_count() const {
    if (steps >= 0) return steps;
    // the reference computes steps = totalTime / dt in float and runs timeStep = 1 .. steps-1
    const int s = (int)((float)totalTime / (float)dt);
    return s > 1 ? s - 1 : 0;
}

Scene load_scene(const std::string& scenePath) {
    const Json j = parse_json_file(scenePath);
    Scene s;
    if (!j["mesh_path"].is_string()) throw std::runtime_error("Missing path to mesh.");
    std::filesystem::path mp(j["mesh_path"].str);
    if (mp.is_relative()) mp = std::filesystem::path(scenePath).parent_path() / mp;
    s.meshPath = mp.lexically_normal().string();
    if (!j["dt"].is_number()) throw std::runtime_error("Missing required param: dt");
    if (!j["viscosity"].is_number()) throw std::runtime_error("Missing required param: viscosity");
    if (!j["total_time"].is_number()) throw std::runtime_error("Missing required param: total_time");
    s.dt = j["dt"].num;
    s.viscosity = j["viscosity"].num;
    s.totalTime = j["total_time"].num;
    if (j["steps"].is_number()) s.steps = (int)j["steps"].num;
    if (j["solver"].is_string()) s.solver = j["solver"].str;
    load_mesh(s.meshPath, s);
    return s;
}

void load_mesh(const std::string& meshPath, Scene& s) {
    const Json j = parse_json_file(meshPath);
    s.nElements = (int)j["elementsCount"].num;
    s.nNodes = (int)j["velocityNodesCount"].num;
    s.nPressure = (int)j["pressureNodesCount"].num;
    const int es = (int)j["elementSize"].num;
    if (es != 6) throw std::runtime_error("Only P2-P1 elements (elementSize 6) are supported");
    if (s.nNodes <= 0 || s.nPressure <= 0) throw std::runtime_error("mesh has no nodes");
    const Json& nodes = j["nodes"];
    const Json& els = j["elements"];
    if ((int)nodes.size() < s.nNodes || (int)els.size() < s.nElements)
        throw std::runtime_error("mesh arrays are shorter than the declared counts");
    s.xy.resize(2 * (size_t)s.nNodes);
    for (int i = 0; i < s.nNodes; ++i) {
        if (nodes[i].size() != 2) throw std::runtime_error("Expected 2D grid. All nodes must be of (x, y) pairs of size 2");
        s.xy[2 * i] = (float)nodes[i][0].num;
        s.xy[2 * i + 1] = (float)nodes[i][1].num;
    }
    s.elements.resize(6 * (size_t)s.nElements);
    for (int e = 0; e < s.nElements; ++e) {
        if ((int)els[e].size() != es) throw std::runtime_error("Mismatch between declared element size and actual element size");
        for (int k = 0; k < 6; ++k) s.elements[6 * (size_t)e + k] = (int)els[e][k].num;
    }
    const Json& ud = j["uDirichlet"];
    const Json& pd = j["pDirichlet"];
    // an expression that uses t makes the data time-dependent: evaluated here at t = 0, on the device per step
    auto index = [&](const std::string& e) {
        for (size_t i = 0; i < s.expressions.size(); ++i)
            if (s.expressions[i] == e) return (int)i;
        s.expressions.push_back(e);
        if (e.find('t') != std::string::npos) s.timeDependent = true;
        return (int)s.expressions.size() - 1;
    };
    auto vars_at = [&](int node) {
        std::map<char, double> v{{'x', (double)s.xy[2 * node]}, {'y', (double)s.xy[2 * node + 1]}};
        if (s.timeDependent) v['t'] = 0.0;
        return v;
    };
    for (size_t g = 0; g < ud.size(); ++g) index(ud[g]["u"].str), index(ud[g]["v"].str);
    for (size_t g = 0; g < pd.size(); ++g) index(pd[g]["p"].str);
    for (size_t g = 0; g < ud.size(); ++g) {
        const Expression u(ud[g]["u"].str), v(ud[g]["v"].str);
        const int iu = index(ud[g]["u"].str), iv = index(ud[g]["v"].str);
        const Json& nn = ud[g]["nodes"];
        for (size_t k = 0; k < nn.size(); ++k) {
            const int node = (int)nn[k].num;
            if (node < 0 || node >= s.nNodes) throw std::runtime_error("velocity Dirichlet node out of range");
            const auto vars = vars_at(node);
            s.uNodes.push_back(node);
            s.gu.push_back(u.evaluate(vars));
            s.gv.push_back(v.evaluate(vars));
            s.uExpr.push_back(iu);
            s.vExpr.push_back(iv);
        }
    }
    for (size_t g = 0; g < pd.size(); ++g) {
        const Expression p(pd[g]["p"].str);
        const int ip = index(pd[g]["p"].str);
        const Json& nn = pd[g]["nodes"];
        for (size_t k = 0; k < nn.size(); ++k) {
            const int node = (int)nn[k].num;
            if (node < 0 || node >= s.nPressure) throw std::runtime_error("pressure Dirichlet node out of range");
            s.pNodes.push_back(node);
            s.gp.push_back(p.evaluate(vars_at(node)));
            s.pExpr.push_back(ip);
        }
    }
}

void write_solution(const std::string& folder, int timeStep, int nNodes, int nPressure, const double* uv,
                    const double* p) {
    const std::string path = folder + "/out_" + std::to_string(timeStep) + ".json";
    std::ofstream f(path);
    if (!f) throw std::runtime_error("Failed to open file for writing the result: " + path);
    auto arr = [&](const char* key, const double* a, int n, bool last) {
        f << "    \"" << key << "\": [\n";
        for (int i = 0; i < n; ++i) f << "        " << json_number(a[i]) << (i + 1 < n ? ",\n" : "\n");
        f << "    ]" << (last ? "\n" : ",\n");
    };
    f << "{\n";
    arr("p", p, nPressure, false);
    f << "    \"timeStep\": " << timeStep << ",\n";
    arr("u", uv, nNodes, false);
    arr("v", uv + nNodes, nNodes, true);
    f << "}\n";
}

int read_solution(const std::string& path, int nNodes, int nPressure, std::vector<double>& uv,
                  std::vector<double>& p) {
    const Json j = parse_json_file(path);
    const Json &u = j["u"], &v = j["v"], &pp = j["p"];
    if ((int)u.size() != nNodes || (int)v.size() != nNodes || (int)pp.size() != nPressure)
        throw std::runtime_error("solution file " + path + " does not match the mesh's node counts");
    uv.assign(2 * (size_t)nNodes, 0.0);
    p.assign(nPressure, 0.0);
    for (int i = 0; i < nNodes; ++i) {
        uv[i] = u[i].num;
        uv[nNodes + i] = v[i].num;
    }
    for (int i = 0; i < nPressure; ++i) p[i] = pp[i].num;
    if (!j["timeStep"].is_number()) throw std::runtime_error("solution file " + path + " has no timeStep");
    return (int)j["timeStep"].num;
}

}  // namespace nsfhost
