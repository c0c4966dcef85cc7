// nsfem: the command-line driver, a drop-in for the reference executable (cpp/main.cpp:87-146).
//
//   nsfem -sceneFile=<scene.json> [-outPath=<dir>] [-numThreads=<n>] [-steps=<n>] [-solver=fp64|mixed]
//         [-device=<i>] [-tol=<eps>]
//
// Loads the scene and mesh (host, C++), then hands everything to the GPU through the C ABI: assembly, and the
// operator-split loop of NavierStokesAssembly::semiLagrangianSolve (include/assembly.h:1477-1557) with the
// fields resident on the device.  With -outPath, out_<step>.json is written after every step (exportSolution,
// include/assembly.h:953-978); the SVG/OpenCV plots are not produced.  -numThreads is accepted for
// compatibility; the host side here is single-threaded setup only.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "nsfem_gb300.h"
#include "scene.h"

namespace {

struct Param {
    const char* description;
    bool isInt;
    bool required;
};

const std::map<std::string, Param> kParams = {
    {"sceneFile", {"Path to the file describing the simulation", false, true}},
    {"numThreads", {"The number of threads which the simulator should use. All threads by default.", true, false}},
    {"outPath", {"Path to a folder where the resulting caches and images will be saved", false, false}},
    {"steps", {"Exact number of time steps (default: int(total_time/dt) - 1, as the reference)", true, false}},
    {"solver", {"Linear solver: fp64 (plain FP64 CG) or mixed (FP32 inner CG, FP64 refinement)", false, false}},
    {"device", {"CUDA device index", true, false}},
    {"tol", {"Relative residual of every CG solve (default 1e-8)", false, false}},
    {"resume", {"Continue from a result file out_<t>.json of an earlier run (steps t+1 .. steps)", false, false}},
};

void usage(FILE* f) {
    fprintf(f, "Supported options\n");
    for (const auto& kv : kParams)
        fprintf(f, "  -%s=<%s>%s  %s\n", kv.first.c_str(), kv.second.isInt ? "int" : "string",
                kv.second.required ? " (required)" : "", kv.second.description);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc == 2 && strcmp(argv[1], "-help") == 0) {
        usage(stdout);
        return 0;
    }
    std::map<std::string, std::string> args;
    for (int i = 1; i < argc; ++i) {
        const char* a = argv[i];
        const char* eq = strchr(a, '=');
        if (a[0] != '-' || !eq) {
            fprintf(stderr, "[Error] Malformed argument: %s\n", a);
            usage(stderr);
            return 1;
        }
        const std::string name(a + 1, eq);
        if (!kParams.count(name)) {
            fprintf(stderr, "[Error] Unknown parameter: %s\n", name.c_str());
            usage(stderr);
            return 1;
        }
        args[name] = eq + 1;
    }
    for (const auto& kv : kParams)
        if (kv.second.required && !args.count(kv.first)) {
            fprintf(stderr, "[Error] Missing required parameter: %s\n", kv.first.c_str());
            usage(stderr);
            return 1;
        }

    nsfhost::Scene scene;
    try {
        scene = nsfhost::load_scene(args["sceneFile"]);
    } catch (const std::exception& e) {
        fprintf(stderr, "[Error] %s\n", e.what());
        return 1;
    }
    if (args.count("steps")) scene.steps = atoi(args["steps"].c_str());
    if (args.count("solver")) scene.solver = args["solver"];
    const int device = args.count("device") ? atoi(args["device"].c_str()) : 0;
    const std::string outPath = args.count("outPath") ? args["outPath"] : "";
    const int steps = scene.step_count();

    printf("Begin solution using semi Lagrangian method\n");
    printf("Elements: %d\n", scene.nElements);
    printf("Velocity nodes: %d\n", scene.nNodes);
    printf("Pressure nodes: %d\n", scene.nPressure);
    printf("Total time: %f\n", scene.totalTime);
    printf("dt: %f\n", scene.dt);
    printf("Total steps: %d\n", steps);
    if (outPath.empty()) printf("[Warning] No output folder. Results of the solver will not be written to disk\n");
    else printf("Output folder: %s\n", outPath.c_str());

    nsf_device* h = nullptr;
    int st = nsf_create(device, &h);
    if (st != NSF_OK) {
        fprintf(stderr, "[Error] cannot initialise CUDA device %d (status %d)\n", device, st);
        return 1;
    }
    auto fail = [&](int status) {
        fprintf(stderr, "[Error] %s\n", nsf_last_error(h));
        nsf_destroy(h);
        return status == NSF_OK ? 1 : 1;
    };
    if (args.count("tol") && (st = nsf_set_tolerance(h, atof(args["tol"].c_str()))) != NSF_OK) return fail(st);
    const int mode = scene.solver == "mixed" ? NSF_SOLVER_MIXED : NSF_SOLVER_FP64;
    if ((st = nsf_set_solver(h, mode, -1)) != NSF_OK) return fail(st);
    const auto t0 = std::chrono::steady_clock::now();
    st = nsf_sim_setup(h, scene.nNodes, scene.xy.data(), scene.nElements, scene.elements.data(), scene.nPressure,
                       (int)scene.uNodes.size(), scene.uNodes.data(), scene.gu.data(), scene.gv.data(),
                       (int)scene.pNodes.size(), scene.pNodes.data(), scene.gp.data(), scene.viscosity, scene.dt);
    if (st != NSF_OK) return fail(st);
    const auto t1 = std::chrono::steady_clock::now();
    std::vector<double> uv(2 * (size_t)scene.nNodes), p(scene.nPressure);
    try {
        int firstStep = 1;
        if (args.count("resume")) {
            firstStep = nsfhost::read_solution(args["resume"], scene.nNodes, scene.nPressure, uv, p) + 1;
            if ((st = nsf_sim_set_fields(h, uv.data(), p.data())) != NSF_OK) return fail(st);
            printf("Resuming after time step %d\n", firstStep - 1);
        }
        if (scene.timeDependent) {
            // Dirichlet data that use t: evaluated on the device at the end time of every step
            std::vector<const char*> ex;
            for (const auto& e : scene.expressions) ex.push_back(e.c_str());
            if ((st = nsf_sim_set_bc_expressions(h, (int)ex.size(), ex.data(), scene.uExpr.data(), scene.vExpr.data(),
                                                 scene.pExpr.data(), (firstStep - 1) * scene.dt)) != NSF_OK)
                return fail(st);
        }
        if (!args.count("resume") && !outPath.empty()) {
            if ((st = nsf_sim_get_fields(h, uv.data(), p.data())) != NSF_OK) return fail(st);
            nsfhost::write_solution(outPath, 0, scene.nNodes, scene.nPressure, uv.data(), p.data());
        }
        std::vector<int> it(5);
        long long total[5] = {0, 0, 0, 0, 0};
        for (int step = firstStep; step <= steps; ++step) {
            if ((st = nsf_sim_step(h, 1, it.data())) != NSF_OK) return fail(st);
            for (int k = 0; k < 5; ++k) total[k] += it[k];
            if (!outPath.empty()) {
                if ((st = nsf_sim_get_fields(h, uv.data(), p.data())) != NSF_OK) return fail(st);
                nsfhost::write_solution(outPath, step, scene.nNodes, scene.nPressure, uv.data(), p.data());
            }
        }
        const auto t2 = std::chrono::steady_clock::now();
        const double setupS = std::chrono::duration<double>(t1 - t0).count();
        const double runS = std::chrono::duration<double>(t2 - t1).count();
        printf("Setup (upload, point-location tree, assembly): %.3f s\n", setupS);
        printf("Time stepping: %.3f s (%.3f ms/step)\n", runS, steps > 0 ? 1e3 * runS / steps : 0.0);
        printf("CG iterations: diffusion %lld / %lld, pressure %lld, mass %lld / %lld\n", total[0], total[1],
               total[2], total[3], total[4]);
    } catch (const std::exception& e) {
        fprintf(stderr, "[Error] %s\n", e.what());
        nsf_destroy(h);
        return 1;
    }
    nsf_destroy(h);
    return 0;
}
