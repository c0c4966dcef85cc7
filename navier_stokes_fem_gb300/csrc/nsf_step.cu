// The whole operator-split step of many mesh instances in ONE persistent cooperative launch (the batched form).
//
// Each instance (a lid-driven cavity of its own size, viscosity and time step) is served by a team: a contiguous
// range of CTAs of the launch.  The team runs the reference's loop body (include/assembly.h:1516-1556) for its
// instance without leaving the kernel: advection, the two diffusion solves, the pressure solve, the two mass
// solves whose right-hand sides are the gradient rows of the new pressure, and the Dirichlet re-imposition.
// Consecutive phases are separated by the team's bounded barrier only; teams never wait on one another, so an
// instance of 300 nodes and one of 260,000 run side by side.  Velocity is updated in place (u <- du + u), so one
// launch describes every step and the step is captured once as a CUDA graph and replayed.
//
// Team sizes are the "tile shape" of the plan: a small autotuner (batch_autotune) times every team on real
// steps and re-divides the co-resident CTAs in proportion to measured work (CTAs x time), keeping the plan with
// the shortest step.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "nsf_device.cuh"
#include "nsf_locate_device.cuh"

namespace nsf {

struct CsrView {
    const int* rowptr;
    const int* col;
    const double* val;
    const float* val32;
    const float* rowsum32;
    const int* sellStart;
    const int* sellCol;
    const double* sellVal;
    const float* sellVal32;
};

struct StepInstance {
    TreeView tree;
    int nNodes, nP;
    float fdt;
    CsrView M, D, K, B, G;   // velocity mass, diffusion, pressure stiffness, -(1/dt) Div, -dt Grad
    double *uv, *tmp, *p, *rhsV, *rhsP;
    const unsigned char *bcV, *bcP;
    const double *gV0, *gV1, *gP, *liftV0, *liftV1, *liftP;
    double *r, *q, *p0, *p1;
    float *r32, *d32, *q32, *p32a, *p32b;
    double* partials;
    GridSync* sync;
    CgInfo* info;            // kStepInfoCap steps x 5 solves
    int* stepCounter;
    unsigned long long* teamNs;
    int firstBlock, nBlocks;
};

struct StepParams {
    int mode;
    double tol2, innerTol2;
    int maxOuter;
    long long timeoutNs;
};

__device__ __forceinline__ CgArgs solve_args(const StepInstance& I, const StepParams& sp, const CsrView& A, int n) {
    CgArgs a{};
    a.n = n;
    a.rowptr = A.rowptr;
    a.col = A.col;
    a.val = A.val;
    a.val32 = A.val32;
    a.rowsum32 = A.rowsum32;
    a.sellStart = A.sellStart;
    a.sellCol = A.sellCol;
    a.sellVal = A.sellVal;
    a.sellVal32 = A.sellVal32;
    a.r = I.r;
    a.q = I.q;
    a.pbuf0 = I.p0;
    a.pbuf1 = I.p1;
    a.r32 = I.r32;
    a.d32 = I.d32;
    a.q32 = I.q32;
    a.p32a = I.p32a;
    a.p32b = I.p32b;
    a.partials = I.partials;
    a.sync = I.sync;
    a.maxIt = n;
    a.tol2 = sp.tol2;
    a.innerTol2 = sp.innerTol2;
    a.maxOuter = sp.maxOuter;
    a.timeoutNs = sp.timeoutNs;
    return a;
}

// One out-of-line copy of each solver serves the step's three solve sites (register allocation per solver, not
// for six inlined copies at once).
__device__ __noinline__ int step_cg_fp64(Team& t, const CgArgs& a, double* stage, double* smem) {
    return team_cg_fp64(t, a, stage, smem);
}
__device__ __noinline__ int step_cg_mixed(Team& t, const CgArgs& a, double* stage, double* smem) {
    return team_cg_mixed(t, a, stage, smem);
}
// the velocity systems (P2 rows of 9 and 19 entries): the pipelined wide product
__device__ __noinline__ int step_cg_fp64_wide(Team& t, const CgArgs& a, double* stage, double* smem) {
    return team_cg_fp64<true>(t, a, stage, smem);
}
__device__ __noinline__ int step_cg_mixed_wide(Team& t, const CgArgs& a, double* stage, double* smem) {
    return team_cg_mixed<true>(t, a, stage, smem);
}
__device__ __forceinline__ int run_cg(Team& t, const CgArgs& a, int mode, double* stage, double* smem) {
    return mode == NSF_SOLVER_MIXED ? step_cg_mixed(t, a, stage, smem) : step_cg_fp64(t, a, stage, smem);
}
__device__ __forceinline__ int run_cg_wide(Team& t, const CgArgs& a, int mode, double* stage, double* smem) {
    return mode == NSF_SOLVER_MIXED ? step_cg_mixed_wide(t, a, stage, smem) : step_cg_fp64_wide(t, a, stage, smem);
}

__global__ void __launch_bounds__(kCgThreads, 2) step_kernel(const StepInstance* __restrict__ insts,
                                                             const int* __restrict__ blockInst, StepParams sp) {
    NSF_KERNEL_SHARED();
    const StepInstance& I = insts[blockInst[blockIdx.x]];
    Team t{I.sync, I.partials, I.nBlocks, (int)blockIdx.x - I.firstBlock, 0ULL, sp.timeoutNs};
    const long long t0 = global_ns();
    const int step = *(const volatile int*)I.stepCounter;
    CgInfo* info = I.info + (size_t)(step % kStepInfoCap) * 5;
    const int Nv = I.nNodes;
    const int bs = blockDim.x;
    int rb, re;

    // advection: back-trace in float, locate, P2 interpolation in double (uv -> tmp)
    team_rows(Nv, t, rb, re);
    for (int i = rb + (int)threadIdx.x; i < re; i += bs) {
        const float2 pos = I.tree.xy[i];
        const double ui = I.uv[i], vi = I.uv[Nv + i];
        const float px = __fsub_rn(pos.x, __fmul_rn((float)ui, I.fdt));
        const float py = __fsub_rn(pos.y, __fmul_rn((float)vi, I.fdt));
        float xi = 0.f, eta = 0.f;
        int nn = -1;
        const int e = locate_point(I.tree, px, py, xi, eta, nn);
        if (e >= 0) {
            double N[6];
            p2_eval_d((double)xi, (double)eta, N);
            const int* en = I.tree.el + 6 * (size_t)e;
            double su = 0.0, sv = 0.0;
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                su = __dadd_rn(su, __dmul_rn(N[k], I.uv[en[k]]));
                sv = __dadd_rn(sv, __dmul_rn(N[k], I.uv[Nv + en[k]]));
            }
            I.tmp[i] = su;
            I.tmp[Nv + i] = sv;
        } else {
            const int src = nn >= 0 ? nn : i;
            I.tmp[i] = I.uv[src];
            I.tmp[Nv + i] = I.uv[Nv + src];
        }
    }
    if (!t.barrier(100)) return;

    // diffusion solves: (M + dt nu K) u = M u_adv - lift, Dirichlet rows -> g; x0 = u_adv
    for (int ch = 0; ch < 2; ++ch) {
        CgArgs a = solve_args(I, sp, I.D, Nv);
        a.bRowptr = I.M.rowptr;
        a.bCol = I.M.col;
        a.bVal = I.M.val;
        a.bSellStart = I.M.sellStart;
        a.bSellCol = I.M.sellCol;
        a.bSellVal = I.M.sellVal;
        a.bX = I.tmp + (size_t)ch * Nv;
        a.lift = ch ? I.liftV1 : I.liftV0;
        a.bcMask = I.bcV;
        a.bcValue = ch ? I.gV1 : I.gV0;
        a.bOut = I.rhsV + (size_t)ch * Nv;
        a.b = a.bOut;
        a.x0 = I.tmp + (size_t)ch * Nv;
        a.x = I.uv + (size_t)ch * Nv;
        a.info = info + ch;
        if (run_cg_wide(t, a, sp.mode, stage, smem) == NSF_ERR_BARRIER_TIMEOUT) return;
    }
    // pressure: Kp p = -(1/dt) Div u - lift, pinned nodes -> g; x0 = p
    {
        CgArgs a = solve_args(I, sp, I.K, I.nP);
        a.bRowptr = I.B.rowptr;
        a.bCol = I.B.col;
        a.bVal = I.B.val;
        a.bX = I.uv;
        a.lift = I.liftP;
        a.bcMask = I.bcP;
        a.bcValue = I.gP;
        a.bOut = I.rhsP;
        a.b = a.bOut;
        a.x0 = I.p;
        a.x = I.p;
        a.info = info + 2;
        if (run_cg(t, a, sp.mode, stage, smem) == NSF_ERR_BARRIER_TIMEOUT) return;
    }
    // velocity correction: M du = (-dt Grad p) per component, x0 = u; the right-hand side is built from the
    // gradient rows of the component (row offset ch*Nv) inside the solve
    for (int ch = 0; ch < 2; ++ch) {
        CgArgs a = solve_args(I, sp, I.M, Nv);
        a.bRowptr = I.G.rowptr + (size_t)ch * Nv;
        a.bCol = I.G.col;
        a.bVal = I.G.val;
        a.bX = I.p;
        a.bOut = I.rhsV + (size_t)ch * Nv;
        a.b = a.bOut;
        a.x0 = I.uv + (size_t)ch * Nv;
        a.x = I.tmp + (size_t)ch * Nv;
        a.info = info + 3 + ch;
        if (run_cg_wide(t, a, sp.mode, stage, smem) == NSF_ERR_BARRIER_TIMEOUT) return;
    }
    // u <- du + u with the Dirichlet values re-imposed (include/assembly.h:686-707), in place
    team_rows(Nv, t, rb, re);
    for (int i = rb + (int)threadIdx.x; i < re; i += bs) {
        const bool d = I.bcV[i];
        I.uv[i] = d ? I.gV0[i] : I.tmp[i] + I.uv[i];
        I.uv[Nv + i] = d ? I.gV1[i] : I.tmp[Nv + i] + I.uv[Nv + i];
    }
    if (t.rank == 0 && threadIdx.x == 0) {
        *I.teamNs = (unsigned long long)(global_ns() - t0);
        *I.stepCounter = step + 1;
    }
}

// ---------------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------------
static CsrView view(const Csr& A) {
    return CsrView{A.rowptr.get(), A.col.get(), A.val.get(), A.val32.get(), A.rowsum32.get(),
                   A.hasSell ? A.sellStart.get() : nullptr, A.sellCol.get(), A.sellVal.get(), A.sellVal32.get()};
}

int step_kernel_capacity(int device) {
    int sms = 0, occ = 0;
    NSF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, step_kernel, kCgThreads, 0));
    return sms * std::min(occ, 2);
}

// Lays the current team sizes out over the grid and uploads the per-instance descriptors.
void batch_upload_plan(nsf_device* h) {
    std::vector<StepInstance> desc(h->batch.size());
    std::vector<int> blockInst;
    int first = 0;
    size_t maxBlocks = 1;
    for (auto& in : h->batch) maxBlocks = std::max(maxBlocks, (size_t)in->blocks);
    h->batchSync.alloc(h->batch.size());
    for (size_t i = 0; i < h->batch.size(); ++i) {
        Instance& in = *h->batch[i];
        in.partials.ensure(6 * (size_t)in.blocks);
        StepInstance& d = desc[i];
        std::memset(&d, 0, sizeof(d));
        d.tree = TreeView{in.mesh.xy.get(), in.mesh.el.get(), in.mesh.tree.triSorted.get(), in.mesh.tree.box.get(),
                          in.mesh.tree.nLeaves};
        d.nNodes = in.mesh.nNodes;
        d.nP = in.mesh.nP;
        d.fdt = (float)in.sim.dt;
        d.M = view(in.mats[NSF_VELOCITY_MASS]);
        d.D = view(in.mats[NSF_DIFFUSION]);
        d.K = view(in.mats[NSF_PRESSURE_STIFFNESS]);
        d.B = view(in.mats[NSF_VELOCITY_DIVERGENCE]);
        d.G = view(in.mats[NSF_PRESSURE_DIVERGENCE]);
        SimState& S = in.sim;
        d.uv = S.uv.get();
        d.tmp = S.tmp.get();
        d.p = S.p.get();
        d.rhsV = S.rhsV.get();
        d.rhsP = S.rhsP.get();
        d.bcV = S.bcV.get();
        d.bcP = S.bcP.get();
        d.gV0 = S.gV[0].get();
        d.gV1 = S.gV[1].get();
        d.gP = S.gP.get();
        d.liftV0 = S.liftV[0].get();
        d.liftV1 = S.liftV[1].get();
        d.liftP = S.liftP.get();
        d.r = in.r.get();
        d.q = in.q.get();
        d.p0 = in.p0.get();
        d.p1 = in.p1.get();
        d.r32 = in.r32.get();
        d.d32 = in.d32.get();
        d.q32 = in.q32.get();
        d.p32a = in.p32a.get();
        d.p32b = in.p32b.get();
        d.partials = in.partials.get();
        d.sync = h->batchSync.get() + i;
        d.info = in.info.get();
        d.stepCounter = in.stepCounter.get();
        d.teamNs = in.teamNs.get();
        d.firstBlock = first;
        d.nBlocks = in.blocks;
        for (int b = 0; b < in.blocks; ++b) blockInst.push_back((int)i);
        first += in.blocks;
    }
    if (first > h->batchCapacity) throw Error{NSF_ERR_BAD_ARG, "plan needs more CTAs than can be co-resident"};
    h->batchGrid = first;
    h->batchDesc.alloc(sizeof(StepInstance) * desc.size());
    NSF_CUDA(cudaMemcpyAsync(h->batchDesc.get(), desc.data(), sizeof(StepInstance) * desc.size(),
                             cudaMemcpyHostToDevice, h->stream));
    h->batchBlockInst.upload(blockInst.data(), blockInst.size(), h->stream);
    NSF_CUDA(cudaStreamSynchronize(h->stream));
}

void batch_launch_step(nsf_device* h) {
    NSF_CUDA(cudaMemsetAsync(h->batchSync.get(), 0, sizeof(GridSync) * h->batch.size(), h->stream));
    StepParams sp{h->solverMode, h->tol * h->tol, h->innerTol * h->innerTol, 64, h->timeoutNs};
    const StepInstance* desc = reinterpret_cast<const StepInstance*>(h->batchDesc.get());
    const int* bi = h->batchBlockInst.get();
    void* params[] = {(void*)&desc, (void*)&bi, (void*)&sp};
    NSF_CUDA(cudaLaunchCooperativeKernel((const void*)step_kernel, dim3(h->batchGrid), dim3(kCgThreads), params, 0,
                                         h->stream));
    count_launch();
}

// Integer team sizes proportional to `work`, each >= 1, summing to `total` (largest remainders).
static std::vector<int> apportion(const std::vector<double>& work, int total) {
    const size_t n = work.size();
    std::vector<int> out(n, 1);
    const double W = std::accumulate(work.begin(), work.end(), 0.0);
    int left = total - (int)n;
    if (left <= 0 || W <= 0) return out;
    std::vector<double> share(n), frac(n);
    int used = 0;
    for (size_t i = 0; i < n; ++i) {
        share[i] = left * work[i] / W;
        const int f = (int)std::floor(share[i]);
        out[i] += f;
        used += f;
        frac[i] = share[i] - f;
    }
    std::vector<size_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return frac[a] > frac[b]; });
    for (size_t k = 0; k < order.size() && used < left; ++k, ++used) out[order[k]]++;
    return out;
}

// Autotuner: starts from a size model (work ~ nnz x sqrt(pressure unknowns)), runs `rounds` real steps on a
// saved copy of the fields, re-divides the CTAs by measured CTAs x time, and keeps the fastest plan.
void batch_autotune(nsf_device* h, int rounds) {
    const size_t n = h->batch.size();
    const int total = h->batchCapacity;
    std::vector<double> work(n);
    for (size_t i = 0; i < n; ++i) {
        Instance& in = *h->batch[i];
        const double nnz = (double)in.mats[NSF_DIFFUSION].nnz + in.mats[NSF_VELOCITY_MASS].nnz +
                           in.mats[NSF_PRESSURE_STIFFNESS].nnz;
        work[i] = nnz * std::sqrt((double)in.mesh.nP);
    }
    // save the fields so the trial steps leave the simulation where it was
    std::vector<DevBuf<double>> saveUV(n), saveP(n);
    std::vector<int> saveCounter(n);
    for (size_t i = 0; i < n; ++i) {
        Instance& in = *h->batch[i];
        saveUV[i].alloc(in.sim.uv.n);
        saveP[i].alloc(in.sim.p.n);
        NSF_CUDA(cudaMemcpyAsync(saveUV[i].get(), in.sim.uv.get(), sizeof(double) * in.sim.uv.n,
                                 cudaMemcpyDeviceToDevice, h->stream));
        NSF_CUDA(cudaMemcpyAsync(saveP[i].get(), in.sim.p.get(), sizeof(double) * in.sim.p.n,
                                 cudaMemcpyDeviceToDevice, h->stream));
    }
    std::vector<int> best;
    double bestMs = 1e300;
    h->autotuneLog.clear();
    h->autotuneMs.clear();
    cudaEvent_t e0, e1;
    NSF_CUDA(cudaEventCreate(&e0));
    NSF_CUDA(cudaEventCreate(&e1));
    for (int round = 0; round <= rounds; ++round) {
        std::vector<int> plan = apportion(work, total);
        for (size_t i = 0; i < n; ++i) h->batch[i]->blocks = plan[i];
        batch_upload_plan(h);
        NSF_CUDA(cudaEventRecord(e0, h->stream));
        batch_launch_step(h);
        NSF_CUDA(cudaEventRecord(e1, h->stream));
        NSF_CUDA(cudaStreamSynchronize(h->stream));
        float ms = 0;
        NSF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        h->autotuneLog.insert(h->autotuneLog.end(), plan.begin(), plan.end());
        h->autotuneMs.push_back(ms);
        if (ms < bestMs) { bestMs = ms; best = plan; }
        for (size_t i = 0; i < n; ++i) {
            unsigned long long ns = 0;
            NSF_CUDA(cudaMemcpy(&ns, h->batch[i]->teamNs.get(), sizeof(ns), cudaMemcpyDeviceToHost));
            work[i] = std::max(1.0, (double)ns) * plan[i];
        }
        // restore the fields and the step counters
        for (size_t i = 0; i < n; ++i) {
            Instance& in = *h->batch[i];
            NSF_CUDA(cudaMemcpyAsync(in.sim.uv.get(), saveUV[i].get(), sizeof(double) * in.sim.uv.n,
                                     cudaMemcpyDeviceToDevice, h->stream));
            NSF_CUDA(cudaMemcpyAsync(in.sim.p.get(), saveP[i].get(), sizeof(double) * in.sim.p.n,
                                     cudaMemcpyDeviceToDevice, h->stream));
            NSF_CUDA(cudaMemsetAsync(in.stepCounter.get(), 0, sizeof(int), h->stream));
        }
        NSF_CUDA(cudaStreamSynchronize(h->stream));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (size_t i = 0; i < n; ++i) h->batch[i]->blocks = best[i];
    batch_upload_plan(h);
}

void batch_capture_graph(nsf_device* h) {
    if (h->batchGraphExec) { cudaGraphExecDestroy(h->batchGraphExec); h->batchGraphExec = nullptr; }
    if (h->batchGraph) { cudaGraphDestroy(h->batchGraph); h->batchGraph = nullptr; }
    NSF_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    try {
        batch_launch_step(h);
    } catch (...) {
        cudaGraph_t g;
        cudaStreamEndCapture(h->stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    NSF_CUDA(cudaStreamEndCapture(h->stream, &h->batchGraph));
    NSF_CUDA(cudaGraphInstantiate(&h->batchGraphExec, h->batchGraph, 0));
}

}  // namespace nsf
