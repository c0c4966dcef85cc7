// Persistent conjugate-gradient megakernels for sm_103a.
//
// Replaces the reference's conjugateGradientMegakernel (gpu/matrix_math.cu:251-286, host driver
// cpp/gpu_simulation_device.cpp:385-515): one cooperative launch runs the whole CG loop on the device.
// Differences from the reference, by design:
//   * 3 grid-wide barriers per FP64 iteration instead of 4 (q = A p and p.q | x, r and r.r | p = r + beta p).
//     GB300 issues only about 2 FP64 FMAs per cycle per SM, which at one FMA per non-zero already matches the
//     HBM stream of a 12-byte CSR entry, so the FP64 kernel spends exactly one DFMA per non-zero and materialises
//     p rather than recomputing it per gathered entry;
//   * the SpMV is warp-chunked CSR: a warp takes 32 consecutive rows, streams their contiguous non-zeros with
//     coalesced loads (four independent loads per lane in flight), stages value and gathered vector element in
//     shared memory, and each lane sums its own row in entry order (the reference assigns one thread per row and
//     walks each row's entries one dependent load after another, gpu/matrix_math.cu:20-47);
//   * deterministic reductions: warp xor-shuffle -> per-block partial -> after the barrier every block sums the
//     partials in one fixed order, so all blocks hold bit-identical alpha/beta (the reference uses float
//     atomicAdd, gpu/matrix_math.cu:163-193);
//   * every barrier wait is bounded by %globaltimer; on expiry the kernel raises an abort word, every block
//     leaves, and the host reports NSF_ERR_BARRIER_TIMEOUT (the reference's spin barrier can deadlock);
//   * stopping rule ||r|| <= tol*||b|| (relative), FP64 vectors and scalars;
//   * optional fused right-hand side: b_i = mask_i ? g_i : (B x_b)_i - lift_i is built in the prologue, so the
//     diffusion and pressure right-hand sides of the operator-split step (include/assembly.h:497-523, 575-595)
//     cost no extra launch.
// The mixed-precision form runs CG with FP32 matrix values and FP32 vectors (FP64 dots and scalars) and refines
// it with FP64 reliable updates: the true residual b - A x is recomputed with the FP64 matrix whenever the FP32
// residual has dropped by a fixed factor, without restarting the recurrence.
#include "nsf_pcg_device.cuh"

namespace nsf {

// ---------------------------------------------------------------------------------------------------
// single-solve kernels: the team is the whole cooperative grid
// ---------------------------------------------------------------------------------------------------
// Wide = true: the pipelined product for matrices with slices wider than kSellChunk entries per row (P2 systems);
// each kernel is instantiated for both so that the narrow systems keep their own register allocation.
template <bool Wide>
__global__ void __launch_bounds__(kCgThreads, 2) cg_fp64_kernel(CgArgs a) {
    NSF_KERNEL_SHARED();
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    team_cg_fp64<Wide>(t, a, stage, smem);
}

// The FP64 CG with one grid barrier per iteration (pipelined recurrences; needs the matrix's SELL copy).
template <bool Wide>
__global__ void __launch_bounds__(kCgThreads, 2) cg_fp64_pipe_kernel(CgArgs a) {
    NSF_KERNEL_SHARED();
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    team_cg_fp64_pipelined<Wide>(t, a, stage, smem);
}

// The narrow mixed kernel streams its FP32 matrix through per-warp TMA rings (kRingBytes of dynamic shared memory).
template <bool Wide>
__global__ void __launch_bounds__(kCgThreads, 2) cg_mixed_kernel(CgArgs a) {
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    if constexpr (Wide) {
        NSF_KERNEL_SHARED();
        team_cg_mixed<Wide>(t, a, stage, smem);
    } else {
        NSF_RING_SHARED();
        SellRing ring = ring_init(dsm, a.sync, a.timeoutNs);
        team_cg_mixed<Wide>(t, a, stage, smem, &ring);
    }
}

template <bool Wide>
__global__ void __launch_bounds__(kCgThreads, 2) pcg_fp64_kernel(CgArgs a) {
    NSF_KERNEL_SHARED();
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    team_pcg_fp64<Wide>(t, a, stage, smem);
}

// The mixed PCG kernels stream the FP32 factor (and the narrow matrix) through per-warp TMA rings.
template <bool Wide>
__global__ void __launch_bounds__(kCgThreads, 2) pcg_mixed_kernel(CgArgs a) {
    NSF_RING_SHARED();
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    SellRing ring = ring_init(dsm, a.sync, a.timeoutNs);
    team_pcg_mixed<Wide>(t, a, stage, smem, &ring);
}

// The split mixed PCG for narrow matrices: the refresh launch (FP64 true residual, tests, sweeps; rare) keeps the
// 2-CTA register budget and the TMA rings, the inner-iteration launch runs the FP32 loop alone at 4 CTAs per SM,
// twice the warps to hide the latency of the gathers.
__global__ void __launch_bounds__(kCgThreads, 2) pcg_mixed_refresh_kernel(CgArgs a) {
    NSF_RING_SHARED();
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    SellRing ring = ring_init(dsm, a.sync, a.timeoutNs);
    team_pcg_mixed_refresh(t, a, stage, smem, &ring);
}

// (C16: the matrix and both factor parts have 16-bit column copies.)
template <bool C16>
__global__ void __launch_bounds__(kCgThreads, 4) pcg_mixed_inner_kernel(CgArgs a) {
    NSF_KERNEL_SHARED();
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    team_pcg_mixed_inner<C16>(t, a, stage, smem, nullptr);
}

// The same iterations as one 1024-thread CTA per SM, the form the split solver launches: the same 32 warps per
// SM and 64 registers per thread, a quarter of the grid barrier's arrivals (1.5 % per iteration on the 2048²
// pressure system, 9-13 % per step on systems of 0.26-1 M rows, where the barriers weigh more).  Two or more
// colours and a SELL copy only: there is no staging area for the CSR product.
constexpr int kInnerCtaThreads = 1024;
// (H16: the factor's FP16 value copies, with C16.)
template <bool C16, bool H16 = false>
__global__ void __launch_bounds__(kInnerCtaThreads, 1) pcg_mixed_inner_kernel_cta1024(CgArgs a) {
    __shared__ double smem[kSmemSlots];
    if (!a.sellStart) return;   // (the host never launches it without one)
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    team_pcg_mixed_inner<C16, true, false, H16>(t, a, nullptr, smem, nullptr);
}

// The reduced (Schur complement) iterations of a two-colour system in the 1024-thread form (a.f.reduced);
// Resident: with the CTA-private row state in dynamic shared memory, where it fits.
template <bool C16, bool Resident = false>
__global__ void __launch_bounds__(kInnerCtaThreads, 1) pcg_mixed_inner_kernel_reduced(CgArgs a) {
    __shared__ double smem[kSmemSlots];
    if (!a.sellStart || a.f.colours != 2 || !a.f.reduced) return;   // (the host never launches it otherwise)
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    team_pcg_mixed_inner_reduced<C16, Resident>(t, a, smem);
}

// The same iterations with the Schur complement formed explicitly (a.f.schur): one product phase per iteration.
template <bool Resident = false>
__global__ void __launch_bounds__(kInnerCtaThreads, 1) pcg_mixed_inner_kernel_schur(CgArgs a) {
    __shared__ double smem[kSmemSlots];
    if (a.f.colours != 2 || !a.f.reduced || !a.f.schur || !a.f.sStart) return;   // (the host never launches it otherwise)
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    team_pcg_mixed_inner_reduced<true, Resident, true>(t, a, smem);
}

// The same 1024-thread form with the row state only its CTA reads (the FP32 correction, and r and q of its colour-1
// rows) in dynamic shared memory for the whole launch: two colours only, and only where that state fits.
template <bool C16, bool H16 = false>
__global__ void __launch_bounds__(kInnerCtaThreads, 1) pcg_mixed_inner_kernel_resident(CgArgs a) {
    __shared__ double smem[kSmemSlots];
    if (!a.sellStart || a.f.colours != 2) return;   // (the host never launches it otherwise)
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    team_pcg_mixed_inner<C16, true, true, H16>(t, a, nullptr, smem, nullptr);
}

// Shared-memory bytes pcg_mixed_inner_kernel_resident needs on `grid` CTAs for a factor's colour blocks: per CTA
// its share of each block (team_block's rule) as d, plus r and q of its colour-1 share.
static size_t resident_bytes_schur(const FactorView& f, int grid) {
    const int slices = (f.colourRow[2] - f.colourRow[1]) / kSlice;
    return sizeof(float) * 4 * (size_t)((slices + grid - 1) / grid) * kSlice;
}

static size_t resident_bytes(const FactorView& f, int grid) {
    auto share = [&](int c) {
        const int slices = (f.colourRow[c + 1] - f.colourRow[c]) / kSlice;
        return (size_t)((slices + grid - 1) / grid) * kSlice;
    };
    return sizeof(float) * (share(0) + 3 * share(1));
}

// The split plain mixed CG for wide (P2) systems: refresh launches (fold, FP64 true residual, tests) at 2 CTAs per
// SM and FP32 iteration launches at 4.
static __device__ void team_cg_mixed_refresh(Team& t, const CgArgs& a, double* stage, double* smem) {
    int where = 10;
    PcgLoop L;
    if (a.loopInit) {
        cg_mixed_start<true>(t, a, stage);
        cg_loop_init(L, a);
    } else {
        L = *a.loop;
    }
    if (!cg_mixed_refresh<true>(t, a, stage, smem, L, where)) {
        write_info(t, a, L.it, NSF_ERR_BARRIER_TIMEOUT, L.refresh, L.rr64, L.bb);
        L.state = kLoopDone;
    } else if (L.state == kLoopDone) {
        cg_mixed_finish<true>(t, a, stage, smem, L);
    }
    pcg_loop_store(t, a, L);
}

static __device__ void team_cg_mixed_inner(Team& t, const CgArgs& a, double* stage, double* smem) {
    int where = 400;
    // the fields the FP32 iterations read or write (the rest of the state stays in memory)
    const PcgLoop& G = *a.loop;
    PcgLoop L;
    L.beta = G.beta;
    L.flip = G.flip;
    L.rr = G.rr;
    L.rrPrev = G.rrPrev;
    L.rrRef = G.rrRef;
    L.target = G.target;
    L.scale = G.scale;
    L.cycleTol2 = G.cycleTol2;
    L.it = G.it;
    L.itRef = G.itRef;
    const bool ok = cg_mixed_inner<true, true>(t, a, stage, smem, nullptr, L, where);
    if (!ok) write_info(t, a, L.it, NSF_ERR_BARRIER_TIMEOUT, G.refresh, G.rr64, G.bb);
    if (t.rank == 0 && threadIdx.x == 0) {
        a.loop->beta = L.beta;
        a.loop->flip = L.flip;
        a.loop->rr = L.rr;
        a.loop->rrPrev = L.rrPrev;
        a.loop->it = L.it;
        a.loop->lastCycle = L.lastCycle;
        a.loop->innerBreakdown = L.innerBreakdown;
        a.loop->state = ok ? L.state : kLoopDone;
    }
}

__global__ void __launch_bounds__(kCgThreads, 2) cg_mixed_refresh_kernel(CgArgs a) {
    NSF_KERNEL_SHARED();
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    team_cg_mixed_refresh(t, a, stage, smem);
}

__global__ void __launch_bounds__(kCgThreads, 4) cg_mixed_inner_kernel(CgArgs a) {
    NSF_KERNEL_SHARED();
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    team_cg_mixed_inner(t, a, stage, smem);
}

// One 1024-thread CTA per SM, as pcg_mixed_inner_kernel_cta1024 (a SELL copy only).
__global__ void __launch_bounds__(kInnerCtaThreads, 1) cg_mixed_inner_kernel_cta1024(CgArgs a) {
    __shared__ double smem[kSmemSlots];
    if (!a.sellStart) return;   // (the host never launches it without one)
    Team t = Team::grid(a.sync, a.partials, a.timeoutNs);
    team_cg_mixed_inner(t, a, nullptr, smem);
}

// ---------------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------------
// The persistent solver kernels with the dynamic shared memory each is launched with (the TMA rings).
struct CgKernel {
    const void* fn;
    size_t dsm;
};
static const CgKernel kCgKernels[8] = {
    {(const void*)cg_fp64_kernel<false>, 0},          {(const void*)cg_mixed_kernel<false>, kRingBytes},
    {(const void*)pcg_fp64_kernel<false>, 0},         {(const void*)pcg_mixed_kernel<false>, kRingBytes},
    {(const void*)cg_fp64_kernel<true>, 0},           {(const void*)cg_mixed_kernel<true>, 0},
    {(const void*)pcg_fp64_kernel<true>, 0},          {(const void*)pcg_mixed_kernel<true>, kRingBytes}};

static const CgKernel& cg_kernel(int mode, bool wide) {
    const int m = mode == NSF_SOLVER_MIXED ? 1 : mode == NSF_SOLVER_PCG_FP64 ? 2 : mode == NSF_SOLVER_PCG_MIXED ? 3 : 0;
    return kCgKernels[(wide ? 4 : 0) + m];
}

// Co-resident CTAs per SM of every persistent solver kernel (the grid must fit all of them); also raises the
// dynamic shared-memory limit of the ring kernels.
static int cg_occupancy() {
    int occ = 1 << 30;
    for (const CgKernel& k : kCgKernels) {
        if (k.dsm) NSF_CUDA(cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.dsm));
        int o = 0;
        NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k.fn, kCgThreads, k.dsm));
        occ = std::min(occ, o);
    }
    NSF_CUDA(cudaFuncSetAttribute((const void*)pcg_mixed_refresh_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kRingBytes));
    int o = 0;
    NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, (const void*)pcg_mixed_refresh_kernel, kCgThreads,
                                                           kRingBytes));
    return std::min(occ, o);
}

// CTAs per SM of the split solvers' inner-iteration kernels (at most 4)
static int inner_occupancy() {
    int o = 0, o16 = 0, c = 0, r = 0;
    NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, (const void*)pcg_mixed_inner_kernel<false>, kCgThreads,
                                                           0));
    NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o16, (const void*)pcg_mixed_inner_kernel<true>,
                                                           kCgThreads, 0));
    o = std::min(o, o16);
    NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, (const void*)cg_mixed_inner_kernel, kCgThreads, 0));
    NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, (const void*)cg_mixed_refresh_kernel, kCgThreads, 0));
    if (r < 2) throw Error{NSF_ERR_CUDA, "mixed refresh kernel cannot be resident at 2 CTAs per SM"};
    return std::min(4, std::min(o, c));
}

void cg_configure(CgWorkspace& ws, int device) {
    int sms = 0, coop = 0;
    NSF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    NSF_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
    if (!coop) throw Error{NSF_ERR_NO_DEVICE, "device does not support cooperative launches"};
    const int perSm = std::min(2, cg_occupancy());
    if (perSm < 1) throw Error{NSF_ERR_CUDA, "CG kernel cannot be resident"};
    ws.grid = sms * perSm;
    ws.block = kCgThreads;
    ws.gridInner = sms * std::max(perSm, inner_occupancy());
    // the 1024-thread inner kernels: one CTA per SM (0 if one of them cannot be resident)
    int o1024 = 1;
    for (const void* fn : {(const void*)pcg_mixed_inner_kernel_cta1024<true, true>,
                           (const void*)pcg_mixed_inner_kernel_cta1024<true>,
                           (const void*)pcg_mixed_inner_kernel_cta1024<false>, (const void*)cg_mixed_inner_kernel_cta1024}) {
        int o = 0;
        NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fn, kInnerCtaThreads, 0));
        o1024 = std::min(o1024, o);
    }
    ws.gridInner1024 = sms * o1024;
    // the resident form: the largest dynamic shared memory at which it still runs one 1024-thread CTA per SM
    ws.residentMaxBytes = 0;
    if (o1024 == 1) {
        int optin = 0;
        NSF_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
        size_t best = 0;
        for (const void* fn : {(const void*)pcg_mixed_inner_kernel_resident<true, true>,
                               (const void*)pcg_mixed_inner_kernel_resident<true>,
                               (const void*)pcg_mixed_inner_kernel_resident<false>,
                               (const void*)pcg_mixed_inner_kernel_reduced<true, true>,
                               (const void*)pcg_mixed_inner_kernel_reduced<false, true>,
                               (const void*)pcg_mixed_inner_kernel_schur<true>}) {
            cudaFuncAttributes fa{};
            NSF_CUDA(cudaFuncGetAttributes(&fa, fn));
            const int dyn = optin - (int)fa.sharedSizeBytes;
            NSF_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
            int o = 0;
            NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fn, kInnerCtaThreads, (size_t)dyn));
            const size_t ok = o >= 1 ? (size_t)dyn : 0;
            best = best == 0 ? ok : std::min(best, ok);
        }
        ws.residentMaxBytes = best;
    }
    // the pipelined FP64 CG runs on the same grid; it is offered only where that grid is co-resident for it
    ws.pipeOk = true;
    for (const void* fn : {(const void*)cg_fp64_pipe_kernel<false>, (const void*)cg_fp64_pipe_kernel<true>}) {
        int o = 0;
        NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fn, kCgThreads, 0));
        if (o < perSm) ws.pipeOk = false;
    }
    ws.partials.alloc((size_t)9 * std::max(ws.grid, ws.gridInner));   // (the pipelined FP64 CG uses 9 regions)
    ws.sync.alloc(1);
    ws.info.alloc(4096);
    ws.loop.alloc(1);
}

void cg_pipe_launch(CgWorkspace& ws, const CgArgs& args, bool wide, cudaStream_t s) {
    NSF_CUDA(cudaMemsetAsync(ws.sync.get(), 0, sizeof(GridSync), s));
    CgArgs a = args;
    a.wbuf0 = ws.w.get();
    a.wbuf1 = ws.bp.get();
    void* params[] = {&a};
    const void* fn = wide ? (const void*)cg_fp64_pipe_kernel<true> : (const void*)cg_fp64_pipe_kernel<false>;
    NSF_CUDA(cudaLaunchCooperativeKernel(fn, dim3(ws.grid), dim3(ws.block), params, 0, s));
    count_launch();
}

void cg_launch(CgWorkspace& ws, const CgArgs& args, int mode, bool wide, cudaStream_t s) {
    NSF_CUDA(cudaMemsetAsync(ws.sync.get(), 0, sizeof(GridSync), s));
    CgArgs a = args;
    void* params[] = {&a};
    const CgKernel& k = cg_kernel(mode, wide);
    NSF_CUDA(cudaLaunchCooperativeKernel(k.fn, dim3(ws.grid), dim3(ws.block), params, k.dsm, s));
    count_launch();
}

// A split solve: the refresh launch, then inner-iteration and refresh launches while the state says so.
// (inner1024: the 1024-thread form, used when given, resident on the device and the matrix has a SELL copy; else
// inner256 at ws.gridInner CTAs.)
static void split_launch(CgWorkspace& ws, CgArgs a, const void* refresh, size_t refreshDsm, const void* inner1024,
                         const void* inner256, cudaStream_t s, size_t inner1024Dsm = 0) {
    a.loop = ws.loop.get();
    auto launch = [&](const void* fn, int grid, int block, size_t dsm) {
        NSF_CUDA(cudaMemsetAsync(ws.sync.get(), 0, sizeof(GridSync), s));
        void* params[] = {&a};
        NSF_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(block), params, dsm, s));
        count_launch();
    };
    const bool cta1024 = inner1024 && ws.gridInner1024 > 0 && a.sellStart;
    const void* inner = cta1024 ? inner1024 : inner256;
    const int innerGrid = cta1024 ? ws.gridInner1024 : ws.gridInner;
    const int innerBlock = cta1024 ? kInnerCtaThreads : ws.block;
    a.loopInit = 1;
    launch(refresh, ws.grid, ws.block, refreshDsm);
    a.loopInit = 0;
    // every refresh counts one outer cycle and the solve ends at maxOuter of them, so this loop is bounded
    for (int cycle = 0; cycle <= a.maxOuter + 1; ++cycle) {
        int state = 0;
        NSF_CUDA(cudaMemcpyAsync(&state, &a.loop->state, sizeof(int), cudaMemcpyDeviceToHost, s));
        NSF_CUDA(cudaStreamSynchronize(s));
        if (state != kLoopInner) return;
        launch(inner, innerGrid, innerBlock, cta1024 ? inner1024Dsm : 0);
        launch(refresh, ws.grid, ws.block, refreshDsm);
    }
    throw Error{NSF_ERR_CUDA, "mixed-precision solve did not finish within its refresh budget"};
}

void cg_mixed_split_launch(CgWorkspace& ws, const CgArgs& a, cudaStream_t s) {
    split_launch(ws, a, (const void*)cg_mixed_refresh_kernel, 0, (const void*)cg_mixed_inner_kernel_cta1024,
                 (const void*)cg_mixed_inner_kernel, s);
}

int pcg_mixed_split_launch(CgWorkspace& ws, CgArgs a, cudaStream_t s) {
    if (a.f.reduced) {   // the reduced iterations: two colours and a SELL copy, checked by the caller
        const bool c16 = a.sellCol16 != nullptr;
        // the CTA-private row state in shared memory where it fits (the full resident form's footprint; the Schur
        // form keeps four vectors of its colour-1 share: d, r, q and 1 / L_11)
        const size_t need = a.f.schur ? resident_bytes_schur(a.f, ws.gridInner1024) : resident_bytes(a.f, ws.gridInner1024);
        const bool res = ws.residentMaxBytes > 0 && need <= ws.residentMaxBytes;
        const void* inner = a.f.schur
                                ? (res ? (const void*)pcg_mixed_inner_kernel_schur<true>
                                       : (const void*)pcg_mixed_inner_kernel_schur<false>)
                            : res ? (c16 ? (const void*)pcg_mixed_inner_kernel_reduced<true, true>
                                         : (const void*)pcg_mixed_inner_kernel_reduced<false, true>)
                                  : (c16 ? (const void*)pcg_mixed_inner_kernel_reduced<true>
                                         : (const void*)pcg_mixed_inner_kernel_reduced<false>);
        split_launch(ws, a, (const void*)pcg_mixed_refresh_kernel, kRingBytes, inner, nullptr, s, res ? need : 0);
        return a.f.schur ? (res ? 6 : 5) : res ? 4 : 3;
    }
    // the fused iterations (two or more colours) in the 1024-thread form; 16-bit columns where all three copies exist
    const bool c16 = a.sellCol16 && a.f.loCol16 && a.f.upCol16 && a.f.colours >= 2;
    const bool h16 = c16 && a.f.loVal16 && a.f.upVal16;   // FP16 factor values (16-bit columns only)
    const void* inner1024 = a.f.colours < 2 ? nullptr
                            : h16           ? (const void*)pcg_mixed_inner_kernel_cta1024<true, true>
                            : c16           ? (const void*)pcg_mixed_inner_kernel_cta1024<true>
                                            : (const void*)pcg_mixed_inner_kernel_cta1024<false>;
    const void* inner256 = c16 ? (const void*)pcg_mixed_inner_kernel<true> : (const void*)pcg_mixed_inner_kernel<false>;
    // two colours and the row state fits one CTA per SM: the resident form
    size_t dsm = 0;
    if (a.f.colours == 2 && a.sellStart && ws.gridInner1024 > 0 && ws.residentMaxBytes > 0) {
        const size_t need = resident_bytes(a.f, ws.gridInner1024);
        if (need <= ws.residentMaxBytes) {
            inner1024 = h16   ? (const void*)pcg_mixed_inner_kernel_resident<true, true>
                        : c16 ? (const void*)pcg_mixed_inner_kernel_resident<true>
                              : (const void*)pcg_mixed_inner_kernel_resident<false>;
            dsm = need;
        }
    }
    split_launch(ws, a, (const void*)pcg_mixed_refresh_kernel, kRingBytes, inner1024, inner256, s, dsm);
    if (!(inner1024 && ws.gridInner1024 > 0 && a.sellStart)) return 0;
    return dsm > 0 ? 2 : 1;
}

// The FP64 solver's persistent grid for `device`, by the same rule as cg_configure, touching no device memory.
int cg_fp64_grid(int device, int* block) {
    int sms = 0, coop = 0;
    NSF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    NSF_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
    if (!coop) throw Error{NSF_ERR_NO_DEVICE, "device does not support cooperative launches"};
    const int perSm = std::min(2, cg_occupancy());
    if (perSm < 1) throw Error{NSF_ERR_CUDA, "CG kernel cannot be resident"};
    *block = kCgThreads;
    return sms * perSm;
}

// Launches the FP64 solver with caller-provided workspace pointers (everything in `a` already set).
void cg_launch_fp64_raw(const CgArgs& args, int grid, int block, cudaStream_t s) {
    NSF_CUDA(cudaMemsetAsync(args.sync, 0, sizeof(GridSync), s));
    CgArgs a = args;
    void* params[] = {&a};
    NSF_CUDA(cudaLaunchCooperativeKernel((const void*)cg_fp64_kernel<false>, dim3(grid), dim3(block), params, 0, s));
    count_launch();
}

}  // namespace nsf
