// The multi-kernel FP64 conjugate gradient (NSF_CG_FORM_MULTI_KERNEL).
//
// Replaces the reference's conjugateGradientMultiKernel (cpp/gpu_simulation_device.cpp:293-383), the solve its
// conjugateGradient(..., useMegakernel = false) runs: r0 = b - A x0, p0 = r0, then per iteration
// alpha = r.r / p.Ap, x += alpha p, r -= alpha Ap, beta = r'.r' / r.r, p = r' + beta p, stopping when r.r falls
// under the tolerance.  The reference issues six launches per iteration (spRMult, dotProduct, two saxpy,
// dotProduct, saxpby) and synchronises the host twice per iteration to read p.Ap and r.r from mapped memory and
// form alpha and beta there.  Here:
//   * three launches per iteration, each an ordinary (non-cooperative) grid whose boundary is the grid-wide sync:
//     q = A p with the partial sums of p.q; x += alpha p and r -= alpha q with those of r.r; p = r + beta p;
//   * the scalars never leave the device: the last CTA to post its partial sum of a reduction (a counter taken
//     after a memory fence) sums all partials in one fixed order and writes alpha, beta, the iteration count and
//     the stopping state, so every run is deterministic and the next kernel reads them from device memory;
//   * kNsfMultiIters iterations are captured once per solve as a CUDA graph and replayed; after the solve has
//     stopped, its kernels return at once, so the host reads the 48-byte state only once per replay, one replay
//     behind the device (the next replay is already queued);
//   * the same products, chunks and per-row arithmetic as the three-barrier megakernel (cg_fp64_kernel), so the
//     two forms take the same iterations on the same system, and the same relative stopping rule.
// It is the ablation the reference keeps beside its megakernel; the persistent kernels stay the default.
#include "nsf_device.cuh"

namespace nsf {

constexpr int kNsfMultiIters = 8;   // iterations per graph replay

namespace {

// Every CTA posts its partial sums, then counts itself in; true in the CTA that arrived last, which then sees
// every other CTA's partials (each was written before that CTA's fence and count).
__device__ bool last_cta(unsigned int* arrived) {
    __shared__ int last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int prev = atomicAdd(arrived, 1u);
        last = prev == gridDim.x - 1;
        if (last) __threadfence();
    }
    __syncthreads();
    return last != 0;
}

__device__ __forceinline__ Team multi_team(const CgArgs& a) {
    return Team{nullptr, a.partials, (int)gridDim.x, (int)blockIdx.x, 0ULL, 0LL};
}

// (b), x = x0, r = b - A x0, p = r; the last CTA forms r.r and b.b and the stopping target.
template <bool Wide>
__global__ void __launch_bounds__(kCgThreads, 2) cg_multi_start_kernel(CgArgs a, CgMultiState* st) {
    NSF_KERNEL_SHARED();
    const Team t = multi_team(a);
    const int G = t.size;
    int rb, re;
    team_rows(a.n, t, rb, re);
    const double* b = a.bRowptr ? a.bOut : a.b;
    build_rhs<Wide>(a, rb, re, stage);
    double rrp = 0, bbp = 0;
    matrix_product<double, double, false, kResidU<Wide>, Wide>(
        a.sellStart, a.sellCol, a.sellVal, a.rowptr, a.col, a.val, rb, re, stage, [&](int c) { return a.x0[c]; },
        [&](int row, double acc, double x0i) {
            const double bi = b[row];
            const double ri = bi - acc;
            a.r[row] = ri;
            a.pbuf0[row] = ri;
            if (a.x != a.x0) a.x[row] = x0i;
            rrp = fma(ri, ri, rrp);
            bbp = fma(bi, bi, bbp);
        });
    rrp = block_sum(rrp, smem);
    bbp = block_sum(bbp, smem);
    if (threadIdx.x == 0) { a.partials[2 * G + t.rank] = rrp; a.partials[3 * G + t.rank] = bbp; }
    if (!last_cta(&st->arrived)) return;
    const double rr = grid_sum(a.partials + 2 * G, G, smem);
    const double bb = grid_sum(a.partials + 3 * G, G, smem);
    if (threadIdx.x == 0) {
        const double target = bb > 0 ? a.tol2 * bb : a.tol2 * rr;
        int status = NSF_ERR_NOT_CONVERGED;
        if (!(rr == rr) || !(bb == bb) || isinf(rr) || isinf(bb)) status = NSF_ERR_BREAKDOWN;
        else if (rr <= target) status = NSF_OK;
        st->rr = rr;
        st->bb = bb;
        st->target = target;
        st->it = 0;
        st->maxIt = a.maxIt;
        st->status = status;
        st->done = status != NSF_ERR_NOT_CONVERGED || a.maxIt <= 0;
        st->arrived = 0;
    }
}

// q = A p and p.q; the last CTA forms alpha = r.r / p.q (or stops the solve on a breakdown).
template <bool Wide>
__global__ void __launch_bounds__(kCgThreads, 2) cg_multi_product_kernel(CgArgs a, CgMultiState* st) {
    NSF_KERNEL_SHARED();
    if (ld_volatile(&st->done)) return;   // the same value in every CTA: it was written by an earlier kernel
    const Team t = multi_team(a);
    int rb, re;
    team_rows(a.n, t, rb, re);
    const double* p = a.pbuf0;
    double pq = 0;
    auto gq = [&](int c) { return p[c]; };
    auto eq = [&](int row, double acc, double pr) {
        a.q[row] = acc;
        pq = fma(pr, acc, pq);
    };
    if (!Wide && a.sellMaxW <= 5)
        matrix_product<double, double, false, 5, Wide>(a.sellStart, a.sellCol, a.sellVal, a.rowptr, a.col, a.val, rb,
                                                       re, stage, gq, eq);
    else
        matrix_product<double, double, false, kUnroll, Wide>(a.sellStart, a.sellCol, a.sellVal, a.rowptr, a.col,
                                                             a.val, rb, re, stage, gq, eq);
    pq = block_sum(pq, smem);
    if (threadIdx.x == 0) a.partials[t.rank] = pq;
    if (!last_cta(&st->arrived)) return;
    const double pqs = grid_sum(a.partials, t.size, smem);
    if (threadIdx.x == 0) {
        if (!(pqs > 0.0) || isinf(pqs)) {
            st->status = NSF_ERR_BREAKDOWN;
            st->done = 1;
        } else {
            st->alpha = st->rr / pqs;
        }
        st->arrived = 0;
    }
}

// x += alpha p, r -= alpha q and r.r; the last CTA counts the iteration, forms beta and applies the stopping rule.
__global__ void __launch_bounds__(kCgThreads, 2) cg_multi_update_kernel(CgArgs a, CgMultiState* st) {
    NSF_KERNEL_SHARED();
    (void)stage;
    if (ld_volatile(&st->done)) return;
    const Team t = multi_team(a);
    int rb, re;
    team_rows(a.n, t, rb, re);
    const double alpha = st->alpha;
    const double* p = a.pbuf0;
    const int bs = blockDim.x;
    double rrn = 0;
    for (int i0 = rb + (int)threadIdx.x; i0 < re; i0 += kRows * bs) {
        double pi[kRows], qi[kRows], xi[kRows], ri[kRows];
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
            const int i = i0 + u * bs;
            if (i < re) { pi[u] = p[i]; qi[u] = a.q[i]; xi[u] = a.x[i]; ri[u] = a.r[i]; }
        }
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
            const int i = i0 + u * bs;
            if (i < re) {
                a.x[i] = fma(alpha, pi[u], xi[u]);
                const double rn = fma(-alpha, qi[u], ri[u]);
                a.r[i] = rn;
                rrn = fma(rn, rn, rrn);
            }
        }
    }
    rrn = block_sum(rrn, smem);
    if (threadIdx.x == 0) a.partials[t.size + t.rank] = rrn;
    if (!last_cta(&st->arrived)) return;
    const double rrs = grid_sum(a.partials + t.size, t.size, smem);
    if (threadIdx.x == 0) {
        const int it = st->it + 1;
        st->it = it;
        if (!(rrs == rrs) || isinf(rrs)) {
            st->status = NSF_ERR_BREAKDOWN;
            st->done = 1;
        } else {
            st->beta = rrs / st->rr;
            st->rr = rrs;
            if (rrs <= st->target) {
                st->status = NSF_OK;
                st->done = 1;
            } else if (it >= st->maxIt) {
                st->done = 1;   // status stays NSF_ERR_NOT_CONVERGED
            }
        }
        st->arrived = 0;
    }
}

// p = r + beta p.
__global__ void __launch_bounds__(kCgThreads, 2) cg_multi_direction_kernel(CgArgs a, CgMultiState* st) {
    if (ld_volatile(&st->done)) return;
    const Team t = multi_team(a);
    int rb, re;
    team_rows(a.n, t, rb, re);
    const double beta = st->beta;
    double* p = a.pbuf0;
    const int bs = blockDim.x;
    for (int i0 = rb + (int)threadIdx.x; i0 < re; i0 += kRows * bs) {
        double pi[kRows], ri[kRows];
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
            const int i = i0 + u * bs;
            if (i < re) { pi[u] = p[i]; ri[u] = a.r[i]; }
        }
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
            const int i = i0 + u * bs;
            if (i < re) p[i] = fma(beta, pi[u], ri[u]);
        }
    }
}

// The solve's record in the handle's info ring, as the persistent kernels write it.
__global__ void cg_multi_finish_kernel(const CgMultiState* st, CgInfo* info) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    info->iterations = st->it;
    info->status = st->status;
    info->outer = 1;
    info->fallback = 0;
    info->rr = st->rr;
    info->bb = st->bb;
}

// Ends a stream capture that an exception left open, so the handle's stream stays usable.
struct CaptureGuard {
    cudaStream_t s;
    bool open = true;
    ~CaptureGuard() {
        if (open) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(s, &g);
            if (g) cudaGraphDestroy(g);
        }
    }
};

struct GraphGuard {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t e = nullptr;
    ~GraphGuard() {
        if (e) cudaGraphExecDestroy(e);   // (a replay still in flight is released when it completes)
        if (g) cudaGraphDestroy(g);
    }
};

}  // namespace

void cg_multi_launch(CgWorkspace& ws, const CgArgs& args, bool wide, cudaStream_t s) {
    CgArgs a = args;
    if (!ws.multi.get()) ws.multi.alloc(1);
    CgMultiHost& hs = ws.multiHost;
    if (!hs.slot) {
        NSF_CUDA(cudaHostAlloc((void**)&hs.slot, 2 * sizeof(CgMultiState), cudaHostAllocDefault));
        for (cudaEvent_t& e : hs.ev) NSF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    CgMultiState* st = ws.multi.get();
    const dim3 grid(ws.grid), block(ws.block);
    NSF_CUDA(cudaMemsetAsync(st, 0, sizeof(CgMultiState), s));
    if (wide) cg_multi_start_kernel<true><<<grid, block, 0, s>>>(a, st);
    else cg_multi_start_kernel<false><<<grid, block, 0, s>>>(a, st);
    NSF_CUDA(cudaGetLastError());
    count_launch();

    // kNsfMultiIters iterations, captured once for this solve's arguments
    GraphGuard gg;
    {
        CaptureGuard cap{s};
        NSF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < kNsfMultiIters; ++k) {
            if (wide) cg_multi_product_kernel<true><<<grid, block, 0, s>>>(a, st);
            else cg_multi_product_kernel<false><<<grid, block, 0, s>>>(a, st);
            cg_multi_update_kernel<<<grid, block, 0, s>>>(a, st);
            cg_multi_direction_kernel<<<grid, block, 0, s>>>(a, st);
        }
        NSF_CUDA(cudaGetLastError());
        cap.open = false;
        NSF_CUDA(cudaStreamEndCapture(s, &gg.g));
    }
    NSF_CUDA(cudaGraphInstantiate(&gg.e, gg.g, 0));

    // every iteration the solve may take lies within maxReplays replays, and the last of them stops it
    const long long maxReplays = ((long long)std::max(a.maxIt, 0) + kNsfMultiIters - 1) / kNsfMultiIters;
    long long issued = 0, checked = 0;
    auto issue = [&] {
        const int k = (int)(issued & 1);
        NSF_CUDA(cudaGraphLaunch(gg.e, s));
        count_launch(3 * kNsfMultiIters);
        NSF_CUDA(cudaMemcpyAsync(hs.slot + k, st, sizeof(CgMultiState), cudaMemcpyDeviceToHost, s));
        NSF_CUDA(cudaEventRecord(hs.ev[k], s));
        ++issued;
    };
    if (maxReplays > 0) {
        // the start kernel may already have stopped the solve: its state decides whether any replay runs
        NSF_CUDA(cudaMemcpyAsync(hs.slot, st, sizeof(CgMultiState), cudaMemcpyDeviceToHost, s));
        NSF_CUDA(cudaStreamSynchronize(s));
        if (!hs.slot[0].done) issue();
    }
    while (checked < issued) {
        if (issued < maxReplays) issue();   // keep the next replay queued while this one is checked
        const int k = (int)(checked & 1);
        NSF_CUDA(cudaEventSynchronize(hs.ev[k]));
        const bool done = hs.slot[k].done != 0;
        ++checked;
        if (done) break;
    }
    cg_multi_finish_kernel<<<1, 32, 0, s>>>(st, a.info);
    NSF_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace nsf
