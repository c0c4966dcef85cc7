// Persistent conjugate-gradient megakernels for sm_103a.
//
// Replaces the reference's conjugateGradientMegakernel (gpu/matrix_math.cu:251-286, host driver
// cpp/gpu_simulation_device.cpp:385-515): one cooperative launch runs the whole CG loop on the device.
// Differences from the reference, by design:
//   * 2 grid-wide barriers per iteration instead of 4.  The search direction of iteration k is never
//     materialised before the SpMV: the SpMV gathers p_j = r_j + beta*p_prev_j on the fly from a
//     double-buffered p, and each row's owner stores the identical fma result for the axpy phase.
//   * deterministic reductions: warp xor-shuffle -> per-block partial -> after the barrier every block sums the
//     partials in one fixed order, so all blocks hold bit-identical alpha/beta (the reference uses float
//     atomicAdd, gpu/matrix_math.cu:163-193);
//   * every barrier wait is bounded by %globaltimer; on expiry the kernel raises an abort word, every block
//     leaves, and the host reports NSF_ERR_BARRIER_TIMEOUT (the reference's spin barrier can deadlock);
//   * stopping rule ||r|| <= tol*||b|| (relative), FP64 vectors and scalars;
//   * optional fused right-hand side: b_i = mask_i ? g_i : (B x_b)_i - lift_i is built in the prologue, so the
//     diffusion and pressure right-hand sides of the operator-split step (include/assembly.h:497-523, 575-595)
//     cost no extra launch or pass.
// The mixed-precision form keeps FP32 matrix values and FP32 vectors in an inner CG (FP64 dots and scalars)
// inside an FP64 iterative-refinement loop whose true residual b - A x is recomputed with the FP64 matrix.
#include "nsf_internal.cuh"

#include <cooperative_groups.h>

namespace nsf {

constexpr int kCgThreads = 512;
constexpr int kGroup = 4;   // lanes that share one CSR row in the SpMV phases

// ---------------------------------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_add_release(unsigned long long* p, unsigned long long v) {
    asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ long long global_ns() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }

// streaming loads for the matrix (read once per iteration; keep L2 for the gathered vectors)
__device__ __forceinline__ int ld_stream(const int* p) { return __ldcs(p); }
__device__ __forceinline__ double ld_stream(const double* p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float* p) { return __ldcs(p); }

// Grid barrier: monotone arrival counter, one arrival per block, bounded wait.
struct GridBarrier {
    GridSync* s;
    unsigned long long target;
    unsigned long long nblocks;
    long long timeoutNs;

    __device__ bool sync(int where) {
        __shared__ int ok;
        __syncthreads();
        if (threadIdx.x == 0) {
            target += nblocks;
            __threadfence();
            red_add_release(&s->arrived, 1ULL);
            int res = 1;
            const long long t0 = global_ns();
            while (ld_acquire(&s->arrived) < target) {
                if (ld_volatile(&s->abort)) { res = 0; break; }
                if (global_ns() - t0 >= timeoutNs) {
                    if (atomicCAS(&s->abort, 0, 1) == 0) s->where = where;
                    res = 0;
                    break;
                }
            }
            __threadfence();
            ok = res;
        }
        __syncthreads();
        return ok != 0;
    }
};

// Sum of one double over the block; result valid in thread 0.  Fixed order -> deterministic.
__device__ double block_sum(double v, double* smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += smem[w];
    __syncthreads();
    return t;
}

// Sum of the per-block partials of one region, identical in every block and thread.
__device__ double grid_sum(const double* part, int G, double* smem) {
    double v = 0;
    if (threadIdx.x < 32) {
        for (int i = threadIdx.x; i < G; i += 32) v += part[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) smem[32] = v;
    }
    __syncthreads();
    v = smem[32];
    __syncthreads();
    return v;
}

__device__ __forceinline__ unsigned group_mask() { return 0xFu << ((threadIdx.x & 31) & ~(kGroup - 1)); }

template <typename T> __device__ __forceinline__ T group_reduce(T v) {
    const unsigned m = group_mask();
    v += __shfl_xor_sync(m, v, 1);
    v += __shfl_xor_sync(m, v, 2);
    return v;
}

// Row-range of this block: contiguous chunks keep each block's gathers local.
__device__ __forceinline__ void block_rows(int n, int& rb, int& re) {
    const int chunk = (n + gridDim.x - 1) / gridDim.x;
    rb = min(n, (int)blockIdx.x * chunk);
    re = min(n, rb + chunk);
}

// Fused right-hand side of one row (4-lane group): mask ? g : (B x_b)_row - lift_row
__device__ __forceinline__ double rhs_row(const CgArgs& a, int row, int sub) {
    double acc = 0;
    const int s = a.bRowptr[row], e = a.bRowptr[row + 1];
    for (int k = s + sub; k < e; k += kGroup) acc = fma(ld_stream(a.bVal + k), a.bX[ld_stream(a.bCol + k)], acc);
    acc = group_reduce(acc);
    if (a.bcMask && a.bcMask[row]) return a.bcValue[row];
    return a.lift ? acc - a.lift[row] : acc;
}

__device__ void write_info(const CgArgs& a, int it, int status, int outer, double rr, double bb) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.info->iterations = it;
        a.info->status = status;
        a.info->outer = outer;
        a.info->rr = rr;
        a.info->bb = bb;
    }
}

// ---------------------------------------------------------------------------------------------------
// FP64 persistent CG
// partial regions: 0 = p.q, 1 = r.r, 2 = r0.r0, 3 = b.b
// ---------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kCgThreads) cg_fp64_kernel(CgArgs a) {
    __shared__ double smem[33];
    const int G = gridDim.x;
    GridBarrier bar{a.sync, 0ULL, (unsigned long long)G, a.timeoutNs};
    int rb, re;
    block_rows(a.n, rb, re);
    const int sub = threadIdx.x & (kGroup - 1);
    const int grp = threadIdx.x / kGroup;
    const int ngrp = blockDim.x / kGroup;
    const bool fusedRhs = a.bRowptr != nullptr;
    const double* b = fusedRhs ? a.bOut : a.b;

    // prologue: (b), x = x0, r0 = b - A x0, p0 = r0
    double rrp = 0, bbp = 0;
    for (int row = rb + grp; row < re; row += ngrp) {
        double bi;
        if (fusedRhs) {
            bi = rhs_row(a, row, sub);
            if (sub == 0 && a.bOut) a.bOut[row] = bi;
        } else {
            bi = a.b[row];
        }
        double acc = 0;
        const int s = a.rowptr[row], e = a.rowptr[row + 1];
        for (int k = s + sub; k < e; k += kGroup) acc = fma(ld_stream(a.val + k), a.x0[ld_stream(a.col + k)], acc);
        acc = group_reduce(acc);
        if (sub == 0) {
            const double ri = bi - acc;
            a.r[row] = ri;
            a.pbuf0[row] = ri;
            if (a.x != a.x0) a.x[row] = a.x0[row];
            rrp = fma(ri, ri, rrp);
            bbp = fma(bi, bi, bbp);
        }
    }
    rrp = block_sum(rrp, smem);
    bbp = block_sum(bbp, smem);
    if (threadIdx.x == 0) { a.partials[2 * G + blockIdx.x] = rrp; a.partials[3 * G + blockIdx.x] = bbp; }
    if (!bar.sync(1)) { write_info(a, 0, NSF_ERR_BARRIER_TIMEOUT, 1, 0, 0); return; }
    double rr = grid_sum(a.partials + 2 * G, G, smem);
    const double bb = grid_sum(a.partials + 3 * G, G, smem);
    const double target = bb > 0 ? a.tol2 * bb : a.tol2 * rr;
    (void)b;

    int it = 0, status = NSF_ERR_NOT_CONVERGED;
    if (!(rr == rr) || !(bb == bb) || isinf(rr) || isinf(bb)) status = NSF_ERR_BREAKDOWN;
    else if (rr <= target) status = NSF_OK;
    double beta = 0.0;
    double* pprev = a.pbuf0;
    double* pcur = a.pbuf1;
    while (status == NSF_ERR_NOT_CONVERGED && it < a.maxIt) {
        // phase A: p = r + beta p_prev (own rows), q = A p (p gathered on the fly), partial p.q
        double pq = 0;
        for (int row = rb + grp; row < re; row += ngrp) {
            double acc = 0;
            const int s = a.rowptr[row], e = a.rowptr[row + 1];
            for (int k = s + sub; k < e; k += kGroup) {
                const int c = ld_stream(a.col + k);
                const double pj = fma(beta, pprev[c], a.r[c]);
                acc = fma(ld_stream(a.val + k), pj, acc);
            }
            acc = group_reduce(acc);
            if (sub == 0) {
                const double pi = fma(beta, pprev[row], a.r[row]);
                pcur[row] = pi;
                a.q[row] = acc;
                pq = fma(pi, acc, pq);
            }
        }
        pq = block_sum(pq, smem);
        if (threadIdx.x == 0) a.partials[blockIdx.x] = pq;
        if (!bar.sync(2)) { write_info(a, it, NSF_ERR_BARRIER_TIMEOUT, 1, rr, bb); return; }
        const double pqs = grid_sum(a.partials, G, smem);
        if (!(pqs > 0.0) || isinf(pqs)) { status = NSF_ERR_BREAKDOWN; break; }
        const double alpha = rr / pqs;
        // phase B: x += alpha p, r -= alpha q, partial r.r
        double rrn = 0;
        for (int i = rb + (int)threadIdx.x; i < re; i += blockDim.x) {
            const double pi = pcur[i], qi = a.q[i];
            a.x[i] = fma(alpha, pi, a.x[i]);
            const double ri = fma(-alpha, qi, a.r[i]);
            a.r[i] = ri;
            rrn = fma(ri, ri, rrn);
        }
        rrn = block_sum(rrn, smem);
        if (threadIdx.x == 0) a.partials[G + blockIdx.x] = rrn;
        if (!bar.sync(3)) { write_info(a, it, NSF_ERR_BARRIER_TIMEOUT, 1, rr, bb); return; }
        const double rrs = grid_sum(a.partials + G, G, smem);
        ++it;
        if (!(rrs == rrs) || isinf(rrs)) { status = NSF_ERR_BREAKDOWN; break; }
        beta = rrs / rr;
        rr = rrs;
        if (rr <= target) { status = NSF_OK; break; }
        double* t = pprev; pprev = pcur; pcur = t;
    }
    write_info(a, it, status, 1, rr, bb);
}

// ---------------------------------------------------------------------------------------------------
// Mixed precision: FP64 iterative refinement around an FP32 inner CG (FP64 dots/scalars)
// partial regions: 0 = p.q (inner), 1 = r.r (inner), 2 = r64.r64, 3 = b.b, 4 = r32.r32 (inner start)
// ---------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kCgThreads) cg_mixed_kernel(CgArgs a) {
    __shared__ double smem[33];
    const int G = gridDim.x;
    GridBarrier bar{a.sync, 0ULL, (unsigned long long)G, a.timeoutNs};
    int rb, re;
    block_rows(a.n, rb, re);
    const int sub = threadIdx.x & (kGroup - 1);
    const int grp = threadIdx.x / kGroup;
    const int ngrp = blockDim.x / kGroup;
    const bool fusedRhs = a.bRowptr != nullptr;

    // x = x0 (own rows); neighbours read x0 in the first residual pass, so no barrier is needed here
    if (a.x != a.x0)
        for (int i = rb + (int)threadIdx.x; i < re; i += blockDim.x) a.x[i] = a.x0[i];

    int it = 0, outer = 0, status = NSF_ERR_NOT_CONVERGED;
    double rr64 = 0, bb = 0, target = 0;
    int where = 10;
    while (true) {
        // R phase: r = b - A64 x (x0 on the first pass), r32 = (float) r, d = 0
        const double* xs = outer == 0 ? a.x0 : a.x;
        double rrp = 0, bbp = 0, rip = 0;
        for (int row = rb + grp; row < re; row += ngrp) {
            double bi;
            if (fusedRhs && outer == 0) {
                bi = rhs_row(a, row, sub);
                if (sub == 0) a.bOut[row] = bi;
            } else {
                bi = fusedRhs ? a.bOut[row] : a.b[row];
            }
            double acc = 0;
            const int s = a.rowptr[row], e = a.rowptr[row + 1];
            for (int k = s + sub; k < e; k += kGroup) acc = fma(ld_stream(a.val + k), xs[ld_stream(a.col + k)], acc);
            acc = group_reduce(acc);
            if (sub == 0) {
                const double ri = bi - acc;
                const float r32 = (float)ri;
                a.r32[row] = r32;
                a.p32a[row] = r32;
                a.d32[row] = 0.0f;
                rrp = fma(ri, ri, rrp);
                bbp = fma(bi, bi, bbp);
                rip = fma((double)r32, (double)r32, rip);
            }
        }
        rrp = block_sum(rrp, smem);
        bbp = block_sum(bbp, smem);
        rip = block_sum(rip, smem);
        if (threadIdx.x == 0) {
            a.partials[2 * G + blockIdx.x] = rrp;
            a.partials[3 * G + blockIdx.x] = bbp;
            a.partials[4 * G + blockIdx.x] = rip;
        }
        if (!bar.sync(where++)) { write_info(a, it, NSF_ERR_BARRIER_TIMEOUT, outer, rr64, bb); return; }
        rr64 = grid_sum(a.partials + 2 * G, G, smem);
        if (outer == 0) {
            bb = grid_sum(a.partials + 3 * G, G, smem);
            target = bb > 0 ? a.tol2 * bb : a.tol2 * rr64;
        }
        double rr = grid_sum(a.partials + 4 * G, G, smem);
        if (!(rr64 == rr64) || isinf(rr64)) { status = NSF_ERR_BREAKDOWN; break; }
        if (rr64 <= target) { status = NSF_OK; break; }
        if (outer >= a.maxOuter || it >= a.maxIt) break;
        ++outer;

        // inner FP32 CG on A32 d = r32 to a relative reduction innerTol
        const double innerTarget = a.innerTol2 * rr;
        double beta = 0.0;
        float* pprev = a.p32a;
        float* pcur = a.p32b;
        bool innerBreak = false;
        while (it < a.maxIt) {
            const float betaf = (float)beta;
            double pq = 0;
            for (int row = rb + grp; row < re; row += ngrp) {
                float acc = 0.f;
                const int s = a.rowptr[row], e = a.rowptr[row + 1];
                for (int k = s + sub; k < e; k += kGroup) {
                    const int c = ld_stream(a.col + k);
                    const float pj = fmaf(betaf, pprev[c], a.r32[c]);
                    acc = fmaf(ld_stream(a.val32 + k), pj, acc);
                }
                acc = group_reduce(acc);
                if (sub == 0) {
                    const float pi = fmaf(betaf, pprev[row], a.r32[row]);
                    pcur[row] = pi;
                    a.q32[row] = acc;
                    pq = fma((double)pi, (double)acc, pq);
                }
            }
            pq = block_sum(pq, smem);
            if (threadIdx.x == 0) a.partials[blockIdx.x] = pq;
            if (!bar.sync(where++)) { write_info(a, it, NSF_ERR_BARRIER_TIMEOUT, outer, rr64, bb); return; }
            const double pqs = grid_sum(a.partials, G, smem);
            if (!(pqs > 0.0) || isinf(pqs)) { innerBreak = true; break; }
            const double alpha = rr / pqs;
            const float alphaf = (float)alpha;
            double rrn = 0;
            for (int i = rb + (int)threadIdx.x; i < re; i += blockDim.x) {
                const float pi = pcur[i], qi = a.q32[i];
                a.d32[i] = fmaf(alphaf, pi, a.d32[i]);
                const float ri = fmaf(-alphaf, qi, a.r32[i]);
                a.r32[i] = ri;
                rrn = fma((double)ri, (double)ri, rrn);
            }
            rrn = block_sum(rrn, smem);
            if (threadIdx.x == 0) a.partials[G + blockIdx.x] = rrn;
            if (!bar.sync(where++)) { write_info(a, it, NSF_ERR_BARRIER_TIMEOUT, outer, rr64, bb); return; }
            const double rrs = grid_sum(a.partials + G, G, smem);
            ++it;
            if (!(rrs == rrs) || isinf(rrs)) { innerBreak = true; break; }
            beta = rrs / rr;
            rr = rrs;
            if (rr <= innerTarget) break;
            float* t = pprev; pprev = pcur; pcur = t;
        }
        // x += d (FP64), then the next true residual needs every block's update
        for (int i = rb + (int)threadIdx.x; i < re; i += blockDim.x) a.x[i] += (double)a.d32[i];
        if (!bar.sync(where++)) { write_info(a, it, NSF_ERR_BARRIER_TIMEOUT, outer, rr64, bb); return; }
        if (innerBreak && it >= a.maxIt) break;
    }
    write_info(a, it, status, outer, rr64, bb);
}

// ---------------------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------------------
void cg_configure(CgWorkspace& ws, int device) {
    int sms = 0, coop = 0;
    NSF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    NSF_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
    if (!coop) throw Error{NSF_ERR_NO_DEVICE, "device does not support cooperative launches"};
    int occ64 = 0, occMixed = 0;
    NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ64, cg_fp64_kernel, kCgThreads, 0));
    NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occMixed, cg_mixed_kernel, kCgThreads, 0));
    const int perSm = std::min(2, std::min(occ64, occMixed));
    if (perSm < 1) throw Error{NSF_ERR_CUDA, "CG kernel cannot be resident"};
    ws.grid = sms * perSm;
    ws.block = kCgThreads;
    ws.partials.alloc((size_t)6 * ws.grid);
    ws.sync.alloc(1);
    ws.info.alloc(4096);
}

void cg_launch(CgWorkspace& ws, const CgArgs& args, int mode, cudaStream_t s) {
    NSF_CUDA(cudaMemsetAsync(ws.sync.get(), 0, sizeof(GridSync), s));
    CgArgs a = args;
    void* params[] = {&a};
    const void* fn = mode == NSF_SOLVER_MIXED ? (const void*)cg_mixed_kernel : (const void*)cg_fp64_kernel;
    NSF_CUDA(cudaLaunchCooperativeKernel(fn, dim3(ws.grid), dim3(ws.block), params, 0, s));
    count_launch();
}

// The FP64 solver's persistent grid for `device`, by the same rule as cg_configure, touching no device memory.
int cg_fp64_grid(int device, int* block) {
    int sms = 0, coop = 0, occ64 = 0, occMixed = 0;
    NSF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    NSF_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
    if (!coop) throw Error{NSF_ERR_NO_DEVICE, "device does not support cooperative launches"};
    NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ64, cg_fp64_kernel, kCgThreads, 0));
    NSF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occMixed, cg_mixed_kernel, kCgThreads, 0));
    const int perSm = std::min(2, std::min(occ64, occMixed));
    if (perSm < 1) throw Error{NSF_ERR_CUDA, "CG kernel cannot be resident"};
    *block = kCgThreads;
    return sms * perSm;
}

// Launches the FP64 solver with caller-provided workspace pointers (everything in `a` already set).
void cg_launch_fp64_raw(const CgArgs& args, int grid, int block, cudaStream_t s) {
    NSF_CUDA(cudaMemsetAsync(args.sync, 0, sizeof(GridSync), s));
    CgArgs a = args;
    void* params[] = {&a};
    NSF_CUDA(cudaLaunchCooperativeKernel((const void*)cg_fp64_kernel, dim3(grid), dim3(block), params, 0, s));
    count_launch();
}

}  // namespace nsf
