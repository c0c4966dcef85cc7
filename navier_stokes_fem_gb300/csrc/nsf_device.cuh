// Device-side building blocks of the persistent CG solvers, shared by the single-solve kernels (nsf_cg.cu) and
// the persistent operator-split step kernel (nsf_step.cu).  See nsf_cg.cu for the design notes.
#pragma once
#include "nsf_internal.cuh"

namespace nsf {

constexpr int kCgThreads = 512;
constexpr int kWarps = kCgThreads / 32;
constexpr int kStage = 128;   // staged (value, gathered x) pairs per warp
constexpr int kMaxInnerBetweenRefresh = 4000;   // mixed precision: FP32 iterations between FP64 true residuals

// TMA bulk-copy pipeline of the streamed SpMV: kPipe stages, each a contiguous slice of the CTA's column
// indices and values (kStreamBytes per stage).  The dynamic shared memory of every CG kernel is kPipe stages
// (the warp-chunked SpMV's staging area reuses the same bytes in other phases).
constexpr int kPipe = 3;
constexpr int kStreamBytes = 32768;
constexpr int kDynSmem = kPipe * kStreamBytes;
static_assert(kWarps * 2 * kStage * (int)sizeof(double) <= kDynSmem, "staging area must fit the stream buffers");

// ---------------------------------------------------------------------------------------------------
// memory-model and timing helpers
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

// A team: `size` consecutive CTAs of a persistent launch that cooperate on one system (the whole grid for a
// single solve; a share of the grid per instance in the batched step).  Its barrier is a monotone arrival
// counter with one arrival per CTA and a bounded wait; a one-CTA team needs only __syncthreads.
struct Team {
    GridSync* sync;
    double* partials;   // kPartialRegions slots of `size` entries each
    int size;
    int rank;
    unsigned long long target;
    long long timeoutNs;

    static __device__ Team grid(GridSync* s, double* partials, long long timeoutNs) {
        return Team{s, partials, (int)gridDim.x, (int)blockIdx.x, 0ULL, timeoutNs};
    }

    __device__ bool barrier(int where) {
        __shared__ int ok;
        if (size == 1) {
            __syncthreads();
            return true;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            target += (unsigned long long)size;
            __threadfence();
            red_add_release(&sync->arrived, 1ULL);
            int res = 1;
            const long long t0 = global_ns();
            while (ld_acquire(&sync->arrived) < target) {
                if (ld_volatile(&sync->abort)) { res = 0; break; }
                if (global_ns() - t0 >= timeoutNs) {
                    if (atomicCAS(&sync->abort, 0, 1) == 0) sync->where = where;
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
static __device__ double block_sum(double v, double* smem) {
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
static __device__ double grid_sum(const double* part, int G, double* smem) {
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

// Row-range of this CTA within its team: contiguous chunks keep each CTA's gathers local.
__device__ __forceinline__ void team_rows(int n, const Team& t, int& rb, int& re) {
    const int chunk = (n + t.size - 1) / t.size;
    rb = min(n, t.rank * chunk);
    re = min(n, rb + chunk);
}

// Warp-chunked CSR product over rows [rb, re) of this block.  Warps take 32 consecutive rows at a time; the
// rows' non-zeros are contiguous, so the warp loads them with coalesced loads, four per lane in flight before
// any is used, and stages each entry's value and gathered vector element in shared memory (kStage entries per
// warp).  Each lane then sums its own row in entry order with one fused multiply-add per non-zero - on GB300 the
// FP64 pipe (about 2 DFMA per cycle per SM) is as tight as HBM, so no other FP64 work is done per non-zero.
// gather(c) yields the vector entry of column c; epi(row, sum) runs on the lane owning `row`.
// With Diff = true the product is taken in difference form, sum_j a_ij (x_j - x_i): the lane subtracts its own
// row's entry before multiplying (the diagonal term vanishes), and epi adds rowsum_i * x_i.  For matrices whose
// rows sum to (almost) zero - stiffness matrices - this removes the catastrophic cancellation of the plain sum on
// smooth vectors, so an FP32 product stays accurate on the smallest eigenmodes; and because the rounded operator
// keeps the exact row sums, its rounding error annihilates constants.
template <typename TV, typename TA, bool Diff = false, typename Gather, typename Epi>
__device__ __forceinline__ void warp_spmv(const int* __restrict__ rowptr, const int* __restrict__ col,
                                          const TV* __restrict__ val, int rb, int re, TA* stage, Gather gather,
                                          Epi epi) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    TA* sv = stage + warp * (2 * kStage);
    TA* sg = sv + kStage;
    for (int r0 = rb + warp * 32; r0 < re; r0 += nwarps * 32) {
        const int nrows = min(32, re - r0);
        const int row = r0 + lane;
        const bool own = lane < nrows;
        const int s = own ? rowptr[row] : 0;
        const int cEnd = rowptr[r0 + nrows];
        const int sNext = __shfl_down_sync(0xffffffffu, s, 1);
        const int e = lane + 1 < nrows ? sNext : cEnd;
        const int cBeg = __shfl_sync(0xffffffffu, s, 0);
        const TA self = (Diff && own) ? gather(row) : TA(0);
        TA acc = TA(0);
        for (int base = cBeg; base < cEnd; base += kStage) {
            const int cnt = min(kStage, cEnd - base);
            int c[kStage / 32];
            TV v[kStage / 32];
#pragma unroll
            for (int u = 0; u < kStage / 32; ++u) {
                const int k = u * 32 + lane;
                const bool in = k < cnt;
                c[u] = in ? ld_stream(col + base + k) : -1;
                v[u] = in ? ld_stream(val + base + k) : TV(0);
            }
#pragma unroll
            for (int u = 0; u < kStage / 32; ++u) {
                const int k = u * 32 + lane;
                if (c[u] >= 0) {
                    sg[k] = gather(c[u]);
                    sv[k] = TA(v[u]);
                }
            }
            __syncwarp();
            if (own) {
                const int a0 = max(s, base), a1 = min(e, base + cnt);
                if (Diff)
                    for (int k = a0; k < a1; ++k) acc = fma(sv[k - base], sg[k - base] - self, acc);
                else
                    for (int k = a0; k < a1; ++k) acc = fma(sv[k - base], sg[k - base], acc);
            }
            __syncwarp();
        }
        if (own) epi(row, acc);
    }
}

// ---------------------------------------------------------------------------------------------------
// Streamed SpMV: the CTA's column indices and values arrive in shared memory through TMA bulk copies
// (cp.async.bulk, completion on an mbarrier), kPipe stages in flight, so the matrix stream needs no registers
// and no dependent loads; threads only read row pointers, gather the vector and sum from shared memory.
// ---------------------------------------------------------------------------------------------------
template <typename TV> __host__ __device__ constexpr int stream_entries() {
    return (int)((kStreamBytes / (4 + sizeof(TV))) / 4) * 4;
}

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Per-CTA state of the copy pipeline; `seq` counts stages over the whole kernel so every buffer's mbarrier
// phase is known without extra state.
struct Stream {
    unsigned long long* bar;   // kPipe mbarriers (shared)
    unsigned char* buf;        // kPipe * kStreamBytes (dynamic shared)
    int* ctl;                  // 2 shared ints: next stage's first row, abort
    double* carry;             // 1 shared double: partial sum of a row that continues into the next stage
    unsigned seq;
    long long timeoutNs;

    __device__ void init() {
        if (threadIdx.x == 0) {
            for (int i = 0; i < kPipe; ++i) mbar_init(bar + i, 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        seq = 0;
        __syncthreads();
    }
};

// Shared memory of a CG kernel: `smem` (reduction slots), the copy pipeline `st` over the kDynSmem dynamic bytes,
// and `stage`, the warp-chunked SpMV's staging area on the same bytes.  Launch with kDynSmem dynamic bytes.
#define NSF_KERNEL_SHARED(timeout)                                                        \
    extern __shared__ __align__(128) unsigned char nsf_dyn[];                              \
    __shared__ double smem[33];                                                            \
    __shared__ unsigned long long nsf_bars[kPipe];                                         \
    __shared__ int nsf_ctl[2];                                                             \
    __shared__ double nsf_carry[2];                                                        \
    Stream st{nsf_bars, nsf_dyn, nsf_ctl, nsf_carry, 0u, (timeout)};                       \
    st.init();                                                                             \
    double* stage = reinterpret_cast<double*>(nsf_dyn)

// Issue the copies of one stage: entries [c0, c1) of col and val (c0 a multiple of 4, c1 - c0 a multiple of 4).
template <typename TV>
__device__ __forceinline__ void stream_issue(Stream& st, unsigned slot, const int* col, const TV* val, int c0, int c1) {
    constexpr int S = stream_entries<TV>();
    unsigned char* base = st.buf + (size_t)slot * kStreamBytes;
    const unsigned n = (unsigned)(c1 - c0);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(st.bar + slot, n * (unsigned)(4 + sizeof(TV)));
    bulk_g2s(base, col + c0, n * 4u, st.bar + slot);
    bulk_g2s(base + (size_t)S * 4, val + c0, n * (unsigned)sizeof(TV), st.bar + slot);
}

// Rows [rb, re) of this CTA: epi(row, sum) for every row, sum = sum_j a_ij gather(j) (or the difference form with
// Diff, see warp_spmv).  Returns false if a copy did not complete within the time limit.
template <typename TV, typename TA, bool Diff, typename Gather, typename Epi>
__device__ bool stream_spmv(Stream& st, const int* __restrict__ rowptr, const int* __restrict__ col,
                            const TV* __restrict__ val, int nnzTotal, int rb, int re, Gather gather, Epi epi) {
    constexpr int S = stream_entries<TV>();
    if (rb >= re) return true;
    const int E0 = rowptr[rb], E1 = rowptr[re];
    const int base0 = E0 & ~3;
    // Bulk copies need 16-byte aligned sources: with an unaligned col or val (a caller's sub-allocation) every
    // entry is read directly.  Entries past the last multiple of 4 are always read directly.
    const bool aligned = ((reinterpret_cast<unsigned long long>(col) | reinterpret_cast<unsigned long long>(val)) &
                          15ULL) == 0;
    const int copyLimit = aligned ? (nnzTotal & ~3) : 0;
    const int nst = (E1 - base0 + S - 1) / S;
    auto copy_range = [&](int s, int& c0, int& c1) {
        c0 = base0 + s * S;
        c1 = min(c0 + S, min((E1 + 3) & ~3, copyLimit));
        if (c1 < c0) c1 = c0;
    };
    // the buffers were last written through the generic proxy (staging of other phases): order those writes
    // before the copies that overwrite them
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    // prologue: stages 0 .. kPipe-2
    if (threadIdx.x == 0) {
        for (int s = 0; s < kPipe - 1 && s < nst; ++s) {
            int c0, c1;
            copy_range(s, c0, c1);
            if (c1 > c0) stream_issue<TV>(st, (st.seq + s) % kPipe, col, val, c0, c1);
            else mbar_expect_tx(st.bar + (st.seq + s) % kPipe, 0);
        }
        st.ctl[0] = rb;
        st.ctl[1] = rb;   // stays put through a stage that no row touches (E0 == E1)
        st.carry[0] = 0.0;
    }
    __syncthreads();
    bool ok = true;
    int s = 0;
    for (; s < nst; ++s) {
        const unsigned g = st.seq + s, slot = g % kPipe, parity = (g / kPipe) & 1;
        if (threadIdx.x == 0 && s + kPipe - 1 < nst) {   // refill the buffer freed by stage s-1
            int c0, c1;
            copy_range(s + kPipe - 1, c0, c1);
            const unsigned sl = (g + kPipe - 1) % kPipe;
            if (c1 > c0) stream_issue<TV>(st, sl, col, val, c0, c1);
            else mbar_expect_tx(st.bar + sl, 0);
        }
        // wait for this stage (bounded)
        {
            const long long t0 = global_ns();
            while (!mbar_test(st.bar + slot, parity)) {
                if (global_ns() - t0 > st.timeoutNs) { ok = false; break; }
            }
        }
        if (__syncthreads_or(!ok)) { ok = false; break; }
        int c0, c1;
        copy_range(s, c0, c1);
        const int ws = max(E0, base0 + s * S), we = min(E1, base0 + (s + 1) * S);
        const int* colS = reinterpret_cast<const int*>(st.buf + (size_t)slot * kStreamBytes);
        const TV* valS = reinterpret_cast<const TV*>(st.buf + (size_t)slot * kStreamBytes + (size_t)S * 4);
        const int first = st.ctl[0];
        for (int r = first + (int)threadIdx.x; r < re; r += blockDim.x) {
            const int rs = rowptr[r];
            if (rs >= we) break;
            const int rend = rowptr[r + 1];
            const int a0 = max(rs, ws), a1 = min(rend, we);
            const TA self = Diff ? gather(r) : TA(0);
            TA acc = (r == first && rs < ws) ? (TA)st.carry[0] : TA(0);
            for (int e = a0; e < a1; ++e) {
                int c;
                TV v;
                if (e < c1) { c = colS[e - c0]; v = valS[e - c0]; }
                else { c = col[e]; v = val[e]; }            // the last few entries of the matrix (alignment)
                if (Diff) acc = fma(TA(v), gather(c) - self, acc);
                else acc = fma(TA(v), gather(c), acc);
            }
            if (rend > we) {                  // continues in the next stage
                st.carry[1] = (double)acc;
                st.ctl[1] = r;
            } else {
                epi(r, acc);
                if (rend == we) st.ctl[1] = r + 1;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            st.ctl[0] = st.ctl[1];
            st.carry[0] = st.carry[1];
        }
        // the next iteration's refill (thread 0) targets the buffer this stage used: everyone is done with it
        __syncthreads();
    }
    if (!ok) {
        // a copy did not land in time: before the CTA leaves, wait (bounded again) for the stages still in flight,
        // s .. min(nst, s + kPipe) - 1, so that no copy writes into shared memory after the kernel ends
        if (threadIdx.x == 0) {
            const int last = min(nst, s + kPipe);
            for (int k = s; k < last; ++k) {
                const unsigned g = st.seq + k;
                const long long t0 = global_ns();
                while (!mbar_test(st.bar + g % kPipe, (g / kPipe) & 1))
                    if (global_ns() - t0 > st.timeoutNs) break;
            }
        }
        __syncthreads();
        return false;
    }
    st.seq += (unsigned)nst;
    {           // rows without entries after the last non-zero of the range (none in assembled matrices)
        for (int r = st.ctl[0] + (int)threadIdx.x; r < re; r += blockDim.x)
            if (rowptr[r] == E1) epi(r, TA(0));
        __syncthreads();
    }
    return ok;
}

static __device__ void write_info(const Team& t, const CgArgs& a, int it, int status, int outer, double rr, double bb) {
    if (t.rank == 0 && threadIdx.x == 0) {
        a.info->iterations = it;
        a.info->status = status;
        a.info->outer = outer;
        a.info->fallback = 0;
        a.info->rr = rr;
        a.info->bb = bb;
    }
}

// A matrix copy that did not land in time: raise the team's abort word (its other CTAs leave at their next
// barrier) and report the timeout status.
static __device__ int stream_timeout(const Team& t, const CgArgs& a, int it, int outer, double rr, double bb) {
    if (threadIdx.x == 0) atomicExch(&t.sync->abort, 1);
    if (threadIdx.x == 0 && t.rank == 0) {
        a.info->iterations = it;
        a.info->status = NSF_ERR_BARRIER_TIMEOUT;
        a.info->outer = outer;
        a.info->fallback = 0;
        a.info->rr = rr;
        a.info->bb = bb;
    }
    return NSF_ERR_BARRIER_TIMEOUT;
}

// b for this block's rows: the given vector, or the fused right-hand side mask ? g : (B x_b) - lift, stored
// to a.bOut by the owning lane (the same lane reads it back in the residual pass).
static __device__ void build_rhs(const CgArgs& a, int rb, int re, double* stage) {
    if (!a.bRowptr) return;
    warp_spmv<double, double>(a.bRowptr, a.bCol, a.bVal, rb, re, stage,
                              [&](int c) { return a.bX[c]; },
                              [&](int row, double acc) {
                                  double bi = a.lift ? acc - a.lift[row] : acc;
                                  if (a.bcMask && a.bcMask[row]) bi = a.bcValue[row];
                                  a.bOut[row] = bi;
                              });
}

// ---------------------------------------------------------------------------------------------------
// FP64 persistent CG
// partial regions: 0 = p.q, 1 = r.r, 2 = r0.r0, 3 = b.b
// ---------------------------------------------------------------------------------------------------
static __device__ int team_cg_fp64(Team& t, const CgArgs& a, double* stage, double* smem, Stream& st) {
    const int G = t.size;
    const int nnzTotal = a.rowptr[a.n];
    int rb, re;
    team_rows(a.n, t, rb, re);
    const double* b = a.bRowptr ? a.bOut : a.b;

    // prologue: (b), x = x0, r0 = b - A x0, p0 = r0
    build_rhs(a, rb, re, stage);
    double rrp = 0, bbp = 0;
    warp_spmv<double, double>(a.rowptr, a.col, a.val, rb, re, stage, [&](int c) { return a.x0[c]; },
                              [&](int row, double acc) {
                                  const double bi = b[row];
                                  const double ri = bi - acc;
                                  a.r[row] = ri;
                                  a.pbuf0[row] = ri;
                                  if (a.x != a.x0) a.x[row] = a.x0[row];
                                  rrp = fma(ri, ri, rrp);
                                  bbp = fma(bi, bi, bbp);
                              });
    rrp = block_sum(rrp, smem);
    bbp = block_sum(bbp, smem);
    if (threadIdx.x == 0) { a.partials[2 * G + t.rank] = rrp; a.partials[3 * G + t.rank] = bbp; }
    if (!t.barrier(1)) { write_info(t, a, 0, NSF_ERR_BARRIER_TIMEOUT, 1, 0, 0); return NSF_ERR_BARRIER_TIMEOUT; }
    double rr = grid_sum(a.partials + 2 * G, G, smem);
    const double bb = grid_sum(a.partials + 3 * G, G, smem);
    const double target = bb > 0 ? a.tol2 * bb : a.tol2 * rr;

    int it = 0, status = NSF_ERR_NOT_CONVERGED;
    if (!(rr == rr) || !(bb == bb) || isinf(rr) || isinf(bb)) status = NSF_ERR_BREAKDOWN;
    else if (rr <= target) status = NSF_OK;
    double* p = a.pbuf0;
    const int bs = blockDim.x;
    while (status == NSF_ERR_NOT_CONVERGED && it < a.maxIt) {
        // phase A: q = A p (streamed matrix), partial p.q
        double pq = 0;
        const bool copied = stream_spmv<double, double, false>(st, a.rowptr, a.col, a.val, nnzTotal, rb, re,
                                                              [&](int c) { return p[c]; },
                                                              [&](int row, double acc) {
                                                                  a.q[row] = acc;
                                                                  pq = fma(p[row], acc, pq);
                                                              });
        if (!copied) return stream_timeout(t, a, it, 1, rr, bb);
        pq = block_sum(pq, smem);
        if (threadIdx.x == 0) a.partials[t.rank] = pq;
        if (!t.barrier(2)) { write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, 1, rr, bb); return NSF_ERR_BARRIER_TIMEOUT; }
        const double pqs = grid_sum(a.partials, G, smem);
        if (!(pqs > 0.0) || isinf(pqs)) { status = NSF_ERR_BREAKDOWN; break; }
        const double alpha = rr / pqs;
        // phase B: x += alpha p, r -= alpha q, partial r.r (four rows per thread in flight)
        double rrn = 0;
        for (int i0 = rb + (int)threadIdx.x; i0 < re; i0 += 4 * bs) {
            double pi[4], qi[4], xi[4], ri[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + u * bs;
                if (i < re) { pi[u] = p[i]; qi[u] = a.q[i]; xi[u] = a.x[i]; ri[u] = a.r[i]; }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
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
        if (threadIdx.x == 0) a.partials[G + t.rank] = rrn;
        if (!t.barrier(3)) { write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, 1, rr, bb); return NSF_ERR_BARRIER_TIMEOUT; }
        const double rrs = grid_sum(a.partials + G, G, smem);
        ++it;
        if (!(rrs == rrs) || isinf(rrs)) { status = NSF_ERR_BREAKDOWN; break; }
        const double beta = rrs / rr;
        rr = rrs;
        if (rr <= target) { status = NSF_OK; break; }
        // phase C: p = r + beta p; the next product gathers p across blocks, hence the third barrier
        for (int i0 = rb + (int)threadIdx.x; i0 < re; i0 += 4 * bs) {
            double pi[4], ri[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + u * bs;
                if (i < re) { pi[u] = p[i]; ri[u] = a.r[i]; }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int i = i0 + u * bs;
                if (i < re) p[i] = fma(beta, pi[u], ri[u]);
            }
        }
        if (!t.barrier(4)) { write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, 1, rr, bb); return NSF_ERR_BARRIER_TIMEOUT; }
    }
    write_info(t, a, it, status, 1, rr, bb);
    return status;
}

// ---------------------------------------------------------------------------------------------------
// Mixed precision: FP32 CG with FP64 reliable updates.
// The search direction p, the product q = A32 p, the residual r32 and the accumulated correction d32 are FP32;
// the dot products and alpha/beta are FP64.  x, b and the true residual stay FP64: whenever the FP32 residual
// has fallen by the factor delta (innerTol) since the last true residual, d32 is folded into x, the residual
// b - A64 x is recomputed with the FP64 matrix and replaces r32, and the recurrence continues with the same
// search direction.  This is iterative refinement that keeps the Krylov recurrence instead of restarting it, so
// the FP32 matrix error costs little in iteration count even on the ill-conditioned pressure system.
// The FP32 product gathers p_j = r32_j + beta p_prev_j on the fly (FP32 arithmetic is cheap on GB300), which
// saves the third barrier of the FP64 kernel.
// partial regions: 0 = p.q, 1 = r32.r32, 2 = r64.r64, 3 = b.b, 4 = r32.r32 after a refresh
// ---------------------------------------------------------------------------------------------------
static __device__ int team_cg_mixed(Team& t, const CgArgs& a, double* stage, double* smem, Stream& st) {
    const int nnzTotal = a.rowptr[a.n];
    float* stage32 = reinterpret_cast<float*>(stage);
    const int G = t.size;
    int rb, re;
    team_rows(a.n, t, rb, re);
    const double* b = a.bRowptr ? a.bOut : a.b;
    const int bs = blockDim.x;

    build_rhs(a, rb, re, stage);
    // x = x0 (own rows); the first true residual gathers x0, not x, so no barrier is needed here
    if (a.x != a.x0)
        for (int i = rb + (int)threadIdx.x; i < re; i += bs) a.x[i] = a.x0[i];

    int it = 0, refresh = 0, status = NSF_ERR_NOT_CONVERGED, where = 10, stalls = 0;
    double rr64 = 0, bb = 0, target = 0, rr = 0, rrPrev = 1.0, beta = 0.0, rrBest = INFINITY;
    float* pprev = a.p32a;
    float* pcur = a.p32b;
    bool first = true;       // the first true residual gathers x0 and sets the target
    bool resetP = true;      // (re)start the recurrence: p_prev := r32, beta := 0
    while (true) {
        // true residual: r = b - A64 x; r32 = (float) r; d32 = 0
        const double* xs = first ? a.x0 : a.x;
        double rrp = 0, bbp = 0, rip = 0;
        float* pp0 = pprev;
        const bool f0 = resetP;
        warp_spmv<double, double>(a.rowptr, a.col, a.val, rb, re, stage, [&](int c) { return xs[c]; },
                                  [&](int row, double acc) {
                                      const double bi = b[row];
                                      const double ri = bi - acc;
                                      const float r32 = (float)ri;
                                      a.r32[row] = r32;
                                      if (f0) pp0[row] = r32;
                                      a.d32[row] = 0.0f;
                                      rrp = fma(ri, ri, rrp);
                                      bbp = fma(bi, bi, bbp);
                                      rip = fma((double)r32, (double)r32, rip);
                                  });
        rrp = block_sum(rrp, smem);
        bbp = block_sum(bbp, smem);
        rip = block_sum(rip, smem);
        if (threadIdx.x == 0) {
            a.partials[2 * G + t.rank] = rrp;
            a.partials[3 * G + t.rank] = bbp;
            a.partials[4 * G + t.rank] = rip;
        }
        if (!t.barrier(where++)) { write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, refresh, rr64, bb); return NSF_ERR_BARRIER_TIMEOUT; }
        rr64 = grid_sum(a.partials + 2 * G, G, smem);
        if (first) {
            bb = grid_sum(a.partials + 3 * G, G, smem);
            target = bb > 0 ? a.tol2 * bb : a.tol2 * rr64;
        }
        const double rrTrue = grid_sum(a.partials + 4 * G, G, smem);
        if (!(rr64 == rr64) || isinf(rr64)) { status = NSF_ERR_BREAKDOWN; break; }
        if (rr64 <= target) { status = NSF_OK; break; }
        if (it >= a.maxIt || refresh >= a.maxOuter) break;
        // stagnation guard: a refresh cycle normally cuts the true residual norm by ~1/delta.  Three consecutive
        // cycles that gain less than 10% mean the FP32 recurrence cannot resolve this system, and the solve
        // finishes in FP64 below.  (CG residuals are not monotone, so single weak cycles are tolerated.)
        if (refresh > 0 && rr64 > 0.81 * rrBest) {
            if (++stalls >= 3) break;
        } else {
            stalls = 0;
        }
        rrBest = fmin(rrBest, rr64);
        // continue the recurrence from the refreshed residual: beta' = |r_new|^2 / |r_prev|^2
        beta = resetP ? 0.0 : rrTrue / rrPrev;
        resetP = false;
        rr = rrTrue;
        const double rrRef = rrTrue;
        const int itRef = it;
        ++refresh;
        first = false;

        bool innerBreakdown = false;
        while (it < a.maxIt) {
            const float betaf = (float)beta;
            const float* pp = pprev;
            float* pc = pcur;
            const float* r32 = a.r32;
            double pq = 0;
            // q = A32 p in difference form: sum_j a_ij (p_j - p_i) + rowsum_i p_i (exact row sums, see warp_spmv)
            const bool copied = stream_spmv<float, float, true>(st, a.rowptr, a.col, a.val32, nnzTotal, rb, re,
                                                                [&](int c) { return fmaf(betaf, pp[c], r32[c]); },
                                                                [&](int row, float acc) {
                                                                    const float pi = fmaf(betaf, pp[row], r32[row]);
                                                                    acc = fmaf(a.rowsum32[row], pi, acc);
                                                                    pc[row] = pi;
                                                                    a.q32[row] = acc;
                                                                    pq = fma((double)pi, (double)acc, pq);
                                                                });
            if (!copied) return stream_timeout(t, a, it, refresh, rr64, bb);
            pq = block_sum(pq, smem);
            if (threadIdx.x == 0) a.partials[t.rank] = pq;
            if (!t.barrier(where++)) { write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, refresh, rr64, bb); return NSF_ERR_BARRIER_TIMEOUT; }
            const double pqs = grid_sum(a.partials, G, smem);
            if (!(pqs > 0.0) || isinf(pqs)) { innerBreakdown = true; break; }
            const float alphaf = (float)(rr / pqs);
            double rrn = 0;
            for (int i0 = rb + (int)threadIdx.x; i0 < re; i0 += 4 * bs) {
                float pi[4], qi[4], di[4], ri[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = i0 + u * bs;
                    if (i < re) { pi[u] = pc[i]; qi[u] = a.q32[i]; di[u] = a.d32[i]; ri[u] = a.r32[i]; }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = i0 + u * bs;
                    if (i < re) {
                        a.d32[i] = fmaf(alphaf, pi[u], di[u]);
                        const float rn = fmaf(-alphaf, qi[u], ri[u]);
                        a.r32[i] = rn;
                        rrn = fma((double)rn, (double)rn, rrn);
                    }
                }
            }
            rrn = block_sum(rrn, smem);
            if (threadIdx.x == 0) a.partials[G + t.rank] = rrn;
            if (!t.barrier(where++)) { write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, refresh, rr64, bb); return NSF_ERR_BARRIER_TIMEOUT; }
            const double rrs = grid_sum(a.partials + G, G, smem);
            ++it;
            { float* t = pprev; pprev = pcur; pcur = t; }
            if (!(rrs == rrs) || isinf(rrs)) { innerBreakdown = true; break; }
            beta = rrs / rr;
            rrPrev = rr;
            rr = rrs;
            if (rr <= a.innerTol2 * rrRef || rr <= target) break;   // time for a true residual
            if (it - itRef >= kMaxInnerBetweenRefresh) break;        // bound the work between true residuals
        }
        // fold the correction into x (FP64); the next true residual gathers x across blocks
        for (int i = rb + (int)threadIdx.x; i < re; i += bs) a.x[i] += (double)a.d32[i];
        if (!t.barrier(where++)) { write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, refresh, rr64, bb); return NSF_ERR_BARRIER_TIMEOUT; }
        if (innerBreakdown) resetP = true;   // restart the recurrence from the true residual
    }
    if (status == NSF_ERR_NOT_CONVERGED && it < a.maxIt) {
        // fall back to the plain FP64 method from the current iterate (x is complete after the last barrier);
        // the right-hand side is final too, so the fused build is not repeated
        CgArgs f = a;
        f.bRowptr = nullptr;
        f.b = b;
        f.x0 = a.x;
        f.maxIt = a.maxIt - it;
        const int fst = team_cg_fp64(t, f, stage, smem, st);
        if (fst == NSF_ERR_BARRIER_TIMEOUT) return fst;
        if (t.rank == 0 && threadIdx.x == 0) {
            a.info->iterations += it;
            a.info->outer = refresh;
            a.info->fallback = 1;   // finished in FP64
        }
        return fst;
    }
    write_info(t, a, it, status, refresh, rr64, bb);
    return status;
}

}  // namespace nsf
