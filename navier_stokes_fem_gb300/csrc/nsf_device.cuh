// Device-side building blocks of the persistent CG solvers, shared by the single-solve kernels (nsf_cg.cu) and
// the persistent operator-split step kernel (nsf_step.cu).  See nsf_cg.cu for the design notes.
#pragma once
#include "nsf_internal.cuh"
#include "nsf_tc.cuh"

namespace nsf {

constexpr int kCgThreads = 256;
constexpr int kWarps = kCgThreads / 32;
constexpr int kStage = 128;   // staged (value, gathered x) pairs per warp
constexpr int kMaxInnerBetweenRefresh = 4000;   // mixed precision: FP32 iterations between FP64 true residuals
constexpr int kRows = 4;      // rows per thread with their loads in flight in the vector phases
constexpr int kRowsLean = 2;  // (the kernels that run at 4 CTAs per SM)
// reduction slots of a CG kernel's shared memory: [0, 32) block_sum (one per warp), 32 grid_sum, 33 block_scalar,
// 34-35 a Decision (decision_put / decision_get)
constexpr int kSmemSlots = 36;

// Shared memory of a CG kernel: reduction slots and the warp-chunked CSR product's staging area (the ring
// kernels stage in their ring memory instead, NSF_RING_SHARED).
#define NSF_KERNEL_SHARED()          \
    __shared__ double smem[kSmemSlots]; \
    __shared__ double stage[kWarps * 2 * kStage]
#define NSF_RING_SHARED()                                     \
    __shared__ double smem[kSmemSlots];                       \
    extern __shared__ __align__(128) unsigned char dsm[];     \
    double* stage = reinterpret_cast<double*>(dsm)


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
// L2 load of data another block wrote before a barrier (never a stale L1 line)
__device__ __forceinline__ double ld_cg(const double* p) { return __ldcg(p); }

// streaming loads for the matrix (read once per iteration; keep L2 for the gathered vectors)
__device__ __forceinline__ int ld_stream(const int* p) { return __ldcs(p); }
__device__ __forceinline__ double ld_stream(const double* p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float* p) { return __ldcs(p); }
__device__ __forceinline__ unsigned short ld_stream(const unsigned short* p) { return __ldcs(p); }
__device__ __forceinline__ __half ld_stream(const __half* p) {
    return __ushort_as_half(__ldcs(reinterpret_cast<const unsigned short*>(p)));
}

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
        // The CTA's writes reach thread 0's release through the bar.sync before it (release is cumulative), and the
        // other CTAs' writes reach every thread's later loads through thread 0's acquire and the bar.sync after it,
        // so no separate fences are needed.  The wait polls the counter alone and looks at the abort flag and the
        // clock every 32nd poll (the first poll included, so a zero limit expires at once).
        __syncthreads();
        if (threadIdx.x == 0) {
            target += (unsigned long long)size;
            red_add_release(&sync->arrived, 1ULL);
            int res = 1;
            const long long t0 = global_ns();
            unsigned polls = 0;
            while (ld_acquire(&sync->arrived) < target) {
                if ((polls++ & 31u) != 0) continue;
                if (ld_volatile(&sync->abort)) { res = 0; break; }
                if (global_ns() - t0 >= timeoutNs) {
                    if (atomicCAS(&sync->abort, 0, 1) == 0) sync->where = where;
                    res = 0;
                    break;
                }
            }
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

// hi + lo += a * b in double-float arithmetic (Dekker's exact product and Knuth's two-sum on FP32 operations):
// about 44 significant bits for a per-thread partial dot product without touching the FP64 pipe, which on GB300
// is narrower than the FP32 one by a factor of 64.  The _rn intrinsics keep the compiler from contracting them.
__device__ __forceinline__ void df_acc(float& hi, float& lo, float a, float b) {
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);
    const float s = __fadd_rn(hi, p);
    const float bp = __fsub_rn(s, hi);
    const float se = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(p, bp));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(se, pe));
}

// hi + lo += (bh + bl) over the warp's lanes by xor shuffles: the double-float sum of the 32 lanes' pairs, the
// same in every lane (Knuth's two-sum on FP32 operations, fixed order).
__device__ __forceinline__ void warp_sum_df(float& hi, float& lo) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float bh = __shfl_xor_sync(0xffffffffu, hi, o);
        const float bl = __shfl_xor_sync(0xffffffffu, lo, o);
        const float sh = __fadd_rn(hi, bh);
        const float bp = __fsub_rn(sh, hi);
        const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(sh, bp)), __fsub_rn(bh, bp));
        hi = sh;
        lo = __fadd_rn(__fadd_rn(lo, bl), e);
    }
}

// block_sum of a double-float pair (hi + lo, the FP32 dot accumulators): both stages (lanes, then the warps'
// pairs in warp 0) add pairs in FP32 with two-sums, so the FP64 pipe, which on GB300 is too narrow for per-thread
// scalar work, sees one conversion per block.  Result valid in thread 0; fixed order -> deterministic.
static __device__ double block_sum_df(float hi, float lo, double* smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* pair = reinterpret_cast<float*>(smem);   // warp w: (hi, lo) at 2w, 2w + 1 (slots [0, 32))
    warp_sum_df(hi, lo);
    if (lane == 0) {
        pair[2 * warp] = hi;
        pair[2 * warp + 1] = lo;
    }
    __syncthreads();
    double t = 0;
    if (warp == 0) {
        const bool in = lane < (int)(blockDim.x >> 5);
        float h = in ? pair[2 * lane] : 0.f, l = in ? pair[2 * lane + 1] : 0.f;
        warp_sum_df(h, l);
        if (lane == 0) t = (double)h + (double)l;
    }
    __syncthreads();
    return t;
}

// Sum of the per-block partials of one region, identical in every block and thread.  Warp 0 loads them (each
// lane a strided share, all loads in flight at once) and reduces in a fixed order; the sum reaches the other
// threads through shared memory, so the FP64 work is one warp's, not every thread's.
static __device__ double grid_sum(const double* part, int G, double* smem) {
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        double p[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) p[k] = lane + 32 * k < G ? ld_cg(part + lane + 32 * k) : 0.0;
        double v = (p[0] + p[1]) + (p[2] + p[3]);
        for (int i = lane + 128; i < G; i += 32) v += ld_cg(part + i);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) smem[32] = v;
    }
    __syncthreads();
    const double t = smem[32];
    __syncthreads();
    return t;
}

// A decision of thread 0 handed to every thread of the block: an FP32 coefficient and a code.  The FP32
// iteration loops use them so that their FP64 state and tests live in thread 0 alone: GB300's FP64 pipe
// retires about 2 lanes per cycle per SM, so a per-thread FP64 test costs 16 cycles per warp.
struct Decision {
    float v;
    int code;
};

// The sum of the team's per-CTA partials as grid_sum forms it, valid in thread 0 only (no broadcast).
static __device__ double grid_sum0(const double* part, int G) {
    double v = 0.0;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        double p[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) p[k] = lane + 32 * k < G ? ld_cg(part + lane + 32 * k) : 0.0;
        v = (p[0] + p[1]) + (p[2] + p[3]);
        for (int i = lane + 128; i < G; i += 32) v += ld_cg(part + i);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    return v;
}

// Thread 0 posts a decision (decision_put); every thread of the block receives it (decision_get).
__device__ __forceinline__ void decision_put(double* smem, float v, int code) {
    reinterpret_cast<float*>(smem + 34)[0] = v;
    reinterpret_cast<int*>(smem + 35)[0] = code;
}
__device__ __forceinline__ Decision decision_get(double* smem) {
    __syncthreads();
    const Decision d{reinterpret_cast<const float*>(smem + 34)[0], reinterpret_cast<const int*>(smem + 35)[0]};
    __syncthreads();
    return d;
}

// f() evaluated once by thread 0 and handed to every thread of the block (scalar FP64 work such as the CG
// coefficients' divisions, kept off the narrow FP64 pipe's per-thread budget).
template <typename F>
__device__ __forceinline__ double block_scalar(double* smem, F f) {
    if (threadIdx.x == 0) smem[33] = f();
    __syncthreads();
    const double v = smem[33];
    __syncthreads();
    return v;
}

// Row-range of this CTA within its team: contiguous chunks keep each CTA's gathers local; chunks are whole
// 32-row slices so that the SELL-32 product of a CTA covers exactly its rows.
__device__ __forceinline__ void team_rows(int n, const Team& t, int& rb, int& re) {
    const int slices = (n + 31) / 32;
    const int chunk = ((slices + t.size - 1) / t.size) * 32;
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
// SELL-32 product (the CG kernels' hot loop).  Rows are grouped in slices of 32; slice s stores its rows'
// entries column-major, entry k of row 32s + lane at sliceStart[s] + 32k + lane, padded to the slice's longest
// row with value 0 and the row's own column.  A warp owns a slice: every load of the matrix is one coalesced
// 128-byte (FP32) or 256-byte (FP64) line, with no shared-memory staging and no block-wide synchronisation, and
// each lane sums its row in CSR entry order with one fused multiply-add per entry (padding adds exact zeros),
// so the result equals the CSR row sum bit for bit.  Up to kUnroll entries per lane have their matrix loads and
// then their vector gathers in flight at once.  The matrix is read with evict-first loads so that the gathered
// vectors stay in L2.
// ---------------------------------------------------------------------------------------------------
constexpr int kSlice = 32;
constexpr int kUnroll = kSellChunk;

// pre() value of the difference-form products that also carries the row's FP32 row sum (loaded with the row's own
// vector entry when the slice starts, not after its sum); row_self() is the entry Diff subtracts.
template <typename TA> struct DiffPre {
    TA self;
    TA rs;
};
template <typename TA> __device__ __forceinline__ TA row_self(TA v) { return v; }
template <typename TA> __device__ __forceinline__ TA row_self(const DiffPre<TA>& v) { return v.self; }

// Column indices of a SELL-32 matrix are 32-bit (TC = int) or, when every slice's columns span fewer than 65535,
// 16-bit offsets from a per-slice base (TC = unsigned short; kCol16Pad marks a padding entry of column -1).

// Loads entries [k0, k0 + U) of a lane's row in a slice (column -1 past the slice width W); cb is the slice's
// column base of a 16-bit column array.
template <int U, typename TV, typename TC = int>
__device__ __forceinline__ void sell_chunk(const TC* __restrict__ cp, const TV* __restrict__ vp, int W, int k0,
                                           int (&c)[U], TV (&v)[U], int cb = 0) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const bool in = k0 + u < W;
        if constexpr (sizeof(TC) == 2) {
            // a padding entry's value is zeroed too: the 16-bit copy of a matrix stores its diagonal as padding
            const int d = in ? (int)ld_stream(cp + (k0 + u) * kSlice) : kCol16Pad;
            const TV x = in ? ld_stream(vp + (k0 + u) * kSlice) : TV(0);
            c[u] = d == kCol16Pad ? -1 : cb + d;
            v[u] = d == kCol16Pad ? TV(0) : x;
        } else {
            c[u] = in ? ld_stream(cp + (k0 + u) * kSlice) : -1;
            v[u] = in ? ld_stream(vp + (k0 + u) * kSlice) : TV(0);
        }
    }
}

// A warp walks its slices sFirst, sFirst + nw, ... as NS independent streams (the warp's slice list cut in NS
// consecutive parts), each with the next slice's first U matrix entries loaded while the current slice's gathers
// are in flight: a step costs one memory latency and serves NS slices.  The slices' start offsets are fetched 32
// at a time, one per lane, and handed out by shuffles.
// pre(row) is evaluated when a slice starts (its loads overlap the slice's), and its value goes to epi(row, sum,
// pre); with Diff it must be the row's own vector entry.  Rows [rb, re): rb a multiple of 32 unless rb == re.
// With 16-bit columns (TC = unsigned short) colBase holds each slice's column base.
template <typename TV, typename TA, bool Diff, int NS = 1, int U = kUnroll, typename TC = int, typename Gather,
          typename Pre, typename Epi>
__device__ __forceinline__ void sell_rows(const int* __restrict__ sliceStart, const TC* __restrict__ col,
                                          const TV* __restrict__ val, int rb, int re, Gather gather, Pre pre,
                                          Epi epi, const int* __restrict__ colBase = nullptr) {
    constexpr bool C16 = sizeof(TC) == 2;
    using PreT = decltype(pre(0));
    if (rb >= re) return;   // (an empty range may start inside the last, partial slice)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int s1 = (re + kSlice - 1) / kSlice;
    const int sFirst = rb / kSlice + warp;
    if (sFirst >= s1) return;
    const int count = (s1 - sFirst + nw - 1) / nw;   // this warp's slices
    const int per = (count + NS - 1) / NS;           // per stream: stream q takes i in [q per, (q + 1) per)
    int mb[NS], me[NS], base[NS], W[NS], c[NS][U];
    int mcb[NS], cb[NS];   // 16-bit columns: the slices' column bases (lane j: slice i0 + j) and the current one's
    TV v[NS][U];
    auto meta_load = [&](int q, int i0) {   // lane j: start / end of stream q's slice i0 + j
        const int idx = sFirst + (q * per + i0 + lane) * nw;
        const bool in = idx < s1 && i0 + lane < per;
        mb[q] = in ? sliceStart[idx] : 0;
        me[q] = in ? sliceStart[idx + 1] : 0;
        if constexpr (C16) mcb[q] = in ? colBase[idx] : 0;
    };
#pragma unroll
    for (int q = 0; q < NS; ++q) {
        meta_load(q, 0);
        base[q] = __shfl_sync(0xffffffffu, mb[q], 0);
        W[q] = (__shfl_sync(0xffffffffu, me[q], 0) - base[q]) / kSlice;
        cb[q] = C16 ? __shfl_sync(0xffffffffu, mcb[q], 0) : 0;
        sell_chunk<U, TV, TC>(col + base[q] + lane, val + base[q] + lane, W[q], 0, c[q], v[q], cb[q]);
    }
    for (int k = 0; k < per; ++k) {
        int row[NS], Wc[NS], bc[NS], cbc[NS];
        bool live[NS];
        PreT pv[NS];
        TA g[NS][U];
        TV vk[NS][U];
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            const int i = q * per + k;
            live[q] = i < count;
            row[q] = (sFirst + i * nw) * kSlice + lane;
            pv[q] = live[q] && row[q] < re ? pre(row[q]) : PreT{};
#pragma unroll
            for (int u = 0; u < U; ++u) {
                g[q][u] = c[q][u] >= 0 ? gather(c[q][u]) : TA(0);
                vk[q][u] = v[q][u];
            }
        }
        // the streams' next slices: first entries in flight with this step's gathers
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            Wc[q] = W[q];
            bc[q] = base[q];
            cbc[q] = cb[q];
            int baseN = 0, WN = 0, cbN = 0;
            if (k + 1 < per && q * per + k + 1 < count) {
                if (((k + 1) & 31) == 0) meta_load(q, k + 1);
                baseN = __shfl_sync(0xffffffffu, mb[q], (k + 1) & 31);
                WN = (__shfl_sync(0xffffffffu, me[q], (k + 1) & 31) - baseN) / kSlice;
                if constexpr (C16) cbN = __shfl_sync(0xffffffffu, mcb[q], (k + 1) & 31);
            }
            sell_chunk<U, TV, TC>(col + baseN + lane, val + baseN + lane, WN, 0, c[q], v[q], cbN);
            base[q] = baseN;
            W[q] = WN;
            cb[q] = cbN;
        }
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            if (!live[q]) continue;
            TA self = TA(0);
            if constexpr (Diff) self = row_self<TA>(pv[q]);
            TA acc = TA(0);
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (u < Wc[q]) {
                    if (Diff) acc = fma(TA(vk[q][u]), g[q][u] - self, acc);
                    else acc = fma(TA(vk[q][u]), g[q][u], acc);
                }
            }
            // rows longer than U entries (P2 matrices): the rest of the slice, chunk by chunk
            for (int k0 = U; k0 < Wc[q]; k0 += U) {
                int c2[U];
                TV v2[U];
                TA g2[U];
                sell_chunk<U, TV, TC>(col + bc[q] + lane, val + bc[q] + lane, Wc[q], k0, c2, v2, cbc[q]);
#pragma unroll
                for (int u = 0; u < U; ++u) g2[u] = c2[u] >= 0 ? gather(c2[u]) : TA(0);
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (c2[u] >= 0) {
                        if (Diff) acc = fma(TA(v2[u]), g2[u] - self, acc);
                        else acc = fma(TA(v2[u]), g2[u], acc);
                    }
                }
            }
            if (row[q] < re) epi(row[q], acc, pv[q]);
        }
    }
}

// Wide matrices (slices wider than U entries per row: the P2 mass, diffusion and divergence matrices).  Each of a
// warp's NS streams is a software pipeline over chunks of U entries per lane: the next chunk's matrix loads (the
// rest of this slice, or the next slice's first chunk) are issued together with this chunk's gathers, so a chunk
// costs one memory latency and a slice of width W costs ceil(W / U) of them (sell_rows spends two per chunk after
// the first).  Same contract as sell_rows; pre(row) is evaluated when the slice's predecessor finishes.
template <int U, typename TV>
__device__ __forceinline__ void sell_chunk_at(const int* __restrict__ col, const TV* __restrict__ val, int off,
                                              int rem, int (&c)[U], TV (&v)[U]) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const bool in = u < rem;
        c[u] = in ? ld_stream(col + off + u * kSlice) : -1;
        v[u] = in ? ld_stream(val + off + u * kSlice) : TV(0);
    }
}

template <typename TV, typename TA, bool Diff, int NS = 1, int U = kUnroll, typename Gather, typename Pre,
          typename Epi>
__device__ __forceinline__ void sell_rows_wide(const int* __restrict__ sliceStart, const int* __restrict__ col,
                                               const TV* __restrict__ val, int rb, int re, Gather gather, Pre pre,
                                               Epi epi) {
    using PreT = decltype(pre(0));
    if (rb >= re) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int s1 = (re + kSlice - 1) / kSlice;
    const int sFirst = rb / kSlice + warp;
    if (sFirst >= s1) return;
    const int count = (s1 - sFirst + nw - 1) / nw;
    const int per = (count + NS - 1) / NS;
    // per stream: k = slice ordinal, kEnd = its end, off / rem = offset and entries left of the chunk in flight
    int mb[NS], me[NS], k[NS], kEnd[NS], off[NS], rem[NS], c[NS][U];
    TV v[NS][U];
    TA acc[NS];
    PreT pv[NS];
#pragma unroll
    for (int q = 0; q < NS; ++q) kEnd[q] = max(0, min(per, count - q * per));
    auto meta_load = [&](int q, int i0) {   // lane j: start / end of stream q's slice i0 + j
        const int i = i0 + lane;
        const bool in = i < kEnd[q];
        const int idx = sFirst + (q * per + i) * nw;
        mb[q] = in ? sliceStart[idx] : 0;
        me[q] = in ? sliceStart[idx + 1] : 0;
    };
#pragma unroll
    for (int q = 0; q < NS; ++q) {
        k[q] = 0;
        acc[q] = TA(0);
        meta_load(q, 0);
        off[q] = __shfl_sync(0xffffffffu, mb[q], 0);
        rem[q] = (__shfl_sync(0xffffffffu, me[q], 0) - off[q]) / kSlice;
        off[q] += lane;
        sell_chunk_at<U, TV>(col, val, off[q], rem[q], c[q], v[q]);
        const int row = (sFirst + q * per * nw) * kSlice + lane;
        pv[q] = kEnd[q] > 0 && row < re ? pre(row) : PreT{};
    }
    while (true) {
        bool any = false;
#pragma unroll
        for (int q = 0; q < NS; ++q) any = any || k[q] < kEnd[q];
        if (!any) break;
        int remC[NS];
        TA g[NS][U];
        TV vk[NS][U];
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            remC[q] = rem[q];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                g[q][u] = c[q][u] >= 0 ? gather(c[q][u]) : TA(0);
                vk[q][u] = v[q][u];
            }
        }
        // each stream's next chunk in flight with this step's gathers
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            if (k[q] >= kEnd[q]) continue;
            if (rem[q] > U) {
                off[q] += U * kSlice;
                rem[q] -= U;
            } else {
                const int kn = k[q] + 1;
                int o = 0, e = 0;
                if (kn < kEnd[q]) {
                    if ((kn & 31) == 0) meta_load(q, kn);
                    o = __shfl_sync(0xffffffffu, mb[q], kn & 31);
                    e = __shfl_sync(0xffffffffu, me[q], kn & 31);
                }
                off[q] = o + lane;
                rem[q] = (e - o) / kSlice;
            }
            sell_chunk_at<U, TV>(col, val, off[q], rem[q], c[q], v[q]);
        }
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            if (k[q] >= kEnd[q]) continue;
            TA self = TA(0);
            if constexpr (Diff) self = row_self<TA>(pv[q]);
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (u < remC[q]) {
                    if (Diff) acc[q] = fma(TA(vk[q][u]), g[q][u] - self, acc[q]);
                    else acc[q] = fma(TA(vk[q][u]), g[q][u], acc[q]);
                }
            }
            if (remC[q] <= U) {   // the slice's last chunk: its rows are complete
                const int row = (sFirst + (q * per + k[q]) * nw) * kSlice + lane;
                if (row < re) epi(row, acc[q], pv[q]);
                acc[q] = TA(0);
                ++k[q];
                if (k[q] < kEnd[q]) {
                    const int rn = row + nw * kSlice;
                    pv[q] = rn < re ? pre(rn) : PreT{};
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------------
// TMA-fed SELL-32 product for narrow FP32 matrices (every slice at most kRingWidth entries per row: the pressure
// system and the preconditioner's factor).  Each warp owns a ring of kRingDepth shared-memory stages; lane 0 issues
// one bulk asynchronous copy (cp.async.bulk with an evict-first L2 policy, completion counted on the stage's
// mbarrier) per array and slice, kRingDepth slices ahead of the warp, so the matrix stream stays in flight without
// holding registers and the gathered vectors keep L2.  A step takes kRingStep slices, whose gathers are in flight
// together.  All copies a call issues are consumed in the same call.
// ---------------------------------------------------------------------------------------------------
constexpr int kRingDepth = 6;
constexpr int kRingStep = 2;
constexpr int kRingWidth = kSellChunk;
constexpr int kRingStage = kRingWidth * kSlice;   // entries per array and stage
constexpr size_t kRingDataPerWarp = (size_t)kRingDepth * kRingStage * 8;
constexpr size_t kRingBytes = kRingDataPerWarp * kWarps + (size_t)kRingDepth * kWarps * sizeof(uint64_t);
static_assert(kRingDataPerWarp * kWarps >= sizeof(double) * kWarps * 2 * kStage,
              "the ring kernels use the ring memory as the CSR product's staging area");

// Waits on asynchronous copies never give up sooner than this, whatever the grid-barrier limit (even a zero
// one, used to test the time-out path): a warp must not leave a stage while its copy may still land.
constexpr long long kAsyncWaitFloorNs = 200000000LL;

struct SellRing {
    int* col;           // [kRingDepth][kRingStage] of this warp
    float* val;
    uint64_t* bar;      // [kRingDepth]
    unsigned seq;       // slices this warp has taken through the ring: stage seq % D, phase parity (seq / D) & 1
    uint64_t policy;    // L2 evict-first
    GridSync* sync;     // its abort word is raised when a stage's wait times out
    long long timeoutNs;
};

// Every thread calls this at kernel start; dsm is the launch's dynamic shared memory (kRingBytes, 128-byte aligned).
__device__ __forceinline__ SellRing ring_init(unsigned char* dsm, GridSync* sync, long long timeoutNs) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* base = dsm + (size_t)warp * kRingDataPerWarp;
    SellRing r;
    r.col = reinterpret_cast<int*>(base);
    r.val = reinterpret_cast<float*>(base + (size_t)kRingDepth * kRingStage * 4);
    r.bar = reinterpret_cast<uint64_t*>(dsm + kRingDataPerWarp * kWarps) + warp * kRingDepth;
    r.seq = 0;
    r.policy = tc::policy_evict_first();
    r.sync = sync;
    r.timeoutNs = timeoutNs > kAsyncWaitFloorNs ? timeoutNs : kAsyncWaitFloorNs;
    if (lane == 0)
        for (int d = 0; d < kRingDepth; ++d) tc::mbar_init(&r.bar[d], 1);
    __syncwarp();
    return r;
}

// Rows [rb, re) of a narrow FP32 SELL-32 matrix through the warp's ring; the contract of sell_rows (padding
// entries may carry column -1).  On a wait time-out the team's abort word is raised (its next barrier fails), the
// copies still in flight are waited for (bounded) and the call returns.
template <typename TA, bool Diff, typename Gather, typename Pre, typename Epi>
__device__ __forceinline__ void sell_rows_ring(SellRing& ring, const int* __restrict__ sliceStart,
                                               const int* __restrict__ col, const float* __restrict__ val, int rb,
                                               int re, Gather gather, Pre pre, Epi epi) {
    using PreT = decltype(pre(0));
    constexpr int S = kRingStep;
    static_assert(32 % S == 0 && kRingDepth >= 2 * S, "ring step");
    if (rb >= re) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int s1 = (re + kSlice - 1) / kSlice;
    const int sFirst = rb / kSlice + warp;
    if (sFirst >= s1) return;
    const int count = (s1 - sFirst + nw - 1) / nw;   // this warp's slices (slice i: sFirst + i nw)
    // lane j holds the start / end of slice 32 b + j for the block b of the slices being consumed (mb0, me0) and
    // for the next block (mb1, me1)
    int mb0, me0, mb1, me1;
    auto meta = [&](int blk, int& mb, int& me) {
        const int i = blk * 32 + lane;
        const bool in = i < count;
        const int idx = sFirst + i * nw;
        mb = in ? sliceStart[idx] : 0;
        me = in ? sliceStart[idx + 1] : 0;
    };
    meta(0, mb0, me0);
    meta(1, mb1, me1);
    int cur = 0;
    auto issue = [&](int i) {   // every lane calls (shuffles); lane 0 starts the copies of slice i
        const bool same = (i >> 5) == cur;
        const int o = __shfl_sync(0xffffffffu, same ? mb0 : mb1, i & 31);
        const int e = __shfl_sync(0xffffffffu, same ? me0 : me1, i & 31);
        if (lane == 0) {
            const unsigned st = (ring.seq + (unsigned)i) % kRingDepth;
            const uint32_t bytes = (uint32_t)(e - o) * 4u;   // W * 32 entries of 4 bytes per array
            tc::fence_proxy_async();                        // the stage's earlier reads before the async writes
            tc::mbar_expect_tx(&ring.bar[st], 2u * bytes);
            if (bytes) {
                tc::bulk_g2s_hint(ring.col + st * kRingStage, col + o, bytes, &ring.bar[st], ring.policy);
                tc::bulk_g2s_hint(ring.val + st * kRingStage, val + o, bytes, &ring.bar[st], ring.policy);
            }
        }
    };
    int issued = min(kRingDepth, count);
    for (int i = 0; i < issued; ++i) issue(i);
    PreT pv[S];
#pragma unroll
    for (int q = 0; q < S; ++q) {
        const int row = (sFirst + q * nw) * kSlice + lane;
        pv[q] = q < count && row < re ? pre(row) : PreT{};
    }
    int i = 0;
    bool ok = true;
    for (; i < count; i += S) {
        int W[S], c[S][kRingWidth];
        float v[S][kRingWidth];
#pragma unroll
        for (int q = 0; q < S; ++q) {
            const int k = (i + q) & 31;
            W[q] = i + q < count ? (__shfl_sync(0xffffffffu, me0, k) - __shfl_sync(0xffffffffu, mb0, k)) / kSlice : 0;
            bool got = true;
            const unsigned seq = ring.seq + (unsigned)(i + q);
            if (i + q < count) got = tc::mbar_wait(&ring.bar[seq % kRingDepth], (seq / kRingDepth) & 1u, ring.timeoutNs);
            ok = ok && __all_sync(0xffffffffu, got);
            const int* sc = ring.col + (seq % kRingDepth) * kRingStage + lane;
            const float* sv = ring.val + (seq % kRingDepth) * kRingStage + lane;
#pragma unroll
            for (int u = 0; u < kRingWidth; ++u) {
                c[q][u] = ok && u < W[q] ? sc[u * kSlice] : -1;
                v[q][u] = ok && u < W[q] ? sv[u * kSlice] : 0.0f;
            }
        }
        if (!ok) {
            if (lane == 0 && atomicCAS(&ring.sync->abort, 0, 1) == 0) ring.sync->where = 900;
            break;
        }
        __syncwarp();   // every lane has read the step's stages: refill them kRingDepth slices ahead
#pragma unroll
        for (int q = 0; q < S; ++q)
            if (issued < count) {
                issue(issued);
                ++issued;
            }
        TA g[S][kRingWidth];
#pragma unroll
        for (int q = 0; q < S; ++q)
#pragma unroll
            for (int u = 0; u < kRingWidth; ++u) g[q][u] = c[q][u] >= 0 ? gather(c[q][u]) : TA(0);
#pragma unroll
        for (int q = 0; q < S; ++q) {
            if (i + q >= count) continue;
            TA self = TA(0);
            if constexpr (Diff) self = row_self<TA>(pv[q]);
            TA acc = TA(0);
#pragma unroll
            for (int u = 0; u < kRingWidth; ++u) {
                if (u < W[q]) {
                    if (Diff) acc = fma(TA(v[q][u]), g[q][u] - self, acc);
                    else acc = fma(TA(v[q][u]), g[q][u], acc);
                }
            }
            const int row = (sFirst + (i + q) * nw) * kSlice + lane;
            if (row < re) epi(row, acc, pv[q]);
        }
#pragma unroll
        for (int q = 0; q < S; ++q) {
            const int row = (sFirst + (i + S + q) * nw) * kSlice + lane;
            if (i + S + q < count) pv[q] = row < re ? pre(row) : PreT{};
        }
        if (((i + S) & 31) == 0) {
            ++cur;
            mb0 = mb1;
            me0 = me1;
            meta(cur + 1, mb1, me1);
        }
    }
    // after a time-out: the copies still in flight land before the ring is left (bounded waits)
    for (int j = i; j < issued; ++j) {
        const unsigned seq = ring.seq + (unsigned)j;
        tc::mbar_wait(&ring.bar[seq % kRingDepth], (seq / kRingDepth) & 1u, ring.timeoutNs);
    }
    __syncwarp();
    ring.seq += (unsigned)issued;
}

// sum_j a_ij gather(j) (or its difference form) with epi(row, sum, gather(row)).
template <typename TV, typename TA, bool Diff, int U = kUnroll, bool Wide = false, typename Gather, typename Epi>
__device__ __forceinline__ void sell_spmv(const int* __restrict__ sliceStart, const int* __restrict__ col,
                                          const TV* __restrict__ val, int rb, int re, Gather gather, Epi epi) {
    if constexpr (Wide) sell_rows_wide<TV, TA, Diff, 1, U>(sliceStart, col, val, rb, re, gather, gather, epi);
    else sell_rows<TV, TA, Diff, 1, U>(sliceStart, col, val, rb, re, gather, gather, epi);
}

// q = A p over the CTA's rows with epi(row, sum, p_row): the SELL-32 copy when the matrix has one, else the
// warp-chunked CSR product (caller-owned CSR arrays, e.g. the allocation-free entry point).
template <typename TV, typename TA, bool Diff, int U = kUnroll, bool Wide = false, typename Gather, typename Epi>
__device__ __forceinline__ void matrix_product(const int* sellStart, const int* sellCol, const TV* sellVal,
                                               const int* rowptr, const int* col, const TV* val, int rb, int re,
                                               TA* stage, Gather gather, Epi epi) {
    if (sellStart) {
        sell_spmv<TV, TA, Diff, U, Wide>(sellStart, sellCol, sellVal, rb, re, gather, epi);
    } else {
        warp_spmv<TV, TA, Diff>(rowptr, col, val, rb, re, stage, gather,
                                [&](int row, TA acc) { epi(row, acc, gather(row)); });
    }
}

// The FP32 difference-form product of the mixed solvers, q_i = sum_j a_ij (p_j - p_i) + rowsum_i p_i: through
// the warp's ring for narrow matrices when the kernel has one, else the register-pipelined SELL-32 product (or the
// CSR product without a SELL copy).  epi(row, sum with the row-sum term, p_row).
// (C16: the narrow register-pipelined product over the 16-bit column copy, which the caller has checked exists;
// that copy stores the diagonal entries as padding, whose difference-form terms are exactly zero.)
template <bool Wide, int U = kUnroll, bool C16 = false, typename Gather, typename Epi>
__device__ __forceinline__ void product32(SellRing* ring, const CgArgs& a, int rb, int re, float* stage,
                                          Gather gather, Epi epi) {
    auto pre = [&](int row) { return DiffPre<float>{gather(row), a.rowsum32[row]}; };
    auto fin = [&](int row, float acc, const DiffPre<float>& q) { epi(row, fmaf(q.rs, q.self, acc), q.self); };
    if constexpr (C16 && !Wide) {
        sell_rows<float, float, true, 1, U, unsigned short>(a.sellStart, a.sellCol16, a.sellVal32, rb, re, gather,
                                                            pre, fin, a.sellColBase);
        return;
    }
    if constexpr (!Wide) {
        if (ring && a.sellStart) {
            sell_rows_ring<float, true>(*ring, a.sellStart, a.sellCol, a.sellVal32, rb, re, gather, pre, fin);
            return;
        }
    }
    if (a.sellStart) {
        if constexpr (Wide) sell_rows_wide<float, float, true, 1, U>(a.sellStart, a.sellCol, a.sellVal32, rb, re,
                                                                   gather, pre, fin);
        else sell_rows<float, float, true, 1, U>(a.sellStart, a.sellCol, a.sellVal32, rb, re, gather, pre, fin);
    } else {
        warp_spmv<float, float, true>(a.rowptr, a.col, a.val32, rb, re, stage, gather,
                                      [&](int row, float acc) { fin(row, acc, pre(row)); });
    }
}

// entries per lane and chunk of the FP64 residual and right-hand-side passes: 4 in the narrow kernels (register
// budget), 8 in the wide ones (P2 rows of 9 and 19 entries take 2 and 3 chunks instead of 3 and 5)
template <bool Wide> constexpr int kResidU = Wide ? 8 : 4;
// chunk of the FP32 product of a wide system in the mixed CG's iterations: the P2 rows of these meshes have 9
// entries (edge midpoints, three quarters of the rows) or 19 (vertices), one and two chunks of 10 instead of two
// and three of 8, and a chunk is a memory latency (12 spills at 64 registers)
constexpr int kWideChunk32 = 10;

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

// b for this block's rows: the given vector, or the fused right-hand side mask ? g : (B x_b) - lift, stored
// to a.bOut by the owning lane (the same lane reads it back in the residual pass).
template <bool Wide = false>
static __device__ void build_rhs(const CgArgs& a, int rb, int re, double* stage) {
    if (!a.bRowptr) return;
    matrix_product<double, double, false, kResidU<Wide>, Wide>(a.bSellStart, a.bSellCol, a.bSellVal, a.bRowptr, a.bCol, a.bVal, rb, re,
                                          stage, [&](int c) { return a.bX[c]; },
                                          [&](int row, double acc, double) {
                                              double bi = a.lift ? acc - a.lift[row] : acc;
                                              if (a.bcMask && a.bcMask[row]) bi = a.bcValue[row];
                                              a.bOut[row] = bi;
                                          });
}

// ---------------------------------------------------------------------------------------------------
// FP64 persistent CG
// partial regions: 0 = p.q, 1 = r.r, 2 = r0.r0, 3 = b.b
// ---------------------------------------------------------------------------------------------------
template <bool Wide = false>
static __device__ int team_cg_fp64(Team& t, const CgArgs& a, double* stage, double* smem) {
    const int G = t.size;
    int rb, re;
    team_rows(a.n, t, rb, re);
    const double* b = a.bRowptr ? a.bOut : a.b;

    // prologue: (b), x = x0, r0 = b - A x0, p0 = r0
    build_rhs<Wide>(a, rb, re, stage);
    double rrp = 0, bbp = 0;
    matrix_product<double, double, false, kResidU<Wide>, Wide>(a.sellStart, a.sellCol, a.sellVal, a.rowptr, a.col, a.val, rb, re, stage,
                                          [&](int c) { return a.x0[c]; },
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
        auto gq = [&](int c) { return p[c]; };
        auto eq = [&](int row, double acc, double pr) {
            a.q[row] = acc;
            pq = fma(pr, acc, pq);
        };
        // chunks as wide as the widest slice when that is 5 (a structured P1 system without its exact zeros)
        if (!Wide && a.sellMaxW <= 5)
            matrix_product<double, double, false, 5, Wide>(a.sellStart, a.sellCol, a.sellVal, a.rowptr, a.col, a.val,
                                                           rb, re, stage, gq, eq);
        else
            matrix_product<double, double, false, kUnroll, Wide>(a.sellStart, a.sellCol, a.sellVal, a.rowptr, a.col,
                                                                 a.val, rb, re, stage, gq, eq);
        pq = block_sum(pq, smem);
        if (threadIdx.x == 0) a.partials[t.rank] = pq;
        if (!t.barrier(2)) { write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, 1, rr, bb); return NSF_ERR_BARRIER_TIMEOUT; }
        const double pqs = grid_sum(a.partials, G, smem);
        if (!(pqs > 0.0) || isinf(pqs)) { status = NSF_ERR_BREAKDOWN; break; }
        const double alpha = block_scalar(smem, [&] { return rr / pqs; });
        // phase B: x += alpha p, r -= alpha q, partial r.r (four rows per thread in flight)
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
        if (threadIdx.x == 0) a.partials[G + t.rank] = rrn;
        if (!t.barrier(3)) { write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, 1, rr, bb); return NSF_ERR_BARRIER_TIMEOUT; }
        const double rrs = grid_sum(a.partials + G, G, smem);
        ++it;
        if (!(rrs == rrs) || isinf(rrs)) { status = NSF_ERR_BREAKDOWN; break; }
        const double beta = block_scalar(smem, [&] { return rrs / rr; });
        rr = rrs;
        if (rr <= target) { status = NSF_OK; break; }
        // phase C: p = r + beta p; the next product gathers p across blocks, hence the third barrier
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
        if (!t.barrier(4)) { write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, 1, rr, bb); return NSF_ERR_BARRIER_TIMEOUT; }
    }
    write_info(t, a, it, status, 1, rr, bb);
    return status;
}

// ---------------------------------------------------------------------------------------------------
// FP64 pipelined CG: one grid barrier per iteration (Ghysels & Vanroose, "Hiding global synchronization latency
// in the preconditioned Conjugate Gradient algorithm", Parallel Computing 40, 2014; here without a preconditioner).
// Besides x, r and p it carries s = A p, w = A r and z = A s as recurrences, so the only product of an iteration
// is q = A w_i on a vector finished before the previous barrier, and every other update is row-local:
//     gamma = r.r, delta = w.r (summed from the previous iteration's partials)
//     beta = gamma / gamma_prev, alpha = gamma / (delta - beta gamma / alpha_prev)   (beta = 0, alpha = gamma / delta
//                                                                                    at the first iteration)
//     z = A w + beta z,  s = w + beta s,  p = r + beta p,  x += alpha p,  r -= alpha s,  w' = w - alpha z,
// with the partials of r'.r' and w'.r' formed in the same pass.  In exact arithmetic it is the CG of team_cg_fp64;
// in floating point its recurrences drift from the true residual, so every kPipeReplaceEvery iterations, and
// whenever the recursive residual meets the tolerance, r, w, s and z are replaced by b - A x, A r, A p and A s
// (residual replacement, after Cools, Yetkin, Agullo, Giraud and Vanroose 2018) and the recurrence continues; the
// replacement's true residual is also the stopping test.
// w is written to the other of two buffers (the product of this iteration still gathers the current one), and the
// partials alternate between region pairs {0, 1} and {2, 3}: one barrier separates an iteration's partial writes
// from the next iteration's reads, and the next writes go to the other pair.  Regions 4 and 5: b.b and r.r;
// 6, 7 and 8: r.s, p.w and p.s after a replacement.
// Vectors: r = a.r, s = a.q, p = a.pbuf0, z = a.pbuf1, w = a.wbuf0 / a.wbuf1.  Needs the SELL copy.
// ---------------------------------------------------------------------------------------------------
struct PipeRow {
    double z, s, p, r, x, w;
};

constexpr int kPipeMaxChecks = 16;      // replacements after the recursive residual met the tolerance, per solve
// Iterations between residual replacements.  Left alone, the recurrences drift: on the 256^2 cavity's pressure
// system the recursive residual met 1e-8 after 1562 iterations with the true one at 1.5e-7 (plain CG: 1557
// iterations).  Replaced every 25 to 400 iterations the pipelined form took exactly plain CG's 1557 (a NumPy model
// of this routine); a replacement costs four products and two barriers.
constexpr int kPipeReplaceEvery = 100;

template <bool Wide = false, typename Gather, typename Epi>
__device__ __forceinline__ void pipe_product(const CgArgs& a, int rb, int re, double* stage, Gather gather, Epi epi) {
    matrix_product<double, double, false, kResidU<Wide>, Wide>(a.sellStart, a.sellCol, a.sellVal, a.rowptr, a.col,
                                                               a.val, rb, re, stage, gather, epi);
}

template <bool Wide = false>
static __device__ int team_cg_fp64_pipelined(Team& t, const CgArgs& a, double* stage, double* smem) {
    const int G = t.size;
    int rb, re;
    team_rows(a.n, t, rb, re);
    const double* b = a.bRowptr ? a.bOut : a.b;
    build_rhs<Wide>(a, rb, re, stage);
    int it = 0, where = 1, checks = 0;
#define NSF_PIPE_BARRIER()                                                                        \
    if (!t.barrier(where++)) {                                                                    \
        write_info(t, a, it, NSF_ERR_BARRIER_TIMEOUT, 1 + checks, rr, bb);                        \
        return NSF_ERR_BARRIER_TIMEOUT;                                                           \
    }
    double rr = 0, bb = 0;
    // r = b - A x (x = x0 first, copied to x), its r.r in region 5 (and b.b in region 4 the first time)
    auto true_residual = [&](const double* xs, bool first) {
        double rrp = 0, bbp = 0;
        pipe_product<Wide>(a, rb, re, stage, [&](int c) { return xs[c]; }, [&](int row, double acc, double xi) {
            const double bi = b[row];
            const double ri = bi - acc;
            a.r[row] = ri;
            if (first && a.x != xs) a.x[row] = xi;
            rrp = fma(ri, ri, rrp);
            bbp = fma(bi, bi, bbp);
        });
        rrp = block_sum(rrp, smem);
        bbp = block_sum(bbp, smem);
        if (threadIdx.x == 0) {
            a.partials[5 * G + t.rank] = rrp;
            if (first) a.partials[4 * G + t.rank] = bbp;
        }
    };
    true_residual(a.x0, true);
    NSF_PIPE_BARRIER();
    bb = grid_sum(a.partials + 4 * G, G, smem);
    rr = grid_sum(a.partials + 5 * G, G, smem);
    const double target = bb > 0 ? a.tol2 * bb : a.tol2 * rr;
    if (!(rr == rr) || !(bb == bb) || isinf(rr) || isinf(bb)) {
        write_info(t, a, 0, NSF_ERR_BREAKDOWN, 1, rr, bb);
        return NSF_ERR_BREAKDOWN;
    }
    if (rr <= target || a.maxIt <= 0) {
        const int st = rr <= target ? NSF_OK : NSF_ERR_NOT_CONVERGED;
        write_info(t, a, 0, st, 1, rr, bb);
        return st;
    }
    // w = A r into the buffer the first iteration reads, with the partials of r.r and w.r in pair 0
    {
        double gp = 0, dp = 0;
        pipe_product<Wide>(a, rb, re, stage, [&](int c) { return a.r[c]; }, [&](int row, double acc, double ri) {
            a.wbuf0[row] = acc;
            gp = fma(ri, ri, gp);
            dp = fma(acc, ri, dp);
        });
        gp = block_sum(gp, smem);
        dp = block_sum(dp, smem);
        if (threadIdx.x == 0) { a.partials[t.rank] = gp; a.partials[G + t.rank] = dp; }
        NSF_PIPE_BARRIER();
    }
    int status = NSF_ERR_NOT_CONVERGED;
    double gammaPrev = 1.0, alphaPrev = 1.0;
    bool explicitDen = false;
    int lastReplaced = 0;
    for (int k = 0;;) {
        const int par = k & 1;
        const double gamma = grid_sum(a.partials + (2 * par) * G, G, smem);
        const double delta = grid_sum(a.partials + (2 * par + 1) * G, G, smem);
        if (!(gamma == gamma) || isinf(gamma)) { status = NSF_ERR_BREAKDOWN; break; }
        double* wc = par ? a.wbuf1 : a.wbuf0;
        const bool met = gamma <= target;
        if (met || it >= a.maxIt || (k > 0 && it - lastReplaced >= kPipeReplaceEvery)) {
            // replacement: r = b - A x and s = A p (p is the recurrence's once an iteration has run) ...
            double rrp = 0;
            pipe_product<Wide>(a, rb, re, stage, [&](int c) { return a.x[c]; }, [&](int row, double acc, double) {
                const double ri = b[row] - acc;
                a.r[row] = ri;
                rrp = fma(ri, ri, rrp);
            });
            if (k > 0)
                pipe_product<Wide>(a, rb, re, stage, [&](int c) { return a.pbuf0[c]; },
                                   [&](int row, double acc, double) { a.q[row] = acc; });
            rrp = block_sum(rrp, smem);
            if (threadIdx.x == 0) a.partials[5 * G + t.rank] = rrp;
            NSF_PIPE_BARRIER();
            rr = grid_sum(a.partials + 5 * G, G, smem);
            if (met) ++checks;
            if (!(rr == rr) || isinf(rr)) { status = NSF_ERR_BREAKDOWN; break; }
            if (rr <= target) { status = NSF_OK; break; }
            if (it >= a.maxIt || checks >= kPipeMaxChecks) break;
            // ... then w = A r and z = A s with r.r and w.r for this k, and, since the short form of p.Ap below
            // rests on orthogonality relations the replacement breaks, r.s, p.w and p.s for the explicit
            // p.Ap = (r + beta p).(w + beta s) of the next iteration (regions 6, 7, 8)
            pipe_product<Wide>(a, rb, re, stage, [&](int c) { return a.r[c]; },
                               [&](int row, double acc, double) { wc[row] = acc; });
            double gp = 0, dp = 0, rsp = 0, pwp = 0, psp = 0;
            pipe_product<Wide>(a, rb, re, stage, [&](int c) { return k > 0 ? a.q[c] : 0.0; },
                               [&](int row, double acc, double) {
                                   const double ri = a.r[row], wi = wc[row];
                                   gp = fma(ri, ri, gp);
                                   dp = fma(wi, ri, dp);
                                   if (k > 0) {
                                       a.pbuf1[row] = acc;
                                       const double si = a.q[row], pi = a.pbuf0[row];
                                       rsp = fma(ri, si, rsp);
                                       pwp = fma(pi, wi, pwp);
                                       psp = fma(pi, si, psp);
                                   }
                               });
            gp = block_sum(gp, smem);
            dp = block_sum(dp, smem);
            rsp = block_sum(rsp, smem);
            pwp = block_sum(pwp, smem);
            psp = block_sum(psp, smem);
            if (threadIdx.x == 0) {
                a.partials[(2 * par) * G + t.rank] = gp;
                a.partials[(2 * par + 1) * G + t.rank] = dp;
                a.partials[6 * G + t.rank] = rsp;
                a.partials[7 * G + t.rank] = pwp;
                a.partials[8 * G + t.rank] = psp;
            }
            NSF_PIPE_BARRIER();
            explicitDen = k > 0;
            lastReplaced = it;
            continue;   // the same k: its gamma and delta are the replaced ones
        }
        const double beta = k == 0 ? 0.0 : gamma / gammaPrev;
        double den = k == 0 ? delta : delta - beta * gamma / alphaPrev;
        if (explicitDen) {
            const double rs = grid_sum(a.partials + 6 * G, G, smem);
            const double pw = grid_sum(a.partials + 7 * G, G, smem);
            const double ps = grid_sum(a.partials + 8 * G, G, smem);
            den = delta + beta * (rs + pw) + beta * beta * ps;
            explicitDen = false;
        }
        if (!(den > 0.0) || isinf(den)) { status = NSF_ERR_BREAKDOWN; break; }
        const double alpha = block_scalar(smem, [&] { return gamma / den; });
        double* wn = par ? a.wbuf0 : a.wbuf1;
        double gn = 0, dn = 0;
        auto gw = [&](int c) { return wc[c]; };
        auto pre = [&](int row) {
            PipeRow q;
            q.r = a.r[row];
            q.x = a.x[row];
            q.w = wc[row];
            if (k > 0) { q.z = a.pbuf1[row]; q.s = a.q[row]; q.p = a.pbuf0[row]; }
            else { q.z = 0.0; q.s = 0.0; q.p = 0.0; }
            return q;
        };
        auto epi = [&](int row, double acc, const PipeRow& q) {
            const double z = fma(beta, q.z, acc);
            const double sv = fma(beta, q.s, q.w);
            const double pv = fma(beta, q.p, q.r);
            a.pbuf1[row] = z;
            a.q[row] = sv;
            a.pbuf0[row] = pv;
            a.x[row] = fma(alpha, pv, q.x);
            const double rn = fma(-alpha, sv, q.r);
            const double wv = fma(-alpha, z, q.w);
            a.r[row] = rn;
            wn[row] = wv;
            gn = fma(rn, rn, gn);
            dn = fma(wv, rn, dn);
        };
        if constexpr (Wide) sell_rows_wide<double, double, false, 1, kUnroll>(a.sellStart, a.sellCol, a.sellVal, rb,
                                                                           re, gw, pre, epi);
        else if (a.sellMaxW <= 5) sell_rows<double, double, false, 1, 5>(a.sellStart, a.sellCol, a.sellVal, rb, re,
                                                                        gw, pre, epi);
        else sell_rows<double, double, false, 1, kUnroll>(a.sellStart, a.sellCol, a.sellVal, rb, re, gw, pre, epi);
        gn = block_sum(gn, smem);
        dn = block_sum(dn, smem);
        const int np = (k + 1) & 1;
        if (threadIdx.x == 0) { a.partials[(2 * np) * G + t.rank] = gn; a.partials[(2 * np + 1) * G + t.rank] = dn; }
        NSF_PIPE_BARRIER();
        ++it;
        ++k;
        gammaPrev = gamma;
        alphaPrev = alpha;
    }
#undef NSF_PIPE_BARRIER
    write_info(t, a, it, status, 1 + checks, rr, bb);
    return status;
}

// ---------------------------------------------------------------------------------------------------
// Mixed precision: FP32 CG with FP64 reliable updates.
// The search direction p, the product q = A32 p, the residual r32 and the accumulated correction d32 are FP32;
// the dot products and alpha/beta are FP64.  x, b and the true residual stay FP64: whenever the FP32 residual
// has fallen by the cycle's tolerance since the last true residual, d32 is folded into x, the residual b - A64 x
// is recomputed with the FP64 matrix and replaces r32, and the recurrence continues with the same search
// direction.  This is iterative refinement that keeps the Krylov recurrence instead of restarting it, so the FP32
// matrix error costs little in iteration count even on the ill-conditioned pressure system.
// Narrow systems form p_j = r32_j + beta p_prev_j per gathered entry (saving a barrier); wide (P2) systems write p
// first and gather it once.  The solve is two steps over a PcgLoop state - a refresh (fold, true residual, tests)
// and the FP32 iterations up to the next refresh - run in one launch (team_cg_mixed) or, for wide systems, as
// separate launches (the inner one at 4 CTAs per SM).
// partial regions: 0 = p.q, 1 = r32.r32, 2 = r64.r64, 3 = b.b, 4 = r32.r32 after a refresh
// ---------------------------------------------------------------------------------------------------
// Power-of-two scaling of the FP32 recurrences.  The FP32 vectors (residual, search direction, correction) carry
// the true residual times L.scale; a refresh that finds their mean square outside [2^-kScaleWindow, 2^kScaleWindow]
// multiplies them by the power of two that brings it near 1.  Sums and products of FP32 values scale exactly by
// powers of two, so the iterates and iteration counts do not depend on the scale of the system or of its
// right-hand side (subnormals aside); unscaled, a residual near 1e-19 already made p.q underflow in FP32.
constexpr int kScaleWindow = 24;
__device__ __forceinline__ double rescale_factor(double meanSquare) {
    if (!(meanSquare > 0.0) || isinf(meanSquare)) return 1.0;
    const int e = ilogb(meanSquare);
    if (e >= -kScaleWindow && e <= kScaleWindow) return 1.0;
    const int k = -(e >> 1);   // floor(e / 2): the same factor for systems a power of four apart
    return ldexp(1.0, max(-60, min(60, k)));
}

// The FP32 correction d is folded into the FP64 iterate every kFoldEvery iterations of a cycle, inside the x/r
// update (x_i += d_i / scale, d_i = 0; a row's own entries only, so no barrier), so that d's FP32 sums restart
// from zero and their rounding (about eps32 |d| per update) stays small.  Summed over a whole cycle of thousands
// of iterations, that rounding put high-frequency noise into x which the recursive residual does not see: on the
// first steps of the 2048 cavity it made refresh cycles look drifted and cost 31,078 pressure iterations over
// steps 1-5 of the run against 23,698 with the fold (the FP64 PCG's 5,985 and 6,010 at steps 1 and 2 are matched).
constexpr int kFoldEvery = 16;
__device__ __forceinline__ bool fold_iteration(const PcgLoop& L) { return (L.it + 1 - L.itRef) % kFoldEvery == 0; }
// d_i's new value, after folding it into x_i when `fold` is set
__device__ __forceinline__ float fold_correction(const CgArgs& a, int i, float dNew, bool fold, double inv) {
    if (!fold) return dNew;
    a.x[i] += (double)dNew * inv;
    return 0.0f;
}

__device__ __forceinline__ void cg_loop_init(PcgLoop& L, const CgArgs& a) {
    L.rr64 = L.bb = L.target = L.rz = L.beta = 0.0;
    L.scale = 1.0;
    L.rrBest = L.rrCycle = INFINITY;
    L.rrRef = 0.0;
    L.rr = 0.0;
    L.rrPrev = 1.0;
    L.cycleTol2 = a.innerTol2;
    L.lastCycle = 0;
    L.it = L.refresh = L.stalls = L.itRef = 0;
    L.first = 1;
    L.resetP = 1;
    L.flip = 0;
    L.innerBreakdown = 0;
    L.rflip = 0;
    L.state = kLoopRefresh;
    L.status = NSF_ERR_NOT_CONVERGED;
}

// The start of the solve (first step only): the fused right-hand side and x = x0 (own rows; the first true
// residual gathers x0, not x, so no barrier is needed).
template <bool Wide = false>
static __device__ void cg_mixed_start(Team& t, const CgArgs& a, double* stage) {
    int rb, re;
    team_rows(a.n, t, rb, re);
    build_rhs<Wide>(a, rb, re, stage);
    if (a.x != a.x0)
        for (int i = rb + (int)threadIdx.x; i < re; i += blockDim.x) a.x[i] = a.x0[i];
}

template <bool Wide = false>
static __device__ bool cg_mixed_refresh(Team& t, const CgArgs& a, double* stage, double* smem, PcgLoop& L,
                                        int& where) {
    const int G = t.size, bs = blockDim.x;
    int rb, re;
    team_rows(a.n, t, rb, re);
    const double* b = a.bRowptr ? a.bOut : a.b;
    const double sc = L.scale;
    if (!L.first) {   // fold the correction into x (FP64); the true residual gathers x across blocks
        const double inv = 1.0 / sc;
        for (int i = rb + (int)threadIdx.x; i < re; i += bs) a.x[i] += (double)a.d32[i] * inv;
        if (!t.barrier(where++)) return false;
        if (L.innerBreakdown) L.resetP = 1;   // restart the recurrence from the true residual
    }
    // true residual: r = b - A64 x; r32 = (float) (scale r); d32 = 0
    const double* xs = L.first ? a.x0 : a.x;
    double rrp = 0, bbp = 0, rip = 0;
    float* pp0 = L.flip ? a.p32b : a.p32a;
    const bool f0 = L.resetP != 0;
    matrix_product<double, double, false, kResidU<Wide>, Wide>(
        a.sellStart, a.sellCol, a.sellVal, a.rowptr, a.col, a.val, rb, re, stage, [&](int c) { return xs[c]; },
        [&](int row, double acc, double) {
            const double bi = b[row];
            const double ri = bi - acc;
            const float r32 = (float)(ri * sc);
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
    if (!t.barrier(where++)) return false;
    L.rr64 = grid_sum(a.partials + 2 * G, G, smem);
    if (L.first) {
        L.bb = grid_sum(a.partials + 3 * G, G, smem);
        L.target = L.bb > 0 ? a.tol2 * L.bb : a.tol2 * L.rr64;
    }
    const double rrTrue = grid_sum(a.partials + 4 * G, G, smem);
    L.state = kLoopDone;
    if (!(L.rr64 == L.rr64) || isinf(L.rr64)) { L.status = NSF_ERR_BREAKDOWN; return true; }
    if (L.rr64 <= L.target) { L.status = NSF_OK; return true; }
    if (L.it >= a.maxIt || L.refresh >= a.maxOuter) return true;
    // stagnation guard: a refresh cycle normally cuts the true residual norm by ~1/delta.  Three consecutive
    // cycles that gain less than 10% mean the FP32 recurrence cannot resolve this system, and the solve
    // finishes in FP64.  (CG residuals are not monotone, so single weak cycles are tolerated.)
    if (L.refresh > 0 && L.rr64 > 0.81 * L.rrBest) {
        if (++L.stalls >= 3) return true;
    } else {
        L.stalls = 0;
    }
    L.rrBest = fmin(L.rrBest, L.rr64);
    // Short refresh cycles (a well-conditioned system: the velocity systems refresh every ~3 iterations at
    // innerTol 0.1) lengthen while the FP32 recurrence stays accurate: when the true residual matches the
    // recursive one within 2x in norm, the next cycle may reduce 10x further (to 1e-4 at most); when they differ by
    // more than 4x the interval returns towards innerTol.  Long cycles (the ill-conditioned pressure system, whose
    // refreshes cost nothing next to ~1000 FP32 iterations) keep innerTol.
    if (L.refresh > 0 && L.rr > 0.0) {
        const double drift = L.rr64 * sc * sc / L.rr;
        if (drift < 4.0 && L.lastCycle < 32) L.cycleTol2 = fmax(L.cycleTol2 * 1e-2, 1e-8);
        else if (drift > 16.0) L.cycleTol2 = fmin(L.cycleTol2 * 1e2, a.innerTol2);
    }
    // continue the recurrence from the refreshed residual: beta' = |r_new|^2 / |r_prev|^2
    L.beta = L.resetP ? 0.0 : block_scalar(smem, [&] { return rrTrue / L.rrPrev; });
    L.resetP = 0;
    double rrS = rrTrue;
    const double f = rescale_factor(rrTrue / a.n);
    if (f != 1.0) {   // own rows of r32 and of the direction the next product extends; gathered after a barrier
        const float ff = (float)f;
        for (int i = rb + (int)threadIdx.x; i < re; i += bs) {
            a.r32[i] *= ff;
            pp0[i] *= ff;
        }
        rrS *= f * f;
        L.scale = sc * f;
        if (!t.barrier(where++)) return false;
    }
    L.rr = rrS;
    L.rrRef = rrS;
    L.itRef = L.it;
    ++L.refresh;
    L.first = 0;
    L.state = kLoopInner;
    return true;
}

template <bool Wide = false, bool Lean = false>
static __device__ bool cg_mixed_inner(Team& t, const CgArgs& a, double* stage, double* smem, SellRing* ring,
                                      PcgLoop& L, int& where) {
    float* stage32 = reinterpret_cast<float*>(stage);
    const int G = t.size, bs = blockDim.x;
    constexpr int R = Lean ? kRowsLean : kRows;
    int rb, re;
    team_rows(a.n, t, rb, re);
    L.innerBreakdown = 0;
    const double targetS = L.target * L.scale * L.scale;   // the stopping test in the FP32 vectors' scale
    const double invScale = 1.0 / L.scale;
    while (L.it < a.maxIt) {
        const float betaf = (float)L.beta;
        const float* pp = L.flip ? a.p32b : a.p32a;
        float* pc = L.flip ? a.p32a : a.p32b;
        const float* r32 = a.r32;
        // q = A32 p in difference form: sum_j a_ij (p_j - p_i) + rowsum_i p_i (exact row sums, see warp_spmv);
        // p.q accumulates in double-float so that the FP64 pipe does no per-row work
        float pqHi = 0.f, pqLo = 0.f;
        if constexpr (Wide) {
            // P2 rows (9 and 19 entries): p = r32 + beta p_prev is written first, so that the product gathers one
            // vector instead of forming p per gathered entry from two (one more barrier, half the gathers)
            for (int i0 = rb + (int)threadIdx.x; i0 < re; i0 += R * bs) {
#pragma unroll
                for (int u = 0; u < R; ++u) {
                    const int i = i0 + u * bs;
                    if (i < re) pc[i] = fmaf(betaf, pp[i], r32[i]);
                }
            }
            if (!t.barrier(where++)) return false;
            product32<Wide, kWideChunk32>(ring, a, rb, re, stage32, [&](int c) { return pc[c]; },
                            [&](int row, float acc, float pi) {
                                a.q32[row] = acc;
                                df_acc(pqHi, pqLo, pi, acc);
                            });
        } else {
            auto gp = [&](int c) { return fmaf(betaf, pp[c], r32[c]); };
            auto ep = [&](int row, float acc, float pi) {
                pc[row] = pi;
                a.q32[row] = acc;
                df_acc(pqHi, pqLo, pi, acc);
            };
            if (a.sellMaxW <= 5) product32<Wide, 5>(ring, a, rb, re, stage32, gp, ep);
            else product32<Wide>(ring, a, rb, re, stage32, gp, ep);
        }
        const double pq = block_sum_df(pqHi, pqLo, smem);
        if (threadIdx.x == 0) a.partials[t.rank] = pq;
        if (!t.barrier(where++)) return false;
        const double pqs = grid_sum(a.partials, G, smem);
        if (!(pqs > 0.0) || isinf(pqs)) { L.innerBreakdown = 1; break; }
        const float alphaf = (float)block_scalar(smem, [&] { return L.rr / pqs; });
        const bool fold = fold_iteration(L);
        float rrHi = 0.f, rrLo = 0.f;
        for (int i0 = rb + (int)threadIdx.x; i0 < re; i0 += R * bs) {
            float pi[R], qi[R], di[R], ri[R];
#pragma unroll
            for (int u = 0; u < R; ++u) {
                const int i = i0 + u * bs;
                if (i < re) { pi[u] = pc[i]; qi[u] = a.q32[i]; di[u] = a.d32[i]; ri[u] = a.r32[i]; }
            }
#pragma unroll
            for (int u = 0; u < R; ++u) {
                const int i = i0 + u * bs;
                if (i < re) {
                    a.d32[i] = fold_correction(a, i, fmaf(alphaf, pi[u], di[u]), fold, invScale);
                    const float rn = fmaf(-alphaf, qi[u], ri[u]);
                    a.r32[i] = rn;
                    df_acc(rrHi, rrLo, rn, rn);
                }
            }
        }
        const double rrn = block_sum_df(rrHi, rrLo, smem);
        if (threadIdx.x == 0) a.partials[G + t.rank] = rrn;
        if (!t.barrier(where++)) return false;
        const double rrs = grid_sum(a.partials + G, G, smem);
        ++L.it;
        L.flip ^= 1;
        if (!(rrs == rrs) || isinf(rrs)) { L.innerBreakdown = 1; break; }
        L.beta = block_scalar(smem, [&] { return rrs / L.rr; });
        L.rrPrev = L.rr;
        L.rr = rrs;
        if (L.rr <= L.cycleTol2 * L.rrRef || L.rr <= targetS) break;   // time for a true residual
        if (L.it - L.itRef >= kMaxInnerBetweenRefresh) break;           // bound the work between true residuals
    }
    L.lastCycle = L.it - L.itRef;
    L.state = kLoopRefresh;
    return true;
}

// The end of a plain mixed solve (state kLoopDone): when it stalled short of the tolerance with budget left, the
// plain FP64 method from the current iterate (x is complete; the right-hand side is final, so the fused build is
// not repeated); then the solve's info.
template <bool Wide = false>
static __device__ int cg_mixed_finish(Team& t, const CgArgs& a, double* stage, double* smem, const PcgLoop& L) {
    if (L.status == NSF_ERR_NOT_CONVERGED && L.it < a.maxIt) {
        CgArgs f = a;
        f.bRowptr = nullptr;
        f.b = a.bRowptr ? a.bOut : a.b;
        f.x0 = a.x;
        f.maxIt = a.maxIt - L.it;
        const int fst = team_cg_fp64<Wide>(t, f, stage, smem);
        if (fst == NSF_ERR_BARRIER_TIMEOUT) return fst;
        if (t.rank == 0 && threadIdx.x == 0) {
            a.info->iterations += L.it;
            a.info->outer = L.refresh;
            a.info->fallback = 1;   // finished in FP64
        }
        return fst;
    }
    write_info(t, a, L.it, L.status, L.refresh, L.rr64, L.bb);
    return L.status;
}

template <bool Wide = false>
static __device__ int team_cg_mixed(Team& t, const CgArgs& a, double* stage, double* smem, SellRing* ring = nullptr) {
    cg_mixed_start<Wide>(t, a, stage);
    PcgLoop L;
    cg_loop_init(L, a);
    int where = 10;
    while (true) {
        if (!cg_mixed_refresh<Wide>(t, a, stage, smem, L, where) ||
            (L.state == kLoopInner && !cg_mixed_inner<Wide>(t, a, stage, smem, ring, L, where))) {
            write_info(t, a, L.it, NSF_ERR_BARRIER_TIMEOUT, L.refresh, L.rr64, L.bb);
            return NSF_ERR_BARRIER_TIMEOUT;
        }
        if (L.state == kLoopDone) break;
    }
    return cg_mixed_finish<Wide>(t, a, stage, smem, L);
}

}  // namespace nsf
