// Dense layers of the learned preconditioner on the tensor cores: Y = epilogue(X W^T) with X gathered row by row
// from up to three FP32 sources (edge features plus the two end nodes' features, say), rounded to BF16 in shared
// memory, W in BF16, FP32 accumulation in tensor memory.
//
// One CTA of 128 threads owns a 128-row tile at a time (persistent over tiles).  The threads stage the tile in the
// canonical no-swizzle K-major layout, one thread issues K / 16 tcgen05.mma (M = 128, N <= 128, K = 16) into TMEM
// and commits them to an mbarrier, then each warp reads its 32 TMEM lanes (= 32 rows) back with tcgen05.ld for the
// fused epilogue (bias, ReLU, ReLU-mask for the backward pass, residual).  Every wait is bounded; on a time-out the
// kernel raises the error word, waits (bounded) for its MMAs, frees TMEM and leaves.
#include <algorithm>
#include <vector>

#include "nsf_internal.cuh"
#include "nsf_tc.cuh"
#include "nsf_learn.h"

namespace nsf {

namespace {
constexpr int kTcThreads = 128;
constexpr int kTcM = 128;

__device__ __forceinline__ float seg_value(const TcArgs& g, int row, int k) {
    int s = 0;
    while (s + 1 < g.nseg && k >= g.seg[s].width) {
        k -= g.seg[s].width;
        ++s;
    }
    const TcSeg& sg = g.seg[s];
    const int src = sg.index ? sg.index[row] : row;
    return src >= 0 ? sg.base[(size_t)src * sg.width + k] : 0.0f;
}
}  // namespace

__global__ void __launch_bounds__(kTcThreads, 1) tc_dense_kernel(TcArgs g) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmemBase;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int K = g.K, N = g.N;
    __nv_bfloat16* sA = reinterpret_cast<__nv_bfloat16*>(sm);
    __nv_bfloat16* sB = reinterpret_cast<__nv_bfloat16*>(sm + (size_t)kTcM * K * 2);
    const uint32_t ncols = N <= 32 ? 32u : (N <= 64 ? 64u : 128u);
    if (warp == 0) tc::tmem_alloc(&tmemBase, ncols);
    if (tid == 0) tc::mbar_init(&mbar, 1);
    for (int e = tid; e < N * K; e += kTcThreads) {
        const int n = e / K, k = e - n * K;
        sB[tc::core_offset(n, k, K)] = g.B[e];
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmemBase;
    const uint32_t idesc = tc::idesc_bf16(kTcM, N);
    const uint32_t aBase = tc::smem_u32(sA), bBase = tc::smem_u32(sB);
    const uint32_t sbo = (uint32_t)K * 16u;   // 8-row groups of a K-wide tile
    const int tiles = (g.rows + kTcM - 1) / kTcM;
    uint32_t phase = 0;
    bool ok = true;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int r0 = tile * kTcM;
        if (g.vec8) {
            // 8 consecutive k of one row per item: two 16-byte loads from the row's source, one 16-byte store of
            // 8 BF16 values (contiguous in the core-matrix layout); four items' loads in flight per thread
            const int kg = K >> 3, items = kTcM * kg;
            for (int e0 = tid; e0 < items; e0 += 4 * kTcThreads) {
                float4 lo[4], hi[4];
                int off[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int e = e0 + u * kTcThreads;
                    lo[u] = hi[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                    off[u] = -1;
                    if (e < items) {
                        const int r = e / kg, g8 = e - r * kg;
                        int k = g8 << 3, sgi = 0;
                        while (sgi + 1 < g.nseg && k >= g.seg[sgi].width) {
                            k -= g.seg[sgi].width;
                            ++sgi;
                        }
                        const TcSeg& sg = g.seg[sgi];
                        const int row = r0 + r;
                        const int src = row < g.rows ? (sg.index ? sg.index[row] : row) : -1;
                        if (src >= 0) {
                            const float4* q = reinterpret_cast<const float4*>(sg.base + (size_t)src * sg.width + k);
                            lo[u] = q[0];
                            hi[u] = q[1];
                        }
                        off[u] = tc::core_offset(r, g8 << 3, K);
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (off[u] < 0) continue;
                    union {
                        __nv_bfloat162 h[4];
                        uint4 v;
                    } pk;
                    pk.h[0] = __floats2bfloat162_rn(lo[u].x, lo[u].y);
                    pk.h[1] = __floats2bfloat162_rn(lo[u].z, lo[u].w);
                    pk.h[2] = __floats2bfloat162_rn(hi[u].x, hi[u].y);
                    pk.h[3] = __floats2bfloat162_rn(hi[u].z, hi[u].w);
                    *reinterpret_cast<uint4*>(sA + off[u]) = pk.v;
                }
            }
        } else {
            for (int e = tid; e < kTcM * K; e += kTcThreads) {
                const int r = e / K, k = e - r * K;
                const float v = r0 + r < g.rows ? seg_value(g, r0 + r, k) : 0.0f;
                sA[tc::core_offset(r, k, K)] = __float2bfloat16_rn(v);
            }
        }
        tc::fence_proxy_async();   // generic-proxy stores -> visible to the tensor core (async proxy)
        tc::fence_before();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            for (int s = 0; s < K / 16; ++s)
                tc::mma_bf16(tmem, tc::smem_desc(aBase + s * 256u, 128u, sbo), tc::smem_desc(bBase + s * 256u, 128u, sbo),
                             idesc, s > 0);
            tc::mma_commit(&mbar);
        }
        if (!tc::mbar_wait(&mbar, phase, g.timeoutNs)) ok = false;
        if (__syncthreads_or(!ok)) {
            ok = false;
            break;
        }
        phase ^= 1u;
        tc::fence_after();
        const int row = r0 + warp * 32 + lane;
        for (int c0 = 0; c0 < N; c0 += 32) {
            float v[32];
            tc::tmem_load32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (row < g.rows) {
                float* y = g.Y + (size_t)row * N + c0;
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    float a = v[j];
                    if (g.bias) a += g.bias[c0 + j];
                    switch (g.epi) {
                        case TC_EPI_RELU:
                            if (g.Ypre) g.Ypre[(size_t)row * N + c0 + j] = a;
                            a = fmaxf(a, 0.0f);
                            break;
                        case TC_EPI_RELU_MASK:   // backward through a ReLU: keep where the pre-activation was > 0
                            a = g.aux[(size_t)row * N + c0 + j] > 0.0f ? a : 0.0f;
                            break;
                        default:
                            break;
                    }
                    if (g.resid) a += g.resid[(size_t)row * N + c0 + j];
                    y[j] = a;
                }
            }
        }
        tc::fence_before();
        __syncthreads();   // TMEM and the A tile are reused by the next tile
    }
    if (!ok) {
        if (tid == 0) atomicExch(g.error, 1);
        tc::mbar_wait(&mbar, phase, g.timeoutNs);   // the MMAs in flight, if any (bounded again)
        __syncthreads();
    }
    tc::fence_after();
    if (warp == 0) tc::tmem_free(tmem, ncols);
}

// Y[rows x N] = epilogue(X W^T) with X the concatenated segments (K columns) and W given as N x K BF16 rows.
void tc_dense(const TcArgs& a, cudaStream_t s, int sms) {
    if (a.K % 16 || a.K <= 0 || a.K > 128 || a.N % 16 || a.N <= 0 || a.N > 128) throw bad_arg("dense layer shape");
    if (a.rows <= 0) return;
    int w = 0;
    for (int i = 0; i < a.nseg; ++i) w += a.seg[i].width;
    if (w != a.K) throw bad_arg("segment widths must add up to K");
    const size_t smem = (size_t)kTcM * a.K * 2 + (size_t)a.N * a.K * 2;
    // 16-byte staging when every segment's rows are 16-byte aligned groups of 8 values
    TcArgs b = a;
    // the MMA waits never give up sooner than 200 ms (TMEM is freed only after the MMAs in flight completed)
    b.timeoutNs = std::max(a.timeoutNs, 200000000LL);
    b.vec8 = 1;
    for (int i = 0; i < a.nseg; ++i)
        if (a.seg[i].width % 8 || reinterpret_cast<uintptr_t>(a.seg[i].base) % 16) b.vec8 = 0;
    static bool attr = false;
    if (!attr) {
        NSF_CUDA(cudaFuncSetAttribute(tc_dense_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024));
        attr = true;
    }
    const int tiles = (a.rows + kTcM - 1) / kTcM;
    tc_dense_kernel<<<std::min(tiles, std::max(sms, 1)), kTcThreads, smem, s>>>(b);
    NSF_CUDA(cudaGetLastError());
    count_launch();
}

// ---------------------------------------------------------------------------------------------------
// Weight gradients of a dense layer on the tensor cores:
//     part[b][k][o] = sum over CTA b's rows r of bf16(X[r][k]) * bf16(G[r][o])   (k < K)
//     part[b][K][o] = sum over the same rows of bf16(G[r][o])                      (the bias)
// with FP32 accumulation in TMEM.  The MMA's M dimension is the input feature (K + 1 <= 128, the rows above K stay
// zero), N the layer's outputs, and its reduction dimension the edges or nodes: a CTA walks its rows in chunks of
// kWgR, stages each chunk of X^T (features x rows) and G^T (outputs x rows) transposed into the K-major core-matrix
// layout - two buffers, so that one chunk is staged while the MMAs of the previous one run - and one thread issues
// kWgR / 16 MMAs per chunk and commits them to that buffer's mbarrier.  Bounded waits; TMEM freed on every path.
// ---------------------------------------------------------------------------------------------------
namespace {
constexpr int kWgR = 128;                  // rows per chunk: the MMAs' reduction extent
constexpr int kWgM = 128;                  // MMA rows: input features plus the bias row, zero-padded
constexpr size_t kWgABytes = (size_t)kWgM * kWgR * 2;

__device__ __forceinline__ void stage8(__nv_bfloat16* dst, const float (&v)[8]) {
    union {
        __nv_bfloat162 h[4];
        uint4 u;
    } pk;
#pragma unroll
    for (int j = 0; j < 4; ++j) pk.h[j] = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
    *reinterpret_cast<uint4*>(dst) = pk.u;
}
}  // namespace

__global__ void __launch_bounds__(kTcThreads, 1) tc_wgrad_kernel(TcWgradArgs g) {
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint64_t mbar[2];
    __shared__ uint32_t tmemBase;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int K = g.K, N = g.N;
    const size_t bBytes = (size_t)N * kWgR * 2;
    const uint32_t ncols = N <= 32 ? 32u : (N <= 64 ? 64u : 128u);
    if (warp == 0) tc::tmem_alloc(&tmemBase, ncols);
    if (tid == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
    }
    // both A buffers zero once: the feature rows above K are never written again
    for (size_t e = tid; e < 2 * kWgABytes / 16; e += kTcThreads)
        reinterpret_cast<uint4*>(sm)[e] = make_uint4(0u, 0u, 0u, 0u);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmemBase;
    const uint32_t idesc = tc::idesc_bf16(kWgM, N);
    const uint32_t sbo = (uint32_t)kWgR * 16u;
    const int r0 = blockIdx.x * g.chunk, r1 = min(g.rows, r0 + g.chunk);
    const int nChunks = r1 > r0 ? (r1 - r0 + kWgR - 1) / kWgR : 0;
    bool ok = true;
    int last = -1;                     // the last chunk whose MMAs were issued
    for (int c = 0; c < nChunks && ok; ++c) {
        const int buf = c & 1;
        if (c >= 2 && !tc::mbar_wait(&mbar[buf], ((c - 2) >> 1) & 1, g.timeoutNs)) ok = false;   // buffer free
        if (__syncthreads_or(!ok)) {
            ok = false;
            break;
        }
        const int rb = r0 + c * kWgR;
        __nv_bfloat16* const tA = reinterpret_cast<__nv_bfloat16*>(sm + (buf ? kWgABytes : 0));
        __nv_bfloat16* const tB = reinterpret_cast<__nv_bfloat16*>(sm + 2 * kWgABytes + (buf ? bBytes : 0));
        // X^T: item (k, group of 8 rows): 8 values of feature k, contiguous along the reduction in the layout;
        // lanes take consecutive features of the same rows, so each of the 8 loads is one coalesced row segment
        const int itemsA = (K + 1) * (kWgR / 8);
        for (int it = tid; it < itemsA; it += kTcThreads) {
            const int rg = it / (K + 1), k = it - rg * (K + 1);
            float v[8];
            // the segment holding feature k, picked by selects (no dynamically indexed local array)
            const int w0 = g.seg[0].width, w1 = g.nseg > 1 ? g.seg[1].width : 0;
            const int sgi = k < w0 ? 0 : (k < w0 + w1 || g.nseg < 3 ? 1 : 2);
            const int kk = sgi == 0 ? k : (sgi == 1 ? k - w0 : k - w0 - w1);
            const float* const base = sgi == 0 ? g.seg[0].base : (sgi == 1 ? g.seg[1].base : g.seg[2].base);
            const int* const index = sgi == 0 ? g.seg[0].index : (sgi == 1 ? g.seg[1].index : g.seg[2].index);
            const int width = sgi == 0 ? w0 : (sgi == 1 ? w1 : g.seg[2].width);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int row = rb + 8 * rg + j;
                float x = 0.0f;
                if (row < r1) {
                    if (k == K) {
                        x = 1.0f;
                    } else {
                        const int src = index ? index[row] : row;
                        x = src >= 0 ? base[(size_t)src * width + kk] : 0.0f;
                    }
                }
                v[j] = x;
            }
            stage8(tA + tc::core_offset(k, 8 * rg, kWgR), v);
        }
        // G^T: item (output o, group of 8 rows)
        const int itemsB = N * (kWgR / 8);
        for (int it = tid; it < itemsB; it += kTcThreads) {
            const int rg = it / N, o = it - rg * N;
            float v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int row = rb + 8 * rg + j;
                v[j] = row < r1 ? g.G[(size_t)row * N + o] : 0.0f;
            }
            stage8(tB + tc::core_offset(o, 8 * rg, kWgR), v);
        }
        tc::fence_proxy_async();   // generic-proxy stores -> visible to the tensor core (async proxy)
        tc::fence_before();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            const uint32_t aBase = tc::smem_u32(tA), bBase = tc::smem_u32(tB);
            for (int s = 0; s < kWgR / 16; ++s)
                tc::mma_bf16(tmem, tc::smem_desc(aBase + s * 256u, 128u, sbo),
                             tc::smem_desc(bBase + s * 256u, 128u, sbo), idesc, c > 0 || s > 0);
            tc::mma_commit(&mbar[buf]);
        }
        last = c;
    }
    if (ok && last >= 0 && !tc::mbar_wait(&mbar[last & 1], (last >> 1) & 1, g.timeoutNs)) ok = false;
    if (__syncthreads_or(!ok)) ok = false;
    if (ok) {
        tc::fence_after();
        const int f = warp * 32 + lane;          // TMEM lane = MMA row = input feature
        float* out = g.part + (size_t)blockIdx.x * (K + 1) * N;
        for (int c0 = 0; c0 < N; c0 += 32) {
            float v[32];
            if (nChunks > 0) tc::tmem_load32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            else
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] = 0.0f;
            if (f <= K)
#pragma unroll
                for (int j = 0; j < 32; ++j) out[(size_t)f * N + c0 + j] = v[j];
        }
    } else {
        if (tid == 0) atomicExch(g.error, 1);
        if (last >= 0) tc::mbar_wait(&mbar[last & 1], (last >> 1) & 1, g.timeoutNs);   // MMAs in flight (bounded)
        __syncthreads();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0) tc::tmem_free(tmem, ncols);
}

int tc_wgrad_blocks(int rows, int sms) {
    const int chunks = (rows + kWgR - 1) / kWgR;
    return std::max(1, std::min(chunks, std::max(sms, 1)));
}

// Per-CTA weight-gradient partials of X^T G (and colsum G) on the tensor cores; returns the number of CTAs (rows of
// partials).  N a multiple of 16 (<= 128), K + 1 <= 128.
int tc_wgrad(const TcWgradArgs& a, cudaStream_t s, int sms) {
    if (a.N % 16 || a.N <= 0 || a.N > 128 || a.K <= 0 || a.K + 1 > kWgM) throw bad_arg("weight-gradient shape");
    if (a.rows <= 0) return 0;
    int w = 0;
    for (int i = 0; i < a.nseg; ++i) w += a.seg[i].width;
    if (w != a.K) throw bad_arg("segment widths must add up to K");
    const int chunks = (a.rows + kWgR - 1) / kWgR;
    const int blocks = tc_wgrad_blocks(a.rows, sms);
    TcWgradArgs b = a;
    b.chunk = ((chunks + blocks - 1) / blocks) * kWgR;
    b.timeoutNs = std::max(a.timeoutNs, 200000000LL);
    const size_t smem = 2 * kWgABytes + 2 * (size_t)a.N * kWgR * 2;
    static bool attr = false;
    if (!attr) {
        NSF_CUDA(cudaFuncSetAttribute(tc_wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
        attr = true;
    }
    tc_wgrad_kernel<<<blocks, kTcThreads, smem, s>>>(b);
    NSF_CUDA(cudaGetLastError());
    count_launch();
    return blocks;
}

}  // namespace nsf

// ---------------------------------------------------------------------------------------------------
// C entry point: one dense layer on host arrays (the tensor-core path's known-answer check)
// ---------------------------------------------------------------------------------------------------
extern "C" int nsf_tc_dense(nsf_device* h, int rows, int K, int N, const float* X, const float* W,
                            const float* bias, int epilogue, float* Y) {
    if (!h || !X || !W || !Y || rows <= 0) return NSF_ERR_BAD_ARG;
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    try {
        NSF_CUDA(cudaSetDevice(h->device));
        if (epilogue != nsf::TC_EPI_NONE && epilogue != nsf::TC_EPI_RELU) throw nsf::bad_arg("epilogue: 0 or 1");
        std::vector<__nv_bfloat16> B((size_t)N * K);
        for (int k = 0; k < K; ++k)
            for (int o = 0; o < N; ++o) B[(size_t)o * K + k] = __float2bfloat16_rn(W[(size_t)k * N + o]);
        nsf::DevBuf<float> x, y, b;
        nsf::DevBuf<__nv_bfloat16> w;
        nsf::DevBuf<int> err;
        x.upload(X, (size_t)rows * K, h->stream);
        w.upload(B.data(), B.size(), h->stream);
        if (bias) b.upload(bias, (size_t)N, h->stream);
        y.alloc((size_t)rows * N);
        err.alloc(1);
        err.zero(h->stream);
        nsf::TcArgs a{};
        a.seg[0] = {x.get(), nullptr, K};
        a.nseg = 1;
        a.rows = rows;
        a.K = K;
        a.B = w.get();
        a.N = N;
        a.bias = bias ? b.get() : nullptr;
        a.epi = epilogue;
        a.Y = y.get();
        a.error = err.get();
        a.timeoutNs = h->timeoutNs;
        nsf::tc_dense(a, h->stream, h->smCount);
        int e = 0;
        NSF_CUDA(cudaMemcpyAsync(Y, y.get(), sizeof(float) * rows * N, cudaMemcpyDeviceToHost, h->stream));
        NSF_CUDA(cudaMemcpyAsync(&e, err.get(), sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        NSF_CUDA(cudaStreamSynchronize(h->stream));
        if (e) throw nsf::Error{NSF_ERR_BARRIER_TIMEOUT, "tensor-core layer timed out"};
        return NSF_OK;
    } catch (const nsf::Error& e) {
        h->lastError = e.msg;
        return e.status;
    }
}

// The weight-gradient kernel on host arrays: its known-answer check.
extern "C" int nsf_tc_weight_gradient(nsf_device* h, int rows, int K, int N, const float* X, const float* G, float* dW,
                                      float* db) {
    if (!h || !X || !G || !dW || !db || rows <= 0) return NSF_ERR_BAD_ARG;
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    try {
        NSF_CUDA(cudaSetDevice(h->device));
        nsf::DevBuf<float> x, g, part;
        nsf::DevBuf<int> err;
        x.upload(X, (size_t)rows * K, h->stream);
        g.upload(G, (size_t)rows * N, h->stream);
        const int blocks = nsf::tc_wgrad_blocks(rows, h->smCount);
        part.alloc((size_t)blocks * (K + 1) * N);
        err.alloc(1);
        err.zero(h->stream);
        nsf::TcWgradArgs a{};
        a.seg[0] = {x.get(), nullptr, K};
        a.nseg = 1;
        a.K = K;
        a.rows = rows;
        a.G = g.get();
        a.N = N;
        a.part = part.get();
        a.error = err.get();
        a.timeoutNs = h->timeoutNs;
        const int used = nsf::tc_wgrad(a, h->stream, h->smCount);
        std::vector<float> hp((size_t)used * (K + 1) * N);
        int e = 0;
        NSF_CUDA(cudaMemcpyAsync(hp.data(), part.get(), sizeof(float) * hp.size(), cudaMemcpyDeviceToHost, h->stream));
        NSF_CUDA(cudaMemcpyAsync(&e, err.get(), sizeof(int), cudaMemcpyDeviceToHost, h->stream));
        NSF_CUDA(cudaStreamSynchronize(h->stream));
        if (e) throw nsf::Error{NSF_ERR_BARRIER_TIMEOUT, "tensor-core weight gradient timed out"};
        for (int k = 0; k <= K; ++k)
            for (int o = 0; o < N; ++o) {
                double sum = 0.0;
                for (int b = 0; b < used; ++b) sum += hp[((size_t)b * (K + 1) + k) * N + o];
                if (k < K) dW[(size_t)k * N + o] = (float)sum;
                else db[o] = (float)sum;
            }
        return NSF_OK;
    } catch (const nsf::Error& e) {
        h->lastError = e.msg;
        return e.status;
    }
}
