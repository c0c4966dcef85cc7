// Internal interfaces of the learned preconditioner: the tensor-core dense layer (nsf_tc_gemm.cu) and the
// message-passing network with its trainer (nsf_learn.cu).
#pragma once
#include <cuda_bf16.h>

#include "nsf_internal.cuh"

namespace nsf {

// One source of the dense layer's input rows: row r reads base[(index ? index[r] : r) * width + 0 .. width)
// (index -1: zeros).
struct TcSeg {
    const float* base;
    const int* index;
    int width;
};

enum TcEpilogue {
    TC_EPI_NONE = 0,        // y = acc (+ bias) (+ resid)
    TC_EPI_RELU = 1,        // ypre = acc + bias; y = max(ypre, 0) (+ resid)
    TC_EPI_RELU_MASK = 2    // y = aux > 0 ? acc : 0  (gradient through a ReLU whose pre-activation is aux)
};

struct TcArgs {
    TcSeg seg[3];
    int nseg;
    int rows;
    int K;                        // sum of the segment widths, a multiple of 16 (<= 128)
    const __nv_bfloat16* B;       // N x K, row-major (the K-major B operand): y = x W^T for W = B
    int N;                        // multiple of 16 (<= 128)
    const float* bias;            // N or null
    int epi;
    const float* aux;             // rows x N (TC_EPI_RELU_MASK)
    float* Y;                     // rows x N
    float* Ypre;                  // rows x N or null (TC_EPI_RELU)
    const float* resid;           // rows x N or null
    int* error;                   // raised on a barrier time-out
    long long timeoutNs;
    int vec8;                     // set by tc_dense: stage the A tile 8 values (16 bytes) at a time
};

void tc_dense(const TcArgs& a, cudaStream_t s, int sms);

// Weight gradients of a dense layer: part[b][k][o] = sum over CTA b's rows of bf16(X[r][k]) bf16(G[r][o]) (k < K)
// and part[b][K][o] = sum of bf16(G[r][o]) (the bias), FP32 accumulation on the tensor cores.
struct TcWgradArgs {
    TcSeg seg[3];
    int nseg;
    int K;                        // sum of the segment widths, K + 1 <= 128
    int rows;
    const float* G;               // rows x N
    int N;                        // multiple of 16 (<= 128)
    int chunk;                    // rows per CTA (set by tc_wgrad)
    float* part;                  // CTAs x (K + 1) x N
    int* error;                   // raised on a time-out
    long long timeoutNs;
};
int tc_wgrad(const TcWgradArgs& a, cudaStream_t s, int sms);
// CTAs (= partial rows) tc_wgrad uses for `rows` rows on `sms` SMs
int tc_wgrad_blocks(int rows, int sms);

}  // namespace nsf
