// The learned preconditioner: an edge-based message-passing network over the graph of the multicolour factor
// pattern that outputs the factor L (M = L L^T) of a system matrix, with its CUDA forward, backward and Adam
// kernels and the C ABI to train it on systems the plain method produced and to install its factor on a slot.
//
// The reference builds an incomplete-Cholesky preconditioner for CG (include/assembly.h:33-35, 1338-1344); this
// network replaces the incomplete factorisation on the same multicolour pattern (nsf_precond.cu).  It works on the
// diagonally scaled system A^ = D^-1/2 A D^-1/2:
//     node features [1, deg/8, sum_j a^_ij, sum_j a^_ij^2], edge features [1, a^_cp, a^_cp^2, dcolour / C]
//     h0 = relu(fn Wn0 + bn0), e0 = relu(fe We0 + be0)                          (width 32, FP32 cores)
//     3 layers: e += relu([e, h_c, h_p] W1e + b1e) W2e + b2e                     (tensor cores, BF16/FP32)
//               m_i = mean of e over the edges incident to i
//               h += relu([h, m] W1n + b1n) W2n + b2n                            (tensor cores)
//     L^_cp = e . wde + bde,  L^_ii = softplus(h . wdn + bdn),  L = D^1/2 L^
//     loss = || L^ L^T x^ - b^ ||^2 / || b^ ||^2 with x^ = D^1/2 x, b^ = D^-1/2 b (x a solution of A x = b)
// The backward pass's input-gradient products and the message-passing layers' weight gradients run on the tensor
// cores too (BF16 operands, FP32 accumulation; the 4-feature embeddings and the 1-output decoders keep FP32
// reductions); every reduction has a fixed order (deterministic).  Every gather of the message passing is a fixed-order loop
// over incidence lists, so forward and backward are deterministic as well.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "nsf_learn.h"

namespace nsf {

constexpr int kH = 32;
constexpr int kLayers = 3;
constexpr int kFn = 4, kFe = 4;

namespace {

int grid_for(int64_t work, int threads) {
    const int64_t g = (work + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 32));
}

// ---------------------------------------------------------------------------------------------------
// parameters: one flat FP32 vector, tensors in a fixed order (weights stored K_in x N_out, row-major)
// ---------------------------------------------------------------------------------------------------
struct PT {
    size_t off = 0;
    int rows = 0, cols = 0;   // a bias has rows = 1
    size_t size() const { return (size_t)rows * cols; }
};
struct NetLayout {
    PT Wn0, bn0, We0, be0;
    struct Layer {
        PT W1e, b1e, W2e, b2e, W1n, b1n, W2n, b2n;
    } L[kLayers];
    PT wde, bde, wdn, bdn;
    size_t count = 0;
    NetLayout() {
        auto add = [&](PT& p, int r, int c) {
            p.off = count;
            p.rows = r;
            p.cols = c;
            count += (size_t)r * c;
        };
        add(Wn0, kFn, kH);
        add(bn0, 1, kH);
        add(We0, kFe, kH);
        add(be0, 1, kH);
        for (auto& l : L) {
            add(l.W1e, 3 * kH, kH);
            add(l.b1e, 1, kH);
            add(l.W2e, kH, kH);
            add(l.b2e, 1, kH);
            add(l.W1n, 2 * kH, kH);
            add(l.b1n, 1, kH);
            add(l.W2n, kH, kH);
            add(l.b2n, 1, kH);
        }
        add(wde, 1, kH);
        add(bde, 1, 1);
        add(wdn, 1, kH);
        add(bdn, 1, 1);
    }
};

// ---------------------------------------------------------------------------------------------------
// small kernels
// ---------------------------------------------------------------------------------------------------
// node features from the matrix: deg, sum a^_ij, sum a^_ij^2 over the off-diagonal pattern; 1/sqrt(a_ii)
__global__ void node_features_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                                     const double* __restrict__ av, const int* __restrict__ aDiag, float* fn,
                                     float* sqrtD) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double di = av[aDiag[i]];
        const double si = 1.0 / sqrt(di);
        int deg = 0;
        double s1 = 0.0, s2 = 0.0;
        for (int k = rp[i]; k < rp[i + 1]; ++k) {
            const int j = ci[k];
            if (j == i) continue;
            ++deg;
            // a^_ij = a_ij / sqrt(a_ii a_jj): the column's diagonal is looked up through its own row
            double dj = 0.0;
            for (int q = rp[j]; q < rp[j + 1]; ++q)
                if (ci[q] == j) {
                    dj = av[q];
                    break;
                }
            const double a = av[k] * si / sqrt(dj);
            s1 += a;
            s2 += a * a;
        }
        fn[4 * (size_t)i + 0] = 1.0f;
        fn[4 * (size_t)i + 1] = (float)(deg / 8.0);
        fn[4 * (size_t)i + 2] = (float)s1;
        fn[4 * (size_t)i + 3] = (float)s2;
        sqrtD[i] = (float)sqrt(di);
    }
}

// edge features and the end points of each lower entry (child = row, parent = column)
__global__ void edge_features_kernel(int n, const int* __restrict__ lrp, const int* __restrict__ lci,
                                     const int* __restrict__ aIdx, const int* __restrict__ aDiag,
                                     const double* __restrict__ av, const unsigned char* __restrict__ colour,
                                     int colours, int* c, float* fe) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double di = av[aDiag[i]];
        for (int k = lrp[i]; k < lrp[i + 1]; ++k) {
            const int j = lci[k];
            const double a = av[aIdx[k]] / sqrt(di * av[aDiag[j]]);
            c[k] = i;
            fe[4 * (size_t)k + 0] = 1.0f;
            fe[4 * (size_t)k + 1] = (float)a;
            fe[4 * (size_t)k + 2] = (float)(a * a);
            fe[4 * (size_t)k + 3] = (float)((double)colour[i] - colour[j]) / (float)colours;
        }
    }
}

// y = relu(x W + b) for a K-wide input (the encoders; K = 4), pre-activation kept
__global__ void encoder_kernel(int rows, int K, const float* __restrict__ x, const float* __restrict__ W,
                               const float* __restrict__ b, float* pre, float* y) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)rows * kH;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(t / kH), o = (int)(t % kH);
        float a = b[o];
        for (int k = 0; k < K; ++k) a = fmaf(x[(size_t)r * K + k], W[k * kH + o], a);
        pre[t] = a;
        y[t] = fmaxf(a, 0.0f);
    }
}

// m_i = (sum of e over edges with child i, then over edges with parent i) / max(1, incident count)
__global__ void aggregate_kernel(int n, const int* __restrict__ lrp, const int* __restrict__ uprp,
                                 const int* __restrict__ upEdge, const float* __restrict__ e, float* m) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)n * kH;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t / kH), o = (int)(t % kH);
        float s = 0.0f;
        for (int k = lrp[i]; k < lrp[i + 1]; ++k) s += e[(size_t)k * kH + o];
        for (int q = uprp[i]; q < uprp[i + 1]; ++q) s += e[(size_t)upEdge[q] * kH + o];
        const int cnt = (lrp[i + 1] - lrp[i]) + (uprp[i + 1] - uprp[i]);
        m[t] = s / (float)max(cnt, 1);
    }
}

// adjoint of aggregate_kernel: dE[k] += dM[c_k] / cnt(c_k) + dM[p_k] / cnt(p_k)
__global__ void aggregate_adjoint_kernel(int m, const int* __restrict__ c, const int* __restrict__ p,
                                         const int* __restrict__ lrp, const int* __restrict__ uprp,
                                         const float* __restrict__ dY, int ldY, int colY, float* dE) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)m * kH;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / kH), o = (int)(t % kH);
        const int a = c[k], b = p[k];
        const int ca = max((lrp[a + 1] - lrp[a]) + (uprp[a + 1] - uprp[a]), 1);
        const int cb = max((lrp[b + 1] - lrp[b]) + (uprp[b + 1] - uprp[b]), 1);
        dE[t] += dY[(size_t)a * ldY + colY + o] / (float)ca + dY[(size_t)b * ldY + colY + o] / (float)cb;
    }
}

// adjoint of the gather of node features onto edges: dH[i] += sum over edges with child i of dX[k][colC..] and
// over edges with parent i of dX[k][colP..]
__global__ void gather_adjoint_kernel(int n, const int* __restrict__ lrp, const int* __restrict__ uprp,
                                      const int* __restrict__ upEdge, const float* __restrict__ dX, int ldX, int colC,
                                      int colP, float* dH) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)n * kH;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t / kH), o = (int)(t % kH);
        float s = 0.0f;
        for (int k = lrp[i]; k < lrp[i + 1]; ++k) s += dX[(size_t)k * ldX + colC + o];
        for (int q = uprp[i]; q < uprp[i + 1]; ++q) s += dX[(size_t)upEdge[q] * ldX + colP + o];
        dH[t] += s;
    }
}

// y[:, 0:32] (+)= x[:, col:col+32] for a row-major source of width ld (a column slice copy / add)
__global__ void slice_kernel(int rows, const float* __restrict__ x, int ld, int col, float* y, int add) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)rows * kH;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(t / kH), o = (int)(t % kH);
        const float v = x[(size_t)r * ld + col + o];
        y[t] = add ? y[t] + v : v;
    }
}

__global__ void relu_mask_kernel(int64_t count, const float* __restrict__ pre, float* d) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x)
        if (!(pre[t] > 0.0f)) d[t] = 0.0f;
}

// decoder: lower[k] = e[k] . wde + bde;  tdiag[i] = h[i] . wdn + bdn;  diag = softplus(tdiag)
__global__ void decoder_kernel(int m, int n, const float* __restrict__ e, const float* __restrict__ h,
                               const float* __restrict__ theta, size_t wde, size_t bde, size_t wdn, size_t bdn,
                               float* lower, float* tdiag, float* diag) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)m + n;
         t += (int64_t)gridDim.x * blockDim.x) {
        if (t < m) {
            float a = theta[bde];
            for (int o = 0; o < kH; ++o) a = fmaf(e[(size_t)t * kH + o], theta[wde + o], a);
            lower[t] = a;
        } else {
            const int64_t i = t - m;
            float a = theta[bdn];
            for (int o = 0; o < kH; ++o) a = fmaf(h[(size_t)i * kH + o], theta[wdn + o], a);
            tdiag[i] = a;
            diag[i] = a > 20.0f ? a : log1pf(expf(a));
        }
    }
}

// y = L^T x (per column p: d_p x_p + sum over edges with parent p of lower_k x_{c_k})
__global__ void ltx_kernel(int n, const int* __restrict__ uprp, const int* __restrict__ upEdge,
                           const int* __restrict__ c, const float* __restrict__ lower,
                           const float* __restrict__ diag, const float* __restrict__ x, float* y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float s = diag[i] * x[i];
        for (int q = uprp[i]; q < uprp[i + 1]; ++q) {
            const int k = upEdge[q];
            s = fmaf(lower[k], x[c[k]], s);
        }
        y[i] = s;
    }
}

// z = L y (per row c: d_c y_c + sum over edges with child c of lower_k y_{p_k}); rho = z - b
__global__ void lx_kernel(int n, const int* __restrict__ lrp, const int* __restrict__ p,
                          const float* __restrict__ lower, const float* __restrict__ diag,
                          const float* __restrict__ y, const float* __restrict__ b, float* rho) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float s = diag[i] * y[i];
        for (int k = lrp[i]; k < lrp[i + 1]; ++k) s = fmaf(lower[k], y[p[k]], s);
        rho[i] = s - (b ? b[i] : 0.0f);
    }
}

// per-block partial sums of x[i] * y[i] (deterministic: fixed blocks, fixed order)
__global__ void dot_partial_kernel(int n, const float* __restrict__ x, const float* __restrict__ y, double* part) {
    __shared__ double sh[256];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        s += (double)x[i] * (double)y[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// gradient of the loss at the decoder outputs: gz = 2 rho / bb (given), u = L^T gz;
// dlower[k] = gz[c_k] y[p_k] + u[p_k] x[c_k],  dt[i] = (gz_i y_i + u_i x_i) * sigmoid(tdiag_i)
__global__ void decoder_grad_kernel(int m, int n, const int* __restrict__ c, const int* __restrict__ p,
                                    const float* __restrict__ gz, const float* __restrict__ u,
                                    const float* __restrict__ y, const float* __restrict__ x,
                                    const float* __restrict__ tdiag, float* dlower, float* dt) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)m + n;
         t += (int64_t)gridDim.x * blockDim.x) {
        if (t < m) {
            dlower[t] = gz[c[t]] * y[p[t]] + u[p[t]] * x[c[t]];
        } else {
            const int64_t i = t - m;
            dt[i] = (gz[i] * y[i] + u[i] * x[i]) / (1.0f + expf(-tdiag[i]));
        }
    }
}

// dE[k][o] = dlower[k] * w[o] (the decoder's input gradient, for edges or nodes)
__global__ void outer_kernel(int rows, const float* __restrict__ d, const float* __restrict__ theta, size_t w,
                             float* out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)rows * kH;
         t += (int64_t)gridDim.x * blockDim.x)
        out[t] = d[t / kH] * theta[w + t % kH];
}

// Weight gradient partials: part[b][k][o] = sum over the block's rows of X[r][k] * G[r][o] (K x N, plus a row of
// ones for the bias: k = K).  X is the concatenation of up to three gathered segments, like the dense layers.
constexpr int kWgRows = 64;
__global__ void wgrad_kernel(TcSeg s0, TcSeg s1, TcSeg s2, int nseg, int K, int rows, const float* __restrict__ G,
                             int N, int chunk, float* part) {
    extern __shared__ float wsm[];
    float* sx = wsm;                      // kWgRows x (K + 1)
    float* sg = wsm + kWgRows * (K + 1);  // kWgRows x N
    const TcSeg segs[3] = {s0, s1, s2};
    const int r0 = blockIdx.x * chunk, r1 = min(rows, r0 + chunk);
    const int outs = (K + 1) * N;
    float acc[16];
    const int per = (outs + blockDim.x - 1) / blockDim.x;   // <= 16 for K <= 96, N = 32, 256 threads
    for (int j = 0; j < 16; ++j) acc[j] = 0.0f;
    for (int rb = r0; rb < r1; rb += kWgRows) {
        const int nr = min(kWgRows, r1 - rb);
        for (int e = threadIdx.x; e < nr * (K + 1); e += blockDim.x) {
            const int r = e / (K + 1), k = e % (K + 1);
            float v = 1.0f;
            if (k < K) {
                int s = 0, kk = k;
                while (s + 1 < nseg && kk >= segs[s].width) {
                    kk -= segs[s].width;
                    ++s;
                }
                const int src = segs[s].index ? segs[s].index[rb + r] : rb + r;
                v = src >= 0 ? segs[s].base[(size_t)src * segs[s].width + kk] : 0.0f;
            }
            sx[e] = v;
        }
        for (int e = threadIdx.x; e < nr * N; e += blockDim.x) sg[e] = G[(size_t)(rb + e / N) * N + e % N];
        __syncthreads();
        for (int j = 0; j < per; ++j) {
            const int q = threadIdx.x + j * blockDim.x;
            if (q < outs) {
                const int k = q / N, o = q % N;
                float a = acc[j];
                for (int r = 0; r < nr; ++r) a = fmaf(sx[r * (K + 1) + k], sg[r * N + o], a);
                acc[j] = a;
            }
        }
        __syncthreads();
    }
    for (int j = 0; j < per; ++j) {
        const int q = threadIdx.x + j * blockDim.x;
        if (q < outs) part[(size_t)blockIdx.x * outs + q] = acc[j];
    }
}

// grad[wOff + k*N + o] += sum_b part[b][k][o] (k < K); grad[bOff + o] += sum_b part[b][K][o]
__global__ void wgrad_reduce_kernel(int blocks, int K, int N, const float* __restrict__ part, float* grad,
                                    size_t wOff, size_t bOff) {
    const int outs = (K + 1) * N;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < outs; q += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < blocks; ++b) s += part[(size_t)b * outs + q];
        const int k = q / N, o = q % N;
        if (k < K) grad[wOff + (size_t)k * N + o] += (float)s;
        else grad[bOff + o] += (float)s;
    }
}

// weights -> BF16 B operands: forward W^T (N_out x K_in) and backward W (K_in x N_out)
__global__ void to_bf16_kernel(int K, int N, const float* __restrict__ W, __nv_bfloat16* fwd, __nv_bfloat16* bwd) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < K * N; t += gridDim.x * blockDim.x) {
        const int k = t / N, o = t % N;
        const __nv_bfloat16 v = __float2bfloat16_rn(W[t]);
        fwd[(size_t)o * K + k] = v;
        bwd[t] = v;
    }
}

__global__ void adam_kernel(size_t count, float* theta, const float* __restrict__ grad, float* m, float* v, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < count; t += (size_t)gridDim.x * blockDim.x) {
        const float g = grad[t];
        const float mt = b1 * m[t] + (1.0f - b1) * g;
        const float vt = b2 * v[t] + (1.0f - b2) * g * g;
        m[t] = mt;
        v[t] = vt;
        theta[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
    }
}

}  // namespace

// ---------------------------------------------------------------------------------------------------
// systems and the tape
// ---------------------------------------------------------------------------------------------------
struct LSystem {
    int n = 0, m = 0, colours = 0, slot = -1;
    DevBuf<int> c, p, lrp, uprp, upEdge;
    DevBuf<float> fn, fe, sqrtD, xh, bh;
};

struct LTape {
    int n = 0, m = 0;
    DevBuf<float> E[kLayers + 1], H[kLayers + 1], PU[kLayers], U[kLayers], PV[kLayers], V[kLayers], MG[kLayers];
    DevBuf<float> e0pre, h0pre, lower, tdiag, diag, y, rho, gz, u, dlower, dt;
    DevBuf<float> dE, dE2, dH, dH2, dPU, dPV, dX, dY;
    void ensure(int n_, int m_) {
        if (n_ <= n && m_ <= m) return;
        n = std::max(n, n_);
        m = std::max(m, m_);
        const size_t en = (size_t)m * kH, nn = (size_t)n * kH;
        for (auto& b : E) b.alloc(en);
        for (auto& b : H) b.alloc(nn);
        for (int l = 0; l < kLayers; ++l) {
            PU[l].alloc(en);
            U[l].alloc(en);
            PV[l].alloc(nn);
            V[l].alloc(nn);
            MG[l].alloc(nn);
        }
        e0pre.alloc(en);
        h0pre.alloc(nn);
        lower.alloc(std::max(m, 1));
        tdiag.alloc(n);
        diag.alloc(n);
        y.alloc(n);
        rho.alloc(n);
        gz.alloc(n);
        u.alloc(n);
        dlower.alloc(std::max(m, 1));
        dt.alloc(n);
        dE.alloc(en);
        dE2.alloc(en);
        dH.alloc(nn);
        dH2.alloc(nn);
        dPU.alloc(en);
        dPV.alloc(nn);
        dX.alloc((size_t)m * 3 * kH);
        dY.alloc((size_t)n * 2 * kH);
    }
};

}  // namespace nsf

struct nsf_learner {
    nsf_device* h = nullptr;
    nsf::NetLayout net;
    nsf::DevBuf<float> theta, am, av, grad, part;
    nsf::DevBuf<__nv_bfloat16> wb;    // BF16 B operands: per layer W1e, W2e, W1n, W2n, forward then backward
    size_t wbOff[nsf::kLayers][4][2] = {};
    std::vector<std::unique_ptr<nsf::LSystem>> systems;
    nsf::LTape tape;
    nsf::DevBuf<int> err;
    nsf::DevBuf<double> dots;
    int step = 0;
    std::string lastError;
};

namespace nsf {
namespace {

const int kDotBlocks = 256;

struct Learner {
    nsf_learner* L;
    cudaStream_t s;
    int sms;
    explicit Learner(nsf_learner* l) : L(l), s(l->h->stream), sms(l->h->smCount) {}

    const PT* weights(int l, int w) const {
        const auto& y = L->net.L[l];
        const PT* t[4] = {&y.W1e, &y.W2e, &y.W1n, &y.W2n};
        return t[w];
    }
    const __nv_bfloat16* wfwd(int l, int w) const { return L->wb.get() + L->wbOff[l][w][0]; }
    const __nv_bfloat16* wbwd(int l, int w) const { return L->wb.get() + L->wbOff[l][w][1]; }
    const float* P(const PT& t) const { return L->theta.get() + t.off; }

    void refresh_bf16() {
        for (int l = 0; l < kLayers; ++l)
            for (int w = 0; w < 4; ++w) {
                const PT* t = weights(l, w);
                to_bf16_kernel<<<grid_for(t->size(), 256), 256, 0, s>>>(t->rows, t->cols, P(*t),
                                                                        L->wb.get() + L->wbOff[l][w][0],
                                                                        L->wb.get() + L->wbOff[l][w][1]);
                NSF_CUDA(cudaGetLastError());
                count_launch();
            }
    }

    void dense(TcSeg a, TcSeg b, TcSeg c, int nseg, int rows, const __nv_bfloat16* B, int N, const float* bias,
               int epi, const float* aux, float* Y, float* Ypre, const float* resid) {
        TcArgs t{};
        t.seg[0] = a;
        t.seg[1] = b;
        t.seg[2] = c;
        t.nseg = nseg;
        t.rows = rows;
        t.K = a.width + (nseg > 1 ? b.width : 0) + (nseg > 2 ? c.width : 0);
        t.B = B;
        t.N = N;
        t.bias = bias;
        t.epi = epi;
        t.aux = aux;
        t.Y = Y;
        t.Ypre = Ypre;
        t.resid = resid;
        t.error = L->err.get();
        t.timeoutNs = L->h->timeoutNs;
        tc_dense(t, s, sms);
    }

    // grad[w] += X^T G, grad[b] += colsum G (X = up to three gathered segments, K columns)
    void wgrad(TcSeg a, TcSeg b, TcSeg c, int nseg, int rows, const float* G, int N, const PT& w, const PT& bias) {
        if (rows <= 0) return;
        const int K = a.width + (nseg > 1 ? b.width : 0) + (nseg > 2 ? c.width : 0);
        const int blocks = std::min(4 * std::max(sms, 1), (rows + kWgRows - 1) / kWgRows);
        const int chunk = (rows + blocks - 1) / blocks;
        const size_t outs = (size_t)(K + 1) * N;
        L->part.ensure(outs * blocks);
        const size_t smem = sizeof(float) * kWgRows * ((K + 1) + N);
        wgrad_kernel<<<blocks, 256, smem, s>>>(a, b, c, nseg, K, rows, G, N, chunk, L->part.get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
        wgrad_reduce_kernel<<<grid_for(outs, 128), 128, 0, s>>>(blocks, K, N, L->part.get(), L->grad.get(), w.off,
                                                                bias.off);
        NSF_CUDA(cudaGetLastError());
        count_launch();
    }

    // The message-passing layers' weight gradients on the tensor cores: bf16(X)^T bf16(G) and the bias colsum,
    // FP32 accumulation in TMEM, per-CTA partials summed in a fixed order.
    void wgrad_tc(TcSeg a, TcSeg b, TcSeg c, int nseg, int rows, const float* G, int N, const PT& w,
                  const PT& bias) {
        if (rows <= 0) return;
        TcWgradArgs t{};
        t.seg[0] = a;
        t.seg[1] = b;
        t.seg[2] = c;
        t.nseg = nseg;
        t.K = a.width + (nseg > 1 ? b.width : 0) + (nseg > 2 ? c.width : 0);
        t.rows = rows;
        t.G = G;
        t.N = N;
        const size_t outs = (size_t)(t.K + 1) * N;
        L->part.ensure(outs * tc_wgrad_blocks(rows, sms));
        t.part = L->part.get();
        t.error = L->err.get();
        t.timeoutNs = L->h->timeoutNs;
        const int blocks = tc_wgrad(t, s, sms);
        wgrad_reduce_kernel<<<grid_for(outs, 128), 128, 0, s>>>(blocks, t.K, N, L->part.get(), L->grad.get(), w.off,
                                                                bias.off);
        NSF_CUDA(cudaGetLastError());
        count_launch();
    }

    double dot(int n, const float* x, const float* y) {
        dot_partial_kernel<<<kDotBlocks, 256, 0, s>>>(n, x, y, L->dots.get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
        std::vector<double> h(kDotBlocks);
        NSF_CUDA(cudaMemcpyAsync(h.data(), L->dots.get(), sizeof(double) * kDotBlocks, cudaMemcpyDeviceToHost, s));
        NSF_CUDA(cudaStreamSynchronize(s));
        double t = 0.0;
        for (double v : h) t += v;
        return t;
    }

    void forward(const LSystem& S) {
        LTape& T = L->tape;
        T.ensure(S.n, S.m);
        const NetLayout& N = L->net;
        const int n = S.n, m = S.m;
        encoder_kernel<<<grid_for((int64_t)n * kH, 256), 256, 0, s>>>(n, kFn, S.fn.get(), P(N.Wn0), P(N.bn0),
                                                                      T.h0pre.get(), T.H[0].get());
        encoder_kernel<<<grid_for((int64_t)m * kH, 256), 256, 0, s>>>(m, kFe, S.fe.get(), P(N.We0), P(N.be0),
                                                                      T.e0pre.get(), T.E[0].get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
        count_launch();
        const TcSeg none{nullptr, nullptr, 0};
        for (int l = 0; l < kLayers; ++l) {
            const auto& y = N.L[l];
            if (m > 0) {
                dense({T.E[l].get(), nullptr, kH}, {T.H[l].get(), S.c.get(), kH}, {T.H[l].get(), S.p.get(), kH}, 3, m,
                      wfwd(l, 0), kH, P(y.b1e), TC_EPI_RELU, nullptr, T.U[l].get(), T.PU[l].get(), nullptr);
                dense({T.U[l].get(), nullptr, kH}, none, none, 1, m, wfwd(l, 1), kH, P(y.b2e), TC_EPI_NONE, nullptr,
                      T.E[l + 1].get(), nullptr, T.E[l].get());
            }
            aggregate_kernel<<<grid_for((int64_t)n * kH, 256), 256, 0, s>>>(n, S.lrp.get(), S.uprp.get(),
                                                                            S.upEdge.get(), T.E[l + 1].get(),
                                                                            T.MG[l].get());
            NSF_CUDA(cudaGetLastError());
            count_launch();
            dense({T.H[l].get(), nullptr, kH}, {T.MG[l].get(), nullptr, kH}, none, 2, n, wfwd(l, 2), kH, P(y.b1n),
                  TC_EPI_RELU, nullptr, T.V[l].get(), T.PV[l].get(), nullptr);
            dense({T.V[l].get(), nullptr, kH}, none, none, 1, n, wfwd(l, 3), kH, P(y.b2n), TC_EPI_NONE, nullptr,
                  T.H[l + 1].get(), nullptr, T.H[l].get());
        }
        decoder_kernel<<<grid_for((int64_t)m + n, 256), 256, 0, s>>>(m, n, T.E[kLayers].get(), T.H[kLayers].get(),
                                                                     L->theta.get(), N.wde.off, N.bde.off, N.wdn.off,
                                                                     N.bdn.off, T.lower.get(), T.tdiag.get(),
                                                                     T.diag.get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
    }

    // loss of system S and its gradient accumulated into grad (scaled by `scale`)
    double loss_backward(const LSystem& S, float scale) {
        LTape& T = L->tape;
        const NetLayout& N = L->net;
        const int n = S.n, m = S.m;
        const TcSeg none{nullptr, nullptr, 0};
        ltx_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, S.uprp.get(), S.upEdge.get(), S.c.get(), T.lower.get(),
                                                    T.diag.get(), S.xh.get(), T.y.get());
        lx_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, S.lrp.get(), S.p.get(), T.lower.get(), T.diag.get(), T.y.get(),
                                                   S.bh.get(), T.rho.get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
        count_launch();
        const double bb = dot(n, S.bh.get(), S.bh.get());
        const double rr = dot(n, T.rho.get(), T.rho.get());
        const double loss = bb > 0 ? rr / bb : rr;
        // gz = 2 rho / bb (times the batch scale); u = L^T gz
        {
            const float f = (float)(2.0 / (bb > 0 ? bb : 1.0)) * scale;
            scale_copy(n, T.rho.get(), f, T.gz.get());
        }
        ltx_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, S.uprp.get(), S.upEdge.get(), S.c.get(), T.lower.get(),
                                                    T.diag.get(), T.gz.get(), T.u.get());
        decoder_grad_kernel<<<grid_for((int64_t)m + n, 256), 256, 0, s>>>(m, n, S.c.get(), S.p.get(), T.gz.get(),
                                                                          T.u.get(), T.y.get(), S.xh.get(),
                                                                          T.tdiag.get(), T.dlower.get(), T.dt.get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
        count_launch();
        wgrad({T.E[kLayers].get(), nullptr, kH}, none, none, 1, m, T.dlower.get(), 1, N.wde, N.bde);
        wgrad({T.H[kLayers].get(), nullptr, kH}, none, none, 1, n, T.dt.get(), 1, N.wdn, N.bdn);
        outer_kernel<<<grid_for((int64_t)m * kH, 256), 256, 0, s>>>(m, T.dlower.get(), L->theta.get(), N.wde.off,
                                                                    T.dE.get());
        outer_kernel<<<grid_for((int64_t)n * kH, 256), 256, 0, s>>>(n, T.dt.get(), L->theta.get(), N.wdn.off,
                                                                    T.dH.get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
        count_launch();
        for (int l = kLayers - 1; l >= 0; --l) {
            const auto& y = N.L[l];
            // node update: h' = h + relu([h, m] W1n + b1n) W2n + b2n
            wgrad_tc({T.V[l].get(), nullptr, kH}, none, none, 1, n, T.dH.get(), kH, y.W2n, y.b2n);
            dense({T.dH.get(), nullptr, kH}, none, none, 1, n, wbwd(l, 3), kH, nullptr, TC_EPI_RELU_MASK,
                  T.PV[l].get(), T.dPV.get(), nullptr, nullptr);
            wgrad_tc({T.H[l].get(), nullptr, kH}, {T.MG[l].get(), nullptr, kH}, none, 2, n, T.dPV.get(), kH, y.W1n,
                     y.b1n);
            dense({T.dPV.get(), nullptr, kH}, none, none, 1, n, wbwd(l, 2), 2 * kH, nullptr, TC_EPI_NONE, nullptr,
                  T.dY.get(), nullptr, nullptr);
            slice_kernel<<<grid_for((int64_t)n * kH, 256), 256, 0, s>>>(n, T.dH.get(), kH, 0, T.dH2.get(), 0);
            slice_kernel<<<grid_for((int64_t)n * kH, 256), 256, 0, s>>>(n, T.dY.get(), 2 * kH, 0, T.dH2.get(), 1);
            NSF_CUDA(cudaGetLastError());
            count_launch();
            count_launch();
            if (m > 0) {
                aggregate_adjoint_kernel<<<grid_for((int64_t)m * kH, 256), 256, 0, s>>>(
                    m, S.c.get(), S.p.get(), S.lrp.get(), S.uprp.get(), T.dY.get(), 2 * kH, kH, T.dE.get());
                NSF_CUDA(cudaGetLastError());
                count_launch();
                // edge update: e' = e + relu([e, h_c, h_p] W1e + b1e) W2e + b2e
                wgrad_tc({T.U[l].get(), nullptr, kH}, none, none, 1, m, T.dE.get(), kH, y.W2e, y.b2e);
                dense({T.dE.get(), nullptr, kH}, none, none, 1, m, wbwd(l, 1), kH, nullptr, TC_EPI_RELU_MASK,
                      T.PU[l].get(), T.dPU.get(), nullptr, nullptr);
                wgrad_tc({T.E[l].get(), nullptr, kH}, {T.H[l].get(), S.c.get(), kH}, {T.H[l].get(), S.p.get(), kH},
                         3, m, T.dPU.get(), kH, y.W1e, y.b1e);
                dense({T.dPU.get(), nullptr, kH}, none, none, 1, m, wbwd(l, 0), 3 * kH, nullptr, TC_EPI_NONE,
                      nullptr, T.dX.get(), nullptr, nullptr);
                slice_kernel<<<grid_for((int64_t)m * kH, 256), 256, 0, s>>>(m, T.dE.get(), kH, 0, T.dE2.get(), 0);
                slice_kernel<<<grid_for((int64_t)m * kH, 256), 256, 0, s>>>(m, T.dX.get(), 3 * kH, 0, T.dE2.get(), 1);
                gather_adjoint_kernel<<<grid_for((int64_t)n * kH, 256), 256, 0, s>>>(
                    n, S.lrp.get(), S.uprp.get(), S.upEdge.get(), T.dX.get(), 3 * kH, kH, 2 * kH, T.dH2.get());
                NSF_CUDA(cudaGetLastError());
                count_launch();
                count_launch();
                count_launch();
                std::swap(T.dE, T.dE2);
            }
            std::swap(T.dH, T.dH2);
        }
        relu_mask_kernel<<<grid_for((int64_t)n * kH, 256), 256, 0, s>>>((int64_t)n * kH, T.h0pre.get(), T.dH.get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
        wgrad({S.fn.get(), nullptr, kFn}, none, none, 1, n, T.dH.get(), kH, N.Wn0, N.bn0);
        if (m > 0) {
            relu_mask_kernel<<<grid_for((int64_t)m * kH, 256), 256, 0, s>>>((int64_t)m * kH, T.e0pre.get(),
                                                                            T.dE.get());
            NSF_CUDA(cudaGetLastError());
            count_launch();
            wgrad({S.fe.get(), nullptr, kFe}, none, none, 1, m, T.dE.get(), kH, N.We0, N.be0);
        }
        return loss;
    }

    void scale_copy(int n, const float* x, float f, float* y);
};

__global__ void scale_copy_kernel(int n, const float* __restrict__ x, float f, float* y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = x[i] * f;
}

void Learner::scale_copy(int n, const float* x, float f, float* y) {
    scale_copy_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, x, f, y);
    NSF_CUDA(cudaGetLastError());
    count_launch();
}

}  // namespace
}  // namespace nsf

// ---------------------------------------------------------------------------------------------------
// systems: the graph, features and (for training) the scaled solution / right-hand side of a slot's matrix
// ---------------------------------------------------------------------------------------------------
namespace nsf {
namespace {

__global__ void scale_pair_kernel(int n, const double* __restrict__ x, const double* __restrict__ b,
                                  const float* __restrict__ sqrtD, float* xh, float* bh) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        xh[i] = (float)(x[i] * (double)sqrtD[i]);
        bh[i] = (float)(b[i] / (double)sqrtD[i]);
    }
}

// factor of A from the network's output: L_cp = sqrt(a_cc) L^_cp, L_ii = sqrt(a_ii) L^_ii
__global__ void factor_from_net_kernel(int n, int m, const int* __restrict__ c, const float* __restrict__ sqrtD,
                                       const float* __restrict__ lower, const float* __restrict__ diag,
                                       double* lVal, double* dOut) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)m + n;
         t += (int64_t)gridDim.x * blockDim.x) {
        if (t < m) {
            lVal[t] = (double)sqrtD[c[t]] * (double)lower[t];
        } else {
            const int64_t i = t - m;
            dOut[i] = (double)sqrtD[i] * (double)fmaxf(diag[i], 1e-6f);
        }
    }
}

std::unique_ptr<LSystem> build_system(nsf_device* h, int slot, const double* x, const double* b) {
    Factor& F = factor_for(h, slot, false);
    const Csr& A = h->mats[slot];
    cudaStream_t s = h->stream;
    auto S = std::make_unique<LSystem>();
    S->n = F.rows;
    S->m = (int)F.nnzL;
    S->colours = F.colours;
    S->slot = slot;
    const int n = S->n, m = S->m;
    std::vector<int> lrp((size_t)n + 1), lci((size_t)std::max(m, 1));
    NSF_CUDA(cudaMemcpyAsync(lrp.data(), F.lRowptr.get(), sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
    if (m) NSF_CUDA(cudaMemcpyAsync(lci.data(), F.lCol.get(), sizeof(int) * m, cudaMemcpyDeviceToHost, s));
    NSF_CUDA(cudaStreamSynchronize(s));
    // edges incident to each node as the parent, in ascending edge order
    std::vector<int> uprp((size_t)n + 1, 0), upEdge((size_t)std::max(m, 1));
    for (int k = 0; k < m; ++k) ++uprp[(size_t)lci[k] + 1];
    for (int i = 0; i < n; ++i) uprp[i + 1] += uprp[i];
    std::vector<int> fill(uprp.begin(), uprp.end() - 1);
    for (int k = 0; k < m; ++k) upEdge[fill[lci[k]]++] = k;
    S->lrp.upload(lrp.data(), lrp.size(), s);
    S->p.upload(lci.data(), lci.size(), s);
    S->uprp.upload(uprp.data(), uprp.size(), s);
    S->upEdge.upload(upEdge.data(), upEdge.size(), s);
    S->c.alloc((size_t)std::max(m, 1));
    S->fn.alloc((size_t)4 * n);
    S->fe.alloc((size_t)4 * std::max(m, 1));
    S->sqrtD.alloc((size_t)n);
    node_features_kernel<<<grid_for(n, 128), 128, 0, s>>>(n, A.rowptr.get(), A.col.get(), A.val.get(),
                                                          F.aIndexDiag.get(), S->fn.get(), S->sqrtD.get());
    edge_features_kernel<<<grid_for(n, 128), 128, 0, s>>>(n, F.lRowptr.get(), F.lCol.get(), F.aIndexL.get(),
                                                          F.aIndexDiag.get(), A.val.get(), F.colourOf.get(),
                                                          F.colours, S->c.get(), S->fe.get());
    NSF_CUDA(cudaGetLastError());
    count_launch();
    count_launch();
    if (x && b) {
        DevBuf<double> xd, bd;
        xd.upload(x, (size_t)n, s);
        bd.upload(b, (size_t)n, s);
        S->xh.alloc((size_t)n);
        S->bh.alloc((size_t)n);
        scale_pair_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, xd.get(), bd.get(), S->sqrtD.get(), S->xh.get(),
                                                           S->bh.get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
        NSF_CUDA(cudaStreamSynchronize(s));   // xd / bd are released on return
    }
    NSF_CUDA(cudaStreamSynchronize(s));
    return S;
}

// deterministic initial parameters (He-style; residual branches x0.1; decoder at L^ = I)
std::vector<float> init_params(const NetLayout& N, uint64_t seed) {
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    auto next = [&]() {   // splitmix64
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    auto normal = [&]() {   // Box-Muller
        const double u1 = ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        const double u2 = ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    };
    std::vector<float> th(N.count, 0.0f);
    auto fillW = [&](const PT& p, double gain) {
        const double sd = gain * std::sqrt(2.0 / p.rows);
        for (size_t i = 0; i < p.size(); ++i) th[p.off + i] = (float)(sd * normal());
    };
    fillW(N.Wn0, 1.0);
    fillW(N.We0, 1.0);
    for (const auto& l : N.L) {
        fillW(l.W1e, 1.0);
        fillW(l.W2e, 0.1);
        fillW(l.W1n, 1.0);
        fillW(l.W2n, 0.1);
    }
    th[N.bdn.off] = (float)std::log(std::exp(1.0) - 1.0);   // softplus -> 1
    return th;
}

}  // namespace
}  // namespace nsf

using namespace nsf;

#define LEARN_BEGIN(L)                                      \
    if (!(L) || !(L)->h) return NSF_ERR_BAD_ARG;            \
    std::lock_guard<std::recursive_mutex> lk_((L)->h->mu);  \
    try {                                                   \
        NSF_CUDA(cudaSetDevice((L)->h->device));

#define LEARN_END(L)                                        \
    }                                                       \
    catch (const nsf::Error& e) {                           \
        (L)->lastError = e.msg;                             \
        return e.status;                                    \
    }                                                       \
    catch (const std::exception& e) {                       \
        (L)->lastError = e.what();                          \
        return NSF_ERR_CUDA;                                \
    }                                                       \
    return NSF_OK;

static void learner_check_error(nsf_learner* L) {
    int e = 0;
    NSF_CUDA(cudaMemcpyAsync(&e, L->err.get(), sizeof(int), cudaMemcpyDeviceToHost, L->h->stream));
    NSF_CUDA(cudaStreamSynchronize(L->h->stream));
    if (e) throw Error{NSF_ERR_BARRIER_TIMEOUT, "a tensor-core layer timed out waiting for its MMAs"};
}

extern "C" {

int nsf_learn_create(nsf_device* h, uint64_t seed, nsf_learner** out) {
    if (!h || !out) return NSF_ERR_BAD_ARG;
    *out = nullptr;
    auto L = std::make_unique<nsf_learner>();
    L->h = h;
    LEARN_BEGIN(L.get())
    const NetLayout& N = L->net;
    const std::vector<float> th = init_params(N, seed);
    L->theta.upload(th.data(), th.size(), h->stream);
    L->am.alloc(N.count);
    L->av.alloc(N.count);
    L->grad.alloc(N.count);
    L->am.zero(h->stream);
    L->av.zero(h->stream);
    size_t off = 0;
    for (int l = 0; l < kLayers; ++l) {
        Learner tmp(L.get());
        for (int w = 0; w < 4; ++w) {
            const size_t sz = tmp.weights(l, w)->size();
            L->wbOff[l][w][0] = off;
            L->wbOff[l][w][1] = off + sz;
            off += 2 * sz;
        }
    }
    L->wb.alloc(off);
    L->err.alloc(1);
    L->err.zero(h->stream);
    L->dots.alloc(256);
    Learner(L.get()).refresh_bf16();
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    *out = L.release();
    return NSF_OK;
    LEARN_END(L.get())
}

void nsf_learn_destroy(nsf_learner* L) {
    if (!L) return;
    {
        std::lock_guard<std::recursive_mutex> lk(L->h->mu);
        cudaSetDevice(L->h->device);
        cudaStreamSynchronize(L->h->stream);
        L->systems.clear();
        L->tape = LTape();
    }
    delete L;
}

const char* nsf_learn_last_error(const nsf_learner* L) { return L ? L->lastError.c_str() : "null learner"; }

int nsf_learn_param_count(nsf_learner* L, int64_t* count) {
    LEARN_BEGIN(L)
    if (count) *count = (int64_t)L->net.count;
    LEARN_END(L)
}

int nsf_learn_get_params(nsf_learner* L, float* theta) {
    LEARN_BEGIN(L)
    if (!theta) throw bad_arg("null array");
    NSF_CUDA(cudaMemcpyAsync(theta, L->theta.get(), sizeof(float) * L->net.count, cudaMemcpyDeviceToHost, L->h->stream));
    NSF_CUDA(cudaStreamSynchronize(L->h->stream));
    LEARN_END(L)
}

int nsf_learn_set_params(nsf_learner* L, const float* theta) {
    LEARN_BEGIN(L)
    if (!theta) throw bad_arg("null array");
    for (size_t i = 0; i < L->net.count; ++i)
        if (!std::isfinite(theta[i])) throw bad_arg("parameters must be finite");
    NSF_CUDA(cudaMemcpyAsync(L->theta.get(), theta, sizeof(float) * L->net.count, cudaMemcpyHostToDevice, L->h->stream));
    L->am.zero(L->h->stream);
    L->av.zero(L->h->stream);
    L->step = 0;
    Learner(L).refresh_bf16();
    NSF_CUDA(cudaStreamSynchronize(L->h->stream));
    LEARN_END(L)
}

int nsf_learn_add_system(nsf_learner* L, int slot, const double* x, const double* b, int* index) {
    LEARN_BEGIN(L)
    if (!x || !b) throw bad_arg("null vector");
    L->systems.push_back(build_system(L->h, slot, x, b));
    if (index) *index = (int)L->systems.size() - 1;
    LEARN_END(L)
}

int nsf_learn_clear_systems(nsf_learner* L) {
    LEARN_BEGIN(L)
    L->systems.clear();
    LEARN_END(L)
}

int nsf_learn_system_size(nsf_learner* L, int index, int* nodes, int64_t* edges) {
    LEARN_BEGIN(L)
    if (index < 0 || index >= (int)L->systems.size()) throw bad_arg("system index out of range");
    if (nodes) *nodes = L->systems[index]->n;
    if (edges) *edges = L->systems[index]->m;
    LEARN_END(L)
}

// Network output on a stored system: L^ off-diagonal values (edge order = the factor pattern) and diagonal.
int nsf_learn_forward(nsf_learner* L, int index, float* lower, float* diag) {
    LEARN_BEGIN(L)
    if (index < 0 || index >= (int)L->systems.size()) throw bad_arg("system index out of range");
    const LSystem& S = *L->systems[index];
    Learner(L).forward(S);
    learner_check_error(L);
    if (lower && S.m)
        NSF_CUDA(cudaMemcpyAsync(lower, L->tape.lower.get(), sizeof(float) * S.m, cudaMemcpyDeviceToHost, L->h->stream));
    if (diag) NSF_CUDA(cudaMemcpyAsync(diag, L->tape.diag.get(), sizeof(float) * S.n, cudaMemcpyDeviceToHost, L->h->stream));
    NSF_CUDA(cudaStreamSynchronize(L->h->stream));
    LEARN_END(L)
}

int nsf_learn_loss_grad(nsf_learner* L, int index, double* loss, float* grad) {
    LEARN_BEGIN(L)
    if (index < 0 || index >= (int)L->systems.size()) throw bad_arg("system index out of range");
    const LSystem& S = *L->systems[index];
    if (!S.xh.get()) throw bad_arg("system has no training pair");
    Learner G(L);
    L->grad.zero(L->h->stream);
    G.forward(S);
    const double v = G.loss_backward(S, 1.0f);
    learner_check_error(L);
    if (loss) *loss = v;
    if (grad)
        NSF_CUDA(cudaMemcpyAsync(grad, L->grad.get(), sizeof(float) * L->net.count, cudaMemcpyDeviceToHost, L->h->stream));
    NSF_CUDA(cudaStreamSynchronize(L->h->stream));
    LEARN_END(L)
}

// Adam over `steps` steps; each step averages the gradient of `batch` systems drawn (seeded) from the store.
int nsf_learn_train(nsf_learner* L, int steps, int batch, double lr, uint64_t seed, float* losses) {
    LEARN_BEGIN(L)
    if (L->systems.empty()) throw Error{NSF_ERR_STATE, "no training systems"};
    if (steps < 0 || batch < 1 || !(lr > 0)) throw bad_arg("steps >= 0, batch >= 1, lr > 0");
    Learner G(L);
    uint64_t st = seed ^ 0xD1B54A32D192ED03ull;
    auto pick = [&]() {
        st ^= st << 13;
        st ^= st >> 7;
        st ^= st << 17;
        return (int)(st % L->systems.size());
    };
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int k = 0; k < steps; ++k) {
        L->grad.zero(L->h->stream);
        double sum = 0.0;
        for (int j = 0; j < batch; ++j) {
            const LSystem& S = *L->systems[pick()];
            G.forward(S);
            sum += G.loss_backward(S, 1.0f / batch);
        }
        ++L->step;
        const float c1 = 1.0f - std::pow(b1, (float)L->step), c2 = 1.0f - std::pow(b2, (float)L->step);
        adam_kernel<<<grid_for((int64_t)L->net.count, 256), 256, 0, L->h->stream>>>(
            L->net.count, L->theta.get(), L->grad.get(), L->am.get(), L->av.get(), (float)lr, b1, b2, eps, c1, c2);
        NSF_CUDA(cudaGetLastError());
        count_launch();
        G.refresh_bf16();
        if (losses) losses[k] = (float)(sum / batch);
    }
    learner_check_error(L);
    LEARN_END(L)
}

// Runs the network on the slot's current matrix (of `target`, or of the learner's own handle when null) and
// installs L as that slot's preconditioner (kind LEARNED).  Both handles must live on the same GPU.
int nsf_learn_apply(nsf_learner* L, nsf_device* target, int slot) {
    LEARN_BEGIN(L)
    nsf_device* T = target ? target : L->h;
    if (T->device != L->h->device) throw bad_arg("the target handle is on another GPU");
    std::lock_guard<std::recursive_mutex> lkT(T->mu);
    std::unique_ptr<LSystem> S = build_system(T, slot, nullptr, nullptr);   // synchronises T's stream
    Learner(L).forward(*S);
    Factor& F = factor_for(T, slot, false);
    factor_from_net_kernel<<<grid_for((int64_t)S->m + S->n, 256), 256, 0, L->h->stream>>>(
        S->n, S->m, S->c.get(), S->sqrtD.get(), L->tape.lower.get(), L->tape.diag.get(), F.lVal.get(), F.diag.get());
    NSF_CUDA(cudaGetLastError());
    count_launch();
    learner_check_error(L);
    factor_fill(F, L->h->stream);
    NSF_CUDA(cudaStreamSynchronize(L->h->stream));
    F.kind = NSF_PRECOND_LEARNED;
    F.shift = 0.0;
    T->pcgOff[slot] = false;
    LEARN_END(L)
}

}  // extern "C"
