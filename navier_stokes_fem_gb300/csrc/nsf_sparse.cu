// Sparse matrix-vector products and small vector kernels of the operator-split step.
//
// Replaces spRMultKernel / spRMultSubKernel (gpu/matrix_math.cu:20-98), which assign one thread per CSR row:
// here four lanes share a row so consecutive lanes read consecutive values/column indices, and the step's
// right-hand-side fix-ups (Dirichlet lift subtraction and value imposition, include/assembly.h:505-523,
// 575-595, 695-707) are fused into the product's epilogue.
#include "nsf_internal.cuh"

namespace nsf {

constexpr int kSpmvThreads = 256;
constexpr int kLanes = 4;

__device__ __forceinline__ double lane_group_sum(double v) {
    const unsigned m = 0xFu << ((threadIdx.x & 31) & ~(kLanes - 1));
    v += __shfl_xor_sync(m, v, 1);
    v += __shfl_xor_sync(m, v, 2);
    return v;
}

// y = A x, or with the right-hand-side epilogue y_i = mask_i ? g_i : (A x)_i - lift_i
__global__ void __launch_bounds__(kSpmvThreads) spmv_kernel(int rows, const int* __restrict__ rowptr,
                                                            const int* __restrict__ col,
                                                            const double* __restrict__ val,
                                                            const double* __restrict__ x,
                                                            const double* __restrict__ lift,
                                                            const unsigned char* __restrict__ mask,
                                                            const double* __restrict__ g, double* __restrict__ y) {
    const int sub = threadIdx.x & (kLanes - 1);
    const int groups = (int)(gridDim.x * blockDim.x) / kLanes;
    for (int row = (int)(blockIdx.x * blockDim.x + threadIdx.x) / kLanes; row < rows; row += groups) {
        double acc = 0;
        const int s = rowptr[row], e = rowptr[row + 1];
        for (int k = s + sub; k < e; k += kLanes) acc = fma(__ldcs(val + k), x[__ldcs(col + k)], acc);
        acc = lane_group_sum(acc);
        if (sub == 0) {
            if (mask && mask[row]) acc = g[row];
            else if (lift) acc -= lift[row];
            y[row] = acc;
        }
    }
}

// y = (y + a), then Dirichlet values imposed: the end of applyPressure (include/assembly.h:686-707)
__global__ void axpy_bc_kernel(int n, const double* __restrict__ a, double* __restrict__ y,
                               const unsigned char* __restrict__ mask, const double* __restrict__ g) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double v = y[i] + a[i];
        if (mask && mask[i]) v = g[i];
        y[i] = v;
    }
}

__global__ void to_fp32_kernel(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

// FP64 row sums, rounded once to FP32: the diagonal term of the difference-form FP32 product
__global__ void rowsum_kernel(int rows, const int* __restrict__ rowptr, const double* __restrict__ val,
                              float* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) s += val[k];
        out[i] = (float)s;
    }
}

static int grid_for(int64_t work, int threads) {
    int64_t g = (work + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 32));
}

void spmv_launch(const Csr& A, const double* x, double* y, cudaStream_t s) {
    spmv_kernel<<<grid_for((int64_t)A.rows * kLanes, kSpmvThreads), kSpmvThreads, 0, s>>>(
        A.rows, A.rowptr.get(), A.col.get(), A.val.get(), x, nullptr, nullptr, nullptr, y);
    NSF_CUDA(cudaGetLastError());
    count_launch();
}

void spmv_rhs_launch(const Csr& A, const double* x, const double* lift, const unsigned char* mask,
                     const double* bcValue, double* y, cudaStream_t s) {
    spmv_kernel<<<grid_for((int64_t)A.rows * kLanes, kSpmvThreads), kSpmvThreads, 0, s>>>(
        A.rows, A.rowptr.get(), A.col.get(), A.val.get(), x, lift, mask, bcValue, y);
    NSF_CUDA(cudaGetLastError());
    count_launch();
}

void axpy_bc_launch(int n, const double* a, double* y, const unsigned char* mask, const double* bcValue,
                    cudaStream_t s) {
    axpy_bc_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, a, y, mask, bcValue);
    NSF_CUDA(cudaGetLastError());
    count_launch();
}

void make_fp32_values(Csr& A, cudaStream_t s) {
    if (A.has32) return;
    A.val32.alloc((size_t)A.nnz);
    to_fp32_kernel<<<grid_for(A.nnz, 256), 256, 0, s>>>(A.nnz, A.val.get(), A.val32.get());
    NSF_CUDA(cudaGetLastError());
    count_launch();
    A.rowsum32.alloc((size_t)A.rows);
    rowsum_kernel<<<grid_for(A.rows, 256), 256, 0, s>>>(A.rows, A.rowptr.get(), A.val.get(), A.rowsum32.get());
    NSF_CUDA(cudaGetLastError());
    count_launch();
    A.has32 = true;
}

}  // namespace nsf
