// Sparse matrix-vector products and small vector kernels of the operator-split step.
//
// Replaces spRMultKernel / spRMultSubKernel (gpu/matrix_math.cu:20-98), which assign one thread per CSR row:
// here four lanes share a row so consecutive lanes read consecutive values/column indices, and the step's
// right-hand-side fix-ups (Dirichlet lift subtraction and value imposition, include/assembly.h:505-523,
// 575-595, 695-707) are fused into the product's epilogue.
#include "nsf_internal.cuh"

#include <climits>

#include <cub/device/device_reduce.cuh>
#include <cub/device/device_scan.cuh>

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

// ---------------------------------------------------------------------------------------------------
// SELL-32 copy of a CSR matrix (the layout the CG kernels stream; see sell_spmv in nsf_device.cuh)
// ---------------------------------------------------------------------------------------------------
// Entries kept in the SELL copies: every non-zero and the diagonal.  Exact zeros of the assembled pattern (the
// diagonal couplings of right-angled P1 triangles, eliminated Dirichlet couplings: about a quarter of a structured
// pressure matrix) contribute +0 to every row sum, so leaving them out changes no product for finite vectors.
__device__ __forceinline__ bool sell_keep(const double* val, const int* col, int k, int row) {
    return val[k] != 0.0 || col[k] == row;
}

__global__ void sell_width_kernel(int rows, int nSlices, const int* __restrict__ rowptr, const int* __restrict__ col,
                                  const double* __restrict__ val, long long* __restrict__ width) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nSlices; s += gridDim.x * blockDim.x) {
        int w = 0;
        for (int l = 0; l < 32; ++l) {
            const int r = s * 32 + l;
            if (r >= rows) continue;
            int c = 0;
            for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) c += sell_keep(val, col, k, r);
            w = max(w, c);
        }
        width[s] = (long long)w * 32;
    }
}

__global__ void narrow_kernel(int n, const long long* __restrict__ in, int* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = (int)in[i];
}

// One thread per (slice, lane): the row's kept entries in CSR order (kept by their FP64 value), then padding
// (value 0, the row's own column, or column 0 for the rows of a tall matrix beyond its column count).
template <typename T>
__global__ void sell_fill_kernel(int rows, int cols, int nSlices, const int* __restrict__ rowptr, const int* __restrict__ col,
                                 const double* __restrict__ keepVal, const T* __restrict__ val,
                                 const int* __restrict__ start, int* __restrict__ scol, T* __restrict__ sval) {
    const long long total = (long long)nSlices * 32;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int r = (int)i, s = r / 32, lane = r % 32;
        const int base = start[s], W = (start[s + 1] - base) / 32;
        const int e = r < rows ? rowptr[r + 1] : 0;
        int q = r < rows ? rowptr[r] : 0;
        const int self = r < rows && r < cols ? r : 0;
        for (int k = 0; k < W; ++k) {
            while (q < e && !sell_keep(keepVal, col, q, r)) ++q;
            const int idx = base + k * 32 + lane;
            const bool in = q < e;
            if (scol) scol[idx] = in ? col[q] : self;
            sval[idx] = in ? val[q] : T(0);
            if (in) ++q;
        }
    }
}

// Entry i of slice sl (lane = i mod 32) is a padding entry of the 16-bit copy: column -1, or (noDiag) the row's
// own column.
__device__ __forceinline__ bool col16_pad(int c, int sl, int lane, bool noDiag) {
    return c < 0 || (noDiag && c == sl * 32 + lane);
}

// One warp per slice: the slice's smallest and largest column (padding entries left out).
__global__ void col16_base_kernel(int nSlices, const int* __restrict__ start, const int* __restrict__ col,
                                  bool noDiag, int* __restrict__ base, int* __restrict__ overflow) {
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (int sl = blockIdx.x * wpb + (threadIdx.x >> 5); sl < nSlices; sl += gridDim.x * wpb) {
        const int b = start[sl], e = start[sl + 1];   // e - b is a multiple of 32: every lane runs the same trips
        int lo = INT_MAX, hi = -1;
        for (int i = b + lane; i < e; i += 32) {
            const int c = col[i];
            if (!col16_pad(c, sl, lane, noDiag)) {
                lo = min(lo, c);
                hi = max(hi, c);
            }
        }
        for (int o = 16; o; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0) {
            base[sl] = hi < 0 ? 0 : lo;
            if (hi >= 0 && hi - lo >= kCol16Pad) atomicOr(overflow, 1);
        }
    }
}

__global__ void col16_fill_kernel(int nSlices, const int* __restrict__ start, const int* __restrict__ col,
                                  bool noDiag, const int* __restrict__ base, unsigned short* __restrict__ col16) {
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (int sl = blockIdx.x * wpb + (threadIdx.x >> 5); sl < nSlices; sl += gridDim.x * wpb) {
        const int b = start[sl], e = start[sl + 1], cb = base[sl];
        for (int i = b + lane; i < e; i += 32) {
            const int c = col[i];
            col16[i] = (unsigned short)(col16_pad(c, sl, lane, noDiag) ? kCol16Pad : c - cb);
        }
    }
}

bool sell_col16(int nSlices, const int* start, const int* col, bool noDiag, DevBuf<int>& base,
                DevBuf<unsigned short>& col16, cudaStream_t s) {
    base.release();
    col16.release();
    if (nSlices <= 0) return false;
    int entries = 0;
    NSF_CUDA(cudaMemcpyAsync(&entries, start + nSlices, sizeof(int), cudaMemcpyDeviceToHost, s));
    DevBuf<int> flag;
    flag.alloc(1);
    flag.zero(s);
    base.alloc((size_t)nSlices);
    const int blocks = grid_for((int64_t)nSlices * 32, 256);
    col16_base_kernel<<<blocks, 256, 0, s>>>(nSlices, start, col, noDiag, base.get(), flag.get());
    NSF_CUDA(cudaGetLastError());
    count_launch();
    int over = 0;
    NSF_CUDA(cudaMemcpyAsync(&over, flag.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
    NSF_CUDA(cudaStreamSynchronize(s));
    if (over || entries <= 0) {
        base.release();
        return false;
    }
    col16.alloc((size_t)entries);
    col16_fill_kernel<<<blocks, 256, 0, s>>>(nSlices, start, col, noDiag, base.get(), col16.get());
    NSF_CUDA(cudaGetLastError());
    count_launch();
    NSF_CUDA(cudaStreamSynchronize(s));
    return true;
}

void prepare_col16(Csr& A, cudaStream_t s) {
    if (!A.hasSell || A.col16Tried) return;
    A.col16Tried = true;
    A.hasCol16 = sell_col16(A.nSlices, A.sellStart.get(), A.sellCol.get(), true, A.sellColBase, A.sellCol16, s);
}

void prepare_matrix(Csr& A, bool fp32, cudaStream_t s) {
    if (fp32) make_fp32_values(A, s);
    if (!A.hasSell) {
        A.col16Tried = A.hasCol16 = false;
        A.sellColBase.release();
        A.sellCol16.release();
        A.nSlices = (A.rows + 31) / 32;
        DevBuf<long long> width, start64;
        width.alloc((size_t)A.nSlices);
        start64.alloc((size_t)A.nSlices + 1);
        sell_width_kernel<<<grid_for(A.nSlices, 256), 256, 0, s>>>(A.rows, A.nSlices, A.rowptr.get(), A.col.get(),
                                                                  A.val.get(), width.get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
        NSF_CUDA(cudaMemsetAsync(start64.get(), 0, sizeof(long long), s));
        size_t tmpBytes = 0;
        NSF_CUDA(cub::DeviceScan::InclusiveSum(nullptr, tmpBytes, width.get(), start64.get() + 1, A.nSlices, s));
        DevBuf<unsigned char> tmp;
        tmp.alloc(tmpBytes);
        NSF_CUDA(cub::DeviceScan::InclusiveSum(tmp.get(), tmpBytes, width.get(), start64.get() + 1, A.nSlices, s));
        DevBuf<long long> widest;
        widest.alloc(1);
        size_t maxBytes = 0;
        NSF_CUDA(cub::DeviceReduce::Max(nullptr, maxBytes, width.get(), widest.get(), A.nSlices, s));
        DevBuf<unsigned char> maxTmp;
        maxTmp.alloc(maxBytes);
        NSF_CUDA(cub::DeviceReduce::Max(maxTmp.get(), maxBytes, width.get(), widest.get(), A.nSlices, s));
        long long total = 0, wmax = 0;
        NSF_CUDA(cudaMemcpyAsync(&total, start64.get() + A.nSlices, sizeof(long long), cudaMemcpyDeviceToHost, s));
        NSF_CUDA(cudaMemcpyAsync(&wmax, widest.get(), sizeof(long long), cudaMemcpyDeviceToHost, s));
        NSF_CUDA(cudaStreamSynchronize(s));
        A.maxWidth = (int)(wmax / 32);
        if (total > INT32_MAX) throw Error{NSF_ERR_BAD_ARG, "padded matrix exceeds 2^31-1 entries"};
        // (total may be below nnz: exact zeros are left out)
        A.sellStart.alloc((size_t)A.nSlices + 1);
        narrow_kernel<<<grid_for(A.nSlices + 1, 256), 256, 0, s>>>(A.nSlices + 1, start64.get(), A.sellStart.get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
        A.sellCol.alloc((size_t)std::max(total, 1LL));
        A.sellVal.alloc((size_t)std::max(total, 1LL));
        sell_fill_kernel<double><<<grid_for((int64_t)A.nSlices * 32, 256), 256, 0, s>>>(
            A.rows, A.cols, A.nSlices, A.rowptr.get(), A.col.get(), A.val.get(), A.val.get(), A.sellStart.get(),
            A.sellCol.get(), A.sellVal.get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
        NSF_CUDA(cudaStreamSynchronize(s));   // width / start64 / tmp are released on return
        A.hasSell = true;
    }
    if (fp32 && !A.hasSell32) {
        A.sellVal32.alloc(A.sellVal.n);
        sell_fill_kernel<float><<<grid_for((int64_t)A.nSlices * 32, 256), 256, 0, s>>>(
            A.rows, A.cols, A.nSlices, A.rowptr.get(), A.col.get(), A.val.get(), A.val32.get(), A.sellStart.get(), nullptr,
            A.sellVal32.get());
        NSF_CUDA(cudaGetLastError());
        count_launch();
        A.hasSell32 = true;
    }
}

}  // namespace nsf
