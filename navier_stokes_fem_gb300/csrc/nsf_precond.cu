// Preconditioner factors for the PCG kernels (nsf_pcg_device.cuh): multicolour structure, incomplete Cholesky,
// and installation of externally computed (learned) factor values.
//
// The reference enables an incomplete-Cholesky preconditioner for its CPU CG under USE_PRECONDITIONING
// (include/assembly.h:33-35, 1338-1344; SMM::IC0Preconditioner from the sparse_matrix_math submodule).  On the GPU
// a triangular solve in natural order is a long chain of dependent rows, so the factor is taken in multicolour
// order instead: the matrix graph is coloured (DSatur), and L_ij (i != j) lives on the matrix pattern where
// colour(j) < colour(i).
// Every colour of a sweep is then one parallel phase.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <queue>
#include <tuple>
#include <vector>
#include <thread>
#include <atomic>

#include "nsf_internal.cuh"

namespace nsf {

namespace {

int grid_for(int64_t work, int threads) {
    const int64_t g = (work + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 32));
}

// SELL-32 layout of a CSR whose row count is a multiple of 32 (rows 32 s .. 32 s + 31 form slice s); entries of
// row 32 s + lane at start[s] + 32 k + lane, padded with column -1.  `from` is carried along per entry.
struct HostSell {
    std::vector<int> start, col, from;
    int maxWidth = 0;
};

HostSell build_sell(int rows, const std::vector<int>& rowptr, const std::vector<int>& col,
                    const std::vector<int>& from) {
    const int nSlices = rows / 32;
    HostSell S;
    S.start.assign((size_t)nSlices + 1, 0);
    int64_t total = 0;
    for (int s = 0; s < nSlices; ++s) {
        int w = 0;
        for (int l = 0; l < 32; ++l) w = std::max(w, rowptr[s * 32 + l + 1] - rowptr[s * 32 + l]);
        S.maxWidth = std::max(S.maxWidth, w);
        S.start[s] = (int)total;
        total += (int64_t)w * 32;
        if (total > INT32_MAX) throw Error{NSF_ERR_BAD_ARG, "factor too large for 32-bit offsets"};
    }
    S.start[nSlices] = (int)total;
    S.col.assign((size_t)total, -1);
    S.from.assign((size_t)total, -1);
    for (int s = 0; s < nSlices; ++s)
        for (int l = 0; l < 32; ++l) {
            const int r = s * 32 + l;
            for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) {
                const size_t idx = (size_t)S.start[s] + (size_t)(k - rowptr[r]) * 32 + l;
                S.col[idx] = col[k];
                S.from[idx] = from[k];
            }
        }
    return S;
}

__global__ void ap_values_kernel(int64_t nnz, const int* __restrict__ from, const double* __restrict__ aVal,
                                 double* __restrict__ apVal) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
        const int f = from[k];
        apVal[k] = f >= 0 ? aVal[f] : 1.0;
    }
}

// The diagonal of the permuted matrix (1 on padding rows), and its FP32 inverse.
__global__ void ap_diag_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                               const double* __restrict__ val, double* __restrict__ diag, float* __restrict__ inv) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {   // (grid_for caps)
        double d = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
            if (col[k] == i) d = val[k];
        diag[i] = d;
        inv[i] = d != 0.0 ? (float)(1.0 / d) : 0.0f;
    }
}

// DSatur colouring of the matrix graph (Brelaz 1979): repeatedly colour the uncoloured row whose neighbours
// already use the most distinct colours (ties: more neighbours, then the lower row index) with the smallest colour
// none of them uses.  On the triangulated grids of this solver it finds 3 colours where first-fit in row order
// needs 4, and every colour is one sweep phase.  Deterministic; the oracle restates it with the same tie rule.
int dsatur_colour(int n, const std::vector<int>& rp, const std::vector<int>& ci, const std::vector<double>& av,
                  std::vector<unsigned char>& colour) {
    colour.assign((size_t)n, 255);
    std::vector<unsigned> used((size_t)n, 0);      // colours among coloured neighbours (bit mask)
    std::vector<int> deg((size_t)n, 0);
    for (int i = 0; i < n; ++i)
        for (int k = rp[i]; k < rp[i + 1]; ++k) deg[i] += ci[k] != i && av[k] != 0.0;
    // max-heap of (saturation, degree, -row) with lazy deletion
    using Key = std::tuple<int, int, int>;
    std::priority_queue<Key> heap;
    for (int i = 0; i < n; ++i) heap.push(Key{0, deg[i], -i});
    int colours = 0;
    while (!heap.empty()) {
        const Key top = heap.top();
        heap.pop();
        const int i = -std::get<2>(top);
        if (colour[i] != 255 || std::get<0>(top) != __builtin_popcount(used[i])) continue;
        int c = 0;
        while (c < 32 && (used[i] >> c & 1u)) ++c;
        if (c >= kMaxColours) throw Error{NSF_ERR_BAD_ARG, "matrix graph needs more than 16 colours"};
        colour[i] = (unsigned char)c;
        colours = std::max(colours, c + 1);
        for (int k = rp[i]; k < rp[i + 1]; ++k) {
            const int j = ci[k];
            if (j == i || av[k] == 0.0 || colour[j] != 255 || (used[j] >> c & 1u)) continue;
            used[j] |= 1u << c;
            heap.push(Key{__builtin_popcount(used[j]), deg[j], -j});
        }
    }
    return colours;
}

}  // namespace

// Colouring, the canonical pattern of L, the colour-permuted system and the sweep layouts for the matrix A.
void factor_structure(Factor& F, const Csr& A, cudaStream_t s) {
    if (!A.valid() || A.rows != A.cols) throw bad_arg("preconditioner needs a square matrix");
    const int n = A.rows;
    std::vector<int> rp((size_t)n + 1), ci((size_t)A.nnz);
    std::vector<double> av((size_t)A.nnz);
    NSF_CUDA(cudaMemcpyAsync(rp.data(), A.rowptr.get(), sizeof(int) * rp.size(), cudaMemcpyDeviceToHost, s));
    if (A.nnz) {
        NSF_CUDA(cudaMemcpyAsync(ci.data(), A.col.get(), sizeof(int) * ci.size(), cudaMemcpyDeviceToHost, s));
        NSF_CUDA(cudaMemcpyAsync(av.data(), A.val.get(), sizeof(double) * av.size(), cudaMemcpyDeviceToHost, s));
    }
    NSF_CUDA(cudaStreamSynchronize(s));

    // colouring of the graph of the non-zero entries (DSatur, see dsatur_colour); exact zeros of the assembled
    // pattern couple nothing, so neighbours through them may share a colour and carry no factor entry
    std::vector<unsigned char> colour;
    const int colours = dsatur_colour(n, rp, ci, av, colour);

    // canonical strictly-lower pattern: neighbours of a smaller colour, ordered by (colour, column)
    std::vector<int> lrp((size_t)n + 1, 0), lci, aIdx, aDiag((size_t)n, -1);
    lci.reserve((size_t)A.nnz / 2 + 1);
    aIdx.reserve((size_t)A.nnz / 2 + 1);
    std::vector<std::pair<int, int>> row;
    for (int i = 0; i < n; ++i) {
        row.clear();
        for (int k = rp[i]; k < rp[i + 1]; ++k) {
            const int j = ci[k];
            if (j == i) aDiag[i] = k;
            else if (av[k] != 0.0 && colour[j] < colour[i]) row.push_back({j, k});
        }
        if (aDiag[i] < 0) throw Error{NSF_ERR_BAD_ARG, "row " + std::to_string(i) + " has no diagonal entry"};
        std::sort(row.begin(), row.end(), [&](const std::pair<int, int>& a, const std::pair<int, int>& b) {
            return colour[a.first] != colour[b.first] ? colour[a.first] < colour[b.first] : a.first < b.first;
        });
        for (auto& e : row) {
            lci.push_back(e.first);
            aIdx.push_back(e.second);
        }
        lrp[i + 1] = (int)lci.size();
    }
    const int64_t nnzL = (int64_t)lci.size();

    // permuted order: colour blocks, rows ascending inside a block, each block padded to whole slices
    std::vector<int> perm, iperm((size_t)n);
    F.colourRow[0] = 0;
    for (int c = 0; c < colours; ++c) {
        for (int i = 0; i < n; ++i)
            if (colour[i] == c) {
                iperm[i] = (int)perm.size();
                perm.push_back(i);
            }
        while (perm.size() % 32) perm.push_back(-1);
        F.colourRow[c + 1] = (int)perm.size();
    }
    const int np = (int)perm.size();

    // P A P^T: row i' = perm[i'], columns renumbered and sorted; padding rows are identity rows
    std::vector<int> aprp((size_t)np + 1, 0), apci, apfrom;
    apci.reserve((size_t)A.nnz + (size_t)(np - n));
    apfrom.reserve(apci.capacity());
    for (int r = 0; r < np; ++r) {
        const int o = perm[r];
        if (o < 0) {
            apci.push_back(r);
            apfrom.push_back(-1);
        } else {
            row.clear();
            for (int k = rp[o]; k < rp[o + 1]; ++k) row.push_back({iperm[ci[k]], k});
            std::sort(row.begin(), row.end());
            for (auto& e : row) {
                apci.push_back(e.first);
                apfrom.push_back(e.second);
            }
        }
        aprp[r + 1] = (int)apci.size();
    }
    // L and L^T in permuted rows and columns; values come from the canonical array (index carried in `from`)
    std::vector<int> lprp((size_t)np + 1, 0), lpci, lpfrom;
    lpci.reserve((size_t)nnzL);
    lpfrom.reserve((size_t)nnzL);
    for (int r = 0; r < np; ++r) {
        const int o = perm[r];
        if (o >= 0)
            for (int k = lrp[o]; k < lrp[o + 1]; ++k) {   // (colour, column) order == ascending permuted column
                lpci.push_back(iperm[lci[k]]);
                lpfrom.push_back(k);
            }
        lprp[r + 1] = (int)lpci.size();
    }
    std::vector<int> uprp((size_t)np + 1, 0);
    for (int64_t k = 0; k < nnzL; ++k) ++uprp[(size_t)lpci[k] + 1];
    for (int r = 0; r < np; ++r) uprp[r + 1] += uprp[r];
    std::vector<int> upci((size_t)nnzL), upfrom((size_t)nnzL), fill(uprp.begin(), uprp.end() - 1);
    for (int r = 0; r < np; ++r)   // rows ascending: each upper row comes out sorted by (permuted) column
        for (int k = lprp[r]; k < lprp[r + 1]; ++k) {
            const int j = lpci[k];
            upci[fill[j]] = r;
            upfrom[fill[j]] = lpfrom[k];
            ++fill[j];
        }
    HostSell lo = build_sell(np, lprp, lpci, lpfrom);
    HostSell up = build_sell(np, uprp, upci, upfrom);

    F.rows = n;
    F.colours = colours;
    F.nPerm = np;
    F.nnzL = nnzL;
    F.colourOf.upload(colour.data(), colour.size(), s);
    F.lRowptr.upload(lrp.data(), lrp.size(), s);
    F.lCol.upload(lci.data(), lci.size(), s);
    F.aIndexL.upload(aIdx.data(), aIdx.size(), s);
    F.aIndexDiag.upload(aDiag.data(), aDiag.size(), s);
    F.perm.upload(perm.data(), perm.size(), s);
    F.loMaxW = lo.maxWidth;
    F.upMaxW = up.maxWidth;
    F.loStart.upload(lo.start.data(), lo.start.size(), s);
    F.loCol.upload(lo.col.data(), lo.col.size(), s);
    F.loFrom.upload(lo.from.data(), lo.from.size(), s);
    F.upStart.upload(up.start.data(), up.start.size(), s);
    F.upCol.upload(up.col.data(), up.col.size(), s);
    F.upFrom.upload(up.from.data(), up.from.size(), s);
    // 16-bit column copies for the inner iterations (both parts or neither)
    F.col16 = sell_col16(np / 32, F.loStart.get(), F.loCol.get(), false, F.loColBase, F.loCol16, s) &&
              sell_col16(np / 32, F.upStart.get(), F.upCol.get(), false, F.upColBase, F.upCol16, s);
    if (!F.col16) {
        F.loColBase.release();
        F.loCol16.release();
        F.upColBase.release();
        F.upCol16.release();
    }
    F.lVal.alloc(std::max<int64_t>(nnzL, 1));
    F.diag.alloc((size_t)n);
    F.loVal.alloc(std::max<size_t>(lo.col.size(), 1));
    F.loVal32.alloc(std::max<size_t>(lo.col.size(), 1));
    F.upVal.alloc(std::max<size_t>(up.col.size(), 1));
    F.upVal32.alloc(std::max<size_t>(up.col.size(), 1));
    F.loVal16.alloc(std::max<size_t>(lo.col.size(), 1));
    F.upVal16.alloc(std::max<size_t>(up.col.size(), 1));
    F.range16.alloc(1);
    F.dinv.alloc((size_t)np);
    F.dinv32.alloc((size_t)np);
    // the permuted matrix, its values gathered from A, and its SELL copies (FP64 and FP32)
    Csr& P = F.Ap;
    P.rows = P.cols = np;
    P.nnz = (int64_t)apci.size();
    P.rowptr.upload(aprp.data(), aprp.size(), s);
    P.col.upload(apci.data(), apci.size(), s);
    F.apFrom.upload(apfrom.data(), apfrom.size(), s);
    P.val.alloc((size_t)P.nnz);
    P.values_changed();
    ap_values_kernel<<<grid_for(P.nnz, 256), 256, 0, s>>>(P.nnz, F.apFrom.get(), A.val.get(), P.val.get());
    NSF_CUDA(cudaGetLastError());
    F.aDiag.alloc((size_t)np);
    F.aInv32.alloc((size_t)np);
    ap_diag_kernel<<<grid_for(np, 256), 256, 0, s>>>(np, P.rowptr.get(), P.col.get(), P.val.get(), F.aDiag.get(),
                                                     F.aInv32.get());
    NSF_CUDA(cudaGetLastError());
    count_launch();
    prepare_matrix(P, true, s);
    NSF_CUDA(cudaStreamSynchronize(s));
    F.ready = false;
    F.kind = NSF_PRECOND_NONE;
}

// ---------------------------------------------------------------------------------------------------
// incomplete Cholesky on the multicolour pattern, one colour per launch (rows of a colour are independent):
//   L_ij = (a_ij - sum_{m in L(i) and L(j)} L_im L_jm) / L_jj  in the (colour, column) order of row i,
//   L_ii = sqrt(a_ii (1 + shift) - sum_j L_ij^2)
// ---------------------------------------------------------------------------------------------------
__global__ void ic0_colour_kernel(int r0, int r1, const int* __restrict__ perm, const int* __restrict__ lRowptr,
                                  const int* __restrict__ lCol, const int* __restrict__ aIndexL,
                                  const int* __restrict__ aIndexDiag, const double* __restrict__ aVal, double shift,
                                  double* lVal, double* diag, int* fail) {
    for (int idx = r0 + blockIdx.x * blockDim.x + threadIdx.x; idx < r1; idx += gridDim.x * blockDim.x) {
        const int i = perm[idx];
        if (i < 0) continue;
        const int b = lRowptr[i], e = lRowptr[i + 1];
        double sq = 0.0;
        for (int k = b; k < e; ++k) {
            const int j = lCol[k];
            double s = aVal[aIndexL[k]];
            const int jb = lRowptr[j], je = lRowptr[j + 1];
            for (int k2 = b; k2 < k; ++k2) {
                const int m = lCol[k2];
                for (int kj = jb; kj < je; ++kj)
                    if (lCol[kj] == m) {
                        s -= lVal[k2] * lVal[kj];
                        break;
                    }
            }
            const double l = s / diag[j];
            lVal[k] = l;
            sq += l * l;
        }
        const double aii = aVal[aIndexDiag[i]];
        double d = aii * (1.0 + shift) - sq;
        if (!(d > 1e-12 * fabs(aii))) {   // breakdown: flag it (the host retries with a larger shift)
            atomicExch(fail, 1);
            d = fabs(aii) > 0 ? fabs(aii) : 1.0;
        }
        diag[i] = sqrt(d);
    }
}

// A value's FP16 copy, and whether it is outside FP16's normal range (a non-zero magnitude below 2^-14, where
// subnormals lose precision, or above 65504).
__device__ __forceinline__ __half to_half_checked(double v, int* range16) {
    const double m = fabs(v);
    if (m != 0.0 && (m < 6.103515625e-05 || m > 65504.0)) atomicExch(range16, 1);
    return __double2half(v);
}

// FP32 copy of a value: the FP16 value widened when the factor keeps FP16 copies (every consumer of the FP32 values,
// the refresh kernel's sweeps included, then applies the same M as the FP16 inner iterations), else the value
// rounded once.
__global__ void factor_fill_kernel(int64_t nLo, int64_t nUp, int n, const int* __restrict__ perm,
                                   const int* __restrict__ loFrom, const int* __restrict__ upFrom,
                                   const double* __restrict__ lVal,
                                   const double* __restrict__ diag, double* loVal, float* loVal32, double* upVal,
                                   float* upVal32, double* dinv, float* dinv32, __half* loVal16, __half* upVal16,
                                   int* range16, int pass) {
    const int64_t total = nLo + nUp + n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < nLo) {
            const int f = loFrom[i];
            const double v = f >= 0 ? lVal[f] : 0.0;
            if (pass == 0) {
                loVal[i] = v;
                loVal16[i] = to_half_checked(v, range16);
            } else {
                loVal32[i] = pass == 2 ? __half2float(loVal16[i]) : (float)v;
            }
        } else if (i < nLo + nUp) {
            const int64_t k = i - nLo;
            const int f = upFrom[k];
            const double v = f >= 0 ? lVal[f] : 0.0;
            if (pass == 0) {
                upVal[k] = v;
                upVal16[k] = to_half_checked(v, range16);
            } else {
                upVal32[k] = pass == 2 ? __half2float(upVal16[k]) : (float)v;
            }
        } else if (pass == 0) {
            const int64_t r = i - nLo - nUp;
            const int o = perm[r];
            const double d = o >= 0 ? 1.0 / diag[o] : 1.0;
            dinv[r] = d;
            dinv32[r] = (float)d;
        }
    }
}

// Copies the canonical factor values into the sweep layouts (FP64 and FP32) and 1 / L_ii.
// With FP16 copies when every value fits FP16's normal range (pass 0 writes FP64, FP16 and 1 / L_ii and checks
// the range; pass 1 or 2 then writes the FP32 copies from the FP64 or the FP16 values).
void factor_fill(Factor& F, cudaStream_t s) {
    const int64_t nLo = (int64_t)F.loCol.n, nUp = (int64_t)F.upCol.n;
    F.range16.zero(s);
    auto launch = [&](int pass) {
        factor_fill_kernel<<<grid_for(nLo + nUp + F.nPerm, 256), 256, 0, s>>>(
            nLo, nUp, F.nPerm, F.perm.get(), F.loFrom.get(), F.upFrom.get(), F.lVal.get(), F.diag.get(),
            F.loVal.get(), F.loVal32.get(), F.upVal.get(), F.upVal32.get(), F.dinv.get(), F.dinv32.get(),
            F.loVal16.get(), F.upVal16.get(), F.range16.get(), pass);
        NSF_CUDA(cudaGetLastError());
        count_launch();
    };
    launch(0);
    int outOfRange = 0;
    NSF_CUDA(cudaMemcpyAsync(&outOfRange, F.range16.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
    NSF_CUDA(cudaStreamSynchronize(s));
    F.has16 = outOfRange == 0;
    launch(F.has16 ? 2 : 1);
    F.ready = true;
}

// IC(0) of A on F's pattern; retries with a growing diagonal shift on breakdown.  Returns the shift used.
double factor_ic0(Factor& F, const Csr& A, cudaStream_t s) {
    DevBuf<int> fail;
    fail.alloc(1);
    double shift = 0.0;
    for (int attempt = 0; attempt < 8; ++attempt) {
        fail.zero(s);
        for (int c = 0; c < F.colours; ++c) {
            const int r0 = F.colourRow[c], r1 = F.colourRow[c + 1];
            ic0_colour_kernel<<<grid_for(r1 - r0, 128), 128, 0, s>>>(
                r0, r1, F.perm.get(), F.lRowptr.get(), F.lCol.get(), F.aIndexL.get(), F.aIndexDiag.get(),
                A.val.get(), shift, F.lVal.get(), F.diag.get(), fail.get());
            NSF_CUDA(cudaGetLastError());
            count_launch();
        }
        int failed = 0;
        NSF_CUDA(cudaMemcpyAsync(&failed, fail.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
        NSF_CUDA(cudaStreamSynchronize(s));
        if (!failed) {
            factor_fill(F, s);
            F.kind = NSF_PRECOND_IC0;
            F.shift = shift;
            return shift;
        }
        shift = shift == 0.0 ? 1e-3 : shift * 10.0;
    }
    throw Error{NSF_ERR_BREAKDOWN, "incomplete Cholesky broke down even with a diagonal shift of 1e4"};
}

// S = A_11 - A_10 A_00^-1 A_01 over the colour-1 rows of the permuted matrix, in FP64 on the host (rows in parallel):
// row i holds a_ii, its colour-1 entries, and -a_ij a_jk / a_jj for every colour-0 neighbour j and colour-1
// neighbour k of j, columns ascending.  Colour-0 rows are left empty.
bool factor_schur(Factor& F, cudaStream_t s) {
    if (F.schurTried) return F.hasSchur;
    F.schurTried = true;
    if (F.colours != 2) return false;
    const Csr& A = F.Ap;
    const int n = A.rows, c1 = F.colourRow[1], c2 = F.colourRow[2];
    std::vector<int> rp((size_t)n + 1), ci((size_t)A.nnz);
    std::vector<double> av((size_t)A.nnz);
    NSF_CUDA(cudaMemcpyAsync(rp.data(), A.rowptr.get(), sizeof(int) * rp.size(), cudaMemcpyDeviceToHost, s));
    NSF_CUDA(cudaMemcpyAsync(ci.data(), A.col.get(), sizeof(int) * ci.size(), cudaMemcpyDeviceToHost, s));
    NSF_CUDA(cudaMemcpyAsync(av.data(), A.val.get(), sizeof(double) * av.size(), cudaMemcpyDeviceToHost, s));
    NSF_CUDA(cudaStreamSynchronize(s));
    std::vector<double> diag((size_t)c1, 0.0);
    for (int j = 0; j < c1; ++j)
        for (int k = rp[j]; k < rp[j + 1]; ++k)
            if (ci[k] == j) diag[j] = av[k];
    const int rows = c2 - c1;
    std::vector<std::vector<std::pair<int, double>>> srow((size_t)rows);
    const int threads = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    std::atomic<int> bad{0};
    for (int w = 0; w < threads; ++w)
        pool.emplace_back([&, w] {
            std::vector<std::pair<int, double>> acc;
            for (int r = w; r < rows; r += threads) {
                const int i = c1 + r;
                acc.clear();
                auto add = [&](int c, double v) {
                    for (auto& e : acc)
                        if (e.first == c) { e.second += v; return; }
                    acc.push_back({c, v});
                };
                for (int q = rp[i]; q < rp[i + 1]; ++q) {
                    const int j = ci[q];
                    if (j >= c1) { add(j, av[q]); continue; }
                    if (diag[j] == 0.0) { bad = 1; continue; }
                    const double f = av[q] / diag[j];
                    for (int t = rp[j]; t < rp[j + 1]; ++t)
                        if (ci[t] >= c1) add(ci[t], -f * av[t]);
                }
                std::sort(acc.begin(), acc.end());
                srow[r] = acc;
            }
        });
    for (auto& t : pool) t.join();
    if (bad) return false;
    std::vector<int> sp((size_t)n + 1, 0), sc;
    std::vector<double> sv;
    for (int r = 0; r < rows; ++r) sp[(size_t)c1 + r + 1] = (int)srow[r].size();
    for (int i = 0; i < n; ++i) sp[i + 1] += sp[i];
    sc.reserve((size_t)sp[n]);
    sv.reserve((size_t)sp[n]);
    for (int r = 0; r < rows; ++r)
        for (const auto& e : srow[r]) {
            sc.push_back(e.first);
            sv.push_back(e.second);
        }
    Csr& S = F.S;
    S.rows = S.cols = n;
    S.nnz = (int64_t)sc.size();
    S.rowptr.upload(sp.data(), sp.size(), s);
    S.col.upload(sc.data(), sc.size(), s);
    S.val.upload(sv.data(), sv.size(), s);
    S.values_changed();
    prepare_matrix(S, true, s);
    prepare_col16(S, s);
    NSF_CUDA(cudaStreamSynchronize(s));
    if (!S.hasCol16) {
        F.S = Csr();
        return false;
    }
    F.hasSchur = true;
    return true;
}

FactorView factor_view(const Factor& F, CgWorkspace& ws) {
    FactorView v;
    v.colours = F.colours;
    for (int c = 0; c <= F.colours; ++c) v.colourRow[c] = F.colourRow[c];
    v.nNatural = F.rows;
    v.perm = F.perm.get();
    v.loMaxW = F.loMaxW;
    v.upMaxW = F.upMaxW;
    v.loStart = F.loStart.get();
    v.loCol = F.loCol.get();
    v.loVal = F.loVal.get();
    v.loVal32 = F.loVal32.get();
    v.upStart = F.upStart.get();
    v.upCol = F.upCol.get();
    v.upVal = F.upVal.get();
    v.upVal32 = F.upVal32.get();
    v.loVal16 = F.has16 ? F.loVal16.get() : nullptr;
    v.upVal16 = F.has16 ? F.upVal16.get() : nullptr;
    if (F.col16) {
        v.loCol16 = F.loCol16.get();
        v.loColBase = F.loColBase.get();
        v.upCol16 = F.upCol16.get();
        v.upColBase = F.upColBase.get();
    }
    v.dinv = F.dinv.get();
    v.dinv32 = F.dinv32.get();
    v.aDiag = F.aDiag.get();
    v.aInv32 = F.aInv32.get();
    if (F.hasSchur) {
        v.sMaxW = F.S.maxWidth;
        v.sStart = F.S.sellStart.get();
        v.sCol16 = F.S.sellCol16.get();
        v.sColBase = F.S.sellColBase.get();
        v.sVal32 = F.S.sellVal32.get();
        v.sRowsum32 = F.S.rowsum32.get();
    }
    v.w = ws.w.get();
    v.w32 = ws.w32.get();
    v.xp = ws.xp.get();
    v.bp = ws.bp.get();
    return v;
}

}  // namespace nsf
