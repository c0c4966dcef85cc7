// ORACLE — test infrastructure only.  CPU restatement of the preconditioned CG path: the multicolour
// incomplete-Cholesky factor M = L L^T and PCG with it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline use it, as the checker.
//
// The reference enables an incomplete-Cholesky preconditioner for its CPU CG (USE_PRECONDITIONING,
// include/assembly.h:33-35; SMM::IC0Preconditioner constructed at include/assembly.h:1338-1344 and used by
// SMM::ConjugateGradient at :541,618,660,671).  Its algorithm lives in the sparse_matrix_math submodule, which is
// not vendored (no pinned commit); this file restates the published IC(0) algorithm: Cholesky restricted to the
// matrix pattern, L_ij = (a_ij - sum_{m < j} L_im L_jm) / L_jj, L_ii = sqrt(a_ii - sum_{m < i} L_im^2), taken in
// the multicolour order the GPU path uses (rows coloured by DSatur; L_ij lives where colour(j) < colour(i)), and preconditioned CG (Saad, Iterative Methods, Algorithm 9.1) with the relative stopping rule
// ||r|| <= tol ||b||.  The sweeps sum in the same order as the GPU: a row's lower entries by (colour, column),
// its upper entries by (colour, row) of L, and multiply by 1 / L_ii.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <queue>
#include <tuple>
#include <vector>

extern "C" {

// DSatur colouring (Brelaz 1979) of the graph of the non-zero entries, as the GPU path colours: repeatedly colour
// the uncoloured row whose coloured neighbours use the most distinct colours (ties: more neighbours, then the lower
// row index) with the smallest colour none of them uses.  Returns the number of colours (or -1 above 32).
int orc_mc_colour(int n, const int64_t* rp, const int* ci, const double* av, unsigned char* colour) {
    std::vector<int> c((size_t)n, -1), deg((size_t)n, 0);
    std::vector<unsigned> used((size_t)n, 0);
    for (int i = 0; i < n; ++i)
        for (int64_t k = rp[i]; k < rp[i + 1]; ++k) deg[i] += ci[k] != i && av[k] != 0.0;
    std::priority_queue<std::tuple<int, int, int>> heap;
    for (int i = 0; i < n; ++i) heap.push(std::make_tuple(0, deg[i], -i));
    int colours = 0;
    while (!heap.empty()) {
        const auto top = heap.top();
        heap.pop();
        const int i = -std::get<2>(top);
        int sat = 0;
        for (unsigned m = used[i]; m; m &= m - 1) ++sat;
        if (c[i] >= 0 || std::get<0>(top) != sat) continue;
        int k = 0;
        while (k < 32 && (used[i] >> k & 1u)) ++k;
        if (k >= 32) return -1;
        c[i] = k;
        colour[i] = (unsigned char)k;
        colours = std::max(colours, k + 1);
        for (int64_t e = rp[i]; e < rp[i + 1]; ++e) {
            const int j = ci[e];
            if (j == i || av[e] == 0.0 || c[j] >= 0 || (used[j] >> k & 1u)) continue;
            used[j] |= 1u << k;
            int sj = 0;
            for (unsigned m = used[j]; m; m &= m - 1) ++sj;
            heap.push(std::make_tuple(sj, deg[j], -j));
        }
    }
    return colours;
}

// Strictly lower pattern: row i's non-zero neighbours j with colour(j) < colour(i), ordered by (colour(j), j).  With
// lrp == nullptr only the count is returned.  aIdx/aDiag: positions in the matrix's value array.
int64_t orc_mc_lower(int n, const int64_t* rp, const int* ci, const double* av, const unsigned char* colour,
                     int64_t* lrp, int* lci, int64_t* aIdx, int64_t* aDiag) {
    int64_t count = 0;
    std::vector<std::pair<int, int64_t>> row;
    if (lrp) lrp[0] = 0;
    for (int i = 0; i < n; ++i) {
        row.clear();
        for (int64_t k = rp[i]; k < rp[i + 1]; ++k) {
            const int j = ci[k];
            if (j == i) {
                if (aDiag) aDiag[i] = k;
            } else if (av[k] != 0.0 && colour[j] < colour[i]) {
                row.push_back({j, k});
            }
        }
        std::sort(row.begin(), row.end(), [&](const std::pair<int, int64_t>& a, const std::pair<int, int64_t>& b) {
            return colour[a.first] != colour[b.first] ? colour[a.first] < colour[b.first] : a.first < b.first;
        });
        for (auto& e : row) {
            if (lci) lci[count] = e.first;
            if (aIdx) aIdx[count] = e.second;
            ++count;
        }
        if (lrp) lrp[i + 1] = count;
    }
    return count;
}

// IC(0) on that pattern, rows taken colour by colour.  a_ii is scaled by (1 + shift).  Returns 0, or 1 if a
// pivot was not positive (the diagonal is then |a_ii| so the factor stays usable; the caller retries).
int orc_ic0(int n, int colours, const unsigned char* colour, const int64_t* lrp, const int* lci, const int64_t* aIdx,
            const int64_t* aDiag, const double* aval, double shift, double* lval, double* diag) {
    int failed = 0;
    for (int c = 0; c < colours; ++c)
        for (int i = 0; i < n; ++i) {
            if (colour[i] != c) continue;
            double sq = 0.0;
            for (int64_t k = lrp[i]; k < lrp[i + 1]; ++k) {
                const int j = lci[k];
                double s = aval[aIdx[k]];
                for (int64_t k2 = lrp[i]; k2 < k; ++k2) {
                    const int m = lci[k2];
                    for (int64_t kj = lrp[j]; kj < lrp[j + 1]; ++kj)
                        if (lci[kj] == m) {
                            s -= lval[k2] * lval[kj];
                            break;
                        }
                }
                lval[k] = s / diag[j];
                sq += lval[k] * lval[k];
            }
            const double aii = aval[aDiag[i]];
            double d = aii * (1.0 + shift) - sq;
            if (!(d > 1e-12 * std::fabs(aii))) {
                failed = 1;
                d = std::fabs(aii) > 0 ? std::fabs(aii) : 1.0;
            }
            diag[i] = std::sqrt(d);
        }
    return failed;
}

// PCG with M = L L^T.  Returns 0 converged, 1 iteration cap, 2 breakdown.
int orc_pcg(int n, const int64_t* rp, const int* ci, const double* av, int colours, const unsigned char* colour,
            const int64_t* lrp, const int* lci, const double* lval, const double* diag, const double* b,
            const double* x0, double* x, int maxIt, double tol, int* itersOut, double* relresOut) {
    if (maxIt < 0) maxIt = n;
    std::vector<std::vector<int>> byColour((size_t)colours);
    for (int i = 0; i < n; ++i) byColour[colour[i]].push_back(i);
    // upper part: row j holds (i, L_ij) for every i with j in L's row i, ordered by (colour(i), i)
    std::vector<int64_t> urp((size_t)n + 1, 0);
    for (int64_t k = 0; k < lrp[n]; ++k) ++urp[(size_t)lci[k] + 1];
    for (int i = 0; i < n; ++i) urp[i + 1] += urp[i];
    std::vector<int> uci((size_t)lrp[n]);
    std::vector<double> uval((size_t)lrp[n]);
    std::vector<int64_t> fill(urp.begin(), urp.end() - 1);
    for (int c = 0; c < colours; ++c)
        for (int i : byColour[c])
            for (int64_t k = lrp[i]; k < lrp[i + 1]; ++k) {
                const int j = lci[k];
                uci[fill[j]] = i;
                uval[fill[j]] = lval[k];
                ++fill[j];
            }
    std::vector<double> dinv((size_t)n);
    for (int i = 0; i < n; ++i) dinv[i] = 1.0 / diag[i];
    auto apply = [&](const std::vector<double>& r, std::vector<double>& w) {
        for (int c = 0; c < colours; ++c)
            for (int i : byColour[c]) {
                double acc = 0.0;
                for (int64_t k = lrp[i]; k < lrp[i + 1]; ++k) acc = std::fma(lval[k], w[lci[k]], acc);
                w[i] = (r[i] - acc) * dinv[i];
            }
        for (int c = colours - 1; c >= 0; --c)
            for (int i : byColour[c]) {
                double acc = 0.0;
                for (int64_t k = urp[i]; k < urp[i + 1]; ++k) acc = std::fma(uval[k], w[uci[k]], acc);
                w[i] = (w[i] - acc) * dinv[i];
            }
    };
    auto spmv = [&](const std::vector<double>& v, std::vector<double>& out) {
        for (int i = 0; i < n; ++i) {
            double acc = 0.0;
            for (int64_t k = rp[i]; k < rp[i + 1]; ++k) acc = std::fma(av[k], v[ci[k]], acc);
            out[i] = acc;
        }
    };
    std::vector<double> xx(x0, x0 + n), r((size_t)n), z((size_t)n), p((size_t)n), q((size_t)n);
    spmv(xx, q);
    double bb = 0, rr = 0;
    for (int i = 0; i < n; ++i) {
        r[i] = b[i] - q[i];
        bb += b[i] * b[i];
        rr += r[i] * r[i];
    }
    const double target = bb > 0 ? tol * tol * bb : tol * tol * rr;
    int it = 0, status = 1;
    if (rr <= target) status = 0;
    double rz = 0;
    if (status == 1) {
        apply(r, z);
        for (int i = 0; i < n; ++i) rz += r[i] * z[i];
        p = z;
    }
    while (status == 1 && it < maxIt) {
        spmv(p, q);
        double pq = 0;
        for (int i = 0; i < n; ++i) pq += p[i] * q[i];
        if (!(pq > 0) || !std::isfinite(pq)) { status = 2; break; }
        const double alpha = rz / pq;
        double rrNew = 0;
        for (int i = 0; i < n; ++i) {
            xx[i] += alpha * p[i];
            r[i] -= alpha * q[i];
            rrNew += r[i] * r[i];
        }
        ++it;
        rr = rrNew;
        if (!std::isfinite(rr)) { status = 2; break; }
        if (rr <= target) { status = 0; break; }
        apply(r, z);
        double rzNew = 0;
        for (int i = 0; i < n; ++i) rzNew += r[i] * z[i];
        if (!(rzNew > 0) || !std::isfinite(rzNew)) { status = 2; break; }
        const double beta = rzNew / rz;
        rz = rzNew;
        for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
    std::copy(xx.begin(), xx.end(), x);
    if (itersOut) *itersOut = it;
    if (relresOut) *relresOut = bb > 0 ? std::sqrt(rr / bb) : 0.0;
    return status;
}

}  // extern "C"
