// P2-P1 assembly of the five system matrices and the two Dirichlet lift matrices on the GPU.
//
// Replaces assembleAllMatrices (include/assembly.h:1302-1475): five TBB tasks that build triplet matrices
// element by element on the CPU, with Dirichlet elimination in assembleBCMatrix (include/assembly.h:994-1030).
// Here the host derives each sparsity pattern once from node-element incidence (parallel over rows), greedily
// colours the elements so that no two elements of a colour share a node, and one kernel per colour computes
// every local matrix of its elements (one thread per element, 32 elements per warp) and adds them into the
// CSR values at positions found by binary search in the row.  Colours run in a fixed order, so every entry
// is summed in the same order on every run: deterministic without atomics.
//
// Local matrices follow the reference's functors: precomputed reference-element integrals scaled by the
// element's Jacobian (LocalMassFunctor, include/assembly.h:842-882), the B-operator expansion of the
// stiffness (LocalStiffnessFunctor, :725-791) and of the divergence blocks (LocalDivergenceFunctor, :793-840),
// with the 7-point quadrature of TriangleIntegrator (:259-304).
#include "nsf_internal.cuh"

#include <algorithm>
#include <cstring>
#include <numeric>
#include <thread>

namespace nsf {

struct RefIntegralsDev {
    double mass[6][6];
    double delP2[12][12];
    double delP1[6][6];
    double divP1P2[3][12];
    double divP2P1[6][6];
};
__constant__ RefIntegralsDev c_ref;

// The P2 shape functions and their reference derivatives at the 7 quadrature points, with the weights: the
// per-point values the convection integrand needs (LocalConvection in NavierStokesAssembly::solve,
// include/assembly.h:1581-1625).
struct QuadTableDev {
    double psi[7][6];
    double dxi[7][6];
    double deta[7][6];
    double w[7];
};
__constant__ QuadTableDev c_quad;

static void p2_eval_h(double xi, double eta, double o[6]) {
    o[0] = 1 - 3 * xi - 3 * eta + 2 * xi * xi + 4 * xi * eta + 2 * eta * eta;
    o[1] = 2 * xi * xi - xi;
    o[2] = 2 * eta * eta - eta;
    o[3] = 4 * xi * eta;
    o[4] = 4 * eta - 4 * xi * eta - 4 * eta * eta;
    o[5] = 4 * xi - 4 * xi * xi - 4 * xi * eta;
}

// Reference-element integrals with the reference's quadrature (3 vertices 3/120, 3 midpoints 8/120,
// centroid 27/120).
static RefIntegralsDev reference_integrals() {
    RefIntegralsDev I;
    std::memset(&I, 0, sizeof(I));
    const double qx[7] = {0, 1, 0, 0.5, 0.5, 0, 1.0 / 3.0};
    const double qy[7] = {0, 0, 1, 0, 0.5, 0.5, 1.0 / 3.0};
    const double qw[7] = {3.0 / 120, 3.0 / 120, 3.0 / 120, 8.0 / 120, 8.0 / 120, 8.0 / 120, 27.0 / 120};
    for (int k = 0; k < 7; ++k) {
        const double xi = qx[k], eta = qy[k], w = qw[k];
        double psi[6], chi[3] = {1 - xi - eta, xi, eta};
        p2_eval_h(xi, eta, psi);
        const double dx2[6] = {-3 + 4 * eta + 4 * xi, -1 + 4 * xi, 0, 4 * eta, -4 * eta, 4 - 4 * eta - 8 * xi};
        const double de2[6] = {-3 + 4 * eta + 4 * xi, 0, -1 + 4 * eta, 4 * xi, 4 - 8 * eta - 4 * xi, -4 * xi};
        const double dx1[3] = {-1, 1, 0}, de1[3] = {-1, 0, 1};
        double d2[12], d1[6];
        for (int i = 0; i < 6; ++i) { d2[i] = dx2[i]; d2[6 + i] = de2[i]; }
        for (int i = 0; i < 3; ++i) { d1[i] = dx1[i]; d1[3 + i] = de1[i]; }
        for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) I.mass[i][j] += psi[i] * psi[j] * w;
        for (int a = 0; a < 12; ++a) for (int b = 0; b < 12; ++b) I.delP2[a][b] += d2[a] * d2[b] * w;
        for (int a = 0; a < 6; ++a) for (int b = 0; b < 6; ++b) I.delP1[a][b] += d1[a] * d1[b] * w;
        for (int p = 0; p < 3; ++p)
            for (int j = 0; j < 6; ++j) {
                I.divP1P2[p][j] += chi[p] * dx2[j] * w;
                I.divP1P2[p][j + 6] += chi[p] * de2[j] * w;
            }
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 3; ++j) {
                I.divP2P1[i][j] += psi[i] * dx1[j] * w;
                I.divP2P1[i][j + 3] += psi[i] * de1[j] * w;
            }
    }
    return I;
}

static QuadTableDev quad_table() {
    QuadTableDev Q;
    const double qx[7] = {0, 1, 0, 0.5, 0.5, 0, 1.0 / 3.0};
    const double qy[7] = {0, 0, 1, 0, 0.5, 0.5, 1.0 / 3.0};
    const double qw[7] = {3.0 / 120, 3.0 / 120, 3.0 / 120, 8.0 / 120, 8.0 / 120, 8.0 / 120, 27.0 / 120};
    for (int k = 0; k < 7; ++k) {
        const double xi = qx[k], eta = qy[k];
        p2_eval_h(xi, eta, Q.psi[k]);
        const double dx2[6] = {-3 + 4 * eta + 4 * xi, -1 + 4 * xi, 0, 4 * eta, -4 * eta, 4 - 4 * eta - 8 * xi};
        const double de2[6] = {-3 + 4 * eta + 4 * xi, 0, -1 + 4 * eta, 4 * xi, 4 - 8 * eta - 4 * xi, -4 * xi};
        for (int i = 0; i < 6; ++i) {
            Q.dxi[k][i] = dx2[i];
            Q.deta[k][i] = de2[i];
        }
        Q.w[k] = qw[k];
    }
    return Q;
}

// ---------------------------------------------------------------------------------------------------
// patterns (host, parallel over rows)
// ---------------------------------------------------------------------------------------------------
struct HostCsr {
    int rows = 0, cols = 0;
    std::vector<int> rowptr, col;
};

template <typename F> static void parallel_rows(int rows, F&& f) {
    const int nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    const int chunk = (rows + nt - 1) / nt;
    for (int t = 0; t < nt; ++t) {
        const int a = t * chunk, b = std::min(rows, a + chunk);
        if (a >= b) break;
        th.emplace_back([a, b, &f] {
            std::vector<int> buf;
            buf.reserve(128);
            for (int r = a; r < b; ++r) f(r, buf);
        });
    }
    for (auto& x : th) x.join();
}

// cand(row, buf) appends candidate columns; they are sorted and de-duplicated here.
template <typename Cand> static HostCsr build_pattern(int rows, int cols, Cand&& cand) {
    HostCsr m;
    m.rows = rows;
    m.cols = cols;
    m.rowptr.assign(rows + 1, 0);
    std::vector<int> counts(rows, 0);
    parallel_rows(rows, [&](int r, std::vector<int>& buf) {
        buf.clear();
        cand(r, buf);
        std::sort(buf.begin(), buf.end());
        counts[r] = (int)(std::unique(buf.begin(), buf.end()) - buf.begin());
    });
    int64_t total = 0;
    for (int r = 0; r < rows; ++r) {
        m.rowptr[r] = (int)total;
        total += counts[r];
        if (total > INT32_MAX) throw bad_arg("matrix has more than 2^31-1 non-zeros");
    }
    m.rowptr[rows] = (int)total;
    m.col.resize(total);
    parallel_rows(rows, [&](int r, std::vector<int>& buf) {
        buf.clear();
        cand(r, buf);
        std::sort(buf.begin(), buf.end());
        auto end = std::unique(buf.begin(), buf.end());
        std::copy(buf.begin(), end, m.col.begin() + m.rowptr[r]);
    });
    return m;
}

static void upload_pattern(Csr& A, const HostCsr& p, cudaStream_t s) {
    A.rows = p.rows;
    A.cols = p.cols;
    A.nnz = p.rowptr[p.rows];
    A.rowptr.upload(p.rowptr.data(), p.rowptr.size(), s);
    A.col.upload(p.col.data(), p.col.size(), s);
    A.val.alloc(std::max<int64_t>(A.nnz, 1));
    A.val.zero(s);
    A.values_changed();
}

// ---------------------------------------------------------------------------------------------------
// assembly kernel
// ---------------------------------------------------------------------------------------------------
struct AsmArgs {
    const float2* xy;
    const int* el;
    const int* order;      // elements sorted by colour
    int begin, end;        // this colour's slice of `order`
    int nNodes;
    double dtnu;
    const unsigned char* bcV;
    const unsigned char* bcP;
    // CSR targets (rowptr, col, val)
    const int *mRp, *mCol; double* mVal;       // velocity mass
    const int *dRp, *dCol; double* dVal;       // diffusion (BC eliminated)
    const int *wvRp, *wvCol; double* wvVal;    // velocity lift (row free, col Dirichlet)
    const int *kRp, *kCol; double* kVal;       // pressure stiffness (BC eliminated)
    const int *wpRp, *wpCol; double* wpVal;    // pressure lift
    const int *bRp, *bCol; double* bVal;       // divergence P x 2Nv
    const int *gRp, *gCol; double* gVal;       // gradient 2Nv x P
};

__device__ int g_missingSlots;   // entries a local matrix addressed outside the pattern (must stay 0)

__device__ __forceinline__ int find_slot(const int* rp, const int* col, int row, int c) {
    int lo = rp[row], hi = rp[row + 1] - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (col[mid] < c) lo = mid + 1;
        else hi = mid;
    }
    if (lo > hi || col[lo] != c) {   // cannot happen for patterns built from the same mesh; never write outside
        atomicAdd(&g_missingSlots, 1);
        return -1;
    }
    return lo;
}

__device__ __forceinline__ void add_at(double* val, int slot, double v) {
    if (slot >= 0) val[slot] += v;
}

__global__ void __launch_bounds__(128) assemble_colour_kernel(AsmArgs a) {
    const int k = a.begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.end) return;
    const int e = a.order[k];
    int t[6];
    double xy[12];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        t[i] = a.el[6 * (size_t)e + i];
        const float2 p = a.xy[t[i]];
        xy[2 * i] = p.x;
        xy[2 * i + 1] = p.y;
    }
    // Jacobian determinant (linTriangleTmJacobian) and the B operator (differentialOperator)
    const double jdet = (xy[2] - xy[0]) * (xy[5] - xy[1]) - (xy[3] - xy[1]) * (xy[4] - xy[0]);
    const double jabs = fabs(jdet);
    double B[2][2];
    B[0][0] = xy[5] - xy[1];
    B[0][1] = xy[1] - xy[3];
    B[1][0] = xy[0] - xy[4];
    B[1][1] = xy[2] - xy[0];
    const double bdet = B[0][0] * B[1][1] - B[0][1] * B[1][0];
    const double invJ = 1.0 / fabs(bdet);

    // velocity mass, diffusion, velocity lift
    for (int i = 0; i < 6; ++i) {
        const int row = t[i];
        const bool rb = a.bcV[row];
        for (int j = 0; j < 6; ++j) {
            const int col = t[j];
            const double m = c_ref.mass[i][j] * jabs;
            double kij = 0;
            const double s0 = c_ref.delP2[i][j], s1 = c_ref.delP2[i][6 + j], s2 = c_ref.delP2[6 + i][j],
                         s3 = c_ref.delP2[6 + i][6 + j];
#pragma unroll
            for (int q = 0; q < 2; ++q)
                kij += s0 * B[q][0] * B[q][0] + s1 * B[q][0] * B[q][1] + s2 * B[q][0] * B[q][1] + s3 * B[q][1] * B[q][1];
            kij *= invJ;
            add_at(a.mVal, find_slot(a.mRp, a.mCol, row, col), m);
            if (!rb) {
                const double d = m + kij * a.dtnu;
                if (!a.bcV[col]) add_at(a.dVal, find_slot(a.dRp, a.dCol, row, col), d);
                else add_at(a.wvVal, find_slot(a.wvRp, a.wvCol, row, col), d);
            }
        }
    }
    // pressure stiffness (P1) and pressure lift
    for (int i = 0; i < 3; ++i) {
        const int row = t[i];
        if (a.bcP[row]) continue;
        for (int j = 0; j < 3; ++j) {
            const int col = t[j];
            double kij = 0;
            const double s0 = c_ref.delP1[i][j], s1 = c_ref.delP1[i][3 + j], s2 = c_ref.delP1[3 + i][j],
                         s3 = c_ref.delP1[3 + i][3 + j];
#pragma unroll
            for (int q = 0; q < 2; ++q)
                kij += s0 * B[q][0] * B[q][0] + s1 * B[q][0] * B[q][1] + s2 * B[q][0] * B[q][1] + s3 * B[q][1] * B[q][1];
            kij *= invJ;
            if (!a.bcP[col]) add_at(a.kVal, find_slot(a.kRp, a.kCol, row, col), kij);
            else add_at(a.wpVal, find_slot(a.wpRp, a.wpCol, row, col), kij);
        }
    }
    // divergence (P1 rows x P2 columns, x block then y block) and gradient (P2 rows x P1 columns)
    for (int p = 0; p < 3; ++p) {
        const int row = t[p];
        for (int q = 0; q < 6; ++q) {
            const double dx = B[0][0] * c_ref.divP1P2[p][q] + B[0][1] * c_ref.divP1P2[p][q + 6];
            const double dy = B[1][0] * c_ref.divP1P2[p][q] + B[1][1] * c_ref.divP1P2[p][q + 6];
            add_at(a.bVal, find_slot(a.bRp, a.bCol, row, t[q]), dx);
            add_at(a.bVal, find_slot(a.bRp, a.bCol, row, t[q] + a.nNodes), dy);
        }
    }
    for (int q = 0; q < 6; ++q) {
        for (int p = 0; p < 3; ++p) {
            const double dx = B[0][0] * c_ref.divP2P1[q][p] + B[0][1] * c_ref.divP2P1[q][p + 3];
            const double dy = B[1][0] * c_ref.divP2P1[q][p] + B[1][1] * c_ref.divP2P1[q][p + 3];
            add_at(a.gVal, find_slot(a.gRp, a.gCol, t[q], t[p]), dx);
            add_at(a.gVal, find_slot(a.gRp, a.gCol, t[q] + a.nNodes, t[p]), dy);
        }
    }
}

// The explicit-convection step's right-hand side, rhs -= dt (C(u) + nu K) u for both velocity components, matrix
// free: per element the local convection matrix C_ij = sign sum_q w_q psi_i (u_h B dpsi_j) (the reference's
// integrand psi^T psi U B dpsi, include/assembly.h:1601-1616, with u_h = psi U at the point, applied to the local
// velocities without forming C) and the local stiffness K of the assembly kernel; one thread per element, one launch
// per element colour, so no two threads of a launch add into the same row.
struct ConvArgs {
    const float2* xy;
    const int* el;
    const int* order;
    int begin, end;
    int nNodes;
    double dt, nu;
    const double* uv;   // [u | v]
    double* rhs;        // [u | v], accumulated
};

__global__ void __launch_bounds__(128) convection_rhs_kernel(ConvArgs a) {
    const int k = a.begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.end) return;
    const int e = a.order[k];
    int t[6];
    double xy[12], u[6], v[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        t[i] = a.el[6 * (size_t)e + i];
        const float2 p = a.xy[t[i]];
        xy[2 * i] = p.x;
        xy[2 * i + 1] = p.y;
        u[i] = a.uv[t[i]];
        v[i] = a.uv[t[i] + a.nNodes];
    }
    double B[2][2];
    B[0][0] = xy[5] - xy[1];
    B[0][1] = xy[1] - xy[3];
    B[1][0] = xy[0] - xy[4];
    B[1][1] = xy[2] - xy[0];
    const double bdet = B[0][0] * B[1][1] - B[0][1] * B[1][0];
    const double sign = bdet > 0 ? 1.0 : -1.0;
    const double invJ = 1.0 / fabs(bdet);
    // per quadrature point: the convected derivative of the local u and v, (u_h B dpsi) . U
    double cu[6] = {}, cv[6] = {};
#pragma unroll
    for (int q = 0; q < 7; ++q) {
        double uh = 0, vh = 0;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            uh = fma(c_quad.psi[q][j], u[j], uh);
            vh = fma(c_quad.psi[q][j], v[j], vh);
        }
        const double g0 = uh * B[0][0] + vh * B[1][0];
        const double g1 = uh * B[0][1] + vh * B[1][1];
        double du = 0, dv = 0;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            const double gj = g0 * c_quad.dxi[q][j] + g1 * c_quad.deta[q][j];
            du = fma(gj, u[j], du);
            dv = fma(gj, v[j], dv);
        }
        const double wq = c_quad.w[q] * sign;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            cu[i] = fma(wq * c_quad.psi[q][i], du, cu[i]);
            cv[i] = fma(wq * c_quad.psi[q][i], dv, cv[i]);
        }
    }
    for (int i = 0; i < 6; ++i) {
        double ku = 0, kv = 0;
        for (int j = 0; j < 6; ++j) {
            double kij = 0;
            const double s0 = c_ref.delP2[i][j], s1 = c_ref.delP2[i][6 + j], s2 = c_ref.delP2[6 + i][j],
                         s3 = c_ref.delP2[6 + i][6 + j];
#pragma unroll
            for (int q = 0; q < 2; ++q)
                kij += s0 * B[q][0] * B[q][0] + s1 * B[q][0] * B[q][1] + s2 * B[q][0] * B[q][1] + s3 * B[q][1] * B[q][1];
            kij *= invJ;
            ku = fma(kij, u[j], ku);
            kv = fma(kij, v[j], kv);
        }
        a.rhs[t[i]] -= a.dt * (cu[i] + a.nu * ku);
        a.rhs[t[i] + a.nNodes] -= a.dt * (cv[i] + a.nu * kv);
    }
}

void convection_rhs_launch(const MeshDev& m, const SimState& S, const double* uv, double* rhs, cudaStream_t s) {
    NSF_CUDA(cudaMemsetAsync(rhs, 0, sizeof(double) * 2 * (size_t)m.nNodes, s));
    ConvArgs a{};
    a.xy = m.xy.get();
    a.el = m.el.get();
    a.order = S.elOrder.get();
    a.nNodes = m.nNodes;
    a.dt = S.dt;
    a.nu = S.viscosity;
    a.uv = uv;
    a.rhs = rhs;
    for (size_t c = 0; c + 1 < S.elStart.size(); ++c) {
        a.begin = S.elStart[c];
        a.end = S.elStart[c + 1];
        const int n = a.end - a.begin;
        if (n == 0) continue;
        convection_rhs_kernel<<<(n + 127) / 128, 128, 0, s>>>(a);
        NSF_CUDA(cudaGetLastError());
        count_launch();
    }
}

// Dirichlet rows become identity rows: the diagonal entry is the only one the pattern keeps there.
__global__ void bc_diagonal_kernel(int n, const unsigned char* bc, const int* rp, double* val) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (bc[i]) val[rp[i]] = 1.0;
}

__global__ void scale_kernel(int64_t n, double s, double* v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] *= s;
}

static int blocks(int64_t n, int t) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + t - 1) / t, 152 * 64)); }

// Builds every matrix of a mesh and the greedy element colouring into `mats`.  Returns the colour count.
int assemble_instance(MeshDev& m, SimState& sim, Csr* mats, cudaStream_t s, double viscosity, double dt) {
    const int Nv = m.nNodes, P = m.nP, T = m.nEl;
    const int* el = m.hel.data();
    const std::vector<unsigned char>& bcV = sim.hbcV;
    const std::vector<unsigned char>& bcP = sim.hbcP;

    // node -> element incidence
    std::vector<int> incStart(Nv + 1, 0), inc((size_t)6 * T);
    for (size_t k = 0; k < (size_t)6 * T; ++k) incStart[el[k] + 1]++;
    for (int i = 0; i < Nv; ++i) incStart[i + 1] += incStart[i];
    {
        std::vector<int> fill(incStart.begin(), incStart.end() - 1);
        for (int e = 0; e < T; ++e)
            for (int j = 0; j < 6; ++j) inc[fill[el[6 * (size_t)e + j]]++] = e;
    }
    auto nodesOf = [&](int node, int count, auto&& keep, std::vector<int>& buf, int offset) {
        for (int k = incStart[node]; k < incStart[node + 1]; ++k) {
            const int* en = el + 6 * (size_t)inc[k];
            for (int j = 0; j < count; ++j)
                if (keep(en[j])) buf.push_back(en[j] + offset);
        }
    };
    auto all = [](int) { return true; };
    auto freeV = [&](int c) { return !bcV[c]; };
    auto dirV = [&](int c) { return (bool)bcV[c]; };
    auto freeP = [&](int c) { return !bcP[c]; };
    auto dirP = [&](int c) { return (bool)bcP[c]; };

    HostCsr pM = build_pattern(Nv, Nv, [&](int r, std::vector<int>& b) { nodesOf(r, 6, all, b, 0); });
    HostCsr pD = build_pattern(Nv, Nv, [&](int r, std::vector<int>& b) {
        if (bcV[r]) b.push_back(r);
        else nodesOf(r, 6, freeV, b, 0);
    });
    HostCsr pWv = build_pattern(Nv, Nv, [&](int r, std::vector<int>& b) { if (!bcV[r]) nodesOf(r, 6, dirV, b, 0); });
    HostCsr pK = build_pattern(P, P, [&](int r, std::vector<int>& b) {
        if (bcP[r]) b.push_back(r);
        else nodesOf(r, 3, freeP, b, 0);
    });
    HostCsr pWp = build_pattern(P, P, [&](int r, std::vector<int>& b) { if (!bcP[r]) nodesOf(r, 3, dirP, b, 0); });
    HostCsr pB = build_pattern(P, 2 * Nv, [&](int r, std::vector<int>& b) {
        nodesOf(r, 6, all, b, 0);
        nodesOf(r, 6, all, b, Nv);
    });
    HostCsr pG = build_pattern(2 * Nv, P, [&](int r, std::vector<int>& b) { nodesOf(r % Nv, 3, all, b, 0); });

    upload_pattern(mats[NSF_VELOCITY_MASS], pM, s);
    upload_pattern(mats[NSF_DIFFUSION], pD, s);
    upload_pattern(mats[NSF_VELOCITY_LIFT], pWv, s);
    upload_pattern(mats[NSF_PRESSURE_STIFFNESS], pK, s);
    upload_pattern(mats[NSF_PRESSURE_LIFT], pWp, s);
    upload_pattern(mats[NSF_VELOCITY_DIVERGENCE], pB, s);
    upload_pattern(mats[NSF_PRESSURE_DIVERGENCE], pG, s);

    // greedy colouring in element order: no two elements of one colour share a node
    std::vector<unsigned long long> used(Nv, 0ull);
    std::vector<int> colour(T);
    int nColours = 0;
    for (int e = 0; e < T; ++e) {
        unsigned long long mask = 0;
        for (int j = 0; j < 6; ++j) mask |= used[el[6 * (size_t)e + j]];
        if (mask == ~0ull) throw bad_arg("element colouring needs more than 64 colours");
        const int c = __builtin_ctzll(~mask);
        colour[e] = c;
        nColours = std::max(nColours, c + 1);
        for (int j = 0; j < 6; ++j) used[el[6 * (size_t)e + j]] |= 1ull << c;
    }
    std::vector<int> cStart(nColours + 1, 0), order(T);
    for (int e = 0; e < T; ++e) cStart[colour[e] + 1]++;
    for (int c = 0; c < nColours; ++c) cStart[c + 1] += cStart[c];
    {
        std::vector<int> fill(cStart.begin(), cStart.end() - 1);
        for (int e = 0; e < T; ++e) order[fill[colour[e]]++] = e;
    }
    sim.elOrder.upload(order.data(), order.size(), s);   // (kept for the explicit-convection step)
    sim.elStart = cStart;
    const int* dOrder = sim.elOrder.get();

    const RefIntegralsDev I = reference_integrals();
    NSF_CUDA(cudaMemcpyToSymbolAsync(c_ref, &I, sizeof(I), 0, cudaMemcpyHostToDevice, s));
    const QuadTableDev Q = quad_table();
    NSF_CUDA(cudaMemcpyToSymbolAsync(c_quad, &Q, sizeof(Q), 0, cudaMemcpyHostToDevice, s));

    AsmArgs a{};
    a.xy = m.xy.get();
    a.el = m.el.get();
    a.order = dOrder;
    a.nNodes = Nv;
    a.dtnu = dt * viscosity;
    a.bcV = sim.bcV.get();
    a.bcP = sim.bcP.get();
    auto bind = [&](int slot, const int*& rp, const int*& col, double*& val) {
        rp = mats[slot].rowptr.get();
        col = mats[slot].col.get();
        val = mats[slot].val.get();
    };
    bind(NSF_VELOCITY_MASS, a.mRp, a.mCol, a.mVal);
    bind(NSF_DIFFUSION, a.dRp, a.dCol, a.dVal);
    bind(NSF_VELOCITY_LIFT, a.wvRp, a.wvCol, a.wvVal);
    bind(NSF_PRESSURE_STIFFNESS, a.kRp, a.kCol, a.kVal);
    bind(NSF_PRESSURE_LIFT, a.wpRp, a.wpCol, a.wpVal);
    bind(NSF_VELOCITY_DIVERGENCE, a.bRp, a.bCol, a.bVal);
    bind(NSF_PRESSURE_DIVERGENCE, a.gRp, a.gCol, a.gVal);
    const int zero = 0;
    NSF_CUDA(cudaMemcpyToSymbolAsync(g_missingSlots, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s));
    for (int c = 0; c < nColours; ++c) {
        a.begin = cStart[c];
        a.end = cStart[c + 1];
        const int n = a.end - a.begin;
        if (n == 0) continue;
        assemble_colour_kernel<<<(n + 127) / 128, 128, 0, s>>>(a);
        NSF_CUDA(cudaGetLastError());
    }
    bc_diagonal_kernel<<<blocks(Nv, 256), 256, 0, s>>>(Nv, sim.bcV.get(), a.dRp, a.dVal);
    bc_diagonal_kernel<<<blocks(P, 256), 256, 0, s>>>(P, sim.bcP.get(), a.kRp, a.kVal);
    Csr& Bd = mats[NSF_VELOCITY_DIVERGENCE];
    Csr& Gd = mats[NSF_PRESSURE_DIVERGENCE];
    scale_kernel<<<blocks(Bd.nnz, 256), 256, 0, s>>>(Bd.nnz, -(1.0 / dt), Bd.val.get());
    scale_kernel<<<blocks(Gd.nnz, 256), 256, 0, s>>>(Gd.nnz, -dt, Gd.val.get());
    NSF_CUDA(cudaGetLastError());
    count_launch(nColours + 4);
    int missing = 0;
    NSF_CUDA(cudaMemcpyFromSymbolAsync(&missing, g_missingSlots, sizeof(int), 0, cudaMemcpyDeviceToHost, s));
    NSF_CUDA(cudaStreamSynchronize(s));
    if (missing) throw Error{NSF_ERR_BAD_ARG, std::to_string(missing) + " local entries fell outside the assembled pattern"};
    return nColours;
}

}  // namespace nsf
