// ORACLE — test infrastructure only.  A CPU restatement of the reference solver's per-time-step hot
// path (vasil-pashov/Navier_Stokes_FEM), used by tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline as the checker.  Nothing in the product links or calls this file.
//
// Restated from (paths inside the reference project):
//   include/assembly.h:98-151    Jacobian determinant and the B operator (linTriangleTmJacobian, differentialOperator)
//   include/assembly.h:154-257   P1 / P2 shape functions and their xi/eta derivatives
//   include/assembly.h:259-304   triangle quadrature: 7 points, weights 3,3,3,8,8,8,27 / 120 (8th slot zero)
//   include/assembly.h:725-882   local stiffness / divergence / mass functors (precomputed integrals)
//   include/assembly.h:994-1054  Dirichlet elimination: BC rows -> identity, BC columns -> transposed weights
//   include/assembly.h:1302-1475 the five matrices: M, M + dt*nu*K (BC), Kp (BC), -(1/dt)*Div (P x 2Nv), -dt*Grad (2Nv x P)
//   include/assembly.h:489-712   diffusion solve and pressure projection algebra, incl. initial guesses
//   include/assembly.h:1477-1579 the operator-split loop and velocity Dirichlet re-imposition
//   include/assembly.h:1664-1728 semi-Lagrangian advection: back-trace, locate, P2 interpolation / nearest node
//   cpp/kd_tree_builder.cpp:81-149, gpu_cpu_shared/kd_tree.cuh:40-169, kd_tree_common.cuh:18-61, misc_common.cuh:59-65
//                                the KD tree: buggy grid bbox, midpoint splits, straddlers on both sides,
//                                first-in-leaf containment, nearest-node fallback
//   tex/Chapters/01_chapter_FEM.tex:644-661  conjugate gradient (the reference's CPU CG lives in the absent
//                                sparse_matrix_math submodule; this restatement stops on the RELATIVE residual
//                                ||r|| <= tol * ||b||, which is what the GPU path implements too)
//
// The scalar type is a template parameter: real = double is the FP64 oracle, real = float reproduces the
// reference's own FP32 arithmetic.  Point location always runs in float exactly as the reference does, and
// this file must be compiled with -ffp-contract=off so every float product is rounded on its own.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

// ------------------------------------------------------------------------------------------------
// Shape functions and quadrature (include/assembly.h:154-304)
// ------------------------------------------------------------------------------------------------
template <typename R> static void p2_eval(R xi, R eta, R out[6]) {
    out[0] = 1 - 3 * xi - 3 * eta + 2 * xi * xi + 4 * xi * eta + 2 * eta * eta;
    out[1] = 2 * xi * xi - xi;
    out[2] = 2 * eta * eta - eta;
    out[3] = 4 * xi * eta;
    out[4] = 4 * eta - 4 * xi * eta - 4 * eta * eta;
    out[5] = 4 * xi - 4 * xi * xi - 4 * xi * eta;
}
template <typename R> static void p2_del(R xi, R eta, R dxi[6], R deta[6]) {
    dxi[0] = -3 + 4 * eta + 4 * xi; dxi[1] = -1 + 4 * xi; dxi[2] = 0; dxi[3] = 4 * eta; dxi[4] = -4 * eta;
    dxi[5] = 4 - 4 * eta - 8 * xi;
    deta[0] = -3 + 4 * eta + 4 * xi; deta[1] = 0; deta[2] = -1 + 4 * eta; deta[3] = 4 * xi;
    deta[4] = 4 - 8 * eta - 4 * xi; deta[5] = -4 * xi;
}
template <typename R> static void p1_eval(R xi, R eta, R out[3]) { out[0] = 1 - xi - eta; out[1] = xi; out[2] = eta; }
template <typename R> static void p1_del(R, R, R dxi[3], R deta[3]) {
    dxi[0] = -1; dxi[1] = 1; dxi[2] = 0; deta[0] = -1; deta[1] = 0; deta[2] = 1;
}

template <typename R> struct Quadrature {
    static constexpr int n = 8;   // the reference declares 8 points and fills 7; the 8th is (0,0) with weight 0
    R x[n], y[n], w[n];
    Quadrature() {
        const R px[7] = {0, 1, 0, R(0.5), R(0.5), 0, R(1.0) / R(3.0)};
        const R py[7] = {0, 0, 1, 0, R(0.5), R(0.5), R(1.0) / R(3.0)};
        const R pw[7] = {R(3.0) / R(120.0), R(3.0) / R(120.0), R(3.0) / R(120.0), R(8.0) / R(120.0),
                         R(8.0) / R(120.0), R(8.0) / R(120.0), R(27.0) / R(120.0)};
        for (int i = 0; i < n; ++i) { x[i] = i < 7 ? px[i] : 0; y[i] = i < 7 ? py[i] : 0; w[i] = i < 7 ? pw[i] : 0; }
    }
};

// Reference-element integrals, precomputed once exactly as the local functors' constructors do.
template <typename R> struct RefIntegrals {
    R mass[6][6];            // int psi_i psi_j
    R delP2[12][12];         // int d(psi)_a d(psi)_b, index = k*6 + i with k=0 xi, 1 eta
    R delP1[6][6];
    R divP1P2[3][12];        // int chi_p dpsi_q/dxi (q) and /deta (q+6): LocalDivergenceFunctor<P1,P2>
    R divP2P1[6][6];         // int psi_q dchi_p/dxi (p) and /deta (p+3): LocalDivergenceFunctor<P2,P1>
    RefIntegrals() {
        Quadrature<R> q;
        std::memset(this, 0, sizeof(*this));
        for (int k = 0; k < q.n; ++k) {
            R psi[6], chi[3], dx2[6], de2[6], dx1[3], de1[3];
            p2_eval(q.x[k], q.y[k], psi);
            p1_eval(q.x[k], q.y[k], chi);
            p2_del(q.x[k], q.y[k], dx2, de2);
            p1_del(q.x[k], q.y[k], dx1, de1);
            R d2[12], d1[6];
            for (int i = 0; i < 6; ++i) { d2[i] = dx2[i]; d2[6 + i] = de2[i]; }
            for (int i = 0; i < 3; ++i) { d1[i] = dx1[i]; d1[3 + i] = de1[i]; }
            // each integrand is evaluated fully, then added with its weight (TriangleIntegrator::integrate)
            for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) mass[i][j] += (psi[i] * psi[j]) * q.w[k];
            for (int a = 0; a < 12; ++a) for (int b = 0; b < 12; ++b) delP2[a][b] += (d2[a] * d2[b]) * q.w[k];
            for (int a = 0; a < 6; ++a) for (int b = 0; b < 6; ++b) delP1[a][b] += (d1[a] * d1[b]) * q.w[k];
            for (int p = 0; p < 3; ++p) for (int j = 0; j < 6; ++j) {
                divP1P2[p][j] += (chi[p] * dx2[j]) * q.w[k];
                divP1P2[p][j + 6] += (chi[p] * de2[j]) * q.w[k];
            }
            for (int i = 0; i < 6; ++i) for (int j = 0; j < 3; ++j) {
                divP2P1[i][j] += (psi[i] * dx1[j]) * q.w[k];
                divP2P1[i][j + 3] += (psi[i] * de1[j]) * q.w[k];
            }
        }
    }
};

// B = [[ym-yk, yk-yl], [xk-xm, xl-xk]], det = B00*B11 - B01*B10 (include/assembly.h:132-151)
template <typename R> static void diff_operator(const R* xy, R& det, R B[2][2]) {
    B[0][0] = xy[5] - xy[1];
    B[0][1] = xy[1] - xy[3];
    B[1][0] = xy[0] - xy[4];
    B[1][1] = xy[2] - xy[0];
    det = B[0][0] * B[1][1] - B[0][1] * B[1][0];
}
template <typename R> static R jacobian_det(const R* xy) {
    const R a = xy[2] - xy[0], b = xy[3] - xy[1], c = xy[4] - xy[0], d = xy[5] - xy[1];
    return a * d - b * c;
}

// Local stiffness for `n` shape functions from precomputed derivative-pair integrals (assembly.h:746-788)
template <typename R, int n, int ld> static void local_stiffness(const R* xy, const R (&sq)[ld][ld], R out[n][n]) {
    R B[2][2], J;
    diff_operator(xy, J, B);
    J = R(1.0) / std::abs(J);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            R acc = 0;
            const R s0 = sq[i][j], s1 = sq[i][n + j], s2 = sq[n + i][j], s3 = sq[n + i][n + j];
            for (int k = 0; k < 2; ++k)
                acc += s0 * B[k][0] * B[k][0] + s1 * B[k][0] * B[k][1] + s2 * B[k][0] * B[k][1] + s3 * B[k][1] * B[k][1];
            out[i][j] = acc * J;
        }
}

// Local convection matrix of NavierStokesAssembly::assembleConvectionMatrix (include/assembly.h:1584-1622): at each
// quadrature point the integrand (psi^T psi U B dpsi) sign, U the element's 6 x 2 nodal velocities, evaluated left
// to right as the reference's StaticMatrix products do (each entry summed from zero over the inner index in order),
// then added with its weight (TriangleIntegrator::integrate), so that the float instantiation reproduces the
// reference's arithmetic.
template <typename R> static void local_convection(const R* xy, const R vel[6][2], R out[6][6]) {
    R B[2][2], det;
    diff_operator(xy, det, B);
    const R sign = det > 0 ? R(1) : R(-1);
    const Quadrature<R> q;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) out[i][j] = 0;
    for (int k = 0; k < q.n; ++k) {
        R psi[6], dxi[6], deta[6];
        p2_eval(q.x[k], q.y[k], psi);
        p2_del(q.x[k], q.y[k], dxi, deta);
        R t1[6][6], t2[6][2], t3[6][2];
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) t1[i][j] = R(0) + psi[i] * psi[j];          // psi^T psi
        for (int i = 0; i < 6; ++i)
            for (int c = 0; c < 2; ++c) {                                          // (psi^T psi) U
                R a = 0;
                for (int m = 0; m < 6; ++m) a += t1[i][m] * vel[m][c];
                t2[i][c] = a;
            }
        for (int i = 0; i < 6; ++i)
            for (int c = 0; c < 2; ++c) {                                          // ... B
                R a = 0;
                for (int m = 0; m < 2; ++m) a += t2[i][m] * B[m][c];
                t3[i][c] = a;
            }
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {                                          // ... dpsi, sign, weight
                R a = 0;
                a += t3[i][0] * dxi[j];
                a += t3[i][1] * deta[j];
                out[i][j] += (a * sign) * q.w[k];
            }
    }
}

// ------------------------------------------------------------------------------------------------
// Sparse matrices: triplets summed in insertion order, rows sorted by column (SMM::TripletMatrix -> CSRMatrix)
// ------------------------------------------------------------------------------------------------
template <typename R> struct CSR {
    int rows = 0, cols = 0;
    std::vector<int64_t> rowptr;
    std::vector<int> col;
    std::vector<R> val;
    int64_t nnz() const { return rowptr.empty() ? 0 : rowptr[rows]; }
    void multiply(const R* x, R* y) const {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < rows; ++i) {
            R s = 0;
            for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) s += val[k] * x[col[k]];
            y[i] = s;
        }
    }
    void scale(R a) { for (auto& v : val) v *= a; }
};

// Triplets are added from `parts` contiguous element ranges at once (one per thread); part k holds the entries of
// the k-th range in insertion order, so concatenating the parts in order gives exactly the serial insertion order of
// the element loop.  to_csr keeps that order within every row (a stable counting sort by row, parts in order), then
// stable-sorts each row by column and sums duplicates in that order - the same sums, bit for bit, as one serial pass.
template <typename R> struct Triplets {
    struct Entry { int row, col; R val; };
    int rows, cols;
    std::vector<std::vector<Entry>> parts;
    Triplets(int r, int c, int nparts) : rows(r), cols(c), parts(nparts) {}
    void add(int part, int r, int c, R v) { parts[part].push_back(Entry{r, c, v}); }
    CSR<R> to_csr() {
        const int np = (int)parts.size();
        // cnt[k*rows + r]: entries of row r in part k, turned into that part's first slot in row r
        std::vector<int64_t> cnt((size_t)np * rows, 0);
#pragma omp parallel for schedule(static, 1)
        for (int k = 0; k < np; ++k)
            for (const Entry& e : parts[k]) ++cnt[(size_t)k * rows + e.row];
        std::vector<int64_t> start(rows + 1, 0);
#pragma omp parallel for schedule(static)
        for (int r = 0; r < rows; ++r) {
            int64_t s = 0;
            for (int k = 0; k < np; ++k) s += cnt[(size_t)k * rows + r];
            start[r + 1] = s;
        }
        for (int r = 0; r < rows; ++r) start[r + 1] += start[r];
#pragma omp parallel for schedule(static)
        for (int r = 0; r < rows; ++r) {
            int64_t o = start[r];
            for (int k = 0; k < np; ++k) {
                const int64_t c = cnt[(size_t)k * rows + r];
                cnt[(size_t)k * rows + r] = o;
                o += c;
            }
        }
        std::unique_ptr<std::pair<int, R>[]> tmp(new std::pair<int, R>[start[rows]]);
#pragma omp parallel for schedule(static, 1)
        for (int k = 0; k < np; ++k) {
            for (const Entry& e : parts[k]) tmp[cnt[(size_t)k * rows + e.row]++] = {e.col, e.val};
            std::vector<Entry>().swap(parts[k]);
        }
        std::vector<int64_t>().swap(cnt);
        // per row: stable sort by column, sum duplicates in order (in place), count the distinct columns
        std::vector<int64_t> uniq(rows + 1, 0);
#pragma omp parallel for schedule(dynamic, 1024)
        for (int r = 0; r < rows; ++r) {
            auto b = tmp.get() + start[r], e = tmp.get() + start[r + 1];
            std::stable_sort(b, e, [](const auto& x, const auto& y) { return x.first < y.first; });
            int64_t w = start[r];
            for (int64_t q = start[r]; q < start[r + 1]; ++q) {
                if (w > start[r] && tmp[w - 1].first == tmp[q].first) tmp[w - 1].second += tmp[q].second;
                else tmp[w++] = tmp[q];
            }
            uniq[r + 1] = w - start[r];
        }
        CSR<R> m;
        m.rows = rows; m.cols = cols;
        m.rowptr.assign(rows + 1, 0);
        for (int r = 0; r < rows; ++r) m.rowptr[r + 1] = m.rowptr[r] + uniq[r + 1];
        m.col.resize(m.rowptr[rows]);
        m.val.resize(m.rowptr[rows]);
#pragma omp parallel for schedule(static)
        for (int r = 0; r < rows; ++r) {
            int64_t o = m.rowptr[r];
            for (int64_t q = start[r]; q < start[r] + uniq[r + 1]; ++q) { m.col[o] = tmp[q].first; m.val[o] = tmp[q].second; ++o; }
        }
        return m;
    }
};

// ------------------------------------------------------------------------------------------------
// Conjugate gradient (thesis algorithm, tex/Chapters/01_chapter_FEM.tex:644-661), relative residual stop.
// Returns 0 converged, 1 iteration cap reached, 2 breakdown (p.Ap <= 0 or non-finite).
// ------------------------------------------------------------------------------------------------
template <typename R>
static int conjugate_gradient(const CSR<R>& A, const R* b, const R* x0, R* x, int maxIt, double tol,
                              int* itersOut, double* relresOut) {
    const int n = A.rows;
    if (maxIt < 0) maxIt = n;
    std::vector<R> r(n), p(n), q(n);
    std::vector<R> xx(x0, x0 + n);
    A.multiply(xx.data(), q.data());
    double bb = 0, rr = 0;
#pragma omp parallel for reduction(+ : bb, rr)
    for (int i = 0; i < n; ++i) {
        r[i] = b[i] - q[i];
        p[i] = r[i];
        bb += (double)b[i] * (double)b[i];
        rr += (double)r[i] * (double)r[i];
    }
    const double target = bb > 0 ? tol * tol * bb : tol * tol * rr;
    int it = 0, status = 1;
    if (rr <= target) status = 0;
    while (status == 1 && it < maxIt) {
        A.multiply(p.data(), q.data());
        double pq = 0;
#pragma omp parallel for reduction(+ : pq)
        for (int i = 0; i < n; ++i) pq += (double)p[i] * (double)q[i];
        if (!(pq > 0) || !std::isfinite(pq)) { status = 2; break; }
        const R alpha = (R)(rr / pq);
        double rrNew = 0;
#pragma omp parallel for reduction(+ : rrNew)
        for (int i = 0; i < n; ++i) {
            xx[i] += alpha * p[i];
            r[i] -= alpha * q[i];
            rrNew += (double)r[i] * (double)r[i];
        }
        ++it;
        if (!std::isfinite(rrNew)) { status = 2; break; }
        if (rrNew <= target) { rr = rrNew; status = 0; break; }
        const R beta = (R)(rrNew / rr);
        rr = rrNew;
#pragma omp parallel for
        for (int i = 0; i < n; ++i) p[i] = r[i] + beta * p[i];
    }
    std::copy(xx.begin(), xx.end(), x);
    if (itersOut) *itersOut = it;
    if (relresOut) *relresOut = bb > 0 ? std::sqrt(rr / bb) : 0.0;
    return status;
}

// ------------------------------------------------------------------------------------------------
// KD tree over triangles, as the reference builds and walks it (float throughout)
// ------------------------------------------------------------------------------------------------
struct TreeNode {
    int axis;        // 0 x, 1 y, 2 leaf
    int right;       // internal: index of the right child (left child = this + 1)
    float split;
    int offset;      // leaf: first slot in leafTris (the reference stores it as uint and returns it via float)
    int count;       // leaf: number of triangles
};

struct KDTree {
    const float* xy = nullptr;       // node coordinates, [2*Nv]
    const int* el = nullptr;         // elements, [6*T]
    std::vector<TreeNode> nodes;
    std::vector<int> leafTris;
    int maxDepth = 0;
    static constexpr int kLeafSize = 16;

    void build(const float* xy_, const int* el_, int nNodes, int nEl) {
        xy = xy_; el = el_;
        // grid bbox as FemGrid2D::loadJSON computes it: BBox2D::expand keeps max = the LAST node
        // (misc_common.cuh:59-65), min = the true minimum.
        float mn[2] = {FLT_MAX, FLT_MAX}, mx[2] = {-FLT_MAX, -FLT_MAX};
        for (int i = 0; i < nNodes; ++i) {
            const float px = xy[2 * i], py = xy[2 * i + 1];
            mn[0] = px < mn[0] ? px : mn[0];
            mn[1] = py < mn[1] ? py : mn[1];
            mx[0] = px > px ? px : px;
            mx[1] = py > py ? py : py;
        }
        maxDepth = std::min(29, (int)std::lround(8 + 1.3f * std::log((float)nEl)));
        std::vector<int> all(nEl);
        std::iota(all.begin(), all.end(), 0);
        nodes.clear(); leafTris.clear();
        build_rec(all, mn, mx, 0, 0);
    }
    int build_rec(std::vector<int>& ids, const float mn[2], const float mx[2], int axis, int level) {
        if (level >= maxDepth || (int)ids.size() <= kLeafSize) {
            TreeNode leaf{2, 0, 0.f, (int)leafTris.size(), (int)ids.size()};
            leafTris.insert(leafTris.end(), ids.begin(), ids.end());
            nodes.push_back(leaf);
            return (int)nodes.size();
        }
        const float split = (mn[axis] + mx[axis]) * 0.5f;
        float lmx[2] = {mx[0], mx[1]}, rmn[2] = {mn[0], mn[1]};
        lmx[axis] = split;
        rmn[axis] = split;
        std::vector<int> L, Rr;
        for (int e : ids) {
            const float a = xy[2 * el[6 * e + 0] + axis], b = xy[2 * el[6 * e + 1] + axis], c = xy[2 * el[6 * e + 2] + axis];
            if (a <= split || b <= split || c <= split) L.push_back(e);
            if (a >= split || b >= split || c >= split) Rr.push_back(e);
        }
        std::vector<int>().swap(ids);
        const int self = (int)nodes.size();
        nodes.push_back(TreeNode{axis, 0, split, 0, 0});
        const int rightIndex = build_rec(L, mn, lmx, (axis + 1) % 2, level + 1);
        nodes[self].right = rightIndex;
        return build_rec(Rr, rmn, mx, (axis + 1) % 2, level + 1);
    }

    // isPointInTriagle (kd_tree_common.cuh:18-61): scaled barycentrics, CCW assumed
    static bool in_triangle(float px, float py, float ax, float ay, float bx, float by, float cx, float cy,
                            float& xi, float& eta) {
        const float abx = bx - ax, aby = by - ay, acx = cx - ax, acy = cy - ay, apx = px - ax, apy = py - ay;
        const float D = abx * acy - aby * acx;
        const float sgn = D > 0 ? 1.0f : -1.0f;
        const float s1 = (apx * acy - apy * acx) * sgn;
        if (s1 < 0 || s1 > D) return false;
        const float s2 = (apy * abx - apx * aby) * sgn;
        if (s2 < 0 || s1 > D - s2) return false;
        const float inv = 1.0f / std::fabs(D);
        xi = s1 * inv;
        eta = s2 * inv;
        return true;
    }

    void nn_leaf(float px, float py, const TreeNode& leaf, float& best, int& bestNode) const {
        for (int i = 0; i < leaf.count; ++i) {
            const int e = leafTris[leaf.offset + i];
            for (int j = 0; j < 6; ++j) {
                const int v = el[6 * e + j];
                const float dx = px - xy[2 * v], dy = py - xy[2 * v + 1];
                const float d = dx * dx + dy * dy;
                if (d < best) { best = d; bestNode = v; }
            }
        }
    }
    // near side first, far side only while the split plane is closer than the best distance so far
    void nn_rec(int idx, float px, float py, float& best, int& bestNode) const {
        const TreeNode& nd = nodes[idx];
        if (nd.axis == 2) { nn_leaf(px, py, nd, best, bestNode); return; }
        const float c = nd.axis == 0 ? px : py;
        const int nearC = c <= nd.split ? idx + 1 : nd.right;
        const int farC = c <= nd.split ? nd.right : idx + 1;
        nn_rec(nearC, px, py, best, bestNode);
        const float ds = (c - nd.split) * (c - nd.split);
        if (ds < best) nn_rec(farC, px, py, best, bestNode);
    }

    int find(float px, float py, float& xi, float& eta, int& nearest) const {
        int idx = 0;
        while (nodes[idx].axis != 2) {
            const TreeNode& nd = nodes[idx];
            const float c = nd.axis == 0 ? px : py;
            idx = c <= nd.split ? idx + 1 : nd.right;
        }
        const TreeNode& leaf = nodes[idx];
        for (int i = 0; i < leaf.count; ++i) {
            const int e = leafTris[leaf.offset + i];
            const int* t = el + 6 * e;
            if (in_triangle(px, py, xy[2 * t[0]], xy[2 * t[0] + 1], xy[2 * t[1]], xy[2 * t[1] + 1], xy[2 * t[2]],
                            xy[2 * t[2] + 1], xi, eta))
                return e;
        }
        float best = FLT_MAX;
        nearest = -1;
        nn_rec(0, px, py, best, nearest);
        return -1;
    }
};

// ------------------------------------------------------------------------------------------------
// The solver: matrices, BC data, fields and one operator-split step
// ------------------------------------------------------------------------------------------------
enum Slot { PRESSURE_STIFFNESS = 0, VELOCITY_MASS, DIFFUSION, VELOCITY_DIVERGENCE, PRESSURE_DIVERGENCE,
            VELOCITY_DIRICHLET_WEIGHTS, PRESSURE_DIRICHLET_WEIGHTS, SLOT_COUNT };

struct SolverBase {
    virtual ~SolverBase() = default;
    virtual const void* matrix(int slot, int& rows, int& cols, int64_t& nnz, const int64_t*& rowptr, const int*& col) = 0;
    virtual void matrix_values(int slot, double* out) = 0;
    virtual int cg(int slot, const double* b, const double* x0, double* x, int maxIt, double tol, int* it, double* rr) = 0;
    virtual void advect(const double* u, const double* v, double* uo, double* vo) = 0;
    virtual int step(int nsteps, int* iters) = 0;
    virtual void set_fields(const double* uv, const double* p) = 0;
    virtual void get_fields(double* uv, double* p) = 0;
    virtual void spmv(int slot, const double* x, double* y) = 0;
    virtual void set_tol(double t) = 0;
    virtual void set_bc(const double* u, const double* v, const double* p) = 0;
    virtual void set_scheme(int scheme) = 0;
    KDTree tree;
    std::vector<float> xy;
    std::vector<int> el;
    int Nv = 0, T = 0, P = 0;
};

template <typename R> struct Solver : SolverBase {
    R nu, dt;
    double tol = 1e-8;
    std::vector<int> uNodes, pNodes;          // Dirichlet occurrences in the reference's group order
    std::vector<R> gu, gv, gp;
    CSR<R> mats[SLOT_COUNT];
    std::vector<R> uv, p, tmp, rhsV, rhsP;

    Solver(int nNodes, const float* nodes, int nEl, const int* elements, int nP, int nU, const int* uN,
           const double* u_, const double* v_, int nPbc, const int* pN, const double* p_, double visc, double dt_) {
        Nv = nNodes; T = nEl; P = nP;
        xy.assign(nodes, nodes + 2 * (size_t)nNodes);
        el.assign(elements, elements + 6 * (size_t)nEl);
        nu = (R)visc; dt = (R)dt_;
        uNodes.assign(uN, uN + nU);
        for (int i = 0; i < nU; ++i) { gu.push_back((R)u_[i]); gv.push_back((R)v_[i]); }
        pNodes.assign(pN, pN + nPbc);
        for (int i = 0; i < nPbc; ++i) gp.push_back((R)p_[i]);
        tree.build(xy.data(), el.data(), Nv, T);
        assemble();
        uv.assign(2 * (size_t)Nv, R(0));
        p.assign(P, R(0));
        tmp.assign(2 * (size_t)Nv, R(0));
        rhsV.assign(2 * (size_t)Nv, R(0));
        rhsP.assign(P, R(0));
        impose_velocity(uv.data());
    }

    void element_xy(int e, R out[12]) const {
        for (int k = 0; k < 6; ++k) {
            const int v = el[6 * e + k];
            out[2 * k] = (R)xy[2 * v];
            out[2 * k + 1] = (R)xy[2 * v + 1];
        }
    }

    void assemble() {
        RefIntegrals<R> I;
        std::vector<char> uBC(Nv, 0), pBC(P, 0);
        for (int v : uNodes) uBC[v] = 1;
        for (int v : pNodes) pBC[v] = 1;
        // contiguous element ranges in parallel, one triplet part per range (see Triplets)
        const int parts = std::max(1, std::min(omp_get_max_threads(), T / 4096 + 1));
        Triplets<R> M(Nv, Nv, parts), D(Nv, Nv, parts), Wv(Nv, Nv, parts), Kp(P, P, parts), Wp(P, P, parts),
            Dv(P, 2 * Nv, parts), G(2 * Nv, P, parts);
        // exact sizes per part first (one allocation each instead of repeated growth)
#pragma omp parallel for schedule(static, 1) num_threads(parts)
        for (int part = 0; part < parts; ++part) {
            const int e0 = (int)((int64_t)T * part / parts), e1 = (int)((int64_t)T * (part + 1) / parts);
            size_t nD = 0, nW = 0, nK = 0, nWp = 0;
            for (int e = e0; e < e1; ++e) {
                const int* t = &el[6 * (size_t)e];
                int fu = 0, fp = 0;
                for (int i = 0; i < 6; ++i) fu += !uBC[t[i]];
                for (int i = 0; i < 3; ++i) fp += !pBC[t[i]];
                nD += (size_t)fu * fu;
                nW += (size_t)fu * (6 - fu);
                nK += (size_t)fp * fp;
                nWp += (size_t)fp * (3 - fp);
            }
            const size_t ne = (size_t)(e1 - e0);
            M.parts[part].reserve(36 * ne);
            D.parts[part].reserve(nD + (part == parts - 1 ? (size_t)Nv : 0));
            Wv.parts[part].reserve(nW);
            Kp.parts[part].reserve(nK + (part == parts - 1 ? (size_t)P : 0));
            Wp.parts[part].reserve(nWp);
            Dv.parts[part].reserve(36 * ne);
            G.parts[part].reserve(36 * ne);
        }
#pragma omp parallel for schedule(static, 1) num_threads(parts)
        for (int part = 0; part < parts; ++part)
        for (int e = (int)((int64_t)T * part / parts); e < (int)((int64_t)T * (part + 1) / parts); ++e) {
            const int* t = &el[6 * (size_t)e];
            R exy[12];
            element_xy(e, exy);
            // velocity mass (LocalMassFunctor) and diffusion = mass + stiffness * dt * nu
            const R jabs = std::abs(jacobian_det(exy));
            R mloc[6][6], kloc[6][6];
            for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) mloc[i][j] = I.mass[i][j] * jabs;
            local_stiffness<R, 6, 12>(exy, I.delP2, kloc);
            for (int i = 0; i < 6; ++i) {
                const bool rb = uBC[t[i]];
                for (int j = 0; j < 6; ++j) {
                    M.add(part, t[i], t[j], mloc[i][j]);
                    const R d = mloc[i][j] + kloc[i][j] * dt * nu;
                    const bool cb = uBC[t[j]];
                    if (!rb && !cb) D.add(part, t[i], t[j], d);
                    else if (!rb && cb) Wv.add(part, t[j], t[i], d);
                }
            }
            // pressure stiffness (P1) with pressure Dirichlet elimination
            R kp[3][3];
            local_stiffness<R, 3, 6>(exy, I.delP1, kp);
            for (int i = 0; i < 3; ++i) {
                const bool rb = pBC[t[i]];
                for (int j = 0; j < 3; ++j) {
                    const bool cb = pBC[t[j]];
                    if (!rb && !cb) Kp.add(part, t[i], t[j], kp[i][j]);
                    else if (!rb && cb) Wp.add(part, t[j], t[i], kp[i][j]);
                }
            }
            // divergence blocks (LocalDivergenceFunctor): B rows with the precomputed mixed integrals
            R det, B[2][2];
            diff_operator(exy, det, B);
            for (int pp = 0; pp < 3; ++pp)
                for (int q = 0; q < 6; ++q) {
                    const R dx = B[0][0] * I.divP1P2[pp][q] + B[0][1] * I.divP1P2[pp][q + 6];
                    const R dy = B[1][0] * I.divP1P2[pp][q] + B[1][1] * I.divP1P2[pp][q + 6];
                    Dv.add(part, t[pp], t[q], dx);
                    Dv.add(part, t[pp], t[q] + Nv, dy);
                }
            for (int q = 0; q < 6; ++q)
                for (int pp = 0; pp < 3; ++pp) {
                    const R dx = B[0][0] * I.divP2P1[q][pp] + B[0][1] * I.divP2P1[q][pp + 3];
                    const R dy = B[1][0] * I.divP2P1[q][pp] + B[1][1] * I.divP2P1[q][pp + 3];
                    G.add(part, t[q], t[pp], dx);
                    G.add(part, t[q] + Nv, t[pp], dy);
                }
        }
        // BC rows become identity rows, once per distinct BC node (the reference walks an unordered_set)
        for (int v = 0; v < Nv; ++v) if (uBC[v]) D.add(parts - 1, v, v, R(1));
        for (int v = 0; v < P; ++v) if (pBC[v]) Kp.add(parts - 1, v, v, R(1));
        mats[VELOCITY_MASS] = M.to_csr();
        mats[DIFFUSION] = D.to_csr();
        mats[VELOCITY_DIRICHLET_WEIGHTS] = Wv.to_csr();
        mats[PRESSURE_STIFFNESS] = Kp.to_csr();
        mats[PRESSURE_DIRICHLET_WEIGHTS] = Wp.to_csr();
        mats[VELOCITY_DIVERGENCE] = Dv.to_csr();
        mats[VELOCITY_DIVERGENCE].scale(-(R(1) / dt));
        mats[PRESSURE_DIVERGENCE] = G.to_csr();
        mats[PRESSURE_DIVERGENCE].scale(-dt);
    }

    const void* matrix(int slot, int& rows, int& cols, int64_t& nnz, const int64_t*& rowptr, const int*& col) override {
        const CSR<R>& m = mats[slot];
        rows = m.rows; cols = m.cols; nnz = m.nnz(); rowptr = m.rowptr.data(); col = m.col.data();
        return m.val.data();
    }
    void matrix_values(int slot, double* out) override {
        const CSR<R>& m = mats[slot];
        for (int64_t k = 0; k < m.nnz(); ++k) out[k] = (double)m.val[k];
    }
    void spmv(int slot, const double* x, double* y) override {
        const CSR<R>& m = mats[slot];
        std::vector<R> xx(x, x + m.cols), yy(m.rows);
        m.multiply(xx.data(), yy.data());
        for (int i = 0; i < m.rows; ++i) y[i] = (double)yy[i];
    }
    int cg(int slot, const double* b, const double* x0, double* x, int maxIt, double t, int* it, double* rr) override {
        const int n = mats[slot].rows;
        std::vector<R> bb(b, b + n), xx0(x0, x0 + n), xx(n);
        const int s = conjugate_gradient(mats[slot], bb.data(), xx0.data(), xx.data(), maxIt, t, it, rr);
        for (int i = 0; i < n; ++i) x[i] = (double)xx[i];
        return s;
    }

    // the velocity Dirichlet values at every listed occurrence (imposeVelocityDirichlet)
    void impose_velocity(R* w) const {
        for (size_t k = 0; k < uNodes.size(); ++k) { w[uNodes[k]] = gu[k]; w[uNodes[k] + Nv] = gv[k]; }
    }

    // semi-Lagrangian advection of both velocity channels (assembly.h:1664-1728)
    void advect_impl(const R* u, const R* v, R* uo, R* vo) const {
        const float fdt = (float)dt;
#pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < Nv; ++i) {
            const float sx = xy[2 * i] - (float)u[i] * fdt;
            const float sy = xy[2 * i + 1] - (float)v[i] * fdt;
            float xi = 0, eta = 0;
            int nearest = -1;
            const int e = tree.find(sx, sy, xi, eta, nearest);
            if (e > -1) {
                R N[6];
                p2_eval((R)xi, (R)eta, N);
                R su = 0, sv = 0;
                for (int k = 0; k < 6; ++k) {
                    const int nd = el[6 * (size_t)e + k];
                    su += N[k] * u[nd];
                    sv += N[k] * v[nd];
                }
                uo[i] = su; vo[i] = sv;
            } else {
                uo[i] = u[nearest]; vo[i] = v[nearest];
            }
        }
    }
    void advect(const double* u, const double* v, double* uo, double* vo) override {
        std::vector<R> a(u, u + Nv), b(v, v + Nv), c(Nv), d(Nv);
        advect_impl(a.data(), b.data(), c.data(), d.data());
        for (int i = 0; i < Nv; ++i) { uo[i] = (double)c[i]; vo[i] = (double)d[i]; }
    }

    void set_tol(double t) override { tol = t; }
    // replaces the Dirichlet values of every listed occurrence (time-dependent data: the caller evaluates them at
    // each step's time and calls this before the step); the lifts are formed from them inside each step
    void set_bc(const double* u_, const double* v_, const double* p_) override {
        for (size_t i = 0; i < gu.size(); ++i) { gu[i] = (R)u_[i]; gv[i] = (R)v_[i]; }
        for (size_t i = 0; i < gp.size(); ++i) gp[i] = (R)p_[i];
    }

    int solve(int slot, const R* b, const R* x0, R* x, int* it) {
        double rr;
        return conjugate_gradient(mats[slot], b, x0, x, -1, tol, it, &rr);
    }

    // one operator-split time step (assembly.h:1516-1556); iters[5] = diffusion u, v, pressure, mass u, v
    int one_step(int* iters) {
        int st = 0;
        R* u = uv.data();
        R* t = tmp.data();
        advect_impl(u, u + Nv, t, t + Nv);
        const CSR<R>& Wv = mats[VELOCITY_DIRICHLET_WEIGHTS];
        for (int ch = 0; ch < 2; ++ch) {   // diffusionSolve, U then V
            R* rhs = rhsV.data() + (size_t)ch * Nv;
            mats[VELOCITY_MASS].multiply(t + (size_t)ch * Nv, rhs);
            for (size_t k = 0; k < uNodes.size(); ++k) {
                const int nd = uNodes[k];
                const R g = ch == 0 ? gu[k] : gv[k];
                rhs[nd] = g;
                for (int64_t q = Wv.rowptr[nd]; q < Wv.rowptr[nd + 1]; ++q) rhs[Wv.col[q]] -= Wv.val[q] * g;
            }
            st |= solve(DIFFUSION, rhs, t + (size_t)ch * Nv, u + (size_t)ch * Nv, &iters[ch]);
        }
        // applyPressure
        mats[VELOCITY_DIVERGENCE].multiply(u, rhsP.data());
        const CSR<R>& Wp = mats[PRESSURE_DIRICHLET_WEIGHTS];
        for (size_t k = 0; k < pNodes.size(); ++k) {
            const int nd = pNodes[k];
            rhsP[nd] = gp[k];
            for (int64_t q = Wp.rowptr[nd]; q < Wp.rowptr[nd + 1]; ++q) rhsP[Wp.col[q]] -= Wp.val[q] * gp[k];
        }
        std::vector<R> pin(p);
        st |= solve(PRESSURE_STIFFNESS, rhsP.data(), pin.data(), p.data(), &iters[2]);
        mats[PRESSURE_DIVERGENCE].multiply(p.data(), rhsV.data());
        st |= solve(VELOCITY_MASS, rhsV.data(), u, t, &iters[3]);
        st |= solve(VELOCITY_MASS, rhsV.data() + Nv, u + Nv, t + Nv, &iters[4]);
#pragma omp parallel for
        for (int64_t i = 0; i < 2 * (int64_t)Nv; ++i) t[i] += u[i];
        impose_velocity(t);
        uv.swap(tmp);
        return st;
    }
    // One step of NavierStokesAssembly::solve (include/assembly.h:1137-1297), the explicit-convection scheme the
    // reference's driver never calls: rhs = -dt (C(u) + nu K) u from the element matrices (the loop at
    // :1151-1165 over the convection and the un-eliminated stiffness matrices, here element by element), the
    // tentative velocity M y = rhs from x0 = u per component, u += y, Dirichlet values; the pressure solve of
    // one_step; the correction M y = -dt Grad p from x0 = u, u += y.  iters[5] = tentative u, v, pressure,
    // correction u, v.
    int one_step_explicit(int* iters) {
        int st = 0;
        R* u = uv.data();
        R* t = tmp.data();
        const RefIntegrals<R> I;
        std::fill(rhsV.begin(), rhsV.end(), R(0));
        for (int e = 0; e < T; ++e) {
            R exy[12], vel[6][2], kloc[6][6], cloc[6][6];
            element_xy(e, exy);
            const int* en = el.data() + 6 * (size_t)e;
            for (int m = 0; m < 6; ++m) { vel[m][0] = u[en[m]]; vel[m][1] = u[en[m] + Nv]; }
            local_stiffness<R, 6, 12>(exy, I.delP2, kloc);
            local_convection(exy, vel, cloc);
            for (int i = 0; i < 6; ++i)
                for (int j = 0; j < 6; ++j) {
                    const R part = -dt * (cloc[i][j] + nu * kloc[i][j]);
                    rhsV[en[i]] += part * vel[j][0];
                    rhsV[en[i] + Nv] += part * vel[j][1];
                }
        }
        for (int ch = 0; ch < 2; ++ch) {
            const size_t o = (size_t)ch * Nv;
            st |= solve(VELOCITY_MASS, rhsV.data() + o, u + o, t + o, &iters[ch]);
            for (int i = 0; i < Nv; ++i) u[o + i] += t[o + i];
        }
        impose_velocity(u);
        mats[VELOCITY_DIVERGENCE].multiply(u, rhsP.data());
        const CSR<R>& Wp = mats[PRESSURE_DIRICHLET_WEIGHTS];
        for (size_t k = 0; k < pNodes.size(); ++k) {
            const int nd = pNodes[k];
            rhsP[nd] = gp[k];
            for (int64_t q = Wp.rowptr[nd]; q < Wp.rowptr[nd + 1]; ++q) rhsP[Wp.col[q]] -= Wp.val[q] * gp[k];
        }
        std::vector<R> pin(p);
        st |= solve(PRESSURE_STIFFNESS, rhsP.data(), pin.data(), p.data(), &iters[2]);
        mats[PRESSURE_DIVERGENCE].multiply(p.data(), rhsV.data());
        for (int ch = 0; ch < 2; ++ch) {
            const size_t o = (size_t)ch * Nv;
            st |= solve(VELOCITY_MASS, rhsV.data() + o, u + o, t + o, &iters[3 + ch]);
            for (int i = 0; i < Nv; ++i) u[o + i] += t[o + i];
        }
        return st;
    }
    int scheme = 0;   // 0: semiLagrangianSolve, 1: solve (explicit convection)
    void set_scheme(int s_) override { scheme = s_; }
    int step(int nsteps, int* iters) override {
        int st = 0;
        for (int s = 0; s < nsteps; ++s) st |= scheme == 1 ? one_step_explicit(iters + 5 * s) : one_step(iters + 5 * s);
        return st;
    }
    void set_fields(const double* w, const double* pp) override {
        for (size_t i = 0; i < uv.size(); ++i) uv[i] = (R)w[i];
        for (int i = 0; i < P; ++i) p[i] = (R)pp[i];
    }
    void get_fields(double* w, double* pp) override {
        for (size_t i = 0; i < uv.size(); ++i) w[i] = (double)uv[i];
        for (int i = 0; i < P; ++i) pp[i] = (double)p[i];
    }
};

}  // namespace oracle

using namespace oracle;

namespace oracle {
// Local element matrices of `n` triangles (vertices x0 y0 x1 y1 x2 y2 each), computed the way assemble() computes
// them, in float (realBits 32, the reference's arithmetic) or double; same layouts as the reference build's
// ref_local_matrices (oracle/ref_assembly_shim.cpp), which pins them.
template <typename R>
static void local_matrices(int n, const float* v, double* mass, double* stiffV, double* stiffP, double* divVx,
                           double* divVy, double* divPx, double* divPy) {
    RefIntegrals<R> I;
    for (int e = 0; e < n; ++e) {
        R exy[12] = {};
        for (int k = 0; k < 6; ++k) exy[k] = (R)v[6 * e + k];
        const R jabs = std::abs(jacobian_det(exy));
        R kloc[6][6], kp[3][3];
        local_stiffness<R, 6, 12>(exy, I.delP2, kloc);
        local_stiffness<R, 3, 6>(exy, I.delP1, kp);
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                mass[36 * e + 6 * i + j] = (double)(I.mass[i][j] * jabs);
                stiffV[36 * e + 6 * i + j] = (double)kloc[i][j];
            }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) stiffP[9 * e + 3 * i + j] = (double)kp[i][j];
        R det, B[2][2];
        diff_operator(exy, det, B);
        for (int pp = 0; pp < 3; ++pp)
            for (int q = 0; q < 6; ++q) {
                divVx[18 * e + 6 * pp + q] = (double)(B[0][0] * I.divP1P2[pp][q] + B[0][1] * I.divP1P2[pp][q + 6]);
                divVy[18 * e + 6 * pp + q] = (double)(B[1][0] * I.divP1P2[pp][q] + B[1][1] * I.divP1P2[pp][q + 6]);
            }
        for (int q = 0; q < 6; ++q)
            for (int pp = 0; pp < 3; ++pp) {
                divPx[18 * e + 3 * q + pp] = (double)(B[0][0] * I.divP2P1[q][pp] + B[0][1] * I.divP2P1[q][pp + 3]);
                divPy[18 * e + 3 * q + pp] = (double)(B[1][0] * I.divP2P1[q][pp] + B[1][1] * I.divP2P1[q][pp + 3]);
            }
    }
}
}  // namespace oracle

extern "C" {

// realBits: 64 -> FP64 oracle, 32 -> the reference's FP32 arithmetic.
void* orc_create(int nNodes, const float* nodes, int nEl, const int* elements, int nP, int nU, const int* uNodes,
                 const double* gu, const double* gv, int nPbc, const int* pNodes, const double* gp, double viscosity,
                 double dt, int realBits) {
    if (realBits == 32)
        return new Solver<float>(nNodes, nodes, nEl, elements, nP, nU, uNodes, gu, gv, nPbc, pNodes, gp, viscosity, dt);
    return new Solver<double>(nNodes, nodes, nEl, elements, nP, nU, uNodes, gu, gv, nPbc, pNodes, gp, viscosity, dt);
}
void orc_destroy(void* h) { delete (SolverBase*)h; }
void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int orc_max_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void orc_matrix_shape(void* h, int slot, int* rows, int* cols, int64_t* nnz) {
    const int64_t* rp; const int* c;
    ((SolverBase*)h)->matrix(slot, *rows, *cols, *nnz, rp, c);
}
void orc_matrix_get(void* h, int slot, int64_t* rowptr, int* col, double* val) {
    int rows, cols; int64_t nnz; const int64_t* rp; const int* c;
    SolverBase* s = (SolverBase*)h;
    s->matrix(slot, rows, cols, nnz, rp, c);
    std::memcpy(rowptr, rp, sizeof(int64_t) * (rows + 1));
    std::memcpy(col, c, sizeof(int) * nnz);
    s->matrix_values(slot, val);
}
void orc_spmv(void* h, int slot, const double* x, double* y) { ((SolverBase*)h)->spmv(slot, x, y); }
int orc_cg(void* h, int slot, const double* b, const double* x0, double* x, int maxIt, double tol, int* iters,
           double* relres) {
    return ((SolverBase*)h)->cg(slot, b, x0, x, maxIt, tol, iters, relres);
}
void orc_locate(void* h, int n, const float* pts, int* elem, float* xi, float* eta, int* nearest) {
    SolverBase* s = (SolverBase*)h;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) {
        float a = 0, b = 0;
        int nn = -1;
        elem[i] = s->tree.find(pts[2 * i], pts[2 * i + 1], a, b, nn);
        xi[i] = a; eta[i] = b;
        nearest[i] = elem[i] >= 0 ? -1 : nn;
    }
}
int orc_tree_size(void* h, int* nNodes, int* nLeafTris, int* maxDepth) {
    SolverBase* s = (SolverBase*)h;
    *nNodes = (int)s->tree.nodes.size();
    *nLeafTris = (int)s->tree.leafTris.size();
    *maxDepth = s->tree.maxDepth;
    return 0;
}
void orc_local_matrices(int realBits, int n, const float* v, double* mass, double* stiffV, double* stiffP,
                        double* divVx, double* divVy, double* divPx, double* divPy) {
    if (realBits == 32) oracle::local_matrices<float>(n, v, mass, stiffV, stiffP, divVx, divVy, divPx, divPy);
    else oracle::local_matrices<double>(n, v, mass, stiffV, stiffP, divVx, divVy, divPx, divPy);
}

// The ported tree alone (no assembly), for point-location checks on large meshes.
struct TreeOnly {
    std::vector<float> xy;
    std::vector<int> el;
    KDTree tree;
};
void* orc_tree_create(int nNodes, const float* nodes, int nEl, const int* elements) {
    TreeOnly* t = new TreeOnly;
    t->xy.assign(nodes, nodes + 2 * (size_t)nNodes);
    t->el.assign(elements, elements + 6 * (size_t)nEl);
    t->tree.build(t->xy.data(), t->el.data(), nNodes, nEl);
    return t;
}
void orc_tree_destroy(void* h) { delete (TreeOnly*)h; }
void orc_tree_locate(void* h, int n, const float* pts, int* elem, float* xi, float* eta, int* nearest) {
    const KDTree& tree = ((TreeOnly*)h)->tree;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) {
        float a = 0, b = 0;
        int nn = -1;
        elem[i] = tree.find(pts[2 * i], pts[2 * i + 1], a, b, nn);
        xi[i] = a; eta[i] = b;
        nearest[i] = elem[i] >= 0 ? -1 : nn;
    }
}
// leaf entries (the reference's leafTriangleIndexes length: its largest leaf offset is below it) and tree depth
void orc_tree_stats(void* h, int64_t* nodes, int64_t* leafEntries, int* maxDepth) {
    const KDTree& tree = ((TreeOnly*)h)->tree;
    *nodes = (int64_t)tree.nodes.size();
    *leafEntries = (int64_t)tree.leafTris.size();
    *maxDepth = tree.maxDepth;
}
void orc_advect(void* h, const double* u, const double* v, double* uo, double* vo) { ((SolverBase*)h)->advect(u, v, uo, vo); }
int orc_step(void* h, int nsteps, int* iters) { return ((SolverBase*)h)->step(nsteps, iters); }
void orc_set_tolerance(void* h, double tol) { ((SolverBase*)h)->set_tol(tol); }
void orc_set_bc(void* h, const double* u, const double* v, const double* p) { ((SolverBase*)h)->set_bc(u, v, p); }
void orc_set_scheme(void* h, int scheme) { ((SolverBase*)h)->set_scheme(scheme); }
// The oracle's local convection matrices of `n` triangles (vertices x0 y0 .. x2 y2, velocities u0..u5 v0..v5), in
// float (realBits 32, the reference's arithmetic) or double; row-major 6 x 6 per triangle.
void orc_local_convection(int realBits, int n, const float* v, const double* vel, double* out) {
    for (int e = 0; e < n; ++e) {
        if (realBits == 32) {
            float xy[12] = {}, u[6][2], c[6][6];
            for (int k = 0; k < 6; ++k) xy[k] = v[6 * e + k];
            for (int k = 0; k < 6; ++k) { u[k][0] = (float)vel[12 * e + k]; u[k][1] = (float)vel[12 * e + 6 + k]; }
            local_convection(xy, u, c);
            for (int k = 0; k < 36; ++k) out[36 * e + k] = c[k / 6][k % 6];
        } else {
            double xy[12] = {}, u[6][2], c[6][6];
            for (int k = 0; k < 6; ++k) xy[k] = v[6 * e + k];
            for (int k = 0; k < 6; ++k) { u[k][0] = vel[12 * e + k]; u[k][1] = vel[12 * e + 6 + k]; }
            local_convection(xy, u, c);
            for (int k = 0; k < 36; ++k) out[36 * e + k] = c[k / 6][k % 6];
        }
    }
}
void orc_set_fields(void* h, const double* uv, const double* p) { ((SolverBase*)h)->set_fields(uv, p); }
void orc_get_fields(void* h, double* uv, double* p) { ((SolverBase*)h)->get_fields(uv, p); }

// standalone predicate, for known-answer tests of the containment test itself
int orc_point_in_triangle(const float* pabc, float* xi, float* eta) {
    return KDTree::in_triangle(pabc[0], pabc[1], pabc[2], pabc[3], pabc[4], pabc[5], pabc[6], pabc[7], *xi, *eta) ? 1 : 0;
}

}  // extern "C"
