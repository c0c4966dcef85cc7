// The C ABI (include/nsfem_gb300.h): device handle, matrix upload, solves, point location, advection and the
// resident operator-split step.  See the header for the reference interface each entry point replaces.
#include "nsf_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <map>
#include <numeric>
#include <stdexcept>

using namespace nsf;

namespace nsf {

// Validates and uploads a mesh, then builds its point-location tree.
void upload_mesh_into(MeshDev& m, cudaStream_t s, int nNodes, const float* xy, int nElements, const int* elements,
                      int nPressure) {
    if (nNodes <= 0 || nElements <= 0 || !xy || !elements) throw bad_arg("empty mesh");
    if (nPressure <= 0 || nPressure > nNodes) throw bad_arg("pressure node count out of range");
    for (int64_t k = 0; k < (int64_t)6 * nElements; ++k)
        if (elements[k] < 0 || elements[k] >= nNodes) throw bad_arg("element references a node out of range");
    for (int64_t k = 0; k < (int64_t)2 * nNodes; ++k)
        if (!std::isfinite(xy[k])) throw bad_arg("non-finite node coordinate");
    m.nNodes = nNodes;
    m.nEl = nElements;
    m.nP = nPressure;
    m.hxy.assign(xy, xy + 2 * (size_t)nNodes);
    m.hel.assign(elements, elements + 6 * (size_t)nElements);
    m.xy.upload((const float2*)xy, nNodes, s);
    m.el.upload(elements, 6 * (size_t)nElements, s);
    tree_build(m, s);
}

void setup_instance(MeshDev& m, SimState& S, Csr* mats, cudaStream_t s, int nNodes, const float* xy, int nElements,
                    const int* elements, int nPressure, int nVelocityBC, const int* velocityBCNodes, const double* bcU,
                    const double* bcV, int nPressureBC, const int* pressureBCNodes, const double* bcP, double viscosity,
                    double dt) {
    if (!(dt > 0) || !(viscosity >= 0)) throw bad_arg("dt must be positive and viscosity non-negative");
    if (nVelocityBC < 0 || nPressureBC < 0) throw bad_arg("negative boundary count");
    if ((nVelocityBC > 0 && (!velocityBCNodes || !bcU || !bcV)) || (nPressureBC > 0 && (!pressureBCNodes || !bcP)))
        throw bad_arg("null boundary array");
    upload_mesh_into(m, s, nNodes, xy, nElements, elements, nPressure);
    S.ready = false;
    S.viscosity = viscosity;
    S.dt = dt;
    S.t0 = 0;
    S.steps = 0;
    S.bcTimeDependent = false;
    S.nBcNodeV = S.nBcNodeP = 0;
    S.scheme = NSF_SCHEME_SEMI_LAGRANGIAN;
    S.hOccV.assign(velocityBCNodes, velocityBCNodes + nVelocityBC);
    S.hOccP.assign(pressureBCNodes, pressureBCNodes + nPressureBC);
    const int Nv = nNodes, P = nPressure;
    // Dirichlet data: mask, imposed value (last listed occurrence) and lift weight (sum over occurrences,
    // because the reference subtracts the lift once per listed occurrence, include/assembly.h:505-523)
    S.hbcV.assign(Nv, 0);
    S.hbcP.assign(P, 0);
    std::vector<double> gset[2] = {std::vector<double>(Nv, 0.0), std::vector<double>(Nv, 0.0)};
    std::vector<double> glift[2] = {std::vector<double>(Nv, 0.0), std::vector<double>(Nv, 0.0)};
    std::vector<double> gsetP(P, 0.0), gliftP(P, 0.0);
    for (int k = 0; k < nVelocityBC; ++k) {
        const int nd = velocityBCNodes[k];
        if (nd < 0 || nd >= Nv) throw bad_arg("velocity Dirichlet node out of range");
        S.hbcV[nd] = 1;
        gset[0][nd] = bcU[k];
        gset[1][nd] = bcV[k];
        glift[0][nd] += bcU[k];
        glift[1][nd] += bcV[k];
    }
    for (int k = 0; k < nPressureBC; ++k) {
        const int nd = pressureBCNodes[k];
        if (nd < 0 || nd >= P) throw bad_arg("pressure Dirichlet node out of range");
        S.hbcP[nd] = 1;
        gsetP[nd] = bcP[k];
        gliftP[nd] += bcP[k];
    }
    S.bcV.upload(S.hbcV.data(), Nv, s);
    S.bcP.upload(S.hbcP.data(), P, s);
    for (int ch = 0; ch < 2; ++ch) {
        S.hgV[ch] = gset[ch];
        S.gV[ch].upload(gset[ch].data(), Nv, s);
    }
    S.hgP = gsetP;
    S.gP.upload(gsetP.data(), P, s);
    S.nColours = assemble_instance(m, S, mats, s, viscosity, dt);
    // constant lift vectors: lift = W g (the Dirichlet data do not depend on time: the expressions see x, y only)
    DevBuf<double> g;
    for (int ch = 0; ch < 2; ++ch) {
        g.upload(glift[ch].data(), Nv, s);
        S.liftV[ch].alloc(Nv);
        spmv_launch(mats[NSF_VELOCITY_LIFT], g.get(), S.liftV[ch].get(), s);
        NSF_CUDA(cudaStreamSynchronize(s));
    }
    g.upload(gliftP.data(), P, s);
    S.liftP.alloc(P);
    spmv_launch(mats[NSF_PRESSURE_LIFT], g.get(), S.liftP.get(), s);
    NSF_CUDA(cudaStreamSynchronize(s));
    // fields: u = 0 with Dirichlet values (imposeVelocityDirichlet), p = 0
    std::vector<double> uv0(2 * (size_t)Nv, 0.0);
    for (int k = 0; k < nVelocityBC; ++k) {
        uv0[velocityBCNodes[k]] = bcU[k];
        uv0[velocityBCNodes[k] + (size_t)Nv] = bcV[k];
    }
    S.uv.upload(uv0.data(), uv0.size(), s);
    S.tmp.alloc(2 * (size_t)Nv);
    S.tmp.zero(s);
    S.rhsV.alloc(2 * (size_t)Nv);
    S.rhsP.alloc(P);
    S.p.alloc(P);
    S.p.zero(s);
    NSF_CUDA(cudaStreamSynchronize(s));
}

Factor& factor_for(nsf_device* h, int slot, bool needValues) {
    if (slot < 0 || slot >= NSF_SLOT_COUNT) throw bad_arg("matrix slot out of range");
    Factor& F = h->factors[slot];
    const Csr& A = h->mats[slot];
    if (!A.valid()) throw Error{NSF_ERR_STATE, "matrix slot " + std::to_string(slot) + " is empty"};
    if (F.rows != A.rows || !F.lRowptr.get()) factor_structure(F, A, h->stream);
    if (needValues && !F.ready) throw Error{NSF_ERR_STATE, "slot " + std::to_string(slot) + " has no factor values"};
    return F;
}

// ---- host buffers that the GPU's own kernels copy ---------------------------------------------------------
// On a coherent CPU-GPU link (Grace), copy-engine transfers that follow a stretch of GPU work are slow: right after
// a step of the 2048 cavity, 12-24 ms device to host and 7-17 ms host to device for its 302 MB of fields, against
// 1.7 ms for a copy kernel in either direction, and 1.6 ms for the copy engine once warm.  Page-locked buffers
// from nsf_host_alloc are mapped for the device and zeroed by a kernel when they are allocated (the first kernel
// access to host pages is slow, so it happens there), and the field transfers to and from them run as copy
// kernels; other host pointers go through cudaMemcpyAsync.
struct HostBlock {
    size_t bytes;
    char* dev;   // its device address
};
std::mutex g_hostMu;
std::map<uintptr_t, HostBlock> g_hostBlocks;   // by host address

// The device address of [p, p + bytes) when it lies inside one block from nsf_host_alloc, else null.
void* host_block_device(const void* p, size_t bytes) {
    std::lock_guard<std::mutex> lk(g_hostMu);
    const uintptr_t a = (uintptr_t)p;
    auto it = g_hostBlocks.upper_bound(a);
    if (it == g_hostBlocks.begin()) return nullptr;
    --it;
    if (a + bytes > it->first + it->second.bytes) return nullptr;
    return it->second.dev + (a - it->first);
}

// dst[0, bytes) = src[0, bytes) (src null: zeros), 16-byte words when both addresses and the size allow it, four
// of them in flight per thread
__global__ void copy_bytes_kernel(char* __restrict__ dst, const char* __restrict__ src, size_t bytes) {
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (size_t)gridDim.x * blockDim.x;
    if ((((uintptr_t)dst | (uintptr_t)src | bytes) & 15) == 0) {
        int4* d = reinterpret_cast<int4*>(dst);
        const int4* s = reinterpret_cast<const int4*>(src);
        const size_t n = bytes / 16;
        for (size_t i0 = tid; i0 < n; i0 += 4 * nt) {
            int4 v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const size_t i = i0 + u * nt;
                v[u] = i < n && s ? s[i] : make_int4(0, 0, 0, 0);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const size_t i = i0 + u * nt;
                if (i < n) d[i] = v[u];
            }
        }
    } else {
        for (size_t i = tid; i < bytes; i += nt) dst[i] = src ? src[i] : 0;
    }
}

void copy_kernel_launch(nsf_device* h, void* dst, const void* src, size_t bytes) {
    copy_bytes_kernel<<<h->smCount * 4, 256, 0, h->stream>>>(static_cast<char*>(dst), static_cast<const char*>(src),
                                                            bytes);
    NSF_CUDA(cudaGetLastError());
    count_launch();
}

// A field transfer between the device and the host on the handle's stream (see HostBlock).
void field_copy(nsf_device* h, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
    if (bytes == 0) return;
    const bool toDevice = kind == cudaMemcpyHostToDevice;
    void* mapped = host_block_device(toDevice ? src : dst, bytes);
    if (mapped) copy_kernel_launch(h, toDevice ? dst : mapped, toDevice ? mapped : src, bytes);
    else NSF_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, h->stream));
}

}  // namespace nsf

std::atomic<long long> nsf::g_launches{0};

#define NSF_BEGIN(h)                                 \
    if (!(h)) return NSF_ERR_BAD_ARG;                   \
    std::lock_guard<std::recursive_mutex> lk_((h)->mu); \
    try {                                               \
        NSF_CUDA(cudaSetDevice((h)->device));

#define NSF_END(h)                                      \
    }                                                   \
    catch (const nsf::Error& e) {                       \
        (h)->lastError = e.msg;                         \
        return e.status;                                \
    }                                                   \
    catch (const std::exception& e) {                   \
        (h)->lastError = e.what();                      \
        return NSF_ERR_CUDA;                            \
    }                                                   \
    (h)->lastError.clear();                             \
    return NSF_OK;

namespace {

DevBuf<double>& scratch(nsf_device* h, int which) { return h->scratch[which]; }

void check_slot(int slot) {
    if (slot < 0 || slot >= NSF_SLOT_COUNT) throw bad_arg("matrix slot out of range");
}

const char* status_text(int st) {
    switch (st) {
        case NSF_OK: return "ok";
        case NSF_ERR_NOT_CONVERGED: return "Max iterations reached!";
        case NSF_ERR_BREAKDOWN: return "CG breakdown (matrix not SPD or non-finite values)";
        case NSF_ERR_BARRIER_TIMEOUT: return "grid barrier wait timed out";
        default: return "error";
    }
}

void ensure_workspace(nsf_device* h, int rows) {
    CgWorkspace& ws = h->ws;
    ws.r.ensure(rows);
    ws.q.ensure(rows);
    ws.p0.ensure(rows);
    ws.p1.ensure(rows);
    ws.r32.ensure(rows);
    ws.r32b.ensure(rows);
    ws.d32.ensure(rows);
    ws.q32.ensure(rows);
    ws.p32a.ensure(rows);
    ws.p32b.ensure(rows);
    ws.w.ensure(rows);
    ws.w32.ensure(rows);
    ws.xp.ensure(rows);
    ws.bp.ensure(rows);
}

cudaEvent_t pool_event(nsf_device* h) {
    if (h->evUsed == h->evPool.size()) {
        cudaEvent_t e;
        NSF_CUDA(cudaEventCreate(&e));
        h->evPool.push_back(e);
    }
    return h->evPool[h->evUsed++];
}

// The plain FP64 CG form for a system: pipelined (one grid barrier per iteration) where the barriers are a
// measurable share of an iteration, the three-barrier form on large systems, where the pipelined form's two extra
// vector passes and extra FP64 operations per row cost more than two barriers.
bool use_pipelined_cg(const nsf_device* h, const Csr& S) {
    if (!h->ws.pipeOk || !S.sellStart.get()) return false;
    if (h->cgForm == NSF_CG_FORM_PIPELINED) return true;
    if (h->cgForm == NSF_CG_FORM_THREE_SYNC) return false;
    return S.rows < NSF_CG_PIPELINED_MAX_ROWS;
}

// The reduced (Schur complement) iteration of the split mixed PCG (NSF_PCG_FORM_AUTO and _REDUCED): two colours,
// a SELL copy and the 1024-thread inner grid.
bool use_reduced_pcg(const nsf_device* h, const Csr& S, const FactorView& f) {
    if (h->pcgForm == NSF_PCG_FORM_FULL) return false;
    return f.colours == 2 && S.sellStart.get() && h->ws.gridInner1024 > 0 && f.aDiag && f.aInv32;
}

// Launch one persistent solve; returns the index of its CgInfo slot.
int launch_solve(nsf_device* h, int slot, int mode, const double* b, const double* x0, double* x, int maxIt,
                 double tol, const CgArgs* fused) {
    Csr& A = h->mats[slot];
    if (!A.valid()) throw Error{NSF_ERR_STATE, "matrix slot " + std::to_string(slot) + " is empty"};
    if (A.rows != A.cols) throw bad_arg("CG needs a square matrix");
    const bool pcg = mode == NSF_SOLVER_PCG_MIXED || mode == NSF_SOLVER_PCG_FP64;
    if (pcg && (!h->factors[slot].ready || h->factors[slot].rows != A.rows))
        mode = mode == NSF_SOLVER_PCG_MIXED ? NSF_SOLVER_MIXED : NSF_SOLVER_FP64;   // no factor: plain CG
    const bool precond = mode == NSF_SOLVER_PCG_MIXED || mode == NSF_SOLVER_PCG_FP64;
    // a preconditioned solve runs on the factor's colour-permuted copy of the matrix
    Csr& S = precond ? h->factors[slot].Ap : A;
    prepare_matrix(S, mode == NSF_SOLVER_MIXED || mode == NSF_SOLVER_PCG_MIXED, h->stream);
    if (mode == NSF_SOLVER_PCG_MIXED) prepare_col16(S, h->stream);   // the inner iterations' narrow product
    ensure_workspace(h, S.rows);
    CgWorkspace& ws = h->ws;
    const int infoIndex = h->infoCursor;
    h->infoCursor = (h->infoCursor + 1) % (int)ws.info.n;
    CgArgs a{};
    if (fused) a = *fused;
    a.n = S.rows;
    a.rowptr = S.rowptr.get();
    a.col = S.col.get();
    a.val = S.val.get();
    a.val32 = S.val32.get();
    a.rowsum32 = S.rowsum32.get();
    a.sellStart = S.sellStart.get();
    a.sellCol = S.sellCol.get();
    a.sellCol16 = S.hasCol16 ? S.sellCol16.get() : nullptr;
    a.sellColBase = S.hasCol16 ? S.sellColBase.get() : nullptr;
    a.sellVal = S.sellVal.get();
    a.sellVal32 = S.sellVal32.get();
    a.sellMaxW = S.maxWidth;
    a.b = b;
    a.x0 = x0;
    a.x = x;
    a.r = ws.r.get();
    a.q = ws.q.get();
    a.pbuf0 = ws.p0.get();
    a.pbuf1 = ws.p1.get();
    a.r32 = ws.r32.get();
    a.r32b = ws.r32b.get();
    a.d32 = ws.d32.get();
    a.q32 = ws.q32.get();
    a.p32a = ws.p32a.get();
    a.p32b = ws.p32b.get();
    a.partials = ws.partials.get();
    a.sync = ws.sync.get();
    a.info = ws.info.get() + infoIndex;
    a.maxIt = maxIt < 0 ? A.rows : maxIt;
    if (precond) {
        a.f = factor_view(h->factors[slot], ws);
        a.f.natB = b;          // the solve itself runs on the permuted copies
        a.f.natX0 = x0;
        a.f.natX = x;
        a.b = ws.bp.get();
        a.x0 = ws.xp.get();
        a.x = ws.xp.get();
        // over the cap (the plain method's count) the solve falls back to plain FP64 CG with the caller's own
        // budget; when the caller's budget is the tighter limit there is no fallback
        const int cap = h->pcgCap[slot] > 0 ? h->pcgCap[slot] : A.rows;
        a.fallbackMaxIt = cap < a.maxIt ? a.maxIt : 0;
        a.maxIt = std::min(a.maxIt, cap);
    }
    if ((size_t)infoIndex >= h->infoMode.size()) h->infoMode.resize(ws.info.n, 0);
    h->infoMode[infoIndex] = mode;
    a.tol2 = tol * tol;
    a.innerTol2 = h->innerTol * h->innerTol;
    a.maxOuter = 64;
    a.timeoutNs = h->timeoutNs;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (h->profile) {
        e0 = pool_event(h);
        e1 = pool_event(h);
        NSF_CUDA(cudaEventRecord(e0, h->stream));
    }
    const bool wide = S.maxWidth > kSellChunk;
    if (mode == NSF_SOLVER_PCG_MIXED && !wide) {
        a.f.reduced = use_reduced_pcg(h, S, a.f) ? 1 : 0;
        // the Schur complement formed explicitly (once per factor) where its 16-bit copy fits
        if (a.f.reduced && h->pcgForm != NSF_PCG_FORM_REDUCED && factor_schur(h->factors[slot], h->stream)) {
            const FactorView v = factor_view(h->factors[slot], ws);
            a.f.schur = 1;
            a.f.sMaxW = v.sMaxW;
            a.f.sStart = v.sStart;
            a.f.sCol16 = v.sCol16;
            a.f.sColBase = v.sColBase;
            a.f.sVal32 = v.sVal32;
            a.f.sRowsum32 = v.sRowsum32;
        }
        h->innerForm[slot] = pcg_mixed_split_launch(ws, a, h->stream);
    }
    else if (mode == NSF_SOLVER_MIXED && wide)
        cg_mixed_split_launch(ws, a, h->stream);
    else if (mode == NSF_SOLVER_FP64 && h->cgForm == NSF_CG_FORM_MULTI_KERNEL)
        cg_multi_launch(ws, a, wide, h->stream);
    else if (mode == NSF_SOLVER_FP64 && use_pipelined_cg(h, S))
        cg_pipe_launch(ws, a, wide, h->stream);
    else
        cg_launch(ws, a, mode, wide, h->stream);
    if (h->profile) {
        NSF_CUDA(cudaEventRecord(e1, h->stream));
        h->records.push_back({slot, mode, A.rows, A.nnz, e0, e1, infoIndex});
    }
    return infoIndex;
}

CgInfo read_info(nsf_device* h, int index) {
    CgInfo info;
    NSF_CUDA(cudaMemcpyAsync(&info, h->ws.info.get() + index, sizeof(CgInfo), cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    return info;
}

void throw_solve_status(const CgInfo& info, const std::string& what) {
    if (info.status != NSF_OK)
        throw Error{info.status, what + ": " + status_text(info.status) + " after " + std::to_string(info.iterations) +
                                     " iterations"};
}

void upload_csr(nsf_device* h, int slot, int rows, int cols, int64_t nnz, const int* rowptr, const int* col,
                const double* val) {
    check_slot(slot);
    if (rows <= 0 || cols <= 0 || nnz < 0) throw bad_arg("matrix dimensions must be positive");
    if (nnz > INT32_MAX) throw bad_arg("matrix has more than 2^31-1 non-zeros");
    if (rowptr[0] != 0 || rowptr[rows] != nnz) throw bad_arg("row pointers do not span [0, nnz]");
    for (int r = 0; r < rows; ++r) {
        if (rowptr[r + 1] < rowptr[r]) throw bad_arg("row pointers decrease");
        for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) {
            if (col[k] < 0 || col[k] >= cols) throw bad_arg("column index out of range");
            if (k > rowptr[r] && col[k] <= col[k - 1]) throw bad_arg("columns must ascend within a row");
        }
    }
    Csr& A = h->mats[slot];
    A.rows = rows;
    A.cols = cols;
    A.nnz = nnz;
    A.rowptr.upload(rowptr, rows + 1, h->stream);
    A.col.upload(col, std::max<int64_t>(nnz, 0), h->stream);
    A.val.upload(val, std::max<int64_t>(nnz, 0), h->stream);
    A.values_changed();
    h->factors[slot] = Factor();
    h->pcgOff[slot] = false;
    NSF_CUDA(cudaStreamSynchronize(h->stream));
}

void sim_require(nsf_device* h) {
    if (!h->sim.ready) throw Error{NSF_ERR_STATE, "nsf_sim_setup has not been called"};
}

// Launches one operator-split step on the resident fields; `infos` receives 5 info indices.
void sim_step_launch(nsf_device* h, int infos[5]) {
    SimState& S = h->sim;
    MeshDev& m = h->mesh;
    const int Nv = m.nNodes;
    // mixed precision per system, unless that system already had to finish in FP64 (see run_steps)
    auto mode = [&](int slot) {
        const bool pre = (h->solverMode == NSF_SOLVER_PCG_MIXED || h->solverMode == NSF_SOLVER_PCG_FP64) &&
                         h->factors[slot].ready && !h->pcgOff[slot];
        const bool mixed = (h->solverMode == NSF_SOLVER_MIXED || h->solverMode == NSF_SOLVER_PCG_MIXED) &&
                           !h->mixedOff[slot];
        if (pre) return mixed ? NSF_SOLVER_PCG_MIXED : NSF_SOLVER_PCG_FP64;
        return mixed ? NSF_SOLVER_MIXED : NSF_SOLVER_FP64;
    };
    cudaStream_t s = h->stream;
    double* uv = S.uv.get();
    double* tmp = S.tmp.get();
    // time-dependent Dirichlet data at the time this step ends
    ++S.steps;
    if (S.bcTimeDependent) bc_update_launch(S, m, h->mats, S.t0 + (double)S.steps * S.dt, s);
    // advection (include/assembly.h:1519-1524)
    advect_launch(m, S.dt, uv, uv + Nv, tmp, tmp + Nv, s);
    // diffusion solves, u then v (include/assembly.h:1529-1545, 489-558): rhs = M u_adv - lift, g on Dirichlet rows
    for (int ch = 0; ch < 2; ++ch) {
        CgArgs f{};
        Csr& M = h->mats[NSF_VELOCITY_MASS];
        prepare_matrix(M, false, s);
        f.bRowptr = M.rowptr.get();
        f.bCol = M.col.get();
        f.bVal = M.val.get();
        f.bSellStart = M.sellStart.get();
        f.bSellCol = M.sellCol.get();
        f.bSellVal = M.sellVal.get();
        f.bX = tmp + (size_t)ch * Nv;
        f.lift = S.liftV[ch].get();
        f.bcMask = S.bcV.get();
        f.bcValue = S.gV[ch].get();
        f.bOut = S.rhsV.get() + (size_t)ch * Nv;
        infos[ch] = launch_solve(h, NSF_DIFFUSION, mode(NSF_DIFFUSION), f.bOut, tmp + (size_t)ch * Nv, uv + (size_t)ch * Nv, -1,
                                 h->tol, &f);
    }
    // pressure projection (include/assembly.h:560-712): rhs_p = -(1/dt) Div u - lift, pinned nodes -> g
    {
        CgArgs f{};
        Csr& Bd = h->mats[NSF_VELOCITY_DIVERGENCE];
        prepare_matrix(Bd, false, s);
        f.bRowptr = Bd.rowptr.get();
        f.bCol = Bd.col.get();
        f.bVal = Bd.val.get();
        f.bSellStart = Bd.sellStart.get();
        f.bSellCol = Bd.sellCol.get();
        f.bSellVal = Bd.sellVal.get();
        f.bX = uv;
        f.lift = S.liftP.get();
        f.bcMask = S.bcP.get();
        f.bcValue = S.gP.get();
        f.bOut = S.rhsP.get();
        infos[2] = launch_solve(h, NSF_PRESSURE_STIFFNESS, mode(NSF_PRESSURE_STIFFNESS), f.bOut, S.p.get(), S.p.get(), -1, h->tol, &f);
    }
    // velocity correction: M du = -dt Grad p per component with x0 = u, then u_out = du + u, Dirichlet re-imposed
    spmv_launch(h->mats[NSF_PRESSURE_DIVERGENCE], S.p.get(), S.rhsV.get(), s);
    for (int ch = 0; ch < 2; ++ch)
        infos[3 + ch] = launch_solve(h, NSF_VELOCITY_MASS, mode(NSF_VELOCITY_MASS), S.rhsV.get() + (size_t)ch * Nv,
                                     uv + (size_t)ch * Nv, tmp + (size_t)ch * Nv, -1, h->tol, nullptr);
    for (int ch = 0; ch < 2; ++ch)
        axpy_bc_launch(Nv, uv + (size_t)ch * Nv, tmp + (size_t)ch * Nv, S.bcV.get(), S.gV[ch].get(), s);
    std::swap(S.uv, S.tmp);
}

// One step of NavierStokesAssembly::solve (include/assembly.h:1137-1297), the explicit-convection scheme; `infos`
// receives 5 info indices (tentative u, v, pressure, correction u, v).  The reference solves its mass systems with
// the velocity as the initial guess of the increment, and so does this.
void sim_step_explicit_launch(nsf_device* h, int infos[5]) {
    SimState& S = h->sim;
    MeshDev& m = h->mesh;
    const int Nv = m.nNodes;
    auto mode = [&](int slot) {
        const bool pre = (h->solverMode == NSF_SOLVER_PCG_MIXED || h->solverMode == NSF_SOLVER_PCG_FP64) &&
                         h->factors[slot].ready && !h->pcgOff[slot];
        const bool mixed = (h->solverMode == NSF_SOLVER_MIXED || h->solverMode == NSF_SOLVER_PCG_MIXED) &&
                           !h->mixedOff[slot];
        if (pre) return mixed ? NSF_SOLVER_PCG_MIXED : NSF_SOLVER_PCG_FP64;
        return mixed ? NSF_SOLVER_MIXED : NSF_SOLVER_FP64;
    };
    cudaStream_t s = h->stream;
    double* uv = S.uv.get();
    double* tmp = S.tmp.get();
    ++S.steps;
    if (S.bcTimeDependent) bc_update_launch(S, m, h->mats, S.t0 + (double)S.steps * S.dt, s);
    // tentative velocity (include/assembly.h:1151-1196): rhs = -dt (C(u) + nu K) u; M y = rhs from x0 = u; u += y
    convection_rhs_launch(m, S, uv, S.rhsV.get(), s);
    for (int ch = 0; ch < 2; ++ch)
        infos[ch] = launch_solve(h, NSF_VELOCITY_MASS, mode(NSF_VELOCITY_MASS), S.rhsV.get() + (size_t)ch * Nv,
                                 uv + (size_t)ch * Nv, tmp + (size_t)ch * Nv, -1, h->tol, nullptr);
    // u += y with the Dirichlet values imposed (imposeVelocityDirichlet, :1198): into tmp, then swapped
    for (int ch = 0; ch < 2; ++ch)
        axpy_bc_launch(Nv, uv + (size_t)ch * Nv, tmp + (size_t)ch * Nv, S.bcV.get(), S.gV[ch].get(), s);
    std::swap(S.uv, S.tmp);
    uv = S.uv.get();
    tmp = S.tmp.get();
    // pressure (:1204-1241): rhs_p = -(1/dt) Div u with the Dirichlet rows and lift, solved from the previous p
    {
        CgArgs f{};
        Csr& Bd = h->mats[NSF_VELOCITY_DIVERGENCE];
        prepare_matrix(Bd, false, s);
        f.bRowptr = Bd.rowptr.get();
        f.bCol = Bd.col.get();
        f.bVal = Bd.val.get();
        f.bSellStart = Bd.sellStart.get();
        f.bSellCol = Bd.sellCol.get();
        f.bSellVal = Bd.sellVal.get();
        f.bX = uv;
        f.lift = S.liftP.get();
        f.bcMask = S.bcP.get();
        f.bcValue = S.gP.get();
        f.bOut = S.rhsP.get();
        infos[2] = launch_solve(h, NSF_PRESSURE_STIFFNESS, mode(NSF_PRESSURE_STIFFNESS), f.bOut, S.p.get(), S.p.get(),
                                -1, h->tol, &f);
    }
    // correction (:1250-1281): M y = -dt Grad p from x0 = u; u += y (no Dirichlet values imposed afterwards)
    spmv_launch(h->mats[NSF_PRESSURE_DIVERGENCE], S.p.get(), S.rhsV.get(), s);
    for (int ch = 0; ch < 2; ++ch)
        infos[3 + ch] = launch_solve(h, NSF_VELOCITY_MASS, mode(NSF_VELOCITY_MASS), S.rhsV.get() + (size_t)ch * Nv,
                                     uv + (size_t)ch * Nv, tmp + (size_t)ch * Nv, -1, h->tol, nullptr);
    for (int ch = 0; ch < 2; ++ch) axpy_bc_launch(Nv, uv + (size_t)ch * Nv, tmp + (size_t)ch * Nv, nullptr, nullptr, s);
    std::swap(S.uv, S.tmp);
}

constexpr int kSolveSlot[5] = {NSF_DIFFUSION, NSF_DIFFUSION, NSF_PRESSURE_STIFFNESS, NSF_VELOCITY_MASS,
                                NSF_VELOCITY_MASS};
constexpr int kSolveSlotExplicit[5] = {NSF_VELOCITY_MASS, NSF_VELOCITY_MASS, NSF_PRESSURE_STIFFNESS,
                                        NSF_VELOCITY_MASS, NSF_VELOCITY_MASS};

void run_steps(nsf_device* h, int nsteps, int* iterations) {
    sim_require(h);
    if (nsteps < 0) throw bad_arg("nsteps must be >= 0");
    const int chunk = std::max(1, (int)(h->ws.info.n / 5) - 1);
    int done = 0;
    std::vector<int> idx;
    while (done < nsteps) {
        const int n = std::min(chunk, nsteps - done);
        idx.assign((size_t)5 * n, 0);
        for (int k = 0; k < n; ++k) {
            if (h->sim.scheme == NSF_SCHEME_EXPLICIT_CONVECTION) sim_step_explicit_launch(h, &idx[(size_t)5 * k]);
            else sim_step_launch(h, &idx[(size_t)5 * k]);
        }
        std::vector<CgInfo> all(h->ws.info.n);
        NSF_CUDA(cudaMemcpyAsync(all.data(), h->ws.info.get(), sizeof(CgInfo) * all.size(), cudaMemcpyDeviceToHost,
                                 h->stream));
        NSF_CUDA(cudaStreamSynchronize(h->stream));
        static const char* namesSL[5] = {"diffusion u", "diffusion v", "pressure", "mass u", "mass v"};
        static const char* namesEx[5] = {"tentative u", "tentative v", "pressure", "correction u", "correction v"};
        const bool ex = h->sim.scheme == NSF_SCHEME_EXPLICIT_CONVECTION;
        const char* const* names = ex ? namesEx : namesSL;
        const int* slots = ex ? kSolveSlotExplicit : kSolveSlot;
        for (int k = 0; k < n; ++k)
            for (int j = 0; j < 5; ++j) {
                const CgInfo& info = all[idx[(size_t)5 * k + j]];
                if (iterations) iterations[(size_t)5 * (done + k) + j] = info.iterations;
                if (info.fallback) {
                    const int used = h->infoMode[idx[(size_t)5 * k + j]];
                    if (used == NSF_SOLVER_PCG_MIXED || used == NSF_SOLVER_PCG_FP64)
                        h->pcgOff[slots[j]] = true;    // the factor did not pay: plain CG from now on
                    else
                        h->mixedOff[slots[j]] = true;  // FP32 cannot resolve this system
                }
                if (info.status != NSF_OK)
                    throw Error{info.status, "step " + std::to_string(done + k + 1) + ", " + names[j] + " solve: " +
                                                 status_text(info.status) + " after " +
                                                 std::to_string(info.iterations) + " iterations"};
            }
        done += n;
    }
}

}  // namespace

extern "C" {

int nsf_create(int device, nsf_device** out) {
    if (!out) return NSF_ERR_BAD_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return NSF_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) return NSF_ERR_BAD_ARG;
    nsf_device* h = new nsf_device();
    h->device = device;
    try {
        NSF_CUDA(cudaSetDevice(device));
        NSF_CUDA(cudaDeviceGetAttribute(&h->smCount, cudaDevAttrMultiProcessorCount, device));
        NSF_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        cg_configure(h->ws, device);
    } catch (const Error& e) {
        fprintf(stderr, "nsf_create: %s\n", e.msg.c_str());
        delete h;
        return e.status;
    }
    *out = h;
    return NSF_OK;
}

void nsf_destroy(nsf_device* h) {
    if (!h) return;
    {
        std::lock_guard<std::recursive_mutex> lk(h->mu);
        cudaSetDevice(h->device);
        if (h->stream) cudaStreamSynchronize(h->stream);
        for (auto e : h->evPool) cudaEventDestroy(e);
        for (int i = 0; i < NSF_SLOT_COUNT; ++i) h->mats[i] = Csr();
        for (int i = 0; i < NSF_SLOT_COUNT; ++i) h->factors[i] = Factor();
        for (int i = 0; i < 4; ++i) scratch(h, i).release();
        if (h->stream) cudaStreamDestroy(h->stream);
    }
    delete h;
}

const char* nsf_last_error(const nsf_device* h) { return h ? h->lastError.c_str() : "null handle"; }

int nsf_device_info(nsf_device* h, int* smCount, int* cgGridBlocks, int* cgBlockThreads) {
    NSF_BEGIN(h)
    if (smCount) *smCount = h->smCount;
    if (cgGridBlocks) *cgGridBlocks = h->ws.grid;
    if (cgBlockThreads) *cgBlockThreads = h->ws.block;
    NSF_END(h)
}

int nsf_synchronize(nsf_device* h) {
    NSF_BEGIN(h)
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    NSF_END(h)
}

int nsf_upload_matrix_csr(nsf_device* h, int slot, int rows, int cols, int64_t nnz, const int* rowptr,
                          const int* col, const double* val) {
    NSF_BEGIN(h)
    if (!rowptr || (nnz > 0 && (!col || !val))) throw bad_arg("null array");
    upload_csr(h, slot, rows, cols, nnz, rowptr, col, val);
    NSF_END(h)
}

int nsf_upload_matrix_triplets(nsf_device* h, int slot, int rows, int cols, int64_t count, const int* row,
                               const int* col, const double* val) {
    NSF_BEGIN(h)
    if (count < 0 || (count > 0 && (!row || !col || !val))) throw bad_arg("null array");
    std::vector<int64_t> order(count);
    std::iota(order.begin(), order.end(), 0);
    for (int64_t k = 0; k < count; ++k)
        if (row[k] < 0 || row[k] >= rows || col[k] < 0 || col[k] >= cols) throw bad_arg("triplet index out of range");
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        return row[a] != row[b] ? row[a] < row[b] : col[a] < col[b];
    });
    std::vector<int> rp(rows + 1, 0), c;
    std::vector<double> v;
    for (int64_t k = 0; k < count; ++k) {
        const int64_t i = order[k];
        if (!c.empty() && k > 0 && row[order[k - 1]] == row[i] && col[order[k - 1]] == col[i]) {
            v.back() += val[i];
        } else {
            c.push_back(col[i]);
            v.push_back(val[i]);
            rp[row[i] + 1]++;
        }
    }
    for (int r = 0; r < rows; ++r) rp[r + 1] += rp[r];
    upload_csr(h, slot, rows, cols, (int64_t)c.size(), rp.data(), c.data(), v.data());
    NSF_END(h)
}

int nsf_matrix_shape(nsf_device* h, int slot, int* rows, int* cols, int64_t* nnz) {
    NSF_BEGIN(h)
    check_slot(slot);
    const Csr& A = h->mats[slot];
    if (rows) *rows = A.rows;
    if (cols) *cols = A.cols;
    if (nnz) *nnz = A.nnz;
    NSF_END(h)
}

int nsf_download_matrix(nsf_device* h, int slot, int* rowptr, int* col, double* val) {
    NSF_BEGIN(h)
    check_slot(slot);
    const Csr& A = h->mats[slot];
    if (!A.valid()) throw Error{NSF_ERR_STATE, "matrix slot is empty"};
    if (rowptr) NSF_CUDA(cudaMemcpyAsync(rowptr, A.rowptr.get(), sizeof(int) * (A.rows + 1), cudaMemcpyDeviceToHost, h->stream));
    if (col && A.nnz) NSF_CUDA(cudaMemcpyAsync(col, A.col.get(), sizeof(int) * A.nnz, cudaMemcpyDeviceToHost, h->stream));
    if (val && A.nnz) NSF_CUDA(cudaMemcpyAsync(val, A.val.get(), sizeof(double) * A.nnz, cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    NSF_END(h)
}

int nsf_spmv(nsf_device* h, int slot, const double* x, double* y) {
    NSF_BEGIN(h)
    check_slot(slot);
    const Csr& A = h->mats[slot];
    if (!A.valid()) throw Error{NSF_ERR_STATE, "matrix slot is empty"};
    if (!x || !y) throw bad_arg("null vector");
    DevBuf<double>& dx = scratch(h, 0);
    DevBuf<double>& dy = scratch(h, 1);
    dx.upload(x, A.cols, h->stream);
    dy.ensure(A.rows);
    spmv_launch(A, dx.get(), dy.get(), h->stream);
    NSF_CUDA(cudaMemcpyAsync(y, dy.get(), sizeof(double) * A.rows, cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    NSF_END(h)
}

int nsf_conjugate_gradient_dev(nsf_device* h, int slot, const double* b_dev, const double* x0_dev, double* x_dev,
                               int maxIterations, double eps, int mode, int* iterations, double* relResidual) {
    NSF_BEGIN(h)
    check_slot(slot);
    if (!b_dev || !x0_dev || !x_dev) throw bad_arg("null vector");
    if (mode < NSF_SOLVER_FP64 || mode > NSF_SOLVER_PCG_FP64) throw bad_arg("unknown solver mode");
    if (!(eps > 0)) throw bad_arg("eps must be positive");
    const int idx = launch_solve(h, slot, mode, b_dev, x0_dev, x_dev, maxIterations, eps, nullptr);
    const CgInfo info = read_info(h, idx);
    if (iterations) *iterations = info.iterations;
    if (relResidual) *relResidual = info.bb > 0 ? std::sqrt(info.rr / info.bb) : 0.0;
    throw_solve_status(info, "conjugate gradient");
    NSF_END(h)
}

int nsf_conjugate_gradient(nsf_device* h, int slot, const double* b, const double* x0, double* x, int maxIterations,
                           double eps, int mode, int* iterations, double* relResidual) {
    NSF_BEGIN(h)
    check_slot(slot);
    const Csr& A = h->mats[slot];
    if (!A.valid()) throw Error{NSF_ERR_STATE, "matrix slot is empty"};
    if (!b || !x0 || !x) throw bad_arg("null vector");
    if (mode < NSF_SOLVER_FP64 || mode > NSF_SOLVER_PCG_FP64) throw bad_arg("unknown solver mode");
    if (!(eps > 0)) throw bad_arg("eps must be positive");
    DevBuf<double>& db = scratch(h, 0);
    DevBuf<double>& dx0 = scratch(h, 1);
    DevBuf<double>& dx = scratch(h, 2);
    db.upload(b, A.rows, h->stream);
    dx0.upload(x0, A.rows, h->stream);
    dx.ensure(A.rows);
    const int idx = launch_solve(h, slot, mode, db.get(), dx0.get(), dx.get(), maxIterations, eps, nullptr);
    NSF_CUDA(cudaMemcpyAsync(x, dx.get(), sizeof(double) * A.rows, cudaMemcpyDeviceToHost, h->stream));
    const CgInfo info = read_info(h, idx);
    if (iterations) *iterations = info.iterations;
    if (relResidual) *relResidual = info.bb > 0 ? std::sqrt(info.rr / info.bb) : 0.0;
    throw_solve_status(info, "conjugate gradient");
    NSF_END(h)
}

int nsf_conjugate_gradient_f32(nsf_device* h, int slot, const float* b, const float* x0, float* x, int maxIterations,
                               float eps) {
    NSF_BEGIN(h)
    check_slot(slot);
    const Csr& A = h->mats[slot];
    if (!A.valid()) throw Error{NSF_ERR_STATE, "matrix slot is empty"};
    if (!b || !x0 || !x) throw bad_arg("null vector");
    std::vector<double> bd(b, b + A.rows), xd0(x0, x0 + A.rows), xd(A.rows);
    int st = nsf_conjugate_gradient(h, slot, bd.data(), xd0.data(), xd.data(), maxIterations, eps, NSF_SOLVER_FP64,
                                    nullptr, nullptr);
    for (int i = 0; i < A.rows; ++i) x[i] = (float)xd[i];
    if (st != NSF_OK) throw Error{st, h->lastError};
    NSF_END(h)
}

int nsf_upload_mesh(nsf_device* h, int nNodes, const float* xy, int nElements, const int* elements, int nPressure) {
    NSF_BEGIN(h)
    upload_mesh_into(h->mesh, h->stream, nNodes, xy, nElements, elements, nPressure);
    h->sim.ready = false;
    NSF_END(h)
}

int nsf_locate(nsf_device* h, int n, const float* pts, int* elem, float* xi, float* eta, int* nearest) {
    NSF_BEGIN(h)
    if (h->mesh.nEl == 0) throw Error{NSF_ERR_STATE, "no mesh uploaded"};
    if (n < 0 || (n > 0 && (!pts || !elem || !xi || !eta || !nearest))) throw bad_arg("null array");
    if (n == 0) return NSF_OK;
    DevBuf<float2> dp;
    DevBuf<int> de, dn;
    DevBuf<float> dxi, deta;
    dp.upload((const float2*)pts, n, h->stream);
    de.alloc(n);
    dn.alloc(n);
    dxi.alloc(n);
    deta.alloc(n);
    locate_launch(h->mesh, n, dp.get(), de.get(), dxi.get(), deta.get(), dn.get(), h->stream);
    NSF_CUDA(cudaMemcpyAsync(elem, de.get(), sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaMemcpyAsync(nearest, dn.get(), sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaMemcpyAsync(xi, dxi.get(), sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaMemcpyAsync(eta, deta.get(), sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    NSF_END(h)
}

int nsf_advect(nsf_device* h, int numNodes, const float* u, const float* v, float dt, float* uOut, float* vOut) {
    NSF_BEGIN(h)
    if (h->mesh.nEl == 0) throw Error{NSF_ERR_STATE, "no mesh uploaded"};
    if (numNodes != h->mesh.nNodes) throw bad_arg("numNodes differs from the mesh's node count");
    if (!u || !v || !uOut || !vOut) throw bad_arg("null vector");
    DevBuf<float> a, b, c, d;
    a.upload(u, numNodes, h->stream);
    b.upload(v, numNodes, h->stream);
    c.alloc(numNodes);
    d.alloc(numNodes);
    advect_f32_launch(h->mesh, dt, a.get(), b.get(), c.get(), d.get(), h->stream);
    NSF_CUDA(cudaMemcpyAsync(uOut, c.get(), sizeof(float) * numNodes, cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaMemcpyAsync(vOut, d.get(), sizeof(float) * numNodes, cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    NSF_END(h)
}

int nsf_advect_f64(nsf_device* h, int numNodes, const double* u, const double* v, double dt, double* uOut,
                   double* vOut) {
    NSF_BEGIN(h)
    if (h->mesh.nEl == 0) throw Error{NSF_ERR_STATE, "no mesh uploaded"};
    if (numNodes != h->mesh.nNodes) throw bad_arg("numNodes differs from the mesh's node count");
    if (!u || !v || !uOut || !vOut) throw bad_arg("null vector");
    DevBuf<double>& a = scratch(h, 0);
    DevBuf<double>& c = scratch(h, 1);
    a.ensure(2 * (size_t)numNodes);
    c.ensure(2 * (size_t)numNodes);
    NSF_CUDA(cudaMemcpyAsync(a.get(), u, sizeof(double) * numNodes, cudaMemcpyHostToDevice, h->stream));
    NSF_CUDA(cudaMemcpyAsync(a.get() + numNodes, v, sizeof(double) * numNodes, cudaMemcpyHostToDevice, h->stream));
    advect_launch(h->mesh, dt, a.get(), a.get() + numNodes, c.get(), c.get() + numNodes, h->stream);
    NSF_CUDA(cudaMemcpyAsync(uOut, c.get(), sizeof(double) * numNodes, cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaMemcpyAsync(vOut, c.get() + numNodes, sizeof(double) * numNodes, cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    NSF_END(h)
}

int nsf_sim_setup(nsf_device* h, int nNodes, const float* xy, int nElements, const int* elements, int nPressure,
                  int nVelocityBC, const int* velocityBCNodes, const double* bcU, const double* bcV, int nPressureBC,
                  const int* pressureBCNodes, const double* bcP, double viscosity, double dt) {
    NSF_BEGIN(h)
    h->sim.ready = false;
    for (int i = 0; i < NSF_SLOT_COUNT; ++i) {
        h->factors[i] = Factor();
        h->pcgOff[i] = false;
    }
    setup_instance(h->mesh, h->sim, h->mats, h->stream, nNodes, xy, nElements, elements, nPressure, nVelocityBC,
                   velocityBCNodes, bcU, bcV, nPressureBC, pressureBCNodes, bcP, viscosity, dt);
    ensure_workspace(h, std::max(nNodes, nPressure));
    for (int slot : {NSF_DIFFUSION, NSF_PRESSURE_STIFFNESS, NSF_VELOCITY_MASS})
        prepare_matrix(h->mats[slot], h->solverMode == NSF_SOLVER_MIXED, h->stream);
    prepare_matrix(h->mats[NSF_VELOCITY_DIVERGENCE], false, h->stream);   // the pressure right-hand side's product
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    h->sim.ready = true;
    NSF_END(h)
}

int nsf_sim_set_fields(nsf_device* h, const double* uv, const double* p) {
    NSF_BEGIN(h)
    sim_require(h);
    if (!uv || !p) throw bad_arg("null field");
    const int Nv = h->mesh.nNodes, P = h->mesh.nP;
    field_copy(h, h->sim.uv.get(), uv, sizeof(double) * 2 * Nv, cudaMemcpyHostToDevice);
    field_copy(h, h->sim.p.get(), p, sizeof(double) * P, cudaMemcpyHostToDevice);
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    NSF_END(h)
}

int nsf_sim_get_fields(nsf_device* h, double* uv, double* p) {
    NSF_BEGIN(h)
    sim_require(h);
    const int Nv = h->mesh.nNodes, P = h->mesh.nP;
    if (uv) field_copy(h, uv, h->sim.uv.get(), sizeof(double) * 2 * Nv, cudaMemcpyDeviceToHost);
    if (p) field_copy(h, p, h->sim.p.get(), sizeof(double) * P, cudaMemcpyDeviceToHost);
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    NSF_END(h)
}

int nsf_sim_set_bc_expressions(nsf_device* h, int nExpressions, const char* const* expressions, const int* velocityU,
                               const int* velocityV, const int* pressure, double t0) {
    NSF_BEGIN(h)
    sim_require(h);
    bc_set_programs(h->sim, h->mesh, h->mats, nExpressions, expressions, velocityU, velocityV, pressure, t0,
                    h->stream);
    NSF_END(h)
}

int nsf_sim_set_scheme(nsf_device* h, int scheme) {
    NSF_BEGIN(h)
    sim_require(h);
    if (scheme != NSF_SCHEME_SEMI_LAGRANGIAN && scheme != NSF_SCHEME_EXPLICIT_CONVECTION) throw bad_arg("unknown scheme");
    h->sim.scheme = scheme;
    NSF_END(h)
}

int nsf_sim_time(nsf_device* h, double* t) {
    NSF_BEGIN(h)
    sim_require(h);
    if (!t) throw bad_arg("null output");
    *t = h->sim.t0 + (double)h->sim.steps * h->sim.dt;
    NSF_END(h)
}

int nsf_sim_step(nsf_device* h, int nsteps, int* iterations) {
    NSF_BEGIN(h)
    run_steps(h, nsteps, iterations);
    NSF_END(h)
}

int nsf_sim_step_host(nsf_device* h, const double* uvIn, const double* pIn, int nsteps, double* uvOut, double* pOut,
                      int* iterations) {
    NSF_BEGIN(h)
    sim_require(h);
    const int Nv = h->mesh.nNodes, P = h->mesh.nP;
    if (uvIn) field_copy(h, h->sim.uv.get(), uvIn, sizeof(double) * 2 * Nv, cudaMemcpyHostToDevice);
    if (pIn) field_copy(h, h->sim.p.get(), pIn, sizeof(double) * P, cudaMemcpyHostToDevice);
    run_steps(h, nsteps, iterations);
    if (uvOut) field_copy(h, uvOut, h->sim.uv.get(), sizeof(double) * 2 * Nv, cudaMemcpyDeviceToHost);
    if (pOut) field_copy(h, pOut, h->sim.p.get(), sizeof(double) * P, cudaMemcpyDeviceToHost);
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    NSF_END(h)
}

int nsf_batch_clear(nsf_device* h) {
    NSF_BEGIN(h)
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    if (h->batchGraphExec) { cudaGraphExecDestroy(h->batchGraphExec); h->batchGraphExec = nullptr; }
    if (h->batchGraph) { cudaGraphDestroy(h->batchGraph); h->batchGraph = nullptr; }
    h->batch.clear();
    h->batchReady = false;
    h->batchStepsDone = 0;
    NSF_END(h)
}

int nsf_batch_add(nsf_device* h, int nNodes, const float* xy, int nElements, const int* elements, int nPressure,
                  int nVelocityBC, const int* velocityBCNodes, const double* bcU, const double* bcV, int nPressureBC,
                  const int* pressureBCNodes, const double* bcP, double viscosity, double dt, int* index) {
    NSF_BEGIN(h)
    if (h->batchReady) throw Error{NSF_ERR_STATE, "the batch is finalized; call nsf_batch_clear first"};
    std::unique_ptr<Instance> in(new Instance());
    setup_instance(in->mesh, in->sim, in->mats, h->stream, nNodes, xy, nElements, elements, nPressure, nVelocityBC,
                   velocityBCNodes, bcU, bcV, nPressureBC, pressureBCNodes, bcP, viscosity, dt);
    const size_t n = (size_t)std::max(nNodes, nPressure);
    in->r.alloc(n);
    in->q.alloc(n);
    in->p0.alloc(n);
    in->p1.alloc(n);
    in->r32.alloc(n);
    in->d32.alloc(n);
    in->q32.alloc(n);
    in->p32a.alloc(n);
    in->p32b.alloc(n);
    in->info.alloc((size_t)kStepInfoCap * 5);
    in->info.zero(h->stream);
    in->stepCounter.alloc(1);
    in->stepCounter.zero(h->stream);
    in->teamNs.alloc(1);
    in->teamNs.zero(h->stream);
    for (int slot : {NSF_DIFFUSION, NSF_PRESSURE_STIFFNESS, NSF_VELOCITY_MASS})
        prepare_matrix(in->mats[slot], h->solverMode == NSF_SOLVER_MIXED, h->stream);
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    in->sim.ready = true;
    h->batch.push_back(std::move(in));
    if (index) *index = (int)h->batch.size() - 1;
    NSF_END(h)
}

int nsf_batch_finalize(nsf_device* h, int autotuneRounds) {
    NSF_BEGIN(h)
    if (h->batch.empty()) throw Error{NSF_ERR_STATE, "no instances added"};
    h->batchCapacity = step_kernel_capacity(h->device);
    if ((int)h->batch.size() > h->batchCapacity)
        throw bad_arg("more instances than co-resident CTAs (" + std::to_string(h->batchCapacity) + ")");
    for (auto& in : h->batch)
        for (int slot : {NSF_DIFFUSION, NSF_PRESSURE_STIFFNESS, NSF_VELOCITY_MASS})
            prepare_matrix(in->mats[slot], h->solverMode == NSF_SOLVER_MIXED, h->stream);
    batch_autotune(h, std::max(0, autotuneRounds));
    batch_capture_graph(h);
    h->batchReady = true;
    h->batchStepsDone = 0;
    NSF_END(h)
}

int nsf_batch_step(nsf_device* h, int nsteps, int* iterations) {
    NSF_BEGIN(h)
    if (!h->batchReady) throw Error{NSF_ERR_STATE, "nsf_batch_finalize has not been called"};
    if (nsteps < 0) throw bad_arg("nsteps must be >= 0");
    const size_t n = h->batch.size();
    std::vector<CgInfo> infos((size_t)kStepInfoCap * 5);
    int done = 0;
    while (done < nsteps) {
        const int chunk = std::min(kStepInfoCap, nsteps - done);
        for (int k = 0; k < chunk; ++k) {
            NSF_CUDA(cudaGraphLaunch(h->batchGraphExec, h->stream));
            count_launch();
        }
        NSF_CUDA(cudaStreamSynchronize(h->stream));
        static const char* names[5] = {"diffusion u", "diffusion v", "pressure", "mass u", "mass v"};
        for (size_t i = 0; i < n; ++i) {
            NSF_CUDA(cudaMemcpy(infos.data(), h->batch[i]->info.get(), sizeof(CgInfo) * infos.size(),
                                cudaMemcpyDeviceToHost));
            for (int k = 0; k < chunk; ++k) {
                const int stepIdx = h->batchStepsDone + k;
                const CgInfo* inf = &infos[(size_t)(stepIdx % kStepInfoCap) * 5];
                for (int j = 0; j < 5; ++j) {
                    if (iterations) iterations[((size_t)(done + k) * n + i) * 5 + j] = inf[j].iterations;
                    if (inf[j].status != NSF_OK)
                        throw Error{inf[j].status, "instance " + std::to_string(i) + ", step " +
                                                       std::to_string(stepIdx + 1) + ", " + names[j] + " solve: " +
                                                       status_text(inf[j].status)};
                }
            }
        }
        h->batchStepsDone += chunk;
        done += chunk;
    }
    NSF_END(h)
}

int nsf_batch_get_fields(nsf_device* h, int index, double* uv, double* p) {
    NSF_BEGIN(h)
    if (index < 0 || index >= (int)h->batch.size()) throw bad_arg("instance index out of range");
    const Instance& in = *h->batch[index];
    if (uv) NSF_CUDA(cudaMemcpyAsync(uv, in.sim.uv.get(), sizeof(double) * in.sim.uv.n, cudaMemcpyDeviceToHost, h->stream));
    if (p) NSF_CUDA(cudaMemcpyAsync(p, in.sim.p.get(), sizeof(double) * in.sim.p.n, cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    NSF_END(h)
}

int nsf_batch_set_fields(nsf_device* h, int index, const double* uv, const double* p) {
    NSF_BEGIN(h)
    if (index < 0 || index >= (int)h->batch.size()) throw bad_arg("instance index out of range");
    Instance& in = *h->batch[index];
    if (uv) NSF_CUDA(cudaMemcpyAsync(in.sim.uv.get(), uv, sizeof(double) * in.sim.uv.n, cudaMemcpyHostToDevice, h->stream));
    if (p) NSF_CUDA(cudaMemcpyAsync(in.sim.p.get(), p, sizeof(double) * in.sim.p.n, cudaMemcpyHostToDevice, h->stream));
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    NSF_END(h)
}

int nsf_batch_plan(nsf_device* h, int* blocks, int* gridBlocks, float* trialMs, int maxTrials, int* nTrials) {
    NSF_BEGIN(h)
    if (blocks)
        for (size_t i = 0; i < h->batch.size(); ++i) blocks[i] = h->batch[i]->blocks;
    if (gridBlocks) *gridBlocks = h->batchGrid;
    const int nt = (int)h->autotuneMs.size();
    if (nTrials) *nTrials = nt;
    if (trialMs)
        for (int k = 0; k < std::min(nt, maxTrials); ++k) trialMs[k] = (float)h->autotuneMs[k];
    NSF_END(h)
}

int nsf_set_tolerance(nsf_device* h, double eps) {
    NSF_BEGIN(h)
    if (!(eps > 0)) throw bad_arg("tolerance must be positive");
    h->tol = eps;
    NSF_END(h)
}

int nsf_set_solver(nsf_device* h, int mode, double innerTolerance) {
    NSF_BEGIN(h)
    if (mode < NSF_SOLVER_FP64 || mode > NSF_SOLVER_PCG_FP64) throw bad_arg("unknown solver mode");
    if (innerTolerance > 0) h->innerTol = innerTolerance;
    h->solverMode = mode;
    for (bool& off : h->mixedOff) off = false;
    for (bool& off : h->pcgOff) off = false;
    if ((mode == NSF_SOLVER_MIXED || mode == NSF_SOLVER_PCG_MIXED) && h->sim.ready) {
        for (int slot : {NSF_DIFFUSION, NSF_PRESSURE_STIFFNESS, NSF_VELOCITY_MASS}) prepare_matrix(h->mats[slot], true, h->stream);
        NSF_CUDA(cudaStreamSynchronize(h->stream));
    }
    NSF_END(h)
}

int nsf_precond_schur_nnz(nsf_device* h, int slot, int64_t* nnz) {
    NSF_BEGIN(h)
    check_slot(slot);
    if (!nnz) throw bad_arg("null output");
    const Factor& F = h->factors[slot];
    *nnz = F.hasSchur ? F.S.nnz : 0;
    NSF_END(h)
}

int nsf_set_pcg_form(nsf_device* h, int form) {
    NSF_BEGIN(h)
    if (form < NSF_PCG_FORM_AUTO || form > NSF_PCG_FORM_SCHUR) throw bad_arg("unknown PCG form");
    h->pcgForm = form;
    NSF_END(h)
}

int nsf_set_cg_form(nsf_device* h, int form) {
    NSF_BEGIN(h)
    if (form < NSF_CG_FORM_AUTO || form > NSF_CG_FORM_MULTI_KERNEL) throw bad_arg("unknown CG form");
    h->cgForm = form;
    NSF_END(h)
}

// ---- preconditioners -------------------------------------------------------------------------------
int nsf_precond_pattern(nsf_device* h, int slot, int* colours, int64_t* nnzLower) {
    NSF_BEGIN(h)
    Factor& F = factor_for(h, slot, false);
    if (colours) *colours = F.colours;
    if (nnzLower) *nnzLower = F.nnzL;
    NSF_END(h)
}

int nsf_precond_get_pattern(nsf_device* h, int slot, int* rowptr, int* col, unsigned char* colour) {
    NSF_BEGIN(h)
    Factor& F = factor_for(h, slot, false);
    if (rowptr)
        NSF_CUDA(cudaMemcpyAsync(rowptr, F.lRowptr.get(), sizeof(int) * (F.rows + 1), cudaMemcpyDeviceToHost, h->stream));
    if (col && F.nnzL)
        NSF_CUDA(cudaMemcpyAsync(col, F.lCol.get(), sizeof(int) * F.nnzL, cudaMemcpyDeviceToHost, h->stream));
    if (colour)
        NSF_CUDA(cudaMemcpyAsync(colour, F.colourOf.get(), F.rows, cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    NSF_END(h)
}

int nsf_precond_ic0(nsf_device* h, int slot, double* shiftUsed) {
    NSF_BEGIN(h)
    Factor& F = factor_for(h, slot, false);
    const double sh = factor_ic0(F, h->mats[slot], h->stream);
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    h->pcgOff[slot] = false;
    if (shiftUsed) *shiftUsed = sh;
    NSF_END(h)
}

int nsf_precond_set(nsf_device* h, int slot, const double* lower, const double* diag) {
    NSF_BEGIN(h)
    if (!diag || (!lower && h->factors[slot].nnzL)) throw bad_arg("null array");
    Factor& F = factor_for(h, slot, false);
    if (F.nnzL && !lower) throw bad_arg("null array");
    for (int i = 0; i < F.rows; ++i)
        if (!(diag[i] > 0.0) || !std::isfinite(diag[i])) throw bad_arg("factor diagonal must be positive and finite");
    for (int64_t k = 0; k < F.nnzL; ++k)
        if (!std::isfinite(lower[k])) throw bad_arg("factor values must be finite");
    if (F.nnzL) NSF_CUDA(cudaMemcpyAsync(F.lVal.get(), lower, sizeof(double) * F.nnzL, cudaMemcpyHostToDevice, h->stream));
    NSF_CUDA(cudaMemcpyAsync(F.diag.get(), diag, sizeof(double) * F.rows, cudaMemcpyHostToDevice, h->stream));
    factor_fill(F, h->stream);
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    F.kind = NSF_PRECOND_LEARNED;
    F.shift = 0.0;
    h->pcgOff[slot] = false;
    NSF_END(h)
}

int nsf_precond_get(nsf_device* h, int slot, double* lower, double* diag) {
    NSF_BEGIN(h)
    Factor& F = factor_for(h, slot, true);
    if (lower && F.nnzL)
        NSF_CUDA(cudaMemcpyAsync(lower, F.lVal.get(), sizeof(double) * F.nnzL, cudaMemcpyDeviceToHost, h->stream));
    if (diag) NSF_CUDA(cudaMemcpyAsync(diag, F.diag.get(), sizeof(double) * F.rows, cudaMemcpyDeviceToHost, h->stream));
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    NSF_END(h)
}

int nsf_precond_kind(nsf_device* h, int slot) {
    if (!h || slot < 0 || slot >= NSF_SLOT_COUNT) return -NSF_ERR_BAD_ARG;
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    return h->factors[slot].ready ? h->factors[slot].kind : NSF_PRECOND_NONE;
}

int nsf_precond_index_bytes(nsf_device* h, int slot) {
    if (!h || slot < 0 || slot >= NSF_SLOT_COUNT) return -NSF_ERR_BAD_ARG;
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    const Factor& F = h->factors[slot];
    return F.ready && F.colours >= 2 && F.col16 && F.Ap.hasCol16 ? 2 : 4;
}

int nsf_precond_value_bytes(nsf_device* h, int slot) {
    if (!h || slot < 0 || slot >= NSF_SLOT_COUNT) return -NSF_ERR_BAD_ARG;
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    const Factor& F = h->factors[slot];
    return F.ready && F.has16 ? 2 : 4;
}

int nsf_precond_inner_form(nsf_device* h, int slot, int* form) {
    NSF_BEGIN(h)
    check_slot(slot);
    if (!form) throw bad_arg("null output pointer");
    *form = h->innerForm[slot];
    NSF_END(h)
}

int nsf_precond_clear(nsf_device* h, int slot) {
    NSF_BEGIN(h)
    check_slot(slot);
    h->factors[slot] = Factor();
    h->pcgOff[slot] = false;
    NSF_END(h)
}

int nsf_precond_cap(nsf_device* h, int slot, int maxIterations) {
    NSF_BEGIN(h)
    check_slot(slot);
    if (maxIterations < 0) throw bad_arg("cap must be >= 0");
    h->pcgCap[slot] = maxIterations;
    NSF_END(h)
}

int nsf_set_barrier_timeout(nsf_device* h, double seconds) {
    NSF_BEGIN(h)
    if (!(seconds >= 0)) throw bad_arg("timeout must be >= 0");
    h->timeoutNs = (long long)(seconds * 1e9);
    NSF_END(h)
}

int nsf_profile(nsf_device* h, int enable) {
    NSF_BEGIN(h)
    NSF_CUDA(cudaStreamSynchronize(h->stream));
    h->records.clear();
    h->evUsed = 0;
    h->profile = enable != 0;
    NSF_END(h)
}

int nsf_profile_read(nsf_device* h, int maxRecords, int* slot, int* mode, int* fallback, int* rows, int64_t* nnz, int* iterations,
                     int* outer, float* ms) {
    if (!h) return -NSF_ERR_BAD_ARG;
    std::lock_guard<std::recursive_mutex> lk(h->mu);
    try {
        NSF_CUDA(cudaSetDevice(h->device));
        NSF_CUDA(cudaStreamSynchronize(h->stream));
        std::vector<CgInfo> all(h->ws.info.n);
        NSF_CUDA(cudaMemcpy(all.data(), h->ws.info.get(), sizeof(CgInfo) * all.size(), cudaMemcpyDeviceToHost));
        const int n = std::min<int>(maxRecords, (int)h->records.size());
        for (int i = 0; i < n; ++i) {
            const auto& r = h->records[i];
            float t = 0;
            NSF_CUDA(cudaEventElapsedTime(&t, r.a, r.b));
            if (slot) slot[i] = r.slot;
            if (mode) mode[i] = r.mode;
            if (fallback) fallback[i] = all[r.infoIndex].fallback;
            if (rows) rows[i] = r.rows;
            if (nnz) nnz[i] = r.nnz;
            if (iterations) iterations[i] = all[r.infoIndex].iterations;
            if (outer) outer[i] = all[r.infoIndex].outer;
            if (ms) ms[i] = t;
        }
        return n;
    } catch (const Error& e) {
        h->lastError = e.msg;
        return -e.status;
    }
}

int nsf_timer(nsf_device* h, int op, float* ms) {
    NSF_BEGIN(h)
    static thread_local cudaEvent_t start = nullptr, stop = nullptr;
    if (!start) {
        NSF_CUDA(cudaEventCreate(&start));
        NSF_CUDA(cudaEventCreate(&stop));
    }
    if (op == 0) {
        NSF_CUDA(cudaEventRecord(start, h->stream));
    } else {
        NSF_CUDA(cudaEventRecord(stop, h->stream));
        NSF_CUDA(cudaEventSynchronize(stop));
        float t = 0;
        NSF_CUDA(cudaEventElapsedTime(&t, start, stop));
        if (ms) *ms = t;
    }
    NSF_END(h)
}

int nsf_host_alloc(nsf_device* h, size_t bytes, void** ptr) {
    NSF_BEGIN(h)
    if (!ptr) throw bad_arg("null output pointer");
    if (bytes == 0) throw bad_arg("zero bytes");
    *ptr = nullptr;
    void* p = nullptr;
    NSF_CUDA(cudaHostAlloc(&p, bytes, cudaHostAllocMapped | cudaHostAllocPortable));
    try {
        void* dev = nullptr;
        NSF_CUDA(cudaHostGetDevicePointer(&dev, p, 0));
        copy_kernel_launch(h, dev, nullptr, bytes);   // zeroes it from the GPU: maps its pages for the device now
        NSF_CUDA(cudaStreamSynchronize(h->stream));
        std::lock_guard<std::mutex> lk(g_hostMu);
        g_hostBlocks[(uintptr_t)p] = HostBlock{bytes, static_cast<char*>(dev)};
    } catch (...) {
        cudaFreeHost(p);
        throw;
    }
    *ptr = p;
    NSF_END(h)
}

int nsf_host_free(nsf_device* h, void* ptr) {
    NSF_BEGIN(h)
    if (ptr) {
        NSF_CUDA(cudaStreamSynchronize(h->stream));
        {
            std::lock_guard<std::mutex> lk(g_hostMu);
            g_hostBlocks.erase((uintptr_t)ptr);
        }
        NSF_CUDA(cudaFreeHost(ptr));
    }
    NSF_END(h)
}

int nsf_launch_count(nsf_device* h, int64_t* launches) {
    NSF_BEGIN(h)
    if (!launches) throw bad_arg("null output pointer");
    *launches = g_launches.load();
    NSF_END(h)
}

int nsf_flush_l2(nsf_device* h, size_t bytes) {
    NSF_BEGIN(h)
    h->flush.ensure(bytes);
    NSF_CUDA(cudaMemsetAsync(h->flush.get(), (int)(h->flushToggle++ & 0xFF), bytes, h->stream));
    NSF_END(h)
}

}  // extern "C"

#include "host/expression.h"

extern "C" int nsf_eval_expression_t(const char* expression, double x, double y, double t, double* value,
                                     char* message, size_t messageBytes) {
    try {
        if (!expression || !value) throw std::runtime_error("null argument");
        // through the compiled program that nsf_sim_set_bc_expressions hands to the device
        std::vector<int> ops;
        std::vector<double> consts;
        nsfhost::Expression(expression).compile(ops, consts);
        *value = nsfhost::run_program(ops, consts, x, y, t);
        if (message && messageBytes) message[0] = '\0';
        return NSF_OK;
    } catch (const std::exception& err) {
        if (message && messageBytes) {
            strncpy(message, err.what(), messageBytes - 1);
            message[messageBytes - 1] = '\0';
        }
        return NSF_ERR_BAD_ARG;
    }
}

extern "C" int nsf_eval_expression(const char* expression, double x, double y, double* value, char* message,
                                   size_t messageBytes) {
    try {
        if (!expression || !value) throw std::runtime_error("null argument");
        const nsfhost::Expression e(expression);
        *value = e.evaluate({{'x', x}, {'y', y}});
        if (message && messageBytes) message[0] = '\0';
        return NSF_OK;
    } catch (const std::exception& err) {
        if (message && messageBytes) {
            strncpy(message, err.what(), messageBytes - 1);
            message[messageBytes - 1] = '\0';
        }
        return NSF_ERR_BAD_ARG;
    }
}
