// Internal declarations shared by the GB300 solver's translation units.  Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdarg>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/nsfem_gb300.h"
#include "host/expression.h"

namespace nsf {

// ------------------------------------------------------------------------------------------------
// error handling: every entry point returns an nsf_status and leaves a message on the handle
// ------------------------------------------------------------------------------------------------
struct Error {
    int status;
    std::string msg;
};

#define NSF_CUDA(call)                                                                                  \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            throw ::nsf::Error{NSF_ERR_CUDA, std::string(#call) + " failed: " + cudaGetErrorString(e_) + \
                                                 " (" + __FILE__ + ":" + std::to_string(__LINE__) + ")"}; \
    } while (0)

inline Error bad_arg(const std::string& m) { return Error{NSF_ERR_BAD_ARG, m}; }

// Every launch of one of the library's kernels is counted here (process-wide), for nsf_launch_count.
extern std::atomic<long long> g_launches;
inline void count_launch(long long n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// ------------------------------------------------------------------------------------------------
// device memory owned by a handle
// ------------------------------------------------------------------------------------------------
template <typename T> struct DevBuf {
    T* ptr = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : ptr(o.ptr), n(o.n) { o.ptr = nullptr; o.n = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) { release(); ptr = o.ptr; n = o.n; o.ptr = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        if (count == n && ptr) return;
        release();
        if (count) NSF_CUDA(cudaMalloc((void**)&ptr, count * sizeof(T)));
        n = count;
    }
    void ensure(size_t count) { if (count > n) alloc(count); }
    void upload(const T* host, size_t count, cudaStream_t s) {
        alloc(count);
        if (count) NSF_CUDA(cudaMemcpyAsync(ptr, host, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void zero(cudaStream_t s) { if (n) NSF_CUDA(cudaMemsetAsync(ptr, 0, n * sizeof(T), s)); }
    T* get() const { return ptr; }
};

// CSR matrix resident on the device.  Row pointers and column indices are int32 (nnz < 2^31 is checked at
// upload); FP64 values are always present, FP32 values are made on demand for the mixed-precision solver.
struct Csr {
    int rows = 0, cols = 0;
    int64_t nnz = 0;
    DevBuf<int> rowptr, col;
    DevBuf<double> val;
    DevBuf<float> val32;
    DevBuf<float> rowsum32;   // FP64 row sums rounded to FP32 (the difference-form FP32 product)
    bool has32 = false;
    // SELL-32 copy for the CG kernels: slice s = rows [32s, 32s+32), entries column-major from sellStart[s]
    int nSlices = 0;
    int maxWidth = 0;         // entries per row of the widest slice
    DevBuf<int> sellStart, sellCol;
    DevBuf<double> sellVal;
    DevBuf<float> sellVal32;
    bool hasSell = false, hasSell32 = false;
    // 16-bit copy of sellCol (offsets from a per-slice base; diagonal entries as padding), built on request when
    // every slice fits; for the difference-form FP32 product only
    DevBuf<int> sellColBase;
    DevBuf<unsigned short> sellCol16;
    bool col16Tried = false, hasCol16 = false;
    void values_changed() {
        has32 = hasSell = hasSell32 = false;
        val32.release();
        sellVal32.release();
    }
    bool valid() const { return rows > 0 && rowptr.ptr != nullptr; }
};

// Preconditioner factor M = L L^T (incomplete Cholesky or learned), in multicolour order: rows are greedily
// coloured so that no two neighbours share a colour, and "lower" means a neighbour of a smaller colour.  The
// triangular solves then run colour by colour, every row of a colour in parallel.
constexpr int kMaxColours = 16;
constexpr int kCol16Pad = 0xFFFF;   // padding entry (column -1) of a 16-bit SELL column array

struct FactorView {
    int colours = 0;
    int colourRow[kMaxColours + 1] = {};      // colour c = permuted rows [colourRow[c], colourRow[c+1]) (x 32)
    int nNatural = 0;                         // rows of the caller's system
    const int* perm = nullptr;                // permuted row -> caller's row (-1: padding row)
    int loMaxW = 0, upMaxW = 0;               // entries per row of the widest lower / upper slice
    const int* loStart = nullptr;             // lower part (L_ij, colour j < colour i), SELL-32, permuted rows
    const int* loCol = nullptr;
    const double* loVal = nullptr;
    const float* loVal32 = nullptr;
    const int* upStart = nullptr;             // upper part (L_ji, colour j > colour i)
    const int* upCol = nullptr;
    const double* upVal = nullptr;
    const float* upVal32 = nullptr;
    const __half* loVal16 = nullptr;          // FP16 copies of both parts' values (null: a value is outside FP16's
    const __half* upVal16 = nullptr;          // normal range); the FP32 copies then hold the same rounded values
    const unsigned short* loCol16 = nullptr;  // 16-bit column copies of both parts (null: not built, or a slice's
    const int* loColBase = nullptr;           // columns span 65535 or more)
    const unsigned short* upCol16 = nullptr;
    const int* upColBase = nullptr;
    const double* dinv = nullptr;             // 1 / L_ii per permuted row (1 on padding rows)
    const float* dinv32 = nullptr;
    // the reduced (Schur complement) iteration of a two-colour system: the matrix's own diagonal per permuted row,
    // FP64, and 1 / a_ii in FP32; reduced = 1 selects that iteration in the split mixed PCG
    const double* aDiag = nullptr;
    const float* aInv32 = nullptr;
    int reduced = 0;
    // the Schur complement S = A_11 - A_10 A_00^-1 A_01 formed explicitly (SELL-32 over the permuted rows, colour-0
    // rows empty; FP32 values, FP64 row sums rounded once, 16-bit columns with the diagonal as padding); schur = 1:
    // the reduced iteration multiplies by it in one phase instead of forming u_0 first
    int schur = 0;
    int sMaxW = 0;
    const int* sStart = nullptr;
    const unsigned short* sCol16 = nullptr;
    const int* sColBase = nullptr;
    const float* sVal32 = nullptr;
    const float* sRowsum32 = nullptr;
    double* w = nullptr;                      // work vector: forward-sweep result, then M^-1 r (in place)
    float* w32 = nullptr;
    double* xp = nullptr;                     // the iterate and right-hand side in permuted order
    double* bp = nullptr;
    const double* natB = nullptr;             // the caller's right-hand side, initial guess and solution
    const double* natX0 = nullptr;
    double* natX = nullptr;
};

// The factor of one matrix.  The preconditioned solve runs on the colour-permuted system P A P^T, whose colour
// blocks are padded to whole 32-row slices (padding rows are identity rows with zero right-hand side), so every
// colour phase of the sweeps is a contiguous, slice-aligned row range.
struct Factor {
    int rows = 0, colours = 0, nPerm = 0;
    int64_t nnzL = 0;                          // strictly lower entries
    int colourRow[kMaxColours + 1] = {};
    DevBuf<unsigned char> colourOf;            // per caller row
    DevBuf<int> lRowptr, lCol;                 // canonical CSR of the strictly lower part (caller's rows), entries by
                                               // (colour, column)
    DevBuf<int> aIndexL, aIndexDiag;           // positions of L's entries / the diagonal in the matrix's CSR values
    DevBuf<double> lVal, diag;                 // factor values on the canonical pattern and L_ii
    DevBuf<int> perm;                          // permuted row -> caller's row (-1 padding)
    Csr Ap;                                    // P A P^T (padded), with its SELL copies
    DevBuf<int> apFrom;                        // Ap value k = A.val[apFrom[k]] (-1: padding diagonal, 1.0)
    DevBuf<int> loStart, loCol, loFrom, upStart, upCol, upFrom;
    DevBuf<int> loColBase, upColBase;           // 16-bit column copies of the two parts (when both fit)
    DevBuf<unsigned short> loCol16, upCol16;
    bool col16 = false;
    int loMaxW = 0, upMaxW = 0;
    DevBuf<double> loVal, upVal, dinv;
    DevBuf<float> loVal32, upVal32, dinv32;
    DevBuf<double> aDiag;                      // diagonal of Ap per permuted row (the reduced iteration)
    DevBuf<float> aInv32;                      // 1 / aDiag in FP32
    Csr S;                                     // the explicit Schur complement of a two-colour factor (factor_schur)
    bool schurTried = false, hasSchur = false;
    DevBuf<__half> loVal16, upVal16;           // FP16 copies of the values (see FactorView)
    DevBuf<int> range16;                       // set by factor_fill when a value does not fit FP16's normal range
    bool has16 = false;
    int kind = 0;                              // NSF_PRECOND_NONE / IC0 / LEARNED
    double shift = 0.0;                        // diagonal shift the incomplete factorisation needed
    bool ready = false;
};

// One solve's outcome, written by the CG kernels (device) and read back by the host.
struct CgInfo {
    int iterations;      // inner iterations in total
    int status;          // nsf_status
    int outer;           // FP64 true-residual refreshes (mixed precision), 1 for the FP64 solver
    int fallback;        // 1: the mixed solver stalled and finished with the FP64 method
    double rr;           // final ||r||^2 (recursive residual; FP64 true residual for the mixed solver)
    double bb;           // ||b||^2
};

// grid-barrier word pair; zeroed before every persistent launch
struct GridSync {
    unsigned long long arrived;
    int abort;
    int where;
};

// Control state of a mixed-precision PCG solve: the recurrence scalars and counters, identical in every thread of
// the solve.  The split form keeps it in device memory between its refresh and inner-iteration kernels.
struct PcgLoop {
    double rr64, bb, target, rz, beta, rrBest, rrCycle, rrRef;
    double rr, rrPrev, cycleTol2;   // plain mixed CG: recursive r.r, its previous value, the cycle's tolerance
    double scale;            // the FP32 vectors hold the true residual times this power of two
    int lastCycle;
    int it, refresh, stalls, itRef;
    int first, resetP, flip, innerBreakdown;
    int rflip;               // which residual buffer is current (r32 or r32b; the fused inner iterations alternate)
    int state, status;
};
enum { kLoopInner = 1, kLoopRefresh = 2, kLoopDone = 3 };

// Kernel-level arguments of the persistent CG solvers.
struct CgArgs {
    int n;
    const int* rowptr;
    const int* col;
    const double* val;
    const float* val32;
    const float* rowsum32;   // row sums of the FP64 matrix, rounded once (mixed precision difference form)
    const int* sellStart;    // SELL-32 copy (null: the CSR arrays are used)
    const int* sellCol;
    const unsigned short* sellCol16;   // its 16-bit column copy (null: none)
    const int* sellColBase;
    const double* sellVal;
    const float* sellVal32;
    FactorView f;            // preconditioned solvers only
    const double* b;
    const double* x0;
    double* x;
    double* r;
    double* q;
    double* pbuf0;
    double* pbuf1;
    float* r32;      // mixed precision inner vectors
    float* r32b;     // (the split PCG's second residual buffer)
    float* d32;
    float* q32;
    float* p32a;
    float* p32b;
    double* partials;   // per-CTA partial sums: up to 9 regions of gridDim.x entries
    GridSync* sync;
    CgInfo* info;
    int maxIt;
    int fallbackMaxIt;       // preconditioned solvers: iteration budget of the plain-CG fallback (0: what is left)
    int sellMaxW;            // entries per row of the SELL copy's widest slice
    PcgLoop* loop;           // split mixed PCG: the control state between kernels
    int loopInit;            // split mixed PCG: this refresh kernel starts the solve
    double tol2;
    double innerTol2;
    int maxOuter;
    long long timeoutNs;
    // optional rhs construction fused into the solver prologue:
    //   b_i = bcMask[i] ? bcValue[i] : (Bm x_b)_i - lift[i]   (written to `bOut` and used as b)
    const int* bRowptr;
    const int* bCol;
    const double* bVal;
    const int* bSellStart;   // Bm's SELL-32 copy (null: the CSR arrays above are streamed)
    const int* bSellCol;
    const double* bSellVal;
    const double* bX;
    const double* lift;
    const unsigned char* bcMask;
    const double* bcValue;
    double* bOut;
    double* wbuf0;           // FP64 pipelined CG: the two buffers of w = A r
    double* wbuf1;
};

// Scalars of the multi-kernel FP64 CG (cg_multi_launch), kept on the device between its kernels.
struct CgMultiState {
    double rr, bb, target, alpha, beta;
    int it, status, done, maxIt;
    unsigned int arrived;   // CTAs of the running kernel that have posted their partial sums
};

// Page-locked host slots the multi-kernel CG's state is copied to after each graph replay, and the events the
// host waits on (created on first use, released with the workspace).
struct CgMultiHost {
    CgMultiState* slot = nullptr;   // two slots: one replay is checked while the next one runs
    cudaEvent_t ev[2] = {nullptr, nullptr};
    CgMultiHost() = default;
    CgMultiHost(const CgMultiHost&) = delete;
    CgMultiHost& operator=(const CgMultiHost&) = delete;
    ~CgMultiHost() {
        if (slot) cudaFreeHost(slot);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
};

// the workspace shared by every solve on a handle (sized for the largest system)
struct CgWorkspace {
    DevBuf<double> r, q, p0, p1, w, xp, bp;
    DevBuf<float> r32, r32b, d32, q32, p32a, p32b, w32;
    DevBuf<double> partials;
    DevBuf<GridSync> sync;
    DevBuf<CgInfo> info;     // ring of infos (one per solve in a step)
    DevBuf<PcgLoop> loop;    // split mixed PCG control state
    DevBuf<CgMultiState> multi;   // multi-kernel FP64 CG scalars
    CgMultiHost multiHost;
    int grid = 0;            // persistent grid size (blocks)
    int block = 0;
    int gridInner = 0;       // grid of the split mixed PCG's inner-iteration kernel
    int gridInner1024 = 0;   // (its one-CTA-per-SM form)
    bool pipeOk = false;     // the pipelined FP64 CG kernels are co-resident on `grid`
    size_t residentMaxBytes = 0;   // shared memory the resident inner PCG kernel may take (0: not offered)
};

// launch helpers implemented in nsf_cg.cu / nsf_sparse.cu
void cg_configure(CgWorkspace& ws, int device);
// wide: the matrix has slices wider than kSellChunk entries per row (the kernels' pipelined product for them)
constexpr int kSellChunk = 8;
void cg_launch(CgWorkspace& ws, const CgArgs& a, int mode, bool wide, cudaStream_t s);
// The FP64 CG with one grid barrier per iteration (pipelined recurrences; the matrix must have its SELL copy).
void cg_pipe_launch(CgWorkspace& ws, const CgArgs& a, bool wide, cudaStream_t s);
// The split mixed PCG (narrow matrices): refresh kernel, then inner-iteration and refresh kernels until the solve
// is done; one small device-to-host read per refresh cycle.
// Returns the inner-iteration kernel it ran (nsf_precond_inner_form's values).
int pcg_mixed_split_launch(CgWorkspace& ws, CgArgs a, cudaStream_t s);
// The split plain mixed CG (wide systems): the same launch pattern.
void cg_mixed_split_launch(CgWorkspace& ws, const CgArgs& a, cudaStream_t s);
// The FP64 CG as one ordinary launch per phase (NSF_CG_FORM_MULTI_KERNEL), replayed as CUDA graphs of several
// iterations; returns after the solve finished (the host polls its state once per replay).
void cg_multi_launch(CgWorkspace& ws, const CgArgs& a, bool wide, cudaStream_t s);
void spmv_launch(const Csr& A, const double* x, double* y, cudaStream_t s);
void spmv_rhs_launch(const Csr& A, const double* x, const double* lift, const unsigned char* mask,
                     const double* bcValue, double* y, cudaStream_t s);
void axpy_bc_launch(int n, const double* a, double* y, const unsigned char* mask, const double* bcValue,
                    cudaStream_t s);
void make_fp32_values(Csr& A, cudaStream_t s);
// SELL-32 copy (FP64 values; with fp32 also the FP32 values and row sums) for the CG kernels; no-op when current
void prepare_matrix(Csr& A, bool fp32, cudaStream_t s);
// 16-bit column copy of a SELL-32 column array (16-bit offsets from each slice's smallest column; kCol16Pad for
// padding entries of column -1 and, with noDiag, for the diagonal entries) when every slice's remaining columns
// span fewer than kCol16Pad; false, with nothing allocated, otherwise.  Synchronises the stream.
bool sell_col16(int nSlices, const int* start, const int* col, bool noDiag, DevBuf<int>& base,
                DevBuf<unsigned short>& col16, cudaStream_t s);
// The matrix's 16-bit column copy, after prepare_matrix (tried once per SELL copy), for the difference-form FP32
// product only: its diagonal entries are padding there, since the difference form's diagonal term
// a_ii (p_i - p_i) is exactly zero (and a row's own entry usually lies in another colour block of the permuted
// system than its neighbours, which would put the slice's columns far apart).
void prepare_col16(Csr& A, cudaStream_t s);

// preconditioner factors (nsf_precond.cu)
void factor_structure(Factor& F, const Csr& A, cudaStream_t s);
double factor_ic0(Factor& F, const Csr& A, cudaStream_t s);
void factor_fill(Factor& F, cudaStream_t s);
FactorView factor_view(const Factor& F, CgWorkspace& ws);
// The explicit Schur complement of a two-colour factor's permuted matrix with its SELL copies (once per factor, on the
// host; synchronises the stream).  False, with nothing kept, where its columns do not fit the 16-bit copy.
bool factor_schur(Factor& F, cudaStream_t s);

// ------------------------------------------------------------------------------------------------
// Mesh, point-location tree and simulation state
// ------------------------------------------------------------------------------------------------
struct LocateTree {
    int nLeaves = 0;          // padded to a power of two
    int leafSize = 0;
    int depth = 0;
    DevBuf<int> triSorted;    // [nLeaves * leafSize], -1 padded
    DevBuf<float4> box;       // heap-ordered node boxes (minx, miny, maxx, maxy), 2*nLeaves-1
};

struct MeshDev {
    int nNodes = 0, nEl = 0, nP = 0;
    DevBuf<float2> xy;
    DevBuf<int> el;
    std::vector<float> hxy;
    std::vector<int> hel;
    LocateTree tree;
};

void tree_build(MeshDev& m, cudaStream_t s);
void locate_launch(const MeshDev& m, int n, const float2* pts, int* elem, float* xi, float* eta, int* nearest,
                   cudaStream_t s);
void advect_launch(const MeshDev& m, double dt, const double* u, const double* v, double* uo, double* vo,
                   cudaStream_t s);
void advect_f32_launch(const MeshDev& m, float dt, const float* u, const float* v, float* uo, float* vo,
                       cudaStream_t s);

// A Dirichlet expression compiled for the device (nsfhost::BcOp codes; c holds the constants of kOpConst).
struct BcProgram {
    int n;
    int op[nsfhost::kBcMaxOps];
    double c[nsfhost::kBcMaxOps];
};

struct SimState {
    bool ready = false;
    double viscosity = 0, dt = 0;
    // simulated time of the resident fields: t0 + steps * dt, steps counted from the last nsf_sim_setup or
    // nsf_sim_set_bc_expressions
    double t0 = 0;
    long long steps = 0;
    std::vector<int> hOccV, hOccP;   // the Dirichlet occurrences (node per listed entry) given at setup
    // time-dependent Dirichlet data: programs evaluated on the device at the start of every step
    bool bcTimeDependent = false;
    DevBuf<BcProgram> bcProg;
    DevBuf<int> bcNodeV, bcOccStartV, bcProgU, bcProgV;   // distinct velocity Dirichlet nodes, their occurrences
    DevBuf<int> bcNodeP, bcOccStartP, bcProgP;
    int nBcNodeV = 0, nBcNodeP = 0;
    DevBuf<double> gSumV[2], gSumP;   // per node, the sum of its occurrences' values (the lift's weights)
    // the element colouring of the assembly (no two elements of a colour share a node), kept for the
    // explicit-convection step's matrix-free right-hand side
    DevBuf<int> elOrder;
    std::vector<int> elStart;
    int scheme = NSF_SCHEME_SEMI_LAGRANGIAN;
    DevBuf<double> uv, tmp, p, rhsV, rhsP;
    DevBuf<double> liftV[2], liftP;
    DevBuf<unsigned char> bcV, bcP;
    DevBuf<double> gV[2], gP;      // values imposed on Dirichlet rows (last listed occurrence wins)
    std::vector<double> hgV[2], hgP;
    std::vector<unsigned char> hbcV, hbcP;
    int nColours = 0;
};

// Time-dependent Dirichlet data (nsf_bc.cu): compiles the expressions, stores the programs and evaluates them at
// S.t0; bc_update_launch re-evaluates values, lift weights and lifts at time t on the stream.
void bc_set_programs(SimState& S, const MeshDev& m, Csr* mats, int nExpressions, const char* const* expressions,
                     const int* velocityU, const int* velocityV, const int* pressure, double t0, cudaStream_t s);
void bc_update_launch(SimState& S, const MeshDev& m, Csr* mats, double t, cudaStream_t s);

// rhs = -dt (C(u) + nu K) u for both velocity components (NavierStokesAssembly::solve's tentative-velocity
// right-hand side), matrix free, per element colour (nsf_assembly.cu).
void convection_rhs_launch(const MeshDev& m, const SimState& S, const double* uv, double* rhs, cudaStream_t s);

// One mesh instance of the batched form: its mesh and tree, matrices, fields and CG workspace.
struct Instance {
    MeshDev mesh;
    Csr mats[NSF_SLOT_COUNT];
    SimState sim;
    DevBuf<double> r, q, p0, p1;
    DevBuf<float> r32, d32, q32, p32a, p32b;
    DevBuf<double> partials;                 // 6 slots per CTA of the team
    DevBuf<CgInfo> info;                     // ring of kStepInfoCap steps x 5 solves
    DevBuf<int> stepCounter;
    DevBuf<unsigned long long> teamNs;       // duration of the team's last step (autotuner input)
    int blocks = 1;                          // team size (CTAs) in the current plan
    double work = 1.0;                       // autotuner's work estimate
};
constexpr int kStepInfoCap = 64;

// The persistent step kernel (nsf_step.cu)
int step_kernel_capacity(int device);

// Assembles every matrix of one mesh on the GPU (nsf_assembly.cu); returns the colour count.
int assemble_instance(MeshDev& m, SimState& sim, Csr* mats, cudaStream_t s, double viscosity, double dt);
// Upload, tree, BC data, assembly, lifts and initial fields of one instance (nsf_api.cu).
void setup_instance(MeshDev& m, SimState& S, Csr* mats, cudaStream_t s, int nNodes, const float* xy, int nElements,
                    const int* elements, int nPressure, int nU, const int* uNodes, const double* gu, const double* gv,
                    int nPb, const int* pNodes, const double* gp, double viscosity, double dt);

}  // namespace nsf

// the opaque handle behind the C ABI
struct nsf_device {
    int device = 0;
    int smCount = 0;
    cudaStream_t stream = nullptr;
    std::recursive_mutex mu;
    std::string lastError;
    nsf::Csr mats[NSF_SLOT_COUNT];
    nsf::CgWorkspace ws;
    nsf::MeshDev mesh;
    nsf::SimState sim;
    nsf::DevBuf<double> scratch[4];   // host-pointer entry points stage their vectors here
    nsf::DevBuf<unsigned char> flush; // L2 eviction buffer (nsf_flush_l2)
    unsigned flushToggle = 0;
    double tol = 1e-8;
    double innerTol = 0.1;   // mixed precision: FP32 residual reduction between FP64 true residuals
    long long timeoutNs = 2000000000LL;
    int solverMode = NSF_SOLVER_FP64;
    int pcgForm = NSF_PCG_FORM_AUTO;   // mixed PCG of a two-colour system: full or reduced iteration
    int cgForm = NSF_CG_FORM_AUTO;   // plain FP64 CG: three barriers per iteration or pipelined (one)
    bool mixedOff[NSF_SLOT_COUNT] = {};   // systems whose mixed solve stalled once: solved in FP64 from then on
    nsf::Factor factors[NSF_SLOT_COUNT];  // preconditioners
    int pcgCap[NSF_SLOT_COUNT] = {};      // iteration cap of a preconditioned solve (0: rows)
    int innerForm[NSF_SLOT_COUNT] = {-1, -1, -1, -1, -1, -1, -1};   // the last split mixed PCG's inner kernel
    bool pcgOff[NSF_SLOT_COUNT] = {};     // systems whose preconditioned solve fell back: plain CG from then on
    // per-solve records (profiling of the persistent CG kernels)
    bool profile = false;
    std::vector<cudaEvent_t> evPool;
    size_t evUsed = 0;
    struct SolveRecord { int slot; int mode; int rows; int64_t nnz; cudaEvent_t a, b; int infoIndex; };
    std::vector<SolveRecord> records;
    int infoCursor = 0;
    std::vector<int> infoMode;               // solver mode each info slot's solve ran with
    // batched form: instances, the launch plan and the captured step graph
    std::vector<std::unique_ptr<nsf::Instance>> batch;
    nsf::DevBuf<unsigned char> batchDesc;    // StepInstance array (nsf_step.cu)
    nsf::DevBuf<int> batchBlockInst;
    nsf::DevBuf<nsf::GridSync> batchSync;
    int batchGrid = 0;
    int batchCapacity = 0;                   // co-resident CTAs of the step kernel
    bool batchReady = false;
    cudaGraph_t batchGraph = nullptr;
    cudaGraphExec_t batchGraphExec = nullptr;
    int batchStepsDone = 0;
    std::vector<int> autotuneLog;            // team sizes tried, flattened per round
    std::vector<double> autotuneMs;          // step time of each round
};

namespace nsf {
// the slot's factor with its pattern built (values too when needValues); nsf_api.cu
Factor& factor_for(nsf_device* h, int slot, bool needValues);
void batch_upload_plan(nsf_device* h);
void batch_launch_step(nsf_device* h);
void batch_autotune(nsf_device* h, int rounds);
void batch_capture_graph(nsf_device* h);
}  // namespace nsf
