/*
 * nsfem_gb300.h — C ABI of the GB300 (sm_103a) per-time-step hot path of the P2-P1 Taylor-Hood
 * Navier-Stokes solver (semi-Lagrangian advection, implicit diffusion, pressure projection).
 *
 * The entry points replace, one for one, the GPU device layer the reference solver calls from its
 * assembly driver (vasil-pashov/Navier_Stokes_FEM):
 *   GPUSimulationDeviceManager::init / getDevice   include/gpu_simulation_device.h:208-220, cpp/gpu_simulation_device.cpp:518-550
 *   GPUSimulationDevice::uploadKDTree              cpp/gpu_simulation_device.cpp:72-77
 *   GPUSimulationDevice::uploadMatrix              include/gpu_simulation_device.h:28, cpp/gpu_simulation_device.cpp:133-140
 *   GPUSimulationDevice::advect                    include/gpu_simulation_device.h:29-36, cpp/gpu_simulation_device.cpp:91-131
 *   GPUSimulationDevice::spRMult                   include/gpu_simulation_device.h:38-48, cpp/gpu_simulation_device.cpp:142-165
 *   GPUSimulationDevice::conjugateGradient         include/gpu_simulation_device.h:62-76, cpp/gpu_simulation_device.cpp:293-515
 *   KDTree::findElement (point location)           gpu_cpu_shared/kd_tree.cuh:40-141
 * plus a simulation-level surface that keeps the whole operator-split step resident on the GPU, replacing the
 * per-step host loop of NavierStokesAssembly::semiLagrangianSolve (include/assembly.h:1477-1557) together with
 * assembleAllMatrices (include/assembly.h:1302-1475).
 *
 * Conventions
 *   - Every function returns an nsf_status; 0 is success.  nsf_last_error() gives the message of the last
 *     failure on a handle (the reference's EC::ErrorCode{status, message}, include/error_code.h:9-39).
 *   - Pointers are HOST memory unless the name ends in _dev; calls with host pointers are synchronous.
 *   - The library owns all device memory; callers own host arrays.  A handle may be used from several
 *     threads (calls are serialised by an internal lock, as the reference's concurrent uploadMatrix calls
 *     from TBB tasks require, include/assembly.h:1330,1381,1422).  One CUDA stream per handle.
 *   - Node coordinates are float [x0,y0,x1,y1,...]; elements are int [v0,v1,v2,m12,m02,m01] per triangle,
 *     counter-clockwise; pressure nodes are the first nPressure nodes.
 *   - Solves stop on the RELATIVE residual ||b - A x|| <= eps * ||b|| (eps * ||r0|| when b = 0).  The
 *     reference's GPU CG stops on the absolute ||r||^2 < eps^2 (cpp/gpu_simulation_device.cpp:405,446,511).
 *   - A solve that does not converge still writes its last iterate and returns NSF_ERR_NOT_CONVERGED (the
 *     reference leaves x unwritten); an initial guess that already converges is copied to x.
 */
#ifndef NSFEM_GB300_H
#define NSFEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nsf_device nsf_device;

enum nsf_status {
    NSF_OK = 0,
    NSF_ERR_CUDA = 1,             /* a CUDA runtime call failed (message carries file:line) */
    NSF_ERR_NOT_CONVERGED = 2,    /* "Max iterations reached!" (cpp/gpu_simulation_device.cpp:382,514) */
    NSF_ERR_BREAKDOWN = 3,        /* CG breakdown: p.Ap <= 0 or a non-finite scalar (matrix not SPD, NaN input) */
    NSF_ERR_BARRIER_TIMEOUT = 4,  /* a grid-wide wait inside a persistent kernel ran past its time limit */
    NSF_ERR_BAD_ARG = 5,
    NSF_ERR_STATE = 6,            /* call order violated, e.g. stepping before nsf_sim_setup */
    NSF_ERR_NO_DEVICE = 7
};

/* Matrix slots.  0-4 are GPUSimulationDevice::SimMatrix (include/gpu_simulation_device.h:16-24); 5 and 6 hold
 * the Dirichlet lift weights (velocityDirichletWeights / pressureDirichletWeights, include/assembly.h:363-380),
 * stored row = free node, column = Dirichlet node. */
enum nsf_slot {
    NSF_PRESSURE_STIFFNESS = 0,
    NSF_VELOCITY_MASS = 1,
    NSF_DIFFUSION = 2,
    NSF_VELOCITY_DIVERGENCE = 3,   /* -(1/dt) * Div, P x 2Nv */
    NSF_PRESSURE_DIVERGENCE = 4,   /* -dt * Grad, 2Nv x P */
    NSF_VELOCITY_LIFT = 5,
    NSF_PRESSURE_LIFT = 6,
    NSF_SLOT_COUNT = 7
};

/* CG variants */
enum nsf_solver {
    NSF_SOLVER_FP64 = 0,       /* persistent FP64 CG megakernel: the plain method */
    NSF_SOLVER_MIXED = 1,      /* FP32 matrix/vectors inside, FP64 dots and scalars, FP64 iterative refinement */
    NSF_SOLVER_PCG_MIXED = 2,  /* mixed precision with the slot's preconditioner (plain mixed CG if it has none) */
    NSF_SOLVER_PCG_FP64 = 3    /* FP64 PCG with the slot's preconditioner (plain FP64 CG if it has none) */
};

/* Iteration form of the plain FP64 CG megakernel (nsf_set_cg_form).  The reference's megakernel joins 4 grid-wide
 * syncs per iteration (gpu/matrix_math.cu:251-286). */
enum nsf_cg_form {
    NSF_CG_FORM_AUTO = 0,       /* pipelined below NSF_CG_PIPELINED_MAX_ROWS rows, three barriers above */
    NSF_CG_FORM_THREE_SYNC = 1, /* q = A p and p.q | x, r and r.r | p = r + beta p: three grid barriers */
    NSF_CG_FORM_PIPELINED = 2,  /* one grid barrier per iteration: the recurrences of pipelined CG (Ghysels and
                                 * Vanroose 2014) carry A r, A p and A A p, so the one product per iteration acts on
                                 * a vector finished before the barrier; two more vector passes and about five more
                                 * FP64 operations per row, and a final true-residual check */
    NSF_CG_FORM_MULTI_KERNEL = 3 /* the reference's conjugateGradientMultiKernel (cpp/gpu_simulation_device.cpp:
                                 * 293-383, its conjugateGradient(..., useMegakernel = false)): one ordinary launch
                                 * per phase (q = A p with p.q; x, r and r.r; p = r + beta p), the kernel boundaries
                                 * as the grid-wide syncs, alpha and beta computed on the device by the last CTA of
                                 * each reduction, 8 iterations per CUDA graph replay and the host reading the
                                 * stopping state once per replay instead of twice per iteration */
};

/* Iteration form of the split mixed PCG on a two-colour system (nsf_set_pcg_form).  The reference preconditions
 * with IC0 under USE_PRECONDITIONING (include/assembly.h:33-35, 1338-1344) and has no reduced form. */
enum nsf_pcg_form {
    NSF_PCG_FORM_AUTO = 0,     /* reduced where the system has two colours, with the Schur complement formed
                                * explicitly where its 16-bit column copy fits (NSF_PCG_FORM_SCHUR), else full */
    NSF_PCG_FORM_FULL = 1,     /* PCG on the whole permuted system: product, forward and backward colour sweeps */
    NSF_PCG_FORM_REDUCED = 2,  /* two colours only (else full): the colour-0 unknowns are eliminated exactly (their
                                * block of a two-colour matrix is diagonal) and PCG runs on the Schur complement with
                                * the factor's colour-1 diagonal as preconditioner.  With IC(0) these are the full
                                * form's iterates in exact arithmetic; each iteration reads every matrix row once and
                                * no factor part (85 against 119 us per iteration on the 2048 cavity's pressure
                                * system), while its FP32 iterations take about 5 % more of them there (the Schur
                                * complement's near-constant mode is resolved less well in FP32); the product
                                * S p = A_10 u + A_11 p through u = -A_00^-1 A_01 p, two phases */
    NSF_PCG_FORM_SCHUR = 3     /* the reduced iteration with S = A_11 - A_10 A_00^-1 A_01 formed once on the host
                                * (9 entries per row on the structured meshes): one product phase and two grid
                                * barriers per iteration, the difference form with S's own FP64 row sums */
};

/* NSF_CG_FORM_AUTO's crossover, from GB300 measurements of both forms on the cavity and channel systems */
#define NSF_CG_PIPELINED_MAX_ROWS 2000000

/* preconditioner kinds (nsf_precond_kind) */
enum nsf_precond {
    NSF_PRECOND_NONE = 0,
    NSF_PRECOND_IC0 = 1,       /* incomplete Cholesky on the multicolour pattern */
    NSF_PRECOND_LEARNED = 2    /* factor values installed by nsf_precond_set (the learned preconditioner) */
};

/* ---- device (GPUSimulationDeviceManager::init + getDevice) ------------------------------------------- */
int nsf_create(int device, nsf_device** out);
void nsf_destroy(nsf_device* h);
const char* nsf_last_error(const nsf_device* h);
int nsf_device_info(nsf_device* h, int* smCount, int* cgGridBlocks, int* cgBlockThreads);
int nsf_synchronize(nsf_device* h);

/* ---- matrices (GPUSimulationDevice::uploadMatrix; GPUSparseMatrix::upload, cpp/gpu_sparse_matrix.cpp:7-50) */
/* CSR with rows grouped and columns ascending within a row (the order GPUSparseMatrix::upload asserts). */
int nsf_upload_matrix_csr(nsf_device* h, int slot, int rows, int cols, int64_t nnz, const int* rowptr,
                          const int* col, const double* val);
/* Triplets in any order; duplicates are summed (SMM::TripletMatrix semantics). */
int nsf_upload_matrix_triplets(nsf_device* h, int slot, int rows, int cols, int64_t count, const int* row,
                               const int* col, const double* val);
int nsf_matrix_shape(nsf_device* h, int slot, int* rows, int* cols, int64_t* nnz);
int nsf_download_matrix(nsf_device* h, int slot, int* rowptr, int* col, double* val);

/* ---- sparse algebra (spRMult; conjugateGradient) ----------------------------------------------------- */
int nsf_spmv(nsf_device* h, int slot, const double* x, double* y);
/* mode: nsf_solver.  maxIterations -1 means `rows` (cpp/gpu_simulation_device.cpp:449).  iterations and
 * relResidual may be NULL. */
int nsf_conjugate_gradient(nsf_device* h, int slot, const double* b, const double* x0, double* x,
                           int maxIterations, double eps, int mode, int* iterations, double* relResidual);
/* The reference's own float signature (include/gpu_simulation_device.h:62-76); computes in FP64. */
int nsf_conjugate_gradient_f32(nsf_device* h, int slot, const float* b, const float* x0, float* x,
                               int maxIterations, float eps);
/* Device-pointer form, asynchronous on the handle's stream except for the status read-back. */
int nsf_conjugate_gradient_dev(nsf_device* h, int slot, const double* b_dev, const double* x0_dev, double* x_dev,
                               int maxIterations, double eps, int mode, int* iterations, double* relResidual);

/* ---- preconditioners (IC0Preconditioner under USE_PRECONDITIONING, include/assembly.h:33-35, 1338-1344) -----
 * M = L L^T in multicolour order: the graph of the slot's non-zero entries is coloured by DSatur (most distinct
 * neighbour colours first; ties: more neighbours, then the lower row), and L_ij (i != j) lives on the non-zeros
 * where colour(j) < colour(i).  The solve runs on the colour-permuted matrix.  A preconditioned solve
 * (NSF_SOLVER_PCG_*) that has not converged after the slot's cap of iterations finishes with plain FP64 CG from
 * its current iterate, within the caller's own iteration budget. */
/* Builds the pattern; colours and the number of strictly lower entries may be NULL. */
int nsf_precond_pattern(nsf_device* h, int slot, int* colours, int64_t* nnzLower);
/* The pattern: rowptr[rows + 1] and col[nnzLower] of the strictly lower part, entries of a row ordered by
 * (colour, column), and colour[rows]. */
int nsf_precond_get_pattern(nsf_device* h, int slot, int* rowptr, int* col, unsigned char* colour);
/* Incomplete Cholesky on the pattern, retried with a diagonal shift a_ii (1 + shift) on breakdown. */
int nsf_precond_ic0(nsf_device* h, int slot, double* shiftUsed);
/* Installs factor values (host arrays): lower[nnzLower] on the pattern and diag[rows] = L_ii > 0. */
int nsf_precond_set(nsf_device* h, int slot, const double* lower, const double* diag);
int nsf_precond_get(nsf_device* h, int slot, double* lower, double* diag);
int nsf_precond_kind(nsf_device* h, int slot);
/* Bytes per column index that the FP32 iterations of the slot's mixed PCG read: 2 when its colour-permuted matrix
 * and both factor parts have 16-bit column copies (every 32-row slice's columns within 65535 of each other; decided
 * by the slot's first mixed PCG solve), else 4. */
int nsf_precond_index_bytes(nsf_device* h, int slot);
/* Bytes per factor value that the mixed PCG's FP32 iterations read: 2 when every factor value fits FP16's normal
 * range (the factor then keeps FP16 copies, and its FP32 copies hold the same rounded values, so that every FP32
 * sweep applies the same M), else 4. */
int nsf_precond_value_bytes(nsf_device* h, int slot);
/* The inner-iteration kernel the slot's last split mixed PCG solve ran: 0 four 256-thread CTAs per SM (one colour),
 * 1 one 1024-thread CTA per SM, 2 the same with the row state only a CTA reads resident in its shared memory (two
 * colours, where it fits), 3 the reduced (Schur complement) iteration of nsf_pcg_form, 4 the same with its
 * CTA-private row state resident in shared memory, 5 and 6 the same two with the Schur complement formed
 * explicitly; -1 before the slot's first such solve. */
int nsf_precond_inner_form(nsf_device* h, int slot, int* form);
/* Entries of the slot's explicitly formed Schur complement (NSF_PCG_FORM_SCHUR; 0 before its first such solve). */
int nsf_precond_schur_nnz(nsf_device* h, int slot, int64_t* nnz);
int nsf_precond_clear(nsf_device* h, int slot);
/* Iterations a preconditioned solve of this slot may take before it falls back (0: the matrix size). */
int nsf_precond_cap(nsf_device* h, int slot, int maxIterations);

/* ---- the learned preconditioner ----------------------------------------------------------------------
 * An edge-based message-passing network over the factor pattern's graph outputs L (M = L L^T) for a system
 * matrix; trained on the GPU (forward, backward and Adam kernels; BF16 tensor-core layers with FP32 accumulation)
 * on pairs (A, x, b) the plain method produced, with loss ||L^ L^T x^ - b^||^2 / ||b^||^2 on the diagonally scaled
 * system.  The learner is bound to a device handle and uses its stream. */
typedef struct nsf_learner nsf_learner;
int nsf_learn_create(nsf_device* h, uint64_t seed, nsf_learner** out);
void nsf_learn_destroy(nsf_learner* L);
const char* nsf_learn_last_error(const nsf_learner* L);
int nsf_learn_param_count(nsf_learner* L, int64_t* count);
int nsf_learn_get_params(nsf_learner* L, float* theta);
/* Replaces the parameters (and resets the Adam state). */
int nsf_learn_set_params(nsf_learner* L, const float* theta);
/* Stores a training system: the slot's current matrix (its graph and features) with a solution x of A x = b. */
int nsf_learn_add_system(nsf_learner* L, int slot, const double* x, const double* b, int* index);
int nsf_learn_clear_systems(nsf_learner* L);
int nsf_learn_system_size(nsf_learner* L, int index, int* nodes, int64_t* edges);
/* The network's scaled factor on a stored system: lower[edges] (factor pattern order), diag[nodes]. */
int nsf_learn_forward(nsf_learner* L, int index, float* lower, float* diag);
/* Loss of a stored system and its gradient with respect to the parameters. */
int nsf_learn_loss_grad(nsf_learner* L, int index, double* loss, float* grad);
/* `steps` Adam steps, each on the mean gradient of `batch` systems drawn from the store; losses[steps] or NULL. */
int nsf_learn_train(nsf_learner* L, int steps, int batch, double lr, uint64_t seed, float* losses);
/* Runs the network on the slot's matrix of `target` (NULL: the learner's own handle; same GPU) and installs its
 * factor as that slot's preconditioner. */
int nsf_learn_apply(nsf_learner* L, nsf_device* target, int slot);
/* One tensor-core dense layer on host arrays: Y[rows x N] = epilogue(X[rows x K] W[K x N] + bias), X and W
 * rounded to BF16, FP32 accumulation; epilogue 0 none, 1 ReLU; K and N multiples of 16 up to 128. */
int nsf_tc_dense(nsf_device* h, int rows, int K, int N, const float* X, const float* W, const float* bias,
                 int epilogue, float* Y);
/* A dense layer's weight gradients on the tensor cores, on host arrays: dW[K x N] = X^T G and db[N] = the column
 * sums of G, for X[rows x K] and G[rows x N] rounded to BF16, FP32 accumulation; K + 1 <= 128, N a multiple of 16
 * up to 128. */
int nsf_tc_weight_gradient(nsf_device* h, int rows, int K, int N, const float* X, const float* G, float* dW,
                           float* db);

/* ---- mesh, point location and advection (uploadKDTree; advect; KDTree::findElement) ------------------ */
/* Uploads the mesh and builds the point-location tree on the GPU over triangle centroids. */
int nsf_upload_mesh(nsf_device* h, int nNodes, const float* xy, int nElements, const int* elements, int nPressure);
/* Containing element of each point, with the reference's semantics: the lowest-index triangle whose closed
 * vertex bounding box holds the point and whose barycentric test passes (bit-exact float predicate);
 * elem = -1 and `nearest` = closest mesh node (ties -> lowest index) when no triangle contains it. */
int nsf_locate(nsf_device* h, int n, const float* pts, int* elem, float* xi, float* eta, int* nearest);
/* The reference's advect signature: float velocities in host memory, synchronous. */
int nsf_advect(nsf_device* h, int numNodes, const float* u, const float* v, float dt, float* uOut, float* vOut);
int nsf_advect_f64(nsf_device* h, int numNodes, const double* u, const double* v, double dt, double* uOut,
                   double* vOut);

/* ---- resident simulation (NavierStokesAssembly::init + assembleAllMatrices + semiLagrangianSolve) ---- */
/* Dirichlet data are given per listed occurrence, in the mesh file's group order, with their evaluated
 * values (FemGrid2D::VelocityDirichlet / PressureDirichlet, include/grid.h:13-60).  Assembles every matrix
 * on the GPU and sets u = 0 with Dirichlet values imposed, p = 0. */
int nsf_sim_setup(nsf_device* h, int nNodes, const float* xy, int nElements, const int* elements, int nPressure,
                  int nVelocityBC, const int* velocityBCNodes, const double* bcU, const double* bcV,
                  int nPressureBC, const int* pressureBCNodes, const double* bcP, double viscosity, double dt);
int nsf_sim_set_fields(nsf_device* h, const double* uv, const double* p);   /* uv = [u(Nv) | v(Nv)] */
int nsf_sim_get_fields(nsf_device* h, double* uv, double* p);
/* Runs nsteps operator-split steps on the resident fields.  iterations (5 per step: diffusion u, diffusion v,
 * pressure, mass u, mass v) may be NULL. */
int nsf_sim_step(nsf_device* h, int nsteps, int* iterations);
/* The same, from and to host fields (the reference's host-visible velocity/pressure vectors). */
int nsf_sim_step_host(nsf_device* h, const double* uvIn, const double* pIn, int nsteps, double* uvOut,
                      double* pOut, int* iterations);

/* Operator-split scheme of nsf_sim_step (nsf_sim_set_scheme). */
enum nsf_scheme {
    NSF_SCHEME_SEMI_LAGRANGIAN = 0,     /* NavierStokesAssembly::semiLagrangianSolve (include/assembly.h:1477-1557):
                                         * semi-Lagrangian advection, implicit diffusion, pressure projection */
    NSF_SCHEME_EXPLICIT_CONVECTION = 1  /* NavierStokesAssembly::solve (include/assembly.h:1065-1299), a path the
                                         * reference's driver never calls: tentative velocity M y = -dt (C(u) + nu K) u
                                         * with the convection matrix of the current velocity (include/assembly.h:
                                         * 1581-1625), u += y, Dirichlet values imposed; the same pressure solve; the
                                         * correction M y = -dt Grad p, u += y.  C and K are applied matrix free per
                                         * element.  iterations: tentative u, v, pressure, correction u, v */
};
/* Selects the scheme of the following nsf_sim_step calls (NSF_ERR_STATE before nsf_sim_setup). */
int nsf_sim_set_scheme(nsf_device* h, int scheme);

/* Time-dependent Dirichlet data.  The reference's expression grammar accepts the variable t
 * (cpp/expression.cpp:167-177) but its imposeVelocityDirichlet (include/assembly.h:1559-1579) evaluates the
 * expressions with x and y only; this replaces those host evaluations by device-side ones that may use t.
 * expressions: nExpressions strings in the mesh-file grammar (variables x, y and t; at most 64 operations and a
 * stack depth of 16 each).  velocityU / velocityV: for every velocity Dirichlet occurrence given to nsf_sim_setup,
 * in that order, the index of its u and v expression; pressure: the same for the pressure occurrences.  The call
 * evaluates the data at t0 (imposed values, lifts) and imposes the velocity values on the resident field, as the
 * set-up imposes the constant data; step k after it then uses the data at t0 + k dt, the time the step ends, for
 * its right-hand sides, lifts and re-imposed values (one small kernel and three CSR products per step).  The
 * data stay time-dependent until the next nsf_sim_setup.  The batched form does not take expressions. */
int nsf_sim_set_bc_expressions(nsf_device* h, int nExpressions, const char* const* expressions, const int* velocityU,
                               const int* velocityV, const int* pressure, double t0);
/* Simulated time of the resident fields: t0 (0 after nsf_sim_setup) + steps taken since then x dt. */
int nsf_sim_time(nsf_device* h, double* t);

/* ---- batched form: many independent instances in one persistent launch per step -------------------- */
/* No single counterpart in the reference, which runs one mesh per process: each instance is a complete
 * NavierStokesAssembly problem (same arguments as nsf_sim_setup).  nsf_batch_add assembles one instance and
 * returns its index; nsf_batch_finalize divides the co-resident CTAs among the instances (an autotuner times
 * `autotuneRounds` trial steps on saved fields and keeps the fastest split) and captures the step as a CUDA
 * graph; nsf_batch_step replays it.  iterations: nsteps x count x 5 (diffusion u, v, pressure, mass u, v). */
int nsf_batch_clear(nsf_device* h);
int nsf_batch_add(nsf_device* h, int nNodes, const float* xy, int nElements, const int* elements, int nPressure,
                  int nVelocityBC, const int* velocityBCNodes, const double* bcU, const double* bcV, int nPressureBC,
                  const int* pressureBCNodes, const double* bcP, double viscosity, double dt, int* index);
int nsf_batch_finalize(nsf_device* h, int autotuneRounds);
int nsf_batch_step(nsf_device* h, int nsteps, int* iterations);
int nsf_batch_get_fields(nsf_device* h, int index, double* uv, double* p);
int nsf_batch_set_fields(nsf_device* h, int index, const double* uv, const double* p);
/* The plan in use: CTAs per instance (count entries), total CTAs, and the autotuner's trial step times. */
int nsf_batch_plan(nsf_device* h, int* blocks, int* gridBlocks, float* trialMs, int maxTrials, int* nTrials);

/* ---- configuration, timing, pinned memory ------------------------------------------------------------ */
int nsf_set_tolerance(nsf_device* h, double eps);
int nsf_set_solver(nsf_device* h, int mode, double innerTolerance);
/* form: nsf_cg_form; applies to the plain FP64 CG solves of this handle (the iteration count is that of CG up to
 * rounding: the pipelined recurrences may take a few more iterations on ill-conditioned systems). */
int nsf_set_cg_form(nsf_device* h, int form);
/* form: nsf_pcg_form; applies to the mixed-precision PCG solves (NSF_SOLVER_PCG_MIXED) of narrow systems. */
int nsf_set_pcg_form(nsf_device* h, int form);
int nsf_set_barrier_timeout(nsf_device* h, double seconds);
/* Records CUDA events around every persistent CG launch while enabled (clears previous records). */
int nsf_profile(nsf_device* h, int enable);
/* Returns the number of records written (<= maxRecords).  mode: the nsf_solver that ran; fallback: 1 if the solve
 * finished with plain FP64 CG (a stalled mixed solve, or a preconditioned one over its cap); outer: FP64
 * true-residual refreshes of a mixed solve. */
int nsf_profile_read(nsf_device* h, int maxRecords, int* slot, int* mode, int* fallback, int* rows, int64_t* nnz, int* iterations,
                     int* outer, float* ms);
/* op 0 records a start event on the handle's stream, op 1 a stop event and writes the elapsed ms. */
int nsf_timer(nsf_device* h, int op, float* ms);
/* Page-locked host memory of `bytes` bytes, zeroed and mapped for the device.  Field transfers to or from it
   (nsf_sim_set_fields, nsf_sim_get_fields, nsf_sim_step_host) run as copy kernels on the handle's stream: on a
   coherent CPU-GPU link the copy engines are slow for a while after GPU work (12-24 ms against 1.7 ms for 302 MB
   after a 2048-cavity step).  Other host pointers are copied with cudaMemcpyAsync.  Free with nsf_host_free. */
int nsf_host_alloc(nsf_device* h, size_t bytes, void** ptr);
int nsf_host_free(nsf_device* h, void* ptr);
/* Number of kernels this handle has launched so far (all of the library's own kernels, memsets excluded). */
int nsf_launch_count(nsf_device* h, int64_t* launches);
/* Overwrites a device buffer of `bytes` bytes on the handle's stream (evicts the L2 between timed steps). */
int nsf_flush_l2(nsf_device* h, size_t bytes);

/* ---- allocation-free solve ----------------------------------------------------------------------------- */
/* No counterpart in the reference.  The FP64 CG solve for callers that cannot call cudaMalloc: a host
 * application whose device memory is all owned by its own pool or fixed budget, or a time-critical loop where a
 * cudaMalloc (which can synchronise the device) is not acceptable.  Needs no handle and allocates nothing: the
 * caller passes the CSR matrix (int32 indices, columns ascending per row), b, x0 and x in device memory it
 * owns; the solver's work vectors live in an 8 MB array compiled into the library, which every GPU that loads
 * the library holds until exit.  rows <= NSF_NOALLOC_MAX_ROWS, else NSF_ERR_BAD_ARG with a message on stderr.
 * The matrix is square (rows x rows) with rowptr[0] = 0, rowptr ascending and 0 <= col < rows; these device
 * arrays are not checked (unlike nsf_upload_matrix_csr), so a column index outside [0, rows) reads outside the
 * caller's vectors.
 * The first call on each device looks up that array's device address (cudaGetSymbolAddress) with the device
 * current and keeps it for the rest of the process; make that first call before any stream capture.  After a
 * cudaDeviceReset (or any teardown of the device's primary context) the kept address is stale: do not call this
 * entry point on that device again in the same process.  Calls share the array: calls that overlap on the
 * GPU (other streams or threads) race, so serialise them.  Runs on `stream` (a cudaStream_t, NULL = default)
 * and returns after the solve finished; statuses as nsf_conjugate_gradient, except that the grid-barrier time
 * limit is fixed at 2 s (nsf_set_barrier_timeout applies to handles only). */
#define NSF_NOALLOC_MAX_ROWS 262144
int nsf_conjugate_gradient_noalloc(int rows, const int* rowptr_dev, const int* col_dev, const double* val_dev,
                                   const double* b_dev, const double* x0_dev, double* x_dev, int maxIterations,
                                   double eps, void* stream, int* iterations, double* relResidual);

/* ---- mesh-file boundary expressions (Expression::init + evaluate, cpp/expression.cpp:308-431) ---------- */
/* Evaluates `expression` at (x, y) in double precision.  NSF_ERR_BAD_ARG on a parse error or a variable
 * other than x and y; the message is written to `message` (may be NULL) up to `messageBytes`. */
int nsf_eval_expression(const char* expression, double x, double y, double* value, char* message,
                        size_t messageBytes);
/* The same with the variable t as well, evaluated on the host through the postfix program that
 * nsf_sim_set_bc_expressions compiles for the device, op for op as the device runs it. */
int nsf_eval_expression_t(const char* expression, double x, double y, double t, double* value, char* message,
                          size_t messageBytes);

#ifdef __cplusplus
}
#endif
#endif /* NSFEM_GB300_H */
