// Allocation-free variant of the FP64 CG solve, for callers that cannot call cudaMalloc.
//
// Who needs it: an application that owns all device memory through its own pool or fixed budget and hands the
// solver only the buffers it should touch, or a time-critical loop in which a cudaMalloc is not acceptable
// because it can synchronise the device and stall the other streams.  Such a caller passes the CSR matrix, the
// right-hand side, the initial guess and the output vector in device memory it owns; the solver's own work
// vectors live in a fixed array compiled into this library instead of being allocated.
//
// The array is a file-scope __device__ variable: every GPU that loads the library holds it (8.05 MB: four work
// vectors of NSF_NOALLOC_MAX_ROWS doubles plus reduction slots) until the process exits.  Host code never dereferences its name (on the host it is only a stand-in symbol); the
// device address is obtained with cudaGetSymbolAddress once per device, on the first call made while that
// device is current, so that first call on each device should come before any stream capture.
//
// Calls share the array and it keeps the previous call's contents; the kernel re-initialises everything it
// reads (the barrier word is cleared on the stream before every launch).  Calls whose kernels overlap on the GPU
// (two streams at once, or two host threads) race on the array: serialise them.
#include "nsf_internal.cuh"

#include <cmath>
#include <mutex>

namespace nsf {

int cg_fp64_grid(int device, int* block);
void cg_launch_fp64_raw(const CgArgs& args, int grid, int block, cudaStream_t s);

namespace {

constexpr int kMaxRows = NSF_NOALLOC_MAX_ROWS;
constexpr int kMaxBlocks = 1024;
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
    double r[kMaxRows];
    double q[kMaxRows];
    double p0[kMaxRows];
    double p1[kMaxRows];
    double partials[6 * kMaxBlocks];
    GridSync sync;
    CgInfo info;
};

static __device__ __align__(256) NoAllocScratch g_scratch;

struct DeviceSetup {
    bool ready = false;
    NoAllocScratch* scratch = nullptr;   // device address of g_scratch on this device
    int grid = 0;
    int block = 0;
};

std::mutex g_setupMutex;
DeviceSetup g_setup[kMaxDevices];

// Once per device, with that device current: the device address of the scratch and the persistent grid.
DeviceSetup& setup_current_device() {
    int dev = 0;
    NSF_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw bad_arg("device index beyond the supported range");
    std::lock_guard<std::mutex> lk(g_setupMutex);
    DeviceSetup& s = g_setup[dev];
    if (!s.ready) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_scratch);
        if (e != cudaSuccess)
            throw Error{NSF_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch) failed: ") + cudaGetErrorString(e)};
        s.grid = cg_fp64_grid(dev, &s.block);
        if (s.grid > kMaxBlocks) s.grid = kMaxBlocks;
        s.scratch = static_cast<NoAllocScratch*>(ptr);
        s.ready = true;
    }
    return s;
}

}  // namespace
}  // namespace nsf

extern "C" int nsf_conjugate_gradient_noalloc(int rows, const int* rowptr_dev, const int* col_dev,
                                              const double* val_dev, const double* b_dev, const double* x0_dev,
                                              double* x_dev, int maxIterations, double eps, void* stream,
                                              int* iterations, double* relResidual) {
    using namespace nsf;
    try {
        if (rows <= 0) throw bad_arg("rows must be positive");
        if (rows > kMaxRows)
            throw bad_arg("rows = " + std::to_string(rows) + " exceeds the allocation-free solver's limit of " +
                          std::to_string(kMaxRows) + " rows");
        if (!rowptr_dev || !col_dev || !val_dev || !b_dev || !x0_dev || !x_dev) throw bad_arg("null device pointer");
        if (!(eps > 0)) throw bad_arg("eps must be positive");
        DeviceSetup& s = setup_current_device();
        NoAllocScratch* w = s.scratch;
        const cudaStream_t st = static_cast<cudaStream_t>(stream);
        CgArgs a{};
        a.n = rows;
        a.rowptr = rowptr_dev;
        a.col = col_dev;
        a.val = val_dev;
        a.b = b_dev;
        a.x0 = x0_dev;
        a.x = x_dev;
        a.r = w->r;
        a.q = w->q;
        a.pbuf0 = w->p0;
        a.pbuf1 = w->p1;
        a.partials = w->partials;
        a.sync = &w->sync;
        a.info = &w->info;
        a.maxIt = maxIterations < 0 ? rows : maxIterations;
        a.tol2 = eps * eps;
        a.timeoutNs = 2000000000LL;
        cg_launch_fp64_raw(a, s.grid, s.block, st);
        CgInfo info;
        NSF_CUDA(cudaMemcpyAsync(&info, &w->info, sizeof(CgInfo), cudaMemcpyDeviceToHost, st));
        NSF_CUDA(cudaStreamSynchronize(st));
        if (iterations) *iterations = info.iterations;
        if (relResidual) *relResidual = info.bb > 0 ? std::sqrt(info.rr / info.bb) : 0.0;
        return info.status;
    } catch (const Error& e) {
        fprintf(stderr, "nsf_conjugate_gradient_noalloc: %s\n", e.msg.c_str());
        return e.status;
    }
}
