/* ORACLE (reference build) — test infrastructure only.
 * The reference's gpu_host_common.cpp is linked into oracle/_ref only because KDTreeCPUOwner::upload shares a
 * translation unit with the KD-tree builder.  The checker never touches a GPU, so the CUDA driver entry points
 * that file references resolve to these stand-ins, which all report CUDA_ERROR_NO_DEVICE (100). */
#define NSFEM_STUB(name) int name(void) { return 100; }
NSFEM_STUB(cuCtxGetCurrent)
NSFEM_STUB(cuCtxPopCurrent_v2)
NSFEM_STUB(cuCtxPushCurrent_v2)
NSFEM_STUB(cuDeviceGet)
NSFEM_STUB(cuDeviceGetAttribute)
NSFEM_STUB(cuDeviceGetName)
NSFEM_STUB(cuDevicePrimaryCtxRelease_v2)
NSFEM_STUB(cuDevicePrimaryCtxRetain)
NSFEM_STUB(cuGetErrorName)
NSFEM_STUB(cuGetErrorString)
NSFEM_STUB(cuLaunchKernel)
NSFEM_STUB(cuMemAllocHost_v2)
NSFEM_STUB(cuMemAlloc_v2)
NSFEM_STUB(cuMemFreeHost)
NSFEM_STUB(cuMemFree_v2)
NSFEM_STUB(cuMemHostAlloc)
NSFEM_STUB(cuMemHostGetDevicePointer_v2)
NSFEM_STUB(cuMemcpyDtoDAsync_v2)
NSFEM_STUB(cuMemcpyDtoD_v2)
NSFEM_STUB(cuMemcpyDtoH_v2)
NSFEM_STUB(cuMemcpyHtoD_v2)
NSFEM_STUB(cuModuleGetFunction)
NSFEM_STUB(cuModuleLoadDataEx)
