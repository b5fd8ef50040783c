// Host-memory stand-in for the CUDA runtime calls made by the reference
// engine's compile path (GpuPostflopSolver::init and its destructor).
//
// TEST INFRASTRUCTURE ONLY. This file is linked (with `-cudart none`) into
// oracle/_ref/ref_capture, a program that runs the reference's own tree
// compiler (cuda/gpu_cfr.cu:1331-1827) on the host so that its integer
// artifacts can be dumped as golden fixtures. Device allocations become
// calloc'd host blocks whose sizes are recorded, so the capture can dump
// every array with its true length. Kernel launches, graphs, events and
// streams are inert: the capture never runs an iteration.
//
// Only runtime API names and signatures from the public CUDA headers are
// used here.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>

namespace {
std::map<const void*, size_t>& sizes() {
  static std::map<const void*, size_t> m;
  return m;
}
}  // namespace

// Size in bytes of a block returned by the stubbed cudaMalloc (0 if unknown).
extern "C" size_t refStubAllocSize(const void* p) {
  auto it = sizes().find(p);
  return it == sizes().end() ? 0 : it->second;
}

extern "C" {

cudaError_t cudaMalloc(void** p, size_t n) {
  *p = std::calloc(n ? n : 1, 1);
  if (!*p) return cudaErrorMemoryAllocation;
  sizes()[*p] = n;
  return cudaSuccess;
}

cudaError_t cudaFree(void* p) {
  if (p) {
    sizes().erase(p);
    std::free(p);
  }
  return cudaSuccess;
}

cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
  if (n) std::memmove(d, s, n);
  return cudaSuccess;
}

cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind,
                            cudaStream_t) {
  if (n) std::memmove(d, s, n);
  return cudaSuccess;
}

cudaError_t cudaMemset(void* d, int v, size_t n) {
  std::memset(d, v, n);
  return cudaSuccess;
}

cudaError_t cudaMemsetAsync(void* d, int v, size_t n, cudaStream_t) {
  std::memset(d, v, n);
  return cudaSuccess;
}

cudaError_t cudaStreamCreate(cudaStream_t* s) {
  *s = reinterpret_cast<cudaStream_t>(std::malloc(8));
  return cudaSuccess;
}
cudaError_t cudaStreamDestroy(cudaStream_t s) {
  std::free(reinterpret_cast<void*>(s));
  return cudaSuccess;
}
cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaStreamBeginCapture(cudaStream_t, cudaStreamCaptureMode) {
  return cudaErrorNotSupported;
}
cudaError_t cudaStreamEndCapture(cudaStream_t, cudaGraph_t*) {
  return cudaErrorNotSupported;
}
cudaError_t cudaGraphInstantiate(cudaGraphExec_t*, cudaGraph_t,
                                 unsigned long long) {
  return cudaErrorNotSupported;
}
cudaError_t cudaGraphLaunch(cudaGraphExec_t, cudaStream_t) {
  return cudaErrorNotSupported;
}
cudaError_t cudaGraphDestroy(cudaGraph_t) { return cudaSuccess; }
cudaError_t cudaGraphExecDestroy(cudaGraphExec_t) { return cudaSuccess; }
cudaError_t cudaGraphGetNodes(cudaGraph_t, cudaGraphNode_t*, size_t* n) {
  if (n) *n = 0;
  return cudaSuccess;
}
cudaError_t cudaEventCreate(cudaEvent_t* e) {
  *e = nullptr;
  return cudaSuccess;
}
cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t, cudaEvent_t) {
  *ms = 0.0f;
  return cudaSuccess;
}
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
const char* cudaGetErrorString(cudaError_t) { return "cuda host stub"; }

cudaError_t cudaLaunchKernel(const void*, dim3, dim3, void**, size_t,
                             cudaStream_t) {
  std::fprintf(stderr, "ref_capture: kernel launch is not available on the "
                       "host stub\n");
  return cudaErrorNotSupported;
}

// Registration hooks emitted by nvcc's host-side code; inert here.
void** __cudaRegisterFatBinary(void*) {
  static void* handle = nullptr;
  return &handle;
}
void __cudaRegisterFatBinaryEnd(void**) {}
void __cudaUnregisterFatBinary(void**) {}
void __cudaRegisterFunction(void**, const char*, char*, const char*, int,
                            uint3*, uint3*, dim3*, dim3*, int*) {}
void __cudaRegisterVar(void**, char*, char*, const char*, int, size_t, int,
                       int) {}
cudaError_t __cudaGetKernel(cudaKernel_t* k, const void*) {
  *k = nullptr;
  return cudaSuccess;
}
cudaError_t __cudaLaunchKernel(cudaKernel_t, dim3, dim3, void**, size_t,
                               cudaStream_t) {
  std::fprintf(stderr, "ref_capture: kernel launch is not available on the "
                       "host stub\n");
  return cudaErrorNotSupported;
}
unsigned __cudaPushCallConfiguration(dim3, dim3, size_t, void*) { return 0; }
cudaError_t __cudaPopCallConfiguration(dim3*, dim3*, size_t*, void*) {
  return cudaSuccess;
}

}  // extern "C"
