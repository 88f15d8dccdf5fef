// A stand-in for the CUDA runtime, linked into a test build of the engine library (nvcc
// -cudart none) so that the C ABI's host paths -- allocation, validation, error returns and
// clean-up -- run on a machine without a GPU.
//
// Device memory is host memory; copies and memsets act on it directly.  A kernel launch does
// nothing, unless the library also links the warp emulator of tests/warp_emu, which defines
// emu_dispatch: then the launch runs a host build of the same kernel on emulated warps.  Test hooks count live allocations, catch frees of unknown pointers, and make the
// k-th allocation from now fail with cudaErrorMemoryAllocation, as an out-of-memory device would.

#include <cuda_profiler_api.h>
#include <cuda_runtime_api.h>

#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace {
std::map<void *, size_t> g_live;  // allocation -> bytes
long g_fail_in = -1;              // allocations to go before one fails; -1: none
long g_allocs = 0;                // allocations made
long g_bad_frees = 0;             // frees of pointers that are not live
long g_launches = 0;              // kernel launches
// host stub -> device (mangled) name; filled by the registration constructors of the engine's
// object, which may run before this file's globals are constructed, hence constructed on first use
std::map<const void *, std::string> &kernel_names() {
  static std::map<const void *, std::string> names;
  return names;
}
char g_dummy[64];                 // backing for opaque handles (streams, events, pools)
// a captured stream operation: a memset, or a kernel launch recorded by the warp emulator
struct Op {
  void *ptr = nullptr;
  int value = 0;
  size_t n = 0;
  std::shared_ptr<void> launch;
};
std::vector<Op> *g_capture = nullptr;  // the stream capture in progress, if any
void *g_fatbin_handle[4];
}  // namespace

extern "C" {

// ---- test hooks ----
void fake_cuda_fail_alloc_in(long k) { g_fail_in = k; }
long fake_cuda_live_allocs(void) { return (long)g_live.size(); }
long fake_cuda_live_bytes(void) {
  long b = 0;
  for (auto &kv : g_live) b += (long)kv.second;
  return b;
}
long fake_cuda_allocs(void) { return g_allocs; }
long fake_cuda_bad_frees(void) { return g_bad_frees; }
long fake_cuda_launches(void) { return g_launches; }

// ---- memory ----
cudaError_t cudaMallocAsync(void **p, size_t n, cudaStream_t) {
  *p = nullptr;
  if (g_fail_in == 0) {
    g_fail_in = -1;
    return cudaErrorMemoryAllocation;
  }
  if (g_fail_in > 0) g_fail_in--;
  void *q = std::calloc(1, n ? n : 1);
  if (!q) return cudaErrorMemoryAllocation;
  g_live[q] = n;
  g_allocs++;
  *p = q;
  return cudaSuccess;
}

cudaError_t cudaFreeAsync(void *p, cudaStream_t) {
  if (!p) return cudaSuccess;
  auto it = g_live.find(p);
  if (it == g_live.end()) {
    g_bad_frees++;
    return cudaErrorInvalidValue;
  }
  std::free(p);
  g_live.erase(it);
  return cudaSuccess;
}

cudaError_t cudaMemcpy(void *dst, const void *src, size_t n, cudaMemcpyKind) {
  if (n && (!dst || !src)) return cudaErrorInvalidValue;
  if (n) std::memmove(dst, src, n);
  return cudaSuccess;
}

cudaError_t cudaMemcpyAsync(void *dst, const void *src, size_t n, cudaMemcpyKind kind, cudaStream_t) {
  return cudaMemcpy(dst, src, n, kind);
}

cudaError_t cudaMemsetAsync(void *p, int v, size_t n, cudaStream_t) {
  if (n && !p) return cudaErrorInvalidValue;
  if (g_capture) {
    Op op;
    op.ptr = p;
    op.value = v;
    op.n = n;
    g_capture->push_back(op);
    return cudaSuccess;
  }
  if (n) std::memset(p, v, n);
  return cudaSuccess;
}

// a __device__ variable's host shadow stands in for its device storage
cudaError_t cudaGetSymbolAddress(void **p, const void *symbol) {
  *p = const_cast<void *>(symbol);
  return cudaSuccess;
}

cudaError_t cudaMemcpyFromSymbol(void *dst, const void *symbol, size_t n, size_t offset, cudaMemcpyKind) {
  std::memmove(dst, static_cast<const char *>(symbol) + offset, n);
  return cudaSuccess;
}

// ---- device, streams, events ----
cudaError_t cudaGetDeviceCount(int *n) {
  *n = 1;
  return cudaSuccess;
}
cudaError_t cudaSetDevice(int d) { return d == 0 ? cudaSuccess : cudaErrorInvalidDevice; }
cudaError_t cudaGetDevice(int *d) {
  *d = 0;
  return cudaSuccess;
}
cudaError_t cudaDeviceGetAttribute(int *v, cudaDeviceAttr attr, int) {
  *v = attr == cudaDevAttrMultiProcessorCount ? 152 : 0;
  return cudaSuccess;
}
cudaError_t cudaDeviceGetDefaultMemPool(cudaMemPool_t *pool, int) {
  *pool = reinterpret_cast<cudaMemPool_t>(g_dummy);
  return cudaSuccess;
}
cudaError_t cudaMemPoolSetAttribute(cudaMemPool_t, cudaMemPoolAttr, void *) { return cudaSuccess; }
cudaError_t cudaStreamCreateWithFlags(cudaStream_t *s, unsigned int) {
  *s = reinterpret_cast<cudaStream_t>(g_dummy + 8);
  return cudaSuccess;
}
cudaError_t cudaStreamDestroy(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaEventCreate(cudaEvent_t *ev) {
  *ev = reinterpret_cast<cudaEvent_t>(g_dummy + 16);
  return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t, cudaEvent_t) {
  *ms = 0.001f;
  return cudaSuccess;
}
cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
const char *emu_last_failure(void) __attribute__((weak));  // tests/warp_emu: why a launch failed

const char *cudaGetErrorString(cudaError_t err) {
  if (err == cudaErrorLaunchFailure && emu_last_failure) return emu_last_failure();
  return err == cudaErrorMemoryAllocation ? "out of memory (fake runtime)" : "error (fake runtime)";
}
cudaError_t cudaProfilerStart(void) { return cudaSuccess; }
cudaError_t cudaProfilerStop(void) { return cudaSuccess; }

// ---- kernels: launch configuration accepted, nothing runs ----
cudaError_t cudaFuncSetAttribute(const void *, cudaFuncAttribute, int) { return cudaSuccess; }
cudaError_t cudaOccupancyMaxActiveBlocksPerMultiprocessor(int *n, const void *, int, size_t) {
  *n = 8;
  return cudaSuccess;
}

// ---- CUDA graphs: stream capture records memsets and launches, a graph launch replays them ----
// (kernel launches are recorded only when the warp emulator is linked in: emu_capture)
void *emu_capture(const char *device_name, unsigned gx, unsigned gy, unsigned gz, unsigned bx, unsigned by,
                  unsigned bz, size_t smem, void **args) __attribute__((weak));
int emu_replay(void *launch) __attribute__((weak));
void emu_release(void *launch) __attribute__((weak));

cudaError_t cudaStreamBeginCapture(cudaStream_t, cudaStreamCaptureMode) {
  if (g_capture) return cudaErrorIllegalState;
  g_capture = new std::vector<Op>();
  return cudaSuccess;
}
cudaError_t cudaStreamEndCapture(cudaStream_t, cudaGraph_t *g) {
  if (!g_capture) {
    *g = nullptr;
    return cudaErrorIllegalState;
  }
  *g = reinterpret_cast<cudaGraph_t>(g_capture);
  g_capture = nullptr;
  return cudaSuccess;
}
cudaError_t cudaGraphInstantiate(cudaGraphExec_t *x, cudaGraph_t g, unsigned long long) {
  *x = reinterpret_cast<cudaGraphExec_t>(new std::vector<Op>(*reinterpret_cast<std::vector<Op> *>(g)));
  return cudaSuccess;
}
cudaError_t cudaGraphLaunch(cudaGraphExec_t x, cudaStream_t) {
  for (const Op &op : *reinterpret_cast<std::vector<Op> *>(x)) {
    if (!op.launch) {
      if (op.n) std::memset(op.ptr, op.value, op.n);
      continue;
    }
    g_launches++;
    if (emu_replay && emu_replay(op.launch.get()) != 0) return cudaErrorLaunchFailure;
  }
  return cudaSuccess;
}
cudaError_t cudaGraphExecDestroy(cudaGraphExec_t x) {
  delete reinterpret_cast<std::vector<Op> *>(x);
  return cudaSuccess;
}
cudaError_t cudaGraphDestroy(cudaGraph_t g) {
  delete reinterpret_cast<std::vector<Op> *>(g);
  return cudaSuccess;
}

// ---- what nvcc's generated host code calls at load time and for <<<...>>> ----
void **__cudaRegisterFatBinary(void *) { return g_fatbin_handle; }
void __cudaRegisterFatBinaryEnd(void **) {}
void __cudaUnregisterFatBinary(void **) {}
void __cudaRegisterFunction(void **, const char *host_fun, char *, const char *device_name, int, uint3 *, uint3 *,
                            dim3 *, dim3 *, int *) {
  kernel_names()[host_fun] = device_name;
}
void __cudaRegisterVar(void **, char *, char *, const char *, int, size_t, int, int) {}
// <<<grid, block, shared, stream>>> pushes the configuration; the launch stub pops it again
struct LaunchConfig {
  dim3 grid, block;
  size_t shared;
  cudaStream_t stream;
};
LaunchConfig g_config;
unsigned __cudaPushCallConfiguration(dim3 grid, dim3 block, size_t shared, struct CUstream_st *stream) {
  g_config = LaunchConfig{grid, block, shared, stream};
  return 0;
}
cudaError_t __cudaPopCallConfiguration(dim3 *grid, dim3 *block, size_t *shared, void *stream) {
  *grid = g_config.grid;
  *block = g_config.block;
  *shared = g_config.shared;
  *static_cast<cudaStream_t *>(stream) = g_config.stream;
  return cudaSuccess;
}
cudaError_t __cudaGetKernel(cudaKernel_t *k, const void *fn) {
  *k = reinterpret_cast<cudaKernel_t>(const_cast<void *>(fn));
  return cudaSuccess;
}
// defined by tests/warp_emu when it is linked in: runs the named kernel, 0 on success
int emu_dispatch(const char *device_name, unsigned gx, unsigned gy, unsigned gz, unsigned bx, unsigned by,
                 unsigned bz, size_t smem, void **args) __attribute__((weak));

cudaError_t __cudaLaunchKernel(cudaKernel_t kernel, dim3 grid, dim3 block, void **args, size_t smem, cudaStream_t) {
  auto it = kernel_names().find(reinterpret_cast<const void *>(kernel));
  if (g_capture) {
    if (!emu_capture) return cudaSuccess;  // nothing runs without the emulator, so nothing to record
    if (it == kernel_names().end()) return cudaErrorInvalidDeviceFunction;
    void *launch = emu_capture(it->second.c_str(), grid.x, grid.y, grid.z, block.x, block.y, block.z, smem, args);
    if (!launch) return cudaErrorInvalidDeviceFunction;
    Op op;
    op.launch = std::shared_ptr<void>(launch, emu_release);
    g_capture->push_back(op);
    return cudaSuccess;
  }
  g_launches++;
  if (!emu_dispatch) return cudaSuccess;
  if (it == kernel_names().end()) return cudaErrorInvalidDeviceFunction;
  return emu_dispatch(it->second.c_str(), grid.x, grid.y, grid.z, block.x, block.y, block.z, smem, args) == 0
             ? cudaSuccess
             : cudaErrorLaunchFailure;
}

}  // extern "C"
