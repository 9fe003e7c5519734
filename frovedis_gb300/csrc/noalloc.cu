// fvg_spmv_no_alloc: y = A x (CRS) on device vectors without allocating.
//
// Some callers cannot allocate device memory: a plug-in running inside a
// host framework that owns every device allocation (its allocator contract
// forbids cudaMalloc behind its back), or a latency-critical loop that must
// not pay cudaMalloc/cudaFree's implicit device synchronisation.  This entry
// point serves them: the only scratch the CRS pass needs (one partial sum per
// piece of a long row) lives in the file-scope device array below, which
// every GPU that loads this library holds until the process exits.
#include <mutex>

#include "fvg_internal.cuh"

namespace fvg {
size_t crs_spmv_no_alloc(fvg_ctx* c, DevCRS& a, int storage, const void* x, void* y, void* scratch,
                         size_t scratch_bytes);
}

using namespace fvg;

// 8 MiB: room for 1,048,576 FP64 (2,097,152 FP32) piece partial sums, i.e.
// long rows totalling up to ~512 million nonzeros.
constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;
static __device__ __align__(256) unsigned char g_no_alloc_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

// Makes the context's device current for the whole call (the symbol lookup
// and the launches on the context's stream) and restores the caller's device
// on the way out.
struct DeviceGuard {
  int prev = -1, dev;
  explicit DeviceGuard(int d) : dev(d) {
    FVG_CUDA(cudaGetDevice(&prev));
    if (prev != dev) FVG_CUDA(cudaSetDevice(dev));
  }
  ~DeviceGuard() {
    if (prev >= 0 && prev != dev) cudaSetDevice(prev);
  }
};

// Device address of g_no_alloc_scratch on `device`, which must be current
// (the name is only a host stand-in); looked up once per device.
void* scratch_for(int device) {
  if (device < 0 || device >= kMaxDevices) fail(FVG_ERR_INVALID_ARG, "device id out of range");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[device]) {
    void* ptr = nullptr;
    cudaError_t rc = cudaGetSymbolAddress(&ptr, g_no_alloc_scratch);
    if (rc != cudaSuccess || !ptr) throw_cuda(rc, "cudaGetSymbolAddress(g_no_alloc_scratch)", __FILE__, __LINE__);
    g_scratch_ptr[device] = ptr;
  }
  return g_scratch_ptr[device];
}
}  // namespace

extern "C" FVG_API fvg_status fvg_spmv_no_alloc(fvg_ctx* c, fvg_matrix* M, fvg_dtype storage, fvg_dtype vec_dtype,
                                               const void* x, void* y) {
  if (!c || !M) return FVG_ERR_INVALID_ARG;
  try {
    if (M->ctx != c) fail(FVG_ERR_INVALID_ARG, "the matrix belongs to another (or a destroyed) context");
    if (storage < FVG_F64 || storage > FVG_BF16) fail(FVG_ERR_INVALID_ARG, "unknown storage dtype");
    const int want = (storage == FVG_F64) ? FVG_F64 : FVG_F32;
    if (vec_dtype != want)
      fail(FVG_ERR_INVALID_ARG, storage == FVG_F64 ? "FP64 values need FP64 vectors"
                                                   : "FP32/BF16 values need FP32 vectors here");
    if ((M->A.m > 0 && !y) || (M->A.n > 0 && !x)) fail(FVG_ERR_INVALID_ARG, "null vector");
    DeviceGuard guard(c->device);
    const size_t need = crs_spmv_no_alloc(c, M->A, storage, x, y, nullptr, 0);
    if (need > kNoAllocScratchBytes)
      fail(FVG_ERR_INVALID_ARG, "matrix too large for fvg_spmv_no_alloc: its long rows need " + std::to_string(need) +
                                    " bytes of scratch, the limit is " + std::to_string(kNoAllocScratchBytes));
    void* scratch = scratch_for(c->device);
    crs_spmv_no_alloc(c, M->A, storage, x, y, scratch, kNoAllocScratchBytes);
    return FVG_OK;
  } catch (const fvg::Error& e) {
    c->last_error = e.msg;
    return e.code;
  } catch (...) {
    c->last_error = "internal error";
    return FVG_ERR_INTERNAL;
  }
}
