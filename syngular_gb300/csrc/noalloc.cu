// Overlap <X|Y> without any allocation: the transfer-sweep scratch lives in a
// fixed file-scope device array instead of a caller-provided workspace.
//
// Who needs it: callers that cannot hand the library device memory for
// scratch -- for instance a C or ctypes binding with no allocator of its own
// that runs inside a process whose GPU memory is entirely owned by another
// framework's pool, or a loop that must not allocate after start-up.  They
// still own X, Y and the 2-double result buffer.
//
// Limits: every bond <= SGT_NOALLOC_MAX_BOND (256) and every physical leg <=
// SGT_NOALLOC_MAX_PHYS (16).  The array takes about 9.4 MB of device memory on
// every GPU that loads the library, until the process exits.
//
// The array is shared by every call: each call rewrites what it reads first
// (the transfer matrices are written before they are read, the exponent and
// the unit start matrix are reset at the start), so stale contents from the
// previous call do no harm; but two calls that run at the same time on the
// GPU (different streams, or different host threads) race on the array and
// give wrong results.  Serialise them.
#include <mutex>

#include "common.cuh"

namespace sgt {

constexpr int64_t kNoAllocMaxBond = 256;
constexpr int64_t kNoAllocMaxPhys = 16;
// E ping-pong (2 x bond^2), T (bond * phys * bond), exponent, unit matrix, each
// rounded up to 256 bytes the way the workspace arena carves it.
constexpr int64_t kNoAllocDoubles =
    2 * kNoAllocMaxBond * kNoAllocMaxBond + kNoAllocMaxBond * kNoAllocMaxPhys * kNoAllocMaxBond + 4 * 32;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

int overlap_ws_run(cudaStream_t st, int n, const double* const* X, const int64_t* xs,
                   const double* const* Y, const int64_t* ys, double* result, void* ws, size_t ws_bytes);
size_t overlap_ws_size(int n, const int64_t* xs, const int64_t* ys);

namespace {

// Device address of g_noalloc_scratch, looked up once per device.  In host
// code the symbol is only a host-side stand-in; its device address comes from
// cudaGetSymbolAddress with that device current.
constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

int scratch_for_current_device(void** out) {
  int dev = 0;
  SGT_CUDA(cudaGetDevice(&dev));
  SGT_REQUIRE(dev >= 0 && dev < kMaxDevices, SGT_ERR_INVALID, "overlap_noalloc: device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error("overlap_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev, cudaGetErrorString(e));
      return SGT_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return SGT_OK;
}

}  // namespace
}  // namespace sgt

extern "C" SGT_API int sgt_overlap_sweep_noalloc(int n, const double* const* X, const int64_t* xshape,
                                                 const double* const* Y, const int64_t* yshape,
                                                 double* result, void* stream) {
  using namespace sgt;
  SGT_REQUIRE(X && Y && xshape && yshape && result && n >= 1, SGT_ERR_INVALID,
              "overlap_noalloc: null argument or empty chain");
  for (int k = 0; k < n; ++k) {
    const int64_t* xk = xshape + 3 * k;
    const int64_t* yk = yshape + 3 * k;
    SGT_REQUIRE(xk[0] <= kNoAllocMaxBond && xk[2] <= kNoAllocMaxBond && yk[0] <= kNoAllocMaxBond &&
                    yk[2] <= kNoAllocMaxBond,
                SGT_ERR_INVALID,
                "overlap_noalloc: bond above the fixed scratch limit of %lld at site %d; use sgt_overlap_sweep",
                (long long)kNoAllocMaxBond, k);
    SGT_REQUIRE(xk[1] <= kNoAllocMaxPhys, SGT_ERR_INVALID,
                "overlap_noalloc: physical leg %lld above the fixed scratch limit of %lld at site %d",
                (long long)xk[1], (long long)kNoAllocMaxPhys, k);
  }
  const size_t need = overlap_ws_size(n, xshape, yshape);
  SGT_REQUIRE(need > 0, SGT_ERR_INVALID, "%s", get_error());
  SGT_REQUIRE(need <= sizeof(double) * (size_t)kNoAllocDoubles, SGT_ERR_INVALID,
              "overlap_noalloc: scratch need %zu bytes exceeds the fixed %zu", need,
              sizeof(double) * (size_t)kNoAllocDoubles);
  void* scratch = nullptr;
  SGT_TRY(scratch_for_current_device(&scratch));
  return overlap_ws_run(as_stream(stream), n, X, xshape, Y, yshape, result, scratch,
                        sizeof(double) * (size_t)kNoAllocDoubles);
}
