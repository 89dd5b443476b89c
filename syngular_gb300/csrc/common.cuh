// Shared helpers of the syngular_gb300 CUDA library: status codes, the
// thread-local error message, a bump allocator over the caller's workspace
// and small device utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/syngular_gb300.h"

namespace sgt {

// Records of a benchmark timer (the sgt_*_profile switches): switched on and
// drained by the caller, appended to from whichever host thread launches.
template <class Rec>
struct ProfLog {
  std::atomic<bool> on{false};
  std::mutex mu;
  std::vector<Rec> recs;
  bool active() const { return on.load(std::memory_order_relaxed); }
  void add(const Rec& r) {
    std::lock_guard<std::mutex> g(mu);
    recs.push_back(r);
  }
  std::vector<Rec> take() {
    std::lock_guard<std::mutex> g(mu);
    std::vector<Rec> v;
    v.swap(recs);
    return v;
  }
};

// Thread-local message of the last failure (read through sgt_last_error()).
void set_error(const char* fmt, ...);
const char* get_error();

#define SGT_CUDA(call)                                                                     \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      ::sgt::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
      return SGT_ERR_CUDA;                                                                 \
    }                                                                                      \
  } while (0)

// Every kernel launch of the library bumps a process-wide counter
// (sgt_launch_count), which benchmarks read around their timed region.
void note_launch();

// cudaFuncSetAttribute acts on the current device only.  Raise `attr` of
// `func` to at least `value` on the current device, remembering per device
// what was already set, so that a process using several GPUs opts every one
// of them in.  Returns the CUDA status of the set (cudaSuccess when cached).
cudaError_t func_attr_at_least(const void* func, cudaFuncAttribute attr, int value);

#define SGT_LAUNCHED()                                                                     \
  do {                                                                                     \
    ::sgt::note_launch();                                                                  \
    cudaError_t e_ = cudaGetLastError();                                                   \
    if (e_ != cudaSuccess) {                                                               \
      ::sgt::set_error("%s:%d: kernel launch: %s", __FILE__, __LINE__, cudaGetErrorString(e_)); \
      return SGT_ERR_CUDA;                                                                 \
    }                                                                                      \
  } while (0)

#define SGT_TRY(expr)            \
  do {                           \
    int s_ = (expr);             \
    if (s_ != SGT_OK) return s_; \
  } while (0)

#define SGT_REQUIRE(cond, code, ...) \
  do {                               \
    if (!(cond)) {                   \
      ::sgt::set_error(__VA_ARGS__); \
      return (code);                 \
    }                                \
  } while (0)

// Bump allocator over a caller-provided workspace.  `measure` mode only adds
// up sizes, so the same code path computes the workspace size and carves it.
struct Arena {
  char* base = nullptr;
  size_t cap = 0;
  size_t used = 0;
  bool measure = false;

  static Arena measuring() {
    Arena a;
    a.measure = true;
    return a;
  }
  Arena() = default;
  Arena(void* p, size_t n) : base((char*)p), cap(n) {}

  template <typename T>
  T* take(size_t count) {
    size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
    size_t off = used;
    used += bytes;
    if (measure) return nullptr;
    if (used > cap) return nullptr;
    return reinterpret_cast<T*>(base + off);
  }
  bool ok() const { return measure || used <= cap; }
};

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------------------
// internal entry points shared between translation units
// ---------------------------------------------------------------------------

// Row-major FP64 GEMM (see sgt_gemm_f64).  split_k > 1 splits the K loop over
// blockIdx.z slices that atomically add alpha*partial into C (beta is applied
// once beforehand).
int gemm_f64(cudaStream_t st, bool ta, bool tb, int64_t M, int64_t N, int64_t K, double alpha,
             const double* A, int64_t lda, int64_t sA, const double* B, int64_t ldb, int64_t sB,
             double beta, double* C, int64_t ldc, int64_t sC, int64_t batch, int split_k = 0);
// Deterministic split-K (K in `splits` equal chunks, ws = splits * M * N doubles,
// summed in a fixed order) and the chunk count that fills the GPU.
int gemm_f64_splitk(cudaStream_t st, bool ta, bool tb, int64_t M, int64_t N, int64_t K, double alpha,
                    const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                    double* ws, int splits);
int splitk_count(int64_t M, int64_t N, int64_t K);

// Elementwise helpers.
int fill_f64(cudaStream_t st, double* p, int64_t n, double v);
int copy2d_f64(cudaStream_t st, double* dst, int64_t ldd, const double* src, int64_t lds,
               int64_t rows, int64_t cols);
int scale_f64(cudaStream_t st, double* p, int64_t n, const double* dev_scale, bool inverse);

// Householder QR of a row-major m x n matrix in place; tau has min(m,n)
// entries.  The arena provides the panel scratch.
size_t qr_ws_bytes(int64_t m, int64_t n);
int qr_factor(cudaStream_t st, double* A, int64_t m, int64_t n, int64_t lda, double* tau, Arena& ar);
// Q (m x keep) = H_1 ... H_k I[:, :keep] from the factored A / tau.
size_t formq_ws_bytes(int64_t m, int64_t n, int64_t keep);
int qr_form_q(cudaStream_t st, const double* A, int64_t m, int64_t n, int64_t lda, const double* tau,
              double* Q, int64_t ldq, int64_t keep, Arena& ar);
// Copy the upper-trapezoidal R rows [0, rows) of the factored A into R
// (rows x n, ldr), zeroing below the diagonal and rows >= min(m, n).
int qr_extract_r(cudaStream_t st, const double* A, int64_t m, int64_t n, int64_t lda, double* R,
                 int64_t ldr, int64_t rows);

// dst (contiguous) = src (contiguous row-major, extents ext[0..rank-1]) with
// its axes reordered: output axis j is source axis perm[j] (rank <= 6; env.cu).
int permute_f64(cudaStream_t st, const double* src, double* dst, int rank, const int64_t* ext, const int* perm);

// Transfer-sweep helpers (sweeps.cu): E /= 2^e with max|E| in [0.5, 1), the
// exponent added to *expo; on the last site result = (E[0], *expo).
int rescale_pow2(cudaStream_t st, double* E, int64_t n, double* expo, double* result, bool last);
int zero_scalar(cudaStream_t st, double* p);

// One-sided Jacobi SVD (see sgt_jacobi_svd).
int jacobi_svd(cudaStream_t st, double* A, int64_t m, int64_t n, double* V, double* s, int* status,
               Arena& ar);

}  // namespace sgt
