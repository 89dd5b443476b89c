// Chain-level operations (the C ABI of include/syngular_gb300.h): overlap
// transfer sweep, reference QR truncation, dense decomposition, left/right
// orthonormalisation, TT-SVD rounding and the exported primitives.
//
// Every entry point runs its site loop on the host and enqueues kernels on
// the caller's stream; nothing here synchronises the device.  Scratch comes
// from the caller's workspace through an Arena whose measuring mode computes
// the matching *_workspace_size.
#include <stdarg.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "common.cuh"

namespace sgt {
int mixed_round_chain(cudaStream_t st, int n, const double* const* X, const int64_t* xs, int64_t chi,
                      int precision, double* const* out, double* spectra, double* discarded, int* status,
                      Arena& ar);

// ---- declarations of helpers defined in other translation units ----------
int frob_norm_f64(cudaStream_t st, const double* p, int64_t n, double* out);
int site_contract_mpo_mps(cudaStream_t st, const double* X, int64_t a, int64_t p, int64_t a2,
                          const double* W, int64_t b, int64_t o, int64_t b2, double* P);
int site_contract_mpo_mpo(cudaStream_t st, const double* A, int64_t b, int64_t i, int64_t m,
                          int64_t b2, const double* B, int64_t c, int64_t o, int64_t c2, double* P);
int bond_concat_chain(cudaStream_t st, int n, const double* const* A, const int64_t* ashape,
                      const double* const* B, const int64_t* bshape, double* const* out,
                      const int* positions);
int orthogonality(cudaStream_t st, const double* core, int64_t l, int64_t p, int64_t r, int side,
                  double* out);
int transpose_f64(cudaStream_t st, double* dst, int64_t ldd, const double* src, int64_t lds,
                  int64_t rows, int64_t cols);
size_t qr_tbuf_count(int64_t m, int64_t n);
int qr_factor_t(cudaStream_t st, double* A, int64_t m, int64_t n, int64_t lda, double* tau,
                double* Tbuf, Arena& ar);
int qr_apply_q(cudaStream_t st, const double* A, int64_t m, int64_t n, int64_t lda,
               const double* Tbuf, double* C, int64_t ldc, int64_t c, bool trans, Arena& ar);
int qr_form_q_t(cudaStream_t st, const double* A, int64_t m, int64_t n, int64_t lda,
                const double* Tbuf, double* Q, int64_t ldq, int64_t keep, Arena& ar);
int eye_f64(cudaStream_t st, double* Q, int64_t ldq, int64_t m, int64_t keep);
size_t jacobi_rows_ws_bytes(int64_t n, int64_t m);
int jacobi_rows(cudaStream_t st, double* G, int64_t ldg, int64_t n, int64_t m, double* Vt,
                int64_t ldv, double* s, int* status, Arena& ar);

// ---- error state and launch counter -----------------------------------------
static thread_local char g_err[512] = "";
static unsigned long long g_launches = 0;

void note_launch() { __atomic_fetch_add(&g_launches, 1ull, __ATOMIC_RELAXED); }

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
const char* get_error() { return g_err; }

cudaError_t func_attr_at_least(const void* func, cudaFuncAttribute attr, int value) {
  static std::mutex mu;
  static std::map<std::tuple<const void*, int, int>, int> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_tuple(func, (int)attr, dev);
  auto it = done.find(key);
  if (it != done.end() && it->second >= value) return cudaSuccess;
  e = cudaFuncSetAttribute(func, attr, value);
  if (e == cudaSuccess) done[key] = value;
  return e;
}

namespace {

struct Shape3 {
  int64_t l, p, r;
};

std::vector<Shape3> shapes_of(int n, const int64_t* s) {
  std::vector<Shape3> v(n);
  for (int k = 0; k < n; ++k) v[k] = {s[3 * k], s[3 * k + 1], s[3 * k + 2]};
  return v;
}

int check_chain(int n, const std::vector<Shape3>& s, const char* what) {
  SGT_REQUIRE(n >= 1, SGT_ERR_INVALID, "%s: empty chain", what);
  for (int k = 0; k < n; ++k) {
    SGT_REQUIRE(s[k].l > 0 && s[k].p > 0 && s[k].r > 0, SGT_ERR_INVALID,
                "%s: non-positive extent at site %d", what, k);
    if (k + 1 < n)
      SGT_REQUIRE(s[k].r == s[k + 1].l, SGT_ERR_INVALID,
                  "%s: bond mismatch between sites %d and %d (%lld vs %lld)", what, k, k + 1,
                  (long long)s[k].r, (long long)s[k + 1].l);
  }
  return SGT_OK;
}

// sum of squares of s[keep:] / sum of squares, spectra copy.
__global__ void spectrum_kernel(const double* __restrict__ s, int count, int keep,
                                double* __restrict__ spec_out, double* __restrict__ disc_out) {
  __shared__ double red[2][32];
  double tot = 0.0, drop = 0.0;
  for (int j = threadIdx.x; j < count; j += blockDim.x) {
    double v = s[j];
    if (spec_out) spec_out[j] = v;
    tot = fma(v, v, tot);
    if (j >= keep) drop = fma(v, v, drop);
  }
  for (int o = 16; o > 0; o >>= 1) {
    tot += __shfl_xor_sync(0xffffffffu, tot, o);
    drop += __shfl_xor_sync(0xffffffffu, drop, o);
  }
  if ((threadIdx.x & 31) == 0) red[0][threadIdx.x >> 5] = tot, red[1][threadIdx.x >> 5] = drop;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0, d = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[0][w], d += red[1][w];
    if (disc_out) *disc_out = (t > 0.0) ? d / t : 0.0;
  }
}

// Rescale E by a power of two so that max|E| lies in [0.5, 1); accumulate the
// exponent (exact, no rounding of E).  result = (E[0,0], exponent) at the end.
__global__ void rescale_pow2_kernel(double* __restrict__ E, int64_t n, double* __restrict__ expo,
                                    double* __restrict__ result, int last) {
  __shared__ double red[32];
  __shared__ int s_e;
  double mx = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, fabs(E[i]));
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
    int e = 0;
    if (m > 0.0 && isfinite(m)) frexp(m, &e);
    s_e = e;
    *expo += (double)e;
  }
  __syncthreads();
  const int e = s_e;
  if (e != 0)
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) E[i] = ldexp(E[i], -e);
  __syncthreads();
  if (last && threadIdx.x == 0) {
    result[0] = E[0];
    result[1] = *expo;
  }
}

__global__ void zero_scalar_kernel(double* p) { *p = 0.0; }

// status = -1 if any bond's Jacobi hit the sweep cap, else the largest sweep count.
__global__ void reduce_status_kernel(const int* __restrict__ st, int n, int* __restrict__ out) {
  if (threadIdx.x != 0) return;
  int r = 0;
  for (int k = 1; k < n; ++k) {
    if (st[k] < 0) {
      r = -1;
      break;
    }
    r = max(r, st[k]);
  }
  *out = r;
}

}  // namespace

// Exact power-of-two rescaling of a transfer matrix (see rescale_pow2_kernel),
// shared with the sliced overlap sweep.
int rescale_pow2(cudaStream_t st, double* E, int64_t n, double* expo, double* result, bool last) {
  rescale_pow2_kernel<<<1, 256, 0, st>>>(E, n, expo, result, last ? 1 : 0);
  SGT_LAUNCHED();
  return SGT_OK;
}

int zero_scalar(cudaStream_t st, double* p) {
  zero_scalar_kernel<<<1, 1, 0, st>>>(p);
  SGT_LAUNCHED();
  return SGT_OK;
}

// ============================================================================
// overlap
// ============================================================================
// splitk: use deterministic split-K partials (16 x the largest product in
// the workspace) for the bond-sized FP64 GEMMs; the fixed-capacity entry
// point (noalloc.cu) runs without.
static int overlap_impl(cudaStream_t st, int n, const double* const* X, const int64_t* xs,
                        const double* const* Y, const int64_t* ys, double* result, Arena& ar,
                        bool splitk = true) {
  auto sx = shapes_of(n, xs), sy = shapes_of(n, ys);
  SGT_TRY(check_chain(n, sx, "overlap(X)"));
  SGT_TRY(check_chain(n, sy, "overlap(Y)"));
  int64_t emax = 1, tmax = 1;
  for (int k = 0; k < n; ++k) {
    SGT_REQUIRE(sx[k].p == sy[k].p, SGT_ERR_INVALID, "overlap: physical dims differ at site %d", k);
    emax = std::max(emax, sx[k].r * sy[k].r);
    tmax = std::max(tmax, sx[k].l * sx[k].p * sy[k].r);
  }
  SGT_REQUIRE(sx[0].l == 1 && sy[0].l == 1 && sx[n - 1].r == 1 && sy[n - 1].r == 1, SGT_ERR_INVALID,
              "overlap: boundary bonds must be 1");
  double* E0 = ar.take<double>(emax);
  double* E1 = ar.take<double>(emax);
  double* T = ar.take<double>(tmax);
  double* expo = ar.take<double>(1);
  double* one = ar.take<double>(1);
  double* skw = splitk ? ar.take<double>(16 * std::max(emax, tmax)) : nullptr;
  if (ar.measure) return SGT_OK;
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "overlap: workspace too small");
  SGT_TRY(fill_f64(st, one, 1, 1.0));
  zero_scalar_kernel<<<1, 1, 0, st>>>(expo);
  SGT_LAUNCHED();
  const double* E = one;
  double* bufs[2] = {E0, E1};
  for (int k = 0; k < n; ++k) {
    const int64_t a = sx[k].l, p = sx[k].p, a2 = sx[k].r, c = sy[k].l, c2 = sy[k].r;
    // T (a x p*c2) = E (a x c) * Y_k (c x p*c2)
    SGT_TRY(gemm_f64_splitk(st, false, false, a, p * c2, c, 1.0, E, c, Y[k], p * c2, 0.0, T, p * c2, skw,
                            skw ? splitk_count(a, p * c2, c) : 1));
    double* En = bufs[k & 1];
    // E' (a2 x c2) = X_k^T (a2 x a*p) * T (a*p x c2)
    SGT_TRY(gemm_f64_splitk(st, true, false, a2, c2, a * p, 1.0, X[k], a2, T, c2, 0.0, En, c2, skw,
                            skw ? splitk_count(a2, c2, a * p) : 1));
    rescale_pow2_kernel<<<1, 256, 0, st>>>(En, a2 * c2, expo, result, k == n - 1);
    SGT_LAUNCHED();
    E = En;
  }
  return SGT_OK;
}

// ============================================================================
// reference QR truncation (>> dim)
// ============================================================================
static int qr_truncate_impl(cudaStream_t st, int n, const double* const* cores, const int64_t* shp,
                            int64_t dim, double* const* out, Arena& ar) {
  auto s = shapes_of(n, shp);
  SGT_TRY(check_chain(n, s, "qr_truncate"));
  SGT_REQUIRE(dim >= 1, SGT_ERR_INVALID, "qr_truncate: dim must be >= 1");
  int64_t lmax = 1, cmax = 1, rmax = 1, wmax = 1;
  for (int k = 0; k < n; ++k) {
    const int64_t l = (k == 0) ? s[k].l : dim;
    if (k + 1 < n) {
      SGT_REQUIRE(l * s[k].p >= dim, SGT_ERR_SHAPE,
                  "cannot reshape array of size %lld into shape (%lld,%lld,%lld)",
                  (long long)(l * s[k].p * std::min(l * s[k].p, dim)), (long long)l,
                  (long long)s[k].p, (long long)dim);
      lmax = std::max(lmax, l * s[k].p * s[k].r);
      rmax = std::max(rmax, s[k].r);
      wmax = std::max(wmax, dim * s[k + 1].p * s[k + 1].r);
      cmax = std::max(cmax, l * s[k].p);
    }
  }
  double* L = ar.take<double>(lmax);
  double* tau = ar.take<double>(std::min(cmax, rmax));
  double* Tb = ar.take<double>(qr_tbuf_count(cmax, rmax));
  double* S = ar.take<double>(dim * rmax);
  double* Wb[2] = {ar.take<double>(wmax), ar.take<double>(wmax)};
  size_t scratch_bytes;
  {
    Arena a = Arena::measuring();
    a.take<double>(cmax * 32);
    a.take<double>(32 * 32);
    a.take<double>(cmax * 32);
    a.take<double>(32 * std::max(rmax, dim));
    a.take<double>(32 * std::max(rmax, dim));
    scratch_bytes = a.used;
  }
  char* scratch = ar.take<char>(scratch_bytes);
  if (ar.measure) return SGT_OK;
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "qr_truncate: workspace too small");
  if (n == 1) {
    SGT_TRY(copy2d_f64(st, out[0], 1, cores[0], 1, 1, s[0].l * s[0].p * s[0].r));
    return SGT_OK;
  }
  const double* cur = cores[0];
  int64_t curl = s[0].l;
  for (int k = 0; k < n - 1; ++k) {
    const int64_t m = curl * s[k].p, r = s[k].r;
    SGT_TRY(copy2d_f64(st, L, r, cur, r, m, r));
    Arena a1(scratch, scratch_bytes);
    SGT_TRY(qr_factor_t(st, L, m, r, r, tau, Tb, a1));
    Arena a2(scratch, scratch_bytes);
    SGT_TRY(qr_form_q_t(st, L, m, r, r, Tb, out[k], dim, dim, a2));
    // S = R[:dim, :] (rows beyond min(m, r) are zero)
    SGT_TRY(qr_extract_r(st, L, m, r, r, S, r, dim));
    double* dst = (k + 1 == n - 1) ? out[n - 1] : Wb[k & 1];
    const int64_t pr = s[k + 1].p * s[k + 1].r;
    SGT_TRY(gemm_f64(st, false, false, dim, pr, r, 1.0, S, r, 0, cores[k + 1], pr, 0, 0.0, dst, pr, 0, 1));
    cur = dst;
    curl = dim;
  }
  return SGT_OK;
}

// ============================================================================
// decompose (dense tensor -> cores, left truncated-QR sweep)
// ============================================================================
static int decompose_right_impl(cudaStream_t st, const double* tensor, int n, const int64_t* phys,
                                const int64_t* bonds, double* const* out, Arena& ar);

static int decompose_impl(cudaStream_t st, const double* tensor, int n, const int64_t* phys,
                          const int64_t* bonds, int mode, double* const* out, Arena& ar) {
  if (mode == 1) return decompose_right_impl(st, tensor, n, phys, bonds, out, ar);
  SGT_REQUIRE(mode == 0, SGT_ERR_INVALID, "decompose: mode must be 0 (left) or 1 (right)");
  SGT_REQUIRE(n >= 1, SGT_ERR_INVALID, "decompose: empty chain");
  int64_t total = 1;
  for (int k = 0; k < n; ++k) {
    SGT_REQUIRE(phys[k] > 0, SGT_ERR_INVALID, "decompose: bad physical dim");
    total *= phys[k];
  }
  std::vector<int64_t> lb(n + 1, 1);
  for (int k = 0; k + 1 < n; ++k) {
    SGT_REQUIRE(bonds[k] > 0, SGT_ERR_INVALID, "decompose: bad bond");
    lb[k + 1] = bonds[k];
  }
  // sizes
  int64_t mmax = 1, rowsmax = 1, rest0 = total;
  int64_t bufmax = total;
  {
    int64_t rest = total, l = 1;
    for (int k = 0; k + 1 < n; ++k) {
      const int64_t m = l * phys[k];
      rest /= phys[k];
      SGT_REQUIRE(m >= lb[k + 1], SGT_ERR_SHAPE,
                  "cannot reshape array of size %lld into shape (%lld,%lld,%lld)",
                  (long long)(m * m), (long long)l, (long long)phys[k], (long long)lb[k + 1]);
      mmax = std::max(mmax, m);
      rowsmax = std::max(rowsmax, lb[k + 1]);
      bufmax = std::max(bufmax, lb[k + 1] * rest);
      l = lb[k + 1];
    }
  }
  (void)rest0;
  double* B0 = ar.take<double>(bufmax);
  double* B1 = ar.take<double>(bufmax);
  double* tau = ar.take<double>(mmax);
  double* Tb = ar.take<double>(qr_tbuf_count(mmax, mmax));
  Arena scratch_measure = Arena::measuring();
  // factor scratch: V, G, Y, W (n columns up to total)
  size_t scratch_bytes = 0;
  {
    Arena a = Arena::measuring();
    a.take<double>(mmax * 32);
    a.take<double>(32 * 32);
    a.take<double>(mmax * 32);
    a.take<double>(32 * std::max<int64_t>(total, rowsmax));
    scratch_bytes = a.used;
  }
  (void)scratch_measure;
  char* scratch_base = ar.take<char>(scratch_bytes);
  if (ar.measure) return SGT_OK;
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "decompose: workspace too small");
  if (n == 1) {
    SGT_TRY(copy2d_f64(st, out[0], 1, tensor, 1, 1, total));
    return SGT_OK;
  }
  SGT_TRY(copy2d_f64(st, B0, 1, tensor, 1, 1, total));
  double* cur = B0;
  double* nxt = B1;
  int64_t l = 1, rest = total;
  for (int k = 0; k + 1 < n; ++k) {
    const int64_t m = l * phys[k];
    rest /= phys[k];
    const int64_t ncol = rest, keep = lb[k + 1];
    Arena sc(scratch_base, scratch_bytes);
    SGT_TRY(qr_factor_t(st, cur, m, ncol, ncol, tau, Tb, sc));
    Arena sc2(scratch_base, scratch_bytes);
    SGT_TRY(qr_form_q_t(st, cur, m, ncol, ncol, Tb, out[k], keep, keep, sc2));
    SGT_TRY(qr_extract_r(st, cur, m, ncol, ncol, nxt, ncol, keep));
    std::swap(cur, nxt);
    l = keep;
  }
  SGT_TRY(copy2d_f64(st, out[n - 1], 1, cur, 1, 1, l * phys[n - 1]));
  return SGT_OK;
}

// Right mode (mps:324-347): for k = n-1..1, L = (T as (rest, p_k r_k))^T,
// complete QR keep l_k columns, core_k = Q[:, :l_k]^T, T <- R[:l_k, :]^T.
static int decompose_right_impl(cudaStream_t st, const double* tensor, int n, const int64_t* phys,
                                const int64_t* bonds, double* const* out, Arena& ar) {
  SGT_REQUIRE(n >= 1, SGT_ERR_INVALID, "decompose: empty chain");
  int64_t total = 1;
  for (int k = 0; k < n; ++k) {
    SGT_REQUIRE(phys[k] > 0, SGT_ERR_INVALID, "decompose: bad physical dim");
    total *= phys[k];
  }
  std::vector<int64_t> rb(n + 1, 1);  // rb[k] = left bond of core k
  for (int k = 1; k < n; ++k) {
    SGT_REQUIRE(bonds[k - 1] > 0, SGT_ERR_INVALID, "decompose: bad bond");
    rb[k] = bonds[k - 1];
  }
  int64_t bufmax = total, mmax = 1, rowsmax = 1, colmax = 1;
  {
    int64_t rest = total, r = 1;
    for (int k = n - 1; k >= 1; --k) {
      const int64_t pr = phys[k] * r;
      rest = rest / phys[k];  // rows of T viewed as (rest, p_k r_k), before this step
      SGT_REQUIRE(pr >= rb[k], SGT_ERR_SHAPE,
                  "cannot reshape array of size %lld into shape (%lld,%lld,%lld)",
                  (long long)(pr * pr), (long long)rb[k], (long long)phys[k], (long long)r);
      mmax = std::max(mmax, pr);
      colmax = std::max(colmax, rest);
      rowsmax = std::max(rowsmax, rb[k]);
      bufmax = std::max(bufmax, rest * rb[k]);
      bufmax = std::max(bufmax, pr * rest);
      r = rb[k];
      rest = rest * 1;  // T' = (rest x l_k)
    }
  }
  double* B0 = ar.take<double>(bufmax);
  double* B1 = ar.take<double>(bufmax);
  double* Qb = ar.take<double>(mmax * rowsmax);
  double* tau = ar.take<double>(mmax);
  double* Tb = ar.take<double>(qr_tbuf_count(mmax, std::max(mmax, colmax)));
  size_t scratch_bytes;
  {
    Arena a = Arena::measuring();
    a.take<double>(mmax * 32);
    a.take<double>(32 * 32);
    a.take<double>(mmax * 32);
    a.take<double>(32 * std::max(colmax, rowsmax));
    a.take<double>(32 * std::max(colmax, rowsmax));
    scratch_bytes = a.used;
  }
  char* scratch = ar.take<char>(scratch_bytes);
  if (ar.measure) return SGT_OK;
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "decompose: workspace too small");
  if (n == 1) {
    SGT_TRY(copy2d_f64(st, out[0], 1, tensor, 1, 1, total));
    return SGT_OK;
  }
  const double* T = tensor;  // (rest x p r), row-major
  int64_t rest = total, r = 1;
  double* bufs[2] = {B0, B1};
  int flip = 0;
  for (int k = n - 1; k >= 1; --k) {
    const int64_t pr = phys[k] * r;
    rest /= phys[k];
    const int64_t keep = rb[k];
    double* L = bufs[flip];
    SGT_TRY(transpose_f64(st, L, rest, T, pr, rest, pr));  // L = T^T (pr x rest)
    Arena a1(scratch, scratch_bytes);
    SGT_TRY(qr_factor_t(st, L, pr, rest, rest, tau, Tb, a1));
    Arena a2(scratch, scratch_bytes);
    SGT_TRY(qr_form_q_t(st, L, pr, rest, rest, Tb, Qb, keep, keep, a2));  // (pr x keep)
    SGT_TRY(transpose_f64(st, out[k], pr, Qb, keep, pr, keep));           // core_k = Q^T
    double* Tn = bufs[flip ^ 1];
    // R[:keep, :] (keep x rest) -> Qb-sized scratch is too small in general; use Tn then transpose in place
    SGT_TRY(qr_extract_r(st, L, pr, rest, rest, Tn, rest, keep));
    // T' = R^T (rest x keep), written into L (no longer needed)
    SGT_TRY(transpose_f64(st, L, keep, Tn, rest, keep, rest));
    T = L;
    flip ^= 1;
    r = keep;
  }
  SGT_TRY(copy2d_f64(st, out[0], 1, T, 1, 1, phys[0] * r));
  return SGT_OK;
}

// ============================================================================
// left / right orthonormalisation (in place, shapes kept)
// ============================================================================
static int orth_impl(cudaStream_t st, int n, double* const* cores, const int64_t* shp, bool left,
                     Arena& ar) {
  auto s = shapes_of(n, shp);
  SGT_TRY(check_chain(n, s, left ? "left_orthonormalization" : "right_orthonormalization"));
  int64_t mmax = 1, kmax = 1, cmax = 1, nmax = 1;
  for (int k = 0; k < n; ++k) {
    const int64_t sz = s[k].l * s[k].p * s[k].r;
    cmax = std::max(cmax, sz);
    if (left && k + 1 < n) {
      SGT_REQUIRE(s[k].l * s[k].p >= s[k].r, SGT_ERR_SHAPE,
                  "left_orthonormalization needs l*p >= r at site %d", k);
      mmax = std::max(mmax, s[k].l * s[k].p);
      kmax = std::max(kmax, s[k].r);
    }
    if (!left && k > 0) {
      SGT_REQUIRE(s[k].p * s[k].r >= s[k].l, SGT_ERR_SHAPE,
                  "right_orthonormalization needs p*r >= l at site %d", k);
      mmax = std::max(mmax, s[k].p * s[k].r);
      kmax = std::max(kmax, s[k].l);
    }
    nmax = std::max(nmax, s[k].p * s[k].r);
    nmax = std::max(nmax, s[k].l * s[k].p);
  }
  double* F = ar.take<double>(mmax * kmax);
  double* tau = ar.take<double>(kmax);
  double* Tb = ar.take<double>(qr_tbuf_count(mmax, kmax));
  double* Rb = ar.take<double>(kmax * kmax);
  double* Tmp = ar.take<double>(cmax);
  size_t scratch_bytes;
  {
    Arena a = Arena::measuring();
    a.take<double>(mmax * 32);
    a.take<double>(32 * 32);
    a.take<double>(mmax * 32);
    a.take<double>(32 * std::max(kmax, nmax));
    a.take<double>(32 * std::max(kmax, nmax));
    scratch_bytes = a.used;
  }
  char* scratch = ar.take<char>(scratch_bytes);
  if (ar.measure) return SGT_OK;
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "orthonormalization: workspace too small");
  if (left) {
    for (int k = 0; k + 1 < n; ++k) {
      const int64_t m = s[k].l * s[k].p, r = s[k].r;
      SGT_TRY(copy2d_f64(st, F, r, cores[k], r, m, r));
      Arena a1(scratch, scratch_bytes);
      SGT_TRY(qr_factor_t(st, F, m, r, r, tau, Tb, a1));
      Arena a2(scratch, scratch_bytes);
      SGT_TRY(qr_form_q_t(st, F, m, r, r, Tb, cores[k], r, r, a2));
      SGT_TRY(qr_extract_r(st, F, m, r, r, Rb, r, r));
      const int64_t pr = s[k + 1].p * s[k + 1].r;
      SGT_TRY(gemm_f64(st, false, false, r, pr, r, 1.0, Rb, r, 0, cores[k + 1], pr, 0, 0.0, Tmp, pr, 0, 1));
      SGT_TRY(copy2d_f64(st, cores[k + 1], 1, Tmp, 1, 1, r * pr));
    }
  } else {
    for (int k = n - 1; k > 0; --k) {
      const int64_t l = s[k].l, pr = s[k].p * s[k].r;
      // F (pr x l) = R_k^T
      SGT_TRY(transpose_f64(st, F, l, cores[k], pr, l, pr));
      Arena a1(scratch, scratch_bytes);
      SGT_TRY(qr_factor_t(st, F, pr, l, l, tau, Tb, a1));
      SGT_TRY(qr_extract_r(st, F, pr, l, l, Rb, l, l));
      Arena a2(scratch, scratch_bytes);
      SGT_TRY(qr_form_q_t(st, F, pr, l, l, Tb, Tmp, l, l, a2));  // V (pr x l)
      SGT_TRY(transpose_f64(st, cores[k], pr, Tmp, l, pr, l));    // core_k = V^T
      // core_{k-1} (lp x l) <- core_{k-1} U^T
      const int64_t lp = s[k - 1].l * s[k - 1].p;
      SGT_TRY(gemm_f64(st, false, true, lp, l, l, 1.0, cores[k - 1], l, 0, Rb, l, 0, 0.0, Tmp, l, 0, 1));
      SGT_TRY(copy2d_f64(st, cores[k - 1], 1, Tmp, 1, 1, lp * l));
    }
  }
  return SGT_OK;
}

// ============================================================================
// TT-SVD rounding
// ============================================================================
static void svd_round_plan(int n, const std::vector<Shape3>& s, int64_t chi, std::vector<int64_t>& b,
                           std::vector<int64_t>& x, std::vector<int64_t>& cnt) {
  b.assign(n + 1, 1);
  for (int k = 0; k + 1 < n; ++k) b[k + 1] = std::min(b[k] * s[k].p, s[k].r);
  x.assign(n + 1, 1);
  cnt.assign(n, 0);
  for (int k = n - 1; k >= 1; --k) {
    cnt[k] = std::min(b[k], s[k].p * x[k + 1]);
    x[k] = std::min(chi, cnt[k]);
  }
  x[0] = 1;
}

static int svd_round_impl(cudaStream_t st, int n, const double* const* cores, const int64_t* shp,
                          int64_t chi, int precision, double* const* out, double* spectra,
                          double* discarded, int* status, Arena& ar) {
  auto s = shapes_of(n, shp);
  SGT_TRY(check_chain(n, s, "svd_round"));
  SGT_REQUIRE(chi >= 1, SGT_ERR_INVALID, "svd_round: chi must be >= 1");
  if (precision == SGT_PREC_TF32 || precision == SGT_PREC_TF32X3 || precision == SGT_PREC_BF16X6)
    return mixed_round_chain(st, n, cores, shp, chi, precision, out, spectra, discarded, status, ar);
  SGT_REQUIRE(precision == SGT_PREC_F64, SGT_ERR_INVALID, "svd_round: unsupported precision %d", precision);
  SGT_REQUIRE(s[0].l == 1 && s[n - 1].r == 1, SGT_ERR_INVALID, "svd_round: boundary bonds must be 1");
  std::vector<int64_t> b, x, cnt;
  svd_round_plan(n, s, chi, b, x, cnt);

  // left sweep storage: factored C_k (b_k p_k x r_k) for k < n-1, last carried core
  std::vector<double*> F(n), Tb(n), tau(n);
  int64_t mmax = 1, rmax = 1, smax = 1, cmax = 1;
  for (int k = 0; k < n; ++k) {
    const int64_t m = b[k] * s[k].p;
    F[k] = ar.take<double>(m * s[k].r);
    if (k + 1 < n) {
      tau[k] = ar.take<double>(std::min(m, s[k].r));
      Tb[k] = ar.take<double>(qr_tbuf_count(m, s[k].r));
    }
    mmax = std::max(mmax, m);
    rmax = std::max(rmax, s[k].r);
    smax = std::max(smax, m * s[k].r);
    cmax = std::max(cmax, s[k].p * x[k + 1]);
  }
  double* Rb = ar.take<double>(rmax * rmax);
  // right sweep buffers
  const int64_t sq = std::max(mmax, cmax);
  double* Mc = ar.take<double>(smax);        // copy of M for its QR
  double* G = ar.take<double>(sq * sq);      // Jacobi rows
  double* Vt = ar.take<double>(sq * sq);
  double* sv = ar.take<double>(sq);
  double* US = ar.take<double>(mmax * chi);
  double* Mn = ar.take<double>(smax);        // pushed core (next M)
  double* Qf = ar.take<double>(cmax * mmax);
  double* tauM = ar.take<double>(sq);
  double* TbM = ar.take<double>(qr_tbuf_count(sq, sq));
  int* stat = ar.take<int>(n);
  size_t scratch_bytes;
  {
    Arena a = Arena::measuring();
    a.take<double>(sq * 32);
    a.take<double>(32 * 32);
    a.take<double>(sq * 32);
    a.take<double>(32 * std::max(sq, rmax * 8));
    a.take<double>(32 * std::max(sq, rmax * 8));
    size_t qb = a.used;
    size_t jb = jacobi_rows_ws_bytes(sq, sq);
    scratch_bytes = std::max(qb, jb);
  }
  // the carry GEMM / apply-Q widths can exceed sq: size W for them too
  int64_t wmax = 1;
  for (int k = 0; k < n; ++k) wmax = std::max(wmax, s[k].p * s[k].r);
  size_t extra;
  {
    Arena a = Arena::measuring();
    a.take<double>(mmax * 32);
    a.take<double>(32 * 32);
    a.take<double>(mmax * 32);
    a.take<double>(32 * std::max(wmax, sq));
    a.take<double>(32 * std::max(wmax, sq));
    extra = a.used;
  }
  scratch_bytes = std::max(scratch_bytes, extra);
  char* scratch = ar.take<char>(scratch_bytes);
  if (ar.measure) return SGT_OK;
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "svd_round: workspace too small");

  // ---- left QR sweep ----
  SGT_TRY(copy2d_f64(st, F[0], 1, cores[0], 1, 1, s[0].p * s[0].r));
  for (int k = 0; k + 1 < n; ++k) {
    const int64_t m = b[k] * s[k].p, r = s[k].r, kk = b[k + 1];
    Arena a1(scratch, scratch_bytes);
    SGT_TRY(qr_factor_t(st, F[k], m, r, r, tau[k], Tb[k], a1));
    SGT_TRY(qr_extract_r(st, F[k], m, r, r, Rb, r, kk));
    const int64_t pr = s[k + 1].p * s[k + 1].r;
    SGT_TRY(gemm_f64(st, false, false, kk, pr, r, 1.0, Rb, r, 0, cores[k + 1], pr, 0, 0.0, F[k + 1], pr, 0, 1));
  }
  // ---- right-to-left truncated SVD sweep ----
  const double* M = F[n - 1];
  for (int k = n - 1; k >= 1; --k) {
    const int64_t mrows = b[k], c = s[k].p * x[k + 1], keep = x[k];
    if (mrows >= c) {
      SGT_TRY(copy2d_f64(st, Mc, c, M, c, mrows, c));
      Arena a1(scratch, scratch_bytes);
      SGT_TRY(qr_factor_t(st, Mc, mrows, c, c, tauM, TbM, a1));
      SGT_TRY(qr_extract_r(st, Mc, mrows, c, c, Qf, c, c));  // R (c x c) into Qf
      SGT_TRY(transpose_f64(st, G, c, Qf, c, c, c));          // G = R^T
      Arena a2(scratch, scratch_bytes);
      SGT_TRY(jacobi_rows(st, G, c, c, c, Vt, c, sv, stat + k, a2));
      SGT_TRY(copy2d_f64(st, out[k], c, Vt, c, keep, c));
      SGT_TRY(gemm_f64(st, false, true, mrows, keep, c, 1.0, M, c, 0, Vt, c, 0, 0.0, US, keep, 0, 1));
    } else {
      SGT_TRY(transpose_f64(st, Mc, mrows, M, c, mrows, c));  // Mc = M^T (c x mrows)
      Arena a1(scratch, scratch_bytes);
      SGT_TRY(qr_factor_t(st, Mc, c, mrows, mrows, tauM, TbM, a1));
      SGT_TRY(qr_extract_r(st, Mc, c, mrows, mrows, G, mrows, mrows));  // G = R (mrows x mrows)
      Arena a2(scratch, scratch_bytes);
      SGT_TRY(jacobi_rows(st, G, mrows, mrows, mrows, Vt, mrows, sv, stat + k, a2));
      Arena a3(scratch, scratch_bytes);
      SGT_TRY(qr_form_q_t(st, Mc, c, mrows, mrows, TbM, Qf, mrows, mrows, a3));  // Q (c x mrows)
      // out_k (keep x c) = Vt[:keep] (keep x mrows) * Q^T
      SGT_TRY(gemm_f64(st, false, true, keep, c, mrows, 1.0, Vt, mrows, 0, Qf, mrows, 0, 0.0, out[k], c, 0, 1));
      // US (mrows x keep) = (G[:keep])^T
      SGT_TRY(transpose_f64(st, US, keep, G, mrows, keep, mrows));
    }
    const int64_t count = cnt[k];
    double* spec_k = nullptr;
    if (spectra) {
      int64_t off = 0;
      for (int j = 1; j < k; ++j) off += cnt[j];
      spec_k = spectra + off;
    }
    spectrum_kernel<<<1, 256, 0, st>>>(sv, (int)count, (int)keep, spec_k,
                                       discarded ? discarded + (k - 1) : nullptr);
    SGT_LAUNCHED();
    // push: M_{k-1} (b_{k-1} p_{k-1} x keep) = Q_{k-1} [US; 0]
    const int64_t mprev = b[k - 1] * s[k - 1].p;
    double* dst = (k - 1 == 0) ? out[0] : Mn;
    SGT_TRY(fill_f64(st, dst, mprev * keep, 0.0));
    SGT_TRY(copy2d_f64(st, dst, keep, US, keep, mrows, keep));
    Arena a4(scratch, scratch_bytes);
    SGT_TRY(qr_apply_q(st, F[k - 1], mprev, s[k - 1].r, s[k - 1].r, Tb[k - 1], dst, keep, keep, false, a4));
    if (k - 1 > 0) {
      // M for the next step must not alias Mn (it is rewritten): copy into F[k-1]'s
      // slot, which is no longer needed once Q_{k-1} has been applied.
      SGT_TRY(copy2d_f64(st, F[k - 1], 1, Mn, 1, 1, mprev * keep));
      M = F[k - 1];
    }
  }
  if (n == 1) SGT_TRY(copy2d_f64(st, out[0], 1, cores[0], 1, 1, s[0].p));
  if (status) {
    reduce_status_kernel<<<1, 32, 0, st>>>(stat, n, status);
    SGT_LAUNCHED();
  }
  return SGT_OK;
}

// the fixed-capacity variant (no split-K partials) for sgt_overlap_sweep_noalloc
size_t overlap_ws_size(int n, const int64_t* xs, const int64_t* ys) {
  Arena a = Arena::measuring();
  if (overlap_impl(nullptr, n, nullptr, xs, nullptr, ys, nullptr, a, false) != SGT_OK) return 0;
  return a.used;
}

int overlap_ws_run(cudaStream_t st, int n, const double* const* X, const int64_t* xs,
                   const double* const* Y, const int64_t* ys, double* result, void* ws, size_t ws_bytes) {
  Arena a(ws, ws_bytes);
  return overlap_impl(st, n, X, xs, Y, ys, result, a, false);
}

size_t svd_round_ws(int n, const int64_t* shape, int64_t chi) {
  Arena a = Arena::measuring();
  if (svd_round_impl(nullptr, n, nullptr, shape, chi, SGT_PREC_F64, nullptr, nullptr, nullptr, nullptr, a) !=
      SGT_OK)
    return 0;
  return a.used;
}

int svd_round_run(cudaStream_t st, int n, const double* const* cores, const int64_t* shape, int64_t chi,
                  double* const* out, double* spectra, double* discarded, int* status, Arena& ar) {
  return svd_round_impl(st, n, cores, shape, chi, SGT_PREC_F64, out, spectra, discarded, status, ar);
}

void svd_round_plan_public(int n, const int64_t* shape, int64_t chi, std::vector<int64_t>& b,
                           std::vector<int64_t>& x, std::vector<int64_t>& cnt) {
  svd_round_plan(n, shapes_of(n, shape), chi, b, x, cnt);
}

}  // namespace sgt

// ============================================================================
// extern "C"
// ============================================================================
using namespace sgt;

extern "C" {

int sgt_version(void) { return 1; }
unsigned long long sgt_launch_count(void) { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }
const char* sgt_last_error(void) { return get_error(); }

int sgt_site_contract_mpo_mps(const double* X, int64_t a, int64_t p, int64_t a2, const double* W,
                              int64_t b, int64_t o, int64_t b2, double* P, void* stream) {
  SGT_REQUIRE(X && W && P, SGT_ERR_INVALID, "site_contract_mpo_mps: null pointer");
  SGT_REQUIRE(a > 0 && p > 0 && a2 > 0 && b > 0 && o > 0 && b2 > 0, SGT_ERR_INVALID,
              "site_contract_mpo_mps: non-positive extent");
  return site_contract_mpo_mps(as_stream(stream), X, a, p, a2, W, b, o, b2, P);
}

int sgt_site_contract_mpo_mpo(const double* A, int64_t b, int64_t i, int64_t m, int64_t b2,
                              const double* B, int64_t c, int64_t o, int64_t c2, double* P,
                              void* stream) {
  SGT_REQUIRE(A && B && P, SGT_ERR_INVALID, "site_contract_mpo_mpo: null pointer");
  SGT_REQUIRE(b > 0 && i > 0 && m > 0 && b2 > 0 && c > 0 && o > 0 && c2 > 0, SGT_ERR_INVALID,
              "site_contract_mpo_mpo: non-positive extent");
  return site_contract_mpo_mpo(as_stream(stream), A, b, i, m, b2, B, c, o, c2, P);
}

int sgt_bond_concat(const double* A, int64_t la, int64_t phys, int64_t ra, const double* B,
                    int64_t lb, int64_t rb, int position, double* out, void* stream) {
  SGT_REQUIRE(A && B && out, SGT_ERR_INVALID, "bond_concat: null pointer");
  int64_t as[3] = {la, phys, ra}, bs[3] = {lb, phys, rb};
  return bond_concat_chain(as_stream(stream), 1, &A, as, &B, bs, &out, &position);
}

size_t sgt_bond_concat_chain_workspace_size(int n) {
  (void)n;
  return 0;
}

int sgt_bond_concat_chain(int n, const double* const* A, const int64_t* ashape,
                          const double* const* B, const int64_t* bshape, double* const* out,
                          void* ws, size_t ws_bytes, void* stream) {
  (void)ws;
  (void)ws_bytes;
  SGT_REQUIRE(n >= 1 && A && B && out && ashape && bshape, SGT_ERR_INVALID, "bond_concat_chain: bad args");
  return bond_concat_chain(as_stream(stream), n, A, ashape, B, bshape, out, nullptr);
}

size_t sgt_overlap_workspace_size(int n, const int64_t* xshape, const int64_t* yshape) {
  Arena a = Arena::measuring();
  if (overlap_impl(nullptr, n, nullptr, xshape, nullptr, yshape, nullptr, a) != SGT_OK) return 0;
  return a.used;
}

int sgt_overlap_sweep(int n, const double* const* X, const int64_t* xshape, const double* const* Y,
                      const int64_t* yshape, double* result, void* ws, size_t ws_bytes, void* stream) {
  SGT_REQUIRE(X && Y && xshape && yshape && result, SGT_ERR_INVALID, "overlap: null argument");
  Arena a(ws, ws_bytes);
  return overlap_impl(as_stream(stream), n, X, xshape, Y, yshape, result, a);
}

size_t sgt_qr_truncate_workspace_size(int n, const int64_t* shape, int64_t dim) {
  Arena a = Arena::measuring();
  if (qr_truncate_impl(nullptr, n, nullptr, shape, dim, nullptr, a) != SGT_OK) return 0;
  return a.used;
}

int sgt_qr_truncate_sweep(int n, const double* const* cores, const int64_t* shape, int64_t dim,
                          double* const* out, void* ws, size_t ws_bytes, void* stream) {
  SGT_REQUIRE(cores && shape && out, SGT_ERR_INVALID, "qr_truncate: null argument");
  Arena a(ws, ws_bytes);
  return qr_truncate_impl(as_stream(stream), n, cores, shape, dim, out, a);
}

size_t sgt_decompose_workspace_size(int n, const int64_t* phys, const int64_t* bonds, int mode) {
  Arena a = Arena::measuring();
  if (decompose_impl(nullptr, nullptr, n, phys, bonds, mode, nullptr, a) != SGT_OK) return 0;
  return a.used;
}

int sgt_decompose(const double* tensor, int n, const int64_t* phys, const int64_t* bonds, int mode,
                  double* const* out, void* ws, size_t ws_bytes, void* stream) {
  SGT_REQUIRE(tensor && phys && out && (n == 1 || bonds), SGT_ERR_INVALID, "decompose: null argument");
  Arena a(ws, ws_bytes);
  return decompose_impl(as_stream(stream), tensor, n, phys, bonds, mode, out, a);
}

int sgt_normalize(double* core, int64_t count, double* norm, void* stream) {
  SGT_REQUIRE(core && norm && count > 0, SGT_ERR_INVALID, "normalize: bad argument");
  cudaStream_t st = as_stream(stream);
  SGT_TRY(frob_norm_f64(st, core, count, norm));
  return scale_f64(st, core, count, norm, true);
}

size_t sgt_orthonormalize_workspace_size(int n, const int64_t* shape) {
  Arena a = Arena::measuring(), b = Arena::measuring();
  if (orth_impl(nullptr, n, nullptr, shape, true, a) != SGT_OK) a.used = 0;
  if (orth_impl(nullptr, n, nullptr, shape, false, b) != SGT_OK) b.used = 0;
  return std::max(a.used, b.used);
}

int sgt_left_orthonormalize(int n, double* const* cores, const int64_t* shape, void* ws,
                            size_t ws_bytes, void* stream) {
  SGT_REQUIRE(cores && shape, SGT_ERR_INVALID, "left_orthonormalization: null argument");
  Arena a(ws, ws_bytes);
  return orth_impl(as_stream(stream), n, cores, shape, true, a);
}

int sgt_right_orthonormalize(int n, double* const* cores, const int64_t* shape, void* ws,
                             size_t ws_bytes, void* stream) {
  SGT_REQUIRE(cores && shape, SGT_ERR_INVALID, "right_orthonormalization: null argument");
  Arena a(ws, ws_bytes);
  return orth_impl(as_stream(stream), n, cores, shape, false, a);
}

int sgt_orthogonality(const double* core, int64_t l, int64_t p, int64_t r, int side, double* out,
                      void* stream) {
  SGT_REQUIRE(core && out && (side == 0 || side == 1), SGT_ERR_INVALID, "orthogonality: bad argument");
  return orthogonality(as_stream(stream), core, l, p, r, side, out);
}

int sgt_svd_round_shapes(int n, const int64_t* shape, int64_t chi, int64_t* out_shape,
                         int64_t* spec_count) {
  SGT_REQUIRE(n >= 1 && shape && out_shape, SGT_ERR_INVALID, "svd_round_shapes: bad argument");
  auto s = shapes_of(n, shape);
  SGT_TRY(check_chain(n, s, "svd_round_shapes"));
  std::vector<int64_t> b, x, cnt;
  svd_round_plan(n, s, chi, b, x, cnt);
  for (int k = 0; k < n; ++k) {
    out_shape[3 * k] = x[k];
    out_shape[3 * k + 1] = s[k].p;
    out_shape[3 * k + 2] = x[k + 1];
    if (spec_count && k >= 1) spec_count[k - 1] = cnt[k];
  }
  return SGT_OK;
}

size_t sgt_svd_round_workspace_size(int n, const int64_t* shape, int64_t chi, int precision) {
  Arena a = Arena::measuring();
  if (svd_round_impl(nullptr, n, nullptr, shape, chi, precision, nullptr, nullptr, nullptr, nullptr, a) !=
      SGT_OK)
    return 0;
  return a.used;
}

int sgt_svd_round(int n, const double* const* cores, const int64_t* shape, int64_t chi, int precision,
                  double* const* out, double* spectra, double* discarded, int* status, void* ws,
                  size_t ws_bytes, void* stream) {
  SGT_REQUIRE(cores && shape && out, SGT_ERR_INVALID, "svd_round: null argument");
  Arena a(ws, ws_bytes);
  return svd_round_impl(as_stream(stream), n, cores, shape, chi, precision, out, spectra, discarded,
                        status, a);
}

int sgt_gemm_f64(int transA, int transB, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
                 int64_t lda, int64_t strideA, const double* B, int64_t ldb, int64_t strideB, double beta,
                 double* C, int64_t ldc, int64_t strideC, int64_t batch, void* stream) {
  SGT_REQUIRE(C && (K == 0 || (A && B)), SGT_ERR_INVALID, "gemm_f64: null pointer");
  return gemm_f64(as_stream(stream), transA != 0, transB != 0, M, N, K, alpha, A, lda, strideA, B, ldb,
                  strideB, beta, C, ldc, strideC, batch, 0);
}

size_t sgt_qr_workspace_size(int64_t m, int64_t n, int64_t keep) {
  Arena a = Arena::measuring();
  a.take<double>(qr_tbuf_count(m, n));
  size_t f = qr_ws_bytes(m, n), q = formq_ws_bytes(m, n, std::max<int64_t>(keep, 1));
  return a.used + std::max(f, q);
}

int sgt_qr(double* A, int64_t m, int64_t n, int64_t lda, double* tau, double* Q, int64_t keep, void* ws,
           size_t ws_bytes, void* stream) {
  SGT_REQUIRE(A && tau && m > 0 && n > 0 && lda >= n, SGT_ERR_INVALID, "qr: bad argument");
  SGT_REQUIRE(keep <= m, SGT_ERR_SHAPE, "qr: keep > m");
  Arena a(ws, ws_bytes);
  double* Tb = a.take<double>(qr_tbuf_count(m, n));
  SGT_REQUIRE(a.ok(), SGT_ERR_WORKSPACE, "qr: workspace too small");
  const size_t base = a.used;
  cudaStream_t st = as_stream(stream);
  SGT_TRY(qr_factor_t(st, A, m, n, lda, tau, Tb, a));
  if (Q && keep > 0) {
    a.used = base;
    SGT_TRY(qr_form_q_t(st, A, m, n, lda, Tb, Q, keep, keep, a));
  }
  return SGT_OK;
}

size_t sgt_jacobi_svd_workspace_size(int64_t m, int64_t n) {
  Arena a = Arena::measuring();
  a.take<double>(n * m);
  a.take<double>(n * n);
  return a.used + jacobi_rows_ws_bytes(n, m);
}

int sgt_jacobi_svd(double* A, int64_t m, int64_t n, double* V, double* s, int* status, void* ws,
                   size_t ws_bytes, void* stream) {
  SGT_REQUIRE(A && V && s && m >= n && n > 0, SGT_ERR_INVALID, "jacobi_svd: bad argument (m >= n > 0)");
  Arena a(ws, ws_bytes);
  double* G = a.take<double>(n * m);
  double* Vt = a.take<double>(n * n);
  SGT_REQUIRE(a.ok(), SGT_ERR_WORKSPACE, "jacobi_svd: workspace too small");
  cudaStream_t st = as_stream(stream);
  SGT_TRY(transpose_f64(st, G, m, A, n, m, n));  // G = A^T (n x m)
  SGT_TRY(jacobi_rows(st, G, m, n, m, V, n, s, status, a));
  SGT_TRY(transpose_f64(st, A, n, G, m, n, m));  // A = (A V)
  // V currently holds V^T (rows = singular vectors); return V (columns)
  SGT_TRY(copy2d_f64(st, Vt, n, V, n, n, n));
  SGT_TRY(transpose_f64(st, V, n, Vt, n, n, n));
  return SGT_OK;
}

}  // extern "C"
