// Zip-up MPO x MPS (Stoudenmire & White, New J. Phys. 12, 055026 (2010),
// "zip-up" algorithm): the product W X compressed site by site from the left
// without ever forming the product cores or its chi*D-sized bonds.
//
// A carry C (r x a b: the already compressed left part, contracted with the
// bonds a of X and b of W) moves left to right.  At site k:
//   M[(r, o), (a', b')] = sum_{a, b, i} C[r, (a, b)] X_k[a, i, a'] W_k[b, i, o, b']
// (two FP64 GEMMs with index permutations between them), then the truncated
// SVD of M: the core Z_k = the q = min(chi, rank bound) leading left singular
// vectors, the next carry S V^T = U_q^T M.  The SVD is the library's FP64
// Householder QR plus one-sided Jacobi on the small triangular factor.  The
// last site takes M itself.  The cost per site is O(chi^3 D d) instead of the
// O(chi^3 D^3 d) of rounding the full product; the truncation is optimal for
// each cut given the right part's gauge, so the caller right-orthonormalises X
// first (exact when chi covers every bond's rank).
#include <algorithm>
#include <vector>

#include "common.cuh"

namespace sgt {

int transpose_f64(cudaStream_t st, double* dst, int64_t ldd, const double* src, int64_t lds, int64_t rows,
                  int64_t cols);
size_t jacobi_rows_ws_bytes(int64_t n, int64_t m);
size_t qr_tbuf_count(int64_t m, int64_t n);
int qr_factor_t(cudaStream_t st, double* A, int64_t m, int64_t n, int64_t lda, double* tau, double* Tbuf, Arena& ar);
int qr_form_q_t(cudaStream_t st, const double* A, int64_t m, int64_t n, int64_t lda, const double* Tbuf, double* Q,
                int64_t ldq, int64_t keep, Arena& ar);
int jacobi_rows(cudaStream_t st, double* G, int64_t ldg, int64_t n, int64_t m, double* Vt, int64_t ldv, double* s,
                int* status, Arena& ar);

namespace {

// disc = sum_{j >= keep} s_j^2 / sum_j s_j^2 (one block)
__global__ void zip_discarded_kernel(const double* __restrict__ s, int count, int keep, double* __restrict__ disc) {
  __shared__ double red[2][32];
  double tot = 0.0, drop = 0.0;
  for (int j = threadIdx.x; j < count; j += blockDim.x) {
    const double v = s[j];
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
    *disc = t > 0.0 ? d / t : 0.0;
  }
}

// status = -1 if some bond's Jacobi reached its sweep cap, else the largest sweep count
__global__ void zip_status_kernel(const int* __restrict__ st, int n, int* __restrict__ out) {
  int r = 0;
  for (int k = 0; k < n; ++k) {
    if (st[k] < 0) {
      r = -1;
      break;
    }
    r = max(r, st[k]);
  }
  *out = r;
}

struct ZipSite {
  int64_t r, a, b, i, o, a2, b2, q;  // carry rows, bonds in, legs, bonds out, kept
};

int zip_plan(int n, const int64_t* ws4, const int64_t* xs, int64_t chi, std::vector<ZipSite>& sites) {
  SGT_REQUIRE(n >= 1 && ws4 && xs, SGT_ERR_INVALID, "zipup: empty chain");
  SGT_REQUIRE(chi >= 1, SGT_ERR_INVALID, "zipup: chi must be >= 1");
  sites.assign(n, ZipSite{});
  int64_t r = 1;
  for (int k = 0; k < n; ++k) {
    ZipSite& z = sites[k];
    z.r = r;
    z.a = xs[3 * k];
    z.i = xs[3 * k + 1];
    z.a2 = xs[3 * k + 2];
    z.b = ws4[4 * k];
    z.o = ws4[4 * k + 2];
    z.b2 = ws4[4 * k + 3];
    SGT_REQUIRE(z.a > 0 && z.i > 0 && z.a2 > 0 && z.b > 0 && z.o > 0 && z.b2 > 0, SGT_ERR_INVALID,
                "zipup: non-positive extent at site %d", k);
    SGT_REQUIRE(ws4[4 * k + 1] == z.i, SGT_ERR_INVALID, "zipup: leg mismatch at site %d", k);
    if (k > 0)
      SGT_REQUIRE(z.a == xs[3 * k - 1] && z.b == ws4[4 * k - 1], SGT_ERR_INVALID,
                  "zipup: bond mismatch between sites %d and %d", k - 1, k);
    const int64_t m = z.r * z.o, nn = z.a2 * z.b2;
    z.q = (k + 1 < n) ? std::min(chi, std::min(m, nn)) : 1;
    r = z.q;
  }
  SGT_REQUIRE(sites[0].a == 1 && sites[0].b == 1 && sites[n - 1].a2 == 1 && sites[n - 1].b2 == 1, SGT_ERR_INVALID,
              "zipup: boundary bonds must be 1");
  return SGT_OK;
}

int zipup_impl(cudaStream_t st, int n, const double* const* W, const int64_t* ws4, const double* const* X,
               const int64_t* xs, int64_t chi, double* const* out, double* discarded, int* status, Arena& ar) {
  std::vector<ZipSite> zs;
  SGT_TRY(zip_plan(n, ws4, xs, chi, zs));
  int64_t cmax = 1, tmax = 1, mmax = 1, smax = 1, qmax = 1;
  size_t scratch = 0, tbmax = 1;
  for (int k = 0; k < n; ++k) {
    const ZipSite& z = zs[k];
    const int64_t m = z.r * z.o, nn = z.a2 * z.b2, mn = std::min(m, nn);
    cmax = std::max(cmax, std::max(z.r * z.a * z.b, z.q * nn));
    tmax = std::max(tmax, std::max(z.r * z.b * z.i * z.a2, m * nn));
    mmax = std::max(mmax, m * nn);
    smax = std::max(smax, mn * mn);
    qmax = std::max(qmax, mn);
    if (k + 1 < n) {
      // Householder factors (T blocks kept for forming Q) + panel scratch
      tbmax = std::max(tbmax, qr_tbuf_count(std::max(m, nn), mn));
      scratch = std::max(scratch, qr_ws_bytes(std::max(m, nn), mn));
      if (m > nn) scratch = std::max(scratch, formq_ws_bytes(m, nn, nn));
      scratch = std::max(scratch, jacobi_rows_ws_bytes(mn, mn));
    }
  }
  double* C0 = ar.take<double>(cmax);
  double* C1 = ar.take<double>(cmax);
  double* Cp = ar.take<double>(cmax);
  double* T1 = ar.take<double>(tmax);
  double* T1p = ar.take<double>(tmax);
  double* M = ar.take<double>(mmax);
  double* A = ar.take<double>(mmax);  // QR input (M or M^T), then Q
  double* Q = ar.take<double>(mmax);
  double* R = ar.take<double>(smax);
  double* G = ar.take<double>(smax);
  double* Vt = ar.take<double>(smax);
  double* s = ar.take<double>(qmax);
  double* tau = ar.take<double>(qmax);
  double* Tb = ar.take<double>(tbmax);
  int* stat = ar.take<int>((size_t)n);
  char* scr = ar.take<char>(std::max<size_t>(scratch, 256));
  if (ar.measure) return SGT_OK;
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "zipup: workspace too small");
  SGT_REQUIRE(W && X && out, SGT_ERR_INVALID, "zipup: null argument");
  SGT_CUDA(cudaMemsetAsync(stat, 0, sizeof(int) * n, st));
  SGT_TRY(fill_f64(st, C0, 1, 1.0));
  double* C = C0;
  double* Cn = C1;
  for (int k = 0; k < n; ++k) {
    const ZipSite& z = zs[k];
    const int64_t m = z.r * z.o, nn = z.a2 * z.b2;
    // Cp[(r, b), a] = C[r, a, b]
    {
      const int64_t ext[3] = {z.r, z.a, z.b};
      const int perm[3] = {0, 2, 1};
      SGT_TRY(permute_f64(st, C, Cp, 3, ext, perm));
    }
    // T1[(r, b), (i, a')] = Cp X_k
    SGT_TRY(gemm_f64(st, false, false, z.r * z.b, z.i * z.a2, z.a, 1.0, Cp, z.a, 0, X[k], z.i * z.a2, 0, 0.0, T1,
                     z.i * z.a2, 0, 1));
    // T1p[(r, a'), (b, i)]
    {
      const int64_t ext[4] = {z.r, z.b, z.i, z.a2};
      const int perm[4] = {0, 3, 1, 2};
      SGT_TRY(permute_f64(st, T1, T1p, 4, ext, perm));
    }
    // T2[(r, a'), (o, b')] = T1p W_k[(b, i), (o, b')]  (into T1)
    SGT_TRY(gemm_f64(st, false, false, z.r * z.a2, z.o * z.b2, z.b * z.i, 1.0, T1p, z.b * z.i, 0, W[k], z.o * z.b2,
                     0, 0.0, T1, z.o * z.b2, 0, 1));
    // M[(r, o), (a', b')]
    {
      const int64_t ext[4] = {z.r, z.a2, z.o, z.b2};
      const int perm[4] = {0, 2, 1, 3};
      SGT_TRY(permute_f64(st, T1, k + 1 < n ? M : out[k], 4, ext, perm));
    }
    if (k + 1 == n) break;  // the last core is M itself (r, o, 1)
    const int64_t q = z.q;
    Arena sa(scr, std::max<size_t>(scratch, 256));
    if (m <= nn) {
      // M^T = Q R (n x m); M = R^T Q^T; rows of Vt (Jacobi on the rows of R^T)
      // are M's left singular vectors
      SGT_TRY(transpose_f64(st, A, m, M, nn, m, nn));
      SGT_TRY(qr_factor_t(st, A, nn, m, m, tau, Tb, sa));
      SGT_TRY(qr_extract_r(st, A, nn, m, m, R, m, m));
      SGT_TRY(transpose_f64(st, G, m, R, m, m, m));
      Arena ja(scr, std::max<size_t>(scratch, 256));
      SGT_TRY(jacobi_rows(st, G, m, m, m, Vt, m, s, stat + k, ja));
      // Z_k (m x q) = Vt[:q]^T; next carry (q x n) = Vt[:q] M
      SGT_TRY(transpose_f64(st, out[k], q, Vt, m, q, m));
      SGT_TRY(gemm_f64(st, false, false, q, nn, m, 1.0, Vt, m, 0, M, nn, 0, 0.0, Cn, nn, 0, 1));
      if (discarded) {
        zip_discarded_kernel<<<1, 256, 0, st>>>(s, (int)m, (int)q, discarded + k);
        SGT_LAUNCHED();
      }
    } else {
      // M = Q R (m x n); left singular vectors Q Vt^T (Jacobi on the rows of R)
      SGT_TRY(copy2d_f64(st, A, nn, M, nn, m, nn));
      SGT_TRY(qr_factor_t(st, A, m, nn, nn, tau, Tb, sa));
      SGT_TRY(qr_extract_r(st, A, m, nn, nn, R, nn, nn));
      Arena fa(scr, std::max<size_t>(scratch, 256));
      SGT_TRY(qr_form_q_t(st, A, m, nn, nn, Tb, Q, nn, nn, fa));
      SGT_TRY(copy2d_f64(st, G, nn, R, nn, nn, nn));
      Arena ja(scr, std::max<size_t>(scratch, 256));
      SGT_TRY(jacobi_rows(st, G, nn, nn, nn, Vt, nn, s, stat + k, ja));
      // Z_k (m x q) = Q Vt[:q]^T; next carry (q x n) = Vt[:q] R
      SGT_TRY(gemm_f64(st, false, true, m, q, nn, 1.0, Q, nn, 0, Vt, nn, 0, 0.0, out[k], q, 0, 1));
      SGT_TRY(gemm_f64(st, false, false, q, nn, nn, 1.0, Vt, nn, 0, R, nn, 0, 0.0, Cn, nn, 0, 1));
      if (discarded) {
        zip_discarded_kernel<<<1, 256, 0, st>>>(s, (int)nn, (int)q, discarded + k);
        SGT_LAUNCHED();
      }
    }
    std::swap(C, Cn);
  }
  if (status) {
    zip_status_kernel<<<1, 1, 0, st>>>(stat, n, status);
    SGT_LAUNCHED();
  }
  return SGT_OK;
}

}  // namespace
}  // namespace sgt

using namespace sgt;

extern "C" {

SGT_API int sgt_mpo_mps_zipup_shapes(int n, const int64_t* wshape, const int64_t* xshape, int64_t chi,
                                     int64_t* out_shape) {
  std::vector<ZipSite> zs;
  SGT_TRY(zip_plan(n, wshape, xshape, chi, zs));
  SGT_REQUIRE(out_shape, SGT_ERR_INVALID, "zipup_shapes: null output");
  for (int k = 0; k < n; ++k) {
    out_shape[3 * k] = zs[k].r;
    out_shape[3 * k + 1] = zs[k].o;
    out_shape[3 * k + 2] = zs[k].q;
  }
  return SGT_OK;
}

SGT_API size_t sgt_mpo_mps_zipup_workspace_size(int n, const int64_t* wshape, const int64_t* xshape, int64_t chi) {
  Arena a = Arena::measuring();
  if (zipup_impl(nullptr, n, nullptr, wshape, nullptr, xshape, chi, nullptr, nullptr, nullptr, a) != SGT_OK) return 0;
  return a.used;
}

SGT_API int sgt_mpo_mps_zipup(int n, const double* const* W, const int64_t* wshape, const double* const* X,
                              const int64_t* xshape, int64_t chi, double* const* out, double* discarded,
                              int* status, void* ws, size_t ws_bytes, void* stream) {
  Arena a(ws, ws_bytes);
  return zipup_impl(as_stream(stream), n, W, wshape, X, xshape, chi, out, discarded, status, a);
}

}  // extern "C"
