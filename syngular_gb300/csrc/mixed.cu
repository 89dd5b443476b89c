// MPO x MPS product followed by TT-SVD rounding: the metric operation.
//
// precision = SGT_PREC_F64: raw product cores in FP64, then the Householder
// QR sweep + one-sided Jacobi TT-SVD of sweeps.cu.
//
// precision = SGT_PREC_TF32 / SGT_PREC_TF32X3 (Gram form): the same rounding
// expressed through Gram matrices, so that every O(R^3) step is a tensor-core
// GEMM and no QR is needed.  With P_k the product cores (bond R_k = a_k b_k):
//   G_0 = [1],  G_{k+1} = sum_p P_k[:,p,:]^T G_k P_k[:,p,:]       (left Gram)
//   right to left, with F_{N} = [1]:
//     Y_k = P_k F_{k+1}  (R_k x p*chi_{k+1}),  Z_k = Y_k^T G_k Y_k
//     Z_k = V diag(s^2) V^T;  core_k = V[:, :chi]^T,  F_k = Y_k V[:, :chi]
//   core_0 = P_0 F_1.
// In exact arithmetic Z_k = M_k^T M_k for the unfolding M_k that the
// QR-then-SVD sweep decomposes, so the kept singular vectors / values are the
// same.  GEMMs: tcgen05 kind::tf32 (one pass, or three passes on split
// hi/lo operands); product cores and Gram matrices are held in FP32; the
// eigen-solves are one-sided block Jacobi on the rows of Z_k in one
// thread-block cluster (svd.cu), after which the kept eigenvectors are
// re-orthonormalised in FP64.
#include <float.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <vector>

#include "common.cuh"

namespace sgt {

int site_contract_mpo_mps(cudaStream_t st, const double* X, int64_t a, int64_t p, int64_t a2,
                          const double* W, int64_t b, int64_t o, int64_t b2, double* P);
size_t svd_round_ws(int n, const int64_t* shape, int64_t chi);
int svd_round_run(cudaStream_t st, int n, const double* const* cores, const int64_t* shape, int64_t chi,
                  double* const* out, double* spectra, double* discarded, int* status, Arena& ar);
void svd_round_plan_public(int n, const int64_t* shape, int64_t chi, std::vector<int64_t>& b,
                           std::vector<int64_t>& x, std::vector<int64_t>& cnt);
int tc_gemm_tf32(cudaStream_t st, int passes, int64_t M, int64_t N, int64_t K, float alpha,
                 const float* Ahi, const float* Alo, int64_t lda, const float* Bhi, const float* Blo,
                 int64_t ldb, float beta, float* C, int64_t ldc, int* err, float* part, int64_t part_floats);
int split_tf32(cudaStream_t st, const float* x, float* hi, float* lo, int64_t n);
int split_f64(cudaStream_t st, const double* x, int64_t ldx, float* hi, float* lo, int64_t rows,
              int64_t cols);
size_t jacobi_rows_ws_bytes_f32(int64_t n, int64_t m);
size_t sym_eig_rows_ws_bytes(int64_t n);
int sym_eig_rows_f32(cudaStream_t st, float* Z, int64_t n, float* Vt, float* lam, int* status, Arena& ar,
                     int method);
int jacobi_rows_f32(cudaStream_t st, float* G, int64_t ldg, int64_t n, int64_t m, float* Vt,
                    int64_t ldv, float* s, int* status, Arena& ar);
size_t sym_eig_ws_bytes(int64_t n);
size_t gram_step_scratch_floats(int64_t chi, int64_t d, int64_t chi2, int64_t D, int64_t dout, int64_t D2);
bool gram_step_supported(int64_t D, int64_t d, int64_t dout, int64_t D2);
int gram_step_structured(cudaStream_t st, int passes, const float* Gh, const float* Gl, const double* X,
                         int64_t chi, int64_t d, int64_t chi2, const double* W, int64_t D, int64_t dout,
                         int64_t D2, float* Gout, float* scratch, int* err);
int sym_eig_f32(cudaStream_t st, const float* Z, int64_t ldz, int64_t n, float* Vt, int64_t ldt, float* lam,
                int* status, Arena& ar, bool* done);
int oz_round_impl(cudaStream_t st, int n, const double* const* W, const int64_t* ws4, const double* const* X,
                  const int64_t* xs, int64_t chi, double* const* out, double* spectra, double* discarded, int* status,
                  Arena& ar);
int oz_round_chain(cudaStream_t st, int n, const double* const* X, const int64_t* xs, int64_t chi, double* const* out,
                   double* spectra, double* discarded, int* status, Arena& ar);

namespace {

// P[(a*B+b), o, (a2*B2+b2)] in FP64, stored as hi = tf32(v), lo = fp32(v - hi).
__global__ void product_split_kernel(const double* __restrict__ X, const double* __restrict__ W,
                                     float* __restrict__ Phi, float* __restrict__ Plo, int64_t Bd,
                                     int64_t I, int64_t O, int64_t A2, int64_t B2, int64_t total) {
  const int64_t ncol = A2 * B2;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx % ncol;
    const int64_t r = idx / ncol;
    const int64_t o = r % O, ab = r / O;
    const int64_t b = ab % Bd, a = ab / Bd;
    const int64_t a2 = c / B2, b2 = c % B2;
    double acc = 0.0;
    for (int64_t i = 0; i < I; ++i)
      acc = fma(X[(a * I + i) * A2 + a2], W[((b * I + i) * O + o) * B2 + b2], acc);
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"((float)acc));
    const float fh = __uint_as_float(h);
    Phi[idx] = fh;
    Plo[idx] = (float)(acc - (double)fh);
  }
}

// x (FP64) -> FP32 pair hi + lo with hi = fl32(x), |x - hi - lo| <= 2^-48 |x|
__global__ void f64_pair_kernel(const double* __restrict__ x, float* __restrict__ hi, float* __restrict__ lo,
                                int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i];
    const float h = (float)v;
    hi[i] = h;
    lo[i] = (float)(v - (double)h);
  }
}

// The product core P[(a,b), o, (a2,b2)] = sum_i X[a,i,a2] W[b,i,o,b2] in FP32
// arithmetic from the FP32 pairs of X and W: error-free products (FMA) and
// two-sum accumulation carry ~44 bits, then the TF32 hi / FP32 lo split of
// the result.  One CTA row per (a, b, o) row of P (grid.y), threads along
// (a2, b2): FP32 throughput instead of GB300's FP64 rate, so the kernel is
// bound by writing hi and lo.
__global__ void product_pair_split_kernel(const float* __restrict__ Xh, const float* __restrict__ Xl,
                                          const float* __restrict__ Wh, const float* __restrict__ Wl,
                                          float* __restrict__ Phi, float* __restrict__ Plo, int Bd, int I, int O,
                                          int A2, int B2, int ncol) {
  const int r = blockIdx.y;
  const int o = r % O, ab = r / O, b = ab % Bd, a = ab / Bd;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncol) return;
  const int a2 = c / B2, b2 = c - a2 * B2;
  float sum = 0.f, t = 0.f;
  for (int i = 0; i < I; ++i) {
    const int64_t xi = ((int64_t)a * I + i) * A2 + a2;
    const int64_t wi = (((int64_t)b * I + i) * O + o) * B2 + b2;
    const float xh = Xh[xi], xl = Xl[xi], wh = Wh[wi], wl = Wl[wi];
    const float prod = xh * wh;
    const float e = fmaf(xh, wh, -prod);
    const float cross = fmaf(xh, wl, xl * wh);
    const float s2 = sum + prod;
    const float bb = s2 - sum;
    const float err = (sum - (s2 - bb)) + (prod - bb);
    sum = s2;
    t += err + e + cross;
  }
  const float v = sum + t;
  uint32_t h;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
  const float fh = __uint_as_float(h);
  const int64_t idx = (int64_t)r * ncol + c;
  Phi[idx] = fh;
  Plo[idx] = (sum - fh) + t;
}

// dst[b] (cols x rows, ldd) = src[b]^T (rows x cols, lds), batch stride sb / db.
__global__ void transpose_f32_kernel(float* __restrict__ dst, int64_t ldd, int64_t db,
                                     const float* __restrict__ src, int64_t lds, int64_t sb,
                                     int64_t rows, int64_t cols) {
  __shared__ float tile[32][33];
  const int64_t b = blockIdx.z;
  src += b * sb;
  dst += b * db;
  const int64_t tiles_c = (cols + 31) / 32, tiles_r = (rows + 31) / 32;
  for (int64_t t = blockIdx.x; t < tiles_r * tiles_c; t += gridDim.x) {
    const int64_t r0 = (t / tiles_c) * 32, c0 = (t % tiles_c) * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      int64_t r = r0 + i, c = c0 + threadIdx.x;
      tile[i][threadIdx.x] = (r < rows && c < cols) ? src[r * lds + c] : 0.f;
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      int64_t c = c0 + i, r = r0 + threadIdx.x;
      if (c < cols && r < rows) dst[c * ldd + r] = tile[threadIdx.x][i];
    }
    __syncthreads();
  }
}

// Small-shape fallback: C = alpha (Ahi+Alo)(Bhi+Blo)^T + beta C on CUDA cores.
__global__ void gemm_nt_f32_kernel(int64_t M, int64_t N, int64_t K, float alpha,
                                   const float* __restrict__ Ah, const float* __restrict__ Al,
                                   int64_t lda, const float* __restrict__ Bh,
                                   const float* __restrict__ Bl, int64_t ldb, float beta,
                                   float* __restrict__ C, int64_t ldc) {
  __shared__ float As[16][65];
  __shared__ float Bs[16][65];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  const int64_t m0 = (int64_t)blockIdx.y * 64, n0 = (int64_t)blockIdx.x * 64;
  float acc[4][4] = {};
  for (int64_t k0 = 0; k0 < K; k0 += 16) {
    for (int q = 0; q < 4; ++q) {
      int idx = tid + 256 * q;
      int rr = idx / 16, kk = idx % 16;
      int64_t gk = k0 + kk;
      int64_t gm = m0 + rr, gn = n0 + rr;
      float a = 0.f, b = 0.f;
      if (gm < M && gk < K) a = Ah[gm * lda + gk] + (Al ? Al[gm * lda + gk] : 0.f);
      if (gn < N && gk < K) b = Bh[gn * ldb + gk] + (Bl ? Bl[gn * ldb + gk] : 0.f);
      As[kk][rr] = a;
      Bs[kk][rr] = b;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  for (int i = 0; i < 4; ++i) {
    int64_t gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
    for (int j = 0; j < 4; ++j) {
      int64_t gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      float* c = C + gm * ldc + gn;
      *c = (beta == 0.f) ? alpha * acc[i][j] : fmaf(beta, *c, alpha * acc[i][j]);
    }
  }
}

__global__ void f32_to_f64_kernel(const float* __restrict__ src, int64_t lds, double* __restrict__ dst,
                                  int64_t ldd, int64_t rows, int64_t cols) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows * cols;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / cols, c = i % cols;
    dst[r * ldd + c] = (double)src[r * lds + c];
  }
}

// Z <- (Z + Z^T) / 2 (the GEMM-formed Gram projection is symmetric only up to rounding)
__global__ void symmetrize_kernel(float* __restrict__ Z, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / n, c = i % n;
    if (c <= r) continue;
    const float v = 0.5f * (Z[r * n + c] + Z[c * n + r]);
    Z[r * n + c] = v;
    Z[c * n + r] = v;
  }
}

__global__ void set_one_kernel(float* hi, float* lo) {
  hi[0] = 1.f;
  lo[0] = 0.f;
}

// Eigenvalues lam (descending) of Z_k, whose left Gram factor was scaled by
// 2^-gexp: spectra = sqrt(lam 2^gexp), discarded = sum_{j >= keep} lam_j / sum lam_j.
__global__ void gram_spectrum_kernel(const float* __restrict__ lam, int count, int keep,
                                     double* __restrict__ spec_out, double* __restrict__ disc_out,
                                     const int* __restrict__ gexp) {
  __shared__ double red[2][32];
  double tot = 0.0, drop = 0.0;
  const int ge = gexp ? *gexp : 0;
  for (int j = threadIdx.x; j < count; j += blockDim.x) {
    double v = fmax((double)lam[j], 0.0);
    if (spec_out) spec_out[j] = sqrt(ldexp(v, ge));
    tot += v;
    if (j >= keep) drop += v;
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

// max |x| as the bit pattern of a non-negative float (ordered like the value)
__global__ void absmax_bits_kernel(const float* __restrict__ x, int64_t n, unsigned* __restrict__ out) {
  float m = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(x[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(out, __float_as_uint(m));
}

// x 2^-e split into TF32 hi / FP32 lo, e = the binary exponent of max |x|
// (exact scaling: keeps the FP32 Gram recursion of long chains in range);
// gexp_next = gexp_prev + e.
__global__ void split_scaled_kernel(const float* __restrict__ x, float* __restrict__ hi, float* __restrict__ lo,
                                    int64_t n, const unsigned* __restrict__ maxbits,
                                    const int* __restrict__ gexp_prev, int* __restrict__ gexp_next) {
  const float m = __uint_as_float(*maxbits);
  int e = 0;
  if (m > 0.f && isfinite(m)) frexpf(m, &e);
  if (blockIdx.x == 0 && threadIdx.x == 0) *gexp_next = *gexp_prev + e;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float v = ldexpf(x[i], -e);
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
    const float fh = __uint_as_float(h);
    hi[i] = fh;
    lo[i] = v - fh;
  }
}

__global__ void merge_status_kernel(const int* __restrict__ st, int n, int* __restrict__ out,
                                    const int* __restrict__ tc_err) {
  if (threadIdx.x != 0) return;
  int r = 0;
  for (int k = 1; k < n; ++k) {
    if (st[k] < 0) {
      r = -1;
      break;
    }
    r = max(r, st[k]);
  }
  if (tc_err && *tc_err) r = -2;
  *out = r;
}

// Eigensolver of the projected Gram matrices (sgt_sym_eig_f32 method 1, 2 or 3):
// SGT_EIG_METHOD in the environment sets the initial choice, sgt_eig_method()
// changes it.
std::atomic<int> g_eig_method{0};

int eig_method() {
  int m = g_eig_method.load(std::memory_order_relaxed);
  if (m == 0) {
    const char* e = getenv("SGT_EIG_METHOD");
    const int v = e ? atoi(e) : 1;
    m = (v >= 1 && v <= 3) ? v : 1;
    int expected = 0;
    if (!g_eig_method.compare_exchange_strong(expected, m)) m = expected;
  }
  return m;
}

}  // namespace

// The first-approximation eigensolver of the BF16X6 form: the method chosen
// through sgt_eig_method or SGT_EIG_METHOD when one was chosen, else method 2
// (Jacobi on the rows of the Cholesky factor: about two thirds of the sweeps of
// method 1, and its lower accuracy near the cut is what the refinement after it
// removes).
int eig_method_current() {
  const int m = g_eig_method.load(std::memory_order_relaxed);
  if (m != 0) return m;
  const char* e = getenv("SGT_EIG_METHOD");
  const int v = e ? atoi(e) : 0;
  return (v >= 1 && v <= 3) ? v : 2;
}

namespace {

inline unsigned gs(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(n, 256), 152 * 16));
}

int transpose_f32(cudaStream_t st, float* dst, int64_t ldd, int64_t db, const float* src, int64_t lds,
                  int64_t sb, int64_t rows, int64_t cols, int64_t batch) {
  if (rows <= 0 || cols <= 0 || batch <= 0) return SGT_OK;
  int64_t tiles = cdiv(rows, 32) * cdiv(cols, 32);
  dim3 g((unsigned)std::min<int64_t>(tiles, 1024), 1, (unsigned)batch);
  transpose_f32_kernel<<<g, dim3(32, 8), 0, st>>>(dst, ldd, db, src, lds, sb, rows, cols);
  SGT_LAUNCHED();
  return SGT_OK;
}

struct Site4 {
  int64_t b, i, o, b2;
};

}  // namespace

// C = alpha A B^T + beta C (A: M x K, B: N x K, row-major fp32 hi/lo pairs).
// tcgen05 when TMA can address the operands, CUDA cores otherwise; `part`
// (part_floats floats, may be null) lets the tensor-core GEMM split K when the
// output has few tiles.
int gemm_nt_dispatch(cudaStream_t st, int passes, int64_t M, int64_t N, int64_t K, float alpha, const float* Ah,
            const float* Al, int64_t lda, const float* Bh, const float* Bl, int64_t ldb, float beta,
            float* C, int64_t ldc, int* err, float* part = nullptr, int64_t part_floats = 0) {
  if (M <= 0 || N <= 0) return SGT_OK;
  auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
  const bool tc_ok = K >= 16 && lda % 4 == 0 && ldb % 4 == 0 && al16(Ah) && al16(Bh) &&
                     (passes == 1 || (al16(Al) && al16(Bl))) && M * N * K >= (int64_t)1 << 22;
  if (tc_ok)
    return tc_gemm_tf32(st, passes, M, N, K, alpha, Ah, Al, lda, Bh, Bl, ldb, beta, C, ldc, err, part, part_floats);
  dim3 g((unsigned)cdiv(N, 64), (unsigned)cdiv(M, 64));
  gemm_nt_f32_kernel<<<g, 256, 0, st>>>(M, N, std::max<int64_t>(K, 0), alpha, Ah, passes == 3 ? Al : nullptr,
                                        lda, Bh, passes == 3 ? Bl : nullptr, ldb, beta, C, ldc);
  SGT_LAUNCHED();
  return SGT_OK;
}

// ---------------------------------------------------------------------------
static int mixed_round_impl(cudaStream_t st, int n, const double* const* W, const int64_t* ws4,
                            const double* const* X, const int64_t* xs, int64_t chi, int passes,
                            double* const* out, double* spectra, double* discarded, int* status,
                            Arena& ar) {
  std::vector<Site4> w(n);
  std::vector<int64_t> R(n + 1), Pd(n), shp(3 * n);
  for (int k = 0; k < n; ++k) {
    w[k] = {ws4[4 * k], ws4[4 * k + 1], ws4[4 * k + 2], ws4[4 * k + 3]};
    SGT_REQUIRE(xs[3 * k + 1] == w[k].i, SGT_ERR_INVALID, "mpo_mps_round: leg mismatch at site %d", k);
    R[k] = xs[3 * k] * w[k].b;
    Pd[k] = w[k].o;
  }
  R[n] = xs[3 * (n - 1) + 2] * w[n - 1].b2;
  SGT_REQUIRE(R[0] == 1 && R[n] == 1, SGT_ERR_INVALID, "mpo_mps_round: boundary bonds must be 1");
  for (int k = 0; k < n; ++k) shp[3 * k] = R[k], shp[3 * k + 1] = Pd[k], shp[3 * k + 2] = R[k + 1];
  std::vector<int64_t> bb, x, cnt;
  svd_round_plan_public(n, shp.data(), chi, bb, x, cnt);

  // structured Gram recursion (gram.cu) unless a core's bonds are too large
  // for its shared-memory contraction kernel; then dense GEMMs on the
  // transposed product cores
  bool structured = true;
  int64_t gscratch = 1;
  for (int k = 0; k + 1 < n; ++k) {
    structured = structured && gram_step_supported(w[k].b, w[k].i, w[k].o, w[k].b2);
    gscratch = std::max<int64_t>(gscratch, (int64_t)gram_step_scratch_floats(xs[3 * k], xs[3 * k + 1],
                                                                              xs[3 * k + 2], w[k].b, w[k].o,
                                                                              w[k].b2));
  }
  std::vector<float*> Ph(n), Pl(n), Pth(n), Ptl(n), Gh(n), Gl(n);
  int64_t rmax = 1, cmax = 1, smax = 1;
  for (int k = 0; k < n; ++k) {
    const int64_t sz = R[k] * Pd[k] * R[k + 1];
    Ph[k] = ar.take<float>(sz);
    Pl[k] = ar.take<float>(sz);
    if (!structured) {
      Pth[k] = ar.take<float>(sz);
      Ptl[k] = ar.take<float>(sz);
    }
    Gh[k] = ar.take<float>(R[k] * R[k]);
    Gl[k] = ar.take<float>(R[k] * R[k]);
    rmax = std::max(rmax, R[k + 1]);
    rmax = std::max(rmax, R[k]);
    cmax = std::max(cmax, Pd[k] * x[k + 1]);
    smax = std::max(smax, sz);
  }
  float* Gacc = ar.take<float>(rmax * rmax);
  float* Ht = structured ? nullptr : ar.take<float>(rmax * rmax);
  float* Hth = structured ? nullptr : ar.take<float>(rmax * rmax);
  float* Htl = structured ? nullptr : ar.take<float>(rmax * rmax);
  float* gsc = structured ? ar.take<float>(gscratch) : nullptr;
  float* Ytp = structured ? ar.take<float>(cmax * rmax) : nullptr;
  float* Fth = ar.take<float>(chi * rmax);
  float* Ftl = ar.take<float>(chi * rmax);
  float* Ftn = ar.take<float>(chi * rmax);
  float* Yt = ar.take<float>(cmax * rmax);
  float* Yth = ar.take<float>(cmax * rmax);
  float* Ytl = ar.take<float>(cmax * rmax);
  float* Y = ar.take<float>(cmax * rmax);
  float* Yh = ar.take<float>(cmax * rmax);
  float* Yl = ar.take<float>(cmax * rmax);
  float* GY = ar.take<float>(cmax * rmax);
  float* GYh = ar.take<float>(cmax * rmax);
  float* GYl = ar.take<float>(cmax * rmax);
  float* Z = ar.take<float>(cmax * cmax);
  float* Vt = ar.take<float>(cmax * cmax);
  float* Vh = ar.take<float>(cmax * cmax);
  float* Vl = ar.take<float>(cmax * cmax);
  float* lam = ar.take<float>(cmax);
  double* Vd = ar.take<double>(chi * cmax);
  double* Sd = ar.take<double>(chi * chi);
  int64_t xmax = 1, wmax = 1;
  for (int k = 0; k < n; ++k) {
    xmax = std::max<int64_t>(xmax, xs[3 * k] * xs[3 * k + 1] * xs[3 * k + 2]);
    wmax = std::max<int64_t>(wmax, w[k].b * w[k].i * w[k].o * w[k].b2);
  }
  float* pXh = ar.take<float>(xmax);
  float* pXl = ar.take<float>(xmax);
  float* pWh = ar.take<float>(wmax);
  float* pWl = ar.take<float>(wmax);
  double* skw = ar.take<double>(16 * chi * cmax);  // split-K partials of the FP64 re-orthonormalisation
  // split-K slices of the tensor-core GEMMs whose outputs have few tiles
  const int64_t tcp = std::min<int64_t>((int64_t)1 << 21, 8 * rmax * std::max<int64_t>(cmax, chi));
  float* tcpart = ar.take<float>(tcp);
  int* stat = ar.take<int>(n + 1);
  int* tc_err = ar.take<int>(1);
  int* gexp = ar.take<int>(n + 1);
  unsigned* gmax = ar.take<unsigned>(1);
  const size_t jbytes = std::max(std::max(jacobi_rows_ws_bytes_f32(cmax, cmax), sym_eig_ws_bytes(cmax)),
                                 sym_eig_rows_ws_bytes(cmax));
  char* jscratch = ar.take<char>(jbytes);
  if (ar.measure) return SGT_OK;
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "mpo_mps_round: workspace too small");
  SGT_CUDA(cudaMemsetAsync(stat, 0, sizeof(int) * (n + 1), st));
  SGT_CUDA(cudaMemsetAsync(tc_err, 0, sizeof(int), st));
  SGT_CUDA(cudaMemsetAsync(gexp, 0, sizeof(int) * (n + 1), st));
  // G_{k+1} (in Gacc) -> power-of-two scaled hi / lo, exponent into gexp[k + 1]
  auto split_gram = [&](int k, int64_t count) -> int {
    SGT_CUDA(cudaMemsetAsync(gmax, 0, sizeof(unsigned), st));
    absmax_bits_kernel<<<gs(count), 256, 0, st>>>(Gacc, count, gmax);
    SGT_LAUNCHED();
    split_scaled_kernel<<<gs(count), 256, 0, st>>>(Gacc, Gh[k + 1], Gl[k + 1], count, gmax, gexp + k, gexp + k + 1);
    SGT_LAUNCHED();
    return SGT_OK;
  };

  // ---- product cores in both layouts ----
  for (int k = 0; k < n; ++k) {
    const int64_t sz = R[k] * Pd[k] * R[k + 1];
    const int64_t a2 = xs[3 * k + 2];
    const int64_t nrow = R[k] * Pd[k], ncol = R[k + 1];
    const int64_t xsz = xs[3 * k] * xs[3 * k + 1] * xs[3 * k + 2], wsz = w[k].b * w[k].i * w[k].o * w[k].b2;
    if (nrow <= 65535 && ncol < ((int64_t)1 << 31)) {
      f64_pair_kernel<<<gs(xsz), 256, 0, st>>>(X[k], pXh, pXl, xsz);
      SGT_LAUNCHED();
      f64_pair_kernel<<<gs(wsz), 256, 0, st>>>(W[k], pWh, pWl, wsz);
      SGT_LAUNCHED();
      product_pair_split_kernel<<<dim3((unsigned)cdiv(ncol, 256), (unsigned)nrow), 256, 0, st>>>(
          pXh, pXl, pWh, pWl, Ph[k], Pl[k], (int)w[k].b, (int)w[k].i, (int)w[k].o, (int)a2, (int)w[k].b2, (int)ncol);
      SGT_LAUNCHED();
    } else {
      product_split_kernel<<<gs(sz), 256, 0, st>>>(X[k], W[k], Ph[k], Pl[k], w[k].b, w[k].i, w[k].o, a2,
                                                    w[k].b2, sz);
      SGT_LAUNCHED();
    }
    if (structured) continue;
    // Pt[p] (R' x R) = (P[:, p, :])^T, P[:, p, :] is R x R' with row stride p*R'
    SGT_TRY(transpose_f32(st, Pth[k], R[k], R[k + 1] * R[k], Ph[k], Pd[k] * R[k + 1], R[k + 1], R[k],
                          R[k + 1], Pd[k]));
    SGT_TRY(transpose_f32(st, Ptl[k], R[k], R[k + 1] * R[k], Pl[k], Pd[k] * R[k + 1], R[k + 1], R[k],
                          R[k + 1], Pd[k]));
  }
  // ---- left Gram recursion ----
  set_one_kernel<<<1, 1, 0, st>>>(Gh[0], Gl[0]);
  SGT_LAUNCHED();
  // structured: G_k is kept with its columns in (b, a) order (see gram.cu)
  for (int k = 0; structured && k + 1 < n; ++k) {
    SGT_TRY(gram_step_structured(st, passes, Gh[k], Gl[k], X[k], xs[3 * k], xs[3 * k + 1], xs[3 * k + 2], W[k],
                                 w[k].b, w[k].o, w[k].b2, Gacc, gsc, tc_err));
    SGT_TRY(split_gram(k, R[k + 1] * R[k + 1]));
  }
  for (int k = 0; !structured && k + 1 < n; ++k) {
    const int64_t r = R[k], r2 = R[k + 1];
    for (int64_t pi = 0; pi < Pd[k]; ++pi) {
      const float* Ah = Pth[k] + pi * r2 * r;
      const float* Al = Ptl[k] + pi * r2 * r;
      // Ht (r2 x r) = Pt[p] G_k^T
      SGT_TRY(gemm_nt_dispatch(st, passes, r2, r, r, 1.f, Ah, Al, r, Gh[k], Gl[k], r, 0.f, Ht, r, tc_err));
      SGT_TRY(split_tf32(st, Ht, Hth, Htl, r2 * r));
      // G_{k+1} += Pt[p] Ht^T
      SGT_TRY(gemm_nt_dispatch(st, passes, r2, r2, r, 1.f, Ah, Al, r, Hth, Htl, r, pi == 0 ? 0.f : 1.f, Gacc, r2,
                      tc_err));
    }
    SGT_TRY(split_gram(k, r2 * r2));
  }
  // ---- right-to-left projection and eigen-solves ----
  set_one_kernel<<<1, 1, 0, st>>>(Fth, Ftl);
  SGT_LAUNCHED();
  for (int k = n - 1; k >= 0; --k) {
    const int64_t r = R[k], r2 = R[k + 1], p = Pd[k], xc = x[k + 1], c = p * xc;
    // Yt (c x r): rows p*xc..: Ft (xc x r2) * P[:, p, :]^T
    for (int64_t pi = 0; pi < p; ++pi) {
      SGT_TRY(gemm_nt_dispatch(st, passes, xc, r, r2, 1.f, Fth, Ftl, r2, Ph[k] + pi * r2, Pl[k] + pi * r2, p * r2,
                      0.f, Yt + pi * xc * r, r, tc_err, tcpart, tcp));
    }
    if (k == 0) {
      // core_0[0][p][c] = Yt[p*xc + c][0]
      f32_to_f64_kernel<<<gs(c), 256, 0, st>>>(Yt, 1, out[0], 1, c, 1);
      SGT_LAUNCHED();
      break;
    }
    const int64_t keep = x[k];
    SGT_TRY(split_tf32(st, Yt, Yth, Ytl, c * r));
    // GY^T (c x r) = Yt G_k^T ;  Z (c x c) = Yt GY
    if (structured) {
      // G_k's columns are in (b, a) order: contract with Yt's columns permuted alike
      const int64_t chik = xs[3 * k], Dk = w[k].b;
      SGT_TRY(transpose_f32(st, Ytp, chik, r, Yt, Dk, r, chik, Dk, c));
      SGT_TRY(split_tf32(st, Ytp, Y, Yl, c * r));  // Y / Yl reused as the split of Ytp
      SGT_TRY(gemm_nt_dispatch(st, passes, c, r, r, 1.f, Y, Yl, r, Gh[k], Gl[k], r, 0.f, GY, r, tc_err, tcpart, tcp));
    } else {
      SGT_TRY(gemm_nt_dispatch(st, passes, c, r, r, 1.f, Yth, Ytl, r, Gh[k], Gl[k], r, 0.f, GY, r, tc_err, tcpart,
                               tcp));
    }
    SGT_TRY(split_tf32(st, GY, GYh, GYl, c * r));
    SGT_TRY(gemm_nt_dispatch(st, passes, c, c, r, 1.f, Yth, Ytl, r, GYh, GYl, r, 0.f, Z, c, tc_err, tcpart, tcp));
    symmetrize_kernel<<<gs(c * c), 256, 0, st>>>(Z, c);
    SGT_LAUNCHED();
    // eigenpairs of the symmetric Z: one-sided Jacobi on the rows of Z (block,
    // cluster-resident).  The two-sided solver (eig.cu) converges in fewer
    // sweeps but its FP32 stopping floor costs accuracy next to the cut.
    Arena ja(jscratch, jbytes);
    SGT_TRY(sym_eig_rows_f32(st, Z, c, Vt, lam, stat + k, ja, eig_method()));
    // core_k = Vt[:keep], re-orthonormalised in FP64 by one Newton-Schulz step
    // V <- 1.5 V - 0.5 (V V^T) V (the FP32 rotations leave |V V^T - I| ~ 1e-6)
    f32_to_f64_kernel<<<gs(keep * c), 256, 0, st>>>(Vt, c, Vd, c, keep, c);
    SGT_LAUNCHED();
    SGT_TRY(gemm_f64_splitk(st, false, true, keep, keep, c, 1.0, Vd, c, Vd, c, 0.0, Sd, keep, skw,
                            splitk_count(keep, keep, c)));
    SGT_TRY(copy2d_f64(st, out[k], c, Vd, c, keep, c));
    SGT_TRY(gemm_f64_splitk(st, false, false, keep, c, keep, -0.5, Sd, keep, Vd, c, 1.5, out[k], c, skw,
                            splitk_count(keep, c, keep)));
    double* spec_k = nullptr;
    if (spectra) {
      int64_t off = 0;
      for (int j = 1; j < k; ++j) off += cnt[j];
      spec_k = spectra + off;
    }
    gram_spectrum_kernel<<<1, 256, 0, st>>>(lam, (int)cnt[k], (int)keep, spec_k,
                                            discarded ? discarded + (k - 1) : nullptr, gexp + k);
    SGT_LAUNCHED();
    // Ft_k (keep x r) = Vt[:keep] Y^T with Y = Yt^T (r x c)
    SGT_TRY(transpose_f32(st, Y, c, 0, Yt, r, 0, c, r, 1));
    SGT_TRY(split_tf32(st, Y, Yh, Yl, r * c));
    SGT_TRY(split_f64(st, out[k], c, Vh, Vl, keep, c));
    SGT_TRY(gemm_nt_dispatch(st, passes, keep, r, c, 1.f, Vh, Vl, c, Yh, Yl, c, 0.f, Ftn, r, tc_err, tcpart, tcp));
    SGT_TRY(split_tf32(st, Ftn, Fth, Ftl, keep * r));
  }
  if (status) {
    merge_status_kernel<<<1, 32, 0, st>>>(stat, n, status, tc_err);
    SGT_LAUNCHED();
  }
  return SGT_OK;
}

namespace {
// Identity operator cores eye[k] = I (d_k x d_k) for sites k0 .. k0 + count - 1;
// the physical dims travel by value in the launch (no host buffer that a
// captured graph would have to read again at replay).
constexpr int EYE_CHUNK = 256;
struct EyeDims {
  int d[EYE_CHUNK];
};
__global__ void identity_cores_kernel(double* __restrict__ eye, const EyeDims dims, int k0, int count, int stride) {
  for (int j = blockIdx.x; j < count; j += gridDim.x) {
    const int d = dims.d[j];
    double* e = eye + (int64_t)(k0 + j) * stride;
    for (int i = threadIdx.x; i < d * d; i += blockDim.x) e[i] = (i / d == i % d) ? 1.0 : 0.0;
  }
}
}  // namespace

// TT-SVD rounding of a plain chain in the Gram form: the chain equals the
// product of a bond-1 identity MPO with itself, so the MPO x MPS pipeline
// applies unchanged (one d x d identity core per site, built on the device).
int mixed_round_chain(cudaStream_t st, int n, const double* const* X, const int64_t* xs, int64_t chi,
                      int precision, double* const* out, double* spectra, double* discarded, int* status,
                      Arena& ar) {
  if (precision == SGT_PREC_BF16X6) return oz_round_chain(st, n, X, xs, chi, out, spectra, discarded, status, ar);
  SGT_REQUIRE(precision == SGT_PREC_TF32 || precision == SGT_PREC_TF32X3, SGT_ERR_INVALID,
              "round: precision %d has no Gram form", precision);
  std::vector<int64_t> w4(4 * (size_t)n);
  std::vector<int> dims(n);
  int64_t dmax = 1;
  for (int k = 0; k < n; ++k) {
    const int64_t d = xs[3 * k + 1];
    w4[4 * k] = 1;
    w4[4 * k + 1] = d;
    w4[4 * k + 2] = d;
    w4[4 * k + 3] = 1;
    dims[k] = (int)d;
    dmax = std::max(dmax, d);
  }
  double* eye = ar.take<double>((size_t)n * dmax * dmax);
  std::vector<const double*> W(n, nullptr);
  if (!ar.measure) {
    SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "round: workspace too small");
    for (int k0 = 0; k0 < n; k0 += EYE_CHUNK) {
      EyeDims ed;
      const int count = std::min(EYE_CHUNK, n - k0);
      for (int j = 0; j < count; ++j) ed.d[j] = dims[k0 + j];
      identity_cores_kernel<<<(unsigned)count, 128, 0, st>>>(eye, ed, k0, count, (int)(dmax * dmax));
      SGT_LAUNCHED();
    }
    for (int k = 0; k < n; ++k) W[k] = eye + (int64_t)k * dmax * dmax;
  }
  return mixed_round_impl(st, n, W.data(), w4.data(), X, xs, chi, precision == SGT_PREC_TF32 ? 1 : 3, out, spectra,
                          discarded, status, ar);
}

static int mpo_mps_round_impl(cudaStream_t st, int n, const double* const* W, const int64_t* ws4,
                              const double* const* X, const int64_t* xs, int64_t chi, int precision,
                              double* const* out, double* spectra, double* discarded, int* status,
                              Arena& ar) {
  SGT_REQUIRE(n >= 1 && ws4 && xs, SGT_ERR_INVALID, "mpo_mps_round: bad arguments");
  SGT_REQUIRE(chi >= 1, SGT_ERR_INVALID, "mpo_mps_round: chi must be >= 1");
  for (int k = 0; k + 1 < n; ++k) {
    SGT_REQUIRE(xs[3 * k + 2] == xs[3 * (k + 1)] && ws4[4 * k + 3] == ws4[4 * (k + 1)], SGT_ERR_INVALID,
                "mpo_mps_round: bond mismatch at site %d", k);
  }
  if (precision == SGT_PREC_TF32 || precision == SGT_PREC_TF32X3)
    return mixed_round_impl(st, n, W, ws4, X, xs, chi, precision == SGT_PREC_TF32 ? 1 : 3, out, spectra,
                            discarded, status, ar);
  if (precision == SGT_PREC_BF16X6)
    return oz_round_impl(st, n, W, ws4, X, xs, chi, out, spectra, discarded, status, ar);
  SGT_REQUIRE(precision == SGT_PREC_F64, SGT_ERR_INVALID, "mpo_mps_round: unsupported precision %d",
              precision);
  // plain FP64: raw product into the workspace, then the QR + Jacobi TT-SVD
  std::vector<int64_t> shp(3 * n);
  std::vector<double*> P(n);
  for (int k = 0; k < n; ++k) {
    shp[3 * k] = xs[3 * k] * ws4[4 * k];
    shp[3 * k + 1] = ws4[4 * k + 2];
    shp[3 * k + 2] = xs[3 * k + 2] * ws4[4 * k + 3];
    P[k] = ar.take<double>(shp[3 * k] * shp[3 * k + 1] * shp[3 * k + 2]);
  }
  if (ar.measure) {
    ar.used += svd_round_ws(n, shp.data(), chi);
    return SGT_OK;
  }
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "mpo_mps_round: workspace too small");
  for (int k = 0; k < n; ++k) {
    SGT_TRY(site_contract_mpo_mps(st, X[k], xs[3 * k], xs[3 * k + 1], xs[3 * k + 2], W[k], ws4[4 * k],
                                  ws4[4 * k + 2], ws4[4 * k + 3], P[k]));
  }
  Arena rest(ar.base + ar.used, ar.cap - ar.used);
  return svd_round_run(st, n, P.data(), shp.data(), chi, out, spectra, discarded, status, rest);
}

}  // namespace sgt

using namespace sgt;

extern "C" {

SGT_API size_t sgt_mpo_mps_round_workspace_size(int n, const int64_t* wshape, const int64_t* xshape,
                                                int64_t chi, int precision) {
  Arena a = Arena::measuring();
  if (mpo_mps_round_impl(nullptr, n, nullptr, wshape, nullptr, xshape, chi, precision, nullptr, nullptr,
                         nullptr, nullptr, a) != SGT_OK)
    return 0;
  return a.used;
}

SGT_API int sgt_mpo_mps_round(int n, const double* const* W, const int64_t* wshape, const double* const* X,
                              const int64_t* xshape, int64_t chi, int precision, double* const* out,
                              double* spectra, double* discarded, int* status, void* ws, size_t ws_bytes,
                              void* stream) {
  SGT_REQUIRE(W && X && out, SGT_ERR_INVALID, "mpo_mps_round: null argument");
  Arena a(ws, ws_bytes);
  return mpo_mps_round_impl(as_stream(stream), n, W, wshape, X, xshape, chi, precision, out, spectra,
                            discarded, status, a);
}

}  // extern "C"

extern "C" SGT_API int sgt_eig_method(int method) {
  const int prev = sgt::eig_method();
  if (method >= 1 && method <= 3) sgt::g_eig_method.store(method, std::memory_order_relaxed);
  return prev;
}
