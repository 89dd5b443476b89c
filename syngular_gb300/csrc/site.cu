// Site-local kernels: MPO x MPS / MPO x MPO core contractions, the direct-sum
// (bond concatenation) kernel and small elementwise helpers.
//
// The contractions are outer-product expansions with a tiny inner dimension
// (the physical leg): each thread produces two adjacent outputs of one row and
// stores them as a 16-byte vector when the row is even-sized.  On GB300 they
// are bound by the FP64 FMA rate (p FMAs per 8-byte output, ~0.6 TFMA/s for
// the chip) before the HBM write of the product core.
#include <algorithm>

#include "common.cuh"

namespace sgt {
namespace {

// P[(a*B+b), o, (a2*B2+b2)] = sum_i X[a,i,a2] * W[b,i,o,b2]
// grid.y enumerates rows r = (a*B + b)*O + o (chunked in z for > 65535 rows).
__global__ void contract_mpo_mps_kernel(const double* __restrict__ X, const double* __restrict__ W,
                                        double* __restrict__ P, int64_t Bd, int64_t I, int64_t O,
                                        int64_t A2, int64_t B2, int64_t rows, bool vec) {
  const int64_t r = (int64_t)blockIdx.y + (int64_t)blockIdx.z * 65535;
  if (r >= rows) return;
  const int64_t o = r % O;
  const int64_t ab = r / O;
  const int64_t b = ab % Bd, a = ab / Bd;
  const int64_t ncol = A2 * B2;
  const int64_t c0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 2;
  if (c0 >= ncol) return;
  const double* xr = X + a * I * A2;           // X[a, :, :]
  const double* wr = W + (b * I * O + o) * B2;  // W[b, 0, o, :], stride over i = O*B2
  double v[2];
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    int64_t c = c0 + e;
    double acc = 0.0;
    if (c < ncol) {
      int64_t a2 = c / B2, b2 = c % B2;
      for (int64_t i = 0; i < I; ++i) acc = fma(xr[i * A2 + a2], wr[i * O * B2 + b2], acc);
    }
    v[e] = acc;
  }
  double* out = P + r * ncol + c0;
  if (vec) {
    *reinterpret_cast<double2*>(out) = make_double2(v[0], v[1]);
  } else {
    out[0] = v[0];
    if (c0 + 1 < ncol) out[1] = v[1];
  }
}

// P[(b*C+c), i, o, (b2*C2+c2)] = sum_m A[b,i,m,b2] * B[c,m,o,c2]
// rows r = ((b*C + c)*I + i)*O + o
__global__ void contract_mpo_mpo_kernel(const double* __restrict__ A, const double* __restrict__ Bm,
                                        double* __restrict__ P, int64_t Cd, int64_t I, int64_t Mm,
                                        int64_t O, int64_t B2, int64_t C2, int64_t rows, bool vec) {
  const int64_t r = (int64_t)blockIdx.y + (int64_t)blockIdx.z * 65535;
  if (r >= rows) return;
  const int64_t o = r % O;
  int64_t t = r / O;
  const int64_t i = t % I;
  t /= I;
  const int64_t c = t % Cd, b = t / Cd;
  const int64_t ncol = B2 * C2;
  const int64_t c0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 2;
  if (c0 >= ncol) return;
  const double* ar = A + (b * I + i) * Mm * B2;  // A[b, i, :, :]
  const double* br = Bm + c * Mm * O * C2 + o * C2;  // B[c, 0, o, :], stride over m = O*C2
  double v[2];
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    int64_t cc = c0 + e;
    double acc = 0.0;
    if (cc < ncol) {
      int64_t b2 = cc / C2, c2 = cc % C2;
      for (int64_t m = 0; m < Mm; ++m) acc = fma(ar[m * B2 + b2], br[m * O * C2 + c2], acc);
    }
    v[e] = acc;
  }
  double* out = P + r * ncol + c0;
  if (vec) {
    *reinterpret_cast<double2*>(out) = make_double2(v[0], v[1]);
  } else {
    out[0] = v[0];
    if (c0 + 1 < ncol) out[1] = v[1];
  }
}

struct ConcatSite {
  const double* A;
  const double* B;
  double* out;
  int64_t la, lb, ra, rb, phys;
  int64_t ol, orr;  // output left / right bond
  int64_t begin;    // first flat output index of this site within the launch
  int pos;
};

constexpr int kConcatMax = 96;  // sites per launch (kernel parameter space)

struct ConcatBatch {
  ConcatSite s[kConcatMax];
  int n;
  int64_t total;
};

// One warp per output row (l, p) of one site (grid.y = site): each row is at
// most two contiguous runs copied from A / B or zero-filled, so there is no
// per-element index arithmetic; consecutive lanes move consecutive elements.
__device__ __forceinline__ void copy_run(double* __restrict__ dst, const double* __restrict__ src, int64_t n,
                                         int lane) {
  for (int64_t i = lane; i < n; i += 32) dst[i] = src[i];
}

__device__ __forceinline__ void zero_run(double* __restrict__ dst, int64_t n, int lane) {
  for (int64_t i = lane; i < n; i += 32) dst[i] = 0.0;
}

__global__ void concat_kernel(const __grid_constant__ ConcatBatch batch) {
  const ConcatSite& d = batch.s[blockIdx.y];
  const int64_t rows = d.ol * d.phys;
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int64_t row = (int64_t)blockIdx.x * nw + (threadIdx.x >> 5); row < rows; row += (int64_t)gridDim.x * nw) {
    const int64_t l = row / d.phys, p = row - l * d.phys;
    double* o = d.out + row * d.orr;
    switch (d.pos) {
      case 0:  // first: [A | B] along r
        copy_run(o, d.A + (l * d.phys + p) * d.ra, d.ra, lane);
        copy_run(o + d.ra, d.B + (l * d.phys + p) * d.rb, d.rb, lane);
        break;
      case 2:  // last: stacked along l
        if (l < d.la) copy_run(o, d.A + (l * d.phys + p) * d.ra, d.orr, lane);
        else copy_run(o, d.B + ((l - d.la) * d.phys + p) * d.rb, d.orr, lane);
        break;
      case 3: {  // single site: A + B
        const double* a = d.A + row * d.orr;
        const double* b = d.B + row * d.orr;
        for (int64_t i = lane; i < d.orr; i += 32) o[i] = a[i] + b[i];
        break;
      }
      default:  // middle: block diagonal
        if (l < d.la) {
          copy_run(o, d.A + (l * d.phys + p) * d.ra, d.ra, lane);
          zero_run(o + d.ra, d.rb, lane);
        } else {
          zero_run(o, d.ra, lane);
          copy_run(o + d.ra, d.B + ((l - d.la) * d.phys + p) * d.rb, d.rb, lane);
        }
    }
  }
}

__global__ void fill_kernel(double* p, int64_t n, double v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

__global__ void copy2d_kernel(double* dst, int64_t ldd, const double* src, int64_t lds, int64_t rows,
                              int64_t cols) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows * cols;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / cols, c = i % cols;
    dst[r * ldd + c] = src[r * lds + c];
  }
}

__global__ void scale_kernel(double* p, int64_t n, const double* s, bool inverse) {
  double f = *s;
  if (inverse) f = (f != 0.0) ? 1.0 / f : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] *= f;
}

__global__ void frob_norm_kernel(const double* p, int64_t n, double* out) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc = fma(p[i], p[i], acc);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) *out = sqrt(acc);
  }
}

inline unsigned grid_for(int64_t n, int threads) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(n, threads), 152 * 16));
}

int launch_rows(int64_t rows, int64_t ncol, dim3& grid, int& threads) {
  threads = ncol >= 512 ? 256 : 128;
  int64_t gx = cdiv(cdiv(ncol, 2), threads);
  int64_t gy = std::min<int64_t>(rows, 65535);
  int64_t gz = cdiv(rows, 65535);
  SGT_REQUIRE(gx <= 0x7fffffff && gz <= 65535, SGT_ERR_INVALID, "site contraction too large");
  grid = dim3((unsigned)gx, (unsigned)gy, (unsigned)gz);
  return SGT_OK;
}

}  // namespace

int fill_f64(cudaStream_t st, double* p, int64_t n, double v) {
  if (n <= 0) return SGT_OK;
  fill_kernel<<<grid_for(n, 256), 256, 0, st>>>(p, n, v);
  SGT_LAUNCHED();
  return SGT_OK;
}

int copy2d_f64(cudaStream_t st, double* dst, int64_t ldd, const double* src, int64_t lds,
               int64_t rows, int64_t cols) {
  if (rows <= 0 || cols <= 0) return SGT_OK;
  if (ldd == cols && lds == cols) {
    SGT_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * rows * cols, cudaMemcpyDeviceToDevice, st));
    return SGT_OK;
  }
  copy2d_kernel<<<grid_for(rows * cols, 256), 256, 0, st>>>(dst, ldd, src, lds, rows, cols);
  SGT_LAUNCHED();
  return SGT_OK;
}

int scale_f64(cudaStream_t st, double* p, int64_t n, const double* dev_scale, bool inverse) {
  if (n <= 0) return SGT_OK;
  scale_kernel<<<grid_for(n, 256), 256, 0, st>>>(p, n, dev_scale, inverse);
  SGT_LAUNCHED();
  return SGT_OK;
}

int frob_norm_f64(cudaStream_t st, const double* p, int64_t n, double* out) {
  frob_norm_kernel<<<1, 1024, 0, st>>>(p, n, out);
  SGT_LAUNCHED();
  return SGT_OK;
}

int site_contract_mpo_mps(cudaStream_t st, const double* X, int64_t a, int64_t p, int64_t a2,
                          const double* W, int64_t b, int64_t o, int64_t b2, double* P) {
  int64_t rows = a * b * o, ncol = a2 * b2;
  if (rows == 0 || ncol == 0) return SGT_OK;
  dim3 grid;
  int threads;
  SGT_TRY(launch_rows(rows, ncol, grid, threads));
    const bool vec = (ncol % 2 == 0) && ((reinterpret_cast<uintptr_t>(P) & 15) == 0);
  contract_mpo_mps_kernel<<<grid, threads, 0, st>>>(X, W, P, b, p, o, a2, b2, rows, vec);
  SGT_LAUNCHED();
  return SGT_OK;
}

int site_contract_mpo_mpo(cudaStream_t st, const double* A, int64_t b, int64_t i, int64_t m,
                          int64_t b2, const double* B, int64_t c, int64_t o, int64_t c2, double* P) {
  int64_t rows = b * c * i * o, ncol = b2 * c2;
  if (rows == 0 || ncol == 0) return SGT_OK;
  dim3 grid;
  int threads;
  SGT_TRY(launch_rows(rows, ncol, grid, threads));
    const bool vec = (ncol % 2 == 0) && ((reinterpret_cast<uintptr_t>(P) & 15) == 0);
  contract_mpo_mpo_kernel<<<grid, threads, 0, st>>>(A, B, P, c, i, m, o, b2, c2, rows, vec);
  SGT_LAUNCHED();
  return SGT_OK;
}

static int concat_shape(int pos, int64_t la, int64_t ra, int64_t lb, int64_t rb, int64_t& ol,
                        int64_t& orr) {
  switch (pos) {
    case 0:
      SGT_REQUIRE(la == lb, SGT_ERR_INVALID, "bond_concat: first-site left bonds differ (%lld, %lld)",
                  (long long)la, (long long)lb);
      ol = la, orr = ra + rb;
      return SGT_OK;
    case 1:
      ol = la + lb, orr = ra + rb;
      return SGT_OK;
    case 2:
      SGT_REQUIRE(ra == rb, SGT_ERR_INVALID, "bond_concat: last-site right bonds differ (%lld, %lld)",
                  (long long)ra, (long long)rb);
      ol = la + lb, orr = ra;
      return SGT_OK;
    case 3:
      SGT_REQUIRE(la == lb && ra == rb, SGT_ERR_INVALID, "bond_concat: single-site shapes differ");
      ol = la, orr = ra;
      return SGT_OK;
  }
  set_error("bond_concat: bad position %d", pos);
  return SGT_ERR_INVALID;
}

int bond_concat_chain(cudaStream_t st, int n, const double* const* A, const int64_t* ashape,
                      const double* const* B, const int64_t* bshape, double* const* out,
                      const int* positions) {
  for (int base = 0; base < n; base += kConcatMax) {
    ConcatBatch batch;
    batch.n = std::min(kConcatMax, n - base);
    int64_t total = 0;
    for (int j = 0; j < batch.n; ++j) {
      int k = base + j;
      ConcatSite& d = batch.s[j];
      d.A = A[k], d.B = B[k], d.out = out[k];
      d.la = ashape[3 * k], d.phys = ashape[3 * k + 1], d.ra = ashape[3 * k + 2];
      d.lb = bshape[3 * k], d.rb = bshape[3 * k + 2];
      SGT_REQUIRE(bshape[3 * k + 1] == d.phys, SGT_ERR_INVALID,
                  "bond_concat: physical dims differ at site %d", k);
      d.pos = positions ? positions[k] : (n == 1 ? 3 : (k == 0 ? 0 : (k == n - 1 ? 2 : 1)));
      SGT_TRY(concat_shape(d.pos, d.la, d.ra, d.lb, d.rb, d.ol, d.orr));
      d.begin = total;
      total += d.ol * d.phys * d.orr;
    }
    batch.total = total;
    if (total == 0) continue;
    int64_t maxrows = 1;
    for (int j = 0; j < batch.n; ++j) maxrows = std::max<int64_t>(maxrows, batch.s[j].ol * batch.s[j].phys);
    dim3 grid((unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(maxrows, 8), 1024)), (unsigned)batch.n);
    concat_kernel<<<grid, 256, 0, st>>>(batch);
    SGT_LAUNCHED();
  }
  return SGT_OK;
}

int orthogonality(cudaStream_t st, const double* core, int64_t l, int64_t p, int64_t r, int side,
                  double* out) {
  if (side == 0) {  // L^T L, L = (l*p, r)
    return gemm_f64(st, true, false, r, r, l * p, 1.0, core, r, 0, core, r, 0, 0.0, out, r, 0, 1);
  }
  // R R^T, R = (l, p*r)
  return gemm_f64(st, false, true, l, l, p * r, 1.0, core, p * r, 0, core, p * r, 0, 0.0, out, l, 0, 1);
}

}  // namespace sgt

namespace sgt {
namespace {
__global__ void transpose_kernel(double* __restrict__ dst, int64_t ldd, const double* __restrict__ src,
                                 int64_t lds, int64_t rows, int64_t cols) {
  __shared__ double tile[32][33];
  const int64_t tiles_c = (cols + 31) / 32;
  const int64_t tiles_r = (rows + 31) / 32;
  for (int64_t t = blockIdx.x; t < tiles_r * tiles_c; t += gridDim.x) {
    const int64_t r0 = (t / tiles_c) * 32, c0 = (t % tiles_c) * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      int64_t r = r0 + i, c = c0 + threadIdx.x;
      tile[i][threadIdx.x] = (r < rows && c < cols) ? src[r * lds + c] : 0.0;
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      int64_t c = c0 + i, r = r0 + threadIdx.x;  // dst row = src col
      if (c < cols && r < rows) dst[c * ldd + r] = tile[threadIdx.x][i];
    }
    __syncthreads();
  }
}
}  // namespace

// dst (cols x rows, ldd) = src^T, src (rows x cols, lds)
int transpose_f64(cudaStream_t st, double* dst, int64_t ldd, const double* src, int64_t lds,
                  int64_t rows, int64_t cols) {
  if (rows <= 0 || cols <= 0) return SGT_OK;
  int64_t tiles = cdiv(rows, 32) * cdiv(cols, 32);
  unsigned g = (unsigned)std::min<int64_t>(tiles, 152 * 16);
  transpose_kernel<<<g, dim3(32, 8), 0, st>>>(dst, ldd, src, lds, rows, cols);
  SGT_LAUNCHED();
  return SGT_OK;
}
}  // namespace sgt
