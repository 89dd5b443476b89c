// Site-local kernels: MPO x MPS / MPO x MPO core contractions, the direct-sum
// (bond concatenation) kernel and small elementwise helpers.
//
// The contractions are outer-product expansions with a tiny inner dimension
// (the physical leg), so they are bound by the HBM write of the product core:
// each thread produces two adjacent outputs of one row and stores them as a
// 16-byte vector when the row is even-sized.
#include <algorithm>

#include "common.cuh"

namespace sgt {
namespace {

// One output row of a site contraction:
//   out[j * K2 + k] = sum_t u[t * su + j] * v[t * sv + k],  j < J2, k < K2,
// with few terms t (the physical leg).  The row is written once, so the
// kernels are bound by the HBM write of the product core.  Vector path (K2
// even, 16-byte aligned row): the block has a multiple of K2/2 threads, each
// thread owns one fixed column pair k, k+1 (its v values stay in registers)
// and walks j with a constant stride, so no index division happens inside
// the row and every store is 16 bytes, consecutive threads on consecutive
// addresses.  Scalar path otherwise (32-bit index arithmetic).
template <int REG_TERMS>
__device__ __forceinline__ void outer_row(const double* __restrict__ u, int64_t su, const double* __restrict__ v,
                                          int64_t sv, int terms, int J2, int K2, double* __restrict__ out,
                                          bool vec) {
  const int T = blockDim.x;
  if (vec) {
    const int hp = K2 >> 1;
    const int k = (threadIdx.x % hp) * 2;
    const int jstep = T / hp;
    double va[REG_TERMS][2];
    if (terms <= REG_TERMS) {
#pragma unroll
      for (int t = 0; t < REG_TERMS; ++t)
        if (t < terms) va[t][0] = v[t * sv + k], va[t][1] = v[t * sv + k + 1];
    }
    // pointer walks (no 64-bit index products in the loop: on GB300 the FP64
    // FMAs, two per output pair and term, are the bound, not HBM)
    const int j0 = threadIdx.x / hp;
    const double* up = u + j0;
    double* op = out + (int64_t)j0 * K2 + k;
    const int64_t ostep = (int64_t)jstep * K2;
    for (int j = j0; j < J2; j += jstep, up += jstep, op += ostep) {
      double o0 = 0.0, o1 = 0.0;
      if (terms <= REG_TERMS) {
        const double* ut = up;
#pragma unroll
        for (int t = 0; t < REG_TERMS; ++t)
          if (t < terms) {
            const double x = *ut;
            ut += su;
            o0 = fma(x, va[t][0], o0);
            o1 = fma(x, va[t][1], o1);
          }
      } else {
        for (int t = 0; t < terms; ++t) {
          const double x = up[t * su];
          o0 = fma(x, v[t * sv + k], o0);
          o1 = fma(x, v[t * sv + k + 1], o1);
        }
      }
      *reinterpret_cast<double2*>(op) = make_double2(o0, o1);
    }
  } else {
    const int n = J2 * K2;
    for (int c = threadIdx.x; c < n; c += T) {
      const int j = c / K2, k = c - j * K2;
      double acc = 0.0;
      for (int t = 0; t < terms; ++t) acc = fma(u[t * su + j], v[t * sv + k], acc);
      out[c] = acc;
    }
  }
}

// P[(a*B+b), o, (a2*B2+b2)] = sum_i X[a,i,a2] * W[b,i,o,b2]; one block per
// output row r = (a*B + b)*O + o.
__global__ void __launch_bounds__(256) contract_mpo_mps_kernel(const double* __restrict__ X,
                                                               const double* __restrict__ W, double* __restrict__ P,
                                                               int64_t Bd, int64_t I, int64_t O, int64_t A2,
                                                               int64_t B2, bool vec) {
  const int64_t r = blockIdx.x;
  const int64_t o = r % O, ab = r / O;
  const int64_t b = ab % Bd, a = ab / Bd;
  outer_row<4>(X + a * I * A2, A2, W + (b * I * O + o) * B2, O * B2, (int)I, (int)A2, (int)B2,
               P + r * A2 * B2, vec);
}

// P[(b*C+c), i, o, (b2*C2+c2)] = sum_m A[b,i,m,b2] * B[c,m,o,c2]; one block
// per output row r = ((b*C + c)*I + i)*O + o.
__global__ void __launch_bounds__(256) contract_mpo_mpo_kernel(const double* __restrict__ A,
                                                               const double* __restrict__ Bm, double* __restrict__ P,
                                                               int64_t Cd, int64_t I, int64_t Mm, int64_t O,
                                                               int64_t B2, int64_t C2, bool vec) {
  const int64_t r = blockIdx.x;
  const int64_t o = r % O;
  int64_t t = r / O;
  const int64_t i = t % I;
  t /= I;
  const int64_t c = t % Cd, b = t / Cd;
  outer_row<4>(A + (b * I + i) * Mm * B2, B2, Bm + c * Mm * O * C2 + o * C2, O * C2, (int)Mm, (int)B2, (int)C2,
               P + r * B2 * C2, vec);
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

// Block shape of a row kernel: rows blocks; with the vector path a multiple
// of K2/2 threads (<= 256), else 32..256 threads.
int launch_rows(int64_t rows, int64_t J2, int64_t K2, bool& vec, unsigned& blocks, int& threads) {
  SGT_REQUIRE(rows <= 0x7fffffff && J2 * K2 <= 0x7fffffff, SGT_ERR_INVALID, "site contraction too large");
  blocks = (unsigned)rows;
  const int64_t hp = K2 / 2;
  vec = vec && K2 % 2 == 0 && hp <= 256;
  if (vec) {
    threads = (int)(hp * std::max<int64_t>(1, std::min<int64_t>(256 / hp, J2)));
  } else {
    threads = (int)std::min<int64_t>(256, std::max<int64_t>(32, cdiv(J2 * K2, 32) * 32));
  }
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
  bool vec = (reinterpret_cast<uintptr_t>(P) & 15) == 0;
  unsigned blocks;
  int threads;
  SGT_TRY(launch_rows(rows, a2, b2, vec, blocks, threads));
  contract_mpo_mps_kernel<<<blocks, threads, 0, st>>>(X, W, P, b, p, o, a2, b2, vec);
  SGT_LAUNCHED();
  return SGT_OK;
}

int site_contract_mpo_mpo(cudaStream_t st, const double* A, int64_t b, int64_t i, int64_t m,
                          int64_t b2, const double* B, int64_t c, int64_t o, int64_t c2, double* P) {
  int64_t rows = b * c * i * o, ncol = b2 * c2;
  if (rows == 0 || ncol == 0) return SGT_OK;
  bool vec = (reinterpret_cast<uintptr_t>(P) & 15) == 0;
  unsigned blocks;
  int threads;
  SGT_TRY(launch_rows(rows, b2, c2, vec, blocks, threads));
  contract_mpo_mpo_kernel<<<blocks, threads, 0, st>>>(A, B, P, c, i, m, o, b2, c2, vec);
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
