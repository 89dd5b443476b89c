// The accurate mixed-precision form of the metric operation
// (sgt_mpo_mps_round / sgt_svd_round with SGT_PREC_BF16X6).
//
// Same algebra as the Gram form of mixed.cu (no Householder QR on the R x R
// product unfoldings):
//   G_0 = [1],  G_{k+1} = sum_o P_k[:,o,:]^T G_k P_k[:,o,:]      (left Gram, structured)
//   right to left, F_N = [1]:
//     Y_k = P_k F_{k+1},  Z_k = Y_k^T G_k Y_k = V diag(s^2) V^T,
//     core_k = V[:, :chi]^T,  F_k = Y_k V[:, :chi],  core_0 = P_0 F_1,
// but carried at FP64-class accuracy:
//   * every O(R^3) product is the sliced bf16 GEMM of oz_gemm.cu (tcgen05,
//     ~2^-35 of the operands' scale) instead of split TF32 (~2^-22);
//   * the two small W contractions of the Gram step, the elementwise steps and
//     the intermediate matrices are FP32 pairs ("double-float", ~48 bits):
//     GB300's FP64 pipe is too slow for them;
//   * the bond eigensolve keeps the FP32 cluster Jacobi (svd.cu) as its first
//     approximation and then refines the eigenvectors and eigenvalues against
//     the pair-accurate Z by two steps of Ogita & Aishima's iteration
//     ("Iterative refinement for symmetric eigenvalue decomposition", Japan J.
//     Indust. Appl. Math. 35, 2018): with X the approximate eigenvectors,
//       R = I - X^T X,  S = X^T Z X,  l_i = S_ii / (1 - R_ii),
//       E_ij = (S_ij + l_j R_ij) / (l_j - l_i)  (E_ii = R_ii / 2),
//       X <- X + X E,
//     all four products on the sliced GEMM.  Each step squares the error, so
//     two steps take the FP32 Jacobi's ~1e-6 to the GEMMs' own accuracy.
//     Pairs whose correction would not be small (near-equal eigenvalues)
//     keep E_ij = R_ij / 2, as in the published method's cluster case.
// Product cores are never formed: the left recursion contracts X and W
// separately (steps A-D), and the right sweep forms Y_k = P_k F_{k+1} as
// (F W^T) then X, 2.2e9 instead of 1.7e10 FP64-equivalent flops per site at
// the benchmark's shapes.
#include <cooperative_groups.h>
#include <float.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "oz.cuh"

namespace cg = cooperative_groups;

namespace sgt {

void svd_round_plan_public(int n, const int64_t* shape, int64_t chi, std::vector<int64_t>& b,
                           std::vector<int64_t>& x, std::vector<int64_t>& cnt);
size_t sym_eig_rows_ws_bytes(int64_t n);
int sym_eig_rows_f32(cudaStream_t st, float* Z, int64_t n, float* Vt, float* lam, int* status, Arena& ar,
                     int method);
int eig_method_current();

namespace {

inline unsigned grid_for(int64_t n, int per = 256) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(n, per), 152 * 16));
}

// dst (rows x cols FP64, ldd) = pair src (lds)
__global__ void pair_to_f64_kernel(const float* __restrict__ h, const float* __restrict__ l, int64_t lds,
                                   double* __restrict__ dst, int64_t ldd, int64_t rows, int64_t cols) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows * cols;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / cols, c = i % cols;
    dst[r * ldd + c] = (double)h[r * lds + c] + (double)l[r * lds + c];
  }
}

// Pair transpose, batched: for every batch b, dst[b] (cols x rows, ldd) =
// src[b]^T (rows x cols, lds); batch strides sb / db.
__global__ void pair_transpose_kernel(float* __restrict__ dh, float* __restrict__ dl, int64_t ldd, int64_t db,
                                      const float* __restrict__ sh, const float* __restrict__ sl, int64_t lds,
                                      int64_t sb, int64_t rows, int64_t cols, const int* __restrict__ skip) {
  if (skip && *skip) return;  // uniform for the grid, before any barrier
  __shared__ float th[32][33], tl[32][33];
  const int64_t b = blockIdx.z;
  sh += b * sb;
  sl += b * sb;
  dh += b * db;
  dl += b * db;
  const int64_t tiles_c = (cols + 31) / 32, tiles_r = (rows + 31) / 32;
  for (int64_t t = blockIdx.x; t < tiles_r * tiles_c; t += gridDim.x) {
    const int64_t r0 = (t / tiles_c) * 32, c0 = (t % tiles_c) * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      const int64_t r = r0 + i, c = c0 + threadIdx.x;
      const bool in = r < rows && c < cols;
      th[i][threadIdx.x] = in ? sh[r * lds + c] : 0.f;
      tl[i][threadIdx.x] = in ? sl[r * lds + c] : 0.f;
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      const int64_t c = c0 + i, r = r0 + threadIdx.x;
      if (c < cols && r < rows) {
        dh[c * ldd + r] = th[threadIdx.x][i];
        dl[c * ldd + r] = tl[threadIdx.x][i];
      }
    }
    __syncthreads();
  }
}

// dst (contiguous in the order of the five output dimensions n[0..4]) =
// src at sum_d i_d * st[d]: a pair-valued index permutation.
struct Perm5 {
  int64_t n[5];
  int64_t st[5];
};

__global__ void pair_permute_kernel(float* __restrict__ dh, float* __restrict__ dl, const float* __restrict__ sh,
                                    const float* __restrict__ sl, const Perm5 pm) {
  const int64_t total = pm.n[0] * pm.n[1] * pm.n[2] * pm.n[3] * pm.n[4];
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = t, off = 0;
#pragma unroll
    for (int d = 4; d >= 0; --d) {
      const int64_t i = rem % pm.n[d];
      rem /= pm.n[d];
      off += i * pm.st[d];
    }
    dh[t] = sh[off];
    dl[t] = sl[off];
  }
}

// Steps B and C of the structured Gram step (see gram.cu) in pair arithmetic,
// for a tile of MD_TA values of a and TC values of c'.
//   B: U [a][b][o][e'][c'] = sum_{e,j} T1[a][b][e][j][c'] W[e][j][o][e']
//   C: T3[c'][e'][b'][a][i] = sum_{b,o} W[b][i][o][b'] U[a][b][o][e'][c']
// T1 / T3 are pair matrices (hi, lo); W is FP64 [b][i][o][b'].  T1 comes from
// step A as T1t[(j, c')][(a, b, e)] (c' outer, so that a tile of a values
// reads contiguous runs of (b, e)).  This generic form serves the edge sites;
// gram_mid_df_tiled below the middle ones.
constexpr int MD_TA = 4;

size_t mid_df_smem(int D, int d, int dout, int D2, int TC) {
  return sizeof(float) * 2 *
         ((size_t)D * d * dout * D2 + (size_t)MD_TA * D * D * d * TC + (size_t)MD_TA * D * dout * D2 * TC);
}

__global__ void __launch_bounds__(256) gram_mid_df_kernel(const float* __restrict__ T1h, const float* __restrict__ T1l,
                                                          const double* __restrict__ W, float* __restrict__ T3h,
                                                          float* __restrict__ T3l, int chi, int D, int d, int dout,
                                                          int D2, int chi2, int TC) {
  extern __shared__ float md_smem[];
  const int a0 = blockIdx.x * MD_TA, c0 = blockIdx.y * TC;
  const int bej = D * D * d;
  const int boe = D * dout * D2;
  const int wn = D * d * dout * D2;
  float2* sW = reinterpret_cast<float2*>(md_smem);  // [D][d][dout][D2]
  float2* sT = sW + wn;                              // [TA][bej][TC]
  float2* sU = sT + MD_TA * bej * TC;                // [TA][b][o][e'][TC]
  const int tid = threadIdx.x;
  for (int i = tid; i < wn; i += 256) {
    const double v = W[i];
    const float h = (float)v;
    sW[i] = make_float2(h, (float)(v - (double)h));
  }
  for (int i = tid; i < MD_TA * bej * TC; i += 256) {
    const int t = i % TC, r = (i / TC) % bej, at = i / (TC * bej);
    const int a = a0 + at, c = c0 + t;
    float2 v = make_float2(0.f, 0.f);
    if (a < chi && c < chi2) {
      // r = (b D + e) d + j
      const int b = r / (D * d), e = (r / d) % D, j = r % d;
      const int64_t g = ((int64_t)j * chi2 + c) * ((int64_t)chi * D * D) + ((int64_t)a * D + b) * D + e;
      v = make_float2(T1h[g], T1l[g]);
    }
    sT[i] = v;
  }
  __syncthreads();
  for (int i = tid; i < MD_TA * boe * TC; i += 256) {
    const int t = i % TC;
    int r = i / TC;
    const int e2 = r % D2;
    r /= D2;
    const int o = r % dout;
    r /= dout;
    const int b = r % D, at = r / D;
    const float2* tcol = sT + ((int64_t)at * bej + (int64_t)b * D * d) * TC + t;
    float h = 0.f, l = 0.f;
    for (int e = 0; e < D; ++e)
      for (int j = 0; j < d; ++j) {
        const float2 x = tcol[(e * d + j) * TC];
        const float2 w = sW[((e * d + j) * dout + o) * D2 + e2];
        df_fma(h, l, x.x, x.y, w.x, w.y);
      }
    df_norm(h, l);
    sU[i] = make_float2(h, l);
  }
  __syncthreads();
  const int inner = MD_TA * d;
  const int total = inner * D2 * D2 * TC;
  for (int k = tid; k < total; k += 256) {
    const int ai = k % inner;
    int r = k / inner;
    const int b2 = r % D2;
    r /= D2;
    const int e2 = r % D2;
    const int t = r / D2;
    const int at = ai / d, i = ai % d;
    const int a = a0 + at, c = c0 + t;
    if (a >= chi || c >= chi2) continue;
    float h = 0.f, l = 0.f;
    for (int b = 0; b < D; ++b)
      for (int o = 0; o < dout; ++o) {
        const float2 w = sW[((b * d + i) * dout + o) * D2 + b2];
        const float2 u = sU[((((int64_t)at * D + b) * dout + o) * D2 + e2) * TC + t];
        df_fma(h, l, w.x, w.y, u.x, u.y);
      }
    df_norm(h, l);
    const int64_t idx = (((int64_t)c * D2 + e2) * D2 + b2) * ((int64_t)chi * d) + (int64_t)a * d + i;
    T3h[idx] = h;
    T3l[idx] = l;
  }
}


// Middle sites (D2 = D, dout = d), compile-time sizes: one block per (8 values
// of a, one c').  Step B: a thread owns one (a, b) row and 16 of the 32
// (o, e') columns, step C one (a, e') row and 16 of the (i, b') columns, so
// every shared-memory value feeds 16 independent pair multiply-adds.  The W
// pairs sit in shared memory in both column orders; rows of T and U are
// padded by one pair against bank conflicts; the T3 tile is staged in shared
// memory and stored as runs of (a, i).
constexpr int MT_TA = 8;

template <int D, int d>
constexpr size_t mid_tiled_smem() {
  return sizeof(float2) * (2 * (size_t)(D * d) * (d * D) + 2 * (size_t)MT_TA * D * (D * d + 1));
}

template <int D, int d>
__global__ void __launch_bounds__(256, 2) gram_mid_df_tiled(const float* __restrict__ T1h, const float* __restrict__ T1l,
                                                           const double* __restrict__ W, float* __restrict__ T3h,
                                                           float* __restrict__ T3l, int chi, int chi2) {
  constexpr int K = D * d;       // (e, j) and (b, o) extents
  constexpr int NB = d * D;      // (o, e') and (i, b') extents
  constexpr int KP = K + 1;      // padded row of T / U
  constexpr int HALF = NB / 2;   // columns per thread
  extern __shared__ float2 mt_smem[];
  float2* sWB = mt_smem;               // [(e, j)][(o, e')]
  float2* sWC = sWB + K * NB;          // [(b, o)][(i, b')]
  float2* sT = sWC + K * NB;           // [a][b][(e, j)] (padded), later the T3 stage
  float2* sU = sT + MT_TA * D * KP;    // [a][e'][(b, o)] (padded)
  const int a0 = blockIdx.x * MT_TA, c = blockIdx.y;
  const int tid = threadIdx.x;
  const int64_t RR = (int64_t)chi * D * D;
  for (int idx = tid; idx < K * NB; idx += 256) {
    // idx = ((b d + i) d + o) D + b2 in W's own order
    const int b2 = idx % D, o = (idx / D) % d, i = (idx / (D * d)) % d, b = idx / (D * d * d);
    const double v = W[idx];
    const float h = (float)v;
    const float2 w = make_float2(h, (float)(v - (double)h));
    sWB[idx] = w;                                   // [(b, i)][(o, b2)]
    sWC[(b * d + o) * NB + i * D + b2] = w;         // [(b, o)][(i, b2)]
  }
  for (int idx = tid; idx < MT_TA * d * D * D; idx += 256) {
    const int be = idx % (D * D), j = (idx / (D * D)) % d, at = idx / (D * D * d);
    const int b = be / D, e = be % D, a = a0 + at;
    float2 v = make_float2(0.f, 0.f);
    if (a < chi) {
      const int64_t g = ((int64_t)j * chi2 + c) * RR + (int64_t)a * D * D + be;
      v = make_float2(T1h[g], T1l[g]);
    }
    sT[(at * D + b) * KP + e * d + j] = v;
  }
  __syncthreads();
  // ---- B: U[a][e'][(b, o)] = sum_(e,j) T[a][b][(e,j)] W[(e,j)][(o,e')] ----
  for (int task = tid; task < MT_TA * D * 2; task += 256) {
    const int half = task & 1, b = (task >> 1) % D, at = (task >> 1) / D;
    float h[HALF], l[HALF];
#pragma unroll
    for (int n = 0; n < HALF; ++n) h[n] = l[n] = 0.f;
    const float2* trow = sT + (at * D + b) * KP;
    const float2* wcol = sWB + half * HALF;
#pragma unroll 4
    for (int k = 0; k < K; ++k) {
      const float2 t = trow[k];
#pragma unroll
      for (int n = 0; n < HALF; ++n) {
        const float2 w = wcol[k * NB + n];
        df_fma(h[n], l[n], t.x, t.y, w.x, w.y);
      }
    }
#pragma unroll
    for (int n = 0; n < HALF; ++n) {
      const int col = half * HALF + n, o = col / D, e2 = col % D;
      df_norm(h[n], l[n]);
      sU[(at * D + e2) * KP + b * d + o] = make_float2(h[n], l[n]);
    }
  }
  __syncthreads();
  // ---- C: stage[e'][b'][a][i] = sum_(b,o) U[a][e'][(b,o)] W[(b,o)][(i,b')] ----
  float2* stage = sT;
  for (int task = tid; task < MT_TA * D * 2; task += 256) {
    const int half = task & 1, e2 = (task >> 1) % D, at = (task >> 1) / D;
    float h[HALF], l[HALF];
#pragma unroll
    for (int n = 0; n < HALF; ++n) h[n] = l[n] = 0.f;
    const float2* urow = sU + (at * D + e2) * KP;
    const float2* wcol = sWC + half * HALF;
#pragma unroll 4
    for (int k = 0; k < K; ++k) {
      const float2 u = urow[k];
#pragma unroll
      for (int n = 0; n < HALF; ++n) {
        const float2 w = wcol[k * NB + n];
        df_fma(h[n], l[n], u.x, u.y, w.x, w.y);
      }
    }
#pragma unroll
    for (int n = 0; n < HALF; ++n) {
      const int col = half * HALF + n, i = col / D, b2 = col % D;
      df_norm(h[n], l[n]);
      stage[((e2 * D + b2) * MT_TA + at) * d + i] = make_float2(h[n], l[n]);
    }
  }
  __syncthreads();
  // ---- store: T3[c][e'][b'][(a, i)], runs of MT_TA * d values ----
  constexpr int RUN = MT_TA * d;
  for (int idx = tid; idx < D * D * RUN; idx += 256) {
    const int r = idx % RUN, eb = idx / RUN;
    const int a = a0 + r / d;
    if (a >= chi) continue;
    const int64_t g = ((int64_t)c * D * D + eb) * ((int64_t)chi * d) + (int64_t)a0 * d + r;
    const float2 v = stage[idx];
    T3h[g] = v.x;
    T3l[g] = v.y;
  }
}

// max |h| over n values as the bit pattern of a non-negative float
__global__ void pair_absmax_kernel(const float* __restrict__ h, int64_t n, unsigned* __restrict__ out) {
  float m = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(h[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(out, __float_as_uint(m));
}

// (h, l) *= 2^-e (exact), e = binary exponent of the max; gexp_next = gexp_prev + e
__global__ void pair_scale_kernel(float* __restrict__ h, float* __restrict__ l, int64_t n,
                                  const unsigned* __restrict__ maxbits, const int* __restrict__ gexp_prev,
                                  int* __restrict__ gexp_next) {
  const float m = __uint_as_float(*maxbits);
  int e = 0;
  if (m > 0.f && isfinite(m)) frexpf(m, &e);
  if (blockIdx.x == 0 && threadIdx.x == 0) *gexp_next = *gexp_prev + e;
  if (e == 0) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    h[i] = ldexpf(h[i], -e);
    l[i] = ldexpf(l[i], -e);
  }
}

__global__ void pair_one_kernel(float* h, float* l) {
  h[0] = 1.f;
  l[0] = 0.f;
}

// Z <- (Z + Z^T) / 2 in pair arithmetic
__global__ void pair_symmetrize_kernel(float* __restrict__ h, float* __restrict__ l, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / n, c = i % n;
    if (c <= r) continue;
    float sh = h[r * n + c], sl = l[r * n + c];
    df_add(sh, sl, h[c * n + r], l[c * n + r]);
    sh *= 0.5f;
    sl *= 0.5f;
    h[r * n + c] = sh;
    l[r * n + c] = sl;
    h[c * n + r] = sh;
    l[c * n + r] = sl;
  }
}

// pair (a / b) for b != 0 (one Newton correction of the FP32 quotient)
__device__ __forceinline__ void df_div(float ah, float al, float bh, float bl, float& qh, float& ql) {
  const float q = ah / bh;
  // r = a - q b in pair arithmetic
  const float p = q * bh;
  const float pe = fmaf(q, bh, -p);
  float r = (ah - p) - pe;
  r += al - q * bl;
  const float q2 = r / bh;
  qh = q + q2;
  ql = q2 - (qh - q);
}

// Refinement step, part 1: l_i = S_ii / VV_ii (= S_ii / (1 - R_ii)), pairs.
__global__ void oa_lambda_kernel(const float* __restrict__ Sh, const float* __restrict__ Sl,
                                 const float* __restrict__ Vh, const float* __restrict__ Vl, int n,
                                 float* __restrict__ lh, float* __restrict__ ll) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int64_t d = (int64_t)i * n + i;
    float qh, ql;
    df_div(Sh[d], Sl[d], Vh[d], Vl[d], qh, ql);
    lh[i] = qh;
    ll[i] = ql;
  }
}

// Refinement step, part 2: Et[i][j] = E[j][i], with
//   E_jj = R_jj / 2,  E_ji = (S_ji + l_i R_ji) / (l_i - l_j)  where that is below 1/8
//   and |l_i - l_j| stands above the products' own error (2^-30 of the largest
//   |l|: eigenvalue differences below that are noise), else R_ji / 2;  R = I - VV.
__global__ void oa_correction_kernel(const float* __restrict__ Sh, const float* __restrict__ Sl,
                                     const float* __restrict__ Vh, const float* __restrict__ Vl,
                                     const float* __restrict__ lh, const float* __restrict__ ll, int n,
                                     const unsigned* __restrict__ lmax_bits, float* __restrict__ Eh,
                                     float* __restrict__ El) {
  const float floor_d = ldexpf(__uint_as_float(*lmax_bits), -30);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)n * n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / n), j = (int)(t % n);  // output Et[i][j] = E[j][i]
    const int64_t ji = (int64_t)j * n + i;
    // R_ji = delta_ji - VV_ji
    float rh = -Vh[ji], rl = -Vl[ji];
    if (i == j) df_add(rh, rl, 1.f, 0.f);
    float eh, el;
    if (i == j) {
      eh = 0.5f * rh;
      el = 0.5f * rl;
    } else {
      // numerator S_ji + l_i R_ji
      float nh = Sh[ji], nl = Sl[ji];
      df_fma(nh, nl, lh[i], ll[i], rh, rl);
      df_norm(nh, nl);
      // denominator l_i - l_j
      float dh = lh[i], dl = ll[i];
      df_add(dh, dl, -lh[j], -ll[j]);
      if (fabsf(dh) > 8.f * fabsf(nh) && fabsf(dh) > floor_d && isfinite(nh)) {
        df_div(nh, nl, dh, dl, eh, el);
      } else {
        eh = 0.5f * rh;
        el = 0.5f * rl;
      }
    }
    Eh[t] = eh;
    El[t] = el;
  }
}

// Rank sort of the eigenvalues (descending, ties by index): perm[rank] = i.
__global__ void rank_desc_kernel(const float* __restrict__ lh, int n, int* __restrict__ perm) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float v = lh[i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const float w = lh[j];
      rank += (w > v) || (w == v && j < i);
    }
    perm[rank] = i;
  }
}

// rows perm[0..keep) of the refined Vt: FP64 core (keep x n) and its pair copy
__global__ void gather_rows_kernel(const float* __restrict__ Vh, const float* __restrict__ Vl, int n,
                                   const int* __restrict__ perm, int keep, double* __restrict__ core,
                                   float* __restrict__ Kh, float* __restrict__ Kl) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)keep * n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / n), c = (int)(t % n);
    const int64_t s = (int64_t)perm[r] * n + c;
    const float h = Vh[s], l = Vl[s];
    core[t] = (double)h + (double)l;
    Kh[t] = h;
    Kl[t] = l;
  }
}

// spectra (descending) = sqrt(l 2^gexp), discarded = sum_{j >= keep} l_j / sum l_j
__global__ void oz_spectrum_kernel(const float* __restrict__ lh, const float* __restrict__ ll,
                                   const int* __restrict__ perm, int count, int keep, double* __restrict__ spec,
                                   double* __restrict__ disc, const int* __restrict__ gexp) {
  __shared__ double red[2][32];
  double tot = 0.0, drop = 0.0;
  const int ge = gexp ? *gexp : 0;
  for (int j = threadIdx.x; j < count; j += blockDim.x) {
    const int i = perm[j];
    const double v = fmax((double)lh[i] + (double)ll[i], 0.0);
    if (spec) spec[j] = sqrt(ldexp(v, ge));
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
    if (disc) *disc = (t > 0.0) ? d / t : 0.0;
  }
}

__global__ void oz_status_kernel(const int* __restrict__ st, int n, int* __restrict__ out, const int* __restrict__ err) {
  if (threadIdx.x != 0) return;
  int r = 0;
  for (int k = 1; k < n; ++k) {
    if (st[k] < 0) {
      r = -1;
      break;
    }
    r = max(r, st[k]);
  }
  if (err && *err) r = -2;
  *out = r;
}

// Identity operator cores eye[k] = I (d_k x d_k) for sites k0 .. k0 + count - 1;
// the physical dims travel by value in the launch (no host buffer that a
// captured graph would have to read again at replay).
constexpr int EYE_CHUNK = 256;
struct EyeDims {
  int d[EYE_CHUNK];
};
__global__ void identity_cores_f64_kernel(double* __restrict__ eye, const EyeDims dims, int k0, int count, int stride) {
  for (int j = blockIdx.x; j < count; j += gridDim.x) {
    const int d = dims.d[j];
    double* e = eye + (int64_t)(k0 + j) * stride;
    for (int i = threadIdx.x; i < d * d; i += blockDim.x) e[i] = (i / d == i % d) ? 1.0 : 0.0;
  }
}

// C = alpha (h + l) + beta C in FP64 (beta == 0 does not read C)
__global__ void axpby_pair_f64_kernel(const float* __restrict__ h, const float* __restrict__ l, int64_t lds,
                                      double alpha, double beta, double* __restrict__ C, int64_t ldc, int64_t rows,
                                      int64_t cols) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows * cols;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / cols, c = i % cols;
    const double v = alpha * ((double)h[r * lds + c] + (double)l[r * lds + c]);
    double* dst = C + r * ldc + c;
    *dst = (beta == 0.0) ? v : fma(beta, *dst, v);
  }
}


// ---------------------------------------------------------------------------
// The kept subspace without eigenvectors (callers that do not ask for
// spectra): trace-correcting purification (Niklasson, Phys. Rev. B 66, 155115,
// 2002, "TC2") drives X_0 = Z / |Z|_F to the orthogonal projector onto the
// eigenvectors of the `keep` largest eigenvalues of Z, squaring X, or taking
// 2X - X^2, whichever moves trace(X) toward `keep`; every product on the
// sliced GEMM, so the projector is FP64-class.  A basis of its range:
// Q = L^T X with L the rank-keep pivoted Cholesky factor of X's FP32 part (a
// projector's Cholesky factor has orthonormal columns, so Q starts
// orthonormal to FP32 rounding and its rows lie in X's range to full
// accuracy), then Newton-Schulz steps Q <- 1.5 Q - 0.5 (Q Q^T) Q in pair
// precision.  The rounded
// state depends on the kept subspace only (any orthonormal basis of it is a
// gauge choice), so this replaces the eigensolve when no spectrum is wanted.
// ---------------------------------------------------------------------------

// Deterministic grid reductions: every block writes its partial sums, and the
// last block to finish (an atomic ticket, reset for the next launch) adds them
// in block order.  RED_BLOCKS blocks of 256 threads.
constexpr int RED_BLOCKS = 2 * 152;

template <int NV>
__device__ __forceinline__ void block_sums(double (&v)[NV], double (*red)[32]) {
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v[q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double a = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a += red[q][w];
      v[q] = a;
    }
  }
}

// thread 0 of the last block returns true with the grid totals in v
template <int NV>
__device__ __forceinline__ bool grid_sums(double (&v)[NV], double* __restrict__ part, unsigned* __restrict__ ticket) {
  __shared__ double red[NV][32];
  __shared__ bool s_last;
  block_sums<NV>(v, red);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) part[(int64_t)blockIdx.x * NV + q] = v[q];
    __threadfence();
    s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return false;
  __threadfence();
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    double a = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b) a += __ldcg(part + (int64_t)b * NV + q);
    v[q] = a;
  }
  *ticket = 0u;
  return true;
}

// |h|_F (double) and trace(h + l) of a pair matrix (n x n)
__global__ void __launch_bounds__(256) pair_frob_trace_kernel(const float* __restrict__ h, const float* __restrict__ l,
                                                              int64_t n, double* __restrict__ part,
                                                              unsigned* __restrict__ ticket,
                                                              double* __restrict__ frob, double* __restrict__ trace) {
  double v[2] = {0.0, 0.0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x, t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t i = t0; i < n * n; i += stride) {
    const double a = (double)h[i];
    v[0] += a * a;
  }
  for (int64_t i = t0; i < n; i += stride) v[1] += (double)h[i * n + i] + (double)l[i * n + i];
  if (grid_sums<2>(v, part, ticket)) {
    *frob = sqrt(v[0]);
    *trace = v[1];
  }
}

// X = Z / (|Z|_F (1 + 2^-32)) + 2^-32 I for the dim x dim pair matrix Z: the
// spectrum of Z scaled into [0, 1] and lifted by 2^-32, so that the products'
// noise (eigenvalues of Z at ~-2^-40 |Z| where Z is rank-deficient) cannot
// leave [0, 1], where the purification's X^2 and 2X - X^2 steps keep every
// eigenvalue; a multiple of I changes no eigenvector.
constexpr float PURIFY_LIFT = 2.3283064365386963e-10f;  // 2^-32

__global__ void pair_scale_by_kernel(const float* __restrict__ zh, const float* __restrict__ zl, int64_t dim,
                                     const double* __restrict__ frob, float* __restrict__ xh, float* __restrict__ xl) {
  const double f = *frob;
  const float inv = (f > 0.0) ? (float)(1.0 / (f * (1.0 + (double)PURIFY_LIFT))) : 0.f;
  const int64_t n = dim * dim;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float p = zh[i] * inv;
    const float pe = fmaf(zh[i], inv, -p) + zl[i] * inv;
    float a = p, b = pe;
    df_norm(a, b);
    if (i % (dim + 1) == 0) df_add(a, b, PURIFY_LIFT, 0.f);
    xh[i] = a;
    xl[i] = b;
  }
}

// One purification step after X2 = X X (the sliced GEMM), fused: the TC2
// choice from trace(X) (dcur: X's diagonal, hi then lo, written by the
// previous step) and trace(X2); X <- X2 or 2X - X2 in place, a warp per row;
// the largest |X2 - X| into resid[t]; the new diagonal into dnext; and the
// slices of the new X for the next product, in oz_split_pair's layout (row
// exponent from the row's largest |hi|, zero padding to ldo).  X2 is
// symmetric to the level-4 rounding of the sliced product (~2^-50), so rows
// are updated independently and X is symmetrised once after the loop.  The
// last block to finish (atomic ticket, reset for the next launch) sets ctl[1]
// when resid[t] <= 2^-34: X was a projector to the products' accuracy, and
// every later step returns at once, as do the products (skip flag ctl[1]).
// X2 element i: the product itself (S = 1) or the sum of its S split-K
// partials in split order (the order of the product's own partial sum).
__device__ __forceinline__ void tc2_x2(const float* __restrict__ x2h, const float* __restrict__ x2l, int S,
                                      int64_t mn, int64_t i, float& h, float& l) {
  h = x2h[i];
  l = x2l[i];
  if (S > 1) {
    for (int z = 1; z < S; ++z) {
      const float v = x2h[(int64_t)z * mn + i];
      const float sum = h + v;
      const float bb = sum - h;
      const float e = (h - (sum - bb)) + (v - bb);
      h = sum;
      l += e;
      l += x2l[(int64_t)z * mn + i];
    }
    const float t = h + l;
    l = l - (t - h);
    h = t;
  }
}

__global__ void __launch_bounds__(256) tc2_step_kernel(float* __restrict__ xh, float* __restrict__ xl,
                                                       const float* __restrict__ x2h, const float* __restrict__ x2l,
                                                       int S, int n, int keep, const float* __restrict__ dcur,
                                                       float* __restrict__ dnext, int* __restrict__ ctl,
                                                       unsigned* __restrict__ resid, unsigned* __restrict__ ticket,
                                                       __nv_bfloat16* __restrict__ out, int64_t ldo, int64_t sstride,
                                                       int* __restrict__ ex) {
  __shared__ double red[2][8];
  __shared__ int s_ch;
  __shared__ bool s_last;
  if (ctl[1]) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  {
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const int64_t d = (int64_t)i * n + i;
      float h2, l2;
      tc2_x2(x2h, x2l, S, (int64_t)n * n, d, h2, l2);
      a += (double)dcur[i] + (double)dcur[n + i];
      b += (double)h2 + (double)l2;
    }
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) red[0][warp] = a, red[1][warp] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
      double ta = 0.0, tb = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) ta += red[0][w], tb += red[1][w];
      s_ch = fabs(tb - keep) < fabs(2.0 * ta - tb - keep) ? 1 : 0;
    }
    __syncthreads();
  }
  const int ch = s_ch;
  float worst = 0.f;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp; r < n; r += warps) {
    float mx = 0.f;
    for (int64_t c = lane; c < n; c += 32) {
      const int64_t i = r * n + c;
      float h2, l2;
      tc2_x2(x2h, x2l, S, (int64_t)n * n, i, h2, l2);
      float h = xh[i], l = xl[i];
      worst = fmaxf(worst, fabsf((h2 - h) + (l2 - l)));
      if (ch) {
        h = h2;
        l = l2;
      } else {  // 2X - X^2
        h *= 2.f;
        l *= 2.f;
        df_add(h, l, -h2, -l2);
      }
      xh[i] = h;
      xl[i] = l;
      mx = fmaxf(mx, fabsf(h));
      if (c == r) dnext[r] = h, dnext[n + r] = l;
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int e = 0;
    if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);
    if (lane == 0) ex[r] = e;
    // each lane re-reads only the elements it wrote above
    for (int64_t c = lane; c < n; c += 32) {
      const int64_t i = r * n + c;
      slice_store(ldexpf(xh[i], 6 - e), ldexpf(xl[i], 6 - e), out, sstride, r * ldo + c);
    }
    for (int64_t c = n + lane; c < ldo; c += 32) slice_zero(out, sstride, r * ldo + c);
  }
  for (int o = 16; o > 0; o >>= 1) worst = fmaxf(worst, __shfl_xor_sync(0xffffffffu, worst, o));
  if (lane == 0 && worst > 0.f) atomicMax(resid, __float_as_uint(worst));
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    if (__uint_as_float(atomicAdd(resid, 0u)) <= ldexpf(1.f, -34)) ctl[1] = 1;
    *ticket = 0u;
  }
}

// tc2_x2 for 4 consecutive elements (i a multiple of 4, mn too): the same sums
// in the same order, with 16-byte loads.
__device__ __forceinline__ void tc2_x2_4(const float* __restrict__ x2h, const float* __restrict__ x2l, int S,
                                        int64_t mn, int64_t i, float4& h, float4& l) {
  h = *reinterpret_cast<const float4*>(x2h + i);
  l = *reinterpret_cast<const float4*>(x2l + i);
  if (S > 1) {
    float hv[4] = {h.x, h.y, h.z, h.w}, lv[4] = {l.x, l.y, l.z, l.w};
    for (int z = 1; z < S; ++z) {
      const float4 v4 = *reinterpret_cast<const float4*>(x2h + (int64_t)z * mn + i);
      const float4 w4 = *reinterpret_cast<const float4*>(x2l + (int64_t)z * mn + i);
      const float vv[4] = {v4.x, v4.y, v4.z, v4.w}, ww[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float sum = hv[j] + vv[j];
        const float bb = sum - hv[j];
        const float e = (hv[j] - (sum - bb)) + (vv[j] - bb);
        hv[j] = sum;
        lv[j] += e;
        lv[j] += ww[j];
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float t = hv[j] + lv[j];
      lv[j] = lv[j] - (t - hv[j]);
      hv[j] = t;
    }
    h = make_float4(hv[0], hv[1], hv[2], hv[3]);
    l = make_float4(lv[0], lv[1], lv[2], lv[3]);
  }
}

// tc2_step_kernel with a block of TC2_VEC_THREADS per row and 4 consecutive
// elements per thread (n a multiple of 4, 16-byte aligned buffers): the same
// per-element arithmetic, the row maximum reduced over the block, the slices
// written 8 bytes at a time.  n blocks keep every SM busy where the
// warp-per-row form fills n / 8 blocks.
constexpr int TC2_VEC_THREADS = 128;
__global__ void __launch_bounds__(TC2_VEC_THREADS) tc2_step4_kernel(
    float* __restrict__ xh, float* __restrict__ xl, const float* __restrict__ x2h, const float* __restrict__ x2l,
    int S, int n, int keep, const float* __restrict__ dcur, float* __restrict__ dnext, int* __restrict__ ctl,
    unsigned* __restrict__ resid, unsigned* __restrict__ ticket, __nv_bfloat16* __restrict__ out, int64_t ldo,
    int64_t sstride, int* __restrict__ ex) {
  constexpr int W = TC2_VEC_THREADS / 32;
  __shared__ double red[2][W];
  __shared__ float s_mx[W];
  __shared__ int s_ch;
  __shared__ bool s_last;
  if (ctl[1]) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t mn = (int64_t)n * n;
  {
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < n; i += TC2_VEC_THREADS) {
      float h2, l2;
      tc2_x2(x2h, x2l, S, mn, (int64_t)i * n + i, h2, l2);
      a += (double)dcur[i] + (double)dcur[n + i];
      b += (double)h2 + (double)l2;
    }
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) red[0][warp] = a, red[1][warp] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
      double ta = 0.0, tb = 0.0;
      for (int w = 0; w < W; ++w) ta += red[0][w], tb += red[1][w];
      s_ch = fabs(tb - keep) < fabs(2.0 * ta - tb - keep) ? 1 : 0;
    }
    __syncthreads();
  }
  const int ch = s_ch;
  float worst = 0.f;
  for (int64_t r = blockIdx.x; r < n; r += gridDim.x) {
    float mx = 0.f;
    for (int64_t c = 4 * threadIdx.x; c < n; c += 4 * TC2_VEC_THREADS) {
      const int64_t i = r * n + c;
      float4 h24, l24;
      tc2_x2_4(x2h, x2l, S, mn, i, h24, l24);
      const float4 h4 = *reinterpret_cast<const float4*>(xh + i);
      const float4 l4 = *reinterpret_cast<const float4*>(xl + i);
      const float h2v[4] = {h24.x, h24.y, h24.z, h24.w}, l2v[4] = {l24.x, l24.y, l24.z, l24.w};
      float hv[4] = {h4.x, h4.y, h4.z, h4.w}, lv[4] = {l4.x, l4.y, l4.z, l4.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        worst = fmaxf(worst, fabsf((h2v[j] - hv[j]) + (l2v[j] - lv[j])));
        if (ch) {
          hv[j] = h2v[j];
          lv[j] = l2v[j];
        } else {  // 2X - X^2
          hv[j] *= 2.f;
          lv[j] *= 2.f;
          df_add(hv[j], lv[j], -h2v[j], -l2v[j]);
        }
        mx = fmaxf(mx, fabsf(hv[j]));
        if (c + j == r) dnext[r] = hv[j], dnext[n + r] = lv[j];
      }
      *reinterpret_cast<float4*>(xh + i) = make_float4(hv[0], hv[1], hv[2], hv[3]);
      *reinterpret_cast<float4*>(xl + i) = make_float4(lv[0], lv[1], lv[2], lv[3]);
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) s_mx[warp] = mx;
    __syncthreads();
    mx = s_mx[0];
    for (int w = 1; w < W; ++w) mx = fmaxf(mx, s_mx[w]);
    __syncthreads();  // s_mx is rewritten by the next row
    int e = 0;
    if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);
    if (threadIdx.x == 0) ex[r] = e;
    // each thread re-reads only the elements it wrote above
    for (int64_t c = 4 * threadIdx.x; c < n; c += 4 * TC2_VEC_THREADS) {
      const int64_t i = r * n + c;
      slice_store4(*reinterpret_cast<const float4*>(xh + i), *reinterpret_cast<const float4*>(xl + i), 6 - e, out,
                   sstride, r * ldo + c);
    }
    for (int64_t c = n + 4 * threadIdx.x; c < ldo; c += 4 * TC2_VEC_THREADS) {
      const __nv_bfloat16 z4[4] = {__float2bfloat16_rn(0.f), __float2bfloat16_rn(0.f), __float2bfloat16_rn(0.f),
                                   __float2bfloat16_rn(0.f)};
#pragma unroll
      for (int s = 0; s < OZ_SLICES; ++s)
        *reinterpret_cast<uint2*>(out + (int64_t)s * sstride + r * ldo + c) = *reinterpret_cast<const uint2*>(z4);
    }
  }
  for (int o = 16; o > 0; o >>= 1) worst = fmaxf(worst, __shfl_xor_sync(0xffffffffu, worst, o));
  if (lane == 0 && worst > 0.f) atomicMax(resid, __float_as_uint(worst));
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    if (__uint_as_float(atomicAdd(resid, 0u)) <= ldexpf(1.f, -34)) ctl[1] = 1;
    *ticket = 0u;
  }
}

// identity pair matrix (rows x cols, ld = cols)
__global__ void pair_eye_kernel(float* __restrict__ h, float* __restrict__ l, int64_t rows, int64_t cols) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows * cols;
       i += (int64_t)gridDim.x * blockDim.x) {
    h[i] = (i / cols == i % cols) ? 1.f : 0.f;
    l[i] = 0.f;
  }
}

// diagonal of a pair matrix (n x n) into d (hi then lo)
__global__ void pair_diag_kernel(const float* __restrict__ h, const float* __restrict__ l, int n,
                                 float* __restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    d[i] = h[(int64_t)i * n + i];
    d[n + i] = l[(int64_t)i * n + i];
  }
}

// Pivoted Cholesky of the purified projector's FP32 part, stopped at rank
// `keep` (one block, left-looking: O(c keep^2) work, the remaining diagonal
// in shared memory): A (c x c) ~ L L^T, Lt (keep x c) = L^T.  A is an
// orthogonal projector of rank keep up to rounding, so L^T L = I up to FP32
// rounding too: L is a well-conditioned basis without any sketch.  The
// sliced GEMM then forms L^T X, whose rows lie in the projector's range to
// its full accuracy.  used: c ints of scratch.
// 1 / sqrt(pivot), or 0 for a pivot below 1/(2c): a rank-keep orthogonal
// projector's greedy pivots stay >= 1/c (the Schur complement left after s
// steps has trace keep - s over c - s diagonal entries), so a smaller one
// means the projector had fewer than `keep` directions above the products'
// noise (a bond matrix of lower numerical rank); that column of L is then 0
// instead of noise amplified without bound, and its row of the basis stays 0.
__device__ __forceinline__ float pc_inv_pivot(float b, int c) {
  return b >= 0.5f / (float)c ? 1.f / sqrtf(b) : 0.f;
}

__global__ void __launch_bounds__(1024) pivoted_chol_kernel(const float* __restrict__ A, int c, int keep,
                                                            float* __restrict__ Lt, int* __restrict__ used) {
  extern __shared__ float pc_diag[];  // c floats
  __shared__ float s_val[32];
  __shared__ int s_idx[32];
  __shared__ int s_p;
  __shared__ float s_inv;
  for (int i = threadIdx.x; i < c; i += blockDim.x) {
    pc_diag[i] = A[(int64_t)i * c + i];
    used[i] = 0;
  }
  __syncthreads();
  for (int s = 0; s < keep; ++s) {
    float best = -1.f;
    int bi = 0;
    for (int i = threadIdx.x; i < c; i += blockDim.x) {
      const float v = used[i] ? -1.f : pc_diag[i];
      if (v > best) best = v, bi = i;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) best = ov, bi = oi;
    }
    if ((threadIdx.x & 31) == 0) s_val[threadIdx.x >> 5] = best, s_idx[threadIdx.x >> 5] = bi;
    __syncthreads();
    if (threadIdx.x == 0) {
      float b = -1.f;
      int p = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
        if (s_val[w] > b || (s_val[w] == b && s_idx[w] < p)) b = s_val[w], p = s_idx[w];
      s_p = p;
      used[p] = 1;
      s_inv = pc_inv_pivot(b, c);
    }
    __syncthreads();
    const int p = s_p;
    const float inv = s_inv;
    for (int i = threadIdx.x; i < c; i += blockDim.x) {
      float v = A[(int64_t)i * c + p];
      for (int t = 0; t < s; ++t) v -= Lt[(int64_t)t * c + i] * Lt[(int64_t)t * c + p];
      const float l = v * inv;
      Lt[(int64_t)s * c + i] = l;
      pc_diag[i] -= l * l;
    }
    __syncthreads();
  }
}

// The same factorisation across one cluster of PC_CS CTAs (the kernel above
// is the fallback where this one does not fit).  CTA b owns rows
// [b R, b R + R) of A and of L and keeps its slice of L in shared memory
// (column t of its rows at Ls[t Rp + r]), so a step reads no global memory but
// its part of A's pivot row (A is symmetric).  A step:
//   1. every warp reads the PC_CS published candidates (remaining diagonal,
//      row) over distributed shared memory and takes the largest, ties to the
//      lowest row: the pivot p, owned by CTA p / R;
//   2. the pivot's row of L (columns < s) is copied from the owner's shared
//      memory, where it was published with the candidate;
//   3. group g of the CTA's threads forms the partial dot products of its rows
//      with that row over the columns t = g (mod G), group 0 adds them in
//      order, writes column s of L and lowers the remaining diagonal;
//   4. the CTA publishes its next candidate and that row of L (double
//      buffered by step parity), and the cluster barrier releases them.
// Candidates are 64-bit keys (order-preserving value bits, then the
// complemented row), so the largest key is the largest value at the lowest
// row, as in the one-block kernel.
constexpr int PC_CS = 16;
constexpr int PC_THREADS = 512;

__device__ __forceinline__ unsigned long long pc_key(float v, int row) {
  unsigned u = __float_as_uint(v);
  u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
  return ((unsigned long long)u << 32) | (unsigned)(~(unsigned)row);
}
__device__ __forceinline__ float pc_key_value(unsigned long long k) {
  unsigned u = (unsigned)(k >> 32);
  u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
  return __uint_as_float(u);
}
__device__ __forceinline__ int pc_key_row(unsigned long long k) { return (int)(~(unsigned)(k & 0xffffffffu)); }
__device__ __forceinline__ unsigned long long pc_warp_max(unsigned long long k) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, k, o);
    k = x > k ? x : k;
  }
  return k;
}

__global__ void __launch_bounds__(PC_THREADS) pivoted_chol_cluster_kernel(const float* __restrict__ A, int c,
                                                                          int keep, int R, int Rp,
                                                                          float* __restrict__ Lt) {
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ float pcs[];
  const int G = PC_THREADS / Rp;
  float* Ls = pcs;                             // keep x Rp
  float* part = Ls + (int64_t)keep * Rp;       // G x Rp
  float* diag = part + (int64_t)G * Rp;        // Rp
  float* prow = diag + Rp;                     // keep
  float* crow = prow + keep;                   // 2 x keep: published candidate rows
  int* used = reinterpret_cast<int*>(crow + 2 * keep);  // Rp
  __shared__ unsigned long long s_key[2];
  __shared__ unsigned long long s_wkey[PC_THREADS / 32];
  const int tid = threadIdx.x, r = tid % Rp, g = tid / Rp, lane = tid & 31, warp = tid >> 5;
  const int row0 = (int)cluster.block_rank() * R;
  const int nrows = max(0, min(R, c - row0));
  const int nw = Rp / 32;
  for (int i = tid; i < Rp; i += PC_THREADS) {
    diag[i] = i < nrows ? A[(int64_t)(row0 + i) * c + row0 + i] : 0.f;
    used[i] = i < nrows ? 0 : 1;
  }
  __syncthreads();
  // this CTA's candidate for step 0
  if (g == 0) {
    unsigned long long k = pc_key(used[r] ? -INFINITY : diag[r], row0 + r);
    k = pc_warp_max(k);
    if (lane == 0) s_wkey[warp] = k;
  }
  __syncthreads();
  if (tid == 0) {
    unsigned long long k = 0ull;
    for (int w = 0; w < nw; ++w) k = s_wkey[w] > k ? s_wkey[w] : k;
    s_key[0] = k;
  }
  cluster.sync();
  for (int s = 0; s < keep; ++s) {
    const int cb = s & 1, nb = cb ^ 1;
    // 1. the pivot
    unsigned long long k = 0ull;
    if (lane < PC_CS) k = *cluster.map_shared_rank(&s_key[cb], lane);
    k = pc_warp_max(k);
    const int p = pc_key_row(k);
    const int owner = p / R;
    const float inv = pc_inv_pivot(pc_key_value(k), c);
    // 2. the pivot's row of L; this CTA's part of A's pivot row
    const float* orow = cluster.map_shared_rank(crow + cb * keep, owner);
    for (int t = tid; t < s; t += PC_THREADS) prow[t] = orow[t];
    const float a = (g == 0 && r < nrows) ? A[(int64_t)p * c + row0 + r] : 0.f;
    __syncthreads();
    // 3. partial dot products, then column s
    if (r < nrows) {
      float acc = 0.f;
      for (int t = g; t < s; t += G) acc = fmaf(Ls[(int64_t)t * Rp + r], prow[t], acc);
      part[g * Rp + r] = acc;
    }
    __syncthreads();
    if (g == 0) {
      if (r < nrows) {
        float sum = 0.f;
        for (int q = 0; q < G; ++q) sum += part[q * Rp + r];
        const float l = (a - sum) * inv;
        Ls[(int64_t)s * Rp + r] = l;
        Lt[(int64_t)s * c + row0 + r] = l;
        diag[r] -= l * l;
        if (row0 + r == p) used[r] = 1;
      }
      unsigned long long kk = pc_key(used[r] ? -INFINITY : diag[r], row0 + r);
      kk = pc_warp_max(kk);
      if (lane == 0) s_wkey[warp] = kk;
    }
    __syncthreads();
    // 4. publish the next candidate with its row of L (columns <= s)
    unsigned long long kn = 0ull;
    for (int w = 0; w < nw; ++w) kn = s_wkey[w] > kn ? s_wkey[w] : kn;
    const int lr = pc_key_row(kn) - row0;
    if (tid == 0) s_key[nb] = kn;
    if (lr >= 0 && lr < Rp)
      for (int t = tid; t <= s; t += PC_THREADS) crow[nb * keep + t] = Ls[(int64_t)t * Rp + lr];
    cluster.sync();
  }
}

// disc = 1 - sum_j (T[j] . Q[j]) / trace(Z)   (T = Q Z, rows of Q the kept basis)
__global__ void __launch_bounds__(256) kept_trace_kernel(const float* __restrict__ th, const float* __restrict__ tl,
                                                         const float* __restrict__ qh, const float* __restrict__ ql,
                                                         int64_t count, const double* __restrict__ trace_z,
                                                         double* __restrict__ part, unsigned* __restrict__ ticket,
                                                         double* __restrict__ disc) {
  double v[1] = {0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    v[0] += ((double)th[i] + (double)tl[i]) * ((double)qh[i] + (double)ql[i]);
  if (grid_sums<1>(v, part, ticket)) {
    const double tz = *trace_z;
    *disc = tz > 0.0 ? fmax(0.0, 1.0 - v[0] / tz) : 0.0;
  }
}

// status word of a projector bond: 0 when X converged to a projector
// (the loop stopped, or its last |X^2 - X| is at most 2^-30), -1 otherwise
__global__ void tc2_status_kernel(const int* __restrict__ ctl, const unsigned* __restrict__ resid,
                                  const unsigned* __restrict__ mcw_resid, int* __restrict__ st) {
  *st = (ctl[1] || __uint_as_float(*resid) <= ldexpf(1.f, -30) || __uint_as_float(*mcw_resid) <= ldexpf(1.f, -30))
            ? 0
            : -1;
}

// One McWeeny step X <- 3 X2 - 2 X3 (X2 = X X, X3 = X2 X, pair arithmetic),
// run only when the trace-correcting steps did not reach a projector (ctl[1]
// unset): that happens when the bond matrix has fewer directions above the
// products' noise than `keep`, and the noise eigenvalues form a cluster that
// no trace correction can split within the step budget.  McWeeny's map sends
// eigenvalues below 1/2 to 0 and above to 1 (quadratically), so X becomes the
// projector onto the significant directions (rank below keep); the basis then
// has zero rows for the rest (the pivot guard), which carry no weight.  The
// largest |change| goes to *resid.
__global__ void __launch_bounds__(256) mcweeny_step_kernel(float* __restrict__ xh, float* __restrict__ xl,
                                                          const float* __restrict__ x2h, const float* __restrict__ x2l,
                                                          const float* __restrict__ x3h, const float* __restrict__ x3l,
                                                          int64_t count, const int* __restrict__ ctl,
                                                          unsigned* __restrict__ resid) {
  if (ctl[1]) return;
  float worst = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const float p = 3.f * x2h[i];
    float h = p, l = fmaf(3.f, x2h[i], -p) + 3.f * x2l[i];
    df_add(h, l, -2.f * x3h[i], -2.f * x3l[i]);
    worst = fmaxf(worst, fabsf((h - xh[i]) + (l - xl[i])));
    xh[i] = h;
    xl[i] = l;
  }
  for (int o = 16; o > 0; o >>= 1) worst = fmaxf(worst, __shfl_xor_sync(0xffffffffu, worst, o));
  if ((threadIdx.x & 31) == 0 && worst > 0.f) atomicMax(resid, __float_as_uint(worst));
}

// Blocked right-looking form of the same factorisation, for projectors whose
// factor does not fit one cluster's shared memory (keep x c beyond ~48 K
// floats per CTA: bond problems of 2048 and more).  Aw is a working copy of A
// that holds the Schur complement left by the previous panels; a panel of
// PB_NB pivots is chosen by one block (pivot = largest remaining diagonal,
// ties to the lowest row, as the kernels above; each column is A's pivot row
// minus the panel's earlier columns, A symmetric), then every SM subtracts the
// panel's outer product from Aw.  O(c^2 keep) FP32 work, all of it in the
// trailing updates.
constexpr int PB_NB = 32;

__global__ void __launch_bounds__(1024) pchol_panel_kernel(const float* __restrict__ Aw, int c, int j0, int nb,
                                                           float* __restrict__ Lt, float* __restrict__ d,
                                                           int* __restrict__ used) {
  __shared__ float s_val[32];
  __shared__ int s_idx[32];
  __shared__ int s_p[PB_NB];
  __shared__ float s_inv;
  for (int s = j0; s < j0 + nb; ++s) {
    float best = -1.f;
    int bi = 0;
    for (int i = threadIdx.x; i < c; i += blockDim.x) {
      const float v = used[i] ? -1.f : d[i];
      if (v > best) best = v, bi = i;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) best = ov, bi = oi;
    }
    if ((threadIdx.x & 31) == 0) s_val[threadIdx.x >> 5] = best, s_idx[threadIdx.x >> 5] = bi;
    __syncthreads();
    if (threadIdx.x == 0) {
      float b = -1.f;
      int p = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
        if (s_val[w] > b || (s_val[w] == b && s_idx[w] < p)) b = s_val[w], p = s_idx[w];
      s_p[s - j0] = p;
      used[p] = 1;
      s_inv = pc_inv_pivot(b, c);
    }
    __syncthreads();
    const int p = s_p[s - j0];
    const float inv = s_inv;
    for (int i = threadIdx.x; i < c; i += blockDim.x) {
      float v = Aw[(int64_t)p * c + i];
      for (int t = j0; t < s; ++t) v -= Lt[(int64_t)t * c + i] * Lt[(int64_t)t * c + p];
      const float l = v * inv;
      Lt[(int64_t)s * c + i] = l;
      d[i] -= l * l;
    }
    __syncthreads();
  }
}

// Aw (c x c) -= P^T P with P = Lt rows [j0, j0 + nb), nb <= PB_NB: 64 x 64
// tiles, 4 x 4 outputs per thread, P's two column ranges staged in shared
// memory.
__global__ void __launch_bounds__(256) pchol_update_kernel(float* __restrict__ Aw, int c,
                                                           const float* __restrict__ P, int nb) {
  __shared__ float Ps[PB_NB][64];
  __shared__ float Qs[PB_NB][64];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  const int i0 = blockIdx.y * 64, j0 = blockIdx.x * 64;
  for (int idx = tid; idx < PB_NB * 64; idx += 256) {
    const int t = idx / 64, q = idx % 64;
    Ps[t][q] = (t < nb && i0 + q < c) ? P[(int64_t)t * c + i0 + q] : 0.f;
    Qs[t][q] = (t < nb && j0 + q < c) ? P[(int64_t)t * c + j0 + q] : 0.f;
  }
  __syncthreads();
  float acc[4][4] = {};
#pragma unroll 8
  for (int t = 0; t < PB_NB; ++t) {
    float a[4], b[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) a[u] = Ps[t][ty + 16 * u], b[u] = Qs[t][tx + 16 * u];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int i = i0 + ty + 16 * u;
    if (i >= c) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int j = j0 + tx + 16 * v;
      if (j < c) Aw[(int64_t)i * c + j] -= acc[u][v];
    }
  }
}

__global__ void pchol_init_kernel(const float* __restrict__ A, int c, float* __restrict__ d, int* __restrict__ used) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < c; i += gridDim.x * blockDim.x) {
    d[i] = A[(int64_t)i * c + i];
    used[i] = 0;
  }
}

// Rank-keep pivoted Cholesky factor Lt (keep x c) of the FP32 projector A
// (c x c): the cluster kernel where it fits, else (work: c*c + c floats of
// scratch) the blocked form, else the one-block kernel.
static int g_pchol_blocked = 0;  // SGT_TUNE_PCHOL_BLOCKED
static int g_purify_cleanup = 0;  // SGT_TUNE_PURIFY_CLEANUP
static int g_tc2_vec = 1;         // SGT_TUNE_PURIFY_VECTOR_STEP

int pivoted_chol(cudaStream_t st, const float* A, int64_t c, int64_t keep, float* Lt, int* used, float* work) {
  const int64_t R = cdiv(c, (int64_t)PC_CS);
  int64_t Rp = 32;
  while (Rp < R) Rp *= 2;
  const size_t smem =
      sizeof(float) * ((size_t)keep * (size_t)(Rp + 3) + (size_t)Rp * (size_t)(PC_THREADS / Rp + 2));
  const bool prefer_blocked = work && c >= 64 && __atomic_load_n(&g_pchol_blocked, __ATOMIC_RELAXED);
  if (!prefer_blocked && c >= 2 * PC_CS && Rp <= PC_THREADS && smem <= 200 * 1024) {
    bool ok = func_attr_at_least((const void*)pivoted_chol_cluster_kernel,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
              func_attr_at_least((const void*)pivoted_chol_cluster_kernel,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(PC_CS, 1, 1);
    cfg.blockDim = dim3(PC_THREADS, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = PC_CS;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int clusters = 0;
    ok = ok && cudaOccupancyMaxActiveClusters(&clusters, pivoted_chol_cluster_kernel, &cfg) == cudaSuccess &&
         clusters >= 1;
    if (ok) {
      SGT_CUDA(cudaLaunchKernelEx(&cfg, pivoted_chol_cluster_kernel, A, (int)c, (int)keep, (int)R, (int)Rp, Lt));
      note_launch();
      return SGT_OK;
    }
    cudaGetLastError();  // not here: the blocked or one-block kernel
  }
  if (work && c >= 64) {
    float* Aw = work;
    float* d = work + c * c;
    SGT_CUDA(cudaMemcpyAsync(Aw, A, sizeof(float) * c * c, cudaMemcpyDeviceToDevice, st));
    pchol_init_kernel<<<(unsigned)cdiv(c, 256), 256, 0, st>>>(A, (int)c, d, used);
    SGT_LAUNCHED();
    const dim3 ug((unsigned)cdiv(c, 64), (unsigned)cdiv(c, 64));
    for (int64_t j0 = 0; j0 < keep; j0 += PB_NB) {
      const int nb = (int)std::min<int64_t>(PB_NB, keep - j0);
      pchol_panel_kernel<<<1, 1024, 0, st>>>(Aw, (int)c, (int)j0, nb, Lt, d, used);
      SGT_LAUNCHED();
      if (j0 + nb < keep) {
        pchol_update_kernel<<<ug, 256, 0, st>>>(Aw, (int)c, Lt + j0 * c, nb);
        SGT_LAUNCHED();
      }
    }
    return SGT_OK;
  }
  SGT_REQUIRE(c * sizeof(float) <= 48 * 1024, SGT_ERR_INVALID, "mpo_mps_round: bond problem too large");
  pivoted_chol_kernel<<<1, 1024, c * sizeof(float), st>>>(A, (int)c, (int)keep, Lt, used);
  SGT_LAUNCHED();
  return SGT_OK;
}

struct Site4 {
  int64_t b, i, o, b2;
};

// Largest number of purification steps (the loop stops itself once X is a
// projector; about 2 log2(|Z|_F / gap at the cut) + 6 are needed, ~45 at the
// benchmark's bonds) and Newton-Schulz steps.
constexpr int TC2_ITERS = 90;
constexpr int MCW_ITERS = 6;  // McWeeny clean-up steps, skipped when the purification converged
constexpr int NS_ITERS = 2;
constexpr int NS_EXTRA = 4;   // Newton-Schulz steps after an unconverged purification

// Pair matrix buffers (hi, lo) carved from the arena.
struct Pair {
  float* h = nullptr;
  float* l = nullptr;
};
Pair take_pair(Arena& ar, int64_t count) {
  Pair p;
  p.h = ar.take<float>((size_t)count);
  p.l = ar.take<float>((size_t)count);
  return p;
}

// Slices + per-row exponents of a rows x cols operand.
struct Sliced {
  __nv_bfloat16* s = nullptr;
  int* e = nullptr;
  int64_t rows = 0, cols = 0;
  OzMat mat() const { return oz_mat(s, rows, cols, e); }
};
Sliced take_sliced(Arena& ar, int64_t rows, int64_t cols) {
  Sliced q;
  q.s = ar.take<__nv_bfloat16>(oz_slice_elems(rows, cols));
  q.e = ar.take<int>((size_t)rows);
  q.rows = rows;
  q.cols = cols;
  return q;
}

// `skip` (device int, may be null): nonzero at launch time makes the call a no-op
int split_pair(cudaStream_t st, const Pair& p, int64_t ld, Sliced& q, int64_t rows, int64_t cols,
               const int* skip = nullptr) {
  q.rows = rows;
  q.cols = cols;
  return oz_split_pair(st, p.h, p.l, ld, rows, cols, q.s, q.e, 1, skip);
}

int pair_transpose(cudaStream_t st, Pair dst, int64_t ldd, int64_t db, Pair src, int64_t lds, int64_t sb, int64_t rows,
                   int64_t cols, int64_t batch, const int* skip = nullptr) {
  if (rows <= 0 || cols <= 0 || batch <= 0) return SGT_OK;
  const int64_t tiles = cdiv(rows, 32) * cdiv(cols, 32);
  dim3 g((unsigned)std::min<int64_t>(tiles, 1024), 1, (unsigned)batch);
  pair_transpose_kernel<<<g, dim3(32, 8), 0, st>>>(dst.h, dst.l, ldd, db, src.h, src.l, lds, sb, rows, cols, skip);
  SGT_LAUNCHED();
  return SGT_OK;
}

int mid_tc(int64_t D, int64_t d, int64_t dout, int64_t D2) {
  int TC = 8;
  while (TC > 1 && mid_df_smem((int)D, (int)d, (int)dout, (int)D2, TC) > 200 * 1024) TC /= 2;
  return mid_df_smem((int)D, (int)d, (int)dout, (int)D2, TC) <= 200 * 1024 ? TC : 0;
}

}  // namespace

bool oz_round_supported(int n, const int64_t* ws4) {
  for (int k = 0; k + 1 < n; ++k)
    if (mid_tc(ws4[4 * k], ws4[4 * k + 1], ws4[4 * k + 2], ws4[4 * k + 3]) == 0) return false;
  return true;
}

// ---------------------------------------------------------------------------
// Phase timing of the BF16X6 round (sgt_phase_profile): an event at every
// phase boundary on the round's stream, summed per phase when read.  Process-
// wide and meant for one round at a time on one stream (benchmarks).
enum RoundPhase { PH_LEFT = 0, PH_Y, PH_BOND, PH_PURIFY, PH_BASIS, PH_DISC, PH_CARRY, PH_EIG, PH_COUNT };
struct PhaseMark {
  int phase;  // the phase that starts here (-1: end of a round)
  cudaEvent_t ev;
};
static ProfLog<PhaseMark> g_phase;

static int phase_mark(cudaStream_t st, int phase) {
  if (!g_phase.active()) return SGT_OK;
  cudaEvent_t e;
  SGT_CUDA(cudaEventCreate(&e));
  const cudaError_t r = cudaEventRecord(e, st);
  if (r != cudaSuccess) {
    cudaEventDestroy(e);
    set_error("phase_profile: %s", cudaGetErrorString(r));
    return SGT_ERR_CUDA;
  }
  g_phase.add({phase, e});
  return SGT_OK;
}

int oz_round_impl(cudaStream_t st, int n, const double* const* W, const int64_t* ws4, const double* const* X,
                  const int64_t* xs, int64_t chi, double* const* out, double* spectra, double* discarded, int* status,
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
  SGT_REQUIRE(oz_round_supported(n, ws4), SGT_ERR_INVALID,
              "mpo_mps_round: operator bonds too large for the pair-precision Gram step");
  for (int k = 0; k < n; ++k) shp[3 * k] = R[k], shp[3 * k + 1] = Pd[k], shp[3 * k + 2] = R[k + 1];
  std::vector<int64_t> bb, x, cnt;
  svd_round_plan_public(n, shp.data(), chi, bb, x, cnt);

  // ---- workspace ----
  int64_t rmax = 1, cmax = 1, t1max = 1, t3max = 1;
  size_t gsmax = 1, xtmax = 1, x2max = 1, t3smax = 1;
  int64_t gcrows = 1, xtrows = 1, x2rows = 1, t3rows = 1;
  for (int k = 0; k < n; ++k) {
    rmax = std::max(rmax, std::max(R[k], R[k + 1]));
    cmax = std::max(cmax, Pd[k] * x[k + 1]);
    if (k + 1 < n) {
      const int64_t chi_k = xs[3 * k], d = xs[3 * k + 1], chi2 = xs[3 * k + 2];
      t1max = std::max<int64_t>(t1max, chi_k * w[k].b * w[k].b * d * chi2);
      t3max = std::max<int64_t>(t3max, chi2 * w[k].b2 * w[k].b2 * chi_k * d);
      gsmax = std::max(gsmax, oz_slice_elems(R[k] * R[k] / chi_k, chi_k));
      gcrows = std::max(gcrows, R[k] * R[k] / chi_k);
      xtmax = std::max(xtmax, oz_slice_elems(d * chi2, chi_k));
      xtrows = std::max(xtrows, d * chi2);
      x2max = std::max(x2max, oz_slice_elems(chi2, chi_k * d));
      x2rows = std::max(x2rows, chi2);
      t3smax = std::max(t3smax, oz_slice_elems(chi2 * w[k].b2 * w[k].b2, chi_k * d));
      t3rows = std::max(t3rows, chi2 * w[k].b2 * w[k].b2);
    }
  }
  auto take_raw = [&](size_t elems, int64_t rows) {
    Sliced q;
    q.s = ar.take<__nv_bfloat16>(elems);
    q.e = ar.take<int>((size_t)rows);
    return q;
  };
  // G_k slices with rows of R_k (kept for the right sweep)
  std::vector<Sliced> GsR(n);
  for (int k = 0; k < n; ++k) GsR[k] = take_sliced(ar, R[k], R[k]);
  Sliced Gchi = take_raw(gsmax, gcrows);  // G_k with rows of chi_k (next Gram step), reused
  Pair G = take_pair(ar, rmax * rmax);
  Pair T1 = take_pair(ar, t1max);
  Pair T3 = take_pair(ar, t3max);
  Sliced T3s = take_raw(t3smax, t3rows);
  Sliced Xt = take_raw(xtmax, xtrows), X2 = take_raw(x2max, x2rows);
  // structured Y: F as rows of B', W and X as slice sets, T = F W^T and its permutation
  size_t fsmax = 1, tqsmax = 1, wslmax = 1, xslmax = 1;
  int64_t fsrows = 1, tpmax = 1, tqrows = 1, wslrows = 1, xslrows = 1;
  for (int k = 0; k < n; ++k) {
    const int64_t A = xs[3 * k], I = xs[3 * k + 1], A2 = xs[3 * k + 2], xc = x[k + 1];
    const int64_t Bk = w[k].b, O = w[k].o, B2 = w[k].b2, bio = Bk * I * O;
    fsmax = std::max(fsmax, oz_slice_elems(xc * A2, B2));
    fsrows = std::max(fsrows, xc * A2);
    tpmax = std::max(tpmax, xc * A2 * bio);
    tqsmax = std::max(tqsmax, oz_slice_elems(Bk * O * xc, I * A2));
    tqrows = std::max(tqrows, Bk * O * xc);
    wslmax = std::max(wslmax, oz_slice_elems(bio, B2));
    wslrows = std::max(wslrows, bio);
    xslmax = std::max(xslmax, oz_slice_elems(A, I * A2));
    xslrows = std::max(xslrows, A);
  }
  Sliced Fs = take_raw(fsmax, fsrows), Tqs = take_raw(tqsmax, tqrows);
  Sliced Wsl = take_raw(wslmax, wslrows), Xsl = take_raw(xslmax, xslrows);
  Pair Tp = take_pair(ar, tpmax), Tq = take_pair(ar, tpmax);
  Pair Ft = take_pair(ar, chi * rmax + 1);
  Pair Yt = take_pair(ar, cmax * rmax), Ytp = take_pair(ar, cmax * rmax), GY = take_pair(ar, cmax * rmax);
  Sliced Yts = take_sliced(ar, cmax, rmax), Ytps = take_sliced(ar, cmax, rmax), GYs = take_sliced(ar, cmax, rmax);
  Sliced Ys = take_sliced(ar, rmax, cmax);
  Pair Z = take_pair(ar, cmax * cmax);
  float* Z32 = ar.take<float>((size_t)(cmax * cmax + cmax));  // + the blocked pivoted Cholesky's diagonal
  float* Vt32 = ar.take<float>((size_t)(cmax * cmax));
  float* lam32 = ar.take<float>((size_t)cmax);
  Pair Vt = take_pair(ar, cmax * cmax), Xv = take_pair(ar, cmax * cmax), VV = take_pair(ar, cmax * cmax);
  Pair T = take_pair(ar, cmax * cmax), S = take_pair(ar, cmax * cmax), Et = take_pair(ar, cmax * cmax);
  Pair lamp = take_pair(ar, cmax);
  Sliced Vts = take_sliced(ar, cmax, cmax), Xvs = take_sliced(ar, cmax, cmax), Zs = take_sliced(ar, cmax, cmax);
  Sliced Ts = take_sliced(ar, cmax, cmax), Ets = take_sliced(ar, cmax, cmax);
  Pair Vk = take_pair(ar, chi * cmax);
  Sliced Vks = take_sliced(ar, chi, cmax);
  int* perm = ar.take<int>((size_t)cmax);
  double* dscal = ar.take<double>(2);
  int* ichoice = ar.take<int>(2);  // purification: [0] the step's choice, [1] converged
  double* rpart = ar.take<double>(2 * RED_BLOCKS);
  unsigned* ticket = ar.take<unsigned>(1);
  unsigned* tc2_resid = ar.take<unsigned>(TC2_ITERS);  // purification: largest |X^2 - X| of each step
  unsigned* mcw_resid = ar.take<unsigned>(MCW_ITERS);  // McWeeny clean-up: largest change of each step
  float* tc2_diag = ar.take<float>((size_t)(4 * cmax));  // purification: X's diagonal, two buffers
  // split-K partials: the largest requirement of the products below
  size_t part_bytes = 0;
  for (int k = 0; k < n; ++k) {
    const int64_t r = R[k], r2 = R[k + 1], c = Pd[k] * x[k + 1];
    {
      const int64_t A = xs[3 * k], I = xs[3 * k + 1], A2 = xs[3 * k + 2], xc = x[k + 1];
      const int64_t Bk = w[k].b, O = w[k].o, B2 = w[k].b2;
      part_bytes = std::max(part_bytes, oz_gemm_ws_bytes(xc * A2, Bk * I * O, B2));
      part_bytes = std::max(part_bytes, oz_gemm_ws_bytes(A, Bk * O * xc, I * A2));
    }
    part_bytes = std::max(part_bytes, oz_gemm_ws_bytes(c, r, r));
    part_bytes = std::max(part_bytes, oz_gemm_ws_bytes(c, c, r));
    part_bytes = std::max(part_bytes, oz_gemm_ws_bytes(c, c, c));
    part_bytes = std::max(part_bytes, oz_gemm_ws_bytes(x[k], r, c));
    if (k + 1 < n) {
      const int64_t chi_k = xs[3 * k], d = xs[3 * k + 1], chi2 = xs[3 * k + 2];
      part_bytes = std::max(part_bytes, oz_gemm_ws_bytes(chi_k * w[k].b * w[k].b, d * chi2, chi_k));
      part_bytes = std::max(part_bytes, oz_gemm_ws_bytes(chi2 * w[k].b2 * w[k].b2, chi2, chi_k * d));
    }
  }
  float* part = ar.take<float>(part_bytes / sizeof(float) + 1);
  const int64_t part_floats = (int64_t)(part_bytes / sizeof(float));
  int* stat = ar.take<int>((size_t)n + 1);
  int* err = ar.take<int>(1);
  int* gexp = ar.take<int>((size_t)n + 1);
  unsigned* gmax = ar.take<unsigned>(1);
  const size_t jbytes = sym_eig_rows_ws_bytes(cmax);
  char* jscratch = ar.take<char>(jbytes);
  if (ar.measure) return SGT_OK;
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "mpo_mps_round: workspace too small");
  SGT_CUDA(cudaMemsetAsync(stat, 0, sizeof(int) * (n + 1), st));
  SGT_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned), st));
  SGT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  SGT_CUDA(cudaMemsetAsync(gexp, 0, sizeof(int) * (n + 1), st));

  auto gemm = [&](int64_t M, int64_t N, int64_t K, float alpha, const OzMat& A, const OzMat& B, float beta,
                  Pair C, int64_t ldc) -> int {
    return oz_gemm(st, M, N, K, alpha, A, B, beta, C.h, C.l, ldc, part, part_floats, err);
  };

  SGT_TRY(phase_mark(st, PH_LEFT));
  // ---- left Gram recursion (structured: X and W contractions, no product) ----
  pair_one_kernel<<<1, 1, 0, st>>>(G.h, G.l);
  SGT_LAUNCHED();
  SGT_TRY(split_pair(st, G, 1, GsR[0], 1, 1));
  for (int k = 0; k + 1 < n; ++k) {
    const int64_t chi_k = xs[3 * k], d = xs[3 * k + 1], chi2 = xs[3 * k + 2];
    const int64_t D = w[k].b, dout = w[k].o, D2 = w[k].b2;
    // G_k as rows of chi_k (its columns are in (b, a) order, so a row of chi_k is one b)
    if (k == 0) {
      SGT_TRY(split_pair(st, G, 1, Gchi, 1, 1));
    } else {
      SGT_TRY(split_pair(st, G, chi_k, Gchi, R[k] * R[k] / chi_k, chi_k));
    }
    // Xt[(j,c')][c] = X[c][j][c'],  X2[a'][(a,i)] = X[a][i][a']
    SGT_TRY(oz_split_f64(st, X[k], 1, d * chi2, d * chi2, chi_k, Xt.s, Xt.e, 1));
    Xt.rows = d * chi2;
    Xt.cols = chi_k;
    SGT_TRY(oz_split_f64(st, X[k], 1, chi2, chi2, chi_k * d, X2.s, X2.e, 1));
    X2.rows = chi2;
    X2.cols = chi_k * d;
    // A: T1t ((d chi2) x (chi D D)) = Xt G_k^T, G_k taken as rows of chi
    SGT_TRY(gemm(d * chi2, chi_k * D * D, chi_k, 1.f, Xt.mat(), Gchi.mat(), 0.f, T1, chi_k * D * D));
    // B + C in pair arithmetic
    bool tiled_done = false;
    if (D2 == D && dout == d && chi2 <= 65535) {
      auto run = [&](auto kern, size_t smem) -> int {
        SGT_CUDA(func_attr_at_least((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        dim3 gt((unsigned)cdiv(chi_k, MT_TA), (unsigned)chi2);
        kern<<<gt, 256, smem, st>>>(T1.h, T1.l, W[k], T3.h, T3.l, (int)chi_k, (int)chi2);
        SGT_LAUNCHED();
        tiled_done = true;
        return SGT_OK;
      };
      if (D == 16 && d == 2) SGT_TRY(run(gram_mid_df_tiled<16, 2>, mid_tiled_smem<16, 2>()));
      else if (D == 16 && d == 4) SGT_TRY(run(gram_mid_df_tiled<16, 4>, mid_tiled_smem<16, 4>()));
      else if (D == 8 && d == 2) SGT_TRY(run(gram_mid_df_tiled<8, 2>, mid_tiled_smem<8, 2>()));
      else if (D == 8 && d == 3) SGT_TRY(run(gram_mid_df_tiled<8, 3>, mid_tiled_smem<8, 3>()));
      else if (D == 8 && d == 4) SGT_TRY(run(gram_mid_df_tiled<8, 4>, mid_tiled_smem<8, 4>()));
      else if (D == 16 && d == 3) SGT_TRY(run(gram_mid_df_tiled<16, 3>, mid_tiled_smem<16, 3>()));
      else if (D == 4 && d == 2) SGT_TRY(run(gram_mid_df_tiled<4, 2>, mid_tiled_smem<4, 2>()));
      else if (D == 4 && d == 3) SGT_TRY(run(gram_mid_df_tiled<4, 3>, mid_tiled_smem<4, 3>()));
      else if (D == 4 && d == 4) SGT_TRY(run(gram_mid_df_tiled<4, 4>, mid_tiled_smem<4, 4>()));
    }
    if (!tiled_done) {
      const int TC = mid_tc(D, d, dout, D2);
      const size_t smem = mid_df_smem((int)D, (int)d, (int)dout, (int)D2, TC);
      SGT_CUDA(func_attr_at_least((const void*)gram_mid_df_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
      dim3 g((unsigned)cdiv(chi_k, MD_TA), (unsigned)cdiv(chi2, TC));
      gram_mid_df_kernel<<<g, 256, smem, st>>>(T1.h, T1.l, W[k], T3.h, T3.l, (int)chi_k, (int)D, (int)d, (int)dout,
                                               (int)D2, (int)chi2, TC);
      SGT_LAUNCHED();
    }
    // D: G_{k+1} ((chi2 D2 D2) x chi2) = T3 X2^T
    SGT_TRY(split_pair(st, T3, chi_k * d, T3s, chi2 * D2 * D2, chi_k * d));
    SGT_TRY(gemm(chi2 * D2 * D2, chi2, chi_k * d, 1.f, T3s.mat(), X2.mat(), 0.f, G, chi2));
    // exact power-of-two scaling against range loss over long chains
    const int64_t gn = R[k + 1] * R[k + 1];
    SGT_CUDA(cudaMemsetAsync(gmax, 0, sizeof(unsigned), st));
    pair_absmax_kernel<<<grid_for(gn), 256, 0, st>>>(G.h, gn, gmax);
    SGT_LAUNCHED();
    pair_scale_kernel<<<grid_for(gn), 256, 0, st>>>(G.h, G.l, gn, gmax, gexp + k, gexp + k + 1);
    SGT_LAUNCHED();
    SGT_TRY(split_pair(st, G, R[k + 1], GsR[k + 1], R[k + 1], R[k + 1]));
  }

  // ---- right-to-left projections, bond eigensolves, refinement ----
  pair_one_kernel<<<1, 1, 0, st>>>(Ft.h, Ft.l);
  SGT_LAUNCHED();
  for (int k = n - 1; k >= 0; --k) {
    const int64_t r = R[k], r2 = R[k + 1], p = Pd[k], xc = x[k + 1], c = p * xc;
    SGT_TRY(phase_mark(st, PH_Y));
    // Yt (c x r): Yt[(o, j)][(a, b)] = sum_{i, a', b'} F[j][(a', b')] X[a][i][a'] W[b][i][o][b'],
    // contracted in two products without forming the product core:
    //   S1: T[(j, a')][(b, i, o)] = sum_b' F[(j, a')][b'] W[(b, i, o)][b']          (K = B')
    //   S2: Y2[a][(b, o, j)] = sum_(i, a') X[a][(i, a')] T[(b, o, j)][(i, a')]   (K = d chi')
    //   Yt[(o, j)][(a, b)] = Y2[a][(b, o, j)]
    {
      const int64_t A = xs[3 * k], I = xs[3 * k + 1], A2 = xs[3 * k + 2];
      const int64_t Bk = w[k].b, O = w[k].o, B2 = w[k].b2, bio = Bk * I * O;
      SGT_TRY(split_pair(st, Ft, B2, Fs, xc * A2, B2));
      SGT_TRY(oz_split_f64(st, W[k], B2, 1, bio, B2, Wsl.s, Wsl.e, 1));
      Wsl.rows = bio;
      Wsl.cols = B2;
      SGT_TRY(gemm(xc * A2, bio, B2, 1.f, Fs.mat(), Wsl.mat(), 0.f, Tp, bio));
      Perm5 pq{{Bk, O, xc, I, A2}, {I * O, 1, A2 * bio, O, bio}};
      pair_permute_kernel<<<grid_for(xc * A2 * bio), 256, 0, st>>>(Tq.h, Tq.l, Tp.h, Tp.l, pq);
      SGT_LAUNCHED();
      SGT_TRY(split_pair(st, Tq, I * A2, Tqs, Bk * O * xc, I * A2));
      SGT_TRY(oz_split_f64(st, X[k], I * A2, 1, A, I * A2, Xsl.s, Xsl.e, 1));
      Xsl.rows = A;
      Xsl.cols = I * A2;
      SGT_TRY(gemm(A, Bk * O * xc, I * A2, 1.f, Xsl.mat(), Tqs.mat(), 0.f, GY, Bk * O * xc));
      Perm5 py{{1, O, xc, A, Bk}, {0, xc, 1, Bk * O * xc, O * xc}};
      pair_permute_kernel<<<grid_for(c * r), 256, 0, st>>>(Yt.h, Yt.l, GY.h, GY.l, py);
      SGT_LAUNCHED();
    }
    if (k == 0) {
      // core_0[0][o][j] = Yt[o*xc + j][0]
      pair_to_f64_kernel<<<grid_for(c), 256, 0, st>>>(Yt.h, Yt.l, 1, out[0], 1, c, 1);
      SGT_LAUNCHED();
      break;
    }
    const int64_t keep = x[k];
    if (!spectra && keep >= c) {
      // nothing is cut at this bond (the rank bound keeps all c directions):
      // the identity is an orthonormal basis of the kept space, no bond matrix needed
      pair_eye_kernel<<<grid_for(keep * c), 256, 0, st>>>(Vk.h, Vk.l, keep, c);
      SGT_LAUNCHED();
      pair_to_f64_kernel<<<grid_for(keep * c), 256, 0, st>>>(Vk.h, Vk.l, c, out[k], c, keep, c);
      SGT_LAUNCHED();
      if (discarded) SGT_CUDA(cudaMemsetAsync(discarded + (k - 1), 0, sizeof(double), st));
    } else {
    SGT_TRY(phase_mark(st, PH_BOND));
    // GY (c x r) = Ytp G_k^T, with Ytp = Yt's columns in G_k's (b, a) column order
    const int64_t chik = xs[3 * k], Dk = w[k].b;
    SGT_TRY(pair_transpose(st, Ytp, chik, r, Yt, Dk, r, chik, Dk, c));
    SGT_TRY(split_pair(st, Ytp, r, Ytps, c, r));
    SGT_TRY(gemm(c, r, r, 1.f, Ytps.mat(), GsR[k].mat(), 0.f, GY, r));
    // Z (c x c) = Yt GY^T
    SGT_TRY(split_pair(st, Yt, r, Yts, c, r));
    SGT_TRY(split_pair(st, GY, r, GYs, c, r));
    SGT_TRY(gemm(c, c, r, 1.f, Yts.mat(), GYs.mat(), 0.f, Z, c));
    pair_symmetrize_kernel<<<grid_for(c * c), 256, 0, st>>>(Z.h, Z.l, c);
    SGT_LAUNCHED();
    if (!spectra && keep < c) {
      // ---- kept subspace by purification (no eigenvectors, no spectrum) ----
      SGT_TRY(phase_mark(st, PH_PURIFY));
      pair_frob_trace_kernel<<<RED_BLOCKS, 256, 0, st>>>(Z.h, Z.l, c, rpart, ticket, dscal, dscal + 1);
      SGT_LAUNCHED();
      pair_scale_by_kernel<<<grid_for(c * c), 256, 0, st>>>(Z.h, Z.l, c, dscal, VV.h, VV.l);
      SGT_LAUNCHED();
      Pair X = VV, X2 = T;
      SGT_CUDA(cudaMemsetAsync(ichoice, 0, 2 * sizeof(int), st));
      SGT_CUDA(cudaMemsetAsync(tc2_resid, 0, sizeof(unsigned) * TC2_ITERS, st));
      pair_diag_kernel<<<grid_for(c), 256, 0, st>>>(X.h, X.l, (int)c, tc2_diag);
      SGT_LAUNCHED();
      SGT_TRY(oz_split_pair(st, X.h, X.l, c, c, c, Vts.s, Vts.e, 1));
      Vts.rows = c;
      Vts.cols = c;
      const unsigned sg = (unsigned)std::min<int64_t>(cdiv(c, 8), 152 * 4);
      const unsigned sg4 = (unsigned)std::min<int64_t>(c, 152 * 16);
      auto a16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
      const bool vec4 = c % 4 == 0 && a16(X.h) && a16(X.l) && a16(T.h) && a16(T.l) && a16(part) &&
                        a16(Vts.s) && __atomic_load_n(&g_tc2_vec, __ATOMIC_RELAXED) != 0;
      for (int it = 0; it < TC2_ITERS; ++it) {
        // X2 = X X; a split-K product leaves its partials, which the step adds
        int S = 1;
        SGT_TRY(oz_gemm(st, c, c, c, 1.f, Vts.mat(), Vts.mat(), 0.f, X2.h, X2.l, c, part, part_floats, err,
                        ichoice + 1, &S));
        const float* x2h = S > 1 ? part : X2.h;
        const float* x2l = S > 1 ? part + (int64_t)S * c * c : X2.l;
        if (vec4)
          tc2_step4_kernel<<<sg4, TC2_VEC_THREADS, 0, st>>>(
              X.h, X.l, x2h, x2l, S, (int)c, (int)keep, tc2_diag + (it & 1) * 2 * c,
              tc2_diag + ((it + 1) & 1) * 2 * c, ichoice, tc2_resid + it, ticket, Vts.s, oz_ld(c), c * oz_ld(c), Vts.e);
        else
          tc2_step_kernel<<<sg, 256, 0, st>>>(X.h, X.l, x2h, x2l, S, (int)c, (int)keep, tc2_diag + (it & 1) * 2 * c,
                                               tc2_diag + ((it + 1) & 1) * 2 * c, ichoice, tc2_resid + it, ticket,
                                               Vts.s, oz_ld(c), c * oz_ld(c), Vts.e);
        SGT_LAUNCHED();
      }
      // McWeeny clean-up of a projector the trace correction could not finish
      // (every launch returns at once when ctl[1] says it did; opt-in, since
      // even skipped launches cost ~3% of a sweep that never needs them)
      const bool cleanup = __atomic_load_n(&g_purify_cleanup, __ATOMIC_RELAXED) != 0;
      SGT_CUDA(cudaMemsetAsync(mcw_resid, 0xff, sizeof(unsigned) * MCW_ITERS, st));  // NaN bits: no clean-up ran
      for (int it = 0; cleanup && it < MCW_ITERS; ++it) {
        SGT_TRY(oz_gemm(st, c, c, c, 1.f, Vts.mat(), Vts.mat(), 0.f, X2.h, X2.l, c, part, part_floats, err,
                        ichoice + 1));                                            // X2 = X X
        if (it == 0) SGT_CUDA(cudaMemsetAsync(mcw_resid, 0, sizeof(unsigned) * MCW_ITERS, st));
        SGT_TRY(oz_split_pair(st, X2.h, X2.l, c, c, c, Ts.s, Ts.e, 1, ichoice + 1));
        Ts.rows = c;
        Ts.cols = c;
        SGT_TRY(oz_gemm(st, c, c, c, 1.f, Ts.mat(), Vts.mat(), 0.f, S.h, S.l, c, part, part_floats, err,
                        ichoice + 1));                                            // X3 = X2 X
        mcweeny_step_kernel<<<grid_for(c * c), 256, 0, st>>>(X.h, X.l, X2.h, X2.l, S.h, S.l, c * c, ichoice,
                                                              mcw_resid + it);
        SGT_LAUNCHED();
        SGT_TRY(oz_split_pair(st, X.h, X.l, c, c, c, Vts.s, Vts.e, 1, ichoice + 1));
      }
      tc2_status_kernel<<<1, 1, 0, st>>>(ichoice, tc2_resid + (TC2_ITERS - 1), mcw_resid + (MCW_ITERS - 1),
                                         stat + k);
      SGT_LAUNCHED();
      pair_symmetrize_kernel<<<grid_for(c * c), 256, 0, st>>>(X.h, X.l, c);
      SGT_LAUNCHED();
      SGT_TRY(phase_mark(st, PH_BASIS));
      // basis: Q = L^T X with L the rank-keep pivoted Cholesky factor of X's FP32 part
      SGT_TRY(pivoted_chol(st, X.h, c, keep, Vt32, perm, Z32));  // Z32 (c*c) and lam32 (c) are free here
      SGT_TRY(oz_split_pair(st, Vt32, nullptr, c, keep, c, Ets.s, Ets.e, 1));
      Ets.rows = keep;
      Ets.cols = c;
      SGT_TRY(split_pair(st, X, c, Vts, c, c));
      SGT_TRY(gemm(keep, c, c, 1.f, Ets.mat(), Vts.mat(), 0.f, Vk, c));
      // Newton-Schulz: Q <- 1.5 Q - 0.5 (Q Q^T) Q; after a purification that
      // needed the McWeeny clean-up the start is further from orthonormal, and
      // NS_EXTRA more steps run (skipped on the device otherwise)
      for (int it = 0; it < NS_ITERS + (cleanup ? NS_EXTRA : 0); ++it) {
        const int* sk = it < NS_ITERS ? nullptr : ichoice + 1;
        SGT_TRY(split_pair(st, Vk, c, Vks, keep, c, sk));
        SGT_TRY(oz_gemm(st, keep, keep, c, 1.f, Vks.mat(), Vks.mat(), 0.f, S.h, S.l, keep, part, part_floats, err, sk));
        SGT_TRY(split_pair(st, S, keep, Ts, keep, keep, sk));
        SGT_TRY(pair_transpose(st, Xv, keep, 0, Vk, c, 0, keep, c, 1, sk));
        SGT_TRY(split_pair(st, Xv, keep, Xvs, c, keep, sk));
        SGT_TRY(oz_gemm(st, keep, c, keep, -0.5f, Ts.mat(), Xvs.mat(), 1.5f, Vk.h, Vk.l, c, part, part_floats, err, sk));
      }
      pair_to_f64_kernel<<<grid_for(keep * c), 256, 0, st>>>(Vk.h, Vk.l, c, out[k], c, keep, c);
      SGT_LAUNCHED();
      SGT_TRY(phase_mark(st, PH_DISC));
      if (discarded) {
        // discarded weight = 1 - trace(Q Z Q^T) / trace(Z)
        SGT_TRY(split_pair(st, Vk, c, Vks, keep, c));
        SGT_TRY(split_pair(st, Z, c, Zs, c, c));
        SGT_TRY(gemm(keep, c, c, 1.f, Vks.mat(), Zs.mat(), 0.f, S, c));
        kept_trace_kernel<<<RED_BLOCKS, 256, 0, st>>>(S.h, S.l, Vk.h, Vk.l, keep * c, dscal + 1, rpart, ticket,
                                                       discarded + (k - 1));
        SGT_LAUNCHED();
      }
    } else {
    SGT_TRY(phase_mark(st, PH_EIG));
    // FP32 Jacobi on the leading part of Z: first approximation
    SGT_CUDA(cudaMemcpyAsync(Z32, Z.h, sizeof(float) * c * c, cudaMemcpyDeviceToDevice, st));
    {
      Arena ja(jscratch, jbytes);
      SGT_TRY(sym_eig_rows_f32(st, Z32, c, Vt32, lam32, stat + k, ja, eig_method_current()));
    }
    SGT_CUDA(cudaMemcpyAsync(Vt.h, Vt32, sizeof(float) * c * c, cudaMemcpyDeviceToDevice, st));
    SGT_CUDA(cudaMemsetAsync(Vt.l, 0, sizeof(float) * c * c, st));
    // refinement against the pair-accurate Z
    SGT_TRY(split_pair(st, Z, c, Zs, c, c));
    for (int it = 0; it < 2; ++it) {
      SGT_TRY(split_pair(st, Vt, c, Vts, c, c));
      SGT_TRY(gemm(c, c, c, 1.f, Vts.mat(), Vts.mat(), 0.f, VV, c));   // VV = Vt Vt^T
      SGT_TRY(gemm(c, c, c, 1.f, Vts.mat(), Zs.mat(), 0.f, T, c));     // T = Vt Z
      SGT_TRY(split_pair(st, T, c, Ts, c, c));
      SGT_TRY(gemm(c, c, c, 1.f, Ts.mat(), Vts.mat(), 0.f, S, c));     // S = Vt Z Vt^T
      oa_lambda_kernel<<<grid_for(c), 256, 0, st>>>(S.h, S.l, VV.h, VV.l, (int)c, lamp.h, lamp.l);
      SGT_LAUNCHED();
      SGT_CUDA(cudaMemsetAsync(gmax, 0, sizeof(unsigned), st));
      pair_absmax_kernel<<<grid_for(c), 256, 0, st>>>(lamp.h, c, gmax);
      SGT_LAUNCHED();
      oa_correction_kernel<<<grid_for(c * c), 256, 0, st>>>(S.h, S.l, VV.h, VV.l, lamp.h, lamp.l, (int)c, gmax, Et.h,
                                                             Et.l);
      SGT_LAUNCHED();
      SGT_TRY(split_pair(st, Et, c, Ets, c, c));
      SGT_TRY(pair_transpose(st, Xv, c, 0, Vt, c, 0, c, c, 1));             // Xv = Vt^T
      SGT_TRY(split_pair(st, Xv, c, Xvs, c, c));
      SGT_TRY(gemm(c, c, c, 1.f, Ets.mat(), Xvs.mat(), 1.f, Vt, c));   // Vt += E^T Vt
    }
    // final eigenvalues of the refined vectors
    SGT_TRY(split_pair(st, Vt, c, Vts, c, c));
    SGT_TRY(gemm(c, c, c, 1.f, Vts.mat(), Vts.mat(), 0.f, VV, c));
    SGT_TRY(gemm(c, c, c, 1.f, Vts.mat(), Zs.mat(), 0.f, T, c));
    SGT_TRY(split_pair(st, T, c, Ts, c, c));
    SGT_TRY(gemm(c, c, c, 1.f, Ts.mat(), Vts.mat(), 0.f, S, c));
    oa_lambda_kernel<<<grid_for(c), 256, 0, st>>>(S.h, S.l, VV.h, VV.l, (int)c, lamp.h, lamp.l);
    SGT_LAUNCHED();
    rank_desc_kernel<<<1, 1024, 0, st>>>(lamp.h, (int)c, perm);
    SGT_LAUNCHED();
    gather_rows_kernel<<<grid_for(keep * c), 256, 0, st>>>(Vt.h, Vt.l, (int)c, perm, (int)keep, out[k], Vk.h, Vk.l);
    SGT_LAUNCHED();
    double* spec_k = nullptr;
    if (spectra) {
      int64_t off = 0;
      for (int j = 1; j < k; ++j) off += cnt[j];
      spec_k = spectra + off;
    }
    oz_spectrum_kernel<<<1, 256, 0, st>>>(lamp.h, lamp.l, perm, (int)cnt[k], (int)keep, spec_k,
                                          discarded ? discarded + (k - 1) : nullptr, gexp + k);
    SGT_LAUNCHED();
    }
    }  // bond matrix branches
    SGT_TRY(phase_mark(st, PH_CARRY));
    // Ft_k (keep x r) = Vk Y^T with Y = Yt^T (r x c)
    Pair Y = Ytp;  // Ytp is free again
    SGT_TRY(pair_transpose(st, Y, c, 0, Yt, r, 0, c, r, 1));
    SGT_TRY(split_pair(st, Y, c, Ys, r, c));
    SGT_TRY(split_pair(st, Vk, c, Vks, keep, c));
    SGT_TRY(gemm(keep, r, c, 1.f, Vks.mat(), Ys.mat(), 0.f, Ft, r));
  }
  if (status) {
    oz_status_kernel<<<1, 32, 0, st>>>(stat, n, status, err);
    SGT_LAUNCHED();
  }
  SGT_TRY(phase_mark(st, -1));
  return SGT_OK;
}

// TT-SVD rounding of a plain chain in this form: the chain is the product of
// a bond-1 identity MPO with itself (one d x d identity core per site).
int oz_round_chain(cudaStream_t st, int n, const double* const* X, const int64_t* xs, int64_t chi, double* const* out,
                   double* spectra, double* discarded, int* status, Arena& ar) {
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
      identity_cores_f64_kernel<<<(unsigned)count, 128, 0, st>>>(eye, ed, k0, count, (int)(dmax * dmax));
      SGT_LAUNCHED();
    }
    for (int k = 0; k < n; ++k) W[k] = eye + (int64_t)k * dmax * dmax;
  }
  return oz_round_impl(st, n, W.data(), w4.data(), X, xs, chi, out, spectra, discarded, status, ar);
}

// FP64 in / FP64 out through the sliced GEMM (exported for tests and callers):
// C = alpha A B^T + beta C, A (M x K, lda), B (N x K, ldb), C (M x N, ldc).
static int gemm_f64_sliced_impl(cudaStream_t st, int64_t M, int64_t N, int64_t K, double alpha, const double* A,
                                int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                                Arena& ar) {
  SGT_REQUIRE(M > 0 && N > 0 && K > 0, SGT_ERR_INVALID, "gemm_f64_sliced: empty problem");
  Sliced As = take_sliced(ar, M, K), Bs = take_sliced(ar, N, K);
  Pair Cp = take_pair(ar, M * N);
  const size_t pb = oz_gemm_ws_bytes(M, N, K);
  float* part = ar.take<float>(pb / sizeof(float) + 1);
  int* err = ar.take<int>(1);
  if (ar.measure) return SGT_OK;
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "gemm_f64_sliced: workspace too small");
  SGT_TRY(oz_split_f64(st, A, lda, 1, M, K, As.s, As.e, 1));
  SGT_TRY(oz_split_f64(st, B, ldb, 1, N, K, Bs.s, Bs.e, 1));
  SGT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  SGT_TRY(oz_gemm(st, M, N, K, 1.f, As.mat(), Bs.mat(), 0.f, Cp.h, Cp.l, N, part, (int64_t)(pb / sizeof(float)), err));
  // C = alpha * (Ch + Cl) + beta * C in FP64 (alpha / beta stay FP64)
  axpby_pair_f64_kernel<<<grid_for(M * N), 256, 0, st>>>(Cp.h, Cp.l, N, alpha, beta, C, ldc, M, N);
  SGT_LAUNCHED();
  return SGT_OK;
}

// Overlap <X|Y> with both contractions of every transfer step on the sliced
// GEMM (tensor cores, FP64-class), the transfer matrix E kept in FP64 between
// sites and rescaled by exact powers of two as in the FP64 sweep:
//   T (a x p c2)  = E (a x c) Y_k (c x p c2)        [A = E, B = Y_k^T]
//   E' (a2 x c2)  = X_k^T (a2 x a p) T (a p x c2)   [A = X_k^T, B = T^T]
// The transposed operands are sliced straight from strided FP64 views.
static int overlap_sliced_impl(cudaStream_t st, int n, const double* const* X, const int64_t* xs,
                               const double* const* Y, const int64_t* ys, double* result, Arena& ar) {
  SGT_REQUIRE(n >= 1 && xs && ys, SGT_ERR_INVALID, "overlap: empty chain");
  int64_t emax = 1, tmax = 1, es = 1, ys_ = 1, ts = 1, xs_ = 1;
  size_t pb = 0;
  for (int k = 0; k < n; ++k) {
    const int64_t a = xs[3 * k], p = xs[3 * k + 1], a2 = xs[3 * k + 2];
    const int64_t c = ys[3 * k], c2 = ys[3 * k + 2];
    SGT_REQUIRE(a > 0 && p > 0 && a2 > 0 && c > 0 && c2 > 0 && ys[3 * k + 1] == p, SGT_ERR_INVALID,
                "overlap: bad shapes at site %d", k);
    if (k + 1 < n)
      SGT_REQUIRE(a2 == xs[3 * k + 3] && c2 == ys[3 * k + 3], SGT_ERR_INVALID,
                  "overlap: bond mismatch between sites %d and %d", k, k + 1);
    emax = std::max(emax, a2 * c2);
    tmax = std::max(tmax, a * p * c2);
    es = std::max<int64_t>(es, (int64_t)oz_slice_elems(a, c));
    ys_ = std::max<int64_t>(ys_, (int64_t)oz_slice_elems(p * c2, c));
    ts = std::max<int64_t>(ts, (int64_t)oz_slice_elems(c2, a * p));
    xs_ = std::max<int64_t>(xs_, (int64_t)oz_slice_elems(a2, a * p));
    pb = std::max(pb, oz_gemm_ws_bytes(a, p * c2, c));
    pb = std::max(pb, oz_gemm_ws_bytes(a2, c2, a * p));
  }
  SGT_REQUIRE(xs[0] == 1 && ys[0] == 1 && xs[3 * n - 1] == 1 && ys[3 * n - 1] == 1, SGT_ERR_INVALID,
              "overlap: boundary bonds must be 1");
  int64_t rmax = 1;
  for (int k = 0; k < n; ++k) rmax = std::max(rmax, std::max(xs[3 * k + 2], std::max(ys[3 * k], xs[3 * k])));
  double* E = ar.take<double>(emax);
  double* Td = ar.take<double>(tmax);
  Pair Tp = take_pair(ar, std::max(tmax, emax));
  Sliced Es, Ysl, Tsl, Xsl;
  Es.s = ar.take<__nv_bfloat16>((size_t)es);
  Es.e = ar.take<int>((size_t)rmax);
  Ysl.s = ar.take<__nv_bfloat16>((size_t)ys_);
  Ysl.e = ar.take<int>((size_t)tmax);
  Tsl.s = ar.take<__nv_bfloat16>((size_t)ts);
  Tsl.e = ar.take<int>((size_t)tmax);
  Xsl.s = ar.take<__nv_bfloat16>((size_t)xs_);
  Xsl.e = ar.take<int>((size_t)rmax);
  float* part = ar.take<float>(pb / sizeof(float) + 1);
  const int64_t part_floats = (int64_t)(pb / sizeof(float));
  double* expo = ar.take<double>(1);
  int* err = ar.take<int>(1);
  if (ar.measure) return SGT_OK;
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "overlap: workspace too small");
  SGT_REQUIRE(X && Y && result, SGT_ERR_INVALID, "overlap: null argument");
  SGT_TRY(fill_f64(st, E, 1, 1.0));
  SGT_TRY(zero_scalar(st, expo));
  SGT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  for (int k = 0; k < n; ++k) {
    const int64_t a = xs[3 * k], p = xs[3 * k + 1], a2 = xs[3 * k + 2];
    const int64_t c = ys[3 * k], c2 = ys[3 * k + 2];
    // T = E Y_k: A = E (a x c, row stride c), B = Y_k^T (p c2 x c: element (j, i) = Y_k[i, j])
    SGT_TRY(oz_split_f64(st, E, c, 1, a, c, Es.s, Es.e, 1));
    Es.rows = a;
    Es.cols = c;
    SGT_TRY(oz_split_f64(st, Y[k], 1, p * c2, p * c2, c, Ysl.s, Ysl.e, 1));
    Ysl.rows = p * c2;
    Ysl.cols = c;
    SGT_TRY(oz_gemm(st, a, p * c2, c, 1.f, Es.mat(), Ysl.mat(), 0.f, Tp.h, Tp.l, p * c2, part, part_floats, err));
    pair_to_f64_kernel<<<grid_for(a * p * c2), 256, 0, st>>>(Tp.h, Tp.l, p * c2, Td, p * c2, a, p * c2);
    SGT_LAUNCHED();
    // E' = X_k^T T: A = X_k^T (a2 x a p: element (j, i) = X_k[i, j]), B = T^T (c2 x a p, T as (a p) x c2)
    SGT_TRY(oz_split_f64(st, X[k], 1, a2, a2, a * p, Xsl.s, Xsl.e, 1));
    Xsl.rows = a2;
    Xsl.cols = a * p;
    SGT_TRY(oz_split_f64(st, Td, 1, c2, c2, a * p, Tsl.s, Tsl.e, 1));
    Tsl.rows = c2;
    Tsl.cols = a * p;
    SGT_TRY(oz_gemm(st, a2, c2, a * p, 1.f, Xsl.mat(), Tsl.mat(), 0.f, Tp.h, Tp.l, c2, part, part_floats, err));
    pair_to_f64_kernel<<<grid_for(a2 * c2), 256, 0, st>>>(Tp.h, Tp.l, c2, E, c2, a2, c2);
    SGT_LAUNCHED();
    SGT_TRY(rescale_pow2(st, E, a2 * c2, expo, result, k == n - 1));
  }
  return SGT_OK;
}

}  // namespace sgt

using namespace sgt;

extern "C" SGT_API size_t sgt_overlap_prec_workspace_size(int n, const int64_t* xshape, const int64_t* yshape,
                                                         int precision) {
  if (precision == SGT_PREC_F64) return sgt_overlap_workspace_size(n, xshape, yshape);
  if (precision != SGT_PREC_BF16X6) {
    set_error("overlap: precision %d not supported (SGT_PREC_F64 or SGT_PREC_BF16X6)", precision);
    return 0;
  }
  Arena a = Arena::measuring();
  if (overlap_sliced_impl(nullptr, n, nullptr, xshape, nullptr, yshape, nullptr, a) != SGT_OK) return 0;
  return a.used;
}

extern "C" SGT_API int sgt_overlap_sweep_prec(int n, const double* const* X, const int64_t* xshape,
                                              const double* const* Y, const int64_t* yshape, int precision,
                                              double* result, void* ws, size_t ws_bytes, void* stream) {
  if (precision == SGT_PREC_F64) return sgt_overlap_sweep(n, X, xshape, Y, yshape, result, ws, ws_bytes, stream);
  SGT_REQUIRE(precision == SGT_PREC_BF16X6, SGT_ERR_INVALID,
              "overlap: precision %d not supported (SGT_PREC_F64 or SGT_PREC_BF16X6)", precision);
  Arena a(ws, ws_bytes);
  return overlap_sliced_impl(as_stream(stream), n, X, xshape, Y, yshape, result, a);
}

extern "C" SGT_API size_t sgt_gemm_f64_sliced_workspace_size(int64_t M, int64_t N, int64_t K) {
  Arena a = Arena::measuring();
  if (gemm_f64_sliced_impl(nullptr, M, N, K, 1.0, nullptr, K, nullptr, K, 0.0, nullptr, N, a) != SGT_OK) return 0;
  return a.used;
}

extern "C" SGT_API int sgt_gemm_f64_sliced(int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
                                           const double* B, int64_t ldb, double beta, double* C, int64_t ldc, void* ws,
                                           size_t ws_bytes, void* stream) {
  SGT_REQUIRE(A && B && C && ws, SGT_ERR_INVALID, "gemm_f64_sliced: null argument");
  Arena a(ws, ws_bytes);
  return gemm_f64_sliced_impl(as_stream(stream), M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, a);
}

extern "C" SGT_API int sgt_set_tuning(int key, int value) {
  if (key == SGT_TUNE_SLICED_SPLIT_CTAS) return sgt::oz_set_split_ctas(value);
  if (key == SGT_TUNE_SLICED_SPLIT_MIN_KTILES) return sgt::oz_set_split_min_ktiles(value);
  if (key == SGT_TUNE_PCHOL_BLOCKED || key == SGT_TUNE_PURIFY_CLEANUP || key == SGT_TUNE_PURIFY_VECTOR_STEP) {
    SGT_REQUIRE(value == 0 || value == 1, SGT_ERR_INVALID, "set_tuning: key %d takes 0 or 1, not %d", key, value);
    int* slot = key == SGT_TUNE_PCHOL_BLOCKED   ? &sgt::g_pchol_blocked
                : key == SGT_TUNE_PURIFY_CLEANUP ? &sgt::g_purify_cleanup
                                                 : &sgt::g_tc2_vec;
    __atomic_store_n(slot, value, __ATOMIC_RELAXED);
    return SGT_OK;
  }
  sgt::set_error("set_tuning: unknown key %d", key);
  return SGT_ERR_INVALID;
}

extern "C" SGT_API int sgt_get_tuning(int key) {
  if (key == SGT_TUNE_SLICED_SPLIT_CTAS) return sgt::oz_split_ctas();
  if (key == SGT_TUNE_SLICED_SPLIT_MIN_KTILES) return sgt::oz_split_min_ktiles();
  if (key == SGT_TUNE_PCHOL_BLOCKED) return __atomic_load_n(&sgt::g_pchol_blocked, __ATOMIC_RELAXED);
  if (key == SGT_TUNE_PURIFY_CLEANUP) return __atomic_load_n(&sgt::g_purify_cleanup, __ATOMIC_RELAXED);
  if (key == SGT_TUNE_PURIFY_VECTOR_STEP) return __atomic_load_n(&sgt::g_tc2_vec, __ATOMIC_RELAXED);
  return -1;
}

extern "C" SGT_API int sgt_phase_profile(int enable, double* ms, int count) {
  if (enable) {
    sgt::g_phase.on = true;
    return SGT_OK;
  }
  sgt::g_phase.on = false;
  const std::vector<sgt::PhaseMark> marks = sgt::g_phase.take();
  double acc[sgt::PH_COUNT] = {};
  int rc = SGT_OK;
  for (size_t i = 0; i + 1 < marks.size(); ++i) {
    const auto& a = marks[i];
    if (a.phase < 0) continue;
    float t = 0.f;
    if (cudaEventSynchronize(marks[i + 1].ev) != cudaSuccess ||
        cudaEventElapsedTime(&t, a.ev, marks[i + 1].ev) != cudaSuccess) {
      sgt::set_error("phase_profile: event timing failed");
      rc = SGT_ERR_CUDA;
      break;
    }
    acc[a.phase] += t;
  }
  for (const auto& m : marks) cudaEventDestroy(m.ev);
  if (ms)
    for (int q = 0; q < count && q < sgt::PH_COUNT; ++q) ms[q] = acc[q];
  return rc;
}

extern "C" SGT_API int sgt_sliced_profile(int enable, double* ms, double* flops, long long* launches) {
  return sgt::oz_profile(enable, ms, flops, launches);
}
