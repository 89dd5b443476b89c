// Left Gram recursion of an MPO x MPS product without forming the product.
//
// With the product core P[(a,b), o, (a',b')] = sum_i X[a,i,a'] W[b,i,o,b'],
//   G'[(a',b'),(c',e')] = sum_o P_o^T G P_o
// is evaluated as
//   A. T1[a,b,e,j,c'] = sum_c  G[(a,b),(c,e)] X[c,j,c']          (tcgen05 GEMM, K = chi)
//   B. U [a,b,o,c',e'] = sum_{e,j} T1[a,b,e,j,c'] W[e,j,o,e']      (shared-memory kernel,
//   C. T3[a,i,b',c',e'] = sum_{b,o} W[b,i,o,b'] U[a,b,o,c',e']       K = D*d each)
//   D. G'[(a',b'),(c',e')] = sum_{a,i} X[a,i,a'] T3[a,i,b',c',e']  (tcgen05 GEMM, K = chi*d)
// which costs 2 chi^2 D^2 d chi' (A) + 2 chi'^2 D'^2 chi d (D) plus O(chi chi' D^3 d^2)
// instead of the 4 (chi D)^3 d of dense products (config 2: 3.8e10 vs 5.5e11 flops).
//
// G is kept with its column pair in (b, a) order ("Gp"): step A then reads
// contiguous K = c runs, and step D writes G' directly in that same order
// (rows (c',e'), columns (b',a')), so no transposes are needed between sites.
// B and C run fused in one kernel that also reorders T3 to the K-major layout
// [c'][e'][b'][a][i] of step D and splits it into TF32 hi / FP32 lo.
#include <algorithm>

#include "common.cuh"

namespace sgt {

int tc_gemm_tf32(cudaStream_t st, int passes, int64_t M, int64_t N, int64_t K, float alpha,
                 const float* Ahi, const float* Alo, int64_t lda, const float* Bhi, const float* Blo,
                 int64_t ldb, float beta, float* C, int64_t ldc, int* err);
int gemm_nt_dispatch(cudaStream_t st, int passes, int64_t M, int64_t N, int64_t K, float alpha, const float* Ah,
                     const float* Al, int64_t lda, const float* Bh, const float* Bl, int64_t ldb, float beta,
                     float* C, int64_t ldc, int* err);

namespace {

constexpr int GM_TA = 4;  // a values per block

__device__ __forceinline__ void split_store(float v, float* hi, float* lo, int64_t idx) {
  uint32_t h;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
  const float fh = __uint_as_float(h);
  hi[idx] = fh;
  lo[idx] = v - fh;
}

// Steps B and C for a tile of GM_TA values of a and TC values of c'.
// T1 layout [a][b][e][j][c'] (chi, D, D, d, chi2); W fp64 [b][i][o][b'];
// output T3 hi/lo layout [c'][e'][b'][a][i].
__global__ void __launch_bounds__(256) gram_mid_kernel(const float* __restrict__ T1, const double* __restrict__ W,
                                                       float* __restrict__ T3h, float* __restrict__ T3l, int chi,
                                                       int D, int d, int dout, int D2, int chi2, int TC) {
  extern __shared__ float gm_smem[];
  const int a0 = blockIdx.x * GM_TA, c0 = blockIdx.y * TC;
  const int bej = D * D * d;             // (b, e, j) extent
  const int boe = D * dout * D2;         // (b, o, e') extent
  float* sW = gm_smem;                   // [D][d][dout][D2]
  float* sT = sW + D * d * dout * D2;    // [TA][bej][TC]
  float* sU = sT + GM_TA * bej * TC;     // [TA][b][o][e'][TC]
  const int tid = threadIdx.x;
  for (int i = tid; i < D * d * dout * D2; i += 256) sW[i] = (float)W[i];
  for (int i = tid; i < GM_TA * bej * TC; i += 256) {
    const int t = i % TC, r = (i / TC) % bej, at = i / (TC * bej);
    const int a = a0 + at, c = c0 + t;
    sT[i] = (a < chi && c < chi2) ? T1[((int64_t)a * bej + r) * chi2 + c] : 0.f;
  }
  __syncthreads();
  // B: U[at][b][o][e'][t] = sum_{e,j} T1[at][b][e][j][t] W[e][j][o][e']
  for (int i = tid; i < GM_TA * boe * TC; i += 256) {
    const int t = i % TC;
    int r = i / TC;
    const int e2 = r % D2;
    r /= D2;
    const int o = r % dout;
    r /= dout;
    const int b = r % D, at = r / D;
    const float* tcol = sT + ((int64_t)at * bej + (int64_t)b * D * d) * TC + t;
    float acc = 0.f;
    for (int e = 0; e < D; ++e)
      for (int j = 0; j < d; ++j)
        acc = fmaf(tcol[(e * d + j) * TC], sW[((e * d + j) * dout + o) * D2 + e2], acc);
    sU[i] = acc;
  }
  __syncthreads();
  // C: T3[c'][e'][b'][a][i] = sum_{b,o} W[b][i][o][b'] U[at][b][o][e'][t]
  const int inner = GM_TA * d;  // (at, i) contiguous in the output
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
    float acc = 0.f;
    for (int b = 0; b < D; ++b)
      for (int o = 0; o < dout; ++o)
        acc = fmaf(sW[((b * d + i) * dout + o) * D2 + b2], sU[((((int64_t)at * D + b) * dout + o) * D2 + e2) * TC + t],
                   acc);
    const int64_t idx = (((int64_t)c * D2 + e2) * D2 + b2) * ((int64_t)chi * d) + (int64_t)a * d + i;
    split_store(acc, T3h, T3l, idx);
  }
}

// dst (cols x rows) = src^T split into hi / lo, src fp64 (rows x cols, row-major).
__global__ void transpose_split_f64_kernel(const double* __restrict__ src, int64_t rows, int64_t cols,
                                           float* __restrict__ hi, float* __restrict__ lo) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows * cols;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = i / rows, r = i % rows;  // dst index i = c * rows + r
    const double v = src[r * cols + c];
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"((float)v));
    const float fh = __uint_as_float(h);
    hi[i] = fh;
    lo[i] = (float)(v - (double)fh);
  }
}

size_t mid_smem_bytes(int D, int d, int dout, int D2, int TC) {
  return sizeof(float) * ((size_t)D * d * dout * D2 + (size_t)GM_TA * D * D * d * TC +
                          (size_t)GM_TA * D * dout * D2 * TC);
}

}  // namespace

// Scratch of one structured step (floats): Xt hi/lo, X2 hi/lo, T1, T3 hi/lo.
size_t gram_step_scratch_floats(int64_t chi, int64_t d, int64_t chi2, int64_t D, int64_t dout, int64_t D2) {
  (void)dout;
  auto r64 = [](int64_t v) { return (v + 63) / 64 * 64; };
  const int64_t xt = r64(d * chi2 * chi);
  const int64_t t1 = r64(chi * D * D * d * chi2);
  const int64_t t3 = r64(chi2 * D2 * D2 * chi * d);
  return (size_t)(4 * xt + t1 + 2 * t3);
}

bool gram_step_supported(int64_t D, int64_t d, int64_t dout, int64_t D2) {
  return mid_smem_bytes((int)D, (int)d, (int)dout, (int)D2, 1) <= 200 * 1024;
}

// Gp (hi/lo, R x R, columns in (b,a) order) -> Gout (fp32, R2 x R2, columns in (b',a') order).
int gram_step_structured(cudaStream_t st, int passes, const float* Gh, const float* Gl, const double* X,
                         int64_t chi, int64_t d, int64_t chi2, const double* W, int64_t D, int64_t dout,
                         int64_t D2, float* Gout, float* scratch, int* err) {
  auto r256 = [](int64_t n) { return (n + 63) / 64 * 64; };
  float* Xth = scratch;
  float* Xtl = Xth + r256(d * chi2 * chi);
  float* X2h = Xtl + r256(d * chi2 * chi);
  float* X2l = X2h + r256(d * chi2 * chi);
  float* T1 = X2l + r256(d * chi2 * chi);
  float* T3h = T1 + r256(chi * D * D * d * chi2);
  float* T3l = T3h + r256(chi2 * D2 * D2 * chi * d);
  const unsigned gs = (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(d * chi2 * chi, 256), 1024));
  // Xt[(j,c')][c] = X[c][j][c'] : transpose of X viewed as chi x (d chi2)
  transpose_split_f64_kernel<<<gs, 256, 0, st>>>(X, chi, d * chi2, Xth, Xtl);
  SGT_LAUNCHED();
  // X2[a'][(a,i)] = X[a][i][a'] : transpose of X viewed as (chi d) x chi2
  transpose_split_f64_kernel<<<gs, 256, 0, st>>>(X, chi * d, chi2, X2h, X2l);
  SGT_LAUNCHED();
  // A: T1 ((chi D D) x (d chi2)) = Gp viewed as (chi D D) x chi  times  Xt^T
  SGT_TRY(gemm_nt_dispatch(st, passes, chi * D * D, d * chi2, chi, 1.f, Gh, Gl, chi, Xth, Xtl, chi, 0.f, T1,
                           d * chi2, err));
  // B + C
  int TC = 8;
  while (TC > 1 && mid_smem_bytes((int)D, (int)d, (int)dout, (int)D2, TC) > 160 * 1024) TC /= 2;
  const size_t smem = mid_smem_bytes((int)D, (int)d, (int)dout, (int)D2, TC);
  static size_t smem_set = 0;
  if (smem > smem_set) {
    SGT_CUDA(cudaFuncSetAttribute(gram_mid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    smem_set = smem;
  }
  dim3 g((unsigned)cdiv(chi, GM_TA), (unsigned)cdiv(chi2, TC));
  gram_mid_kernel<<<g, 256, smem, st>>>(T1, W, T3h, T3l, (int)chi, (int)D, (int)d, (int)dout, (int)D2, (int)chi2,
                                        TC);
  SGT_LAUNCHED();
  // D: Gout ((chi2 D2 D2) x chi2) = T3 ((chi2 D2 D2) x (chi d)) times X2^T
  SGT_TRY(gemm_nt_dispatch(st, passes, chi2 * D2 * D2, chi2, chi * d, 1.f, T3h, T3l, chi * d, X2h, X2l, chi * d,
                           0.f, Gout, chi2, err));
  return SGT_OK;
}

}  // namespace sgt
