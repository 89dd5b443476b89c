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
                 int64_t ldb, float beta, float* C, int64_t ldc, int* err, float* part, int64_t part_floats);
int gemm_nt_dispatch(cudaStream_t st, int passes, int64_t M, int64_t N, int64_t K, float alpha, const float* Ah,
                     const float* Al, int64_t lda, const float* Bh, const float* Bl, int64_t ldb, float beta,
                     float* C, int64_t ldc, int* err, float* part = nullptr, int64_t part_floats = 0);

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

// Register-tiled form of steps B and C for middle sites (D2 = D, dout = d,
// D a multiple of 8), compile-time sizes.  Both steps are small GEMMs with
// K = 32-ish and a fixed W operand in shared memory:
//   B: rows (a, b, c') x K (e, j)  -> cols (o, e')   [U = T1 W]
//   C: rows (a, e', c') x K (b, o) -> cols (i, b')   [T3 = U W']
// A thread owns 8 rows (the 8 values of c' of the tile, contiguous in shared
// memory: two 16-byte loads per K step) x 8 columns (one 16-byte pair of W),
// so every 4 shared loads feed 64 FMAs.  U is laid out [a][e'][b][o][c'] for
// step C's row access; step C's tile is staged [c'][e'][b'][a][i] in the T1
// buffer and stored as 32-byte runs (a, i) with the TF32 hi/lo split.
constexpr int GT_TA = 4, GT_TC = 8, GT_THREADS = 256;

template <int D, int d>
__global__ void __launch_bounds__(GT_THREADS) gram_mid_tiled_kernel(const float* __restrict__ T1,
                                                                    const double* __restrict__ W,
                                                                    float* __restrict__ T3h, float* __restrict__ T3l,
                                                                    int chi, int chi2) {
  constexpr int K = D * d;               // (e, j) and (b, o) extents
  constexpr int NB = d * D;              // (o, e') and (i, b') extents
  constexpr int TROWS = GT_TA * D * K;   // T1 tile rows of 8 c' values: [a][b][e][j]
  extern __shared__ __align__(16) float gt_smem[];
  float* sWB = gt_smem;                  // [(e, j)][(o, e')] = W[e][j][o][e']
  float* sWC = sWB + K * NB;             // [(b, o)][(i, b')] = W[b][i][o][b']
  float* sT = sWC + K * NB;              // [a][b][e][j][c'], later the output stage
  float* sU = sT + TROWS * GT_TC;        // [a][e'][b][o][c']
  const int a0 = blockIdx.x * GT_TA, c0 = blockIdx.y * GT_TC;
  const int tid = threadIdx.x;
  for (int idx = tid; idx < K * NB; idx += GT_THREADS) {
    // idx = ((b * d + i) * d + o) * D + b2 in W's own order
    const int b2 = idx % D, o = (idx / D) % d, i = (idx / (D * d)) % d, b = idx / (D * d * d);
    const float w = (float)W[idx];
    sWB[idx] = w;                                          // [(b, i)][(o, b2)]
    sWC[(b * d + o) * NB + i * D + b2] = w;                // [(b, o)][(i, b2)]
  }
  const bool full_c = (c0 + GT_TC <= chi2) && (chi2 % 4 == 0);
  for (int idx = tid; idx < TROWS * (GT_TC / 4); idx += GT_THREADS) {
    const int r = idx / (GT_TC / 4), q = idx % (GT_TC / 4);
    const int at = r / (D * K), a = a0 + at;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a < chi) {
      const float* src = T1 + ((int64_t)a * (D * K) + (r % (D * K))) * chi2 + c0 + 4 * q;
      if (full_c) {
        v = *reinterpret_cast<const float4*>(src);
      } else {
        float t[4];
        for (int u = 0; u < 4; ++u) t[u] = (c0 + 4 * q + u < chi2) ? src[u] : 0.f;
        v = make_float4(t[0], t[1], t[2], t[3]);
      }
    }
    reinterpret_cast<float4*>(sT)[idx] = v;
  }
  __syncthreads();
  // ---- B: U[a][e'][b][o][c'] = sum_(e,j) T1[a][b][(e,j)][c'] W[(e,j)][(o,e')] ----
  for (int task = tid; task < GT_TA * D * (NB / 8); task += GT_THREADS) {
    const int cg = task % (NB / 8), rg = task / (NB / 8);  // rg = at * D + b
    const int at = rg / D, b = rg % D;
    const int n0 = cg * 8, o = n0 / D, e0 = n0 % D;
    float acc[8][8];
#pragma unroll
    for (int t = 0; t < 8; ++t)
#pragma unroll
      for (int n = 0; n < 8; ++n) acc[t][n] = 0.f;
    const float* arow = sT + (int64_t)rg * K * GT_TC;
#pragma unroll 4
    for (int k = 0; k < K; ++k) {
      const float4 x0 = *reinterpret_cast<const float4*>(arow + k * GT_TC);
      const float4 x1 = *reinterpret_cast<const float4*>(arow + k * GT_TC + 4);
      const float4 w0 = *reinterpret_cast<const float4*>(sWB + k * NB + n0);
      const float4 w1 = *reinterpret_cast<const float4*>(sWB + k * NB + n0 + 4);
      const float xa[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
      const float wb[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
      for (int t = 0; t < 8; ++t)
#pragma unroll
        for (int n = 0; n < 8; ++n) acc[t][n] = fmaf(xa[t], wb[n], acc[t][n]);
    }
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      float* dst = sU + ((((int64_t)at * D + e0 + n) * D + b) * d + o) * GT_TC;
      reinterpret_cast<float4*>(dst)[0] = make_float4(acc[0][n], acc[1][n], acc[2][n], acc[3][n]);
      reinterpret_cast<float4*>(dst)[1] = make_float4(acc[4][n], acc[5][n], acc[6][n], acc[7][n]);
    }
  }
  __syncthreads();
  // ---- C: stage[c'][e'][b'][a][i] = sum_(b,o) U[a][e'][(b,o)][c'] W'[(b,o)][(i,b')] ----
  float* stage = sT;
  for (int task = tid; task < GT_TA * D * (NB / 8); task += GT_THREADS) {
    const int cg = task % (NB / 8), rg = task / (NB / 8);  // rg = at * D + e'
    const int at = rg / D, e2 = rg % D;
    const int n0 = cg * 8, i = n0 / D, b20 = n0 % D;
    float acc[8][8];
#pragma unroll
    for (int t = 0; t < 8; ++t)
#pragma unroll
      for (int n = 0; n < 8; ++n) acc[t][n] = 0.f;
    const float* arow = sU + (int64_t)rg * K * GT_TC;
#pragma unroll 4
    for (int k = 0; k < K; ++k) {
      const float4 x0 = *reinterpret_cast<const float4*>(arow + k * GT_TC);
      const float4 x1 = *reinterpret_cast<const float4*>(arow + k * GT_TC + 4);
      const float4 w0 = *reinterpret_cast<const float4*>(sWC + k * NB + n0);
      const float4 w1 = *reinterpret_cast<const float4*>(sWC + k * NB + n0 + 4);
      const float xa[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
      const float wb[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
      for (int t = 0; t < 8; ++t)
#pragma unroll
        for (int n = 0; n < 8; ++n) acc[t][n] = fmaf(xa[t], wb[n], acc[t][n]);
    }
#pragma unroll
    for (int t = 0; t < 8; ++t)
#pragma unroll
      for (int n = 0; n < 8; ++n)
        stage[(((int64_t)(t * D + e2) * D + b20 + n) * GT_TA + at) * d + i] = acc[t][n];
  }
  __syncthreads();
  // ---- store: runs of GT_TA * d values (a, i) per (c', e', b') ----
  constexpr int RUN = GT_TA * d;
  for (int idx = tid; idx < GT_TC * D * D * RUN; idx += GT_THREADS) {
    const int ai = idx % RUN, rest = idx / RUN;  // rest = (t * D + e2) * D + b2
    const int t = rest / (D * D);
    const int at = ai / d, a = a0 + at, c = c0 + t;
    if (a >= chi || c >= chi2) continue;
    const int64_t g = ((int64_t)c * D * D + rest % (D * D)) * ((int64_t)chi * d) + (int64_t)a0 * d + ai;
    split_store(stage[idx], T3h, T3l, g);
  }
}

template <int D, int d>
size_t tiled_smem_bytes() {
  return sizeof(float) * (2 * (size_t)(D * d) * (d * D) + 2 * (size_t)GT_TA * D * (D * d) * GT_TC);
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
  if (D2 == D && dout == d) {
    bool done = false;
    dim3 gt((unsigned)cdiv(chi, GT_TA), (unsigned)cdiv(chi2, GT_TC));
    auto run = [&](auto kern, size_t smem) -> int {
      if (smem > 200 * 1024) return SGT_OK;  // the generic kernel below takes it
      SGT_CUDA(func_attr_at_least((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      kern<<<gt, GT_THREADS, smem, st>>>(T1, W, T3h, T3l, (int)chi, (int)chi2);
      SGT_LAUNCHED();
      done = true;
      return SGT_OK;
    };
    if (D == 16 && d == 2) SGT_TRY(run(gram_mid_tiled_kernel<16, 2>, tiled_smem_bytes<16, 2>()));
    else if (D == 16 && d == 4) SGT_TRY(run(gram_mid_tiled_kernel<16, 4>, tiled_smem_bytes<16, 4>()));
    else if (D == 8 && d == 2) SGT_TRY(run(gram_mid_tiled_kernel<8, 2>, tiled_smem_bytes<8, 2>()));
    else if (D == 8 && d == 3) SGT_TRY(run(gram_mid_tiled_kernel<8, 3>, tiled_smem_bytes<8, 3>()));
    else if (D == 8 && d == 4) SGT_TRY(run(gram_mid_tiled_kernel<8, 4>, tiled_smem_bytes<8, 4>()));
    else if (D == 16 && d == 3) SGT_TRY(run(gram_mid_tiled_kernel<16, 3>, tiled_smem_bytes<16, 3>()));
    if (done) {
      SGT_TRY(gemm_nt_dispatch(st, passes, chi2 * D2 * D2, chi2, chi * d, 1.f, T3h, T3l, chi * d, X2h, X2l,
                               chi * d, 0.f, Gout, chi2, err));
      return SGT_OK;
    }
  }
  int TC = 8;
  while (TC > 1 && mid_smem_bytes((int)D, (int)d, (int)dout, (int)D2, TC) > 160 * 1024) TC /= 2;
  const size_t smem = mid_smem_bytes((int)D, (int)d, (int)dout, (int)D2, TC);
  SGT_CUDA(func_attr_at_least((const void*)gram_mid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
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
