// FP64 row-major batched GEMM used by every plain-FP64 sweep.
//
// GB300 executes FP64 at a small fraction of its other rates (about 2 DFMA per
// clock per SM), so a register-blocked CUDA-core kernel is already bound by
// the FP64 pipe; the design goal here is to keep every SM busy (split-K for
// skinny outputs) rather than to shave memory traffic.
#include "common.cuh"

namespace sgt {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, THREADS = 256;

template <bool TA, bool TB>
__global__ void __launch_bounds__(THREADS) gemm_f64_kernel(
    int64_t M, int64_t N, int64_t K, double alpha, const double* __restrict__ A, int64_t lda,
    int64_t sA, const double* __restrict__ B, int64_t ldb, int64_t sB, double beta,
    double* __restrict__ C, int64_t ldc, int64_t sC, int splits, int64_t kchunk) {
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];

  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int64_t m0 = (int64_t)blockIdx.y * BM;
  const int64_t n0 = (int64_t)blockIdx.x * BN;
  const int64_t bz = blockIdx.z / splits;
  const int kz = blockIdx.z % splits;
  const int64_t kbeg = (int64_t)kz * kchunk;
  const int64_t kend = min(K, kbeg + kchunk);

  A += bz * sA;
  B += bz * sB;
  C += bz * sC;

  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  for (int64_t k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int idx = tid + THREADS * q;
      if (!TA) {  // A is M x K: read along k
        int mm = idx / BK, kk = idx % BK;
        int64_t gm = m0 + mm, gk = k0 + kk;
        As[kk][mm] = (gm < M && gk < kend) ? A[gm * lda + gk] : 0.0;
      } else {  // A stored K x M: read along m
        int kk = idx / BM, mm = idx % BM;
        int64_t gm = m0 + mm, gk = k0 + kk;
        As[kk][mm] = (gm < M && gk < kend) ? A[gk * lda + gm] : 0.0;
      }
      if (!TB) {  // B is K x N: read along n
        int kk = idx / BN, nn = idx % BN;
        int64_t gn = n0 + nn, gk = k0 + kk;
        Bs[kk][nn] = (gn < N && gk < kend) ? B[gk * ldb + gn] : 0.0;
      } else {  // B stored N x K: read along k
        int nn = idx / BK, kk = idx % BK;
        int64_t gn = n0 + nn, gk = k0 + kk;
        Bs[kk][nn] = (gn < N && gk < kend) ? B[gn * ldb + gk] : 0.0;
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }

#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int64_t gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int64_t gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      double* c = C + gm * ldc + gn;
      if (splits > 1) {
        atomicAdd(c, alpha * acc[i][j]);
      } else {
        *c = (beta == 0.0) ? alpha * acc[i][j] : fma(beta, *c, alpha * acc[i][j]);
      }
    }
  }
}

__global__ void scale_matrix_kernel(double* C, int64_t ldc, int64_t sC, int64_t M, int64_t N,
                                    double beta) {
  int64_t b = blockIdx.y;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M * N;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / N, c = i % N;
    double* p = C + b * sC + r * ldc + c;
    *p = (beta == 0.0) ? 0.0 : beta * *p;
  }
}

// C = alpha * sum_z P[z] + beta * C (fixed order over z: deterministic)
__global__ void splitk_reduce_kernel(const double* __restrict__ P, int splits, int64_t M, int64_t N, double alpha,
                                     double beta, double* __restrict__ C, int64_t ldc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M * N; i += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int z = 0; z < splits; ++z) acc += P[(int64_t)z * M * N + i];
    double* c = C + (i / N) * ldc + (i % N);
    *c = (beta == 0.0) ? alpha * acc : fma(beta, *c, alpha * acc);
  }
}
}  // namespace

// Deterministic split-K: the K range is cut into `splits` equal chunks (a
// multiple of the K tile), computed as one batched launch into ws (splits x
// M x N doubles) and summed in a fixed order.  Used where the output has too
// few 64 x 64 tiles to occupy the GPU's FP64 pipes (the bond-sized GEMMs of
// the mixed form and of the overlap sweep).  splits <= 1: plain gemm_f64.
int gemm_f64_splitk(cudaStream_t st, bool ta, bool tb, int64_t M, int64_t N, int64_t K, double alpha,
                    const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                    double* ws, int splits) {
  if (splits > 1 && (K % splits != 0 || (K / splits) % BK != 0)) splits = 1;
  if (splits <= 1 || M <= 0 || N <= 0)
    return gemm_f64(st, ta, tb, M, N, K, alpha, A, lda, 0, B, ldb, 0, beta, C, ldc, 0, 1, 1);
  const int64_t kc = K / splits;
  const int64_t sA = ta ? kc * lda : kc;  // K chunk z of A and B
  const int64_t sB = tb ? kc : kc * ldb;
  SGT_TRY(gemm_f64(st, ta, tb, M, N, kc, 1.0, A, lda, sA, B, ldb, sB, 0.0, ws, N, M * N, splits, 1));
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(M * N, 256), 152 * 8));
  splitk_reduce_kernel<<<g, 256, 0, st>>>(ws, splits, M, N, alpha, beta, C, ldc);
  SGT_LAUNCHED();
  return SGT_OK;
}

// number of K chunks (<= 16) that brings an M x N output to ~128 or more 64 x 64 tiles
int splitk_count(int64_t M, int64_t N, int64_t K) {
  const int64_t tiles = cdiv(M, BM) * cdiv(N, BN);
  int s = 1;
  while (s < 16 && tiles * s * 2 <= 160 && K % (2 * s) == 0 && (K / (2 * s)) % BK == 0 && K / (2 * s) >= 4 * BK)
    s *= 2;
  return s;
}

int gemm_f64(cudaStream_t st, bool ta, bool tb, int64_t M, int64_t N, int64_t K, double alpha,
             const double* A, int64_t lda, int64_t sA, const double* B, int64_t ldb, int64_t sB,
             double beta, double* C, int64_t ldc, int64_t sC, int64_t batch, int split_k) {
  if (M <= 0 || N <= 0 || batch <= 0) return SGT_OK;
  SGT_REQUIRE(batch <= 65535, SGT_ERR_INVALID, "gemm_f64: batch %lld too large", (long long)batch);
  if (K <= 0) {
    if (beta == 1.0) return SGT_OK;
    dim3 g((unsigned)std::min<int64_t>(cdiv(M * N, 256), 4096), (unsigned)batch);
    scale_matrix_kernel<<<g, 256, 0, st>>>(C, ldc, sC, M, N, beta);
    SGT_LAUNCHED();
    return SGT_OK;
  }
  int64_t tiles = cdiv(M, BM) * cdiv(N, BN) * batch;
  int splits = split_k;
  if (splits <= 0) {
    splits = 1;
    const int64_t target = 2 * 152;
    if (tiles < target && K >= 4 * BK * 8) {
      splits = (int)std::min<int64_t>(cdiv(target, tiles), K / (BK * 8));
      if (splits < 1) splits = 1;
    }
  }
  while (batch * splits > 65535) splits = std::max(1, splits / 2);
  int64_t kchunk = cdiv(cdiv(K, splits), BK) * BK;
  splits = (int)cdiv(K, kchunk);
  if (splits > 1 && beta != 1.0) {
    dim3 g((unsigned)std::min<int64_t>(cdiv(M * N, 256), 4096), (unsigned)batch);
    scale_matrix_kernel<<<g, 256, 0, st>>>(C, ldc, sC, M, N, beta);
    SGT_LAUNCHED();
  }
  SGT_REQUIRE(cdiv(M, BM) <= 65535, SGT_ERR_INVALID, "gemm_f64: M too large");
  dim3 grid((unsigned)cdiv(N, BN), (unsigned)cdiv(M, BM), (unsigned)(batch * splits));
#define SGT_GEMM_LAUNCH(TA_, TB_)                                                         \
  gemm_f64_kernel<TA_, TB_><<<grid, THREADS, 0, st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, \
                                                      beta, C, ldc, sC, splits, kchunk)
  if (!ta && !tb) SGT_GEMM_LAUNCH(false, false);
  else if (ta && !tb) SGT_GEMM_LAUNCH(true, false);
  else if (!ta && tb) SGT_GEMM_LAUNCH(false, true);
  else SGT_GEMM_LAUNCH(true, true);
#undef SGT_GEMM_LAUNCH
  SGT_LAUNCHED();
  return SGT_OK;
}

}  // namespace sgt
