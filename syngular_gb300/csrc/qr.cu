// Blocked Householder QR in FP64 (right-looking, compact WY).
//
// Row-major A (m x n).  For every panel of up to NB columns:
//   1. panel_kernel factors the panel with a cluster of CS CTAs: the panel
//      rows are split over the CTAs, each column needs two cluster-wide
//      reductions (column norm, then v^T A for the remaining panel columns),
//      exchanged through distributed shared memory between hardware cluster
//      barriers.  It also writes the explicit unit-lower-trapezoidal V.
//   2. T (block reflector H_1...H_jb = I - V T V^T) from G = V^T V.
//   3. trailing update A2 <- A2 - V ((V T)^T A2) with the FP64 GEMM.
// The reflectors stay in A below the diagonal (LAPACK dgeqrf layout, with
// the same sign convention beta = -sign(alpha) * norm), tau holds the
// scalars and Tbuf the per-panel T factors, so Q can be applied or formed
// later without recomputation.
#include <cooperative_groups.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace sgt {

constexpr int QR_NB = 32;
constexpr int QR_THREADS = 256;
constexpr int QR_WARPS = QR_THREADS / 32;

namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One cluster factors rows [j0, m) x columns [j0, j0+jb) of A.
__global__ void __launch_bounds__(QR_THREADS) panel_kernel(double* __restrict__ A, int64_t m,
                                                           int64_t lda, int64_t j0, int jb,
                                                           double* __restrict__ tau,
                                                           double* __restrict__ Vbuf) {
  cg::cluster_group cluster = cg::this_cluster();
  const int cs = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  __shared__ double s_warp[QR_WARPS][QR_NB];
  __shared__ double s_part[QR_NB];  // this CTA's partial sums, read by the whole cluster
  __shared__ double s_bcast[4];

  const int64_t mr = m - j0;
  const int64_t chunk = (mr + cs - 1) / cs;
  const int64_t lo = j0 + rank * chunk;
  const int64_t hi = min(m, lo + chunk);

  for (int j = 0; j < jb; ++j) {
    const int64_t col = j0 + j;
    const int64_t drow = j0 + j;  // diagonal row
    // (a) partial sum of squares below the diagonal
    double acc = 0.0;
    for (int64_t g = lo + tid; g < hi; g += QR_THREADS) {
      if (g > drow) {
        double x = A[g * lda + col];
        acc = fma(x, x, acc);
      }
    }
    acc = warp_sum(acc);
    if (lane == 0) s_warp[warp][0] = acc;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < QR_WARPS; ++w) t += s_warp[w][0];
      s_part[0] = t;
    }
    cluster.sync();
    if (tid == 0) {
      double sigma = 0.0;
      for (int r = 0; r < cs; ++r) sigma += cluster.map_shared_rank(s_part, r)[0];
      double alpha = A[drow * lda + col];
      double t = 0.0, beta = alpha, scale = 0.0;
      if (sigma > 0.0) {
        double nrm = sqrt(fma(alpha, alpha, sigma));
        beta = (alpha >= 0.0) ? -nrm : nrm;
        t = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
      }
      s_bcast[0] = t;
      s_bcast[1] = beta;
      s_bcast[2] = scale;
    }
    __syncthreads();
    const double t = s_bcast[0], beta = s_bcast[1], scale = s_bcast[2];

    // (d) scale own sub-diagonal rows into v, partial w_c = sum v_g A[g, c]
    double wc[QR_NB];
#pragma unroll
    for (int c = 0; c < QR_NB; ++c) wc[c] = 0.0;
    if (t != 0.0) {
      for (int64_t g = lo + tid; g < hi; g += QR_THREADS) {
        double* row = A + g * lda + j0;
        if (g > drow) {
          double v = row[j] * scale;
          row[j] = v;
#pragma unroll
          for (int c = 0; c < QR_NB; ++c)
            if (c > j && c < jb) wc[c] = fma(v, row[c], wc[c]);
        } else if (g == drow) {  // the diagonal row contributes v = 1
#pragma unroll
          for (int c = 0; c < QR_NB; ++c)
            if (c > j && c < jb) wc[c] += row[c];
        }
      }
    }
#pragma unroll
    for (int c = 0; c < QR_NB; ++c) {
      double v = warp_sum(wc[c]);
      if (lane == 0) s_warp[warp][c] = v;
    }
    __syncthreads();
    if (tid < QR_NB) {
      double v = 0.0;
      for (int w = 0; w < QR_WARPS; ++w) v += s_warp[w][tid];
      s_part[tid] = v;
    }
    cluster.sync();
    if (tid < QR_NB) {
      double v = 0.0;
      for (int r = 0; r < cs; ++r) v += cluster.map_shared_rank(s_part, r)[tid];
      s_warp[0][tid] = v;  // reuse as the broadcast of w
    }
    __syncthreads();
    if (t != 0.0) {
      for (int64_t g = lo + tid; g < hi; g += QR_THREADS) {
        double* row = A + g * lda + j0;
        if (g > drow) {
          double tv = t * row[j];
          for (int c = j + 1; c < jb; ++c) row[c] = fma(-tv, s_warp[0][c], row[c]);
        } else if (g == drow) {
          for (int c = j + 1; c < jb; ++c) row[c] = fma(-t, s_warp[0][c], row[c]);
        }
      }
    }
    if (tid == 0 && drow >= lo && drow < hi) {
      A[drow * lda + col] = beta;
      tau[col] = t;
    }
    // s_warp[0][*] and s_part are rewritten in the next column only after
    // this CTA passes the next cluster barrier, which every CTA reaches only
    // after finishing the reads above.
    __syncthreads();
  }
  // explicit V for the trailing update (own rows only)
  for (int64_t g = lo + tid; g < hi; g += QR_THREADS) {
    const int64_t rr = g - j0;
    const double* row = A + g * lda + j0;
    for (int c = 0; c < jb; ++c) Vbuf[rr * jb + c] = (rr == c) ? 1.0 : (rr > c ? row[c] : 0.0);
  }
}

// T from G = V^T V and tau: T[q][q] = tau_q, T[0:q, q] = -tau_q T[0:q,0:q] G[0:q, q].
// One warp; jb <= 32.
__global__ void build_t_kernel(const double* __restrict__ G, const double* __restrict__ tau, int jb,
                               double* __restrict__ T) {
  __shared__ double sT[QR_NB][QR_NB];
  const int lane = threadIdx.x;
  for (int i = lane; i < QR_NB * QR_NB; i += 32) sT[i / QR_NB][i % QR_NB] = 0.0;
  __syncwarp();
  for (int q = 0; q < jb; ++q) {
    double tq = tau[q];
    double v = 0.0;
    if (lane < q) {
      for (int k = lane; k < q; ++k) v = fma(sT[lane][k], G[k * jb + q], v);
      v = -tq * v;
    }
    __syncwarp();
    if (lane < q) sT[lane][q] = v;
    if (lane == 0) sT[q][q] = tq;
    __syncwarp();
  }
  for (int i = lane; i < jb * jb; i += 32) T[i] = sT[i / jb][i % jb];
}

// Explicit V of panel [j0, j0+jb) from the factored A.
__global__ void extract_v_kernel(const double* __restrict__ A, int64_t m, int64_t lda, int64_t j0,
                                 int jb, double* __restrict__ V) {
  const int64_t mr = m - j0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < mr * jb;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t rr = i / jb;
    int c = (int)(i % jb);
    V[i] = (rr == c) ? 1.0 : (rr > c ? A[(j0 + rr) * lda + j0 + c] : 0.0);
  }
}

__global__ void extract_r_kernel(const double* __restrict__ A, int64_t m, int64_t n, int64_t lda,
                                 double* __restrict__ R, int64_t ldr, int64_t rows) {
  const int64_t k = min(m, n);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows * n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / n, c = i % n;
    R[r * ldr + c] = (r < k && c >= r) ? A[r * lda + c] : 0.0;
  }
}

__global__ void eye_kernel(double* Q, int64_t ldq, int64_t m, int64_t keep) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m * keep;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / keep, c = i % keep;
    Q[r * ldq + c] = (r == c) ? 1.0 : 0.0;
  }
}

inline unsigned grid1d(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(n, 256), 152 * 8));
}

int launch_panel(cudaStream_t st, double* A, int64_t m, int64_t lda, int64_t j0, int jb, double* tau,
                 double* Vbuf) {
  const int64_t mr = m - j0;
  int cs = 1;
  if (mr >= 2048) cs = 8;
  else if (mr >= 1024) cs = 4;
  else if (mr >= 512) cs = 2;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cs, 1, 1);
  cfg.blockDim = dim3(QR_THREADS, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  SGT_CUDA(cudaLaunchKernelEx(&cfg, panel_kernel, A, m, lda, j0, jb, tau, Vbuf));
  note_launch();
  return SGT_OK;
}

}  // namespace

size_t qr_tbuf_count(int64_t m, int64_t n) {
  int64_t k = std::min(m, n);
  return (size_t)cdiv(k, QR_NB) * QR_NB * QR_NB;
}

// Scratch of qr_factor besides Tbuf: V (m x NB), G (NB x NB), Y (m x NB), W (NB x n).
static void qr_scratch(Arena& ar, int64_t m, int64_t n, double** V, double** G, double** Y,
                       double** W) {
  *V = ar.take<double>((size_t)m * QR_NB);
  *G = ar.take<double>(QR_NB * QR_NB);
  *Y = ar.take<double>((size_t)m * QR_NB);
  *W = ar.take<double>((size_t)QR_NB * std::max<int64_t>(n, 1));
}

size_t qr_ws_bytes(int64_t m, int64_t n) {
  Arena a = Arena::measuring();
  double *V, *G, *Y, *W;
  qr_scratch(a, m, n, &V, &G, &Y, &W);
  a.take<double>(qr_tbuf_count(m, n));
  return a.used;
}

int qr_factor_t(cudaStream_t st, double* A, int64_t m, int64_t n, int64_t lda, double* tau,
                double* Tbuf, Arena& ar) {
  const int64_t k = std::min(m, n);
  if (k <= 0) return SGT_OK;
  double *V, *G, *Y, *W;
  qr_scratch(ar, m, n, &V, &G, &Y, &W);
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "qr: workspace too small");
  for (int64_t j0 = 0; j0 < k; j0 += QR_NB) {
    const int jb = (int)std::min<int64_t>(QR_NB, k - j0);
    const int64_t mr = m - j0;
    SGT_TRY(launch_panel(st, A, m, lda, j0, jb, tau, V));
    double* T = Tbuf + (j0 / QR_NB) * QR_NB * QR_NB;
    // G = V^T V
    SGT_TRY(gemm_f64(st, true, false, jb, jb, mr, 1.0, V, jb, 0, V, jb, 0, 0.0, G, jb, 0, 1));
    build_t_kernel<<<1, 32, 0, st>>>(G, tau + j0, jb, T);
    SGT_LAUNCHED();
    const int64_t nc = n - j0 - jb;
    if (nc > 0) {
      double* A2 = A + j0 * lda + j0 + jb;
      // Y = V T (mr x jb); W = Y^T A2 (jb x nc); A2 -= V W
      SGT_TRY(gemm_f64(st, false, false, mr, jb, jb, 1.0, V, jb, 0, T, jb, 0, 0.0, Y, jb, 0, 1));
      SGT_TRY(gemm_f64(st, true, false, jb, nc, mr, 1.0, Y, jb, 0, A2, lda, 0, 0.0, W, nc, 0, 1));
      SGT_TRY(gemm_f64(st, false, false, mr, nc, jb, -1.0, V, jb, 0, W, nc, 0, 1.0, A2, lda, 0, 1));
    }
  }
  return SGT_OK;
}

int qr_factor(cudaStream_t st, double* A, int64_t m, int64_t n, int64_t lda, double* tau, Arena& ar) {
  double* Tbuf = ar.take<double>(qr_tbuf_count(m, n));
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "qr: workspace too small");
  return qr_factor_t(st, A, m, n, lda, tau, Tbuf, ar);
}

// C (rows m x c, ldc) <- Q C  (trans=false)  or  Q^T C (trans=true), Q = H_1 ... H_k.
int qr_apply_q(cudaStream_t st, const double* A, int64_t m, int64_t n, int64_t lda,
               const double* Tbuf, double* C, int64_t ldc, int64_t c, bool trans, Arena& ar) {
  const int64_t k = std::min(m, n);
  if (k <= 0 || c <= 0) return SGT_OK;
  double* V = ar.take<double>((size_t)m * QR_NB);
  double* W = ar.take<double>((size_t)QR_NB * c);
  double* W2 = ar.take<double>((size_t)QR_NB * c);
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "qr_apply_q: workspace too small");
  const int64_t nblk = cdiv(k, QR_NB);
  for (int64_t bi = 0; bi < nblk; ++bi) {
    // Q C applies blocks last-to-first; Q^T C first-to-last.
    const int64_t b = trans ? bi : nblk - 1 - bi;
    const int64_t j0 = b * QR_NB;
    const int jb = (int)std::min<int64_t>(QR_NB, k - j0);
    const int64_t mr = m - j0;
    extract_v_kernel<<<grid1d(mr * jb), 256, 0, st>>>(A, m, lda, j0, jb, V);
    SGT_LAUNCHED();
    const double* T = Tbuf + b * QR_NB * QR_NB;
    double* Cs = C + j0 * ldc;
    // W = V^T Cs (jb x c); W2 = op(T) W; Cs -= V W2   with op(T) = T for Q, T^T for Q^T
    SGT_TRY(gemm_f64(st, true, false, jb, c, mr, 1.0, V, jb, 0, Cs, ldc, 0, 0.0, W, c, 0, 1));
    SGT_TRY(gemm_f64(st, trans, false, jb, c, jb, 1.0, T, jb, 0, W, c, 0, 0.0, W2, c, 0, 1));
    SGT_TRY(gemm_f64(st, false, false, mr, c, jb, -1.0, V, jb, 0, W2, c, 0, 1.0, Cs, ldc, 0, 1));
  }
  return SGT_OK;
}

size_t formq_ws_bytes(int64_t m, int64_t n, int64_t keep) {
  Arena a = Arena::measuring();
  a.take<double>((size_t)m * QR_NB);
  a.take<double>((size_t)QR_NB * keep);
  a.take<double>((size_t)QR_NB * keep);
  return a.used;
}

int qr_form_q_t(cudaStream_t st, const double* A, int64_t m, int64_t n, int64_t lda,
                const double* Tbuf, double* Q, int64_t ldq, int64_t keep, Arena& ar) {
  SGT_REQUIRE(keep <= m, SGT_ERR_SHAPE, "qr_form_q: keep %lld > m %lld", (long long)keep,
              (long long)m);
  if (keep <= 0) return SGT_OK;
  eye_kernel<<<grid1d(m * keep), 256, 0, st>>>(Q, ldq, m, keep);
  SGT_LAUNCHED();
  return qr_apply_q(st, A, m, n, lda, Tbuf, Q, ldq, keep, false, ar);
}

int qr_extract_r(cudaStream_t st, const double* A, int64_t m, int64_t n, int64_t lda, double* R,
                 int64_t ldr, int64_t rows) {
  if (rows <= 0 || n <= 0) return SGT_OK;
  extract_r_kernel<<<grid1d(rows * n), 256, 0, st>>>(A, m, n, lda, R, ldr, rows);
  SGT_LAUNCHED();
  return SGT_OK;
}

int eye_f64(cudaStream_t st, double* Q, int64_t ldq, int64_t m, int64_t keep) {
  if (m * keep <= 0) return SGT_OK;
  eye_kernel<<<grid1d(m * keep), 256, 0, st>>>(Q, ldq, m, keep);
  SGT_LAUNCHED();
  return SGT_OK;
}

}  // namespace sgt
