// One-sided (Hestenes) Jacobi SVD in FP64.
//
// The matrix is held "columns as rows": G (n x m, row-major) where row j is
// column j of A (m x n).  Rotating rows p, q of G orthogonalises columns p, q
// of A; the same rotation is applied to rows of Vt, initialised to I, so on
// convergence G = (A V)^T and Vt = V^T.
//
// Parallel ordering: the round-robin (circle) tournament gives n/2 disjoint
// pairs per step and covers every pair once per sweep of n-1 steps.  A
// cluster of CTAs shares the pairs of a step (one warp per pair, column dot
// products reduced with warp shuffles) and meets at a hardware cluster
// barrier between steps.  Sweeps stop when no pair needed a rotation, or at
// the sweep cap, in which case the status word reports -1 instead of the
// number of sweeps; no wait in this file can spin without bound.
#include <cooperative_groups.h>
#include <float.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace sgt {

constexpr int JAC_THREADS = 256;
constexpr int JAC_WARPS = JAC_THREADS / 32;
constexpr int JAC_MAX_SWEEPS = 60;

namespace {

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ int rr_index(int i, int s, int np) {
  // circle method: position 0 fixed, the others rotate by s
  return i == 0 ? 0 : ((i - 1 + s) % (np - 1)) + 1;
}

template <typename T>
__device__ __forceinline__ T wsum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// T = double: plain FP64.  T = float: the column data and dot products are
// FP32 (warp-shuffle trees); the rotation angle is still formed in FP64.
template <typename T>
__global__ void __launch_bounds__(JAC_THREADS) jacobi_kernel(T* __restrict__ G, int64_t ldg,
                                                             T* __restrict__ Vt, int64_t ldv,
                                                             int n, int64_t m, double tol,
                                                             T* __restrict__ norms,
                                                             int* __restrict__ status) {
  cg::cluster_group cluster = cg::this_cluster();
  const int cs = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gw = rank * JAC_WARPS + warp;
  const int nw = cs * JAC_WARPS;
  const int np = n + (n & 1);
  const int npairs = np / 2;

  __shared__ int s_rot[2];
  if (threadIdx.x < 2) s_rot[threadIdx.x] = 0;
  cluster.sync();

  int sweeps = 0;
  bool converged = (n < 2);
  while (!converged && sweeps < JAC_MAX_SWEEPS) {
    const int par = sweeps & 1;
    int my_rot = 0;
    for (int s = 0; s < np - 1; ++s) {
      for (int i = gw; i < npairs; i += nw) {
        int p = rr_index(i, s, np), q = rr_index(np - 1 - i, s, np);
        if (p >= n || q >= n) continue;
        if (p > q) {
          int t = p;
          p = q;
          q = t;
        }
        T* gp = G + (int64_t)p * ldg;
        T* gq = G + (int64_t)q * ldg;
        T a = 0, b = 0, c = 0;
        for (int64_t e = lane; e < m; e += 32) {
          T x = gp[e], y = gq[e];
          a = fma(x, x, a);
          b = fma(y, y, b);
          c = fma(x, y, c);
        }
        a = wsum_t(a);
        b = wsum_t(b);
        c = wsum_t(c);
        const double da = (double)a, db = (double)b, dc = (double)c;
        if (dc != 0.0 && fabs(dc) > tol * sqrt(da) * sqrt(db)) {
          ++my_rot;
          double zeta = (db - da) / (2.0 * dc);
          double t = copysign(1.0, zeta) / (fabs(zeta) + hypot(1.0, zeta));
          double cd = 1.0 / sqrt(fma(t, t, 1.0));
          const T cs_ = (T)cd, sn = (T)(cd * t);
          for (int64_t e = lane; e < m; e += 32) {
            T x = gp[e], y = gq[e];
            gp[e] = cs_ * x - sn * y;
            gq[e] = sn * x + cs_ * y;
          }
          T* vp = Vt + (int64_t)p * ldv;
          T* vq = Vt + (int64_t)q * ldv;
          for (int e = lane; e < n; e += 32) {
            T x = vp[e], y = vq[e];
            vp[e] = cs_ * x - sn * y;
            vq[e] = sn * x + cs_ * y;
          }
        }
      }
      __threadfence();
      cluster.sync();
    }
    if (lane == 0 && my_rot) atomicAdd(&s_rot[par], my_rot);
    __syncthreads();
    cluster.sync();
    int total = 0;
    for (int r = 0; r < cs; ++r) total += *cluster.map_shared_rank(&s_rot[par], r);
    ++sweeps;
    converged = (total == 0);
    // everyone has read s_rot[par]; the next sweep uses the other slot, and
    // this one is cleared before it is used again two sweeps later
    cluster.sync();
    if (threadIdx.x == 0) s_rot[par] = 0;
  }
  // row norms = singular values
  for (int j = gw; j < n; j += nw) {
    const T* gj = G + (int64_t)j * ldg;
    T a = 0;
    for (int64_t e = lane; e < m; e += 32) a = fma(gj[e], gj[e], a);
    a = wsum_t(a);
    if (lane == 0) norms[j] = sqrt(a);
  }
  if (rank == 0 && threadIdx.x == 0 && status) *status = converged ? sweeps : -1;
  cluster.sync();
}

template <typename T>
__global__ void eye_rows_kernel(T* Vt, int64_t ldv, int n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)n * n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / n, c = i % n;
    Vt[r * ldv + c] = (r == c) ? T(1) : T(0);
  }
}

// perm[j] = position of row j in descending order of norms (ties by index).
template <typename T>
__global__ void rank_kernel(const T* __restrict__ norms, int n, int* __restrict__ perm) {
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    T v = norms[j];
    int r = 0;
    for (int i = 0; i < n; ++i) {
      T w = norms[i];
      r += (w > v) || (w == v && i < j);
    }
    perm[j] = r;
  }
}

template <typename T>
__global__ void permute_rows_kernel(const T* __restrict__ src, int64_t lds, T* __restrict__ dst,
                                    int64_t ldd, int64_t cols, const int* __restrict__ perm, int n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)n * cols;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i / cols, c = i % cols;
    dst[(int64_t)perm[r] * ldd + c] = src[r * lds + c];
  }
}

template <typename T>
__global__ void permute_vec_kernel(const T* __restrict__ src, T* __restrict__ dst,
                                   const int* __restrict__ perm, int n) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
    dst[perm[j]] = src[j];
}

inline unsigned g1(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(n, 256), 152 * 8));
}

}  // namespace

template <typename T>
size_t jacobi_rows_ws_bytes_t(int64_t n, int64_t m) {
  Arena a = Arena::measuring();
  a.take<T>((size_t)n * m);
  a.take<T>((size_t)n * n);
  a.take<T>((size_t)n);
  a.take<int>((size_t)n);
  return a.used;
}

size_t jacobi_rows_ws_bytes(int64_t n, int64_t m) { return jacobi_rows_ws_bytes_t<double>(n, m); }
size_t jacobi_rows_ws_bytes_f32(int64_t n, int64_t m) { return jacobi_rows_ws_bytes_t<float>(n, m); }

// Orthogonalise the n rows (length m) of G; Vt (n x n) receives V^T, s the
// descending singular values, rows of G and Vt sorted accordingly.
template <typename T>
int jacobi_rows_t(cudaStream_t st, T* G, int64_t ldg, int64_t n, int64_t m, T* Vt, int64_t ldv, T* s,
                  int* status, Arena& ar) {
  if (n <= 0) return SGT_OK;
  SGT_REQUIRE(n <= (1 << 20), SGT_ERR_INVALID, "jacobi: n too large");
  T* Gtmp = ar.take<T>((size_t)n * m);
  T* Vtmp = ar.take<T>((size_t)n * n);
  T* norms = ar.take<T>((size_t)n);
  int* perm = ar.take<int>((size_t)n);
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "jacobi: workspace too small");

  eye_rows_kernel<T><<<g1(n * n), 256, 0, st>>>(Vt, ldv, (int)n);
  SGT_LAUNCHED();

  int cs = 1;
  const int64_t pairs = (n + 1) / 2;
  if (pairs >= 16 * JAC_WARPS) cs = 16;
  else if (pairs >= 8 * JAC_WARPS) cs = 8;
  else if (pairs >= 4 * JAC_WARPS) cs = 4;
  else if (pairs >= 2 * JAC_WARPS) cs = 2;
  static bool nonportable = false;
  if (!nonportable) {
    SGT_CUDA(cudaFuncSetAttribute(jacobi_kernel<double>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    SGT_CUDA(cudaFuncSetAttribute(jacobi_kernel<float>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    nonportable = true;
  }
  const double eps = (sizeof(T) == 8) ? DBL_EPSILON : (double)FLT_EPSILON;
  const double tol = eps * sqrt((double)std::max<int64_t>(m, 1));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cs, 1, 1);
  cfg.blockDim = dim3(JAC_THREADS, 1, 1);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  SGT_CUDA(cudaLaunchKernelEx(&cfg, jacobi_kernel<T>, G, ldg, Vt, ldv, (int)n, m, tol, norms, status));
  note_launch();

  rank_kernel<T><<<1, 256, 0, st>>>(norms, (int)n, perm);
  SGT_LAUNCHED();
  permute_rows_kernel<T><<<g1(n * m), 256, 0, st>>>(G, ldg, Gtmp, m, m, perm, (int)n);
  SGT_LAUNCHED();
  permute_rows_kernel<T><<<g1(n * n), 256, 0, st>>>(Vt, ldv, Vtmp, n, n, perm, (int)n);
  SGT_LAUNCHED();
  permute_vec_kernel<T><<<g1(n), 256, 0, st>>>(norms, s, perm, (int)n);
  SGT_LAUNCHED();
  SGT_CUDA(cudaMemcpy2DAsync(G, ldg * sizeof(T), Gtmp, m * sizeof(T), m * sizeof(T), n,
                             cudaMemcpyDeviceToDevice, st));
  SGT_CUDA(cudaMemcpy2DAsync(Vt, ldv * sizeof(T), Vtmp, n * sizeof(T), n * sizeof(T), n,
                             cudaMemcpyDeviceToDevice, st));
  return SGT_OK;
}

int jacobi_rows(cudaStream_t st, double* G, int64_t ldg, int64_t n, int64_t m, double* Vt,
                int64_t ldv, double* s, int* status, Arena& ar) {
  return jacobi_rows_t<double>(st, G, ldg, n, m, Vt, ldv, s, status, ar);
}

int jacobi_rows_f32(cudaStream_t st, float* G, int64_t ldg, int64_t n, int64_t m, float* Vt,
                    int64_t ldv, float* s, int* status, Arena& ar) {
  return jacobi_rows_t<float>(st, G, ldg, n, m, Vt, ldv, s, status, ar);
}

}  // namespace sgt
