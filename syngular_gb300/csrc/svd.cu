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

// Rotation for the pair (p, q) with a = |g_p|^2, b = |g_q|^2, c = g_p.g_q
// (identical on all lanes after the xor-shuffle reductions).  Returns whether
// to rotate, cs / sn and tau = sn / (1 + cs): rotations are applied as
// x' = x - sn (y + tau x), y' = y + sn (x - tau y) (Rutishauser), which keeps
// the pair's norm to O(sn^4) even when 1 + t^2 rounds to 1.  T = float: computed in FP32 on every lane (cheap);
// T = double: computed in FP64 on lane 0 and broadcast -- GB300 runs FP64 at a
// small fraction of its FP32 rate, so 32 redundant lanes would dominate.
template <typename T>
__device__ __forceinline__ bool jacobi_rotation(T a, T b, T c, double tol, double abs_floor, int lane,
                                                T& cs_, T& sn, T& tau) {
  if (sizeof(T) == 4) {
    const float fa = (float)a, fb = (float)b, fc = (float)c;
    if (!(fabsf(fc) > (float)tol * sqrtf(fa) * sqrtf(fb) && fabsf(fc) > (float)abs_floor)) return false;
    const float zeta = (fb - fa) / (2.f * fc);
    const float t = copysignf(1.f, zeta) / (fabsf(zeta) + sqrtf(fmaf(zeta, zeta, 1.f)));
    const float cf = 1.f / sqrtf(fmaf(t, t, 1.f));
    cs_ = (T)cf;
    sn = (T)(cf * t);
    tau = (T)(sn / (1.f + cf));
    return true;
  } else {
    int rot = 0;
    double cd = 1.0, sd = 0.0;
    if (lane == 0) {
      const double da = (double)a, db = (double)b, dc = (double)c;
      if (fabs(dc) > tol * sqrt(da * db) && fabs(dc) > abs_floor) {
        rot = 1;
        const double zeta = (db - da) / (2.0 * dc);
        const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(fma(zeta, zeta, 1.0)));
        cd = 1.0 / sqrt(fma(t, t, 1.0));
        sd = cd * t;
      }
    }
    rot = __shfl_sync(0xffffffffu, rot, 0);
    if (!rot) return false;
    cs_ = (T)__shfl_sync(0xffffffffu, cd, 0);
    sn = (T)__shfl_sync(0xffffffffu, sd, 0);
    tau = (T)(sn / (T(1) + cs_));
    return true;
  }
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
        T cs_, sn, tau;
        if (jacobi_rotation<T>(a, b, c, tol, 0.0, lane, cs_, sn, tau)) {
          ++my_rot;
          for (int64_t e = lane; e < m; e += 32) {
            T x = gp[e], y = gq[e];
            gp[e] = x - sn * (y + tau * x);
            gq[e] = y + sn * (x - tau * y);
          }
          T* vp = Vt + (int64_t)p * ldv;
          T* vq = Vt + (int64_t)q * ldv;
          for (int e = lane; e < n; e += 32) {
            T x = vp[e], y = vq[e];
            vp[e] = x - sn * (y + tau * x);
            vq[e] = y + sn * (x - tau * y);
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

// ---------------------------------------------------------------------------
// Cluster-resident block Jacobi.  The rows are cut into 2*CS blocks of bs rows;
// CTA c of a CS-CTA cluster holds two of them ("slots") in shared memory,
// together with their Vt rows when vt_smem (else Vt stays in global memory,
// addressed by global row).  An outer step orthogonalises every pair of the
// 2*bs local rows (round-robin sub-steps, one warp per pair, warp-shuffle dot
// products, __syncthreads between sub-steps); then the blocks move one
// position along the circle tournament of blocks through DSMEM (source slot 0
// staged in local shared memory, slot 1 in registers, one cluster barrier
// between the remote reads and the local writes).  2*CS-1 outer steps pair
// every two blocks once: one outer sweep.  Rotations whose |g_p.g_q| lies
// below m*(eps*|G|_F)^2 are skipped: such pairs are numerically zero columns
// that FP rounding would otherwise keep re-rotating.
constexpr int BJ_MAX_SLOT_BYTES = 64 * 1024;
constexpr int BJ_THREADS = 512;  // 16 warps: one warp per pair of a sub-step (bs = 16)
constexpr int BJ_WARPS = BJ_THREADS / 32;

template <typename T>
__global__ void __launch_bounds__(BJ_THREADS) bjacobi_kernel(T* __restrict__ G, int64_t ldg,
                                                              T* __restrict__ Vt, int64_t ldv, int n,
                                                              int m, int bs, int vt_smem, double tol,
                                                              T* __restrict__ norms,
                                                              int* __restrict__ status) {
  cg::cluster_group cluster = cg::this_cluster();
  const int cs = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nblk = 2 * cs;
  const int vlen = vt_smem ? n : 0;
  const int row_len = m + vlen;  // elements per slot row: G part then Vt part
  const int slot_elems = bs * row_len;

  extern __shared__ __align__(16) unsigned char bj_raw[];
  T* slots = reinterpret_cast<T*>(bj_raw);  // [2][bs][row_len]
  T* stage = slots + 2 * slot_elems;        // [bs][row_len]
  __shared__ int s_blk[2];
  __shared__ int s_rot[2];
  __shared__ double s_norm;

  auto pos_owner = [&](int q, int& cta, int& slot) {
    if (q < cs) {
      cta = q;
      slot = 0;
    } else {
      cta = nblk - 1 - q;
      slot = 1;
    }
  };
  auto slot_pos = [&](int c, int slot) { return slot == 0 ? c : nblk - 1 - c; };

  // load the two initial blocks (block b at position b)
  for (int sl = 0; sl < 2; ++sl) {
    const int blk = slot_pos(rank, sl);
    if (tid == 0) s_blk[sl] = blk;
    for (int64_t i = tid; i < slot_elems; i += BJ_THREADS) {
      const int r = (int)(i / row_len), e = (int)(i % row_len);
      const int gr = blk * bs + r;
      T v = T(0);
      if (gr < n) v = (e < m) ? G[(int64_t)gr * ldg + e] : ((e - m) == gr ? T(1) : T(0));
      slots[(int64_t)sl * slot_elems + i] = v;
    }
  }
  if (!vt_smem) {
    for (int64_t i = tid; i < (int64_t)n * n; i += BJ_THREADS) {
      // Vt = I in global memory; each CTA initialises its own rows
      const int r = (int)(i / n), c = (int)(i % n);
      const int b = r / bs;
      if (b == slot_pos(rank, 0) || b == slot_pos(rank, 1)) Vt[(int64_t)r * ldv + c] = (r == c) ? T(1) : T(0);
    }
  }
  if (!vt_smem) __threadfence();
  // |G|_F^2 over the cluster
  {
    double acc = 0.0;
    for (int64_t i = tid; i < 2 * (int64_t)slot_elems; i += BJ_THREADS) {
      const int e = (int)(i % row_len);
      if (e < m) {
        const double v = (double)slots[i];
        acc += v * v;
      }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double s_red[BJ_WARPS];
    if (lane == 0) s_red[warp] = acc;
    if (tid < 2) s_rot[tid] = 0;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < BJ_WARPS; ++w) t += s_red[w];
      s_norm = t;
    }
    cluster.sync();
    if (tid == 0) {
      double t = 0.0;
      for (int r = 0; r < cs; ++r) t += *cluster.map_shared_rank(&s_norm, r);
      s_red[0] = t;
    }
    __syncthreads();
    const double eps = (sizeof(T) == 8) ? 2.220446049250313e-16 : 1.1920928955078125e-07;
    const double fl = eps * sqrt(s_red[0]);
    cluster.sync();  // everyone has read s_norm before it is reused
    if (tid == 0) s_norm = (double)m * fl * fl;
    __syncthreads();
  }
  const double abs_floor = s_norm;

  const int W = 2 * bs;  // rows in the working set
  int sweeps = 0;
  bool converged = (n < 2);
  while (!converged && sweeps < JAC_MAX_SWEEPS) {
    const int par = sweeps & 1;
    int my_rot = 0;
    for (int step = 0; step < nblk - 1; ++step) {
      // ---- all pairs of the 2*bs local rows ----
      for (int sub = 0; sub < W - 1; ++sub) {
        for (int i = warp; i < bs; i += BJ_WARPS) {
          int p = rr_index(i, sub, W), q = rr_index(W - 1 - i, sub, W);
          const int gp = s_blk[p / bs] * bs + (p % bs), gq = s_blk[q / bs] * bs + (q % bs);
          if (gp >= n || gq >= n) continue;
          T* rp = slots + (int64_t)(p / bs) * slot_elems + (int64_t)(p % bs) * row_len;
          T* rq = slots + (int64_t)(q / bs) * slot_elems + (int64_t)(q % bs) * row_len;
          T a = 0, b = 0, c = 0;
          for (int e = lane; e < m; e += 32) {
            const T x = rp[e], y = rq[e];
            a = fma(x, x, a);
            b = fma(y, y, b);
            c = fma(x, y, c);
          }
          a = wsum_t(a);
          b = wsum_t(b);
          c = wsum_t(c);
          T cs_, sn, tau;
          if (jacobi_rotation<T>(a, b, c, tol, abs_floor, lane, cs_, sn, tau)) {
            ++my_rot;
            for (int e = lane; e < m; e += 32) {
              const T x = rp[e], y = rq[e];
              rp[e] = x - sn * (y + tau * x);
              rq[e] = y + sn * (x - tau * y);
            }
            T* vp = vt_smem ? rp + m : Vt + (int64_t)gp * ldv;
            T* vq = vt_smem ? rq + m : Vt + (int64_t)gq * ldv;
            for (int e = lane; e < n; e += 32) {
              const T x = vp[e], y = vq[e];
              vp[e] = x - sn * (y + tau * x);
              vq[e] = y + sn * (x - tau * y);
            }
          }
        }
        __syncthreads();
      }
      // ---- move blocks one position along the circle ----
      int src_cta[2], src_slot[2];
      for (int sl = 0; sl < 2; ++sl) {
        const int q = slot_pos(rank, sl);
        const int qs = (q == 0) ? 0 : (q == 1 ? nblk - 1 : q - 1);
        pos_owner(qs, src_cta[sl], src_slot[sl]);
      }
      if (!vt_smem) __threadfence();
      cluster.sync();
      // slot 0's incoming block -> stage (shared), slot 1's -> registers
      const T* r0 = cluster.map_shared_rank(slots, src_cta[0]) + (int64_t)src_slot[0] * slot_elems;
      const T* r1 = cluster.map_shared_rank(slots, src_cta[1]) + (int64_t)src_slot[1] * slot_elems;
      const int nb0 = *cluster.map_shared_rank(&s_blk[src_slot[0]], src_cta[0]);
      const int nb1 = *cluster.map_shared_rank(&s_blk[src_slot[1]], src_cta[1]);
      const int n4 = slot_elems * (int)sizeof(T) / 16;  // uint4 chunks per slot
      const uint4* s0 = reinterpret_cast<const uint4*>(r0);
      const uint4* s1 = reinterpret_cast<const uint4*>(r1);
      uint4* st4 = reinterpret_cast<uint4*>(stage);
      uint4 regs[BJ_MAX_SLOT_BYTES / 16 / BJ_THREADS];
#pragma unroll
      for (int j = 0; j < BJ_MAX_SLOT_BYTES / 16 / BJ_THREADS; ++j) {
        const int idx = tid + j * BJ_THREADS;
        if (idx < n4) {
          st4[idx] = s0[idx];
          regs[j] = s1[idx];
        }
      }
      cluster.sync();
      uint4* d0 = reinterpret_cast<uint4*>(slots);
      uint4* d1 = reinterpret_cast<uint4*>(slots + slot_elems);
#pragma unroll
      for (int j = 0; j < BJ_MAX_SLOT_BYTES / 16 / BJ_THREADS; ++j) {
        const int idx = tid + j * BJ_THREADS;
        if (idx < n4) {
          d0[idx] = st4[idx];
          d1[idx] = regs[j];
        }
      }
      if (tid == 0) {
        s_blk[0] = nb0;
        s_blk[1] = nb1;
      }
      __syncthreads();
    }
    if (lane == 0 && my_rot) atomicAdd(&s_rot[par], my_rot);
    __syncthreads();
    cluster.sync();
    int total = 0;
    for (int r = 0; r < cs; ++r) total += *cluster.map_shared_rank(&s_rot[par], r);
    ++sweeps;
    converged = (total == 0);
    cluster.sync();
    if (tid == 0) s_rot[par] = 0;
  }
  // write back (blocks are back at their initial positions only after whole
  // sweeps, so use the recorded block ids) and row norms
  for (int sl = 0; sl < 2; ++sl) {
    const int blk = s_blk[sl];
    for (int64_t i = tid; i < slot_elems; i += BJ_THREADS) {
      const int r = (int)(i / row_len), e = (int)(i % row_len);
      const int gr = blk * bs + r;
      if (gr >= n) continue;
      const T v = slots[(int64_t)sl * slot_elems + i];
      if (e < m) G[(int64_t)gr * ldg + e] = v;
      else Vt[(int64_t)gr * ldv + (e - m)] = v;
    }
    for (int r = warp; r < bs; r += BJ_WARPS) {
      const int gr = blk * bs + r;
      if (gr >= n) continue;
      const T* row = slots + (int64_t)sl * slot_elems + (int64_t)r * row_len;
      T acc = 0;
      for (int e = lane; e < m; e += 32) acc = fma(row[e], row[e], acc);
      acc = wsum_t(acc);
      if (lane == 0) norms[gr] = sqrt(acc);
    }
  }
  if (rank == 0 && tid == 0 && status) *status = converged ? sweeps : -1;
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

// Convergence threshold on |g_p.g_q| / (|g_p| |g_q|): a few times the rounding
// noise of an m-term dot product, so that noise alone does not keep pairs
// rotating (FP64: 4 eps sqrt(m); FP32: 8 eps sqrt(m)).
template <typename T>
double jacobi_tol(int64_t m) {
  const double eps = (sizeof(T) == 8) ? DBL_EPSILON : (double)FLT_EPSILON;
  const double k = (sizeof(T) == 8) ? 4.0 : 8.0;
  return k * eps * sqrt((double)std::max<int64_t>(m, 1));
}

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

  // cluster-resident block Jacobi when a cluster of up to 16 CTAs can hold
  // the rows (G, and Vt too when it fits), else the L2-resident kernel below
  if (n >= 64 && m <= 4096) {
    int csb = 2;
    while (csb < 16 && csb * 2 * 32 <= n) csb *= 2;  // about 16 rows per block
    for (int vt_smem = 1; vt_smem >= 0; --vt_smem) {
      const int64_t bsz = cdiv(n, 2 * csb);
      const int64_t slot_bytes = bsz * (m + (vt_smem ? n : 0)) * (int64_t)sizeof(T);
      if (slot_bytes > BJ_MAX_SLOT_BYTES || slot_bytes % 16 != 0) continue;
      static bool attr_done[2] = {false, false};
      auto kern = bjacobi_kernel<T>;
      if (!attr_done[sizeof(T) == 8]) {
        SGT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        SGT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      3 * BJ_MAX_SLOT_BYTES));
        attr_done[sizeof(T) == 8] = true;
      }
      const double tolb = jacobi_tol<T>(m);
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(csb, 1, 1);
      cfg.blockDim = dim3(BJ_THREADS, 1, 1);
      cfg.dynamicSmemBytes = (size_t)3 * slot_bytes;
      cfg.stream = st;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = csb;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      int clusters = 0;
      if (cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg) != cudaSuccess || clusters < 1) {
        cudaGetLastError();  // not schedulable here: use the other kernel
        break;
      }
      SGT_CUDA(cudaLaunchKernelEx(&cfg, kern, G, ldg, Vt, ldv, (int)n, (int)m, (int)bsz, vt_smem, tolb, norms,
                                  status));
      note_launch();
      goto sort;
    }
  }
  {
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
  const double tol = jacobi_tol<T>(m);
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
  }
sort:

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
