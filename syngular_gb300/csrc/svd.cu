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

#include <cstdlib>
#include <vector>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace sgt {

constexpr int JAC_THREADS = 256;
constexpr int JAC_WARPS = JAC_THREADS / 32;
constexpr int JAC_MAX_SWEEPS = 60;

namespace {

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
    // zeta, t and tau only choose the angle (any value within a few ulps
    // gives a rotation that zeroes the pair to rounding level): fast
    // reciprocal divisions.  cs stays correctly rounded so that cs and sn
    // form an orthogonal pair to FP32 precision (no drift of the row norms).
    const float zeta = __fdividef(fb - fa, 2.f * fc);
    const float t = __fdividef(copysignf(1.f, zeta), fabsf(zeta) + sqrtf(fmaf(zeta, zeta, 1.f)));
    const float cf = 1.f / sqrtf(fmaf(t, t, 1.f));
    cs_ = (T)cf;
    sn = (T)(cf * t);
    tau = (T)__fdividef((float)sn, 1.f + cf);
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

// Low-latency FP32 rotation for the Gram-form kernel's inner sweep, where the
// dependent chain of one sub-step is the critical path: square roots and
// quotients from the hardware reciprocal (square root) estimates, which only
// choose the angle; cs = 1 / sqrt(1 + t^2) from the estimate plus one Newton
// step y (3/2 - u y^2 / 2), so that cs^2 (1 + t^2) = 1 to about an ulp without
// a systematic bias (a bias would drift the row norms over the thousands of
// rotations a row sees).
__device__ __forceinline__ bool rot_fast(float a, float b, float c, float tol, float abs_floor, float& cs_,
                                         float& sn, float& tau, float& tn) {
  const float sa = a * rsqrtf(a), sb = b * rsqrtf(b);  // a or b = 0: NaN, no rotation (c is 0 there)
  if (!(fabsf(c) > tol * sa * sb && fabsf(c) > abs_floor)) return false;
  const float zeta = __fdividef(b - a, 2.f * c);
  const float az = fabsf(zeta);
  const float q = fmaf(zeta, zeta, 1.f);
  const float sq = (az > 1e18f) ? az : q * rsqrtf(q);
  const float t = __fdividef(copysignf(1.f, zeta), az + sq);
  const float u = fmaf(t, t, 1.f);
  float y = rsqrtf(u);
  y = y * fmaf(-0.5f * u, y * y, 1.5f);
  cs_ = y;
  sn = y * t;
  tau = __fdividef(sn, 1.f + y);
  tn = t;
  return true;
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
  __shared__ double s_part[JAC_WARPS];
  __shared__ double s_norm;
  if (threadIdx.x < 2) s_rot[threadIdx.x] = 0;
  // n > 512: pairs with |g_p . g_q| below m (eps |G|_F)^2 are rounding noise
  // and are not rotated (on such problems rows at the noise level otherwise
  // keep rotating against each other up to the sweep cap; on smaller ones the
  // floor would stop rotations that still move the leading vectors)
  double abs_floor = 0.0;
  if (n > 512) {
    double acc = 0.0;
    for (int j = gw; j < n; j += nw) {
      const T* gj = G + (int64_t)j * ldg;
      for (int64_t e = lane; e < m; e += 32) acc += (double)gj[e] * (double)gj[e];
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) s_part[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < JAC_WARPS; ++w) t += s_part[w];
      s_norm = t;
    }
    cluster.sync();
    double tot = 0.0;
    for (int r = 0; r < cs; ++r) tot += *cluster.map_shared_rank(&s_norm, r);
    const double fl = (sizeof(T) == 4 ? (double)FLT_EPSILON : DBL_EPSILON) * sqrt(tot);
    abs_floor = (double)m * fl * fl;
  }
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
        if (jacobi_rotation<T>(a, b, c, tol, abs_floor, lane, cs_, sn, tau)) {
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

// ---------------------------------------------------------------------------
// Gram-form block Jacobi (FP32).  Same cluster layout and circle of blocks as
// bjacobi_kernel (Vt rows always in shared memory, bs <= 16), but an outer step
// touches the 2*bs working rows [G | Vt] only twice instead of once per pair:
//   1. C = G_w G_w^T, the Gram matrix of the working rows (W x W, W = 32 with
//      zero padding): warp w owns an 8x8 tile, lanes stride the row length and
//      a 5-step shuffle reduce-scatter leaves two sums per lane;
//   2. one round-robin sweep of two-sided rotations C <- R C R^T on the small
//      matrix (double-buffered, one barrier per sub-step; warp i holds pair i,
//      lane j the 2x2 block (i, j); lanes 16..31 rotate rows of Q = prod R);
//   3. [G | Vt]_w <- Q [G | Vt]_w, skipped when no pair rotated.
// The angles are those of the row-pair form (same criterion, same Rutishauser
// update) computed from the tracked Gram entries, so the sweep count and the
// stopping floor are unchanged; shared-memory traffic per step drops from
// O(W^2 (m + n)) to O(W (m + n)).
//
// MODE 0: rows of G, Vt = I.  MODE 2 (G = a symmetric positive
// semi-definite Z, m = n): the rows and columns of Z are gathered in the order
// perm (decreasing diagonal), factored in place as Z_perm + delta I = R^T R by
// a blocked row-oriented Cholesky across the cluster (the owner of block J
// factors its rows, every CTA applies the rank-bs update of its later rows
// from a DSMEM copy of R's block row); the shift delta = 2 n eps max(diag)
// makes the FP32 factorisation stable for rank-deficient Z.  Then the rows of
// R are orthogonalised without Vt (rows of J R = s_j u_j^T, u_j the
// eigenvectors of Z_perm, s_j^2 = lam_j + delta).  On exit G rows are
// lam_j u_j^T and Vt rows u_j^T, both in the original column order, and
// norms = lam_j.  Jacobi on the Cholesky factor needs about two thirds of the
// sweeps of Jacobi on Z (its rows are graded and nearly orthogonal from the
// start), but its vectors come from normalising rows that are orthogonal only
// to the Jacobi tolerance.
constexpr int GJ_W = 32;
constexpr int GJ_SLOT_CAP = BJ_MAX_SLOT_BYTES + 4 * (GJ_W / 2) * (GJ_W / 2);  // rows + tracked Gram
constexpr int GJ_MOVE_REGS = (GJ_SLOT_CAP / 16 + BJ_THREADS - 1) / BJ_THREADS;

template <int MODE>
__global__ void __launch_bounds__(BJ_THREADS) gjacobi_kernel(float* __restrict__ G, int64_t ldg,
                                                             float* __restrict__ Vt, int64_t ldv, int n, int m,
                                                             int bs, double tol, float* __restrict__ norms,
                                                             int* __restrict__ status,
                                                             const int* __restrict__ perm,
                                                             float* __restrict__ qlog, int* __restrict__ blog) {
  cg::cluster_group cluster = cg::this_cluster();
  const int cs = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nblk = 2 * cs;
  const int row_len = (MODE == 1 || MODE == 2) ? m : m + n;  // G part then Vt part
  // MODE 1 pads each row by 4 floats: the apply's 16-byte stores of 8 rows
  // at one column offset then fall in different banks
  const int rs = (MODE == 1 && (row_len & 7) == 0) ? row_len + 4 : row_len;
  const int slot_elems = bs * rs;
  // each slot: bs rows, then the bs x bs Gram matrix of those rows as tracked
  // through the rotations (it travels with the rows)
  const int gstride = (bs * bs + 3) & ~3;
  const int slot_tot = slot_elems + gstride;
  const int weff = 2 * bs;    // working rows (<= GJ_W)

  extern __shared__ __align__(16) unsigned char gj_raw[];
  float* slots = reinterpret_cast<float*>(gj_raw);  // 2 x ([bs][row_len], [bs][bs])
  float* stage = slots + 2 * slot_tot;              // one slot
  __shared__ __align__(16) float sC[2][GJ_W][GJ_W];
  __shared__ __align__(16) float sQ[GJ_W][GJ_W];
  __shared__ __align__(16) float sQt[GJ_W][GJ_W];
  __shared__ int s_off[GJ_W];
  __shared__ int s_blk[2][2];  // [parity][slot]: block ids, double-buffered for the MODE 1 move
  __shared__ int s_rot[2];
  __shared__ int s_any;
  __shared__ double s_norm;
  __shared__ double s_red[BJ_WARPS];

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
  // MODE 1 double-buffers the slots (buffers sl and 2 + sl; the block at the
  // fixed circle position 0 never moves): mp is the parity of the moves done
  int mp = 0;
  auto curo = [&](int sl) -> int64_t {
    if (MODE == 1 && mp && !(rank == 0 && sl == 0)) return (int64_t)(2 + sl) * slot_tot;
    return (int64_t)sl * slot_tot;
  };

  if (tid < GJ_W) s_off[tid] = (tid < weff) ? (tid / bs) * slot_tot + (tid % bs) * rs : -1;
  for (int sl = 0; sl < 2; ++sl) {
    const int blk = slot_pos(rank, sl);
    if (tid == 0) s_blk[0][sl] = blk;
    for (int64_t i = tid; i < (int64_t)bs * row_len; i += BJ_THREADS) {
      const int r = (int)(i / row_len), e = (int)(i % row_len);
      const int gr = blk * bs + r;
      float v = 0.f;
      if (gr < n) {
        if (MODE >= 2) v = (e < m) ? G[(int64_t)perm[gr] * ldg + perm[e]] : 0.f;
        else if (e < m) v = G[(int64_t)gr * ldg + e];
        else v = ((e - m) == gr) ? 1.f : 0.f;
      }
      slots[(int64_t)sl * slot_tot + (int64_t)r * rs + e] = v;
    }
  }
  float shift = 0.f;
  if constexpr (MODE >= 2) {
    // ---- largest diagonal entry over the cluster -> shift and pivot floor ----
    float mx = 0.f;
    for (int sl = 0; sl < 2; ++sl)
      for (int r = tid; r < bs; r += BJ_THREADS) {
        const int gr = slot_pos(rank, sl) * bs + r;
        if (gr < n) mx = fmaxf(mx, slots[(int64_t)sl * slot_tot + (int64_t)r * row_len + gr]);
      }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) s_red[warp] = (double)mx;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < BJ_WARPS; ++w) t = fmax(t, s_red[w]);
      s_norm = t;
    }
    cluster.sync();
    if (tid == 0) {
      double t = 0.0;
      for (int r = 0; r < cs; ++r) t = fmax(t, *cluster.map_shared_rank(&s_norm, r));
      s_red[0] = t;
    }
    __syncthreads();
    const float dfloor = fmaxf(FLT_EPSILON * (float)s_red[0], FLT_MIN);
    // Z + delta I has the eigenvectors of Z and a condition number below
    // 1 / (2 n eps), so its Cholesky factor is stable in FP32 even when Z is
    // numerically rank deficient (static pivoting alone is not: a pivot that
    // is rounding noise can carry off-diagonal entries of the size of the
    // matrix).  delta is removed from the eigenvalues on exit.
    shift = 2.f * (float)n * FLT_EPSILON * (float)s_red[0];
    for (int sl = 0; sl < 2; ++sl)
      for (int r = tid; r < bs; r += BJ_THREADS) {
        const int gr = slot_pos(rank, sl) * bs + r;
        if (gr < n) slots[(int64_t)sl * slot_tot + (int64_t)r * row_len + gr] += shift;
      }
    cluster.sync();  // s_norm / s_red are reused below
    // ---- blocked row-oriented Cholesky, Z_perm = R^T R ----
    float* coefT = &sQ[0][0];  // [2 bs][16]: R_J[i][K] for the CTA's own rows K
    for (int J = 0; J < nblk; ++J) {
      const int j0 = J * bs;
      if (j0 >= n) break;
      int ocs, osl;
      pos_owner(J, ocs, osl);
      const int jrows = min(bs, n - j0);
      if (rank == ocs) {
        float* blk = slots + (int64_t)osl * slot_tot;
        for (int r = 0; r < jrows; ++r) {
          const int gi = j0 + r;
          float* row = blk + (int64_t)r * row_len;
          __syncthreads();
          float d = row[gi];
          if (!(d > dfloor)) d = dfloor;
          const float sd = sqrtf(d), inv = 1.f / sd;
          __syncthreads();
          for (int e = tid; e < n; e += BJ_THREADS) row[e] = (e < gi) ? 0.f : (e == gi ? sd : row[e] * inv);
          __syncthreads();
          const int rem = jrows - r - 1;
          for (int idx = tid; idx < rem * n; idx += BJ_THREADS) {
            const int r2 = r + 1 + idx / n, e = idx % n;
            const int g2 = j0 + r2;
            if (e >= g2) blk[(int64_t)r2 * row_len + e] -= row[g2] * row[e];
          }
        }
      }
      cluster.sync();
      const int c0 = j0 + bs;
      if (c0 < n) {
        const float* src = cluster.map_shared_rank(slots, ocs) + (int64_t)osl * slot_tot;
        const int w = n - c0;
        for (int idx = tid; idx < bs * w; idx += BJ_THREADS) {
          const int i = idx / w, e = c0 + idx % w;
          stage[(int64_t)i * row_len + e] = (i < jrows) ? src[(int64_t)i * row_len + e] : 0.f;
        }
        __syncthreads();
        for (int idx = tid; idx < 2 * bs * 16; idx += BJ_THREADS) {
          const int lr = idx / 16, i = idx % 16;
          const int sl = lr / bs, r = lr % bs;
          const int B = slot_pos(rank, sl), K = B * bs + r;
          coefT[idx] = (i < bs && B > J && K < n) ? stage[(int64_t)i * row_len + K] : 0.f;
        }
        __syncthreads();
        for (int e = c0 + tid; e < n; e += BJ_THREADS) {
          float x[16];
#pragma unroll
          for (int i = 0; i < 16; ++i) x[i] = (i < bs) ? stage[(int64_t)i * row_len + e] : 0.f;
          for (int lr = 0; lr < 2 * bs; ++lr) {
            const int sl = lr / bs, r = lr % bs;
            if (slot_pos(rank, sl) <= J) continue;
            const float4* c4 = reinterpret_cast<const float4*>(coefT + lr * 16);
            float acc = 0.f;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const float4 c = c4[q];
              acc = fmaf(c.x, x[4 * q], acc);
              acc = fmaf(c.y, x[4 * q + 1], acc);
              acc = fmaf(c.z, x[4 * q + 2], acc);
              acc = fmaf(c.w, x[4 * q + 3], acc);
            }
            slots[(int64_t)sl * slot_tot + (int64_t)r * row_len + e] -= acc;
          }
        }
        __syncthreads();
      }
    }
    cluster.sync();
    if constexpr (MODE == 3) {
      // rows of L = R^T: local row i (position) <- column i of R, gathered from
      // the owners of R's rows; slot 0 through the stage buffer, slot 1
      // through registers, one cluster barrier before the local writes; the
      // Vt part starts as I
      constexpr int REGS = BJ_MAX_SLOT_BYTES / 2 / 4 / BJ_THREADS;  // G part <= half a slot
      float hold[REGS];
      for (int sl = 0; sl < 2; ++sl) {
        const int B = slot_pos(rank, sl);
        int k = 0;
        for (int idx = tid; idx < bs * m; idx += BJ_THREADS, ++k) {
          const int r = idx / m, j = idx % m;
          const int i = B * bs + r;
          float v = 0.f;
          if (i < n && j <= i) {
            int ocs, osl;
            pos_owner(j / bs, ocs, osl);
            v = cluster.map_shared_rank(slots, ocs)[(int64_t)osl * slot_tot + (int64_t)(j % bs) * row_len + i];
          }
          if (sl == 0) stage[(int64_t)r * row_len + j] = v;
          else if (k < REGS) hold[k] = v;
        }
      }
      cluster.sync();
      for (int sl = 0; sl < 2; ++sl) {
        const int B = slot_pos(rank, sl);
        int k = 0;
        for (int idx = tid; idx < bs * m; idx += BJ_THREADS, ++k) {
          const int r = idx / m, j = idx % m;
          float* row = slots + (int64_t)sl * slot_tot + (int64_t)r * row_len;
          row[j] = (sl == 0) ? stage[(int64_t)r * row_len + j] : (k < REGS ? hold[k] : 0.f);
        }
        for (int idx = tid; idx < bs * n; idx += BJ_THREADS) {
          const int r = idx / n, c = idx % n;
          slots[(int64_t)sl * slot_tot + (int64_t)r * row_len + m + c] = (B * bs + r == c) ? 1.f : 0.f;
        }
      }
      __syncthreads();
    }
  }
  // |G|_F^2 over the cluster -> floor m (eps |G|_F)^2 on |g_p . g_q|
  {
    double acc = 0.0;
    for (int64_t i = tid; i < 2 * (int64_t)slot_elems; i += BJ_THREADS) {
      const int sl = (int)(i / slot_elems), j = (int)(i % slot_elems);
      if (j % rs < m) {
        const double v = (double)slots[(int64_t)sl * slot_tot + j];
        acc += v * v;
      }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
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
    const double fl = 1.1920928955078125e-07 * sqrt(s_red[0]);
    cluster.sync();
    if (tid == 0) s_norm = (double)m * fl * fl;
    __syncthreads();
  }
  const float abs_floor = (float)s_norm;
  const float ftol = (float)tol;

  // Gram tile of this warp: 8 x 8 of the full 32 x 32, or 4 x 4 of the
  // bs x bs cross block
  const int ti = warp >> 2, tj = warp & 3;

  int sweeps = 0;
  bool converged = (n < 2);
  int my_rot = 0;
  while (!converged && sweeps < JAC_MAX_SWEEPS) {
    const int par = sweeps & 1;
    for (int step = 0; step < nblk - 1; ++step) {
      // ---- 1. Gram matrix of the working rows: all of it on the first step
      // of a sweep, else only the cross block (the two diagonal blocks are
      // the tracked Gram matrices that came with the rows) ----
      const bool all_pairs = (step == 0);
      // 4 x 4 tiles of C, lanes striding the row length, reduce-scatter to one
      // entry per lane pair: all 64 tiles of the 32 x 32 matrix on the first
      // step (4 per warp), else the 16 tiles of the cross block (1 per warp)
      // with the diagonal blocks taken from the tracked Gram matrices
      const int ntile = all_pairs ? 4 : 1;
      for (int tt = 0; tt < ntile; ++tt) {
        int ra0, rb0;  // first row of the tile's A and B rows (local indices)
        if (all_pairs) {
          const int t = warp * 4 + tt;  // 0..63 over an 8 x 8 grid of 4 x 4 tiles
          ra0 = 4 * (t >> 3);
          rb0 = 4 * (t & 7);
        } else {
          ra0 = 4 * ti;
          rb0 = bs + 4 * tj;
        }
        const int alim = all_pairs ? weff : bs, blim = all_pairs ? weff : 2 * bs;
        int offa[4], offb[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          offa[q] = (ra0 + q < alim) ? s_off[ra0 + q] : -1;
          offb[q] = (rb0 + q < blim && (all_pairs || rb0 + q >= bs)) ? s_off[rb0 + q] : -1;
        }
        float v[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) v[k] = 0.f;
        auto gram_scalar = [&]() {
          for (int e = lane; e < m; e += 32) {
            float xa[4], xb[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              xa[q] = offa[q] >= 0 ? slots[offa[q] + e] : 0.f;
              xb[q] = offb[q] >= 0 ? slots[offb[q] + e] : 0.f;
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
              for (int u = 0; u < 4; ++u) v[q * 4 + u] = fmaf(xa[q], xb[u], v[q * 4 + u]);
          }
        };
        if constexpr (MODE == 1) {
          if (((m | rs) & 3) == 0) {
            // 16-byte loads (row offsets and length multiples of 4 floats): a
            // quarter of the iterations of the scalar loop
            const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int e = 4 * lane; e < m; e += 128) {
              float4 xa[4], xb[4];
#pragma unroll
              for (int q = 0; q < 4; ++q) {
                xa[q] = offa[q] >= 0 ? *reinterpret_cast<const float4*>(slots + offa[q] + e) : z4;
                xb[q] = offb[q] >= 0 ? *reinterpret_cast<const float4*>(slots + offb[q] + e) : z4;
              }
#pragma unroll
              for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                  float t = v[q * 4 + u];
                  t = fmaf(xa[q].x, xb[u].x, t);
                  t = fmaf(xa[q].y, xb[u].y, t);
                  t = fmaf(xa[q].z, xb[u].z, t);
                  v[q * 4 + u] = fmaf(xa[q].w, xb[u].w, t);
                }
            }
          } else {
            gram_scalar();
          }
        } else {
          gram_scalar();
        }
#pragma unroll
        for (int h = 8, o = 16; o > 1; h >>= 1, o >>= 1) {
          const bool up = (lane & o) != 0;
#pragma unroll
          for (int k = 0; k < h; ++k) {
            const float send = up ? v[k] : v[k + h];
            const float keep = up ? v[k + h] : v[k];
            v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
          }
        }
        v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
        const int ra = ra0 + ((lane >> 1) >> 2), rb = rb0 + ((lane >> 1) & 3);
        if ((lane & 1) == 0 && ra < alim && rb < blim) {
          sC[0][ra][rb] = v[0];
          if (!all_pairs) sC[0][rb][ra] = v[0];
        }
      }
      if (!all_pairs) {
        for (int idx = tid; idx < 2 * bs * bs; idx += BJ_THREADS) {
          const int sl = idx / (bs * bs), r = idx % (bs * bs);
          sC[0][sl * bs + r / bs][sl * bs + r % bs] = slots[curo(sl) + slot_elems + r];
        }
      }
      for (int i = tid; i < GJ_W * GJ_W; i += BJ_THREADS) sQ[i / GJ_W][i % GJ_W] = (i / GJ_W == i % GJ_W) ? 1.f : 0.f;
      if (tid == 0) s_any = 0;
      __syncthreads();

      // ---- 2. rotations on C, accumulated in Q.  The first step of a sweep
      // takes every pair of the 2 bs working rows (round robin, 2 bs - 1
      // sub-steps); all blocks sit in some working set then, so the later
      // steps need only the pairs across the two blocks (sub-step u pairs
      // local row i with row bs + (i + u) mod bs: bs sub-steps).  Every pair
      // of rows is thus visited once per sweep.
      int cur = 0;
      const int nsub = all_pairs ? weff - 1 : bs;
      auto pair_p = [&](int i, int u) { return all_pairs ? rr_index(i, u, weff) : i; };
      auto pair_q = [&](int i, int u) {
        if (!all_pairs) {
          const int t = i + u;
          return bs + (t >= bs ? t - bs : t);
        }
        return rr_index(weff - 1 - i, u, weff);
      };
      for (int sub = 0; sub < nsub; ++sub) {
        if (warp < bs) {
          // warp i: the rows p_i, q_i of C (2 x 32 entries: lane l holds block
          // (i, l / 2), row p_i or q_i by the parity of l) and of Q (lane = column)
          const int i = warp;
          const int pi = pair_p(i, sub), qi = pair_q(i, sub);
          const int j = lane >> 1, half = lane & 1;
          // the rotation of pair j, on lanes 2j and 2j + 1
          float cj = 1.f, sj = 0.f, tj_ = 0.f, tanj = 0.f;
          int rj = 0, pj = 0, qj = 0;
          if (j < bs) {
            pj = pair_p(j, sub);
            qj = pair_q(j, sub);
            const float a = fmaxf(sC[cur][pj][pj], 0.f), b = fmaxf(sC[cur][qj][qj], 0.f), c = sC[cur][pj][qj];
            float c_, s_, t_, tn_;
            if (rot_fast(a, b, c, ftol, abs_floor, c_, s_, t_, tn_)) {
              rj = 1;
              cj = c_;
              sj = s_;
              tj_ = t_;
              tanj = tn_;
            }
          }
          const int ri = __shfl_sync(0xffffffffu, rj, 2 * i);
          const float si = __shfl_sync(0xffffffffu, sj, 2 * i);
          const float taui = __shfl_sync(0xffffffffu, tj_, 2 * i), tani = __shfl_sync(0xffffffffu, tanj, 2 * i);
          (void)cj;
          const int nxt = cur ^ 1;
          if (j < bs) {
            const float xpp = sC[cur][pi][pj], xpq = sC[cur][pi][qj], xqp = sC[cur][qi][pj], xqq = sC[cur][qi][qj];
            float o0, o1;  // this lane's row (p_i or q_i) at columns p_j and q_j
            if (j == i) {
              if (ri) {
                o0 = half ? 0.f : xpp - tani * xpq;
                o1 = half ? xqq + tani * xpq : 0.f;
              } else {
                o0 = half ? xqp : xpp;
                o1 = half ? xqq : xpq;
              }
            } else {
              float rp = half ? xqp : xpp, rq = half ? xqq : xpq;
              if (ri) {  // rows p_i, q_i
                rp = half ? xqp + si * (xpp - taui * xqp) : xpp - si * (xqp + taui * xpp);
                rq = half ? xqq + si * (xpq - taui * xqq) : xpq - si * (xqq + taui * xpq);
              }
              if (rj) {  // columns p_j, q_j
                o0 = rp - sj * (rq + tj_ * rp);
                o1 = rq + sj * (rp - tj_ * rq);
              } else {
                o0 = rp;
                o1 = rq;
              }
            }
            const int rr = half ? qi : pi;
            sC[nxt][rr][pj] = o0;
            sC[nxt][rr][qj] = o1;
          }
          if (ri && lane < weff) {
            const float x = sQ[pi][lane], y = sQ[qi][lane];
            sQ[pi][lane] = x - si * (y + taui * x);
            sQ[qi][lane] = y + si * (x - taui * y);
          }
          if (ri && lane == 2 * i) {
            ++my_rot;
            s_any = 1;
          }
        }
        __syncthreads();
        cur ^= 1;
      }
      // the diagonal blocks of the rotated Gram matrix travel with the rows
      for (int idx = tid; idx < 2 * bs * bs; idx += BJ_THREADS) {
        const int sl = idx / (bs * bs), r = idx % (bs * bs);
        slots[curo(sl) + slot_elems + r] = sC[cur][sl * bs + r / bs][sl * bs + r % bs];
      }
      if constexpr (MODE == 1) {
        // log Q and the two block ids (-1: no rotation) for gj_replay_kernel
        const int64_t ls = ((int64_t)sweeps * (nblk - 1) + step) * cs + rank;
        if (s_any) {
          float4* qd = reinterpret_cast<float4*>(qlog + ls * (GJ_W * GJ_W));
          for (int i = tid; i < GJ_W * GJ_W / 4; i += BJ_THREADS) qd[i] = reinterpret_cast<const float4*>(&sQ[0][0])[i];
        }
        if (tid == 0) {
          blog[2 * ls] = s_any ? s_blk[mp][0] : -1;
          blog[2 * ls + 1] = s_blk[mp][1];
        }
      }

      // ---- 3. apply Q to the working rows ----
      if (s_any && (row_len & 7) == 0) {
        // register tiles: thread rg = output rows rg, rg + 8, rg + 16, rg + 24
        // x 8 columns (eight consecutive rows per 16-byte store phase, which
        // the padded row stride puts in distinct banks), Q^T rows as one
        // 16-byte broadcast per K step (sQt[k][4 rg + a] = Q[rg + 8 a][k]),
        // X rows as two; all reads finish before the in-place writes
        for (int i = tid; i < GJ_W * GJ_W; i += BJ_THREADS) {
          const int r = i / GJ_W, k = i % GJ_W;
          sQt[k][4 * (r & 7) + (r >> 3)] = sQ[r][k];
        }
        __syncthreads();
        const int rg = lane & 7, cgl = lane >> 3;
        for (int ebase = 0; ebase < row_len; ebase += BJ_THREADS) {
          const int e0 = ebase + (warp * 4 + cgl) * 8;
          float acc[4][8];
#pragma unroll
          for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int u = 0; u < 8; ++u) acc[a][u] = 0.f;
          if (e0 < row_len) {
            for (int k = 0; k < weff; ++k) {
              const float4 q = *reinterpret_cast<const float4*>(&sQt[k][4 * rg]);
              const float* xr = slots + s_off[k] + e0;
              const float4 x0 = *reinterpret_cast<const float4*>(xr);
              const float4 x1 = *reinterpret_cast<const float4*>(xr + 4);
              const float qa[4] = {q.x, q.y, q.z, q.w};
              const float xv[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
#pragma unroll
              for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int u = 0; u < 8; ++u) acc[a][u] = fmaf(qa[a], xv[u], acc[a][u]);
            }
          }
          __syncthreads();
          if (e0 < row_len) {
#pragma unroll
            for (int a = 0; a < 4; ++a) {
              const int r = rg + 8 * a;
              if (r < weff) {
                float4* d = reinterpret_cast<float4*>(slots + s_off[r] + e0);
                d[0] = make_float4(acc[a][0], acc[a][1], acc[a][2], acc[a][3]);
                d[1] = make_float4(acc[a][4], acc[a][5], acc[a][6], acc[a][7]);
              }
            }
          }
          __syncthreads();
        }
      } else if (s_any) {
        for (int e = tid; e < row_len; e += BJ_THREADS) {
          float x[GJ_W];
#pragma unroll
          for (int j = 0; j < GJ_W; ++j) x[j] = (j < weff) ? slots[s_off[j] + e] : 0.f;
#pragma unroll 4
          for (int r = 0; r < weff; ++r) {
            const float4* q4 = reinterpret_cast<const float4*>(&sQ[r][0]);
            float acc = 0.f;
#pragma unroll
            for (int j4 = 0; j4 < GJ_W / 4; ++j4) {
              const float4 q = q4[j4];
              acc = fmaf(q.x, x[4 * j4], acc);
              acc = fmaf(q.y, x[4 * j4 + 1], acc);
              acc = fmaf(q.z, x[4 * j4 + 2], acc);
              acc = fmaf(q.w, x[4 * j4 + 3], acc);
            }
            slots[s_off[r] + e] = acc;
          }
        }
      }

      // ---- 4. move blocks one position along the circle ----
      int src_cta[2], src_slot[2];
      for (int sl = 0; sl < 2; ++sl) {
        const int q = slot_pos(rank, sl);
        const int qs = (q == 0) ? 0 : (q == 1 ? nblk - 1 : q - 1);
        pos_owner(qs, src_cta[sl], src_slot[sl]);
      }
      if constexpr (MODE == 1) {
        // pull straight into the other buffer of each moving slot: a buffer
        // is only overwritten after the next step's cluster barrier, by when
        // every CTA has finished reading it, so one barrier per step suffices
        cluster.sync();
        const int nmp = mp ^ 1;
        const int n4 = slot_tot * (int)sizeof(float) / 16;
        for (int sl = 0; sl < 2; ++sl) {
          if (rank == 0 && sl == 0) continue;
          const int sc = src_cta[sl], ss = src_slot[sl];
          const int64_t soff = (sc == 0 && ss == 0) ? 0 : (int64_t)(mp ? 2 + ss : ss) * slot_tot;
          const int64_t doff = (int64_t)(nmp ? 2 + sl : sl) * slot_tot;
          const uint4* src4 = reinterpret_cast<const uint4*>(cluster.map_shared_rank(slots, sc) + soff);
          uint4* dst4 = reinterpret_cast<uint4*>(slots + doff);
          for (int idx = tid; idx < n4; idx += BJ_THREADS) dst4[idx] = src4[idx];
          if (tid == 0) s_blk[nmp][sl] = *cluster.map_shared_rank(&s_blk[mp][ss], sc);
        }
        if (rank == 0 && tid == 0) s_blk[nmp][0] = s_blk[mp][0];
        mp = nmp;
        if (tid < GJ_W) s_off[tid] = (tid < weff) ? (int)curo(tid / bs) + (tid % bs) * rs : -1;
        __syncthreads();
        continue;
      }
      cluster.sync();
      const float* r0 = cluster.map_shared_rank(slots, src_cta[0]) + (int64_t)src_slot[0] * slot_tot;
      const float* r1 = cluster.map_shared_rank(slots, src_cta[1]) + (int64_t)src_slot[1] * slot_tot;
      const int nb0 = *cluster.map_shared_rank(&s_blk[0][src_slot[0]], src_cta[0]);
      const int nb1 = *cluster.map_shared_rank(&s_blk[0][src_slot[1]], src_cta[1]);
      const int n4 = slot_tot * (int)sizeof(float) / 16;
      const uint4* s0 = reinterpret_cast<const uint4*>(r0);
      const uint4* s1 = reinterpret_cast<const uint4*>(r1);
      uint4* st4 = reinterpret_cast<uint4*>(stage);
      uint4 regs[GJ_MOVE_REGS];
#pragma unroll
      for (int j = 0; j < GJ_MOVE_REGS; ++j) {
        const int idx = tid + j * BJ_THREADS;
        if (idx < n4) {
          st4[idx] = s0[idx];
          regs[j] = s1[idx];
        }
      }
      cluster.sync();
      uint4* d0 = reinterpret_cast<uint4*>(slots);
      uint4* d1 = reinterpret_cast<uint4*>(slots + slot_tot);
#pragma unroll
      for (int j = 0; j < GJ_MOVE_REGS; ++j) {
        const int idx = tid + j * BJ_THREADS;
        if (idx < n4) {
          d0[idx] = st4[idx];
          d1[idx] = regs[j];
        }
      }
      if (tid == 0) {
        s_blk[0][0] = nb0;
        s_blk[0][1] = nb1;
      }
      __syncthreads();
    }
    if (my_rot) atomicAdd(&s_rot[par], my_rot);
    my_rot = 0;
    __syncthreads();
    cluster.sync();
    int total = 0;
    for (int r = 0; r < cs; ++r) total += *cluster.map_shared_rank(&s_rot[par], r);
    ++sweeps;
    converged = (total == 0);
    cluster.sync();
    if (tid == 0) s_rot[par] = 0;
  }
  for (int sl = 0; sl < 2; ++sl) {
    const int blk = s_blk[mp][sl];
    if (MODE == 2) {
      for (int r = warp; r < bs; r += BJ_WARPS) {
        const int gr = blk * bs + r;
        if (gr >= n) continue;
        const float* row = slots + curo(sl) + (int64_t)r * rs;
        float acc = 0.f;
        for (int e = lane; e < m; e += 32) acc = fmaf(row[e], row[e], acc);
        acc = wsum_t(acc);
        const float sg = sqrtf(acc), inv = sg > 0.f ? 1.f / sg : 0.f;
        const float lam = fmaxf(acc - shift, 0.f);
        for (int e = lane; e < m; e += 32) {
          G[(int64_t)gr * ldg + perm[e]] = row[e] * (lam * inv);
          Vt[(int64_t)gr * ldv + perm[e]] = row[e] * inv;
        }
        if (lane == 0) norms[gr] = lam;
      }
      continue;
    }
    if (MODE == 3) {
      for (int r = warp; r < bs; r += BJ_WARPS) {
        const int gr = blk * bs + r;
        if (gr >= n) continue;
        const float* row = slots + curo(sl) + (int64_t)r * rs;
        float acc = 0.f;
        for (int e = lane; e < m; e += 32) acc = fmaf(row[e], row[e], acc);
        acc = wsum_t(acc);
        const float lam = fmaxf(acc - shift, 0.f);
        for (int e = lane; e < n; e += 32) {
          const float v = row[m + e];
          G[(int64_t)gr * ldg + perm[e]] = lam * v;
          Vt[(int64_t)gr * ldv + perm[e]] = v;
        }
        if (lane == 0) norms[gr] = lam;
      }
      continue;
    }
    for (int64_t i = tid; i < (int64_t)bs * row_len; i += BJ_THREADS) {
      const int r = (int)(i / row_len), e = (int)(i % row_len);
      const int gr = blk * bs + r;
      if (gr >= n) continue;
      const float v = slots[curo(sl) + (int64_t)r * rs + e];
      if (e < m) G[(int64_t)gr * ldg + e] = v;
      else Vt[(int64_t)gr * ldv + (e - m)] = v;
    }
    for (int r = warp; r < bs; r += BJ_WARPS) {
      const int gr = blk * bs + r;
      if (gr >= n) continue;
      const float* row = slots + curo(sl) + (int64_t)r * rs;
      float acc = 0.f;
      for (int e = lane; e < m; e += 32) acc = fmaf(row[e], row[e], acc);
      acc = wsum_t(acc);
      if (lane == 0) norms[gr] = sqrtf(acc);
    }
  }
  if (rank == 0 && tid == 0 && status) *status = converged ? sweeps : -1;
  cluster.sync();
}

// Vt = (the logged rotations of gjacobi_kernel<1>, in order) applied to I.
// Columns of Vt transform independently under row rotations, so each CTA
// replays the whole log on a slice of COLS (4 or 8) columns held in shared
// memory (all 2 cs bs block rows) and needs no other CTA; 4-column slices
// spread a 512-column Vt over 128 CTAs instead of 64.  The log of step s + 1
// (the cs rotation matrices, rows padded to 36 floats so that the 16-byte
// loads of the 8 rows a quarter-warp reads fall in distinct banks, and the
// block ids) streams into the other half of a double buffer with cp.async
// while step s computes every working row of its rotated pairs into
// registers; the rows are written back after a barrier.
constexpr int RP_THREADS = 256, RP_QS = GJ_W + 4;

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <int COLS>
__global__ void __launch_bounds__(RP_THREADS) gj_replay_kernel(const float* __restrict__ qlog,
                                                               const int* __restrict__ blog,
                                                               const int* __restrict__ status, int n, int cs, int bs,
                                                               float* __restrict__ Vt, int64_t ldv) {
  extern __shared__ __align__(16) float rp_smem[];
  const int nrows = 2 * cs * bs, weff = 2 * bs;
  float* V = rp_smem;                                   // [nrows][COLS]
  float* Qb = V + nrows * COLS;                      // [2][cs][GJ_W][RP_QS]
  __shared__ int s_b[2][2 * 16];
  const int c0 = blockIdx.x * COLS, tid = threadIdx.x;
  const int qstride = cs * GJ_W * RP_QS;
  for (int i = tid; i < nrows * COLS; i += RP_THREADS) V[i] = (i / COLS == c0 + i % COLS) ? 1.f : 0.f;
  const int st = *status;
  const int sweeps = st > 0 ? st : (st < 0 ? JAC_MAX_SWEEPS : 0);
  const int64_t nsteps = (int64_t)sweeps * (2 * cs - 1);
  const int tasks = cs * weff;  // (pair, working row)
  auto prefetch = [&](int64_t ls, int buf) {
    const float* src = qlog + ls * cs * (GJ_W * GJ_W);
    float* dst = Qb + buf * qstride;
    for (int i = tid; i < cs * GJ_W * GJ_W / 4; i += RP_THREADS) {
      const int cr = i / (GJ_W / 4), q4 = i % (GJ_W / 4);  // cr = pair * GJ_W + row
      cp_async16(dst + cr * RP_QS + 4 * q4, src + 4 * i);
    }
    if (tid < 2 * cs) cp_async4(&s_b[buf][tid], blog + ls * cs * 2 + tid);
    cp_async_commit();
  };
  if (nsteps > 0) prefetch(0, 0);
  for (int64_t ls = 0; ls < nsteps; ++ls) {
    const int cur = (int)(ls & 1);
    if (ls + 1 < nsteps) {
      prefetch(ls + 1, cur ^ 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    int any = 0;
    for (int c = 0; c < cs; ++c) any |= (s_b[cur][2 * c] >= 0);
    float out[2][COLS];
    int orow[2] = {-1, -1};
    if (any) {
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const int t = tid + k * RP_THREADS;
        if (t >= tasks) continue;
        const int c = t / weff, r = t % weff;
        const int A = s_b[cur][2 * c], B = s_b[cur][2 * c + 1];
        if (A < 0) continue;
        const float* q = Qb + cur * qstride + (c * GJ_W + r) * RP_QS;
#pragma unroll
        for (int u = 0; u < COLS; ++u) out[k][u] = 0.f;
        for (int j4 = 0; j4 < weff / 4; ++j4) {
          const float4 q4 = *reinterpret_cast<const float4*>(q + 4 * j4);
          const float qv[4] = {q4.x, q4.y, q4.z, q4.w};
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const int j = 4 * j4 + jj;
            const int vr = (j < bs) ? A * bs + j : B * bs + (j - bs);
#pragma unroll
            for (int h = 0; h < COLS / 4; ++h) {
              const float4 v = *reinterpret_cast<const float4*>(V + vr * COLS + 4 * h);
              out[k][4 * h + 0] = fmaf(qv[jj], v.x, out[k][4 * h + 0]);
              out[k][4 * h + 1] = fmaf(qv[jj], v.y, out[k][4 * h + 1]);
              out[k][4 * h + 2] = fmaf(qv[jj], v.z, out[k][4 * h + 2]);
              out[k][4 * h + 3] = fmaf(qv[jj], v.w, out[k][4 * h + 3]);
            }
          }
        }
        for (int j = 4 * (weff / 4); j < weff; ++j) {
          const int vr = (j < bs) ? A * bs + j : B * bs + (j - bs);
#pragma unroll
          for (int u = 0; u < COLS; ++u) out[k][u] = fmaf(q[j], V[vr * COLS + u], out[k][u]);
        }
        orow[k] = (r < bs) ? A * bs + r : B * bs + (r - bs);
      }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (orow[k] < 0) continue;
      float4* d = reinterpret_cast<float4*>(V + orow[k] * COLS);
#pragma unroll
      for (int h = 0; h < COLS / 4; ++h)
        d[h] = make_float4(out[k][4 * h], out[k][4 * h + 1], out[k][4 * h + 2], out[k][4 * h + 3]);
    }
  }
  __syncthreads();
  for (int i = tid; i < n * COLS; i += RP_THREADS) {
    const int r = i / COLS, c = c0 + i % COLS;
    if (c < n) Vt[(int64_t)r * ldv + c] = V[i];
  }
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
// FP32 multiplier: 1 unless SGT_EIG_TOL (a positive number) overrides it.
// With eps sqrt(m) the rounded MPO x MPS states of the 64-site benchmark chain
// agree with the FP64 form to an infidelity of ~2e-9 (8 eps sqrt(m): ~7e-6)
// at the same sweep count: the last sweeps converge quadratically, so a
// tighter stop costs little, while the pairs straddling the truncation have
// small relative gaps and amplify whatever residual the stop leaves.
static double f32_tol_scale() {
  static const double v = [] {
    const char* e = getenv("SGT_EIG_TOL");
    const double x = e ? atof(e) : 0.0;
    return (x > 0.0 && x < 1e6) ? x : 1.0;
  }();
  return v;
}

template <typename T>
double jacobi_tol(int64_t m) {
  const double eps = (sizeof(T) == 8) ? DBL_EPSILON : (double)FLT_EPSILON;
  const double k = (sizeof(T) == 8) ? 4.0 : f32_tol_scale();
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

// Launch gjacobi_kernel<MODE> when its cluster layout fits (n in [64, 512],
// blocks of <= 16 rows, slots within the shared-memory budget and a cluster
// of that size schedulable); *launched reports whether it was.
static int gj_cluster(int64_t n) {
  int csb = 2;
  while (csb < 16 && cdiv(n, 2 * csb) > GJ_W / 2) csb *= 2;
  return csb;
}

template <int MODE>
static int launch_gjacobi(cudaStream_t st, float* G, int64_t ldg, float* Vt, int64_t ldv, int64_t n, int64_t m,
                          float* norms, int* status, const int* perm, bool* launched, float* qlog = nullptr,
                          int* blog = nullptr) {
  *launched = false;
  if (n < 64 || n > 16 * GJ_W || (MODE >= 2 && m != n)) return SGT_OK;
  const int csb = gj_cluster(n);
  const int64_t bsz = cdiv(n, 2 * csb);
  int64_t rlen = (MODE == 1 || MODE == 2) ? m : m + n;
  if (MODE == 1 && rlen % 8 == 0) rlen += 4;  // the kernel's row padding
  const int64_t slot_bytes = bsz * rlen * (int64_t)sizeof(float);
  if (bsz > GJ_W / 2 || slot_bytes > BJ_MAX_SLOT_BYTES || slot_bytes % 16 != 0) return SGT_OK;
  auto kern = gjacobi_kernel<MODE>;
  SGT_CUDA(func_attr_at_least((const void*)kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  SGT_CUDA(func_attr_at_least((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 3 * GJ_SLOT_CAP));
  const int64_t gram_bytes = ((bsz * bsz + 3) & ~int64_t(3)) * (int64_t)sizeof(float);
  const int64_t dyn = (MODE == 1 ? 4 : 3) * (slot_bytes + gram_bytes);
  if (dyn > 3 * GJ_SLOT_CAP) return SGT_OK;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(csb, 1, 1);
  cfg.blockDim = dim3(BJ_THREADS, 1, 1);
  cfg.dynamicSmemBytes = (size_t)dyn;
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
    cudaGetLastError();
    return SGT_OK;
  }
  SGT_CUDA(cudaLaunchKernelEx(&cfg, kern, G, ldg, Vt, ldv, (int)n, (int)m, (int)bsz, jacobi_tol<float>(m), norms,
                              status, perm, qlog, blog));
  note_launch();
  *launched = true;
  return SGT_OK;
}

// Rows of G and Vt and the norms reordered by decreasing norm (ties by index).
template <typename T>
int sort_rows_t(cudaStream_t st, T* G, int64_t ldg, int64_t n, int64_t m, T* Vt, int64_t ldv, T* s,
                const T* norms, int* perm, T* Gtmp, T* Vtmp) {
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

  // FP32: Gram-form block Jacobi when the rows fit 2 blocks of <= 16 rows per
  // CTA of a cluster of <= 16 CTAs, Vt included
  if constexpr (sizeof(T) == 4) {
    bool launched = false;
    SGT_TRY(launch_gjacobi<0>(st, G, ldg, Vt, ldv, n, m, norms, status, nullptr, &launched));
    if (launched) goto sort;
  }
  // cluster-resident block Jacobi when a cluster of up to 16 CTAs can hold
  // the rows (G, and Vt too when it fits), else the L2-resident kernel below
  if (n >= 64 && m <= 4096) {
    int csb = 2;
    while (csb < 16 && csb * 2 * 32 <= n) csb *= 2;  // about 16 rows per block
    for (int vt_smem = 1; vt_smem >= 0; --vt_smem) {
      const int64_t bsz = cdiv(n, 2 * csb);
      const int64_t slot_bytes = bsz * (m + (vt_smem ? n : 0)) * (int64_t)sizeof(T);
      if (slot_bytes > BJ_MAX_SLOT_BYTES || slot_bytes % 16 != 0) continue;
      auto kern = bjacobi_kernel<T>;
      SGT_CUDA(func_attr_at_least((const void*)kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
      SGT_CUDA(func_attr_at_least((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  3 * BJ_MAX_SLOT_BYTES));
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
  SGT_CUDA(func_attr_at_least((const void*)jacobi_kernel<double>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  SGT_CUDA(func_attr_at_least((const void*)jacobi_kernel<float>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
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
  return sort_rows_t<T>(st, G, ldg, n, m, Vt, ldv, s, norms, perm, Gtmp, Vtmp);
}

int jacobi_rows(cudaStream_t st, double* G, int64_t ldg, int64_t n, int64_t m, double* Vt,
                int64_t ldv, double* s, int* status, Arena& ar) {
  return jacobi_rows_t<double>(st, G, ldg, n, m, Vt, ldv, s, status, ar);
}

int jacobi_rows_f32(cudaStream_t st, float* G, int64_t ldg, int64_t n, int64_t m, float* Vt,
                    int64_t ldv, float* s, int* status, Arena& ar) {
  return jacobi_rows_t<float>(st, G, ldg, n, m, Vt, ldv, s, status, ar);
}

// ---------------------------------------------------------------------------
// Symmetric positive semi-definite eigenproblem Z = V diag(lam) V^T (FP32,
// n x n, Z overwritten).  Vt rows: eigenvectors, lam: eigenvalues, decreasing.
//   method 0: one-sided Jacobi on the rows of Z, rotations accumulated in Vt
//             (rows of Z V are lam_j v_j^T)
//   method 2: diagonal-ordered Cholesky + one-sided Jacobi on the rows of the
//             factor R, vectors by normalisation (gjacobi_kernel<2>)
//   method 3: the same factor, one-sided Jacobi on the rows of L = R^T with
//             the rotations accumulated: the eigenvectors of Z are the rows of
//             the accumulated rotation (R^T R = J^T S^2 J) (gjacobi_kernel<3>)
// status: sweeps, -1 at the sweep cap.

namespace {

__global__ void diag_order_kernel(const float* __restrict__ Z, int64_t ldz, int n, int* __restrict__ order) {
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const float v = Z[(int64_t)j * ldz + j];
    int r = 0;
    for (int i = 0; i < n; ++i) {
      const float w = Z[(int64_t)i * ldz + i];
      r += (w > v) || (w == v && i < j);
    }
    order[r] = j;
  }
}

}  // namespace

// Rotation log of gjacobi_kernel<1>: one 32 x 32 matrix and two block ids
// per CTA per outer step, for the sweep cap.
static size_t gj_log_floats(int64_t n) {
  const int cs = gj_cluster(n);
  return (size_t)JAC_MAX_SWEEPS * (2 * cs - 1) * cs * GJ_W * GJ_W;
}
static size_t gj_log_ints(int64_t n) {
  const int cs = gj_cluster(n);
  return (size_t)JAC_MAX_SWEEPS * (2 * cs - 1) * cs * 2;
}

// Monotone in n: a workspace sized for the largest bond problem of a chain
// also serves its smaller ones.
size_t sym_eig_rows_ws_bytes(int64_t n) {
  Arena a = Arena::measuring();
  a.take<int>((size_t)n);  // diagonal order
  if (n >= 64) {
    const int64_t nl = std::min<int64_t>(n, 16 * GJ_W);
    a.take<float>(gj_log_floats(nl));
    a.take<int>(gj_log_ints(nl));
  }
  return a.used + jacobi_rows_ws_bytes_t<float>(n, n);
}

// Optional event timing of the cluster eigensolver's launches (benchmarks):
// a CUDA event pair around every gjacobi_kernel<1> launch, on its stream,
// and the status word that receives its sweep count.
struct EigProfRec {
  cudaEvent_t a, b;
  const int* status;
  int64_t n;
};
ProfLog<EigProfRec> g_eig_prof;

int sym_eig_rows_f32(cudaStream_t st, float* Z, int64_t n, float* Vt, float* lam, int* status, Arena& ar,
                     int method) {
  if (method < 1 || method > 3 || n < 64 || n > 16 * GJ_W)
    return jacobi_rows_f32(st, Z, n, n, n, Vt, n, lam, status, ar);
  Arena ar0 = ar;  // for the fallbacks below, which need none of the buffers taken here
  if (method == 1) {
    // rows of Z only in shared memory; the rotations are logged and replayed
    // on Vt = I afterwards by all SMs (columns of Vt are independent)
    float* qlog = ar.take<float>(gj_log_floats(n));
    int* blog = ar.take<int>(gj_log_ints(n));
    float* Gtmp = ar.take<float>((size_t)n * n);
    float* Vtmp = ar.take<float>((size_t)n * n);
    float* norms = ar.take<float>((size_t)n);
    int* perm = ar.take<int>((size_t)n);
    SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "sym_eig: workspace too small");
    bool launched = false;
    // timing (benchmarks only) never fails the solve: a record whose events
    // cannot be made is dropped, and its error cleared
    EigProfRec rec{nullptr, nullptr, status, n};
    bool prof = false;
    if (g_eig_prof.active()) {
      prof = cudaEventCreate(&rec.a) == cudaSuccess;
      if (prof && cudaEventCreate(&rec.b) != cudaSuccess) {
        cudaEventDestroy(rec.a);
        rec.a = nullptr;
        prof = false;
      }
      if (prof && cudaEventRecord(rec.a, st) != cudaSuccess) prof = false;
      if (!prof) cudaGetLastError();
    }
    SGT_TRY(launch_gjacobi<1>(st, Z, n, Vt, n, n, n, norms, status, nullptr, &launched, qlog, blog));
    if (rec.b) {
      if (prof && launched && cudaEventRecord(rec.b, st) == cudaSuccess) {
        g_eig_prof.add(rec);
      } else {
        if (prof && launched) cudaGetLastError();
        cudaEventDestroy(rec.a);
        cudaEventDestroy(rec.b);
      }
    }
    if (!launched) return jacobi_rows_f32(st, Z, n, n, n, Vt, n, lam, status, ar0);
    const int cs = gj_cluster(n);
    const int bsz = (int)cdiv(n, 2 * cs);
    // 8-column slices unless that leaves most SMs idle
    const int cols = cdiv(n, 8) >= 128 ? 8 : 4;
    const size_t smem = sizeof(float) * ((size_t)2 * cs * bsz * cols + (size_t)2 * cs * GJ_W * RP_QS);
    {
      const size_t qb = sizeof(float) * (size_t)2 * 16 * GJ_W * RP_QS;
      SGT_CUDA(func_attr_at_least((const void*)gj_replay_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(sizeof(float) * (size_t)2 * 16 * (GJ_W / 2) * 8 + qb)));
      SGT_CUDA(func_attr_at_least((const void*)gj_replay_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(sizeof(float) * (size_t)2 * 16 * (GJ_W / 2) * 4 + qb)));
    }
    if (cols == 8)
      gj_replay_kernel<8><<<(unsigned)cdiv(n, 8), RP_THREADS, smem, st>>>(qlog, blog, status, (int)n, cs, bsz, Vt, n);
    else
      gj_replay_kernel<4><<<(unsigned)cdiv(n, 4), RP_THREADS, smem, st>>>(qlog, blog, status, (int)n, cs, bsz, Vt, n);
    SGT_LAUNCHED();
    SGT_TRY(sort_rows_t<float>(st, Z, n, n, n, Vt, n, lam, norms, perm, Gtmp, Vtmp));
    return SGT_OK;
  }
  int* order = ar.take<int>((size_t)n);
  float* Gtmp = ar.take<float>((size_t)n * n);
  float* Vtmp = ar.take<float>((size_t)n * n);
  float* norms = ar.take<float>((size_t)n);
  int* perm = ar.take<int>((size_t)n);
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "sym_eig: workspace too small");
  diag_order_kernel<<<1, 512, 0, st>>>(Z, n, (int)n, order);
  SGT_LAUNCHED();
  bool launched = false;
  // timing (benchmarks only), as for method 1: never fails the solve
  EigProfRec rec{nullptr, nullptr, status, n};
  bool prof = false;
  if (g_eig_prof.active()) {
    prof = cudaEventCreate(&rec.a) == cudaSuccess;
    if (prof && cudaEventCreate(&rec.b) != cudaSuccess) {
      cudaEventDestroy(rec.a);
      rec.a = nullptr;
      prof = false;
    }
    if (prof && cudaEventRecord(rec.a, st) != cudaSuccess) prof = false;
    if (!prof) cudaGetLastError();
  }
  if (method == 2) SGT_TRY(launch_gjacobi<2>(st, Z, n, Vt, n, n, n, norms, status, order, &launched));
  else SGT_TRY(launch_gjacobi<3>(st, Z, n, Vt, n, n, n, norms, status, order, &launched));
  if (rec.b) {
    if (prof && launched && cudaEventRecord(rec.b, st) == cudaSuccess) {
      g_eig_prof.add(rec);
    } else {
      if (prof && launched) cudaGetLastError();
      cudaEventDestroy(rec.a);
      cudaEventDestroy(rec.b);
    }
  }
  if (!launched) return jacobi_rows_f32(st, Z, n, n, n, Vt, n, lam, status, ar0);
  SGT_TRY(sort_rows_t<float>(st, Z, n, n, n, Vt, n, lam, norms, perm, Gtmp, Vtmp));
  return SGT_OK;
}

}  // namespace sgt

// enable = 1: start recording the cluster eigensolver's launches; 0: stop, wait
// for the recorded events and return the summed kernel milliseconds, the
// algorithmic FP32 flops (sweeps x n(n-1)/2 pair visits x 12 n: three dot
// products and the rotation of two rows of length n per visit) and the number
// of launches.
extern "C" SGT_API int sgt_eig_profile(int enable, double* ms, double* flops, long long* launches) {
  using namespace sgt;
  if (enable) {
    g_eig_prof.on = true;
    return SGT_OK;
  }
  g_eig_prof.on = false;
  const std::vector<EigProfRec> recs = g_eig_prof.take();
  double tot = 0.0, fl = 0.0;
  int rc = SGT_OK;
  for (auto& r : recs) {
    float t = 0.f;
    int sw = 0;
    if (rc == SGT_OK && cudaEventSynchronize(r.b) == cudaSuccess &&
        cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess &&
        (!r.status || cudaMemcpy(&sw, r.status, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess)) {
      tot += t;
      const double sweeps = sw > 0 ? sw : (sw < 0 ? JAC_MAX_SWEEPS : 0);
      fl += sweeps * 0.5 * (double)r.n * (double)(r.n - 1) * 12.0 * (double)r.n;
    } else if (rc == SGT_OK) {
      rc = SGT_ERR_CUDA;
    }
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  if (ms) *ms = tot;
  if (flops) *flops = fl;
  if (launches) *launches = (long long)recs.size();
  return rc;
}
