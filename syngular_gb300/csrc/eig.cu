// Symmetric eigen-decomposition Z = V diag(lam) V^T of the Gram-form bond
// matrices by two-sided block Jacobi, cluster-resident, FP32 data.
//
// Z_k = M^T M for the bond unfolding M, so rotating Z on both sides is the
// one-sided Jacobi SVD of M carried out through its Gram matrix: convergence
// follows the conditioning of M (one-sided Jacobi applied to Z itself would
// follow that of Z^2).
//
// Layout: the (padded) index range is cut into nb = 2*CS blocks of b rows;
// CTA c of a CS-CTA cluster owns row blocks 2c and 2c+1 of Z and of V in
// shared memory for the whole solve (V holds the eigenvectors as columns).
// One step pairs the blocks by the circle tournament; CTA i solves pair i:
//   1. gather the 2b x 2b subproblem S = Z[I u J, I u J] through DSMEM;
//   2. one cyclic Jacobi sweep on S in shared memory, accumulating Q (2b x 2b);
//   3. cluster barrier; every CTA replaces its row blocks by Q^T [Z_I; Z_J]
//      (partner rows and Q read through DSMEM before a second barrier);
//   4. every CTA updates its rows' columns I u J of Z and V by Q for all pairs
//      (warp per row, lane per column, operands exchanged by shuffles).
// nb-1 steps form one outer sweep; sweeps stop when no subproblem needed a
// rotation, or at the cap (status -1).  Rotation angles in FP32; the caller
// re-orthonormalises the kept eigenvectors in FP64.
#include <cooperative_groups.h>
#include <float.h>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace sgt {

namespace {

constexpr int SJ_THREADS = 256;
constexpr int SJ_WARPS = SJ_THREADS / 32;
constexpr int SJ_MAXB = 16;          // rows per block (2b <= 32: one warp covers a subproblem row)
constexpr int SJ_MAX_SWEEPS = 40;

__device__ __forceinline__ int circle_block(int pos, int step, int nb) {
  return pos == 0 ? 0 : ((pos - 1 + step) % (nb - 1)) + 1;
}

// Shared memory carve (floats): Z rows [2b][ld], V rows [2b][ld], staging
// [2b][ld], S [32][33], Q [32][33], Qc [2][32][33], Qt [32][33].
struct SjSmem {
  float* Z;
  float* V;
  float* St;
  float* S;
  float* Q;
  float* Qc;
  float* Qt;
};

__device__ __forceinline__ SjSmem sj_carve(float* base, int b, int ld) {
  SjSmem m;
  m.Z = base;
  m.V = m.Z + 2 * b * ld;
  m.St = m.V + 2 * b * ld;
  m.S = m.St + 2 * b * ld;
  m.Q = m.S + 32 * 33;
  m.Qc = m.Q + 32 * 33;
  m.Qt = m.Qc + 2 * 32 * 33;
  return m;
}

__global__ void __launch_bounds__(SJ_THREADS) sjacobi_kernel(const float* __restrict__ Zin, int64_t ldz, int n,
                                                             int b, float tol, float* __restrict__ Vout,
                                                             int64_t ldv, float* __restrict__ lam,
                                                             int* __restrict__ status) {
  cg::cluster_group cluster = cg::this_cluster();
  const int cs = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nb = 2 * cs;
  const int np = nb * b;  // padded order
  const int ld = np;      // row stride of Z / V rows in shared memory
  const int w2 = 2 * b;   // subproblem order

  extern __shared__ __align__(16) float sj_raw[];
  SjSmem sm = sj_carve(sj_raw, b, ld);
  __shared__ int s_pair_of[64];   // block -> pair index (this step)
  __shared__ int s_side_of[64];   // block -> 0 (I) or 1 (J)
  __shared__ int s_blkI[32], s_blkJ[32];
  __shared__ int s_active[32];    // pair rotated this step (read remotely from solvers)
  __shared__ int s_rot[2];
  __shared__ float s_rot_param[16][3];

  // ---- load own rows: Z (zero padded) and V = I ----
  for (int i = tid; i < w2 * ld; i += SJ_THREADS) {
    const int r = i / ld, c = i % ld;
    const int g = rank * w2 + r;
    sm.Z[i] = (g < n && c < n) ? Zin[(int64_t)g * ldz + c] : 0.f;
    sm.V[i] = (g == c) ? 1.f : 0.f;
  }
  if (tid < 2) s_rot[tid] = 0;
  // numerically-zero floor for off-diagonals: FLT_EPSILON * max diagonal
  __shared__ float s_dmax;
  if (tid == 0) {
    float m = 0.f;
    for (int r = 0; r < w2; ++r) {
      const int g = rank * w2 + r;
      if (g < np) m = fmaxf(m, fabsf(sm.Z[(int64_t)r * ld + g]));
    }
    s_dmax = m;
  }
  cluster.sync();
  float abs_floor;
  {
    float m = 0.f;
    for (int r = 0; r < cs; ++r) m = fmaxf(m, *cluster.map_shared_rank(&s_dmax, r));
    abs_floor = FLT_EPSILON * m;
  }
  cluster.sync();

  int sweeps = 0;
  bool converged = false;
  while (!converged && sweeps < SJ_MAX_SWEEPS) {
    const int par = sweeps & 1;
    int rotated_here = 0;
    for (int step = 0; step < nb - 1; ++step) {
      // pair table (identical in every CTA)
      if (tid < cs) {
        const int I = circle_block(tid, step, nb), J = circle_block(nb - 1 - tid, step, nb);
        s_blkI[tid] = I;
        s_blkJ[tid] = J;
        s_pair_of[I] = tid;
        s_side_of[I] = 0;
        s_pair_of[J] = tid;
        s_side_of[J] = 1;
      }
      __syncthreads();
      // ---- 1. gather S for pair `rank` ----
      const int I = s_blkI[rank], J = s_blkJ[rank];
      for (int i = tid; i < w2 * w2; i += SJ_THREADS) {
        const int rr = i / w2, cc = i % w2;
        const int rb = rr < b ? I : J, cb = cc < b ? I : J;
        const int owner = rb >> 1, slot = rb & 1;
        const float* zrow = cluster.map_shared_rank(sm.Z, owner) + (int64_t)(slot * b + rr % b) * ld;
        sm.S[rr * 33 + cc] = zrow[cb * b + cc % b];
        sm.Q[rr * 33 + cc] = (rr == cc) ? 1.f : 0.f;
      }
      __syncthreads();
      // ---- 2. one cyclic Jacobi sweep on S (order w2, even) ----
      int any = 0;
      for (int sub = 0; sub < w2 - 1; ++sub) {
        if (tid < b) {
          const int p0 = (tid == 0) ? 0 : ((tid - 1 + sub) % (w2 - 1)) + 1;
          const int q0 = ((w2 - 1 - tid - 1 + sub) % (w2 - 1)) + 1;
          const int p = min(p0, q0), q = max(p0, q0);
          const float app = sm.S[p * 33 + p], aqq = sm.S[q * 33 + q], apq = sm.S[p * 33 + q];
          float c = 1.f, s = 0.f, ta = 0.f;
          if (fabsf(apq) > fmaxf(tol * sqrtf(fabsf(app)) * sqrtf(fabsf(aqq)), abs_floor)) {
            const float tau = (aqq - app) / (2.f * apq);
            const float t = copysignf(1.f, tau) / (fabsf(tau) + sqrtf(fmaf(tau, tau, 1.f)));
            c = 1.f / sqrtf(fmaf(t, t, 1.f));
            s = t * c;
            ta = s / (1.f + c);
            any = 1;
          }
          s_rot_param[tid][0] = c;
          s_rot_param[tid][1] = s;
          s_rot_param[tid][2] = ta;
        }
        __syncthreads();
        // rows: S <- J^T S
        for (int i = tid; i < b * w2; i += SJ_THREADS) {
          const int k = i / w2, col = i % w2;
          const int p0 = (k == 0) ? 0 : ((k - 1 + sub) % (w2 - 1)) + 1;
          const int q0 = ((w2 - 1 - k - 1 + sub) % (w2 - 1)) + 1;
          const int p = min(p0, q0), q = max(p0, q0);
          const float s = s_rot_param[k][1], ta = s_rot_param[k][2];
          if (s == 0.f) continue;
          const float x = sm.S[p * 33 + col], y = sm.S[q * 33 + col];
          sm.S[p * 33 + col] = x - s * (y + ta * x);
          sm.S[q * 33 + col] = y + s * (x - ta * y);
        }
        __syncthreads();
        // columns: S <- S J, Q <- Q J
        for (int i = tid; i < 2 * b * w2; i += SJ_THREADS) {
          const int which = i / (b * w2);
          const int j = i % (b * w2);
          const int k = j / w2, row = j % w2;
          const int p0 = (k == 0) ? 0 : ((k - 1 + sub) % (w2 - 1)) + 1;
          const int q0 = ((w2 - 1 - k - 1 + sub) % (w2 - 1)) + 1;
          const int p = min(p0, q0), q = max(p0, q0);
          const float s = s_rot_param[k][1], ta = s_rot_param[k][2];
          if (s == 0.f) continue;
          float* M = which ? sm.Q : sm.S;
          const float x = M[row * 33 + p], y = M[row * 33 + q];
          M[row * 33 + p] = x - s * (y + ta * x);
          M[row * 33 + q] = y + s * (x - ta * y);
        }
        __syncthreads();
      }
      any = __syncthreads_or(any);
      if (tid == 0) s_active[rank] = any;
      rotated_here += any;
      // ---- 3. row update of own blocks: new = Q[:, side]^T [Z_I; Z_J] ----
      cluster.sync();
      for (int sl = 0; sl < 2; ++sl) {
        const int blk = 2 * rank + sl;
        const int pr = s_pair_of[blk], side = s_side_of[blk];
        const int solver = pr;
        const int active = *cluster.map_shared_rank(&s_active[pr], solver);
        if (!active) continue;  // uniform across the CTA
        const int partner = side == 0 ? s_blkJ[pr] : s_blkI[pr];
        const float* qsrc = cluster.map_shared_rank(sm.Q, solver);
        float* qdst = sm.Qc + sl * 32 * 33;
        for (int i = tid; i < w2 * w2; i += SJ_THREADS) qdst[(i / w2) * 33 + i % w2] = qsrc[(i / w2) * 33 + i % w2];
        const float* prow = cluster.map_shared_rank(sm.Z, partner >> 1) + (int64_t)((partner & 1) * b) * ld;
        float* st = sm.St + (int64_t)sl * b * ld;
        for (int i = tid; i < b * ld; i += SJ_THREADS) st[i] = prow[i];
      }
      cluster.sync();  // everyone holds the old partner rows locally now
      for (int sl = 0; sl < 2; ++sl) {
        const int blk = 2 * rank + sl;
        const int pr = s_pair_of[blk], side = s_side_of[blk];
        const int active = *cluster.map_shared_rank(&s_active[pr], pr);
        if (!active) continue;
        const float* q = sm.Qc + sl * 32 * 33;
        float* own = sm.Z + (int64_t)sl * b * ld;
        const float* oth = sm.St + (int64_t)sl * b * ld;
        // rows of I are the first b rows of [Z_I; Z_J]
        const float* zi = side == 0 ? own : oth;
        const float* zj = side == 0 ? oth : own;
        // column by column: thread handles column `col` for all b output rows
        for (int col = tid; col < ld; col += SJ_THREADS) {
          float in[2 * SJ_MAXB];
#pragma unroll
          for (int r = 0; r < SJ_MAXB; ++r) {
            in[r] = r < b ? zi[(int64_t)r * ld + col] : 0.f;
            in[SJ_MAXB + r] = r < b ? zj[(int64_t)r * ld + col] : 0.f;
          }
          for (int r = 0; r < b; ++r) {
            float acc = 0.f;
            const int qc = side * b + r;
#pragma unroll
            for (int k = 0; k < SJ_MAXB; ++k) {
              if (k < b) {
                acc = fmaf(q[k * 33 + qc], in[k], acc);
                acc = fmaf(q[(b + k) * 33 + qc], in[SJ_MAXB + k], acc);
              }
            }
            own[(int64_t)r * ld + col] = acc;
          }
        }
      }
      __syncthreads();
      // ---- 4. column update of own rows (Z and V) for every active pair ----
      for (int pr = 0; pr < cs; ++pr) {
        const int active = *cluster.map_shared_rank(&s_active[pr], pr);
        if (!active) continue;
        const float* qsrc = cluster.map_shared_rank(sm.Q, pr);
        for (int i = tid; i < w2 * w2; i += SJ_THREADS) sm.Qt[(i / w2) * 33 + i % w2] = qsrc[(i / w2) * 33 + i % w2];
        __syncthreads();
        const int Ib = s_blkI[pr], Jb = s_blkJ[pr];
        // warp per row of [Z rows; V rows], lane per column of I u J
        for (int rr = warp; rr < 2 * w2; rr += SJ_WARPS) {
          float* row = (rr < w2 ? sm.Z : sm.V) + (int64_t)(rr % w2) * ld;
          const int colg = lane < w2 ? ((lane < b ? Ib : Jb) * b + lane % b) : 0;
          const float x = lane < w2 ? row[colg] : 0.f;
          float acc = 0.f;
#pragma unroll 8
          for (int k = 0; k < 32; ++k) {
            const float xk = __shfl_sync(0xffffffffu, x, k);
            if (k < w2 && lane < w2) acc = fmaf(xk, sm.Qt[k * 33 + lane], acc);
          }
          if (lane < w2) row[colg] = acc;
        }
        __syncthreads();
      }
      cluster.sync();  // rows final before the next gather
    }
    if (tid == 0) atomicAdd(&s_rot[par], rotated_here > 0 ? 1 : 0);
    __syncthreads();
    cluster.sync();
    int total = 0;
    for (int r = 0; r < cs; ++r) total += *cluster.map_shared_rank(&s_rot[par], r);
    ++sweeps;
    converged = (total == 0);
    cluster.sync();
    if (tid == 0) s_rot[par] = 0;
  }
  // ---- eigenvalues (diagonal) and V rows out ----
  for (int r = tid; r < w2; r += SJ_THREADS) {
    const int g = rank * w2 + r;
    if (g < n) lam[g] = sm.Z[(int64_t)r * ld + g];
  }
  for (int i = tid; i < w2 * ld; i += SJ_THREADS) {
    const int r = i / ld, c = i % ld;
    const int g = rank * w2 + r;
    if (g < n && c < n) Vout[(int64_t)g * ldv + c] = sm.V[i];
  }
  if (rank == 0 && tid == 0 && status) *status = converged ? sweeps : -1;
  cluster.sync();
}

// rank by descending lam (ties by index), then Vt[rank] = column j of V, lam sorted
__global__ void sj_rank_kernel(const float* __restrict__ lam, int n, int* __restrict__ perm) {
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const float v = lam[j];
    int r = 0;
    for (int i = 0; i < n; ++i) {
      const float w = lam[i];
      r += (w > v) || (w == v && i < j);
    }
    perm[j] = r;
  }
}

// Vt[perm[j]][i] = V[i][j]
__global__ void sj_gather_kernel(const float* __restrict__ V, int64_t ldv, int n, const int* __restrict__ perm,
                                 const float* __restrict__ lam, float* __restrict__ Vt, int64_t ldt,
                                 float* __restrict__ lam_sorted) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (int64_t)n * n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx / n), j = (int)(idx % n);
    Vt[(int64_t)perm[j] * ldt + i] = V[(int64_t)i * ldv + j];
    if (i == 0) lam_sorted[perm[j]] = lam[j];
  }
}

}  // namespace

size_t sym_eig_ws_bytes(int64_t n) {
  Arena a = Arena::measuring();
  a.take<float>((size_t)n * n);
  a.take<float>((size_t)n);
  a.take<int>((size_t)n);
  return a.used;
}

// Eigen-decomposition of symmetric Z (n x n fp32, ld): Vt rows = eigenvectors
// by descending eigenvalue, lam = eigenvalues (descending).  Returns
// SGT_ERR_UNSUPPORTED_SIZE (nonzero) when n does not fit the cluster kernel.
int sym_eig_f32(cudaStream_t st, const float* Z, int64_t ldz, int64_t n, float* Vt, int64_t ldt, float* lam,
                int* status, Arena& ar, bool* done) {
  *done = false;
  if (n < 64 || n > 1024) return SGT_OK;
  int cs = 2;
  while (cs < 16 && cdiv(n, 2 * cs) > SJ_MAXB) cs *= 2;
  const int64_t b = cdiv(n, 2 * cs);
  if (b > SJ_MAXB) return SGT_OK;
  const int64_t ld = 2 * cs * b;
  const size_t smem = sizeof(float) * ((size_t)3 * 2 * b * ld + 5 * 32 * 33);
  if (smem > 227 * 1024) return SGT_OK;
  float* V = ar.take<float>((size_t)n * n);
  float* lraw = ar.take<float>((size_t)n);
  int* perm = ar.take<int>((size_t)n);
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "sym_eig: workspace too small");
  SGT_CUDA(func_attr_at_least((const void*)sjacobi_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  // dynamic + static shared memory must stay within the per-block opt-in limit
  if (func_attr_at_least((const void*)sjacobi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return SGT_OK;  // does not fit here: the caller uses the one-sided kernel
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cs, 1, 1);
  cfg.blockDim = dim3(SJ_THREADS, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cs;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, sjacobi_kernel, &cfg) != cudaSuccess || clusters < 1) {
    cudaGetLastError();
    return SGT_OK;
  }
  const float tol = 16.f * FLT_EPSILON;
  SGT_CUDA(cudaLaunchKernelEx(&cfg, sjacobi_kernel, Z, ldz, (int)n, (int)b, tol, V, (int64_t)n, lraw, status));
  note_launch();
  sj_rank_kernel<<<1, 256, 0, st>>>(lraw, (int)n, perm);
  SGT_LAUNCHED();
  const unsigned g = (unsigned)std::min<int64_t>(cdiv(n * n, 256), 152 * 8);
  sj_gather_kernel<<<g, 256, 0, st>>>(V, n, (int)n, perm, lraw, Vt, ldt, lam);
  SGT_LAUNCHED();
  *done = true;
  return SGT_OK;
}

}  // namespace sgt

namespace sgt {
size_t jacobi_rows_ws_bytes_f32(int64_t n, int64_t m);
size_t sym_eig_rows_ws_bytes(int64_t n);
int sym_eig_rows_f32(cudaStream_t st, float* Z, int64_t n, float* Vt, float* lam, int* status, Arena& ar,
                     int method);
}  // namespace sgt

extern "C" SGT_API size_t sgt_sym_eig_f32_workspace_size(int64_t n) {
  return std::max(sgt::sym_eig_ws_bytes(n) + sgt::jacobi_rows_ws_bytes_f32(n, n) + 256 * 4 + sizeof(float) * n * n,
                  sgt::sym_eig_rows_ws_bytes(n));
}

// Eigen-decomposition of a symmetric positive semi-definite FP32 matrix Z
// (n x n, row-major; Z is overwritten): Vt rows = eigenvectors, lam descending.
// method 0: two-sided block Jacobi in one cluster (falls back to 1 when n does
// not fit); method 1: one-sided Jacobi on the rows of Z; method 2: Jacobi on
// the rows of Z's diagonal-ordered Cholesky factor (vectors by normalisation);
// method 3: on the columns of that factor with the rotations accumulated.
extern "C" SGT_API int sgt_sym_eig_f32(float* Z, int64_t n, float* Vt, float* lam, int* status, int method,
                                       void* ws, size_t ws_bytes, void* stream) {
  using namespace sgt;
  SGT_REQUIRE(Z && Vt && lam && n > 0, SGT_ERR_INVALID, "sym_eig: bad argument");
  SGT_REQUIRE(method >= 0 && method <= 3, SGT_ERR_INVALID, "sym_eig: method must be 0..3");
  cudaStream_t st = as_stream(stream);
  Arena ar(ws, ws_bytes);
  bool done = false;
  if (method == 0) SGT_TRY(sym_eig_f32(st, Z, n, n, Vt, n, lam, status, ar, &done));
  if (!done) {
    Arena a2(ws, ws_bytes);
    SGT_TRY(sym_eig_rows_f32(st, Z, n, Vt, lam, status, a2, method));
  }
  return SGT_OK;
}
