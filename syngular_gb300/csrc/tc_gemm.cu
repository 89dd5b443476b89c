// Tensor-core GEMM for sm_103a: tcgen05.mma (kind::tf32) with operands staged
// by TMA into 128B-swizzled shared memory and the accumulator in TMEM.
//
//   C (M x N, fp32, row-major) = alpha * sum_pass A_pass * B_pass^T + beta * C
//
// A is M x K and B is N x K, both row-major fp32 ("K-major" for the MMA).
// passes = 1: plain TF32.  passes = 3: split precision, A = A_hi + A_lo and
// B = B_hi + B_lo with hi the TF32-rounded value, accumulating
// A_hi*B_hi + A_hi*B_lo + A_lo*B_hi in FP32 (about 22 significant bits).
//
// One CTA computes a 128 x 128 tile with 6 warps: lane 0 of warp 0 issues the
// TMA loads into a 3-stage ring, lane 0 of warp 1 issues the MMAs, warps 2..5
// drain the accumulator after every 32-wide K chunk (double-buffered in TMEM)
// and add it into FP32 registers, so the tensor-core accumulation never spans
// more than one chunk (its long-K accumulation truncates).  Warp w may only
// touch TMEM lanes 32*(w%4)..+31, which are tile rows.
// Every mbarrier wait has an iteration limit; on expiry the kernel records an
// error code, skips the remaining work, still frees its TMEM and returns.
//
// Split K: with gridDim.z = S > 1, CTA z walks K-tiles [z kps, (z + 1) kps)
// and stores alpha * its partial tile into slice z of a workspace; a second
// kernel adds the S slices in a fixed order into beta * C (deterministic).
// Used when the output has too few 128 x 128 tiles to occupy the GPU.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <vector>

#include "common.cuh"

namespace sgt {

namespace {

constexpr int TC_BM = 128;
constexpr int TC_BN = 128;
constexpr int TC_BK = 32;  // fp32 elements per stage along K = 128 bytes = one swizzle row
constexpr int TC_STAGES = 3;
constexpr int TC_EPI_WARPS = 4;
constexpr int TC_THREADS = 64 + 32 * TC_EPI_WARPS;  // producer warp, MMA warp, 4 accumulator warps
constexpr int TC_TMEM_COLS = 2 * 128;               // two accumulator buffers of TC_BN columns
constexpr int TILE_BYTES = TC_BM * TC_BK * 4;  // 16 KB (A and B tiles have the same size)
constexpr uint32_t WAIT_LIMIT = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred P1;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, P1;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: true when the phase completed, false after WAIT_LIMIT polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < WAIT_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x,
                                            int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, rows of
// 128 bytes, 8-row core groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);      // start address
  d |= (uint64_t)(1) << 16;                    // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)((1024 >> 4) & 0x3FFF) << 32; // stride byte offset between 8-row groups
  d |= (uint64_t)1 << 46;                      // descriptor version
  d |= (uint64_t)2 << 61;                      // SWIZZLE_128B
  return d;
}

// Instruction descriptor: D = f32, A = B = tf32, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
        "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
        "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

struct TcArgs {
  float* C;
  int64_t ldc;
  int M, N, K;
  float alpha, beta;
  int passes;
  int* err;
  int kps;          // K-tiles per split (all of them without a split)
  int64_t pstride;  // elements between the split slices of C
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Warp roles: warp 0 lane 0 issues TMA loads into a TC_STAGES ring; warp 1
// owns TMEM (2 x 128 columns) and lane 0 issues the MMAs; warps 2..5 drain
// each 32-wide K chunk of the accumulator from TMEM into FP32 registers
// (round-to-nearest adds), so the tensor core never accumulates more than one
// chunk.  Two TMEM buffers let the MMA of chunk c+1 overlap the drain of c.
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_tf32_kernel(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mAl,
                        const __grid_constant__ CUtensorMap mB, const __grid_constant__ CUtensorMap mBl,
                        const TcArgs args) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int npass = args.passes;
  const int tiles_per_stage = (npass == 3) ? 4 : 2;
  unsigned char* ring = smem;
  uint64_t* full = reinterpret_cast<uint64_t*>(ring + (size_t)TC_STAGES * tiles_per_stage * TILE_BYTES);
  uint64_t* empty = full + TC_STAGES;
  uint64_t* accf = empty + TC_STAGES;  // accumulator buffer b holds a finished chunk
  uint64_t* acce = accf + 2;           // accumulator buffer b has been drained
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acce + 2);
  __shared__ int s_fail;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * TC_BN;
  const int kt0 = (int)blockIdx.z * args.kps;
  const int KT = min((args.K + TC_BK - 1) / TC_BK - kt0, args.kps);

  if (threadIdx.x == 0) {
    s_fail = 0;
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], TC_EPI_WARPS);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TC_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  auto tile = [&](int stage, int which) -> unsigned char* {
    return ring + ((size_t)stage * tiles_per_stage + which) * TILE_BYTES;
  };

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer ----
      const uint32_t bytes = (uint32_t)tiles_per_stage * TILE_BYTES;
      for (int kt = 0; kt < KT; ++kt) {
        const int s = kt % TC_STAGES;
        const uint32_t ph = (uint32_t)(kt / TC_STAGES) & 1u;
        if (kt >= TC_STAGES && !mbar_wait(&empty[s], ph ^ 1u)) {
          atomicExch(&s_fail, 1);
          break;
        }
        if (*(volatile int*)&s_fail) break;
        mbar_expect_tx(&full[s], bytes);
        const int kx = (kt0 + kt) * TC_BK;
        tma_load_2d(tile(s, 0), &mA, &full[s], kx, m0);
        tma_load_2d(tile(s, 1), &mB, &full[s], kx, n0);
        if (npass == 3) {
          tma_load_2d(tile(s, 2), &mAl, &full[s], kx, m0);
          tma_load_2d(tile(s, 3), &mBl, &full[s], kx, n0);
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer: one K-tile per accumulator chunk ----
      constexpr uint32_t idesc = idesc_tf32(TC_BM, TC_BN);
      for (int kt = 0; kt < KT; ++kt) {
        const int s = kt % TC_STAGES;
        const uint32_t ph = (uint32_t)(kt / TC_STAGES) & 1u;
        const int b = kt & 1, use = kt >> 1;
        if (use >= 1 && !mbar_wait(&acce[b], (uint32_t)(use - 1) & 1u)) {
          atomicExch(&s_fail, 1);
          break;
        }
        if (!mbar_wait(&full[s], ph)) {
          atomicExch(&s_fail, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + (uint32_t)(b * TC_BN);
        const uint32_t a = smem_u32(tile(s, 0)), bb = smem_u32(tile(s, 1));
        const uint32_t al = smem_u32(tile(s, 2)), bl = smem_u32(tile(s, 3));
#pragma unroll
        for (int kk = 0; kk < TC_BK / 8; ++kk) {  // tf32 MMA consumes K = 8 (32 bytes)
          const uint32_t off = kk * 32;
          if (npass == 3) {  // small cross terms first, then hi*hi
            mma_tf32(d, smem_desc(a + off), smem_desc(bl + off), idesc, kk > 0 ? 1u : 0u);
            mma_tf32(d, smem_desc(al + off), smem_desc(bb + off), idesc, 1u);
            mma_tf32(d, smem_desc(a + off), smem_desc(bb + off), idesc, 1u);
          } else {
            mma_tf32(d, smem_desc(a + off), smem_desc(bb + off), idesc, kk > 0 ? 1u : 0u);
          }
        }
        mma_commit(&empty[s]);
        mma_commit(&accf[b]);
      }
    }
    __syncwarp();
  } else {
    // ---- accumulator warps: drain every chunk into registers ----
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    float acc[TC_BN];
#pragma unroll
    for (int i = 0; i < TC_BN; ++i) acc[i] = 0.f;
    bool ok = true;
    for (int kt = 0; kt < KT && ok; ++kt) {
      const int b = kt & 1, use = kt >> 1;
      if (!mbar_wait(&accf[b], (uint32_t)use & 1u)) {
        atomicExch(&s_fail, 1);
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int c0 = 0; c0 < TC_BN; c0 += 32) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * TC_BN + c0), v);
#pragma unroll
        for (int i = 0; i < 32; ++i) acc[c0 + i] += v[i];
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[b]);
    }
    ok = ok && !*(volatile int*)&s_fail;
    const int row = m0 + q * 32 + lane;
    if (ok && row < args.M) {
      float* crow = args.C + (int64_t)blockIdx.z * args.pstride + (int64_t)row * args.ldc + n0;
#pragma unroll
      for (int i = 0; i < TC_BN; ++i) {
        if (n0 + i < args.N) {
          const float r = args.alpha * acc[i];
          crow[i] = (args.beta == 0.f) ? r : fmaf(args.beta, crow[i], r);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS));
  }
  if (threadIdx.x == 0 && s_fail && args.err) atomicExch(args.err, 1);
}

// C = beta C + sum_z part[z] (slices M x N, row-major), z in order.
__global__ void splitk_sum_f32_kernel(const float* __restrict__ part, int S, int64_t M, int64_t N, float beta,
                                      float* __restrict__ C, int64_t ldc) {
  const int64_t mn = M * N;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < mn; i += (int64_t)gridDim.x * blockDim.x) {
    float acc = part[i];
    for (int z = 1; z < S; ++z) acc += part[(int64_t)z * mn + i];
    float* c = C + (i / N) * ldc + (i % N);
    *c = (beta == 0.f) ? acc : fmaf(beta, *c, acc);
  }
}

// cvt.rna.tf32.f32: hi = TF32 rounding of x, lo = x - hi.
__global__ void split_tf32_kernel(const float* __restrict__ x, float* __restrict__ hi,
                                  float* __restrict__ lo, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float v = x[i];
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
    const float fh = __uint_as_float(h);
    hi[i] = fh;
    if (lo) lo[i] = v - fh;
  }
}

// FP64 -> (hi, lo) fp32 pair for 3xTF32 (lo keeps the residual to ~2^-22).
__global__ void split_f64_kernel(const double* __restrict__ x, int64_t ldx, float* __restrict__ hi,
                                 float* __restrict__ lo, int64_t rows, int64_t cols) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows * cols;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / cols, c = i % cols;
    const double v = x[r * ldx + c];
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"((float)v));
    const float fh = __uint_as_float(h);
    hi[i] = fh;
    if (lo) lo[i] = (float)(v - (double)fh);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int get_encode() {
  if (g_encode) return SGT_OK;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  SGT_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
  SGT_REQUIRE(fn && q == cudaDriverEntryPointSuccess, SGT_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return SGT_OK;
}

// rows x K fp32 row-major with leading dimension ld (elements), box 128 x 32.
int make_map(CUtensorMap* map, const float* ptr, int64_t rows, int64_t K, int64_t ld) {
  SGT_REQUIRE((reinterpret_cast<uintptr_t>(ptr) & 15) == 0, SGT_ERR_INVALID,
              "tc_gemm: operand not 16-byte aligned");
  SGT_REQUIRE((ld * 4) % 16 == 0, SGT_ERR_INVALID, "tc_gemm: leading dimension must be a multiple of 4");
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 4)};
  cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)TC_BM};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(ptr), dims, strides, box,
                        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  SGT_REQUIRE(r == CUDA_SUCCESS, SGT_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return SGT_OK;
}

size_t tc_smem_bytes(int passes) {
  const int tps = (passes == 3) ? 4 : 2;
  return 1024 + (size_t)TC_STAGES * tps * TILE_BYTES + 8 * (2 * TC_STAGES + 4) + 16;
}

// Optional event timing of the tensor-core GEMM launches (benchmarks): each
// launch is bracketed by CUDA events recorded on its own stream.
struct ProfRec {
  cudaEvent_t a, b;
  double flops;
};
ProfLog<ProfRec> g_prof;

}  // namespace

// Number of K splits for an M x N x K product with `part_floats` floats of
// workspace: enough 128 x 128 tiles x splits to cover ~148 SMs, at least 8
// K-tiles (256 K) per split, at most 8 splits.
int tc_splits(int64_t M, int64_t N, int64_t K, int64_t part_floats) {
  const int64_t tiles = cdiv(N, TC_BN) * cdiv(M, TC_BM);
  const int64_t kt = cdiv(K, TC_BK);
  if (part_floats <= 0 || tiles >= 120) return 1;
  int64_t S = std::min<int64_t>(std::min<int64_t>(8, cdiv(148, tiles)), kt / 8);
  while (S > 1 && S * M * N > part_floats) --S;
  if (S <= 1) return 1;
  const int64_t kps = cdiv(kt, S);
  return (int)cdiv(kt, kps);
}

int tc_gemm_tf32(cudaStream_t st, int passes, int64_t M, int64_t N, int64_t K, float alpha,
                 const float* Ahi, const float* Alo, int64_t lda, const float* Bhi, const float* Blo,
                 int64_t ldb, float beta, float* C, int64_t ldc, int* err, float* part, int64_t part_floats) {
  SGT_REQUIRE(passes == 1 || passes == 3, SGT_ERR_INVALID, "tc_gemm: passes must be 1 or 3");
  SGT_REQUIRE(M > 0 && N > 0 && K > 0, SGT_ERR_INVALID, "tc_gemm: empty problem");
  SGT_REQUIRE(M < (1ll << 31) && N < (1ll << 31) && K < (1ll << 31), SGT_ERR_INVALID, "tc_gemm: too large");
  SGT_REQUIRE(passes == 1 || (Alo && Blo), SGT_ERR_INVALID, "tc_gemm: split operands missing");
  SGT_TRY(get_encode());
  CUtensorMap ma, mal, mb, mbl;
  SGT_TRY(make_map(&ma, Ahi, M, K, lda));
  SGT_TRY(make_map(&mb, Bhi, N, K, ldb));
  if (passes == 3) {
    SGT_TRY(make_map(&mal, Alo, M, K, lda));
    SGT_TRY(make_map(&mbl, Blo, N, K, ldb));
  } else {
    mal = ma;
    mbl = mb;
  }
  const size_t smem = tc_smem_bytes(passes);
  SGT_CUDA(func_attr_at_least((const void*)tc_gemm_tf32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)tc_smem_bytes(3)));
  const int S = part ? tc_splits(M, N, K, part_floats) : 1;
  const int KTall = (int)cdiv(K, TC_BK);
  const int kps = (int)cdiv(KTall, S);
  TcArgs args{C, ldc, (int)M, (int)N, (int)K, alpha, beta, passes, err, kps, 0};
  if (S > 1) {  // partial tiles into the workspace, summed below
    args.C = part;
    args.ldc = N;
    args.beta = 0.f;
    args.pstride = M * N;
  }
  dim3 grid((unsigned)cdiv(N, TC_BN), (unsigned)cdiv(M, TC_BM), (unsigned)S);
  SGT_REQUIRE(grid.y <= 65535, SGT_ERR_INVALID, "tc_gemm: M too large");
  ProfRec rec{};
  const bool prof = g_prof.active();
  if (prof) {
    SGT_CUDA(cudaEventCreate(&rec.a));
    SGT_CUDA(cudaEventCreate(&rec.b));
    SGT_CUDA(cudaEventRecord(rec.a, st));
  }
  tc_gemm_tf32_kernel<<<grid, TC_THREADS, smem, st>>>(ma, mal, mb, mbl, args);
  SGT_LAUNCHED();
  if (S > 1) {
    splitk_sum_f32_kernel<<<(unsigned)std::min<int64_t>(cdiv(M * N, 256), 152 * 8), 256, 0, st>>>(part, S, M, N,
                                                                                                  beta, C, ldc);
    SGT_LAUNCHED();
  }
  if (prof) {
    SGT_CUDA(cudaEventRecord(rec.b, st));
    rec.flops = 2.0 * (double)M * (double)N * (double)K;
    g_prof.add(rec);
  }
  return SGT_OK;
}

int split_tf32(cudaStream_t st, const float* x, float* hi, float* lo, int64_t n) {
  if (n <= 0) return SGT_OK;
  unsigned g = (unsigned)std::min<int64_t>(cdiv(n, 256), 152 * 16);
  split_tf32_kernel<<<g, 256, 0, st>>>(x, hi, lo, n);
  SGT_LAUNCHED();
  return SGT_OK;
}

int split_f64(cudaStream_t st, const double* x, int64_t ldx, float* hi, float* lo, int64_t rows,
              int64_t cols) {
  if (rows * cols <= 0) return SGT_OK;
  unsigned g = (unsigned)std::min<int64_t>(cdiv(rows * cols, 256), 152 * 16);
  split_f64_kernel<<<g, 256, 0, st>>>(x, ldx, hi, lo, rows, cols);
  SGT_LAUNCHED();
  return SGT_OK;
}

}  // namespace sgt

extern "C" SGT_API int sgt_tc_gemm_f32(int passes, int64_t M, int64_t N, int64_t K, float alpha,
                                       const float* A_hi, const float* A_lo, int64_t lda,
                                       const float* B_hi, const float* B_lo, int64_t ldb, float beta,
                                       float* C, int64_t ldc, int* err, void* stream) {
  return sgt::tc_gemm_tf32(sgt::as_stream(stream), passes, M, N, K, alpha, A_hi, A_lo, lda, B_hi, B_lo,
                           ldb, beta, C, ldc, err, nullptr, 0);
}

extern "C" SGT_API size_t sgt_tc_gemm_f32_workspace_size(int64_t M, int64_t N, int64_t K) {
  const int S = sgt::tc_splits(M, N, K, (int64_t)1 << 40);
  return S > 1 ? (size_t)S * (size_t)M * (size_t)N * sizeof(float) : 0;
}

extern "C" SGT_API int sgt_tc_gemm_f32_ws(int passes, int64_t M, int64_t N, int64_t K, float alpha,
                                          const float* A_hi, const float* A_lo, int64_t lda, const float* B_hi,
                                          const float* B_lo, int64_t ldb, float beta, float* C, int64_t ldc,
                                          int* err, void* ws, size_t ws_bytes, void* stream) {
  return sgt::tc_gemm_tf32(sgt::as_stream(stream), passes, M, N, K, alpha, A_hi, A_lo, lda, B_hi, B_lo,
                           ldb, beta, C, ldc, err, static_cast<float*>(ws), (int64_t)(ws_bytes / sizeof(float)));
}

extern "C" SGT_API int sgt_tc_profile(int enable, double* ms, double* flops, long long* launches) {
  // enable = 1: start recording; 0: stop, synchronise on the recorded events,
  // return the summed kernel time, algorithmic flops and launch count.
  using namespace sgt;
  if (enable) {
    g_prof.on = true;
    return SGT_OK;
  }
  g_prof.on = false;
  const std::vector<ProfRec> recs = g_prof.take();
  double tot = 0.0, fl = 0.0;
  int rc = SGT_OK;
  for (const auto& r : recs) {
    float t = 0.f;
    if (rc == SGT_OK && cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
      tot += t;
      fl += r.flops;
    } else if (rc == SGT_OK) {
      set_error("tc_profile: event timing failed");
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

extern "C" SGT_API int sgt_split_tf32(const float* x, float* hi, float* lo, int64_t n, void* stream) {
  return sgt::split_tf32(sgt::as_stream(stream), x, hi, lo, n);
}
