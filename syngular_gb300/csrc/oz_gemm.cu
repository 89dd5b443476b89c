// FP64-class GEMM on the bf16 tensor cores (tcgen05 kind::f16) by exact
// slicing, and the FP32-pair ("double-float") helpers around it.
//
//   C (M x N) = alpha * A B^T + beta * C,   A: M x K,  B: N x K  (K contiguous)
//
// Values travel as FP32 pairs hi + lo (|lo| <= ulp(hi) / 2, ~48 significant
// bits): GB300's FP64 pipe is ~1/64 of its FP32 rate, so every elementwise
// step of the accurate forms runs in FP32 error-free arithmetic instead.
//
// Slicing (Ozaki's error-free splitting, with a fixed slice width): row i of
// an operand is scaled by 2^(6 - e_i), e_i the binary exponent of the row's
// largest entry (|x| < 2^e_i), and cut by round-to-nearest into
//   x 2^(6 - e_i) = sum_{s<6} m_s 2^(-7 s) + r,   m_s integers, |m_s| <= 64,
//   |r| <= 2^-36 (so x is kept to 2^-42 of the row's largest entry).
// Slice s is stored in bf16 as m_s 2^(-7 s), which bf16 holds exactly.
//
// The product of slices s of A and t of B is an integer times 2^(-7(s+t)),
// at most 2^12 in magnitude.  The pairs with s + t <= 5 (21 of them)
// accumulate in five TMEM accumulators by level c = min(s + t, 4).  Over a K
// range of at most OZ_KC = 1024, the level-c accumulator (c <= 3) is an
// integer times 2^(-7c) of magnitude at most (c + 1) * 1024 * 2^12 <= 2^24,
// so its FP32 accumulation is exact whatever the tensor core's rounding;
// level 4 gathers the s + t = 4, 5 terms, which carry 2^-28 of the leading
// level's weight, so its FP32 rounding stays near 2^-40 of the result's scale
// (one shared accumulator for levels 3..5 measured 2^-33: its rounding, not
// the slicing, limited the accuracy).
// The epilogue adds the four levels in pair arithmetic and scales by
// 2^(e_i + f_j - 12).  Longer K is split over CTAs (grid z) whose pair
// partials a second kernel adds in a fixed order (deterministic).
//
// Accuracy: about 2^-40 of the row-max times column-max scale per product
// term (level 4's rounding, the dropped s + t = 6 terms and the slice
// remainders), against 2^-22 for split TF32 and 2^-52 for FP64.
//
// CTA: 128 x 96 output tile, 6 warps.  Warp 0 lane 0 issues the TMA loads (a
// 3D map per operand, the slice index is the third coordinate) into a 2-stage
// ring; warp 1 owns TMEM (5 x 96 columns) and lane 0 issues the MMAs; warps
// 2..5 drain the five accumulators once at the end (warp w reads TMEM lanes
// 32 (w % 4)..+31).
// Every mbarrier wait has an iteration limit: on expiry the kernel records
// an error, skips the remaining work, frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "oz.cuh"

namespace sgt {

namespace {

constexpr int OZ_BM = 128;
constexpr int OZ_BN = 96;  // five accumulators of 96 columns fill 480 of TMEM's 512
constexpr int OZ_BK = 32;  // bf16 elements per stage along K = 64 bytes = one 64B-swizzle row
constexpr int OZ_STAGES = 2;
constexpr int OZ_LEVELS = 5;
constexpr int OZ_EPI_WARPS = 4;
constexpr int OZ_THREADS = 64 + 32 * OZ_EPI_WARPS;
constexpr int OZ_TMEM_COLS = 512;  // allocation (a power of two): the whole TMEM of the SM
constexpr int OZ_TILE_A = OZ_BM * OZ_BK * 2;  // 8 KB per A slice tile
constexpr int OZ_TILE_B = OZ_BN * OZ_BK * 2;  // 6 KB per B slice tile
constexpr int OZ_STAGE_BYTES = OZ_SLICES * (OZ_TILE_A + OZ_TILE_B);
static_assert(OZ_LEVELS * OZ_BN <= OZ_TMEM_COLS, "accumulators exceed TMEM");
constexpr uint32_t OZ_WAIT_LIMIT = 1u << 24;

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

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < OZ_WAIT_LIMIT; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// 3D tiled load: box {OZ_BK, 128, 1} at (k, row, slice).
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 64-byte swizzle, rows of
// 64 bytes, 8-row core groups 512 bytes apart.
__device__ __forceinline__ uint64_t smem_desc64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);       // start address
  d |= (uint64_t)(1) << 16;                     // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)((512 >> 4) & 0x3FFF) << 32;   // stride byte offset between 8-row groups
  d |= (uint64_t)1 << 46;                       // descriptor version
  d |= (uint64_t)4 << 61;                       // SWIZZLE_64B
  return d;
}

// Instruction descriptor: D = f32, A = B = bf16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
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

struct OzArgs {
  float* Chi;
  float* Clo;
  int64_t ldc;
  int64_t pstride;  // floats between split-K partial slices (0 without a split)
  const int* ea;    // exponent of row i of A at ea[i * eas]
  const int* eb;
  int64_t eas, ebs;
  int M, N, K;
  float alpha, beta;
  int kps;  // K-tiles per split
  int mfast;  // 1: blockIdx.x walks the M tiles (consecutive CTAs share a B tile), 0: the N tiles
  const int* skip;  // when non-null and nonzero at launch, the launch does nothing
  int* err;
};

// pair (h, l) += v for an exactly representable v (two-sum, then renormalised)
__device__ __forceinline__ void pair_add(float& h, float& l, float v) {
  const float s = h + v;
  const float bb = s - h;
  const float e = (h - (s - bb)) + (v - bb);
  h = s;
  l += e;
}

__global__ void __launch_bounds__(OZ_THREADS, 1)
    oz_gemm_kernel(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB, const OzArgs args) {
  if (args.skip && *args.skip) return;  // uniform for the whole grid, before any barrier or TMEM
  extern __shared__ __align__(1024) unsigned char oz_smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(oz_smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* ring = smem;
  uint64_t* full = reinterpret_cast<uint64_t*>(ring + (size_t)OZ_STAGES * OZ_STAGE_BYTES);
  uint64_t* empty = full + OZ_STAGES;
  uint64_t* accf = empty + OZ_STAGES;  // all MMAs of the tile have completed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accf + 1);
  __shared__ int s_fail;
  __shared__ int s_eb[OZ_BN];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = (args.mfast ? blockIdx.x : blockIdx.y) * OZ_BM;
  const int n0 = (args.mfast ? blockIdx.y : blockIdx.x) * OZ_BN;
  const int kt0 = (int)blockIdx.z * args.kps;
  const int KT = min((args.K + OZ_BK - 1) / OZ_BK - kt0, args.kps);

  if (threadIdx.x == 0) {
    s_fail = 0;
    for (int s = 0; s < OZ_STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accf, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int j = threadIdx.x; j < OZ_BN; j += blockDim.x)
    s_eb[j] = (n0 + j < args.N) ? args.eb[(int64_t)(n0 + j) * args.ebs] : 0;
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(OZ_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  auto tileA = [&](int stage, int s) -> unsigned char* {
    return ring + (size_t)stage * OZ_STAGE_BYTES + (size_t)s * OZ_TILE_A;
  };
  auto tileB = [&](int stage, int s) -> unsigned char* {
    return ring + (size_t)stage * OZ_STAGE_BYTES + (size_t)OZ_SLICES * OZ_TILE_A + (size_t)s * OZ_TILE_B;
  };

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer: all slices of A and B for one K-tile per stage ----
      for (int kt = 0; kt < KT; ++kt) {
        const int s = kt % OZ_STAGES;
        const uint32_t ph = (uint32_t)(kt / OZ_STAGES) & 1u;
        if (kt >= OZ_STAGES && !mbar_wait(&empty[s], ph ^ 1u)) {
          atomicExch(&s_fail, 1);
          break;
        }
        if (*(volatile int*)&s_fail) break;
        mbar_expect_tx(&full[s], (uint32_t)OZ_STAGE_BYTES);
        const int kx = (kt0 + kt) * OZ_BK;
#pragma unroll
        for (int j = 0; j < OZ_SLICES; ++j) {
          tma_load_3d(tileA(s, j), &mA, &full[s], kx, m0, j);
          tma_load_3d(tileB(s, j), &mB, &full[s], kx, n0, j);
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer: the 21 slice pairs of every 16-wide K step ----
      constexpr uint32_t idesc = idesc_bf16(OZ_BM, OZ_BN);
      bool ok = true;
      for (int kt = 0; kt < KT; ++kt) {
        const int s = kt % OZ_STAGES;
        const uint32_t ph = (uint32_t)(kt / OZ_STAGES) & 1u;
        if (!mbar_wait(&full[s], ph)) {
          atomicExch(&s_fail, 1);
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int kk = 0; kk < OZ_BK / 16; ++kk) {  // bf16 MMA consumes K = 16 (32 bytes)
          const uint32_t off = kk * 32;
          // small terms first within each accumulator (level 3 holds s + t = 3, 4, 5)
#pragma unroll
          for (int lv = OZ_SLICES - 1; lv >= 0; --lv) {
#pragma unroll
            for (int a = 0; a <= lv; ++a) {
              const int b = lv - a;
              const int acc = lv < OZ_LEVELS - 1 ? lv : OZ_LEVELS - 1;
              // the first MMA into an accumulator initialises it
              const bool first = (kt == 0 && kk == 0) && (acc < OZ_LEVELS - 1 ? a == 0 : (lv == OZ_SLICES - 1 && a == 0));
              mma_bf16(tmem + (uint32_t)(acc * OZ_BN), smem_desc64(smem_u32(tileA(s, a)) + off),
                       smem_desc64(smem_u32(tileB(s, b)) + off), idesc, first ? 0u : 1u);
            }
          }
        }
        mma_commit(&empty[s]);
      }
      if (ok) mma_commit(accf);
    }
    __syncwarp();
  } else {
    // ---- epilogue: four levels -> FP32 pair, scaled, alpha / beta ----
    const int q = warp & 3;
    bool ok = false;
    for (uint32_t i = 0; KT > 0 && i < OZ_WAIT_LIMIT; ++i) {
      if (mbar_try_wait(accf, 0)) {
        ok = true;
        break;
      }
      if ((i & 1023u) == 1023u && *(volatile int*)&s_fail) break;  // producer / issuer gave up
    }
    ok = __all_sync(0xffffffffu, ok);
    if (!ok) atomicExch(&s_fail, 1);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int row = m0 + q * 32 + lane;
    int ea = 0;
    if (row < args.M) ea = args.ea[(int64_t)row * args.eas];
    const bool split = args.pstride != 0;
    float* chi = args.Chi + (int64_t)blockIdx.z * args.pstride;
    float* clo = args.Clo + (int64_t)blockIdx.z * args.pstride;
    // Without beta, each warp's 32 x 32 block goes out through shared memory
    // (the ring is idle once every MMA has completed): stored row by row, one
    // 128-byte line per instruction, instead of one 4-byte word per row.
    const bool coalesce = split || args.beta == 0.f;
    float* st_h = reinterpret_cast<float*>(ring) + (size_t)q * (2 * 32 * 33);
    float* st_l = st_h + 32 * 33;
#pragma unroll 1
    for (int c0 = 0; c0 < OZ_BN; c0 += 32) {
      float v0[32], v1[32], v2[32], v3[32], v4[32];
      const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0;
      if (ok) {
        tmem_ld32(ta, v0);
        tmem_ld32(ta + OZ_BN, v1);
        tmem_ld32(ta + 2 * OZ_BN, v2);
        tmem_ld32(ta + 3 * OZ_BN, v3);
        tmem_ld32(ta + 4 * OZ_BN, v4);
      } else {
#pragma unroll
        for (int i = 0; i < 32; ++i) v0[i] = v1[i] = v2[i] = v3[i] = v4[i] = 0.f;
      }
      if (!ok || __any_sync(0xffffffffu, *(volatile int*)&s_fail)) continue;  // warp-uniform
      if (coalesce) {
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          float h = v0[i], l = 0.f;
          pair_add(h, l, v1[i]);
          pair_add(h, l, v2[i]);
          pair_add(h, l, v3[i]);
          l += v4[i];
          const float hs = h + l;
          l = l - (hs - h);
          h = hs;
          const float ph = h * args.alpha;
          const float pl = fmaf(h, args.alpha, -ph) + l * args.alpha;
          const int ex = ea + s_eb[c0 + i] - 12;
          st_h[lane * 33 + i] = ldexpf(ph, ex);
          st_l[lane * 33 + i] = ldexpf(pl, ex);
        }
        __syncwarp();
        const int col = n0 + c0 + lane;
        if (col < args.N) {
#pragma unroll 4
          for (int rr = 0; rr < 32; ++rr) {
            const int r2 = m0 + q * 32 + rr;
            if (r2 >= args.M) break;
            const int64_t idx = (int64_t)r2 * args.ldc + col;
            chi[idx] = st_h[rr * 33 + lane];
            clo[idx] = st_l[rr * 33 + lane];
          }
        }
        __syncwarp();
        continue;
      }
      if (row >= args.M) continue;
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const int col = n0 + c0 + i;
        if (col >= args.N) continue;
        // exact: v0 + v1 (integers on grids 1 and 2^-7 up to 2^24), then v2, v3, v4
        float h = v0[i], l = 0.f;
        pair_add(h, l, v1[i]);
        pair_add(h, l, v2[i]);
        pair_add(h, l, v3[i]);
        l += v4[i];
        const float hs = h + l;
        l = l - (hs - h);
        h = hs;
        // alpha (two-product), then the exponent scale (exact power of two)
        const float ph = h * args.alpha;
        const float pl = fmaf(h, args.alpha, -ph) + l * args.alpha;
        const int ex = ea + s_eb[c0 + i] - 12;
        h = ldexpf(ph, ex);
        l = ldexpf(pl, ex);
        const int64_t idx = (int64_t)row * args.ldc + col;
        if (!split && args.beta != 0.f) {
          const float oh = chi[idx], ol = clo[idx];
          const float bh = oh * args.beta;
          const float bl = fmaf(oh, args.beta, -bh) + ol * args.beta;
          pair_add(h, l, bh);
          l += bl;
          const float t = h + l;
          l = l - (t - h);
          h = t;
        }
        chi[idx] = h;
        clo[idx] = l;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(OZ_TMEM_COLS));
  }
  if (threadIdx.x == 0 && s_fail && args.err) atomicExch(args.err, 1);
}

// C = beta C + sum_z part[z] in pair arithmetic, z in order (deterministic).
__global__ void oz_splitk_sum_kernel(const int* __restrict__ skip, const float* __restrict__ ph,
                                     const float* __restrict__ pl, int S, int64_t M,
                                     int64_t N, float beta, float* __restrict__ Chi, float* __restrict__ Clo,
                                     int64_t ldc) {
  if (skip && *skip) return;
  const int64_t mn = M * N;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < mn; i += (int64_t)gridDim.x * blockDim.x) {
    float h = ph[i], l = pl[i];
    for (int z = 1; z < S; ++z) {
      pair_add(h, l, ph[(int64_t)z * mn + i]);
      l += pl[(int64_t)z * mn + i];
    }
    const int64_t c = (i / N) * ldc + (i % N);
    if (beta != 0.f) {
      const float oh = Chi[c], ol = Clo[c];
      const float bh = oh * beta;
      const float bl = fmaf(oh, beta, -bh) + ol * beta;
      pair_add(h, l, bh);
      l += bl;
    }
    const float t = h + l;
    Chi[c] = t;
    Clo[c] = l - (t - h);
  }
}

// One warp per row: exponent of the row's largest |hi|, then the slices.
__global__ void oz_split_pair_kernel(const int* __restrict__ skip, const float* __restrict__ hi,
                                     const float* __restrict__ lo, int64_t ld,
                                     int64_t rows, int64_t cols, __nv_bfloat16* __restrict__ out, int64_t ldo,
                                     int64_t sstride, int* __restrict__ ex, int64_t exs) {
  if (skip && *skip) return;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += warps) {
    const float* hr = hi + r * ld;
    const float* lr = lo ? lo + r * ld : nullptr;
    float mx = 0.f;
    for (int64_t c = lane; c < cols; c += 32) mx = fmaxf(mx, fabsf(hr[c]));
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int e = 0;
    if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);
    if (lane == 0) ex[r * exs] = e;
    for (int64_t c = lane; c < cols; c += 32) {
      const float h = ldexpf(hr[c], 6 - e);
      const float l = lr ? ldexpf(lr[c], 6 - e) : 0.f;
      slice_store(h, l, out, sstride, r * ldo + c);
    }
    for (int64_t c = cols + lane; c < ldo; c += 32) slice_zero(out, sstride, r * ldo + c);
  }
}

// Vector form of the kernel above (cols, ld multiples of 4 and 16-byte aligned
// rows): each lane reads 4 consecutive hi / lo values with one 16-byte load
// and writes each slice's 4 values with one 8-byte store (slice_store4).
__global__ void oz_split_pair4_kernel(const int* __restrict__ skip, const float* __restrict__ hi,
                                      const float* __restrict__ lo, int64_t ld, int64_t rows, int64_t cols,
                                      __nv_bfloat16* __restrict__ out, int64_t ldo, int64_t sstride,
                                      int* __restrict__ ex, int64_t exs) {
  if (skip && *skip) return;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int64_t c4 = cols >> 2;
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += warps) {
    const float4* hr = reinterpret_cast<const float4*>(hi + r * ld);
    const float4* lr = lo ? reinterpret_cast<const float4*>(lo + r * ld) : nullptr;
    float mx = 0.f;
    for (int64_t c = lane; c < c4; c += 32) {
      const float4 h = hr[c];
      mx = fmaxf(mx, fmaxf(fmaxf(fabsf(h.x), fabsf(h.y)), fmaxf(fabsf(h.z), fabsf(h.w))));
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int e = 0;
    if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);
    if (lane == 0) ex[r * exs] = e;
    for (int64_t c = lane; c < c4; c += 32)
      slice_store4(hr[c], lr ? lr[c] : make_float4(0.f, 0.f, 0.f, 0.f), 6 - e, out, sstride, r * ldo + 4 * c);
    for (int64_t c = cols + lane; c < ldo; c += 32) slice_zero(out, sstride, r * ldo + c);
  }
}

// The same from FP64 with general strides (small operands: site cores).
__global__ void oz_split_f64_kernel(const double* __restrict__ x, int64_t rs, int64_t cs, int64_t rows, int64_t cols,
                                    __nv_bfloat16* __restrict__ out, int64_t ldo, int64_t sstride,
                                    int* __restrict__ ex, int64_t exs) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += warps) {
    double mx = 0.0;
    for (int64_t c = lane; c < cols; c += 32) mx = fmax(mx, fabs(x[r * rs + c * cs]));
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int e = 0;
    if (mx > 0.0 && isfinite(mx)) frexp(mx, &e);
    if (lane == 0) ex[r * exs] = e;
    for (int64_t c = lane; c < cols; c += 32) {
      const double v = ldexp(x[r * rs + c * cs], 6 - e);
      const float h = (float)v;
      const float l = (float)(v - (double)h);
      slice_store(h, l, out, sstride, r * ldo + c);
    }
    for (int64_t c = cols + lane; c < ldo; c += 32) slice_zero(out, sstride, r * ldo + c);
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_enc = nullptr;

int get_enc() {
  if (g_enc) return SGT_OK;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  SGT_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
  SGT_REQUIRE(fn && q == cudaDriverEntryPointSuccess, SGT_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  g_enc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return SGT_OK;
}

// rows x K bf16 slices (row stride ld, slice stride sstride, in elements), box 32 x 128 x 1.
int make_slice_map(CUtensorMap* map, const OzMat& m, int64_t rows, int64_t K, int box_rows) {
  SGT_REQUIRE((reinterpret_cast<uintptr_t>(m.s) & 15) == 0, SGT_ERR_INVALID, "oz_gemm: slices not 16-byte aligned");
  SGT_REQUIRE((m.ld * 2) % 16 == 0 && (m.sstride * 2) % 16 == 0 && m.ld >= oz_ld(K), SGT_ERR_INVALID,
              "oz_gemm: row and slice strides must be multiples of 8 elements, rows padded to oz_ld(K)");
  // the padded width: slice rows hold zeros in [K, oz_ld(K)), so the last K-tile reads zeros
  cuuint64_t dims[3] = {(cuuint64_t)oz_ld(K), (cuuint64_t)rows, (cuuint64_t)OZ_SLICES};
  cuuint64_t strides[2] = {(cuuint64_t)(m.ld * 2), (cuuint64_t)(m.sstride * 2)};
  cuuint32_t box[3] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = g_enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16*>(m.s), dims, strides, box,
                     estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  SGT_REQUIRE(r == CUDA_SUCCESS, SGT_ERR_CUDA, "cuTensorMapEncodeTiled (slices) failed (%d)", (int)r);
  return SGT_OK;
}

size_t oz_smem_bytes() { return 1024 + (size_t)OZ_STAGES * OZ_STAGE_BYTES + 8 * (2 * OZ_STAGES + 1) + 16; }

struct OzProf {
  cudaEvent_t a, b;
  double flops;
};
ProfLog<OzProf> g_oz_prof;

}  // namespace

// K splits of an M x N x K product: at least enough for OZ_KC of K per CTA
// (exactness), more while the output has too few tiles to fill the split
// target's CTAs, the splits keep the minimum K-tiles each (default 8 x 32 =
// 256 of K) and the workspace (part_floats) holds them.
// -1 when even the required splits do not fit the workspace.
// CTAs a product with few output tiles is split up to (process-wide tuning,
// sgt_set_tuning(SGT_TUNE_SLICED_SPLIT_CTAS, v)).
// Those splits keep at least this many K-tiles of OZ_BK each
// (SGT_TUNE_SLICED_SPLIT_MIN_KTILES).
static int g_oz_split_ctas = 148;
static int g_oz_split_min_kt = 8;

int oz_set_split_ctas(int v) {
  SGT_REQUIRE(v >= 1 && v <= 4 * 152, SGT_ERR_INVALID, "sliced GEMM split target %d outside [1, 608]", v);
  __atomic_store_n(&g_oz_split_ctas, v, __ATOMIC_RELAXED);
  return SGT_OK;
}
int oz_split_ctas() { return __atomic_load_n(&g_oz_split_ctas, __ATOMIC_RELAXED); }
int oz_set_split_min_ktiles(int v) {
  SGT_REQUIRE(v >= 2 && v <= 32, SGT_ERR_INVALID, "sliced GEMM split K-tiles %d outside [2, 32]", v);
  __atomic_store_n(&g_oz_split_min_kt, v, __ATOMIC_RELAXED);
  return SGT_OK;
}
int oz_split_min_ktiles() { return __atomic_load_n(&g_oz_split_min_kt, __ATOMIC_RELAXED); }

int oz_splits(int64_t M, int64_t N, int64_t K, int64_t part_floats) {
  const int64_t kt = cdiv(K, OZ_BK);
  auto norm = [&](int64_t S) { return cdiv(kt, cdiv(kt, S)); };
  int64_t S = norm(cdiv(K, OZ_KC));
  if (S > 1 && 2 * S * M * N > part_floats) return -1;
  const int64_t tiles = cdiv(N, OZ_BN) * cdiv(M, OZ_BM);
  const int64_t target = oz_split_ctas(), minkt = oz_split_min_ktiles();
  while (tiles * S < target && kt / (S * 2) >= minkt && 2 * norm(2 * S) * M * N <= part_floats) S = norm(2 * S);
  return (int)S;
}

size_t oz_gemm_ws_bytes(int64_t M, int64_t N, int64_t K) {
  const int S = oz_splits(M, N, K, (int64_t)1 << 50);
  return S > 1 ? (size_t)2 * S * M * N * sizeof(float) : 0;
}

int oz_gemm(cudaStream_t st, int64_t M, int64_t N, int64_t K, float alpha, const OzMat& A, const OzMat& B, float beta,
            float* Chi, float* Clo, int64_t ldc, float* part, int64_t part_floats, int* err, const int* skip,
            int* splits) {
  if (M <= 0 || N <= 0) return SGT_OK;
  SGT_REQUIRE(K > 0, SGT_ERR_INVALID, "oz_gemm: empty K");
  SGT_REQUIRE(M < (1ll << 31) && N < (1ll << 31) && K < (1ll << 31), SGT_ERR_INVALID, "oz_gemm: too large");
  SGT_TRY(get_enc());
  CUtensorMap ma, mb;
  SGT_TRY(make_slice_map(&ma, A, M, K, OZ_BM));
  SGT_TRY(make_slice_map(&mb, B, N, K, OZ_BN));
  SGT_CUDA(func_attr_at_least((const void*)oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)oz_smem_bytes()));
  const int S = oz_splits(M, N, K, part ? part_floats : 0);
  SGT_REQUIRE(S >= 1, SGT_ERR_WORKSPACE, "oz_gemm: split-K workspace too small for %lld x %lld x %lld",
              (long long)M, (long long)N, (long long)K);
  SGT_REQUIRE(!splits || S == 1 || beta == 0.f, SGT_ERR_INVALID, "oz_gemm: deferred split-K sum needs beta = 0");
  if (splits) *splits = S;
  const int KTall = (int)cdiv(K, OZ_BK);
  const int kps = (int)cdiv(KTall, S);
  // raster order: the CTAs that share the larger operand's tile run side by
  // side, so that tile is read from DRAM once (the smaller operand stays in L2)
  const int mfast = N > M ? 1 : 0;
  OzArgs args{Chi, Clo, ldc, 0, A.e, B.e, A.estride, B.estride, (int)M, (int)N, (int)K, alpha, beta, kps, mfast,
              skip, err};
  if (S > 1) {
    args.Chi = part;
    args.Clo = part + (int64_t)S * M * N;
    args.ldc = N;
    args.beta = 0.f;
    args.pstride = M * N;
  }
  const unsigned mt = (unsigned)cdiv(M, OZ_BM), nt = (unsigned)cdiv(N, OZ_BN);
  dim3 grid(mfast ? mt : nt, mfast ? nt : mt, (unsigned)S);
  SGT_REQUIRE(grid.y <= 65535, SGT_ERR_INVALID, "oz_gemm: too many tiles along %s", mfast ? "N" : "M");
  OzProf rec{};
  const bool prof = g_oz_prof.active() && !skip;  // a launch that may do nothing is not timed
  if (prof) {
    SGT_CUDA(cudaEventCreate(&rec.a));
    SGT_CUDA(cudaEventCreate(&rec.b));
    SGT_CUDA(cudaEventRecord(rec.a, st));
  }
  oz_gemm_kernel<<<grid, OZ_THREADS, oz_smem_bytes(), st>>>(ma, mb, args);
  SGT_LAUNCHED();
  if (S > 1 && !splits) {
    oz_splitk_sum_kernel<<<(unsigned)std::min<int64_t>(cdiv(M * N, 256), 152 * 8), 256, 0, st>>>(
        skip, part, part + (int64_t)S * M * N, S, M, N, beta, Chi, Clo, ldc);
    SGT_LAUNCHED();
  }
  if (prof) {
    SGT_CUDA(cudaEventRecord(rec.b, st));
    rec.flops = 2.0 * (double)M * (double)N * (double)K;
    g_oz_prof.add(rec);
  }
  return SGT_OK;
}

int oz_split_pair(cudaStream_t st, const float* hi, const float* lo, int64_t ld, int64_t rows, int64_t cols,
                  __nv_bfloat16* out, int* e, int64_t estride, const int* skip) {
  if (rows <= 0 || cols <= 0) return SGT_OK;
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(rows, 8), 152 * 16));
  const bool vec = cols % 4 == 0 && ld % 4 == 0 && (reinterpret_cast<uintptr_t>(hi) & 15) == 0 &&
                   (reinterpret_cast<uintptr_t>(lo) & 15) == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0;
  if (vec)
    oz_split_pair4_kernel<<<g, 256, 0, st>>>(skip, hi, lo, ld, rows, cols, out, oz_ld(cols), rows * oz_ld(cols), e,
                                             estride);
  else
    oz_split_pair_kernel<<<g, 256, 0, st>>>(skip, hi, lo, ld, rows, cols, out, oz_ld(cols), rows * oz_ld(cols), e,
                                            estride);
  SGT_LAUNCHED();
  return SGT_OK;
}

int oz_split_f64(cudaStream_t st, const double* x, int64_t rs, int64_t cs, int64_t rows, int64_t cols,
                 __nv_bfloat16* out, int* e, int64_t estride) {
  if (rows <= 0 || cols <= 0) return SGT_OK;
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(rows, 8), 152 * 16));
  oz_split_f64_kernel<<<g, 256, 0, st>>>(x, rs, cs, rows, cols, out, oz_ld(cols), rows * oz_ld(cols), e, estride);
  SGT_LAUNCHED();
  return SGT_OK;
}

int oz_profile(int enable, double* ms, double* flops, long long* launches) {
  if (enable) {
    g_oz_prof.on = true;
    return SGT_OK;
  }
  g_oz_prof.on = false;
  const std::vector<OzProf> recs = g_oz_prof.take();
  double tot = 0.0, fl = 0.0;
  int rc = SGT_OK;
  for (const auto& r : recs) {
    float t = 0.f;
    if (rc == SGT_OK && cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
      tot += t;
      fl += r.flops;
    } else if (rc == SGT_OK) {
      set_error("sliced_profile: event timing failed");
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

}  // namespace sgt
