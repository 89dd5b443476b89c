// FP64-class GEMM on the bf16 tensor cores by exact slicing (oz_gemm.cu) and
// the FP32-pair helpers of the accurate mixed-precision form.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"

namespace sgt {

constexpr int OZ_SLICES = 6;   // bf16 slices per operand row (6 + 5 * 7 = 41 bits, 2^-42 truncation)
constexpr int OZ_KC = 1024;    // longest K range accumulated exactly by one CTA

// ---------------------------------------------------------------------------
// FP32-pair device arithmetic (error-free transformations)
// ---------------------------------------------------------------------------

// s + e = a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (h, l) += a * b for pairs a = (ah, al), b = (bh, bl): the leading product is
// exact (FMA), the cross terms carry the low parts; l collects the errors.
__device__ __forceinline__ void df_fma(float& h, float& l, float ah, float al, float bh, float bl) {
  const float p = ah * bh;
  float pe = fmaf(ah, bh, -p);
  pe = fmaf(ah, bl, pe);
  pe = fmaf(al, bh, pe);
  float s, e;
  two_sum(h, p, s, e);
  h = s;
  l += e + pe;
}

// renormalise a pair so that |l| <= ulp(h) / 2
__device__ __forceinline__ void df_norm(float& h, float& l) {
  const float s = h + l;
  l = l - (s - h);
  h = s;
}

// (h, l) += (bh, bl)
__device__ __forceinline__ void df_add(float& h, float& l, float bh, float bl) {
  float s, e;
  two_sum(h, bh, s, e);
  h = s;
  l += e + bl;
  df_norm(h, l);
}

// S bf16 slices of a rows x K operand (K contiguous): slice j, row r, column k
// at s[j * sstride + r * ld + k]; row r was scaled by 2^(6 - e[r * estride]).
struct OzMat {
  const __nv_bfloat16* s;
  int64_t ld;
  int64_t sstride;
  const int* e;
  int64_t estride;
};

// x (a pair, scaled so that |x| < 64) -> OZ_SLICES integers m_s with
// x = sum_s m_s 2^(-7 s) + r, |m_s| <= 64, |r| <= 2^-36; slice s stored as the
// bf16 value m_s 2^(-7 s) (exact).
__device__ __forceinline__ void slice_store(float h, float l, __nv_bfloat16* out, int64_t sstride, int64_t idx) {
  float m = rintf(h);
  float rh = h - m;  // exact
  float rl = l;
  out[idx] = __float2bfloat16_rn(m);
#pragma unroll
  for (int s = 1; s < OZ_SLICES; ++s) {
    // renormalise (rh, rl) exactly, move up 7 bits, cut the next integer
    const float t = rh + rl;
    const float bb = t - rh;
    rl = (rh - (t - bb)) + (rl - bb);
    rh = t * 128.f;
    rl *= 128.f;
    m = rintf(rh + rl);
    rh = rh - m;  // exact: |rh - m| <= 1/2 + |rl| and m is the integer nearest rh + rl
    out[(int64_t)s * sstride + idx] = __float2bfloat16_rn(ldexpf(m, -7 * s));
  }
}


// slice_store for 4 consecutive values (hi h, lo l, scaled by 2^sh first):
// one 8-byte store per slice; idx a multiple of 4 (8-byte aligned).
__device__ __forceinline__ void slice_store4(float4 h, float4 l, int sh, __nv_bfloat16* out, int64_t sstride,
                                             int64_t idx) {
  const float hv[4] = {h.x, h.y, h.z, h.w}, lv[4] = {l.x, l.y, l.z, l.w};
  float rh[4], rl[4];
  __nv_bfloat16 q[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float hh = ldexpf(hv[j], sh), ll = ldexpf(lv[j], sh);
    const float m = rintf(hh);
    rh[j] = hh - m;  // exact
    rl[j] = ll;
    q[j] = __float2bfloat16_rn(m);
  }
  *reinterpret_cast<uint2*>(out + idx) = *reinterpret_cast<const uint2*>(q);
#pragma unroll
  for (int s = 1; s < OZ_SLICES; ++s) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float t = rh[j] + rl[j];
      const float bb = t - rh[j];
      rl[j] = (rh[j] - (t - bb)) + (rl[j] - bb);
      rh[j] = t * 128.f;
      rl[j] *= 128.f;
      const float m = rintf(rh[j] + rl[j]);
      rh[j] = rh[j] - m;
      q[j] = __float2bfloat16_rn(ldexpf(m, -7 * s));
    }
    *reinterpret_cast<uint2*>(out + (int64_t)s * sstride + idx) = *reinterpret_cast<const uint2*>(q);
  }
}

__device__ __forceinline__ void slice_zero(__nv_bfloat16* out, int64_t sstride, int64_t idx) {
#pragma unroll
  for (int s = 0; s < OZ_SLICES; ++s) out[(int64_t)s * sstride + idx] = __float2bfloat16_rn(0.f);
}

// Slice storage of a rows x cols operand: the leading dimension rounded up to
// a multiple of 8 elements (TMA strides are multiples of 16 bytes).
inline int64_t oz_ld(int64_t cols) { return (cols + 7) / 8 * 8; }
inline size_t oz_slice_elems(int64_t rows, int64_t cols) { return (size_t)OZ_SLICES * rows * oz_ld(cols); }

// C (pair hi/lo, ldc) = alpha * A B^T + beta * C.  `part` (part_floats floats,
// may be null) holds the split-K partials when K > OZ_KC or the output has few
// tiles; oz_gemm_ws_bytes gives the bytes that allow every split the kernel
// wants.  `err` (device int, may be null) is set when a pipeline wait timed out.
// `skip` (device int, may be null): when nonzero at launch time the call does
// nothing (iterations that a device-side test found converged).
// `splits` (may be null): with it, a split-K product leaves its S partials in
// `part` (hi of split z at part[z M N], lo at part[(S + z) M N], row-major
// M x N, alpha applied, beta must be 0) for the caller to add in split order,
// and *splits = S; S = 1 writes C as usual.
int oz_gemm(cudaStream_t st, int64_t M, int64_t N, int64_t K, float alpha, const OzMat& A, const OzMat& B, float beta,
            float* Chi, float* Clo, int64_t ldc, float* part, int64_t part_floats, int* err,
            const int* skip = nullptr, int* splits = nullptr);
size_t oz_gemm_ws_bytes(int64_t M, int64_t N, int64_t K);
// split-K target of products with few output tiles (see sgt_set_tuning)
int oz_set_split_ctas(int v);
int oz_split_ctas();
int oz_set_split_min_ktiles(int v);
int oz_split_min_ktiles();
int oz_profile(int enable, double* ms, double* flops, long long* launches);

// Slice a pair matrix (element (r, c) = hi[r * ld + c] + lo[r * ld + c]; lo
// may be null) into `out` (oz_slice_elems(rows, cols) bf16, slice stride
// rows * oz_ld(cols)) with one exponent per row into e[r * estride].
int oz_split_pair(cudaStream_t st, const float* hi, const float* lo, int64_t ld, int64_t rows, int64_t cols,
                  __nv_bfloat16* out, int* e, int64_t estride, const int* skip = nullptr);
// The same from FP64 with general strides: element (r, c) = x[r * rs + c * cs].
int oz_split_f64(cudaStream_t st, const double* x, int64_t rs, int64_t cs, int64_t rows, int64_t cols,
                 __nv_bfloat16* out, int* e, int64_t estride);

inline OzMat oz_mat(const __nv_bfloat16* s, int64_t rows, int64_t cols, const int* e) {
  return OzMat{s, oz_ld(cols), rows * oz_ld(cols), e, 1};
}

}  // namespace sgt
