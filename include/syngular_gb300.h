/*
 * syngular_gb300 -- C ABI of the GB300 (sm_103a) matrix-product library.
 *
 * Conventions
 *   - Every pointer argument named for a core, matrix or result is a DEVICE
 *     pointer, except arrays of pointers/shapes (`const double* const* cores`,
 *     `const int64_t* shape`), which live in HOST memory and hold device
 *     pointers / sizes.
 *   - Cores are dense row-major: MPS core (l, p, r); MPO core (l, in, out, r).
 *     Where an operation treats an MPO core as an MPS core (rounding,
 *     orthonormalisation, overlap of vectorised operators) it passes
 *     p = in * out, exactly as the reference's left matricization does.
 *   - `shape` arrays are flattened triples (l_k, p_k, r_k), k = 0..n-1.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *     asynchronous unless stated otherwise; they never synchronise the device.
 *   - Scratch memory is caller-provided: query `*_workspace_size`, pass a
 *     device buffer of at least that many bytes (256-byte aligned).  The
 *     library allocates nothing and frees nothing.
 *   - Return value: SGT_OK or an SGT_ERR_* code; `sgt_last_error()` gives the
 *     message of the last failure on the calling thread.  No C++ exception
 *     crosses this boundary.
 *
 * Each entry point names the reference function (antoine311200/Syngular,
 * path:line) it replaces.  Reference paths: mps = tensor/matrix_product_state.py,
 * mpo = tensor/matrix_product_operator.py.
 */
#ifndef SYNGULAR_GB300_H
#define SYNGULAR_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SGT_API __attribute__((visibility("default")))
#else
#define SGT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define SGT_OK 0
#define SGT_ERR_INVALID 1        /* bad argument (shape mismatch, null pointer, ...) */
#define SGT_ERR_NOT_CONVERGED 2  /* an iterative kernel hit its sweep cap */
#define SGT_ERR_CUDA 3           /* a CUDA runtime call failed */
#define SGT_ERR_WORKSPACE 4      /* workspace smaller than the size query returned */
#define SGT_ERR_SHAPE 5          /* the reference would fail to reshape (e.g. l*p < dim) */

/* Arithmetic of the rounding / contraction entry points that take a `precision`. */
#define SGT_PREC_F64 0     /* plain FP64 everywhere */
#define SGT_PREC_TF32 1    /* GEMM-shaped work on tcgen05 kind::tf32, FP32 accumulate */
#define SGT_PREC_BF16 2    /* reserved, rejected with SGT_ERR_INVALID (see SGT_PREC_BF16X3) */
#define SGT_PREC_BF16X3 3  /* reserved, rejected with SGT_ERR_INVALID: a split bf16 product keeps
                              ~16 mantissa bits (~1.5e-5), short of the ~1e-7 that the Gram form's
                              squared spectrum needs; the split-tf32 form below keeps ~22 bits */
#define SGT_PREC_TF32X3 4  /* split tf32 (hi*hi + hi*lo + lo*hi) on tcgen05, FP32 accumulate */
#define SGT_PREC_BF16X6 5  /* FP64-class: every operand row cut exactly into six 7-bit bf16 slices,
                              the 21 leading slice products on tcgen05 kind::f16 accumulated exactly
                              in TMEM (~2^-41 of the operands' scale); elementwise work in FP32 pairs;
                              kept subspaces by purification on that GEMM (or, when spectra are asked
                              for, FP32 Jacobi eigenvectors refined against the pair-accurate bond
                              matrix) */

SGT_API int sgt_version(void);
SGT_API const char* sgt_last_error(void);
/* Number of kernels this library has launched in the process so far. */
SGT_API unsigned long long sgt_launch_count(void);

/* ----------------------------------------------------------------------
 * Site contractions (raw products, no rounding)
 * -------------------------------------------------------------------- */

/* MPO x MPS site: P[(a,b), o, (a2,b2)] = sum_i X[a,i,a2] * W[b,i,o,b2],
 * fused bond index a*B + b.  Replaces the per-site `contract` of
 * MatrixProductOperator.__matmul__ (mpo:183-191). */
SGT_API int sgt_site_contract_mpo_mps(const double* X, int64_t a, int64_t p, int64_t a2,
                              const double* W, int64_t b, int64_t o, int64_t b2,
                              double* P, void* stream);

/* MPO x MPO site: P[(b,c), i, o, (b2,c2)] = sum_m A[b,i,m,b2] * B[c,m,o,c2],
 * fused bond index b*C + c.  Replaces mpo:279-288 (output leg uses B's
 * `out`, where the reference's reshape assumes A.out == B.out). */
SGT_API int sgt_site_contract_mpo_mpo(const double* A, int64_t b, int64_t i, int64_t m, int64_t b2,
                              const double* B, int64_t c, int64_t o, int64_t c2,
                              double* P, void* stream);

/* ----------------------------------------------------------------------
 * Direct sum (bond concatenation) -- MatrixProductState.__add__ (mps:75-100),
 * MatrixProductOperator.__add__ (mpo:84-108).
 * position: 0 = first site ([A | B] along r), 1 = middle (block diagonal),
 *           2 = last site (stacked along l), 3 = single-site chain (A + B).
 * Output shape: first (la, phys, ra+rb), middle (la+lb, phys, ra+rb),
 *               last (la+lb, phys, ra), single (la, phys, ra).
 * -------------------------------------------------------------------- */
SGT_API int sgt_bond_concat(const double* A, int64_t la, int64_t phys, int64_t ra,
                    const double* B, int64_t lb, int64_t rb, int position,
                    double* out, void* stream);

/* All sites of a chain in one launch (same layout rules as above). */
SGT_API int sgt_bond_concat_chain(int n, const double* const* A, const int64_t* ashape,
                          const double* const* B, const int64_t* bshape,
                          double* const* out, void* ws, size_t ws_bytes, void* stream);
SGT_API size_t sgt_bond_concat_chain_workspace_size(int n);

/* ----------------------------------------------------------------------
 * Overlap <X|Y> without conjugation -- MatrixProductState.__or__ (mps:116-127).
 * Transfer sweep E_{k+1} = sum_p X_k[:,p,:]^T E_k Y_k[:,p,:] with per-site
 * rescaling by exact powers of two.  `result` (device, 2 doubles) receives
 * (mantissa, exponent) with the exponent an integer held in a double:
 * <X|Y> = mantissa * 2^exponent, i.e. ldexp(mantissa, (int)exponent) in C.
 * -------------------------------------------------------------------- */
SGT_API size_t sgt_overlap_workspace_size(int n, const int64_t* xshape, const int64_t* yshape);
SGT_API int sgt_overlap_sweep(int n, const double* const* X, const int64_t* xshape,
                      const double* const* Y, const int64_t* yshape,
                      double* result, void* ws, size_t ws_bytes, void* stream);

/* The same overlap in a chosen arithmetic (precision SGT_PREC_F64: exactly
 * sgt_overlap_sweep; SGT_PREC_BF16X6: both contractions of every transfer
 * step on the sliced bf16 tensor-core GEMM, FP64-class, the transfer matrix
 * kept in FP64 and rescaled by exact powers of two; other codes are rejected).
 * Replaces MatrixProductState.__or__ (mps:116-127) under the precision policy.
 * Result as for sgt_overlap_sweep. */
SGT_API size_t sgt_overlap_prec_workspace_size(int n, const int64_t* xshape, const int64_t* yshape,
                                               int precision);
SGT_API int sgt_overlap_sweep_prec(int n, const double* const* X, const int64_t* xshape,
                                   const double* const* Y, const int64_t* yshape, int precision,
                                   double* result, void* ws, size_t ws_bytes, void* stream);

/* Overlap <X|Y> that allocates nothing and takes no workspace.  It has no
 * counterpart in the reference.  It serves callers that cannot give the
 * library scratch memory -- e.g. a C/ctypes binding whose process leaves all
 * device memory to another framework's pool, or a loop that must not
 * allocate.  Its scratch is a fixed ~9.4 MB device array inside the library
 * (held on every GPU that loads it until exit), so every bond must be <= 256
 * and every physical leg <= 16; larger chains are rejected with
 * SGT_ERR_INVALID (use sgt_overlap_sweep).  The first call on a device looks
 * up that array's device address (make it before any stream capture).  All
 * calls share the array: calls that overlap on the GPU (other streams or host
 * threads) race and must be serialised by the caller.  Result as for
 * sgt_overlap_sweep: (mantissa, exponent), <X|Y> = ldexp(mantissa, exponent). */
SGT_API int sgt_overlap_sweep_noalloc(int n, const double* const* X, const int64_t* xshape,
                                      const double* const* Y, const int64_t* yshape,
                                      double* result, void* stream);

/* ----------------------------------------------------------------------
 * Reference rounding `>> dim` = compress(dim, strict=True), left mode
 * (mps:432-468, mpo:544-580): for k = 0..n-2, complete Householder QR of the
 * left unfolding L_k, core_k <- Q[:, :dim], core_{k+1} <- R[:dim, :] @ R_{k+1}.
 * The caller applies the early exit (dim >= min(bond_shape), mps:367) itself.
 * `out[k]` must hold (l'_k, p_k, r'_k) with r'_k = dim (k < n-1), l'_k = dim
 * (k > 0).  Returns SGT_ERR_SHAPE when some l'_k * p_k < dim.
 * -------------------------------------------------------------------- */
SGT_API size_t sgt_qr_truncate_workspace_size(int n, const int64_t* shape, int64_t dim);
SGT_API int sgt_qr_truncate_sweep(int n, const double* const* cores, const int64_t* shape, int64_t dim,
                          double* const* out, void* ws, size_t ws_bytes, void* stream);

/* ----------------------------------------------------------------------
 * Dense tensor -> cores: decompose (mps:296-350, mpo:418-453).
 * `tensor` holds prod(phys) doubles in row-major order of the (already
 * interleaved, for an operator) site legs; bonds has n-1 entries.  out[k] has
 * shape (bonds[k-1], phys[k], bonds[k]).  mode 0 = "left" (truncated complete
 * QR sweep from the first site), 1 = "right" (from the last site on the
 * transposed unfoldings, mps:324-347).
 * -------------------------------------------------------------------- */
SGT_API size_t sgt_decompose_workspace_size(int n, const int64_t* phys, const int64_t* bonds,
                                            int mode);
SGT_API int sgt_decompose(const double* tensor, int n, const int64_t* phys, const int64_t* bonds,
                          int mode, double* const* out, void* ws, size_t ws_bytes, void* stream);

/* Divide a core by its Frobenius norm in place -- normalize (mps:252-256).
 * `norm` (device, 1 double) receives the norm. */
SGT_API int sgt_normalize(double* core, int64_t count, double* norm, void* stream);

/* ----------------------------------------------------------------------
 * In-place left / right orthonormalisation -- left_orthonormalization
 * (mps:554-566, mpo:673-694), right_orthonormalization (mps:568-580,
 * mpo:696-719).  Shapes are kept (the reference requires l*p >= r, resp.
 * p*r >= l; SGT_ERR_SHAPE otherwise).
 * -------------------------------------------------------------------- */
SGT_API size_t sgt_orthonormalize_workspace_size(int n, const int64_t* shape);
SGT_API int sgt_left_orthonormalize(int n, double* const* cores, const int64_t* shape,
                            void* ws, size_t ws_bytes, void* stream);
SGT_API int sgt_right_orthonormalize(int n, double* const* cores, const int64_t* shape,
                             void* ws, size_t ws_bytes, void* stream);

/* Gram matrix of one core -- left_orthogonality (mps:624-626) with side 0:
 * out (r x r) = L^T L, L = (l*p, r); right_orthogonality (mps:628-630) with
 * side 1: out (l x l) = R R^T, R = (l, p*r). */
SGT_API int sgt_orthogonality(const double* core, int64_t l, int64_t p, int64_t r, int side,
                      double* out, void* stream);

/* ----------------------------------------------------------------------
 * TT-SVD rounding to bond chi (no reference counterpart: the reference's `>>`
 * is the QR truncation above).  Left Householder-QR sweep (bonds reduced to
 * the left rank bound), then right-to-left truncated SVD via one-sided Jacobi.
 * `out_shape` (3n) is filled by sgt_svd_round_shapes.  `spectra` (device,
 * may be NULL) receives, bond after bond k = 1..n-1, the full singular
 * values of that bond's unfolding (sgt_svd_round_shapes gives the counts in
 * `spec_count`); `discarded` (device, n-1 doubles, may be NULL) the
 * discarded weight sum(dropped s^2)/sum(s^2) per bond.  `status` (device
 * int, may be NULL) receives the largest Jacobi sweep count over the bonds,
 * or -1 if some bond's Jacobi SVD reached its sweep cap.
 * -------------------------------------------------------------------- */
SGT_API int sgt_svd_round_shapes(int n, const int64_t* shape, int64_t chi, int64_t* out_shape,
                         int64_t* spec_count);
SGT_API size_t sgt_svd_round_workspace_size(int n, const int64_t* shape, int64_t chi, int precision);
SGT_API int sgt_svd_round(int n, const double* const* cores, const int64_t* shape, int64_t chi,
                  int precision, double* const* out, double* spectra, double* discarded,
                  int* status, void* ws, size_t ws_bytes, void* stream);

/* ----------------------------------------------------------------------
 * The metric operation: raw MPO x MPS product (W @ X without the reference's
 * auto-round, mpo:183-191) followed by TT-SVD rounding to chi, in one call.
 * wshape: 4n entries (b, in, out, b2) per operator core; xshape: 3n entries.
 * Output cores (chi_k, out_k, chi_{k+1}) as given by sgt_svd_round_shapes on
 * the product shapes (a*b, out, a2*b2); spectra / discarded / status as for
 * sgt_svd_round (status -2: a tensor-core pipeline wait timed out).
 * precision SGT_PREC_F64: plain FP64 (product + Householder QR sweep + Jacobi).
 * SGT_PREC_TF32 / SGT_PREC_TF32X3: Gram form on tcgen05 -- product cores and
 * left Gram matrices in FP32, every O(R^3) step a TF32 (one pass) or split
 * 3xTF32 GEMM, eigen-solves by one-sided Jacobi (FP32 columns, FP64 angles).
 * SGT_PREC_BF16X6: the same Gram-form algebra at FP64-class accuracy -- every
 * O(R^3) step the sliced bf16 GEMM below (sgt_gemm_f64_sliced), Gram matrices
 * and intermediates in FP32 pairs, each bond's FP32 Jacobi eigenvectors
 * refined by two Ogita-Aishima steps against the pair-accurate bond matrix;
 * product cores are sliced site by site and never stored whole.  With
 * `spectra` NULL no eigensolve runs: each bond's kept subspace is the range of
 * the projector that trace-correcting purification (X <- X^2 or 2X - X^2 on
 * the sliced GEMM, at most 90 steps, stopped on the device once X^2 = X to
 * 2^-34) makes from the bond matrix, its basis the rows of L^T X (L the
 * pivoted Cholesky factor of X) made orthonormal by Newton-Schulz steps; a
 * bond where nothing is cut takes the identity.  The rounded state depends on
 * the kept subspaces only, so both variants give the same state.
 * -------------------------------------------------------------------- */
SGT_API size_t sgt_mpo_mps_round_workspace_size(int n, const int64_t* wshape, const int64_t* xshape,
                                                int64_t chi, int precision);
SGT_API int sgt_mpo_mps_round(int n, const double* const* W, const int64_t* wshape,
                              const double* const* X, const int64_t* xshape, int64_t chi,
                              int precision, double* const* out, double* spectra,
                              double* discarded, int* status, void* ws, size_t ws_bytes,
                              void* stream);

/* ----------------------------------------------------------------------
 * Zip-up MPO x MPS (Stoudenmire & White 2010): W X compressed to bond chi
 * site by site from the left, never forming the product cores or their
 * chi*D bonds.  A carry C (the compressed left part) moves right; at site k
 * M[(r, o), (a', b')] = sum C[r, (a, b)] X_k[a, i, a'] W_k[b, i, o, b'] is
 * split by a truncated FP64 SVD (Householder QR + one-sided Jacobi on the
 * triangular factor): core k = the leading left singular vectors, the carry
 * = S V^T.  Approximate unless chi covers every bond's rank; near the
 * optimal truncation when X is right-orthonormal (the Python API
 * right-orthonormalises a copy).  The reference lists unfinished modes for
 * this (MATMUL_MODE "variational"/"fit-up", mpo:262-276); no reference
 * result to match.  Shapes: out[k] = (r_k, out_k, r_{k+1}) from
 * sgt_mpo_mps_zipup_shapes; `discarded` (device, n-1 doubles, may be NULL):
 * sum of dropped s^2 / sum s^2 at each bond's SVD; `status` (device int, may
 * be NULL): largest Jacobi sweep count, -1 at a sweep cap.
 * -------------------------------------------------------------------- */
SGT_API int sgt_mpo_mps_zipup_shapes(int n, const int64_t* wshape, const int64_t* xshape, int64_t chi,
                                     int64_t* out_shape);
SGT_API size_t sgt_mpo_mps_zipup_workspace_size(int n, const int64_t* wshape, const int64_t* xshape,
                                                int64_t chi);
SGT_API int sgt_mpo_mps_zipup(int n, const double* const* W, const int64_t* wshape, const double* const* X,
                              const int64_t* xshape, int64_t chi, double* const* out, double* discarded,
                              int* status, void* ws, size_t ws_bytes, void* stream);

/* ----------------------------------------------------------------------
 * DMRG environment blocks (variational/dmrg.py:65-112, DMRG.__left_blocks /
 * DMRG.__right_blocks) and the two-site effective contraction
 * (variational/dmrg.py:143-165, the `site` tensor of each sweep step).
 *
 * Shapes: `wshape` holds quadruples (b, in, out, b') per site; `xshape` (the
 * bra, contracted with the operator's OUT leg) and `yshape` (the ket,
 * contracted with its IN leg) hold triples.  The reference passes the same
 * state for both (dmrg.py:78-81).
 *   side 0: blocks[k] = L_k (x_r, w_r, y_r) for k = 0..count-1,
 *           L_k[a',b',c'] = sum L_{k-1}[a,b,c] X_k[a,o,a'] W_k[b,i,o,b'] Y_k[c,i,c']
 *   side 1: blocks[k] = R_k (x_l, w_l, y_l) for k = n-1 down to n-count,
 *           R_k[a,b,c] = sum X_k[a,o,a'] W_k[b,i,o,b'] Y_k[c,i,c'] R_{k+1}[a',b',c']
 * with the unit 1x1x1 block beyond the chain ends.  The reference computes
 * count = n-2 blocks on each side.  `blocks` is an array of n device pointers
 * (entries outside the computed range are ignored).  Plain FP64, no
 * rescaling.
 * -------------------------------------------------------------------- */
SGT_API size_t sgt_env_blocks_workspace_size(int n, const int64_t* wshape, const int64_t* xshape,
                                             const int64_t* yshape, int side, int count);
SGT_API int sgt_env_blocks(int n, const double* const* W, const int64_t* wshape, const double* const* X,
                           const int64_t* xshape, const double* const* Y, const int64_t* yshape, int side,
                           int count, double* const* blocks, void* ws, size_t ws_bytes, void* stream);

/* out[a,o1,o2,a4] = sum L[a,b,c] M[c,i1,i2,c4] W1[b,i1,o1,b2] W2[b2,i2,o2,b3] R[a4,b3,c4]:
 * the effective operator of sites k, k+1 applied to their merged tensor M
 * (c, in_k, in_{k+1}, c4).  lshape/rshape are triples; L = lshape = NULL
 * stands for the unit block (first step, dmrg.py:143-149; needs b = c = 1),
 * likewise R = rshape = NULL (last step, dmrg.py:150-157).  mshape, w1shape,
 * w2shape are quadruples; `out` holds (a, out_k, out_{k+1}, a4). */
SGT_API size_t sgt_env_two_site_workspace_size(const int64_t* lshape, const int64_t* mshape,
                                               const int64_t* w1shape, const int64_t* w2shape,
                                               const int64_t* rshape);
SGT_API int sgt_env_two_site(const double* L, const int64_t* lshape, const double* M, const int64_t* mshape,
                             const double* W1, const int64_t* w1shape, const double* W2,
                             const int64_t* w2shape, const double* R, const int64_t* rshape, double* out,
                             void* ws, size_t ws_bytes, void* stream);

/* ----------------------------------------------------------------------
 * Dense primitives (exported for composition and tests)
 * -------------------------------------------------------------------- */

/* C = alpha * op(A) op(B) + beta * C, row-major, batched with element strides.
 * op(A) is M x K (A stored K x M when transA), op(B) is K x N. */
SGT_API int sgt_gemm_f64(int transA, int transB, int64_t M, int64_t N, int64_t K, double alpha,
                 const double* A, int64_t lda, int64_t strideA,
                 const double* B, int64_t ldb, int64_t strideB, double beta,
                 double* C, int64_t ldc, int64_t strideC, int64_t batch, void* stream);

/* Householder QR of row-major A (m x n, leading dim lda) in place (R on and
 * above the diagonal, reflectors below), tau gets min(m,n) scalars; then
 * Q (m x keep, keep <= m) = first `keep` columns of the complete Q. */
SGT_API size_t sgt_qr_workspace_size(int64_t m, int64_t n, int64_t keep);
SGT_API int sgt_qr(double* A, int64_t m, int64_t n, int64_t lda, double* tau, double* Q, int64_t keep,
           void* ws, size_t ws_bytes, void* stream);

/* One-sided Jacobi SVD of row-major A (m x n, m >= n): on return A holds
 * U*diag(s) with columns in descending order of s, V (n x n, row-major) the
 * right singular vectors as columns, s the singular values in descending
 * order.  `status` (device int, may be NULL) gets the number of sweeps used,
 * or -1 if the sweep cap was reached; the call itself never waits for the
 * device, so a caller that needs the outcome reads `status` after a sync. */
SGT_API size_t sgt_jacobi_svd_workspace_size(int64_t m, int64_t n);
SGT_API int sgt_jacobi_svd(double* A, int64_t m, int64_t n, double* V, double* s, int* status,
                   void* ws, size_t ws_bytes, void* stream);

/* Tensor-core GEMM (tcgen05, kind::tf32, TMA-staged operands, TMEM accumulator):
 * C (M x N, fp32) = alpha * A B^T + beta * C with A (M x K) and B (N x K)
 * row-major fp32, leading dimensions multiples of 4, 16-byte aligned bases.
 * passes = 1: TF32 inputs.  passes = 3: split precision, A_hi/B_hi the TF32
 * parts and A_lo/B_lo the residuals (from sgt_split_tf32), accumulating
 * A_hi B_hi + A_hi B_lo + A_lo B_hi in FP32.  `err` (device int, may be NULL)
 * is set to 1 if a pipeline wait timed out.  GEMM-shaped work of the
 * mixed-precision forms (product carries, trailing updates, transfer sweeps). */
SGT_API int sgt_tc_gemm_f32(int passes, int64_t M, int64_t N, int64_t K, float alpha,
                            const float* A_hi, const float* A_lo, int64_t lda,
                            const float* B_hi, const float* B_lo, int64_t ldb, float beta,
                            float* C, int64_t ldc, int* err, void* stream);

/* The same GEMM with a workspace: when the output has too few 128 x 128 tiles
 * to occupy the GPU, K is split over up to 8 CTAs per tile, each storing its
 * partial tile into the workspace, and a second kernel adds the slices in a
 * fixed order into beta * C (deterministic).  The size query gives the bytes
 * that allow the full split (0: no split for this shape); a smaller workspace
 * gives fewer splits, none at 0 bytes. */
SGT_API size_t sgt_tc_gemm_f32_workspace_size(int64_t M, int64_t N, int64_t K);
SGT_API int sgt_tc_gemm_f32_ws(int passes, int64_t M, int64_t N, int64_t K, float alpha,
                               const float* A_hi, const float* A_lo, int64_t lda,
                               const float* B_hi, const float* B_lo, int64_t ldb, float beta,
                               float* C, int64_t ldc, int* err, void* ws, size_t ws_bytes, void* stream);

/* Event timing of tensor-core GEMM launches: enable = 1 starts recording a
 * CUDA event pair around every sgt tcgen05 GEMM launch (on its stream);
 * enable = 0 stops, waits for the recorded events and returns the summed
 * kernel milliseconds, algorithmic flops (2 M N K per launch) and launches. */
SGT_API int sgt_tc_profile(int enable, double* ms, double* flops, long long* launches);

/* Event timing of the cluster-resident FP32 eigensolver (the Gram form's bond
 * solve, gjacobi_kernel<1>): enable = 1 starts recording a CUDA event pair
 * around every launch; enable = 0 stops, waits for the events and returns the
 * summed kernel milliseconds, the algorithmic FP32 flops (sweeps x n(n-1)/2
 * pair visits x 12 n per launch, the sweep count read from the launch's
 * status word) and the number of launches.  Like sgt_tc_profile, a process-wide
 * switch for single-threaded benchmarks: not for use while other threads launch
 * work or while a stream is being captured into a graph. */
SGT_API int sgt_eig_profile(int enable, double* ms, double* flops, long long* launches);

/* Symmetric PSD eigen-decomposition in FP32 (the Gram-form bond solve):
 * Z (n x n, overwritten) -> Vt rows = eigenvectors, lam descending.
 * method 0: two-sided block Jacobi in one thread-block cluster (used when it
 * fits, else method 1); method 1: one-sided Jacobi on the rows of Z;
 * method 2: one-sided Jacobi on the rows of the Cholesky factor of Z + delta I
 * (delta = 2 n eps max diag) taken in decreasing-diagonal order: about two
 * thirds of the sweeps, vectors by normalisation (less accurate near the cut);
 * method 3: the same factor, one-sided Jacobi on its columns with the rotations
 * accumulated (the eigenvectors are the rows of the accumulated rotation).
 * status: sweeps performed, -1 at the sweep cap. */
SGT_API size_t sgt_sym_eig_f32_workspace_size(int64_t n);
SGT_API int sgt_sym_eig_f32(float* Z, int64_t n, float* Vt, float* lam, int* status, int method,
                            void* ws, size_t ws_bytes, void* stream);

/* Eigensolver used for the bond problems of the Gram forms (sgt_mpo_mps_round
 * / sgt_svd_round with TF32 / TF32X3 / BF16X6): the sgt_sym_eig_f32 method 1,
 * 2 or 3 (other values leave it unchanged).  Returns the previous choice.
 * Without a choice (this call or the environment variable SGT_EIG_METHOD) the
 * TF32 forms use method 1 and the BF16X6 form method 2, whose lower accuracy
 * near the cut its refinement removes.  Process-wide.  The FP32 Jacobi
 * stopping threshold on |g_p.g_q| / (|g_p||g_q|) is k eps sqrt(m) with k = 1,
 * or the value of SGT_EIG_TOL. */
SGT_API int sgt_eig_method(int method);

/* Batched MPO x MPS + TT-SVD round + overlap over `count` independent
 * instances of uneven size (replaces the per-instance loop a caller of the
 * reference would write around `(W @ X) >> chi` and `X | Z`; no single
 * reference function).  sgt_batched_plan_create sizes every instance's
 * workspace (max of the fused round and the overlap), deals the instances
 * onto `lanes` stream lanes, most estimated work first onto the least-loaded
 * lane (work: per bond the squared product bond times d chi), and returns the
 * workspace one launch
 * needs; it is host-only (no device calls).  sgt_batched_launch forks the
 * lanes off `stream` with events, runs each lane's instances in order inside
 * its own workspace region and joins the lanes back: no allocation, no host
 * synchronisation, capturable into a CUDA graph.  The lanes' streams and
 * events are created on the first launch and released by
 * sgt_batched_plan_destroy.  One plan must not be launched concurrently from
 * two threads. */
typedef struct sgt_batched_plan_s* sgt_batched_plan;
SGT_API int sgt_batched_plan_create(int count, const int* n, const int64_t* const* wshape,
                                    const int64_t* const* xshape, const int64_t* chi, int precision,
                                    int lanes, sgt_batched_plan* plan, size_t* ws_bytes);
SGT_API int sgt_batched_plan_lane(const struct sgt_batched_plan_s* plan, int instance);
SGT_API int sgt_batched_plan_out_shape(const struct sgt_batched_plan_s* plan, int instance,
                                       int64_t* out_shape);
SGT_API int sgt_batched_launch(sgt_batched_plan plan, const double* const* const* W,
                               const double* const* const* X, double* const* const* out,
                               double* const* spectra, double* const* discarded, int* const* status,
                               double* const* overlap, void* ws, size_t ws_bytes, void* stream);
SGT_API void sgt_batched_plan_destroy(sgt_batched_plan plan);

/* FP64-class GEMM on the bf16 tensor cores: C = alpha A B^T + beta C with A
 * (M x K, lda) and B (N x K, ldb) row-major FP64, C (M x N, ldc) FP64.  Every
 * row of A and of B is scaled by a power of two and cut exactly into six
 * 7-bit slices held in bf16; the 21 slice products with slice levels
 * s + t <= 5 run as tcgen05 kind::f16 MMAs whose FP32 accumulation is exact
 * over K ranges of 1024 (longer K is split and the partials added in a fixed
 * order).  Error ~2^-41 of the row-max times column-max scale per term
 * (FP64: 2^-52; split TF32: 2^-22).  The GEMM kind of the SGT_PREC_BF16X6
 * forms, exported for composition and tests. */
SGT_API size_t sgt_gemm_f64_sliced_workspace_size(int64_t M, int64_t N, int64_t K);
SGT_API int sgt_gemm_f64_sliced(int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
                                const double* B, int64_t ldb, double beta, double* C, int64_t ldc, void* ws,
                                size_t ws_bytes, void* stream);

/* Process-wide tuning of the sliced GEMM (no reference counterpart; the
 * batched engine's autotuner sets it).  SGT_TUNE_SLICED_SPLIT_CTAS: a product
 * whose output has fewer 128 x 96 tiles than this many CTAs is split along K
 * (partials added in a fixed order) until it fills about that many CTAs, each
 * split keeping at least SGT_TUNE_SLICED_SPLIT_MIN_KTILES tiles of 32 along K
 * (defaults 148 and 8; ranges 1..608 and 2..32).  Workspace queries made
 * under one setting stay valid under another: a split that would not fit the
 * workspace is not taken.  Results do not depend on the setting beyond FP32
 * pair rounding of the partial sums.  sgt_get_tuning returns the current
 * value (-1 for an unknown key). */
#define SGT_TUNE_SLICED_SPLIT_CTAS 0
#define SGT_TUNE_SLICED_SPLIT_MIN_KTILES 1
/* SGT_TUNE_PCHOL_BLOCKED (0 or 1, default 0): the BF16X6 form's pivoted
 * Cholesky of a purified projector on one 16-CTA cluster with the factor in
 * shared memory where it fits (0), or always blocked (1: 32-pivot panels on one
 * block, trailing updates on all SMs).  Same kept subspace either way. */
#define SGT_TUNE_PCHOL_BLOCKED 2
/* SGT_TUNE_PURIFY_CLEANUP (0 or 1, default 0): after a purification that did
 * not reach a projector (a bond matrix with fewer directions above the
 * products' noise than kept; its status is -1), run McWeeny steps
 * X <- 3X^2 - 2X^3 and extra Newton-Schulz steps on the basis.  Off by default:
 * the steps are enqueued for every bond and skipped on the device when not
 * needed, which still costs about 3% of a sweep that never needs them. */
#define SGT_TUNE_PURIFY_CLEANUP 3
/* SGT_TUNE_PURIFY_VECTOR_STEP (0 or 1, default 1): each purification step
 * after the product X2 = X X updates X, finds its residual and writes X's
 * slices with one 128-thread block per row and 16-byte accesses where the bond
 * dimension is a multiple of 4 (1), or with one warp per row (0).  The same
 * arithmetic element by element: identical results. */
#define SGT_TUNE_PURIFY_VECTOR_STEP 4
SGT_API int sgt_set_tuning(int key, int value);
SGT_API int sgt_get_tuning(int key);

/* Phase timing of the BF16X6 rounding (a benchmark switch, process-wide, for
 * one rounding at a time on one stream): enable = 1 starts recording CUDA
 * events at the phase boundaries; enable = 0 stops, waits for them and writes
 * the milliseconds per phase into ms[0..count-1]: 0 left Gram recursion,
 * 1 right-sweep projections Y_k, 2 bond matrices Z_k, 3 purification,
 * 4 kept basis (pivoted Cholesky, Newton-Schulz), 5 discarded weights,
 * 6 carry F_k to the next bond, 7 eigensolve + refinement (with spectra). */
#define SGT_ROUND_PHASES 8
SGT_API int sgt_phase_profile(int enable, double* ms, int count);

/* Event timing of the sliced bf16 GEMM launches, as sgt_tc_profile (flops
 * counted as 2 M N K per call, the FP64-equivalent work). */
SGT_API int sgt_sliced_profile(int enable, double* ms, double* flops, long long* launches);

/* hi = TF32 rounding of x (round to nearest, ties away), lo = x - hi (lo may be NULL). */
SGT_API int sgt_split_tf32(const float* x, float* hi, float* lo, int64_t n, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SYNGULAR_GB300_H */
