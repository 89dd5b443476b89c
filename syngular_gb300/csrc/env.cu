// DMRG environment blocks and the two-site effective contraction
// (variational/dmrg.py:65-112 and 143-165 of the reference).
//
// An environment block is the partial contraction <X| W |Y> of the sites to
// the left (or right) of a bond: three legs (bra bond, operator bond, ket
// bond).  One site's update is a short chain of FP64 GEMMs on the library's
// register-blocked kernel with two index permutations in between, ordered so
// that every GEMM has the bond-sized dimensions as M and N and the small
// physical/operator legs inside K:
//
//   left  E'[a',b',c'] = sum E[a,b,c] X[a,o,a'] W[b,i,o,b'] Y[c,i,c']
//     T1[(b,c),(o,a')]  = E^T X                       (K = a)
//     P1[c,a',b,o]      = T1 permuted
//     T2[(c,a'),(i,b')] = P1 . W[(b,o),(i,b')]         (K = b*o, W permuted once)
//     P2[a',b',c,i]     = T2 permuted
//     E'[(a',b'),c']    = P2 . Y[(c,i),c']             (K = c*i)
//   right E[a,b,c] = sum X[a,o,a'] W[b,i,o,b'] Y[c,i,c'] E'[a',b',c']  (mirror order)
//
// The reference contracts with opt_einsum; bra and ket are the same state
// there (dmrg.py:78-81, 101-104); here they may differ.  The block before the
// first site (and after the last) is the unit 1x1x1 tensor, which is what the
// reference's first/last step computes by omitting it.  No rescaling: blocks
// are returned as they are, in plain FP64.
#include <algorithm>
#include <vector>

#include "common.cuh"

namespace sgt {

constexpr int PERM_MAX = 6;

namespace {

struct PermArgs {
  int rank;
  int64_t out_extent[PERM_MAX];  // extents of the output axes
  int64_t src_stride[PERM_MAX];  // source stride of the axis that lands at each output position
  int64_t total;
};

// dst (contiguous, axes in `perm` order) <- src (contiguous row-major).  One
// thread per output element, output index decoded innermost-first; the
// innermost output axis is usually a bond, so writes are coalesced.
__global__ void permute_kernel(const double* __restrict__ src, double* __restrict__ dst, const PermArgs a) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < a.total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = idx, off = 0;
#pragma unroll
    for (int q = PERM_MAX - 1; q >= 0; --q) {
      if (q < a.rank) {
        const int64_t e = a.out_extent[q];
        const int64_t c = rem % e;
        rem /= e;
        off += c * a.src_stride[q];
      }
    }
    dst[idx] = src[off];
  }
}

}  // namespace

// dst = src with its axes reordered: output axis j is source axis perm[j].
int permute_f64(cudaStream_t st, const double* src, double* dst, int rank, const int64_t* ext, const int* perm) {
  SGT_REQUIRE(rank >= 1 && rank <= PERM_MAX, SGT_ERR_INVALID, "permute: rank %d outside [1, %d]", rank, PERM_MAX);
  PermArgs a{};
  a.rank = rank;
  int64_t stride[PERM_MAX];
  int64_t s = 1;
  for (int q = rank - 1; q >= 0; --q) {
    stride[q] = s;
    s *= ext[q];
  }
  a.total = s;
  for (int j = 0; j < rank; ++j) {
    a.out_extent[j] = ext[perm[j]];
    a.src_stride[j] = stride[perm[j]];
  }
  if (a.total == 0) return SGT_OK;
  const int64_t blocks = std::min<int64_t>(cdiv(a.total, 256), 152 * 16);
  permute_kernel<<<(unsigned)blocks, 256, 0, st>>>(src, dst, a);
  SGT_LAUNCHED();
  return SGT_OK;
}

namespace {

__global__ void unit_kernel(double* p) { *p = 1.0; }

struct Site3 {
  int64_t l, p, r;
};
struct Site4 {
  int64_t l, i, o, r;
};

// Scratch sizes (doubles) of one left/right update and of the two-site step.
struct EnvScratch {
  int64_t t1 = 1, p1 = 1, wp = 1, t2 = 1, p2 = 1;
  void grow(int64_t a, int64_t b, int64_t c) {
    t1 = std::max(t1, a);
    p1 = std::max(p1, a);
    t2 = std::max(t2, c);
    p2 = std::max(p2, c);
    wp = std::max(wp, b);
  }
};

// One left update: En (A' x B' x C') from E (A x B x C), bra X (A, o, A'),
// operator W (B, i, o, B'), ket Y (C, i, C').
int env_left_step(cudaStream_t st, const double* E, const Site3& x, const Site4& w, const Site3& y, const double* X,
                  const double* W, const double* Y, double* En, double* T1, double* P1, double* Wp, double* T2,
                  double* P2) {
  const int64_t A = x.l, o = x.p, A2 = x.r, B = w.l, i = w.i, B2 = w.r, C = y.l, C2 = y.r;
  // T1[(b,c),(o,a')] = E[a,(b,c)]^T X[a,(o,a')]
  SGT_TRY(gemm_f64(st, true, false, B * C, o * A2, A, 1.0, E, B * C, 0, X, o * A2, 0, 0.0, T1, o * A2, 0, 1));
  {
    const int64_t ext[4] = {B, C, o, A2};
    const int perm[4] = {1, 3, 0, 2};  // -> [c, a', b, o]
    SGT_TRY(permute_f64(st, T1, P1, 4, ext, perm));
  }
  {
    const int64_t ext[4] = {B, i, o, B2};
    const int perm[4] = {0, 2, 1, 3};  // -> [b, o, i, b']
    SGT_TRY(permute_f64(st, W, Wp, 4, ext, perm));
  }
  // T2[(c,a'),(i,b')] = P1[(c,a'),(b,o)] Wp[(b,o),(i,b')]
  SGT_TRY(gemm_f64(st, false, false, C * A2, i * B2, B * o, 1.0, P1, B * o, 0, Wp, i * B2, 0, 0.0, T2, i * B2, 0, 1));
  {
    const int64_t ext[4] = {C, A2, i, B2};
    const int perm[4] = {1, 3, 0, 2};  // -> [a', b', c, i]
    SGT_TRY(permute_f64(st, T2, P2, 4, ext, perm));
  }
  // En[(a',b'),c'] = P2[(a',b'),(c,i)] Y[(c,i),c']
  SGT_TRY(gemm_f64(st, false, false, A2 * B2, C2, C * i, 1.0, P2, C * i, 0, Y, C2, 0, 0.0, En, C2, 0, 1));
  return SGT_OK;
}

// One right update: E (A x B x C) from En (A' x B' x C').
int env_right_step(cudaStream_t st, const double* En, const Site3& x, const Site4& w, const Site3& y,
                   const double* X, const double* W, const double* Y, double* E, double* T1, double* P1, double* Wq,
                   double* T2, double* P2) {
  const int64_t A = x.l, o = x.p, A2 = x.r, B = w.l, i = w.i, B2 = w.r, C = y.l, C2 = y.r;
  // T1[(a,o),(b',c')] = X[(a,o),a'] En[a',(b',c')]
  SGT_TRY(gemm_f64(st, false, false, A * o, B2 * C2, A2, 1.0, X, A2, 0, En, B2 * C2, 0, 0.0, T1, B2 * C2, 0, 1));
  {
    const int64_t ext[4] = {A, o, B2, C2};
    const int perm[4] = {0, 3, 1, 2};  // -> [a, c', o, b']
    SGT_TRY(permute_f64(st, T1, P1, 4, ext, perm));
  }
  {
    const int64_t ext[4] = {B, i, o, B2};
    const int perm[4] = {2, 3, 0, 1};  // -> [o, b', b, i]
    SGT_TRY(permute_f64(st, W, Wq, 4, ext, perm));
  }
  // T2[(a,c'),(b,i)] = P1[(a,c'),(o,b')] Wq[(o,b'),(b,i)]
  SGT_TRY(gemm_f64(st, false, false, A * C2, B * i, o * B2, 1.0, P1, o * B2, 0, Wq, B * i, 0, 0.0, T2, B * i, 0, 1));
  {
    const int64_t ext[4] = {A, C2, B, i};
    const int perm[4] = {0, 2, 3, 1};  // -> [a, b, i, c']
    SGT_TRY(permute_f64(st, T2, P2, 4, ext, perm));
  }
  // E[(a,b),c] = P2[(a,b),(i,c')] Y[c,(i,c')]^T
  SGT_TRY(gemm_f64(st, false, true, A * B, C, i * C2, 1.0, P2, i * C2, 0, Y, i * C2, 0, 0.0, E, C, 0, 1));
  return SGT_OK;
}

int env_blocks_impl(cudaStream_t st, int n, const double* const* W, const int64_t* ws4, const double* const* X,
                    const int64_t* xs, const double* const* Y, const int64_t* ys, int side, int count,
                    double* const* blocks, Arena& ar) {
  SGT_REQUIRE(n >= 1, SGT_ERR_INVALID, "env_blocks: empty chain");
  SGT_REQUIRE(side == 0 || side == 1, SGT_ERR_INVALID, "env_blocks: side must be 0 (left) or 1 (right)");
  SGT_REQUIRE(count >= 0 && count <= n, SGT_ERR_INVALID, "env_blocks: count %d outside [0, %d]", count, n);
  SGT_REQUIRE(ws4 && xs && ys, SGT_ERR_INVALID, "env_blocks: null shape array");
  std::vector<Site3> sx(n), sy(n);
  std::vector<Site4> sw(n);
  EnvScratch sc;
  for (int k = 0; k < n; ++k) {
    sx[k] = {xs[3 * k], xs[3 * k + 1], xs[3 * k + 2]};
    sy[k] = {ys[3 * k], ys[3 * k + 1], ys[3 * k + 2]};
    sw[k] = {ws4[4 * k], ws4[4 * k + 1], ws4[4 * k + 2], ws4[4 * k + 3]};
  }
  for (int k = 0; k < n; ++k) {
    SGT_REQUIRE(sx[k].l > 0 && sx[k].p > 0 && sx[k].r > 0 && sy[k].l > 0 && sy[k].p > 0 && sy[k].r > 0 &&
                    sw[k].l > 0 && sw[k].i > 0 && sw[k].o > 0 && sw[k].r > 0,
                SGT_ERR_INVALID, "env_blocks: non-positive extent at site %d", k);
    SGT_REQUIRE(sx[k].p == sw[k].o, SGT_ERR_INVALID,
                "env_blocks: bra physical leg %lld != operator output leg %lld at site %d", (long long)sx[k].p,
                (long long)sw[k].o, k);
    SGT_REQUIRE(sy[k].p == sw[k].i, SGT_ERR_INVALID,
                "env_blocks: ket physical leg %lld != operator input leg %lld at site %d", (long long)sy[k].p,
                (long long)sw[k].i, k);
    if (k + 1 < n)
      SGT_REQUIRE(sx[k].r == sx[k + 1].l && sy[k].r == sy[k + 1].l && sw[k].r == sw[k + 1].l, SGT_ERR_INVALID,
                  "env_blocks: bond mismatch between sites %d and %d", k, k + 1);
    const int64_t A = sx[k].l, o = sx[k].p, A2 = sx[k].r, B = sw[k].l, i = sw[k].i, B2 = sw[k].r, C = sy[k].l,
                  C2 = sy[k].r;
    if (side == 0)
      sc.grow(B * C * o * A2, B * i * o * B2, C * A2 * i * B2);
    else
      sc.grow(A * o * B2 * C2, B * i * o * B2, A * C2 * B * i);
  }
  SGT_REQUIRE(side == 1 || (sx[0].l == 1 && sy[0].l == 1 && sw[0].l == 1), SGT_ERR_INVALID,
              "env_blocks: left boundary bonds must be 1");
  SGT_REQUIRE(side == 0 || (sx[n - 1].r == 1 && sy[n - 1].r == 1 && sw[n - 1].r == 1), SGT_ERR_INVALID,
              "env_blocks: right boundary bonds must be 1");
  double* T1 = ar.take<double>(sc.t1);
  double* P1 = ar.take<double>(sc.p1);
  double* Wp = ar.take<double>(sc.wp);
  double* T2 = ar.take<double>(sc.t2);
  double* P2 = ar.take<double>(sc.p2);
  double* one = ar.take<double>(1);
  if (ar.measure) return SGT_OK;
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "env_blocks: workspace too small");
  SGT_REQUIRE(W && X && Y && (count == 0 || blocks), SGT_ERR_INVALID, "env_blocks: null argument");
  if (count == 0) return SGT_OK;
  unit_kernel<<<1, 1, 0, st>>>(one);
  SGT_LAUNCHED();
  const double* prev = one;
  for (int j = 0; j < count; ++j) {
    const int k = side == 0 ? j : n - 1 - j;
    SGT_REQUIRE(blocks[k], SGT_ERR_INVALID, "env_blocks: null output block for site %d", k);
    if (side == 0)
      SGT_TRY(env_left_step(st, prev, sx[k], sw[k], sy[k], X[k], W[k], Y[k], blocks[k], T1, P1, Wp, T2, P2));
    else
      SGT_TRY(env_right_step(st, prev, sx[k], sw[k], sy[k], X[k], W[k], Y[k], blocks[k], T1, P1, Wp, T2, P2));
    prev = blocks[k];
  }
  return SGT_OK;
}

// out[a, o1, o2, a4] = sum L[a,b,c] M[c,i1,i2,c4] W1[b,i1,o1,b2] W2[b2,i2,o2,b3] R[a4,b3,c4]
int env_two_site_impl(cudaStream_t st, const double* Lb, const int64_t* ls, const double* M, const int64_t* ms,
                      const double* W1, const int64_t* w1, const double* W2, const int64_t* w2, const double* Rb,
                      const int64_t* rs, double* out, Arena& ar) {
  SGT_REQUIRE(ms && w1 && w2, SGT_ERR_INVALID, "env_two_site: null shape array");
  const int64_t C = ms[0], i1 = ms[1], i2 = ms[2], C4 = ms[3];
  const int64_t B = w1[0], o1 = w1[2], B2 = w1[3], B3 = w2[3], o2 = w2[2];
  const int64_t A = ls ? ls[0] : 1, A4 = rs ? rs[0] : 1;
  for (int q = 0; q < 4; ++q)
    SGT_REQUIRE(ms[q] > 0 && w1[q] > 0 && w2[q] > 0, SGT_ERR_INVALID, "env_two_site: non-positive extent");
  SGT_REQUIRE(w1[1] == i1 && w2[1] == i2 && w2[0] == B2, SGT_ERR_INVALID,
              "env_two_site: operator legs do not match the two-site tensor");
  if (ls)
    SGT_REQUIRE(ls[0] > 0 && ls[1] == B && ls[2] == C, SGT_ERR_INVALID,
                "env_two_site: left block (%lld, %lld, %lld) does not match (., %lld, %lld)", (long long)ls[0],
                (long long)ls[1], (long long)ls[2], (long long)B, (long long)C);
  else
    SGT_REQUIRE(B == 1 && C == 1, SGT_ERR_INVALID, "env_two_site: no left block needs unit left bonds");
  if (rs)
    SGT_REQUIRE(rs[0] > 0 && rs[1] == B3 && rs[2] == C4, SGT_ERR_INVALID,
                "env_two_site: right block (%lld, %lld, %lld) does not match (., %lld, %lld)", (long long)rs[0],
                (long long)rs[1], (long long)rs[2], (long long)B3, (long long)C4);
  else
    SGT_REQUIRE(B3 == 1 && C4 == 1, SGT_ERR_INVALID, "env_two_site: no right block needs unit right bonds");
  const int64_t n1 = A * B * i1 * i2 * C4, n2 = A * i2 * C4 * o1 * B2, n3 = A * C4 * o1 * o2 * B3;
  double* T = ar.take<double>(std::max(n1, std::max(n2, n3)));
  double* P = ar.take<double>(std::max(n1, std::max(n2, n3)));
  double* one = ar.take<double>(1);
  if (ar.measure) return SGT_OK;
  SGT_REQUIRE(ar.ok(), SGT_ERR_WORKSPACE, "env_two_site: workspace too small");
  SGT_REQUIRE(M && W1 && W2 && out && (Lb || !ls) && (Rb || !rs), SGT_ERR_INVALID, "env_two_site: null argument");
  if (!ls || !rs) {
    unit_kernel<<<1, 1, 0, st>>>(one);
    SGT_LAUNCHED();
  }
  const double* Lp = ls ? Lb : one;
  const double* Rp = rs ? Rb : one;
  // T[(a,b),(i1,i2,c4)] = L[(a,b),c] M[c,(i1,i2,c4)]
  SGT_TRY(gemm_f64(st, false, false, A * B, i1 * i2 * C4, C, 1.0, Lp, C, 0, M, i1 * i2 * C4, 0, 0.0, T,
                   i1 * i2 * C4, 0, 1));
  {
    const int64_t ext[5] = {A, B, i1, i2, C4};
    const int perm[5] = {0, 3, 4, 1, 2};  // -> [a, i2, c4, b, i1]
    SGT_TRY(permute_f64(st, T, P, 5, ext, perm));
  }
  // T[(a,i2,c4),(o1,b2)] = P[(a,i2,c4),(b,i1)] W1[(b,i1),(o1,b2)]
  SGT_TRY(gemm_f64(st, false, false, A * i2 * C4, o1 * B2, B * i1, 1.0, P, B * i1, 0, W1, o1 * B2, 0, 0.0, T,
                   o1 * B2, 0, 1));
  {
    const int64_t ext[5] = {A, i2, C4, o1, B2};
    const int perm[5] = {0, 2, 3, 4, 1};  // -> [a, c4, o1, b2, i2]
    SGT_TRY(permute_f64(st, T, P, 5, ext, perm));
  }
  // T[(a,c4,o1),(o2,b3)] = P[(a,c4,o1),(b2,i2)] W2[(b2,i2),(o2,b3)]
  SGT_TRY(gemm_f64(st, false, false, A * C4 * o1, o2 * B3, B2 * i2, 1.0, P, B2 * i2, 0, W2, o2 * B3, 0, 0.0, T,
                   o2 * B3, 0, 1));
  {
    const int64_t ext[5] = {A, C4, o1, o2, B3};
    const int perm[5] = {0, 2, 3, 4, 1};  // -> [a, o1, o2, b3, c4]
    SGT_TRY(permute_f64(st, T, P, 5, ext, perm));
  }
  // out[(a,o1,o2),a4] = P[(a,o1,o2),(b3,c4)] R[a4,(b3,c4)]^T
  SGT_TRY(gemm_f64(st, false, true, A * o1 * o2, A4, B3 * C4, 1.0, P, B3 * C4, 0, Rp, B3 * C4, 0, 0.0, out, A4,
                   0, 1));
  return SGT_OK;
}

}  // namespace
}  // namespace sgt

using namespace sgt;

extern "C" {

size_t sgt_env_blocks_workspace_size(int n, const int64_t* wshape, const int64_t* xshape, const int64_t* yshape,
                                     int side, int count) {
  Arena a = Arena::measuring();
  if (env_blocks_impl(nullptr, n, nullptr, wshape, nullptr, xshape, nullptr, yshape, side, count, nullptr, a) !=
      SGT_OK)
    return 0;
  return a.used;
}

int sgt_env_blocks(int n, const double* const* W, const int64_t* wshape, const double* const* X,
                   const int64_t* xshape, const double* const* Y, const int64_t* yshape, int side, int count,
                   double* const* blocks, void* ws, size_t ws_bytes, void* stream) {
  Arena a(ws, ws_bytes);
  return env_blocks_impl(as_stream(stream), n, W, wshape, X, xshape, Y, yshape, side, count, blocks, a);
}

size_t sgt_env_two_site_workspace_size(const int64_t* lshape, const int64_t* mshape, const int64_t* w1shape,
                                       const int64_t* w2shape, const int64_t* rshape) {
  Arena a = Arena::measuring();
  if (env_two_site_impl(nullptr, nullptr, lshape, nullptr, mshape, nullptr, w1shape, nullptr, w2shape, nullptr,
                        rshape, nullptr, a) != SGT_OK)
    return 0;
  return a.used;
}

int sgt_env_two_site(const double* L, const int64_t* lshape, const double* M, const int64_t* mshape,
                     const double* W1, const int64_t* w1shape, const double* W2, const int64_t* w2shape,
                     const double* R, const int64_t* rshape, double* out, void* ws, size_t ws_bytes, void* stream) {
  Arena a(ws, ws_bytes);
  return env_two_site_impl(as_stream(stream), L, lshape, M, mshape, W1, w1shape, W2, w2shape, R, rshape, out, a);
}

}  // extern "C"
