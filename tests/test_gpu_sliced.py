"""FP64-class sliced bf16 GEMM (tcgen05 kind::f16) and the SGT_PREC_BF16X6
rounding form built on it, against numpy FP64 and the FP64 oracle.

Tolerances: the GEMM keeps ~2^-41 of the row-max times column-max scale per
term (tested at 2^-38 of K times that scale elementwise, and exactly for
small-integer operands, where every slice product and every accumulation is
exact); the rounding form is held to
a plain relative 1e-6 on <X|Z> and <Z|Z> (the accuracy bound of the
mixed-precision target), with its measured error far below that."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import tt_fp64 as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def sliced_gemm(A, B, alpha=1.0, beta=0.0, C=None):
    from syngular_gb300 import _lib as L

    M, K = A.shape
    N = B.shape[0]
    a = torch.as_tensor(A, dtype=torch.float64, device="cuda").contiguous()
    b = torch.as_tensor(B, dtype=torch.float64, device="cuda").contiguous()
    c = (torch.zeros((M, N), dtype=torch.float64, device="cuda") if C is None
         else torch.as_tensor(C, dtype=torch.float64, device="cuda").clone())
    nb = L.query("sgt_gemm_f64_sliced_workspace_size", M, N, K)
    assert nb > 0
    ws = L.workspace(nb)
    L.call("sgt_gemm_f64_sliced", M, N, K, ctypes.c_double(alpha), L.ptr(a), K, L.ptr(b), K, ctypes.c_double(beta),
           L.ptr(c), N, L.ptr(ws), ws.numel(), L.stream_ptr())
    torch.cuda.synchronize()
    return c.cpu().numpy()


@pytest.mark.parametrize("M,N,K", [(200, 300, 1500), (128, 128, 64), (257, 129, 4096), (33, 517, 999)])
def test_exact_on_small_integers(M, N, K):
    """Integer operands of at most 7 bits fit the first slice exactly, so the
    tensor-core result must equal the exact integer product (also across the
    split-K partials when K > 1024)."""
    rng = np.random.default_rng(M + N + K)
    A = rng.integers(-64, 65, size=(M, K)).astype(np.float64)
    B = rng.integers(-64, 65, size=(N, K)).astype(np.float64)
    C = sliced_gemm(A, B)
    np.testing.assert_array_equal(C, A @ B.T)


@pytest.mark.parametrize("M,N,K", [(512, 4096, 4096), (1000, 256, 512), (512, 512, 512), (7, 9, 3), (4096, 64, 256),
                                   (512, 65536, 256)])
def test_accuracy_bound(M, N, K):
    rng = np.random.default_rng(7 * M + N)
    A = rng.standard_normal((M, K)) * np.exp(rng.uniform(-3, 3, size=(M, 1)))
    B = rng.standard_normal((N, K))
    C = sliced_gemm(A, B)
    ref = A @ B.T
    err = np.abs(C - ref)
    # slicing keeps every entry to 2^-42 of its row's (column's) largest entry
    scale = np.max(np.abs(A), axis=1)[:, None] * np.max(np.abs(B), axis=1)[None, :]
    assert np.all(err <= 2.0 ** -38 * K * scale), float(np.max(err / (K * scale)))
    # independent truncation errors: ~2^-41 sqrt(K) of that scale in the median
    assert float(np.median(err / (np.sqrt(K) * scale))) < 2.0 ** -39
    # and far below split TF32 (2^-22) relative to sum_k |a_ik| |b_jk|
    bound = np.abs(A) @ np.abs(B).T
    assert float(np.max(err / bound)) < 2.0 ** -28


def test_alpha_beta():
    rng = np.random.default_rng(3)
    A = rng.standard_normal((130, 70))
    B = rng.standard_normal((90, 70))
    C0 = rng.standard_normal((130, 90))
    C = sliced_gemm(A, B, alpha=-0.75, beta=2.0, C=C0)
    scale = 0.75 * 70 * np.max(np.abs(A)) * np.max(np.abs(B))
    np.testing.assert_allclose(C, -0.75 * (A @ B.T) + 2.0 * C0, rtol=0, atol=2.0 ** -38 * scale)


def dev(cores):
    from syngular_gb300 import _lib

    return [_lib.as_device(c) for c in cores]


def rel_overlaps(X, Z, Zr):
    from syngular_gb300.tensor import _ops

    Xd = dev(X)
    ov, ovr = _ops.overlap(Xd, Z), O.overlap(X, Zr)
    zz, zzr = _ops.overlap(Z, Z), O.overlap(Zr, Zr)
    return abs(ov - ovr) / abs(ovr), abs(zz - zzr) / abs(zzr)


CASES = [(6, 2, 8, 3, 5), (10, 2, 32, 4, 24), (8, 3, 16, 4, 20), (12, 2, 64, 8, 64), (8, 2, 32, 16, 48),
         (7, 3, 16, 8, 30), (14, 2, 64, 16, 40)]


@pytest.mark.parametrize("n,d,chi,D,cut", CASES)
def test_bf16x6_round_matches_oracle(n, d, chi, D, cut):
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(1000 * n + chi)
    X = O.random_mps_cores(rng, n, d, chi)
    W = O.random_mpo_cores(rng, n, d, D)
    Zr, spec_r, disc_r = O.tt_svd_round(O.mpo_mps_product(W, X), cut)
    Z, spec, counts, disc, status = _ops.mpo_mps_round(dev(W), dev(X), cut, L.PREC_BF16X6)
    torch.cuda.synchronize()
    assert int(status.item()) >= 0
    assert [tuple(z.shape) for z in Z] == [z.shape for z in Zr]
    e_ov, e_zz = rel_overlaps(X, Z, Zr)
    assert e_ov < 1e-6 and e_zz < 1e-6, (e_ov, e_zz)
    assert e_ov < 1e-8 and e_zz < 1e-9, (e_ov, e_zz)  # the form's own accuracy, well inside the bound
    s = spec.cpu().numpy()
    off = 0
    for k in range(n - 1):
        m = min(counts[k], len(spec_r[k]))
        kk = min(cut, m)
        np.testing.assert_allclose(s[off:off + kk], spec_r[k][:kk], rtol=0, atol=1e-8 * spec_r[k][0])
        np.testing.assert_allclose(s[off + kk:off + m] ** 2, spec_r[k][kk:m] ** 2, rtol=0, atol=1e-4 * spec_r[k][0] ** 2)
        off += counts[k]
    np.testing.assert_allclose(disc.cpu().numpy()[: n - 1], disc_r, rtol=1e-6, atol=1e-12)


def test_bf16x6_svd_round_chain():
    """sgt_svd_round in the BF16X6 form on a plain chain (a direct sum, so the
    bond matrices are rank-deficient), against the oracle."""
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(21)
    A = O.random_mps_cores(rng, 10, 2, 24)
    B = O.random_mps_cores(rng, 10, 2, 24)
    S = O.direct_sum(A, B)
    Zr, spec_r, _ = O.tt_svd_round(S, 20)
    Z, spec, counts, disc, status = _ops.svd_round(dev(S), 20, L.PREC_BF16X6)
    torch.cuda.synchronize()
    assert int(status.item()) >= 0
    ov, ovr = _ops.overlap(dev(A), Z), O.overlap(A, Zr)
    assert abs(ov - ovr) / abs(ovr) < 1e-8
    zz, zzr = _ops.overlap(Z, Z), O.overlap(Zr, Zr)
    assert abs(zz - zzr) / zzr < 1e-9


@pytest.mark.parametrize("blocked", [0, 1])
@pytest.mark.parametrize("n,d,chi,D,cut", CASES)
def test_bf16x6_round_without_spectra(n, d, chi, D, cut, blocked):
    """Without spectra the BF16X6 form finds each kept subspace by purification
    (no eigensolve): the rounded state, the discarded weights and the right
    orthonormality of the cores match the FP64 oracle, with the projector's
    pivoted Cholesky on one cluster or blocked."""
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(1000 * n + chi)
    X = O.random_mps_cores(rng, n, d, chi)
    W = O.random_mpo_cores(rng, n, d, D)
    Zr, spec_r, disc_r = O.tt_svd_round(O.mpo_mps_product(W, X), cut)
    L.call("sgt_set_tuning", L.TUNE_PCHOL_BLOCKED, blocked)
    try:
        Z, spec, counts, disc, status = _ops.mpo_mps_round(dev(W), dev(X), cut, L.PREC_BF16X6, spectra=False)
        torch.cuda.synchronize()
    finally:
        L.call("sgt_set_tuning", L.TUNE_PCHOL_BLOCKED, 0)
    assert spec is None and int(status.item()) >= 0
    assert [tuple(z.shape) for z in Z] == [z.shape for z in Zr]
    e_ov, e_zz = rel_overlaps(X, Z, Zr)
    assert e_ov < 1e-6 and e_zz < 1e-6, (e_ov, e_zz)
    assert e_ov < 1e-8 and e_zz < 1e-9, (e_ov, e_zz)
    # discarded weights from traces; eigenvalues below ~1e-11 of the largest
    # sit at the products' own error and may fall on either side of the cut
    np.testing.assert_allclose(disc.cpu().numpy()[: n - 1], disc_r, rtol=1e-6, atol=1e-9)
    # right orthonormal cores where the bond truncates (there the kept subspace
    # is a full-rank projector's range)
    for k in range(1, n):
        if disc_r[k - 1] > 1e-9:
            m = Z[k].reshape(Z[k].shape[0], -1).cpu().numpy()
            np.testing.assert_allclose(m @ m.T, np.eye(m.shape[0]), rtol=0, atol=1e-10)


@pytest.mark.parametrize("n,d,chi,D,cut", [(12, 2, 64, 8, 64), (7, 3, 16, 8, 30), (10, 2, 30, 3, 24)])
def test_purify_step_forms_agree(n, d, chi, D, cut):
    """The purification step with a block per row and 16-byte accesses (bond
    dimensions that are multiples of 4) and with a warp per row give the same
    rounded cores, discarded weights and status bit for bit."""
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(7 * n + chi)
    W, X = dev(O.random_mpo_cores(rng, n, d, D)), dev(O.random_mps_cores(rng, n, d, chi))
    out = []
    for vec in (1, 0):
        L.call("sgt_set_tuning", L.TUNE_PURIFY_VECTOR_STEP, vec)
        try:
            Z, _, _, disc, status = _ops.mpo_mps_round(W, X, cut, L.PREC_BF16X6, spectra=False)
            torch.cuda.synchronize()
        finally:
            L.call("sgt_set_tuning", L.TUNE_PURIFY_VECTOR_STEP, 1)
        out.append((Z, disc, int(status.item())))
    (Za, da, sa), (Zb, db, sb) = out
    assert sa == sb and sa >= 0
    assert torch.equal(da, db)
    for a, b in zip(Za, Zb):
        assert torch.equal(a, b)


@pytest.mark.parametrize("n,d,chi,chi2", [(12, 2, 16, 9), (64, 2, 256, 256), (5, 3, 7, 11)])
def test_overlap_on_sliced_gemm(n, d, chi, chi2):
    """The transfer sweep with its contractions on the sliced GEMM against the
    FP64 sweep: <X|Y> within 1e-10 of |X||Y| and <X|X> within 1e-10 relative
    (FP64-class products, FP64 transfer matrix, exact power-of-two rescaling)."""
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(n * 100 + chi)
    X = [L.as_device(c) for c in O.random_mps_cores(rng, n, d, chi)]
    Y = [L.as_device(c) for c in O.random_mps_cores(rng, n, d, chi2)]
    xy = _ops.overlap(X, Y, L.PREC_BF16X6)
    xy64 = _ops.overlap(X, Y)
    xx = _ops.overlap(X, X, L.PREC_BF16X6)
    xx64 = _ops.overlap(X, X)
    yy64 = _ops.overlap(Y, Y)
    assert abs(xy - xy64) <= 1e-10 * np.sqrt(xx64 * yy64)
    assert abs(xx - xx64) <= 1e-10 * xx64
    # the drop-in operator follows MatrixProductState.PRECISION
    from syngular_gb300.tensor import MatrixProductState

    saved = MatrixProductState.PRECISION
    try:
        MatrixProductState.PRECISION = "bf16x6"
        a, b = MatrixProductState.from_sites(X), MatrixProductState.from_sites(Y)
        assert float(a | b) == xy
    finally:
        MatrixProductState.PRECISION = saved


def test_bf16x6_round_rank_below_keep():
    """X + X rounded to 3/2 of X's bond: every bond matrix has rank chi below
    the kept 3 chi / 2, so the purification meets a cluster of noise
    eigenvalues it cannot split (its bonds report status -1).  With the
    clean-up steps (McWeeny, extra Newton-Schulz) the rounded state is 2X to
    1e-8 (without them it measured 3.4e-5 off)."""
    cleanup = 1
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(77)
    n, d, chi = 10, 2, 16
    X = O.random_mps_cores(rng, n, d, chi)
    S = O.direct_sum(X, X)
    L.call("sgt_set_tuning", L.TUNE_PURIFY_CLEANUP, cleanup)
    try:
        Z, spec, counts, disc, status = _ops.svd_round(dev(S), 3 * chi // 2, L.PREC_BF16X6, spectra=False)
        torch.cuda.synchronize()
    finally:
        L.call("sgt_set_tuning", L.TUNE_PURIFY_CLEANUP, 0)
    xx = O.overlap(X, X)
    zz = _ops.overlap(Z, Z)
    zx = _ops.overlap(Z, dev(X))
    assert abs(zz - 4 * xx) <= 1e-8 * 4 * xx
    assert abs(zx - 2 * xx) <= 1e-8 * 2 * xx
