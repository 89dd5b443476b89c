"""GPU parity of the plain FP64 path against the golden fixtures (produced by the
reference) and the numpy oracle.  Tolerance: 1e-12 relative for FP64 results
(gauge-invariant quantities: dense reconstructions, overlaps, Gram matrices,
singular values)."""
import numpy as np
import pytest
import torch

from oracle import tt_fp64 as O
from tests.conftest import rel

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def mps(cores):
    from syngular_gb300.tensor import MatrixProductState

    return MatrixProductState.from_sites([np.asarray(c) for c in cores])


def mpo(cores):
    from syngular_gb300.tensor import MatrixProductOperator

    return MatrixProductOperator.from_sites([np.asarray(c) for c in cores])


def dev(cores):
    from syngular_gb300 import _lib

    return [_lib.as_device(c) for c in cores]


def host(cores):
    return [c.cpu().numpy() for c in cores]


# ---------------------------------------------------------------------------
# primitives
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("M,N,K", [(37, 53, 29), (64, 64, 4096), (130, 7, 300)])
def test_gemm_f64(ta, tb, M, N, K):
    from syngular_gb300 import _lib as L

    rng = np.random.default_rng(M * N + K)
    A = rng.standard_normal((K, M) if ta else (M, K))
    B = rng.standard_normal((N, K) if tb else (K, N))
    C = rng.standard_normal((M, N))
    ref = 1.5 * (A.T if ta else A) @ (B.T if tb else B) - 0.5 * C
    Ad, Bd, Cd = (L.as_device(x) for x in (A, B, C))
    L.call("sgt_gemm_f64", ta, tb, M, N, K, 1.5, L.ptr(Ad), A.shape[1], 0, L.ptr(Bd), B.shape[1], 0,
           -0.5, L.ptr(Cd), N, 0, 1, L.stream_ptr())
    assert rel(Cd.cpu().numpy(), ref) < 1e-13


@pytest.mark.parametrize("m,n,keep", [(40, 30, 30), (300, 200, 250), (3000, 96, 96), (50, 300, 50),
                                      (2500, 700, 100)])
def test_householder_qr(m, n, keep):
    from syngular_gb300 import _lib as L

    rng = np.random.default_rng(m + n)
    A = rng.standard_normal((m, n))
    Ad = L.as_device(A)
    k = min(m, n)
    tau = torch.empty(k, dtype=torch.float64, device="cuda")
    Q = torch.empty((m, keep), dtype=torch.float64, device="cuda")
    ws = L.workspace(L.query("sgt_qr_workspace_size", m, n, keep))
    L.call("sgt_qr", L.ptr(Ad), m, n, n, L.ptr(tau), L.ptr(Q), keep, L.ptr(ws), ws.numel(), L.stream_ptr())
    Qh = Q.cpu().numpy()
    R = np.triu(Ad.cpu().numpy())[:k]
    Qr, Rr = np.linalg.qr(A, mode="complete")
    # same Householder sign convention as LAPACK: factors agree, not just up to gauge
    assert rel(R, Rr[:k]) < 1e-12
    assert rel(Qh, Qr[:, :keep]) < 1e-12
    np.testing.assert_allclose(Qh.T @ Qh, np.eye(keep), atol=1e-13)


@pytest.mark.parametrize("m,n", [(24, 24), (100, 60), (300, 300), (520, 513), (512, 512), (2000, 128)])
def test_jacobi_svd(m, n):
    from syngular_gb300 import _lib as L

    rng = np.random.default_rng(m * 7 + n)
    A = rng.standard_normal((m, n))
    Ad = L.as_device(A)
    V = torch.empty((n, n), dtype=torch.float64, device="cuda")
    s = torch.empty(n, dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = L.workspace(L.query("sgt_jacobi_svd_workspace_size", m, n))
    L.call("sgt_jacobi_svd", L.ptr(Ad), m, n, L.ptr(V), L.ptr(s), L.ptr(status), L.ptr(ws), ws.numel(),
           L.stream_ptr())
    assert int(status.item()) > 0
    sr = np.linalg.svd(A, compute_uv=False)
    np.testing.assert_allclose(s.cpu().numpy(), sr, rtol=1e-12)
    Vh, US = V.cpu().numpy(), Ad.cpu().numpy()
    np.testing.assert_allclose(Vh.T @ Vh, np.eye(n), atol=1e-13)
    assert rel(A @ Vh, US) < 1e-12


def test_site_contractions_match_oracle():
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(11)
    X = O.random_mps_cores(rng, 4, 3, 5)
    W = O.random_mpo_cores(rng, 4, 3, 4)
    W[1] = rng.standard_normal((4, 3, 2, 4))
    W[2] = rng.standard_normal((4, 2, 3, 4))
    X[1] = rng.standard_normal((5, 3, 5))
    P = host(_ops.contract_mpo_mps(dev(W[:1]) + dev(W[1:2]), dev(X[:1]) + dev(X[1:2])))
    ref = O.mpo_mps_product(W[:2], X[:2])
    for a, b in zip(P, ref):
        np.testing.assert_allclose(a, b, rtol=1e-14, atol=1e-14)
    A = O.random_mpo_cores(rng, 3, 3, 2)
    B = [rng.standard_normal((3, 3, 2, 3)) if k == 1 else rng.standard_normal(
        (1 if k == 0 else 3, 3, 2, 3 if k < 2 else 1)) for k in range(3)]
    B[0] = rng.standard_normal((1, 3, 2, 3))
    B[2] = rng.standard_normal((3, 3, 2, 1))
    P = host(_ops.contract_mpo_mpo(dev(A), dev(B)))
    for a, b in zip(P, O.mpo_mpo_product(A, B)):
        np.testing.assert_allclose(a, b, rtol=1e-14, atol=1e-14)


def test_bond_concat_bit_exact():
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(12)
    for n in (1, 2, 5):
        A = O.random_mps_cores(rng, n, 3, 4)
        B = O.random_mps_cores(rng, n, 3, 2)
        got = host(_ops.concat(dev(A), dev(B)))
        for a, b in zip(got, O.direct_sum(A, B)):
            np.testing.assert_array_equal(a, b)


# ---------------------------------------------------------------------------
# reference known answers and fixtures
# ---------------------------------------------------------------------------

def test_config1_golden(golden):
    g = golden("config1.npz")
    for seed in (1, 2):
        c = "seed%d" % seed
        W, X, Y = mpo(g(c, "W")), mps(g(c, "X")), mps(g(c, "Y"))
        P = W @ X
        assert rel(P.to_tensor(), g(c, "P_tensor")) < TOL
        Z = P >> 4
        assert rel(Z.to_tensor(), g(c, "Z_tensor")) < TOL
        assert abs((Z | Y) - g(c, "zy")) <= TOL * abs(g(c, "zy"))
        assert abs((X | Y) - g(c, "xy")) <= TOL * abs(g(c, "xy"))
        Z.left_orthonormalization()
        np.testing.assert_allclose(np.diag(Z.left_orthogonality(0)), g(c, "diag0"), atol=1e-12)
        np.testing.assert_allclose(np.diag(Z.left_orthogonality(1)), g(c, "diag1"), atol=1e-12)
        assert rel(Z.left_orthogonality(0), g(c, "gram0")) < 1e-12


def test_config1_decompose_on_device(golden):
    """Dense seeded tensors -> cores on the GPU; the operator cores agree with
    the reference's (same Householder convention), the product and rounding
    reproduce the fixture."""
    from syngular_gb300.tensor import MatrixProductOperator, MatrixProductState

    g = golden("config1.npz")
    w, x, y = O.config1_inputs(1)
    W = MatrixProductOperator(w, bond_shape=(8, 8)).decompose()
    X = MatrixProductState(x, bond_shape=(8, 8)).decompose()
    Y = MatrixProductState(y, bond_shape=(8, 8)).decompose()
    for a, b in zip(host(W.sites), g("seed1", "W")):
        assert rel(a, b) < 1e-11
    Z = (W @ X) >> 4
    assert rel(Z.to_tensor(), g("seed1", "Z_tensor")) < 1e-11
    assert abs((Z | Y) - g("seed1", "zy")) <= 1e-11 * abs(g("seed1", "zy"))


def test_readme_flow(golden):
    from syngular_gb300.tensor import MatrixProductOperator, MatrixProductState

    g = golden("readme_flow.npz")
    np.random.seed(0)
    W = MatrixProductOperator(np.arange(16 ** 6).reshape((16,) * 6), bond_shape=(16, 16))
    W.decompose()
    X = MatrixProductState(np.arange(16 ** 3).reshape((16,) * 3), bond_shape=(4, 4))
    X.decompose()
    T = MatrixProductOperator.random((16, 16, 16), (16, 16, 16), (8, 8))
    MatrixProductOperator.zeros((16, 16, 16), (16, 16, 16), (4, 4))
    U = MatrixProductState.random((16, 16, 16), (8, 8))
    W = W >> 4
    T = T >> 2
    TW = T + W
    assert TW.bond_shape == tuple(g("readme", "tw_bond_shape"))
    TWT = TW @ T
    assert TWT.bond_shape == tuple(g("readme", "twt_bond_shape"))
    assert [tuple(s) for s in TWT.shape] == [tuple(s) for s in g("readme", "twt_shape")]
    Z = TWT @ X
    assert abs((X | U) - g("readme", "xu")) <= 1e-11 * abs(g("readme", "xu"))
    assert abs((Z | X) - g("readme", "zx")) <= 1e-9 * abs(g("readme", "zx"))
    Z = Z >> 16
    Z.left_orthonormalization()
    assert [tuple(s) for s in Z.shape] == [tuple(s) for s in g("readme", "z_shape")]
    np.testing.assert_allclose(np.diag(Z.left_orthogonality(0)), g("readme", "diag0"), atol=1e-12)
    np.testing.assert_allclose(np.diag(Z.left_orthogonality(1)), g("readme", "diag1"), atol=1e-12)


def test_known_answers(golden):
    from syngular_gb300.tensor import MatrixProductOperator, MatrixProductState

    g = golden("known_answers.npz")
    w = np.arange(16.0).reshape(2, 2, 2, 2)
    x = np.arange(4.0).reshape(2, 2)
    W = MatrixProductOperator(w, bond_shape=(2,)).decompose()
    X = MatrixProductState(x, bond_shape=(2,)).decompose()
    Z = W @ W @ X
    np.testing.assert_allclose(Z.to_tensor().reshape(4), g("mpo_matmul", "out"), rtol=1e-11)
    W4 = MatrixProductOperator(w, bond_shape=(4,)).decompose()
    assert abs(W4[(1, 1), (1, 1)] - 15) < 1e-11
    z = np.arange(4.0 ** 3 * 27).reshape(4, 4, 4, 3, 3, 3)
    Zd = MatrixProductOperator(z, bond_shape=(3, 3)).decompose()
    assert abs(Zd[(3, 1, 0), (1, 2, 1)] - 1420) < 1e-8
    # MPO add chain with auto-round (test/test_mpo.py:256-282)
    Xa = MatrixProductOperator(np.arange(1.0, 17).reshape(2, 2, 2, 2), bond_shape=(3,)).decompose()
    Ya = MatrixProductOperator(np.arange(18.0, 34).reshape(2, 2, 2, 2), bond_shape=(3,)).decompose()
    Za = Xa + Ya + Ya + Ya + Ya + Ya + Ya + Ya + Ya + Ya
    assert abs(Za[(1, 1), (1, 1)] - 313) < 1e-9
    np.testing.assert_allclose(Za.to_tensor(), g("mpo_add", "z_tensor"), atol=1e-9)
    # MPS add / dot / normalize / compress / canonical (test/test_mps.py)
    x8 = np.arange(8.0).reshape(2, 2, 2)
    S = MatrixProductState(x8, bond_shape=(2, 2)).decompose() + MatrixProductState(
        x8, bond_shape=(2, 2)).decompose()
    np.testing.assert_allclose(S.to_tensor(), g("mps_add", "z_tensor"), atol=1e-12)
    x64 = np.arange(64.0).reshape(4, 4, 4)
    X = MatrixProductState(x64, bond_shape=(4, 4)).decompose()
    assert abs(X.dot() - 292.1369541841634) < 1e-9
    X.normalize()
    assert abs(X.dot() - 1.0) < 1e-12
    Xc = MatrixProductState(x64, bond_shape=(4, 4)).decompose() >> 2
    assert [tuple(s) for s in Xc.shape] == [tuple(s) for s in g("mps_compress", "z_shape")]
    assert rel(Xc.to_tensor(), g("mps_compress", "z_tensor")) < 1e-11
    XL = MatrixProductState(x64, bond_shape=(2, 2)).decompose(mode="left")
    XR = MatrixProductState(x64, bond_shape=(2, 2)).decompose(mode="right")
    assert rel(XL.to_tensor(), g("mps_canonical", "left_tensor")) < 1e-11
    assert rel(XR.to_tensor(), g("mps_canonical", "right_tensor")) < 1e-11
    # augment: 31 chained + then >> 2 (test/test_mps.py:22-38)
    Xa = MatrixProductState(x8, bond_shape=(2, 2)).decompose()
    Yz = MatrixProductState.zeros((2, 2, 2), (2, 2))
    Zs = Xa
    for _ in range(31):
        Zs = Zs + Yz
    assert [tuple(s) for s in Zs.shape] == [tuple(s) for s in g("mps_augment", "z_shape")]
    assert rel((Zs >> 2).to_tensor(), g("mps_augment", "zc_tensor")) < 1e-11
    # orthogonality (test/test_mpo.py:66-112)
    Wo = MatrixProductOperator(np.arange(4.0 ** 6).reshape((4,) * 6), bond_shape=(2, 2)).decompose()
    Wo.left_orthonormalization()
    np.testing.assert_allclose(np.diag(Wo.left_orthogonality(0)), g("mpo_orth", "l0"), atol=1e-12)
    np.testing.assert_allclose(np.diag(Wo.left_orthogonality(1)), g("mpo_orth", "l1"), atol=1e-12)
    Wo.right_orthonormalization()
    np.testing.assert_allclose(np.diag(Wo.right_orthogonality(1)), g("mpo_orth", "r1"), atol=1e-12)
    np.testing.assert_allclose(np.diag(Wo.right_orthogonality(2)), g("mpo_orth", "r2"), atol=1e-12)
    assert abs(Wo[(1, 0, 0), (1, 0, 0)] - g("mpo_orth", "w100100")) < 1e-6 * abs(g("mpo_orth", "w100100"))
    # non-strict compress then >> (test/test_mpo.py:115-158)
    Wc = MatrixProductOperator(np.arange(16.0 ** 4).reshape(16, 16, 16, 16), bond_shape=(8,)).decompose()
    Wc.compress(4, mode="left")
    assert [tuple(s) for s in Wc.shape] == [tuple(s) for s in g("mpo_compress", "w_shape")]
    Zc = Wc >> 2
    assert [tuple(s) for s in Zc.shape] == [tuple(s) for s in g("mpo_compress", "z_shape")]
    assert rel(Zc.to_tensor(), g("mpo_compress", "z_tensor")) < 1e-10
    # diagonal operator round trip (test/test_mpo.py:296-330)
    Yd = MatrixProductOperator(g("mpo_compare", "y"), bond_shape=(4,)).decompose().right_orthonormalization()
    np.testing.assert_allclose(Yd.to_tensor(), g("mpo_compare", "y_tensor"), atol=1e-12)


@pytest.mark.parametrize("n", [0, 1, 2])
def test_random_matmul_mps(golden, n):
    g = golden("random_cases.npz")
    c = "matmul_mps%d" % n
    Z = mpo(g(c, "W")) @ mps(g(c, "X"))
    assert [tuple(s) for s in Z.shape] == [tuple(s) for s in g(c, "Z_shape")]
    assert Z.bond_shape == tuple(g(c, "Z_bond_shape"))
    assert rel(Z.to_tensor(), g(c, "Z_tensor")) < TOL


@pytest.mark.parametrize("n", [0, 1])
def test_random_matmul_mpo(golden, n):
    g = golden("random_cases.npz")
    c = "matmul_mpo%d" % n
    Z = mpo(g(c, "A")) @ mpo(g(c, "B"))
    assert [tuple(s) for s in Z.shape] == [tuple(s) for s in g(c, "Z_shape")]
    assert rel(Z.to_tensor(), g(c, "Z_tensor")) < TOL


def test_random_add(golden):
    g = golden("random_cases.npz")
    Z = mps(g("add_mps", "X")) + mps(g("add_mps", "Y"))
    for a, b in zip(host(Z.sites), g("add_mps", "Z")):
        np.testing.assert_array_equal(a, b)
    Z = mpo(g("add_mpo", "A")) + mpo(g("add_mpo", "B"))
    assert [tuple(s) for s in Z.shape] == [tuple(s) for s in g("add_mpo", "Z_shape")]
    assert rel(Z.to_tensor(), g("add_mpo", "Z_tensor")) < TOL


@pytest.mark.parametrize("n", [0, 1, 2])
def test_random_overlap(golden, n):
    g = golden("random_cases.npz")
    c = "overlap%d" % n
    v = mps(g(c, "X")) | mps(g(c, "Y"))
    assert abs(v - g(c, "value")) <= TOL * max(1.0, abs(g(c, "value")))


def test_random_rshift(golden):
    from syngular_gb300.tensor import MatrixProductState

    g = golden("random_cases.npz")
    for dim in (2, 3):
        c = "rshift_mps_d%d" % dim
        Z = mps(g(c, "X")) >> dim
        assert [tuple(s) for s in Z.shape] == [tuple(s) for s in g(c, "Z_shape")]
        assert Z.bond_shape == tuple(g(c, "Z_bond_shape"))
        assert rel(Z.to_tensor(), g(c, "Z_tensor")) < TOL
    Z = mps(g("rshift_pad", "X")).compress(4, strict=True)
    assert [tuple(s) for s in Z.shape] == [tuple(s) for s in g("rshift_pad", "Z_shape")]
    assert rel(Z.to_tensor(), g("rshift_pad", "Z_tensor")) < TOL
    np.testing.assert_allclose(Z.left_orthogonality(0), g("rshift_pad", "Z_gram0"), atol=1e-12)
    W = mpo(g("rshift_mpo", "W"))
    Z = W >> 2
    assert W.bond_shape == tuple(g("rshift_mpo", "src_bond_shape"))
    assert rel(Z.to_tensor(), g("rshift_mpo", "Z_tensor")) < TOL
    # early exit returns the object itself; l*p < dim raises like the reference
    X = mps(g("rshift_mps_d2", "X"))
    assert (X >> 64) is X
    with pytest.raises(ValueError):
        mps(O.random_mps_cores(np.random.default_rng(0), 3, 2, 8)) >> 4
    with pytest.raises(Exception, match="integer"):
        X >> 2.0
    assert isinstance(MatrixProductState.empty(), MatrixProductState)


def test_random_orth_and_decompose(golden):
    from syngular_gb300.tensor import MatrixProductOperator, MatrixProductState

    g = golden("random_cases.npz")
    X = mps(g("orth_mps", "X"))
    X.left_orthonormalization()
    for k in range(3):
        np.testing.assert_allclose(X.left_orthogonality(k), g("orth_mps", "left_gram")[k], atol=1e-12)
    assert rel(O.to_tensor(host(X.sites)), O.to_tensor(g("orth_mps", "left"))) < TOL
    Xr = mps(g("orth_mps", "X"))
    Xr.right_orthonormalization()
    for k in range(3):
        np.testing.assert_allclose(Xr.right_orthogonality(k + 1), g("orth_mps", "right_gram")[k], atol=1e-12)
    assert rel(O.to_tensor(host(Xr.sites)), O.to_tensor(g("orth_mps", "right"))) < TOL
    D = MatrixProductState(g("decompose_mps", "t"), bond_shape=tuple(g("decompose_mps", "bonds"))).decompose()
    assert [tuple(s) for s in D.shape] == [tuple(s) for s in g("decompose_mps", "Z_shape")]
    assert rel(D.to_tensor(), g("decompose_mps", "Z_tensor")) < TOL
    D = MatrixProductOperator(g("decompose_mpo", "t"), bond_shape=tuple(g("decompose_mpo", "bonds"))).decompose()
    assert rel(D.to_tensor(), g("decompose_mpo", "Z_tensor")) < TOL


# ---------------------------------------------------------------------------
# TT-SVD rounding (no reference counterpart: checked against the oracle)
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("n,d,chi,D,cut", [(6, 2, 4, 3, 3), (8, 2, 16, 4, 12), (5, 3, 6, 2, 7),
                                           (12, 2, 64, 8, 64)])
def test_svd_round_matches_oracle(n, d, chi, D, cut):
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(n * 100 + chi)
    X = O.random_mps_cores(rng, n, d, chi)
    W = O.random_mpo_cores(rng, n, d, D)
    P = O.mpo_mps_product(W, X)
    Zr, spec_r, disc_r = O.tt_svd_round(P, cut)
    Pd = _ops.contract_mpo_mps(dev(W), dev(X))
    Z, spec, counts, disc, status = _ops.svd_round(Pd, cut)
    assert int(status.item()) >= 0
    assert [tuple(z.shape) for z in Z] == [z.shape for z in Zr]
    s = spec.cpu().numpy()
    off = 0
    for k in range(n - 1):
        np.testing.assert_allclose(s[off:off + counts[k]], spec_r[k], rtol=1e-11, atol=1e-14 * spec_r[k][0])
        off += counts[k]
    np.testing.assert_allclose(disc.cpu().numpy(), disc_r, rtol=1e-9, atol=1e-15)
    ov = _ops.overlap(dev(X), Z)
    ov_r = O.overlap(X, Zr)
    assert abs(ov - ov_r) <= TOL * 10 * abs(ov_r)
    # gauge-invariant: <Z|Z> and <Z|Zr>
    zz = _ops.overlap(Z, Z)
    assert abs(zz - O.overlap(Zr, Zr)) <= TOL * 10 * zz
    assert abs(_ops.overlap(Z, dev(Zr)) - zz) <= TOL * 10 * zz
    # right-orthonormal cores 1..n-1
    for k in range(1, n):
        G = _ops.orthogonality(Z[k], 1).cpu().numpy()
        np.testing.assert_allclose(G, np.eye(G.shape[0]), atol=1e-12)


def test_svd_round_exact_when_chi_covers_rank():
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(99)
    X = O.random_mps_cores(rng, 7, 2, 3)
    W = O.random_mpo_cores(rng, 7, 2, 2)
    P = O.mpo_mps_product(W, X)
    Z, *_ = _ops.svd_round(_ops.contract_mpo_mps(dev(W), dev(X)), 1000)
    assert rel(O.to_tensor(host(Z)), O.to_tensor(P)) < 1e-12


APPLY_CASES = ["test_apply", "h_site0", "x_site4", "cx_site1", "swap_site3", "rand2_d3", "rand1_d4",
               "rand2_d2_wide"]


@pytest.mark.parametrize("case", APPLY_CASES)
def test_mps_apply(golden, case):
    """MatrixProductState.apply on the device against the reference's cores
    (same QR sign convention, so the cores agree directly) and the oracle; the
    input state is unchanged (strict copy)."""
    g = golden("apply_cases.npz")
    xs, gate, idx = g(case, "x"), g(case, "gate"), int(g(case, "index"))
    X = mps(xs)
    Y = X.apply(gate, idx)
    ref = g(case, "out")
    out = host(Y.sites)
    assert [c.shape for c in out] == [c.shape for c in ref]
    for a, b in zip(out, ref):
        assert rel(a, b) < TOL
    for a, b in zip(out, O.mps_apply(xs, gate, idx)):
        assert rel(a, b) < TOL
    for a, b in zip(host(X.sites), xs):
        np.testing.assert_array_equal(a, b)
    assert Y.shape == X.shape


def test_mps_apply_errors():
    """The reference's failures: no working copy without strict (NameError),
    a window past the last site (IndexError)."""
    rng = np.random.default_rng(3)
    xs = [rng.standard_normal(s) for s in [(1, 2, 2), (2, 2, 2), (2, 2, 1)]]
    X = mps(xs)
    cx = np.eye(4)[[0, 1, 3, 2]].reshape(2, 2, 2, 2)
    with pytest.raises(NameError):
        X.apply(cx, 0, strict=False)
    with pytest.raises(IndexError):
        X.apply(cx, 2)


def test_mul(golden):
    """syngular.mul (tensor/utils.py:8-73) against the reference: shapes and
    reconstructions of MPS x MPO, MPO x MPS and MPO x MPO (each ending with
    >> min_bond), the MPS x MPS overlap, and the site-count error."""
    import syngular_gb300 as syn

    g = golden("mul_cases.npz")
    X, Y = mps(g("mul", "X")), mps(g("mul", "Y"))
    W, V = mpo(g("mul", "W")), mpo(g("mul", "V"))
    xw = syn.mul(X, W)
    assert [tuple(s) for s in xw.shape] == [c.shape for c in g("mul", "XW")]
    assert rel(xw.to_tensor(), g("mul", "XW_tensor")) < TOL
    wx = syn.mul(W, X)
    assert [tuple(s) for s in wx.shape] == [c.shape for c in g("mul", "WX")]
    assert rel(wx.to_tensor(), O.to_tensor(g("mul", "WX"))) < TOL
    xy = syn.mul(X, Y)
    ref = float(g("mul", "XY"))
    assert abs(float(xy) - ref) <= TOL * abs(ref)
    wv = syn.mul(W, V)
    assert [tuple(s) for s in wv.shape] == [c.shape for c in g("mul", "WV")]
    assert rel(wv.to_tensor(), g("mul", "WV_tensor")) < TOL
    with pytest.raises(Exception, match="same number of sites"):
        syn.mul(X, mpo(g("mul", "W")[:2]))
    # test/test_syn.py:10-26: arange operands (exact at this size)
    X, W = mps(g("syn", "X")), mpo(g("syn", "W"))
    assert rel(syn.mul(W, X, mode="standard").to_tensor(), g("syn", "WX_tensor")) < TOL
    assert rel(syn.mul(X, W, mode="standard").to_tensor(), g("syn", "XW_tensor")) < TOL
    assert abs(float(syn.mul(X, X, mode="standard")) - float(g("syn", "XX"))) <= TOL * 14.0
