"""Pin the numpy oracle against fixtures produced by the Python reference."""
import numpy as np
import pytest

from oracle import tt_fp64 as O
from tests.conftest import rel

TOL = 1e-12


def test_config1_flow(golden):
    g = golden("config1.npz")
    for seed in (1, 2):
        c = "seed%d" % seed
        W, X, Y = g(c, "W"), g(c, "X"), g(c, "Y")
        P = O.qr_truncate(O.mpo_mps_product(W, X), 8)
        assert rel(O.to_tensor(P), g(c, "P_tensor")) < TOL
        Z = O.qr_truncate(P, 4)
        assert rel(O.to_tensor(Z), g(c, "Z_tensor")) < TOL
        assert abs(O.overlap(Z, Y) - g(c, "zy")) <= TOL * abs(g(c, "zy"))
        assert abs(O.overlap(X, Y) - g(c, "xy")) <= TOL * abs(g(c, "xy"))
        Zo = O.left_orthonormalize(Z)
        np.testing.assert_allclose(np.diag(O.left_orthogonality(Zo[0])), g(c, "diag0"), atol=1e-12)
        np.testing.assert_allclose(np.diag(O.left_orthogonality(Zo[1])), g(c, "diag1"), atol=1e-12)
        assert [tuple(s.shape) for s in Zo] == [tuple(s) for s in g(c, "Z_shape")]


def test_config1_from_seed_matches_fixture(golden):
    g = golden("config1.npz")
    res = O.config1_flow(1)
    assert rel(O.to_tensor(res["Z"]), g("seed1", "Z_tensor")) < TOL
    assert abs(res["zy"] - g("seed1", "zy")) <= TOL * abs(g("seed1", "zy"))


def test_known_answers(golden):
    g = golden("known_answers.npz")
    # test/test_mpo.py:177-196: W @ W @ X with the lossy auto-round
    w = np.arange(16.0).reshape(2, 2, 2, 2)
    x = np.arange(4.0).reshape(2, 2)
    W = O.mpo_decompose(w, (2,))
    X = O.mps_decompose(x, (2,))
    # `W @ W @ X` is `(W @ W) @ X`; each `@` rounds to the smaller bond
    WW = O.qr_truncate(O.mpo_mpo_product(W, W), 2)
    Z = O.qr_truncate(O.mpo_mps_product(WW, X), min(4, 2))
    out = O.to_tensor(Z).reshape(4)
    np.testing.assert_allclose(out, g("mpo_matmul", "out"), rtol=1e-12)
    np.testing.assert_allclose(g("mpo_matmul", "out"),
                               [1509.179143, 1742.53175013, 2253.42694889, 2522.46360351], rtol=1e-8)
    # test/test_mpo.py:44-64
    Wd = O.mpo_decompose(w, (4,))
    assert abs(O.mpo_to_tensor(Wd)[1, 1, 1, 1] - 15) < 1e-12
    z = np.arange(4.0 ** 3 * 27).reshape(4, 4, 4, 3, 3, 3)
    Zd = O.mpo_decompose(z, (3, 3))
    assert abs(O.mpo_to_tensor(Zd)[3, 1, 0, 1, 2, 1] - g("mpo_decompose", "z")) < 1e-9
    assert abs(g("mpo_decompose", "z") - 1420) < 1e-9
    # test/test_mps.py:51-70
    x8 = np.arange(8.0).reshape(2, 2, 2)
    X = O.mps_decompose(x8, (2, 2))
    S = O.direct_sum(X, X)
    np.testing.assert_allclose(O.to_tensor(S), g("mps_add", "z_tensor"), atol=1e-12)
    np.testing.assert_allclose(O.to_tensor(S), 2 * x8, atol=1e-12)
    # test/test_mps.py:100-126
    x64 = np.arange(64.0).reshape(4, 4, 4)
    X = O.mps_decompose(x64, (4, 4))
    assert abs(O.dot(X) - g("mps_dot", "dot")) < 1e-9
    assert abs(g("mps_dot", "dot") - 292.1369541841634) < 1e-9
    assert abs(O.dot(O.normalize(X)) - 1.0) < 1e-12
    # test/test_mps.py:72-84
    Z = O.qr_truncate(X, 2)
    assert [c.shape for c in Z] == [tuple(s) for s in g("mps_compress", "z_shape")]
    assert rel(O.to_tensor(Z), g("mps_compress", "z_tensor")) < 1e-12


def test_mpo_add_chain(golden):
    """test/test_mpo.py:256-282: X + 9 Y with MPO auto-round to the min bond."""
    g = golden("known_answers.npz")
    x = np.arange(1.0, 17).reshape(2, 2, 2, 2)
    y = np.arange(18.0, 34).reshape(2, 2, 2, 2)
    X = O.mpo_decompose(x, (3,))
    Y = O.mpo_decompose(y, (3,))
    Z, zb = X, O.bond_shape_of(X)
    for _ in range(9):
        mb = min(min(zb), min(O.bond_shape_of(Y)))
        S = O.direct_sum(Z, Y)
        Z = O.qr_truncate(S, mb)
        zb = O.bond_shape_of(S)
    t = O.mpo_to_tensor(Z)
    assert abs(t[1, 1, 1, 1] - 313) < 1e-9
    np.testing.assert_allclose(t, g("mpo_add", "z_tensor"), atol=1e-9)


@pytest.mark.parametrize("n", [0, 1, 2])
def test_random_matmul_mps(golden, n):
    g = golden("random_cases.npz")
    c = "matmul_mps%d" % n
    X, W = g(c, "X"), g(c, "W")
    mb = min(min(O.bond_shape_of(W)), min(O.bond_shape_of(X)))
    Z = O.qr_truncate(O.mpo_mps_product(W, X), mb)
    assert [s.shape for s in Z] == [tuple(s) for s in g(c, "Z_shape")]
    assert rel(O.to_tensor(Z), g(c, "Z_tensor")) < TOL


@pytest.mark.parametrize("n", [0, 1])
def test_random_matmul_mpo(golden, n):
    g = golden("random_cases.npz")
    c = "matmul_mpo%d" % n
    A, B = g(c, "A"), g(c, "B")
    mb = min(min(O.bond_shape_of(A)), min(O.bond_shape_of(B)))
    Z = O.qr_truncate(O.mpo_mpo_product(A, B), mb)
    assert rel(O.mpo_to_tensor(Z), g(c, "Z_tensor")) < TOL


def test_random_add(golden):
    g = golden("random_cases.npz")
    Z = O.direct_sum(g("add_mps", "X"), g("add_mps", "Y"))
    for a, b in zip(Z, g("add_mps", "Z")):
        np.testing.assert_array_equal(a, b)
    A, B = g("add_mpo", "A"), g("add_mpo", "B")
    mb = min(min(O.bond_shape_of(A)), min(O.bond_shape_of(B)))
    Z = O.qr_truncate(O.direct_sum(A, B), mb)
    assert rel(O.mpo_to_tensor(Z), g("add_mpo", "Z_tensor")) < TOL


@pytest.mark.parametrize("n", [0, 1, 2])
def test_random_overlap(golden, n):
    g = golden("random_cases.npz")
    c = "overlap%d" % n
    v = O.overlap(g(c, "X"), g(c, "Y"))
    assert abs(v - g(c, "value")) <= TOL * max(1.0, abs(g(c, "value")))
    m, lg = O.overlap_log(g(c, "X"), g(c, "Y"))
    assert abs(m * np.exp(lg) - g(c, "value")) <= TOL * max(1.0, abs(g(c, "value")))


def test_random_rshift(golden):
    g = golden("random_cases.npz")
    for dim in (2, 3):
        c = "rshift_mps_d%d" % dim
        Z = O.qr_truncate(g(c, "X"), dim)
        assert [s.shape for s in Z] == [tuple(s) for s in g(c, "Z_shape")]
        assert rel(O.to_tensor(Z), g(c, "Z_tensor")) < TOL
    Z = O.qr_truncate(g("rshift_pad", "X"), 4, bond_shape=(2, 6))
    assert rel(O.to_tensor(Z), g("rshift_pad", "Z_tensor")) < TOL
    np.testing.assert_allclose(O.left_orthogonality(Z[0]), g("rshift_pad", "Z_gram0"), atol=1e-12)
    Z = O.qr_truncate(g("rshift_mpo", "W"), 2)
    assert rel(O.mpo_to_tensor(Z), g("rshift_mpo", "Z_tensor")) < TOL
    with pytest.raises(ValueError):
        O.qr_truncate(O.random_mps_cores(np.random.default_rng(0), 3, 2, 8), 4)


def test_random_orth(golden):
    g = golden("random_cases.npz")
    X = g("orth_mps", "X")
    L = O.left_orthonormalize(X)
    R = O.right_orthonormalize(X)
    for k in range(3):
        np.testing.assert_allclose(O.left_orthogonality(L[k]), g("orth_mps", "left_gram")[k], atol=1e-12)
        np.testing.assert_allclose(O.right_orthogonality(R[k + 1]), g("orth_mps", "right_gram")[k], atol=1e-12)
    assert rel(O.to_tensor(L), O.to_tensor(g("orth_mps", "left"))) < TOL
    assert rel(O.to_tensor(R), O.to_tensor(g("orth_mps", "right"))) < TOL


def test_random_decompose(golden):
    g = golden("random_cases.npz")
    Z = O.mps_decompose(g("decompose_mps", "t"), tuple(g("decompose_mps", "bonds")))
    assert [s.shape for s in Z] == [tuple(s) for s in g("decompose_mps", "Z_shape")]
    assert rel(O.to_tensor(Z), g("decompose_mps", "Z_tensor")) < TOL
    Z = O.mpo_decompose(g("decompose_mpo", "t"), tuple(g("decompose_mpo", "bonds")))
    assert rel(O.mpo_to_tensor(Z), g("decompose_mpo", "Z_tensor")) < TOL


def test_tt_svd_round_identities():
    """TT-SVD rounding (no reference counterpart): exact when chi covers the
    rank, the kept spectrum matches dense SVDs of the unfoldings, the discarded
    weight bounds the error (Oseledets 2011, Thm 2.2)."""
    rng = np.random.default_rng(5)
    X = O.random_mps_cores(rng, 6, 2, 4)
    W = O.random_mpo_cores(rng, 6, 2, 3)
    P = O.mpo_mps_product(W, X)
    T = O.to_tensor(P)
    Z, spec, disc = O.tt_svd_round(P, 64)
    assert rel(O.to_tensor(Z), T) < 1e-12
    for k in range(1, 6):
        s = np.linalg.svd(T.reshape(2 ** k, -1), compute_uv=False)
        np.testing.assert_allclose(spec[k - 1][: len(s)][:8], s[: len(spec[k - 1])][:8], rtol=1e-10)
    Z, spec, disc = O.tt_svd_round(P, 3)
    err = np.linalg.norm(O.to_tensor(Z) - T) ** 2 / np.linalg.norm(T) ** 2
    assert err <= sum(disc) * (1 + 1e-9)


APPLY_CASES = ["test_apply", "h_site0", "x_site4", "cx_site1", "swap_site3", "rand2_d3", "rand1_d4",
               "rand2_d2_wide"]


@pytest.mark.parametrize("case", APPLY_CASES)
def test_mps_apply(golden, case):
    """MatrixProductState.apply: the oracle's cores agree with the reference's
    directly (complete QR keeps LAPACK's sign convention), and the input chain is
    left unchanged (strict copy)."""
    g = golden("apply_cases.npz")
    xs = g(case, "x")
    before = [c.copy() for c in xs]
    out = O.mps_apply(xs, g(case, "gate"), int(g(case, "index")))
    ref = g(case, "out")
    assert [c.shape for c in out] == [c.shape for c in ref]
    for a, b in zip(out, ref):
        assert rel(a, b) < TOL
    for a, b in zip(xs, before):
        np.testing.assert_array_equal(a, b)
    if case == "test_apply":
        for a, b in zip(xs, g(case, "x_after")):
            np.testing.assert_array_equal(a, b)


def test_mul(golden):
    """syngular.mul (tensor/utils.py:8-73): the oracle's products against the
    reference's, cores directly (same QR sign convention) and reconstructions."""
    g = golden("mul_cases.npz")
    X, Y, W, V = g("mul", "X"), g("mul", "Y"), g("mul", "W"), g("mul", "V")
    kind, xw = O.mul("mps", X, "mpo", W)
    assert kind == "mps"
    for a, b in zip(xw, g("mul", "XW")):
        assert rel(a, b) < TOL
    assert rel(O.to_tensor(xw), g("mul", "XW_tensor")) < TOL
    _, wx = O.mul("mpo", W, "mps", X)
    for a, b in zip(wx, g("mul", "WX")):
        assert rel(a, b) < TOL
    kind, xy = O.mul("mps", X, "mps", Y)
    assert kind == "scalar" and abs(xy - float(g("mul", "XY"))) <= TOL * abs(xy)
    kind, wv = O.mul("mpo", W, "mpo", V)
    assert kind == "mpo"
    for a, b in zip(wv, g("mul", "WV")):
        assert rel(a, b) < TOL
    assert rel(O.mpo_to_tensor(wv), g("mul", "WV_tensor")) < TOL
    with pytest.raises(Exception, match="same number of sites"):
        O.mul("mps", X, "mpo", W[:2])
    # test/test_syn.py:10-26: arange operands, exact at this size
    X, W = g("syn", "X"), g("syn", "W")
    _, wx = O.mul("mpo", W, "mps", X)
    assert rel(O.to_tensor(wx), g("syn", "WX_tensor")) < TOL
    _, xw = O.mul("mps", X, "mpo", W)
    assert rel(O.to_tensor(xw), g("syn", "XW_tensor")) < TOL
    np.testing.assert_allclose(O.to_tensor(xw).reshape(-1), g("syn", "exact_xw"), rtol=1e-12)
    _, xx = O.mul("mps", X, "mps", X)
    assert abs(xx - float(g("syn", "XX"))) <= TOL * abs(xx)


@pytest.mark.parametrize("case", ["dmrg_a", "dmrg_b"])
def test_dmrg_environment(golden, case):
    """Environment blocks and the sweep's two-site tensors (variational/dmrg.py:65-165)."""
    g = golden("dmrg_cases.npz")
    W, X = g(case, "W"), g(case, "X")
    n = len(W)
    left = O.env_left_blocks(W, X)
    right = O.env_right_blocks(W, X)
    for k in range(n):
        if k <= n - 3:
            assert rel(left[k], g(case, "left/%d" % k)) < TOL
        else:
            assert left[k] is None
        if k >= 2:
            assert rel(right[k], g(case, "right/%d" % k)) < TOL
        else:
            assert right[k] is None
    # the sweep uses the blocks built before it (dmrg.py:41-42), with the state's current sites
    steps = int(g(case, "steps"))
    assert steps == n - 1
    for k in range(steps):
        x0, x1 = g(case, "step/%d/x0" % k), g(case, "step/%d/x1" % k)
        merge = np.tensordot(x0, x1, axes=([2], [0]))
        Lb = None if k == 0 else left[k - 1]
        Rb = None if k == n - 2 else right[k + 2]
        site = O.env_two_site(Lb, merge, W[k], W[k + 1], Rb)
        assert rel(site, g(case, "step/%d/site" % k)) < TOL
