"""Size-independent properties of the oracle's restatements that no reference
test pins: the zip-up product (the reference's "variational" / "fit-up"
MATMUL_MODE branches are empty, tensor/matrix_product_operator.py:262-276) and
the DMRG environment blocks with a bra and a ket that differ
(variational/dmrg.py:65-112 uses one state for both).  CPU only."""
import numpy as np
import pytest

from oracle import tt_fp64 as O


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.mark.parametrize("n,d,chi,D", [(5, 2, 3, 2), (4, 3, 2, 3), (6, 2, 4, 2)])
def test_zipup_exact_when_chi_covers_rank(n, d, chi, D):
    """With chi at least every bond's rank the zip-up is exact: the dense
    tensor equals the raw product's and nothing is discarded."""
    rng = np.random.default_rng(100 * n + chi)
    X, W = O.random_mps_cores(rng, n, d, chi), O.random_mpo_cores(rng, n, d, D)
    Z, disc = O.zipup(W, X, 10 ** 6)
    assert rel(O.to_tensor(Z), O.to_tensor(O.mpo_mps_product(W, X))) < 1e-12
    assert len(disc) == n - 1 and max(disc) < 1e-26


@pytest.mark.parametrize("cut", [1, 2, 4])
def test_zipup_truncated_cores_and_weights(cut):
    """Truncated: every core but the last is left-orthonormal, the bonds are
    min(cut, rank bound), each discarded weight lies in [0, 1), and the norm of
    the result is the norm of its last core (the carry holds the weight)."""
    rng = np.random.default_rng(5)
    n, d, chi, D = 6, 2, 4, 3
    X, W = O.random_mps_cores(rng, n, d, chi), O.random_mpo_cores(rng, n, d, D)
    Z, disc = O.zipup(W, X, cut)
    for z in Z[:-1]:
        m = z.reshape(-1, z.shape[2])
        np.testing.assert_allclose(m.T @ m, np.eye(m.shape[1]), atol=1e-12)
        assert z.shape[2] <= cut
    assert all(0.0 <= w < 1.0 for w in disc)
    assert abs(np.sqrt(O.overlap(Z, Z)) - np.linalg.norm(Z[-1])) <= 1e-12 * np.linalg.norm(Z[-1])


@pytest.mark.parametrize("n,d,chi,D", [(5, 2, 3, 2), (6, 3, 2, 2), (7, 2, 4, 3)])
def test_environment_blocks_split_the_expectation(n, d, chi, D):
    """<X|W|Y> (X on the operator's output leg, Y on its input leg, no
    conjugate) equals sum(L_k * R_{k+1}) at every cut and the two-site tensor
    contracted with the bra's merged pair at every step."""
    rng = np.random.default_rng(17 * n + D)
    X, Y = O.random_mps_cores(rng, n, d, chi), O.random_mps_cores(rng, n, d, chi)
    W = O.random_mpo_cores(rng, n, d, D)
    E = O.overlap(X, O.mpo_mps_product(W, Y))
    left, right = O.env_left_blocks(W, X, Y), O.env_right_blocks(W, X, Y)
    for k in range(1, n - 2):
        assert abs(float(np.sum(left[k] * right[k + 1])) - E) <= 1e-12 * abs(E)
    for k in range(n - 1):
        ket = np.tensordot(Y[k], Y[k + 1], axes=([2], [0]))
        bra = np.tensordot(X[k], X[k + 1], axes=([2], [0]))
        Lb = None if k == 0 else left[k - 1]
        Rb = None if k == n - 2 else right[k + 2]
        site = O.env_two_site(Lb, ket, W[k], W[k + 1], Rb)
        assert abs(float(np.sum(site * bra)) - E) <= 1e-12 * abs(E)
