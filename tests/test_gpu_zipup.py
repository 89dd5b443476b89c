"""Zip-up MPO x MPS (sgt_mpo_mps_zipup, MATMUL_MODE "zip-up") against the
numpy restatement of the same algorithm (oracle.tt_fp64.zipup): FP64, so the
gauge-invariant results (overlaps, norms, discarded weights) agree to 1e-10
relative; with chi covering every bond's rank the result is the exact
product."""
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


def dev(cores):
    from syngular_gb300 import _lib

    return [_lib.as_device(c) for c in cores]


@pytest.mark.parametrize("n,d,chi,D,cut", [(6, 2, 8, 3, 5), (10, 2, 16, 4, 12), (8, 3, 12, 2, 20), (12, 2, 32, 4, 24)])
def test_zipup_matches_oracle(n, d, chi, D, cut):
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(500 + n * chi)
    X = O.random_mps_cores(rng, n, d, chi)
    W = O.random_mpo_cores(rng, n, d, D)
    Y = O.random_mps_cores(rng, n, d, 7)
    Zr, disc_r = O.zipup(W, X, cut)
    Z, disc, status = _ops.mpo_mps_zipup(dev(W), dev(X), cut)
    torch.cuda.synchronize()
    assert int(status.item()) >= 0
    assert [tuple(z.shape) for z in Z] == [z.shape for z in Zr]
    zz_r = O.overlap(Zr, Zr)
    assert abs(_ops.overlap(Z, Z) - zz_r) <= 1e-10 * zz_r
    yy = O.overlap(Y, Y)
    assert abs(_ops.overlap(dev(Y), Z) - O.overlap(Y, Zr)) <= 1e-10 * np.sqrt(yy * zz_r)
    np.testing.assert_allclose(disc.cpu().numpy()[: n - 1], disc_r, rtol=1e-8, atol=1e-14)
    # cores before the last are left-orthonormal
    for k in range(n - 1):
        m = Z[k].reshape(-1, Z[k].shape[-1]).cpu().numpy()
        np.testing.assert_allclose(m.T @ m, np.eye(m.shape[1]), rtol=0, atol=1e-12)


def test_zipup_exact_when_chi_covers_rank():
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(42)
    X = O.random_mps_cores(rng, 7, 2, 6)
    W = O.random_mpo_cores(rng, 7, 2, 3)
    P = O.mpo_mps_product(W, X)
    Z, disc, status = _ops.mpo_mps_zipup(dev(W), dev(X), 1000)
    pp = O.overlap(P, P)
    assert abs(_ops.overlap(Z, Z) - pp) <= 1e-12 * pp
    assert abs(_ops.overlap(Z, dev(P)) - pp) <= 1e-12 * pp
    assert float(disc.max().item()) <= 1e-20


def test_matmul_mode_zipup():
    """The drop-in operator with MATMUL_MODE = "zip-up": the state is made
    right-orthonormal (exact FP64 TT-SVD at its own bonds), then zipped up to
    the min bond; compared with the oracle doing the same."""
    from syngular_gb300.tensor import MatrixProductOperator, MatrixProductState, _ops

    rng = np.random.default_rng(8)
    Xc = O.random_mps_cores(rng, 9, 2, 12)
    Wc = O.random_mpo_cores(rng, 9, 2, 4)
    saved = MatrixProductOperator.MATMUL_MODE
    try:
        MatrixProductOperator.MATMUL_MODE = "zip-up"
        Z = MatrixProductOperator.from_sites(Wc) @ MatrixProductState.from_sites(Xc)
    finally:
        MatrixProductOperator.MATMUL_MODE = saved
    Xr, _s, _d = O.tt_svd_round(Xc, 10 ** 6)
    Zr, _disc = O.zipup(Wc, Xr, 4)
    zz = O.overlap(Zr, Zr)
    assert abs(_ops.overlap(Z.sites, Z.sites) - zz) <= 1e-10 * zz
    assert abs(_ops.overlap(dev(Xc), Z.sites) - O.overlap(Xc, Zr)) <= 1e-10 * np.sqrt(O.overlap(Xc, Xc) * zz)
