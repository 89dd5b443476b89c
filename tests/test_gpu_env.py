"""GPU parity of the DMRG environment blocks and the two-site effective
contraction (reference: variational/dmrg.py:65-165) against the fixtures
written by running the reference, and against the numpy oracle on larger
seeded chains (bra and ket different).  FP64: 1e-12 relative."""
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


def _objs(W, X):
    from syngular_gb300.tensor import MatrixProductOperator, MatrixProductState

    return (MatrixProductOperator.from_sites([np.asarray(c) for c in W]),
            MatrixProductState.from_sites([np.asarray(c) for c in X]))


@pytest.mark.parametrize("case", ["dmrg_a", "dmrg_b"])
def test_blocks_and_sites_match_reference(golden, case):
    from syngular_gb300.tensor import MatrixProductState
    from syngular_gb300.variational import DMRG

    g = golden("dmrg_cases.npz")
    W, X = g(case, "W"), g(case, "X")
    n = len(W)
    op, st = _objs(W, X)
    left = DMRG.left_blocks(op, st)
    right = DMRG.right_blocks(op, st)
    for k in range(n):
        if k <= n - 3:
            assert rel(left[k].cpu().numpy(), g(case, "left/%d" % k)) < TOL
        else:
            assert left[k] is None
        if k >= 2:
            assert rel(right[k].cpu().numpy(), g(case, "right/%d" % k)) < TOL
        else:
            assert right[k] is None
    for k in range(int(g(case, "steps"))):
        sites = [np.asarray(c) for c in X]
        sites[k], sites[k + 1] = g(case, "step/%d/x0" % k), g(case, "step/%d/x1" % k)
        cur = MatrixProductState.from_sites(sites)
        site = DMRG.effective_site(op, cur, left, right, k)
        assert rel(site.cpu().numpy(), g(case, "step/%d/site" % k)) < TOL


@pytest.mark.parametrize("n,d,chi,D", [(6, 2, 16, 4), (10, 2, 64, 8), (5, 3, 40, 5)])
def test_blocks_bra_ket_match_oracle(n, d, chi, D):
    from syngular_gb300.tensor import MatrixProductState
    from syngular_gb300.variational import DMRG

    rng = np.random.default_rng(100 + n)
    X = O.random_mps_cores(rng, n, d, chi)
    Y = O.random_mps_cores(rng, n, d, max(2, chi // 2 + 1))
    W = O.random_mpo_cores(rng, n, d, D)
    op, ket = _objs(W, Y)
    bra = MatrixProductState.from_sites([np.asarray(c) for c in X])
    left = DMRG.left_blocks(op, ket, bra=bra)
    right = DMRG.right_blocks(op, ket, bra=bra)
    lo = O.env_left_blocks(W, X, Y)
    ro = O.env_right_blocks(W, X, Y)
    for k in range(n):
        if lo[k] is not None:
            assert rel(left[k].cpu().numpy(), lo[k]) < TOL
        if ro[k] is not None:
            assert rel(right[k].cpu().numpy(), ro[k]) < TOL
    # <X|W|Y> closes from any split: L_{k} . R_{k+1}
    full = float(np.einsum("abc,abc->", lo[0], ro[1])) if n == 3 else float(np.einsum("abc,abc->", lo[1], ro[2]))
    assert abs(float((left[1] * right[2]).sum()) - full) <= TOL * abs(full) * 10
    # two-site tensor at an interior step, the state as ket (reference convention)
    opx, stx = _objs(W, X)
    lx, rx = DMRG.left_blocks(opx, stx), DMRG.right_blocks(opx, stx)
    k = n // 2 - 1
    site = DMRG.effective_site(opx, stx, lx, rx, k)
    lo = O.env_left_blocks(W, X)
    ro = O.env_right_blocks(W, X)
    merge = np.tensordot(X[k], X[k + 1], axes=([2], [0]))
    ref = O.env_two_site(lo[k - 1] if k > 0 else None, merge, W[k], W[k + 1], ro[k + 2] if k + 2 < n else None)
    assert rel(site.cpu().numpy(), ref) < TOL


def test_env_errors():
    from syngular_gb300 import _lib as L
    from syngular_gb300.variational import DMRG

    rng = np.random.default_rng(3)
    X = O.random_mps_cores(rng, 4, 2, 4)
    W = O.random_mpo_cores(rng, 4, 3, 2)   # operator legs 3 != state leg 2
    op, st = _objs(W, X)
    with pytest.raises(L.SyngularError):
        DMRG.left_blocks(op, st)
    W = O.random_mpo_cores(rng, 4, 2, 2)
    op, st = _objs(W, X)
    with pytest.raises(Exception):
        DMRG.effective_site(op, st, [None] * 4, [None] * 4, 1)
