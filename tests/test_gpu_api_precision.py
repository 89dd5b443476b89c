"""The drop-in API reaches the fused rounding path: with AUTO_ROUND off,
ROUNDING = "svd" and a precision policy, ``(W @ X) >> chi``
(tensor/matrix_product_operator.py:181-192 without the auto-round, then
tensor/matrix_product_state.py:139-143) runs sgt_mpo_mps_round on the two
factors without forming the product, bit for bit the same as the direct call."""
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


@pytest.fixture
def policy():
    from syngular_gb300.tensor import MatrixProductOperator, MatrixProductState

    saved = (MatrixProductOperator.AUTO_ROUND, MatrixProductOperator.PRECISION, MatrixProductOperator.ROUNDING,
             MatrixProductState.ROUNDING, MatrixProductState.PRECISION)
    yield MatrixProductOperator, MatrixProductState
    (MatrixProductOperator.AUTO_ROUND, MatrixProductOperator.PRECISION, MatrixProductOperator.ROUNDING,
     MatrixProductState.ROUNDING, MatrixProductState.PRECISION) = saved


@pytest.mark.parametrize("prec", ["bf16x6", "f64", "tf32x3"])
def test_lazy_product_round_is_the_fused_call(policy, prec):
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    MPO, MPS = policy
    MPO.AUTO_ROUND = False
    MPO.PRECISION = prec
    MPS.ROUNDING = "svd"
    rng = np.random.default_rng(5)
    X = MPS.from_sites(O.random_mps_cores(rng, 10, 2, 16))
    W = MPO.from_sites(O.random_mpo_cores(rng, 10, 2, 8))
    P = W @ X
    assert P.bond_shape == tuple([16 * 8] * 9) and P._sites is None
    Z = P >> 24
    assert P._sites is None, "the product was formed"
    ref, _s, _c, _d, _st = _ops.mpo_mps_round(W.sites, X.sites, 24, {"bf16x6": L.PREC_BF16X6, "f64": L.PREC_F64,
                                                                     "tf32x3": L.PREC_TF32X3}[prec], spectra=False)
    assert len(Z.sites) == len(ref)
    for a, b in zip(Z.sites, ref):
        assert torch.equal(a, b)
    # the overlap through the API equals the FP64 oracle's within the form's bound
    Zr, _, _ = O.tt_svd_round(O.mpo_mps_product([w.cpu().numpy() for w in W.sites],
                                                [x.cpu().numpy() for x in X.sites]), 24)
    ov = X | Z
    ovr = O.overlap([x.cpu().numpy() for x in X.sites], Zr)
    tol = {"bf16x6": 1e-6, "f64": 1e-12, "tf32x3": 1e-2}[prec]
    assert abs(ov - ovr) / abs(ovr) < tol


def test_lazy_product_materialises_on_read(policy):
    from syngular_gb300.tensor import _ops

    MPO, MPS = policy
    MPO.AUTO_ROUND = False
    rng = np.random.default_rng(6)
    X = MPS.from_sites(O.random_mps_cores(rng, 5, 2, 4))
    W = MPO.from_sites(O.random_mpo_cores(rng, 5, 2, 3))
    P = W @ X
    raw = _ops.contract_mpo_mps(W.sites, X.sites)
    for a, b in zip(P.sites, raw):
        assert torch.equal(a, b)
    assert [tuple(s.shape) for s in P.sites] == P.shape


def test_auto_round_svd_on_the_operator_class(policy):
    """AUTO_ROUND on with the operator class's ROUNDING = "svd": `@` ends with
    the fused round to min_bond (mpo:192) in the operator's precision."""
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    MPO, MPS = policy
    MPO.AUTO_ROUND = True
    MPO.ROUNDING = "svd"
    MPO.PRECISION = "bf16x6"
    rng = np.random.default_rng(9)
    X = MPS.from_sites(O.random_mps_cores(rng, 8, 2, 12))
    W = MPO.from_sites(O.random_mpo_cores(rng, 8, 2, 4))
    Z = W @ X
    ref, _s, _c, _d, _st = _ops.mpo_mps_round(W.sites, X.sites, 4, L.PREC_BF16X6, spectra=False)
    for a, b in zip(Z.sites, ref):
        assert torch.equal(a, b)


@pytest.mark.parametrize("prec", ["bf16x6", "f64"])
def test_matmul_mode_opti_is_the_density_matrix_round(policy, prec):
    """MATMUL_MODE = "opti" (the reference's unfinished density-matrix
    compression, mpo:193-273) gives the optimal truncation to min_bond: the
    fused product + TT-SVD round, against the FP64 oracle's rounding."""
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    MPO, MPS = policy
    saved = MPO.MATMUL_MODE
    try:
        MPO.MATMUL_MODE = "opti"
        MPO.PRECISION = prec
        rng = np.random.default_rng(19)
        Xc = O.random_mps_cores(rng, 8, 2, 12)
        Wc = O.random_mpo_cores(rng, 8, 2, 4)
        X, W = MPS.from_sites(Xc), MPO.from_sites(Wc)
        Z = W @ X
        code = L.PREC_BF16X6 if prec == "bf16x6" else L.PREC_F64
        ref, _s, _c, _d, _st = _ops.mpo_mps_round(W.sites, X.sites, 4, code, spectra=False)
        for a, b in zip(Z.sites, ref):
            assert torch.equal(a, b)
        Zo, _sp, _di = O.tt_svd_round(O.mpo_mps_product(Wc, Xc), 4)
        zz = O.overlap(Zo, Zo)
        assert abs(_ops.overlap(X.sites, Z.sites) - O.overlap(Xc, Zo)) <= 1e-8 * np.sqrt(O.overlap(Xc, Xc) * zz)
    finally:
        MPO.MATMUL_MODE = saved
