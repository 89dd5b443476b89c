"""Fused MPO x MPS + TT-SVD round in every precision against the FP64 oracle.

FP64: 1e-12 relative on gauge-invariant quantities.  Mixed precision (Gram form
on tcgen05): the overlap <X|Z> is a small fraction of |X||Z| for a random
operator, so its relative error is reported together with the error
normalised by |X||Z|; tolerances: 3xTF32 normalised 1e-6 and kept singular
values 1e-4 relative to the largest; one-pass TF32 normalised 1e-3."""
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


CASES = [(6, 2, 8, 3, 5), (10, 2, 32, 4, 24), (8, 3, 16, 4, 20), (12, 2, 64, 8, 64), (8, 2, 32, 16, 48),
         (7, 3, 16, 8, 30)]


@pytest.mark.parametrize("n,d,chi,D,cut", CASES)
@pytest.mark.parametrize("prec,tol_norm,tol_spec", [(0, 1e-13, 1e-11), (4, 1e-6, 1e-4), (1, 1e-3, 3e-2)])
def test_mpo_mps_round(n, d, chi, D, cut, prec, tol_norm, tol_spec):
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(1000 * n + chi)
    X = O.random_mps_cores(rng, n, d, chi)
    W = O.random_mpo_cores(rng, n, d, D)
    Zr, spec_r, disc_r = O.tt_svd_round(O.mpo_mps_product(W, X), cut)
    Z, spec, counts, disc, status = _ops.mpo_mps_round(dev(W), dev(X), cut, prec)
    torch.cuda.synchronize()
    assert int(status.item()) >= 0
    assert [tuple(z.shape) for z in Z] == [z.shape for z in Zr]
    Xd = dev(X)
    ov, ovr = _ops.overlap(Xd, Z), O.overlap(X, Zr)
    nx, nz = np.sqrt(O.overlap(X, X)), np.sqrt(O.overlap(Zr, Zr))
    assert abs(ov - ovr) / (nx * nz) < tol_norm
    zz = _ops.overlap(Z, Z)
    assert abs(zz - nz * nz) / (nz * nz) < max(tol_norm * 100, 1e-12)
    s = spec.cpu().numpy()
    off = 0
    for k in range(n - 1):
        m = min(counts[k], len(spec_r[k]), cut)
        np.testing.assert_allclose(s[off:off + m], spec_r[k][:m], rtol=0, atol=tol_spec * spec_r[k][0])
        off += counts[k]
    if prec == 0:
        assert abs(ov - ovr) <= 1e-11 * abs(ovr)
        np.testing.assert_allclose(disc.cpu().numpy(), disc_r, rtol=1e-9, atol=1e-15)


@pytest.mark.parametrize("method", [1, 2, 3])
def test_mpo_mps_round_eig_methods(method):
    """The three bond eigensolvers of the Gram form give the same rounded state
    (3xTF32, a chain whose bond problems are 128 x 128)."""
    from syngular_gb300.tensor import _ops

    n, d, chi, D, cut = 10, 2, 32, 8, 64
    rng = np.random.default_rng(77)
    X = O.random_mps_cores(rng, n, d, chi)
    W = O.random_mpo_cores(rng, n, d, D)
    Zr, spec_r, _ = O.tt_svd_round(O.mpo_mps_product(W, X), cut)
    prev = _ops.eig_method(method)
    try:
        Z, spec, counts, disc, status = _ops.mpo_mps_round(dev(W), dev(X), cut, 4)
        torch.cuda.synchronize()
    finally:
        _ops.eig_method(prev)
    assert int(status.item()) >= 0
    Zd = [torch.from_numpy(z).cuda() for z in Zr]
    nz = np.sqrt(O.overlap(Zr, Zr))
    fid = abs(_ops.overlap(Z, Zd)) / (np.sqrt(abs(_ops.overlap(Z, Z))) * nz)
    assert 1 - fid < 1e-8


@pytest.mark.parametrize("n,d,chi,cut,summed", [(8, 2, 32, 16, False), (6, 3, 20, 12, False), (8, 2, 24, 24, True)])
def test_svd_round_gram_form(n, d, chi, cut, summed):
    """TT-SVD rounding of a plain chain (and of a direct sum) through the Gram
    form: the chain is routed through the MPO x MPS pipeline with bond-1
    identity cores; 3xTF32 against the FP64 oracle."""
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(500 + n * d + chi)
    X = O.random_mps_cores(rng, n, d, chi)
    if summed:
        X = O.direct_sum(X, O.random_mps_cores(rng, n, d, chi))
    Zr, spec_r, disc_r = O.tt_svd_round(X, cut)
    Z, spec, counts, disc, status = _ops.svd_round(dev(X), cut, 4)
    torch.cuda.synchronize()
    assert int(status.item()) >= 0
    assert [tuple(z.shape) for z in Z] == [z.shape for z in Zr]
    Xd = dev(X)
    ov, ovr = _ops.overlap(Xd, Z), O.overlap(X, Zr)
    nx, nz = np.sqrt(O.overlap(X, X)), np.sqrt(O.overlap(Zr, Zr))
    assert abs(ov - ovr) / (nx * nz) < 1e-6
    s = spec.cpu().numpy()
    off = 0
    for k in range(n - 1):
        m = min(counts[k], len(spec_r[k]), cut)
        np.testing.assert_allclose(s[off:off + m], spec_r[k][:m], rtol=0, atol=1e-4 * spec_r[k][0])
        off += counts[k]
    np.testing.assert_allclose(disc.cpu().numpy(), disc_r, rtol=0, atol=1e-5)
