"""Parity of sgt_mpo_mps_round at the benchmark's core shapes (MPS bond 256,
d = 2; MPO bond 16, 2 x 2 legs; product bond 4096; reference operation
``(W @ X) >> chi`` of tensor/matrix_product_operator.py:181-192 with TT-SVD
rounding), in the plain FP64 form (1e-12 relative) and the FP64-class BF16X6
form (plain relative 1e-6 on <X|Z> and <Z|Z>, the mixed-precision accuracy
bound), against the FP64 oracle: live on an 8-site chain, and through golden
values (tests/golden/make_config2_cores.py) on 20- and 24-site chains whose
middle bonds truncate 512 down to 256.  Spectra: kept singular values to 1e-12
(FP64) / 1e-8 (BF16X6) of the largest; the discarded tail as squares, to 1e-12 (FP64) / 1e-4 (BF16X6) of
the largest square: the BF16X6 bond solve works on squared singular values
and its FP32 first approximation resolves eigenvectors only down to ~1e-5 of
the largest eigenvalue (measured), below which the refinement keeps pairs
whose correction would not be small; the kept subspace, and so the rounded
state, is not affected."""
import math

import numpy as np
import pytest
import torch

from oracle import tt_fp64 as O

pytestmark = pytest.mark.gpu

CHI, D, DPHYS = 256, 16, 2


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def dev(cores):
    from syngular_gb300 import _lib

    return [_lib.as_device(c) for c in cores]


def decode(v):
    return math.ldexp(float(v[0]), int(v[1]))


def run(W, X, prec):
    from syngular_gb300.tensor import _ops

    Xd, Wd = dev(X), dev(W)
    Z, spec, counts, disc, status = _ops.mpo_mps_round(Wd, Xd, CHI, prec)
    xz = _ops.decode_overlap(_ops.overlap_device(Xd, Z).cpu().tolist())
    zz = _ops.decode_overlap(_ops.overlap_device(Z, Z).cpu().tolist())
    torch.cuda.synchronize()
    return Z, spec.cpu().numpy(), counts, disc.cpu().numpy(), int(status.item()), xz, zz


@pytest.mark.parametrize("prec_name,tol_ov,tol_spec,tol_tail", [("f64", 1e-12, 1e-12, 1e-12),
                                                                 ("bf16x6", 1e-6, 1e-8, 1e-4)])
def test_eight_sites_live(prec_name, tol_ov, tol_spec, tol_tail):
    from syngular_gb300 import _lib as L

    prec = {"f64": L.PREC_F64, "bf16x6": L.PREC_BF16X6}[prec_name]
    rng = np.random.default_rng(8)
    X = O.random_mps_cores(rng, 8, DPHYS, CHI)
    W = O.random_mpo_cores(rng, 8, DPHYS, D)
    Zr, spec_r, disc_r = O.tt_svd_round(O.mpo_mps_product(W, X), CHI)
    Z, spec, counts, disc, status, xz, zz = run(W, X, prec)
    assert status >= 0
    assert [tuple(z.shape) for z in Z] == [z.shape for z in Zr]
    xzr, zzr = O.overlap(X, Zr), O.overlap(Zr, Zr)
    assert abs(xz - xzr) / abs(xzr) < tol_ov, (xz, xzr)
    assert abs(zz - zzr) / abs(zzr) < tol_ov, (zz, zzr)
    check_spectra(spec, counts, spec_r, 8, CHI, tol_spec, tol_tail)


def check_spectra(spec, counts, spec_r, n, keep, tol_kept, tol_sq_tail):
    """Kept singular values to tol_kept of the largest; the discarded tail as
    squares, |s'^2 - s^2| <= tol_sq_tail s_max^2: a Gram-form solve works on
    s^2, so a singular value near zero is only as good as the square root of
    its eigenvalue's error."""
    off = 0
    for k in range(n - 1):
        m = min(counts[k], len(spec_r[k]))
        s, r = spec[off:off + m], spec_r[k][:m]
        kk = min(keep, m)
        np.testing.assert_allclose(s[:kk], r[:kk], rtol=0, atol=tol_kept * r[0])
        np.testing.assert_allclose(s[kk:] ** 2, r[kk:] ** 2, rtol=0, atol=tol_sq_tail * r[0] ** 2)
        off += counts[k]


def golden_inputs(n, seed):
    rng = np.random.default_rng(seed)
    return O.random_mps_cores(rng, n, DPHYS, CHI), O.random_mpo_cores(rng, n, DPHYS, D)


@pytest.mark.parametrize("case,n,seed", [("n20", 20, 11), ("n24", 24, 12)])
@pytest.mark.parametrize("prec_name,tol_ov,tol_spec,tol_tail", [("f64", 1e-12, 1e-12, 1e-12),
                                                                 ("bf16x6", 1e-6, 1e-8, 1e-4)])
def test_truncating_chains_golden(golden, case, n, seed, prec_name, tol_ov, tol_spec, tol_tail):
    from syngular_gb300 import _lib as L

    prec = {"f64": L.PREC_F64, "bf16x6": L.PREC_BF16X6}[prec_name]
    g = golden("config2_cores.npz")
    X, W = golden_inputs(n, seed)
    Z, spec, counts, disc, status, xz, zz = run(W, X, prec)
    assert status >= 0
    xzr, zzr = decode(g(case, "xz")), decode(g(case, "zz"))
    assert abs(xz - xzr) / abs(xzr) < tol_ov, (xz, xzr)
    assert abs(zz - zzr) / abs(zzr) < tol_ov, (zz, zzr)
    spec_r = g(case, "spectra")
    check_spectra(spec, counts, spec_r, n, CHI, tol_spec, tol_tail)
    np.testing.assert_allclose(disc[: n - 1], g(case, "discarded"), rtol=1e-6, atol=1e-14)
    # the middle bonds really truncate (product rank 512 / 1024 > 256)
    assert max(g(case, "discarded")) > 1e-3


@pytest.mark.parametrize("case,n,seed", [("n20", 20, 11), ("n24", 24, 12)])
def test_truncating_chains_golden_without_spectra(golden, case, n, seed):
    """The BF16X6 form without spectra (kept subspaces by purification, the
    path of ``(W @ X) >> chi`` through the API) at the benchmark's shapes."""
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    g = golden("config2_cores.npz")
    X, W = golden_inputs(n, seed)
    Xd, Wd = dev(X), dev(W)
    Z, spec, counts, disc, status = _ops.mpo_mps_round(Wd, Xd, CHI, L.PREC_BF16X6, spectra=False)
    xz = _ops.decode_overlap(_ops.overlap_device(Xd, Z).cpu().tolist())
    zz = _ops.decode_overlap(_ops.overlap_device(Z, Z).cpu().tolist())
    torch.cuda.synchronize()
    assert int(status.item()) >= 0
    xzr, zzr = decode(g(case, "xz")), decode(g(case, "zz"))
    assert abs(xz - xzr) / abs(xzr) < 1e-6, (xz, xzr)
    assert abs(zz - zzr) / abs(zzr) < 1e-6, (zz, zzr)
    np.testing.assert_allclose(disc.cpu().numpy()[: n - 1], g(case, "discarded"), rtol=1e-6, atol=1e-9)
