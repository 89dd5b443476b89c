"""The allocation-free overlap entry point, through the C ABI.

It exists for callers that cannot give the library scratch memory (no
allocator of their own, or a process whose device memory belongs to another
framework's pool).  Its result must match the workspace-based
`sgt_overlap_sweep` within the FP64 tolerance used everywhere else (1e-12
relative), on two calls in a row: the shared static scratch keeps the first
call's contents, which the second call must not read as live data.  This file
is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def chain(rng, n, d, chi):
    dims = [1] + [chi] * (n - 1) + [1]
    return [torch.from_numpy(rng.standard_normal((dims[k], d, dims[k + 1])) / np.sqrt(chi * d)).cuda()
            for k in range(n)]


def both(X, Y):
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor import _ops

    n = len(X)
    xs, _a = L.shape_array([tuple(c.shape) for c in X])
    ys, _b = L.shape_array([tuple(c.shape) for c in Y])
    xp, _c = L.ptr_array(X)
    yp, _d = L.ptr_array(Y)
    res = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    L.call("sgt_overlap_sweep_noalloc", n, xp, xs, yp, ys, L.ptr(res), L.stream_ptr())
    ref = _ops.overlap_device(X, Y)
    torch.cuda.synchronize()
    return _ops.decode_overlap(res.cpu().tolist()), _ops.decode_overlap(ref.cpu().tolist())


def test_noalloc_overlap_matches_workspace_version_twice():
    rng = np.random.default_rng(42)
    X1, Y1 = chain(rng, 12, 3, 64), chain(rng, 12, 3, 48)
    X2, Y2 = chain(rng, 20, 2, 256), chain(rng, 20, 2, 200)
    for X, Y in ((X1, Y1), (X2, Y2)):
        got, ref = both(X, Y)
        assert np.isfinite(got)
        assert abs(got - ref) <= TOL * abs(ref), (got, ref)
    # and the first case again, after the larger one filled the shared array
    got, ref = both(X1, Y1)
    assert abs(got - ref) <= TOL * abs(ref), (got, ref)


def test_noalloc_rejects_oversize_bond():
    from syngular_gb300 import _lib as L

    rng = np.random.default_rng(1)
    X = chain(rng, 3, 2, 300)
    with pytest.raises(L.SyngularError, match="scratch limit"):
        both(X, X)
