"""FP32 symmetric eigensolvers of the Gram form against numpy FP64.

Z = A^T A with controlled spectra.  Checked: eigenvalues (relative to the
largest), and the angle between the computed and exact subspaces spanned by
the top-k eigenvectors (k below a spectral gap)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def run(Z, method):
    from syngular_gb300 import _lib as L

    n = Z.shape[0]
    Zd = torch.from_numpy(Z.astype(np.float32)).cuda()
    Vt = torch.empty((n, n), dtype=torch.float32, device="cuda")
    lam = torch.empty(n, dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    ws = L.workspace(L.query("sgt_sym_eig_f32_workspace_size", n))
    L.call("sgt_sym_eig_f32", L.ptr(Zd), n, L.ptr(Vt), L.ptr(lam), L.ptr(st), method, L.ptr(ws), ws.numel(),
           L.stream_ptr())
    torch.cuda.synchronize()
    return Vt.cpu().numpy().astype(np.float64), lam.cpu().numpy().astype(np.float64), int(st.item())


@pytest.mark.parametrize("n", [128, 256, 512])
@pytest.mark.parametrize("method", [0, 1])
def test_sym_eig(n, method):
    rng = np.random.default_rng(n + method)
    A = rng.standard_normal((4 * n, n)) / np.sqrt(n)
    Z = A.T @ A
    w, V = np.linalg.eigh(Z)
    w, V = w[::-1], V[:, ::-1]
    Vt, lam, st = run(Z, method)
    assert st > 0
    np.testing.assert_allclose(lam, w, atol=1e-5 * w[0])
    k = n // 2
    # subspace angle: |V_k^T Vhat_k| singular values -> cos of principal angles
    s = np.linalg.svd(V[:, :k].T @ Vt[:k].T, compute_uv=False)
    assert np.min(s) > 1 - 1e-5
    # orthogonality of the computed vectors (FP32)
    np.testing.assert_allclose(Vt @ Vt.T, np.eye(n), atol=5e-5)
