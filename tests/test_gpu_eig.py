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


# per method: (1 - min cos of the top-n/2 subspace angles, |Vt Vt^T - I| max).  Method 2
# takes its vectors by normalising rows that are orthogonal to the Jacobi tolerance
# (8 eps sqrt(n)), so both figures are looser.
TOL = {0: (1e-5, 5e-5), 1: (1e-5, 5e-5), 2: (3e-4, 3e-4), 3: (1e-5, 5e-5)}


CASES = [(n, m) for m in (0, 1, 2, 3) for n in (128, 256, 512)] + [(n, m) for m in (1, 2, 3) for n in (96, 300)]


@pytest.mark.parametrize("n,method", CASES)
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
    assert np.min(s) > 1 - TOL[method][0]
    # orthogonality of the computed vectors (FP32)
    np.testing.assert_allclose(Vt @ Vt.T, np.eye(n), atol=TOL[method][1])


@pytest.mark.parametrize("method", [1, 2, 3])
def test_sym_eig_graded_rank_deficient(method):
    """Eigenvalues decaying to 1e-11 of the largest (below FP32 resolution):
    the resolvable part must come out right and every vector stays unit-norm
    (Cholesky pivots under the floor are raised to it, never zero rows)."""
    n = 256
    rng = np.random.default_rng(7)
    lam_true = np.exp(-np.arange(n) / (n / 25.0))
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    Z = (Q * lam_true) @ Q.T
    Z = (Z + Z.T) / 2
    Vt, lam, st = run(Z, method)
    assert st > 0
    assert np.all(np.isfinite(Vt)) and np.all(np.isfinite(lam))
    big = lam_true > 1e-3
    np.testing.assert_allclose(lam[big], lam_true[big], atol=2e-5)
    np.testing.assert_allclose(np.linalg.norm(Vt, axis=1), 1.0, atol=TOL[method][1] * 4)
    # the top eigenvectors (well separated, lam > 1e-2) agree up to sign
    top = lam_true > 1e-2
    cos = np.abs(np.sum(Vt[top] * Q[:, top].T, axis=1))
    assert np.min(cos) > 1 - 1e-4
