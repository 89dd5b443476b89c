"""tcgen05 TF32 / 3xTF32 GEMM against an FP64 reference of the same product.
Tolerances: TF32 (10-bit mantissa) 5e-3 relative Frobenius error; 3xTF32 1e-6
(split products exact to ~2^-22; the kernel drains the tensor-core accumulator
every 32 of K into round-to-nearest FP32 registers, so long K does not
accumulate the tensor core's truncation)."""
import numpy as np
import pytest
import torch

from tests.conftest import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def run(M, N, K, passes, ldpad=0, beta=0.0, seed=0):
    from syngular_gb300 import _lib as L

    rng = np.random.default_rng(seed)
    lda = ldb = K + ldpad
    A = rng.standard_normal((M, lda)).astype(np.float32)
    B = rng.standard_normal((N, ldb)).astype(np.float32)
    C0 = rng.standard_normal((M, N)).astype(np.float32)
    ref = 0.75 * A[:, :K].astype(np.float64) @ B[:, :K].astype(np.float64).T + beta * C0.astype(np.float64)
    dev = torch.device("cuda")
    Ad, Bd, Cd = (torch.from_numpy(x).to(dev) for x in (A, B, C0))
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    if passes == 3:
        Ah, Al, Bh, Bl = (torch.empty_like(t) for t in (Ad, Ad, Bd, Bd))
        L.call("sgt_split_tf32", L.ptr(Ad), L.ptr(Ah), L.ptr(Al), Ad.numel(), L.stream_ptr())
        L.call("sgt_split_tf32", L.ptr(Bd), L.ptr(Bh), L.ptr(Bl), Bd.numel(), L.stream_ptr())
    else:
        Ah, Al, Bh, Bl = Ad, None, Bd, None
    L.call("sgt_tc_gemm_f32", passes, M, N, K, 0.75, L.ptr(Ah), L.ptr(Al) if Al is not None else None, lda,
           L.ptr(Bh), L.ptr(Bl) if Bl is not None else None, ldb, beta, L.ptr(Cd), N, L.ptr(err), L.stream_ptr())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return rel(Cd.cpu().numpy(), ref)


@pytest.mark.parametrize("M,N,K,pad", [(128, 128, 32, 0), (256, 384, 512, 0), (200, 300, 100, 0),
                                       (1000, 136, 77, 3), (4096, 512, 4096, 0)])
def test_tf32(M, N, K, pad):
    assert run(M, N, K, 1, pad) < 5e-3


@pytest.mark.parametrize("M,N,K", [(128, 128, 32), (300, 260, 1000), (2048, 1024, 2048), (512, 512, 8192)])
def test_3xtf32(M, N, K):
    assert run(M, N, K, 3, beta=0.5) < 1e-6


def run_ws(M, N, K, passes, beta=0.5, seed=1, ws_scale=1.0):
    """Through sgt_tc_gemm_f32_ws (split K when the output has few tiles);
    returns (relative error, result)."""
    from syngular_gb300 import _lib as L

    rng = np.random.default_rng(seed)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    C0 = rng.standard_normal((M, N)).astype(np.float32)
    ref = 0.75 * A.astype(np.float64) @ B.astype(np.float64).T + beta * C0.astype(np.float64)
    dev = torch.device("cuda")
    Ad, Bd, Cd = (torch.from_numpy(x).to(dev) for x in (A, B, C0))
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    Ah, Al, Bh, Bl = (torch.empty_like(t) for t in (Ad, Ad, Bd, Bd))
    L.call("sgt_split_tf32", L.ptr(Ad), L.ptr(Ah), L.ptr(Al), Ad.numel(), L.stream_ptr())
    L.call("sgt_split_tf32", L.ptr(Bd), L.ptr(Bh), L.ptr(Bl), Bd.numel(), L.stream_ptr())
    nbytes = int(L.query("sgt_tc_gemm_f32_workspace_size", M, N, K) * ws_scale) // 16 * 16
    ws = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=dev)
    L.call("sgt_tc_gemm_f32_ws", passes, M, N, K, 0.75, L.ptr(Ah), L.ptr(Al), K, L.ptr(Bh), L.ptr(Bl), K, beta,
           L.ptr(Cd), N, L.ptr(err), L.ptr(ws), nbytes, L.stream_ptr())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    out = Cd.cpu().numpy()
    return rel(out, ref), out


@pytest.mark.parametrize("M,N,K,splits", [(512, 512, 4096, 8), (256, 4096, 4096, 3), (128, 256, 1000, 4),
                                          (4096, 4096, 256, 1)])
def test_3xtf32_split_k(M, N, K, splits):
    """Split K (the Z = Y^T (G Y) and projection shapes of the Gram form, a
    ragged last K-tile, and a shape with enough tiles to need no split):
    3xTF32 accuracy, bitwise repeatable, and a workspace of half the size
    (fewer splits) gives the same accuracy."""
    from syngular_gb300 import _lib as L

    nbytes = L.query("sgt_tc_gemm_f32_workspace_size", M, N, K)
    assert nbytes == (splits * M * N * 4 if splits > 1 else 0)
    e1, c1 = run_ws(M, N, K, 3)
    e2, c2 = run_ws(M, N, K, 3)
    assert e1 < 1e-6
    np.testing.assert_array_equal(c1, c2)
    e3, _ = run_ws(M, N, K, 3, ws_scale=0.5)
    assert e3 < 1e-6
