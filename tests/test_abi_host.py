"""CPU-side checks of the C-ABI library and the host logic (no GPU calls)."""
import os
import re

import numpy as np
import pytest

from tests.conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g

    g.build()
    from syngular_gb300 import _lib

    return _lib.load()


def header_symbols():
    with open(os.path.join(ROOT, "include", "syngular_gb300.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"SGT_API\s+[\w\s\*]+?\b(sgt_\w+)\s*\(", text)))


def test_header_lists_entry_points():
    syms = header_symbols()
    assert "sgt_svd_round" in syms and "sgt_overlap_sweep" in syms
    assert len(syms) >= 20


def test_library_exports_every_header_symbol(lib):
    for name in header_symbols():
        assert hasattr(lib, name), name


def test_ctypes_signatures_cover_header(lib):
    from syngular_gb300 import _lib

    missing = [s for s in header_symbols() if s not in _lib.SIGNATURES]
    assert not missing, missing


def test_version_and_error_string(lib):
    assert lib.sgt_version() >= 1
    assert isinstance(lib.sgt_last_error(), bytes)


def test_workspace_queries_and_shape_checks(lib):
    """Size queries run on the host only; they validate shapes like the calls."""
    from syngular_gb300 import _lib as L

    sh, _k = L.shape_array([(1, 2, 4), (4, 2, 4), (4, 2, 1)])
    assert L.query("sgt_overlap_workspace_size", 3, sh, sh) > 0
    assert L.query("sgt_qr_truncate_workspace_size", 3, sh, 2) > 0
    # l*p < dim at the first site: the reference's reshape fails, so does the query
    assert L.query("sgt_qr_truncate_workspace_size", 3, sh, 4) == 0
    assert b"reshape" in lib.sgt_last_error()
    bad, _b = L.shape_array([(1, 2, 4), (3, 2, 1)])
    assert L.query("sgt_overlap_workspace_size", 2, bad, bad) == 0
    assert b"bond mismatch" in lib.sgt_last_error()
    # split-K slices of the tensor-core GEMM: only for outputs with few tiles
    assert L.query("sgt_tc_gemm_f32_workspace_size", 512, 512, 4096) == 8 * 512 * 512 * 4
    assert L.query("sgt_tc_gemm_f32_workspace_size", 256, 4096, 4096) == 3 * 256 * 4096 * 4
    assert L.query("sgt_tc_gemm_f32_workspace_size", 4096, 4096, 4096) == 0
    assert L.query("sgt_tc_gemm_f32_workspace_size", 128, 128, 64) == 0
    # the reserved bf16 precision codes are rejected by the size queries already
    for prec in (L.PREC_BF16, L.PREC_BF16X3):
        assert L.query("sgt_svd_round_workspace_size", 3, sh, 2, prec) == 0
        assert b"precision" in lib.sgt_last_error()
    # event profiles: stopping with nothing recorded needs no device
    import ctypes

    for name in ("sgt_tc_profile", "sgt_eig_profile"):
        ms, fl, n = ctypes.c_double(1.0), ctypes.c_double(1.0), ctypes.c_longlong(1)
        assert getattr(lib, name)(0, ctypes.byref(ms), ctypes.byref(fl), ctypes.byref(n)) == 0
        assert (ms.value, fl.value, n.value) == (0.0, 0.0, 0)


def test_svd_round_shapes_match_oracle(lib):
    from oracle import tt_fp64 as O
    from syngular_gb300 import _lib as L
    import ctypes

    rng = np.random.default_rng(3)
    for n, d, chi, D, cut in [(6, 2, 8, 3, 5), (5, 3, 4, 2, 7), (8, 2, 16, 4, 6)]:
        X = O.random_mps_cores(rng, n, d, chi)
        W = O.random_mpo_cores(rng, n, d, D)
        P = O.mpo_mps_product(W, X)
        Z, spec, _ = O.tt_svd_round(P, cut)
        sh, _k = L.shape_array([c.shape for c in P])
        out = (ctypes.c_int64 * (3 * n))()
        cnt = (ctypes.c_int64 * (n - 1))()
        assert lib.sgt_svd_round_shapes(n, sh, cut, ctypes.cast(out, L._PI64), ctypes.cast(cnt, L._PI64)) == 0
        got = [(out[3 * k], out[3 * k + 1], out[3 * k + 2]) for k in range(n)]
        assert got == [c.shape for c in Z]
        assert [cnt[k] for k in range(n - 1)] == [len(s) for s in spec]


def test_no_cpu_fallback_without_gpu():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from syngular_gb300.tensor import MatrixProductState

    with pytest.raises(RuntimeError, match="CUDA"):
        MatrixProductState.zeros((2, 2), (2,))


def test_batched_plan_host_only():
    """sgt_batched_plan_create is host-only: workspace sizes, the most-work-first
    deal onto lanes and the rounded shapes, without a GPU."""
    import numpy as np

    from syngular_gb300.batched import NativePlan

    rng = np.random.default_rng(5)
    shapes, chis = [], []
    for _ in range(9):
        n = int(rng.integers(3, 8))
        d = int(rng.choice([2, 3]))
        chi = int(rng.integers(2, 9))
        D = int(rng.choice([1, 2, 3]))
        xb = [1] + [chi] * (n - 1) + [1]
        wb = [1] + [D] * (n - 1) + [1]
        xs = [v for k in range(n) for v in (xb[k], d, xb[k + 1])]
        ws = [v for k in range(n) for v in (wb[k], d, d, wb[k + 1])]
        shapes.append((ws, xs, chi))
    plan = NativePlan(shapes, precision=0, lanes=4)
    assert plan.ws_bytes > 0 and plan.ws_bytes % 256 == 0
    assert sorted(set(plan.lane)) == [0, 1, 2, 3]
    for (ws, xs, chi), oshape in zip(shapes, plan.out_shapes):
        n = len(xs) // 3
        p = [(xs[3 * k] * ws[4 * k], ws[4 * k + 2], xs[3 * k + 2] * ws[4 * k + 3]) for k in range(n)]
        assert len(oshape) == n and oshape[0][0] == 1 and oshape[-1][2] == 1
        for k in range(n - 1):
            assert oshape[k][2] == oshape[k + 1][0] and oshape[k][2] <= chi


def test_bench_dominant_kernel_object(lib):
    """The bench line's dominant_kernel object from the eigensolver's event
    profile: well-formed figures, and an error string instead of a failure."""
    import bench

    assert bench._eig_profile(True) is True
    stats = bench._eig_profile(False)
    assert stats == (0.0, 0.0, 0)
    assert bench._eig_summary(stats, 600.0) == {"kernel": "gjacobi_kernel<1>", "launches": 0}
    flops = 14 * 0.5 * 512 * 511 * 12 * 512 * 55
    d = bench._eig_summary((437.5, flops, 55), 600.0)
    assert d["launches"] == 55 and abs(d["ms_per_launch"] - 437.5 / 55) < 1e-12
    assert 0 < d["frac"] < d["frac_of_cluster_sms"] < 1
    assert abs(d["share_of_step"] - 437.5 / 600.0) < 1e-12
    assert bench._eig_summary("RuntimeError: x", 600.0)["error"] == "RuntimeError: x"


def test_bench_cpu_port_machinery():
    """The CPU arm's machinery on a 3-site chain of the benchmark's core shapes:
    a whole sweep of the numpy FP64 port in a fresh interpreter with a fixed
    BLAS thread count, and the CPU / BLAS description printed beside it."""
    import bench

    r = bench.cpu_full_sweep(1, sites=3)
    assert r["seconds"] > 0 and r["overlap"] == r["overlap"]
    info = bench.cpu_info()
    assert info["cores"] >= 1 and info["numpy"]


def test_sliced_split_tuning_host_only(lib):
    """The sliced GEMM's split-K target is a process-wide host setting: range
    checked, readable, and the workspace query follows it (more splits, more
    partial sums) without any GPU call."""
    from syngular_gb300 import _lib as L

    before = lib.sgt_get_tuning(L.TUNE_SLICED_SPLIT_CTAS)
    assert before == 148
    try:
        assert lib.sgt_set_tuning(L.TUNE_SLICED_SPLIT_CTAS, 0) == L.SGT_ERR_INVALID
        assert lib.sgt_set_tuning(L.TUNE_SLICED_SPLIT_CTAS, 609) == L.SGT_ERR_INVALID
        assert lib.sgt_set_tuning(99, 1) == L.SGT_ERR_INVALID
        assert lib.sgt_get_tuning(99) == -1
        assert lib.sgt_get_tuning(L.TUNE_SLICED_SPLIT_MIN_KTILES) == 8
        assert lib.sgt_get_tuning(L.TUNE_PCHOL_BLOCKED) == 0
        assert lib.sgt_set_tuning(L.TUNE_PCHOL_BLOCKED, 2) == L.SGT_ERR_INVALID
        assert lib.sgt_set_tuning(L.TUNE_PCHOL_BLOCKED, 1) == L.SGT_OK
        assert lib.sgt_get_tuning(L.TUNE_PCHOL_BLOCKED) == 1
        assert lib.sgt_set_tuning(L.TUNE_PCHOL_BLOCKED, 0) == L.SGT_OK
        assert lib.sgt_get_tuning(L.TUNE_PURIFY_CLEANUP) == 0
        assert lib.sgt_set_tuning(L.TUNE_PURIFY_CLEANUP, 5) == L.SGT_ERR_INVALID
        assert lib.sgt_set_tuning(L.TUNE_PURIFY_CLEANUP, 1) == L.SGT_OK
        assert lib.sgt_get_tuning(L.TUNE_PURIFY_CLEANUP) == 1
        assert lib.sgt_set_tuning(L.TUNE_PURIFY_CLEANUP, 0) == L.SGT_OK
        assert lib.sgt_get_tuning(L.TUNE_PURIFY_VECTOR_STEP) == 1
        assert lib.sgt_set_tuning(L.TUNE_PURIFY_VECTOR_STEP, 2) == L.SGT_ERR_INVALID
        assert lib.sgt_set_tuning(L.TUNE_PURIFY_VECTOR_STEP, 0) == L.SGT_OK
        assert lib.sgt_get_tuning(L.TUNE_PURIFY_VECTOR_STEP) == 0
        assert lib.sgt_set_tuning(L.TUNE_PURIFY_VECTOR_STEP, 1) == L.SGT_OK
        assert lib.sgt_set_tuning(L.TUNE_SLICED_SPLIT_MIN_KTILES, 1) == L.SGT_ERR_INVALID
        sizes = []
        for t, kt in ((24, 8), (148, 8), (592, 8), (592, 2)):
            assert lib.sgt_set_tuning(L.TUNE_SLICED_SPLIT_CTAS, t) == L.SGT_OK
            assert lib.sgt_set_tuning(L.TUNE_SLICED_SPLIT_MIN_KTILES, kt) == L.SGT_OK
            assert lib.sgt_get_tuning(L.TUNE_SLICED_SPLIT_CTAS) == t
            sizes.append(lib.sgt_gemm_f64_sliced_workspace_size(512, 512, 512))
        # 512^3: one split at target 24, two while each keeps 8 K-tiles, eight at 2
        assert sizes[0] < sizes[1] == sizes[2] < sizes[3]
    finally:
        lib.sgt_set_tuning(L.TUNE_SLICED_SPLIT_CTAS, before)
        lib.sgt_set_tuning(L.TUNE_SLICED_SPLIT_MIN_KTILES, 8)


def test_env_blocks_size_queries_host_only(lib):
    """The DMRG environment size queries check the chain on the host: a
    consistent chain gives a size on both sides, a bond or leg mismatch 0."""
    from oracle import tt_fp64 as O
    from syngular_gb300 import _lib as L

    rng = np.random.default_rng(1)
    X = O.random_mps_cores(rng, 6, 2, 16)
    W = O.random_mpo_cores(rng, 6, 2, 4)
    ws, _w = L.i64_array([v for w in W for v in w.shape])
    xs, _x = L.shape_array([c.shape for c in X])
    for side in (0, 1):
        assert lib.sgt_env_blocks_workspace_size(6, ws, xs, xs, side, 4) > 0
    bad = [c.shape for c in X]
    bad[3] = (bad[3][0], bad[3][1], bad[3][2] + 1)
    bs, _b = L.shape_array(bad)
    assert lib.sgt_env_blocks_workspace_size(6, ws, bs, xs, 0, 4) == 0
    assert b"bond mismatch" in lib.sgt_last_error()
    W3 = O.random_mpo_cores(rng, 6, 3, 4)
    w3, _w3 = L.i64_array([v for w in W3 for v in w.shape])
    assert lib.sgt_env_blocks_workspace_size(6, w3, xs, xs, 0, 4) == 0
    ls, _l = L.i64_array([1, 1, 1])
    m, _m = L.i64_array([1, 2, 2, 16])
    w1, _1 = L.i64_array(list(W[0].shape))
    w2, _2 = L.i64_array(list(W[1].shape))
    rs, _r = L.i64_array([16, 4, 16])
    assert lib.sgt_env_two_site_workspace_size(ls, m, w1, w2, rs) > 0
    assert lib.sgt_env_two_site_workspace_size(None, m, w1, w2, rs) > 0
    assert lib.sgt_env_two_site_workspace_size(ls, m, w1, w2, None) == 0   # right block needed (b3 = 4)


@pytest.mark.parametrize("n,d,chi,D,cut", [(6, 2, 4, 3, 5), (5, 3, 2, 2, 64), (7, 2, 8, 4, 12)])
def test_zipup_shapes_match_oracle_host_only(lib, n, d, chi, D, cut):
    """The zip-up's output shapes (a host query) are the oracle's core shapes;
    the workspace query sizes the chain, and a bond mismatch is refused with
    the library's message."""
    import ctypes

    from oracle import tt_fp64 as O
    from syngular_gb300 import _lib as L

    rng = np.random.default_rng(n * 10 + cut)
    X, W = O.random_mps_cores(rng, n, d, chi), O.random_mpo_cores(rng, n, d, D)
    Zr, _disc = O.zipup(W, X, cut)
    ws, _w = L.i64_array([v for w in W for v in w.shape])
    xs, _x = L.shape_array([c.shape for c in X])
    out = (ctypes.c_int64 * (3 * n))()
    assert lib.sgt_mpo_mps_zipup_shapes(n, ws, xs, cut, ctypes.cast(out, L._PI64)) == L.SGT_OK
    assert [tuple(out[3 * k:3 * k + 3]) for k in range(n)] == [z.shape for z in Zr]
    assert lib.sgt_mpo_mps_zipup_workspace_size(n, ws, xs, cut) > 0
    bad = [c.shape for c in X]
    bad[2] = (bad[2][0] + 1, bad[2][1], bad[2][2])
    bs, _b = L.shape_array(bad)
    assert lib.sgt_mpo_mps_zipup_shapes(n, ws, bs, cut, ctypes.cast(out, L._PI64)) == L.SGT_ERR_INVALID
    assert b"bond mismatch" in lib.sgt_last_error()
    assert lib.sgt_mpo_mps_zipup_workspace_size(n, ws, xs, 0) == 0


def test_library_resolves_every_symbol_at_load(lib):
    """Every symbol the library uses is defined (bound at load time, not at
    the first call): a declared-but-missing helper would otherwise surface only
    when its entry point runs on a GPU host."""
    import ctypes

    from syngular_gb300 import _lib

    ctypes.CDLL(_lib.LIB_PATH, mode=os.RTLD_NOW | os.RTLD_LOCAL)
