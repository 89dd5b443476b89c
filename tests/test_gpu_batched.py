"""Batched uneven instances (the batched workload at small scale): eager launch,
CUDA-graph capture and replay; every instance against the FP64 oracle."""
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


def make(rng, count):
    from syngular_gb300.batched import Instance

    insts, ref = [], []
    for _ in range(count):
        n = int(rng.integers(4, 10))
        d = int(rng.choice([2, 3, 4]))
        chi = int(rng.integers(4, 17))
        D = int(rng.choice([2, 4]))
        X = O.random_mps_cores(rng, n, d, chi)
        W = O.random_mpo_cores(rng, n, d, D)
        insts.append(Instance(W, X, chi))
        Zr, spec, disc = O.tt_svd_round(O.mpo_mps_product(W, X), chi)
        ref.append((O.overlap(X, Zr), np.sqrt(O.overlap(X, X) * O.overlap(Zr, Zr))))
    return insts, ref


@pytest.mark.parametrize("prec,tol,spectra,per_lane", [(0, 1e-12, True, 0), (4, 1e-6, True, 0),
                                                      (5, 1e-9, False, 2)])
def test_batched_eager_and_graph(prec, tol, spectra, per_lane):
    """Eager launch against the FP64 oracle, then graph replay against the
    eager results; the BF16X6 case runs without spectra (purification) and
    captures the batch as several graphs of two instances per lane."""
    from syngular_gb300.batched import BatchedRound

    rng = np.random.default_rng(77)
    insts, ref = make(rng, 12)
    b = BatchedRound(insts, precision=prec, streams=4, spectra=spectra)
    b.launch()
    torch.cuda.synchronize()
    eager = b.overlaps()
    assert all(s >= 0 for s in b.statuses())
    for v, (r, scale) in zip(eager, ref):
        assert abs(v - r) <= tol * scale
    b.capture(per_lane=per_lane)
    assert len(b.graphs) == (1 if per_lane == 0 else -(-max(len(l) for l in b.lanes) // per_lane))
    for inst in insts:
        inst.ovl.zero_()
    b.replay()
    torch.cuda.synchronize()
    replayed = b.overlaps()
    np.testing.assert_allclose(replayed, eager, rtol=1e-12, atol=0)


def test_autotune_caches_choice(tmp_path, monkeypatch):
    import syngular_gb300.batched as B

    monkeypatch.setattr(B, "TUNE_FILE", str(tmp_path / "tune.json"))
    rng = np.random.default_rng(5)
    insts, _ = make(rng, 6)
    r1 = B.autotune(insts, precision=0, candidates=(1, 2), reps=1)
    assert r1["streams"] in (1, 2) and set(r1["trials"]) <= {"lanes=1", "lanes=2"}
    r2 = B.autotune(insts, precision=0, candidates=(1, 2), reps=1)
    assert r2 == r1


def test_autotune_split_depth(tmp_path, monkeypatch):
    """BF16X6 batch: the tuner also times the sliced GEMM's split-K target and
    leaves the library set to its choice."""
    import syngular_gb300.batched as B
    from syngular_gb300 import _lib as L

    monkeypatch.setattr(B, "TUNE_FILE", str(tmp_path / "tune.json"))
    rng = np.random.default_rng(6)
    insts, _ = make(rng, 6)
    lib = L.load()
    before = (lib.sgt_get_tuning(L.TUNE_SLICED_SPLIT_CTAS), lib.sgt_get_tuning(L.TUNE_SLICED_SPLIT_MIN_KTILES))
    try:
        r = B.autotune(insts, precision=L.PREC_BF16X6, candidates=(2,), reps=1, spectra=False, per_lane=2,
                       splits=((74, 8), (296, 4)))
        assert tuple(r["split"]) in (before, (74, 8), (296, 4))
        assert (lib.sgt_get_tuning(L.TUNE_SLICED_SPLIT_CTAS),
                lib.sgt_get_tuning(L.TUNE_SLICED_SPLIT_MIN_KTILES)) == tuple(r["split"])
        assert "lanes=2,split=74x8" in r["trials"] and "lanes=2,split=296x4" in r["trials"]
    finally:
        L.call("sgt_set_tuning", L.TUNE_SLICED_SPLIT_CTAS, before[0])
        L.call("sgt_set_tuning", L.TUNE_SLICED_SPLIT_MIN_KTILES, before[1])


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (4, 1e-6)])
def test_native_batched_launch(prec, tol):
    """sgt_batched_launch (one library call, lanes forked off the current
    stream) gives every instance the result of its own sgt_mpo_mps_round +
    sgt_overlap_sweep, eagerly and from a captured graph."""
    from syngular_gb300.batched import NativeBatchedRound
    from syngular_gb300.tensor import _ops

    rng = np.random.default_rng(31 + prec)
    insts, ref = make(rng, 7)
    b = NativeBatchedRound(insts, precision=prec, lanes=3)
    b.launch()
    torch.cuda.synchronize()
    first = b.overlaps()
    assert all(s >= 0 for s in b.statuses())
    for inst, got, (ov, nrm) in zip(insts, first, ref):
        assert abs(got - ov) <= tol * nrm
        Z, spec, counts, disc, st = _ops.mpo_mps_round(inst.W, inst.X, inst.chi, prec)
        alone = _ops.overlap(inst.X, Z)
        assert abs(got - alone) <= 1e-12 * nrm
    for inst in insts:
        inst.ovl.zero_()
    b.replay()
    torch.cuda.synchronize()
    assert b.overlaps() == first
