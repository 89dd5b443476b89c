"""Continuous-batching serving loop: admission by HBM budget, overlapping jobs on
separate streams, each result equal alone and in the mix."""
import time

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


def server_with_sessions(rng, count, budget=8 << 30, slots=4):
    from syngular_gb300.serving import RoundServer

    srv = RoundServer(budget_bytes=budget, slots=slots)
    for i in range(count):
        n = int(rng.integers(4, 9))
        d = int(rng.choice([2, 4]))
        chi = int(rng.integers(4, 13))
        D = int(rng.choice([2, 4]))
        srv.add_session("s%d" % i, mps=O.random_mps_cores(rng, n, d, chi), mpo=O.random_mpo_cores(rng, n, d, D))
    return srv


def jobs_for(rng, count, precision=0):
    from syngular_gb300.serving import Job

    jobs = []
    for i in range(count):
        kind = ["round", "add_round", "overlap"][i % 3]
        s = "s%d" % i
        jobs.append(Job(kind=kind, session=s, chi=int(rng.integers(3, 9)), precision=precision, other=s, job_id=i))
    return jobs


def summary(job):
    if job.kind == "overlap":
        from syngular_gb300.tensor._ops import decode_overlap

        return decode_overlap(job.result.cpu().tolist())
    cores = job.result[0]
    from syngular_gb300.tensor import _ops

    return _ops.overlap(cores, cores)


@pytest.mark.parametrize("precision", [0, 5])
def test_mix_equals_alone(precision):
    """Each job's result alone (one slot) equals its result in the mix (four
    slots, overlapping on the device): FP64 and the BF16X6 precision form
    (rounding without spectra, the serving default).  Every kernel of both
    forms sums in a fixed order, so the tolerance is FP64 rounding."""
    rng = np.random.default_rng(3)
    srv = server_with_sessions(rng, 12).start()
    jobs = jobs_for(rng, 12, precision)
    for j in jobs:
        srv.submit(j)
    for j in jobs:
        assert j.done.wait(120), "job did not finish"
        assert j.error is None, j.error
    mixed = [summary(j) for j in jobs]
    srv.stop()
    # alone: one slot, one job at a time
    rng = np.random.default_rng(3)
    solo = server_with_sessions(rng, 12, slots=1).start()
    jobs2 = jobs_for(rng, 12, precision)
    alone = []
    for j in jobs2:
        solo.submit(j)
        assert j.done.wait(120)
        alone.append(summary(j))
    solo.stop()
    np.testing.assert_allclose(mixed, alone, rtol=1e-12, atol=0)


def test_budget_admission_and_rejection():
    from syngular_gb300.serving import Job, latency_stats

    rng = np.random.default_rng(9)
    srv = server_with_sessions(rng, 4, slots=4)
    big = Job(kind="round", session="s0", chi=8, precision=0)
    ok = Job(kind="overlap", session="s1", other="s1")
    f_ok, f_big = srv.footprint(ok), srv.footprint(big)
    assert 0 < f_ok < f_big
    srv.budget = (f_ok + f_big) // 2  # admits the overlap, not the round
    srv.start()
    srv.submit(big)
    assert big.done.wait(60)
    srv.submit(ok)
    assert ok.done.wait(60)
    srv.stop()
    assert ok.error is None and big.error is not None and "budget" in big.error
    st = latency_stats([ok])
    assert st["count"] == 1 and st["p50_ms"] >= 0


def test_bad_job_does_not_stop_the_loop():
    """A job naming an unknown session is rejected on its own; the scheduler
    thread keeps serving the jobs that follow it."""
    from syngular_gb300.serving import Job

    rng = np.random.default_rng(11)
    srv = server_with_sessions(rng, 2, slots=2).start()
    bad = Job(kind="round", session="no-such-session", chi=4, precision=0)
    good = Job(kind="overlap", session="s0", other="s0")
    srv.submit(bad)
    srv.submit(good)
    assert bad.done.wait(60) and good.done.wait(60)
    srv.stop()
    assert bad.error is not None and "KeyError" in bad.error
    assert good.error is None and good.result is not None


@pytest.mark.parametrize("precision", [0, 5])
def test_repeated_jobs_replay_graphs(precision):
    """A job kind seen before on the same sessions replays its captured CUDA
    graph; the replayed results equal the first (eager) run bit for bit, and
    a graph still in use by one job is not replayed by a second in flight."""
    from syngular_gb300.serving import Job

    rng = np.random.default_rng(17)
    srv = server_with_sessions(rng, 2, slots=4).start()
    results = {}
    for kind in ("round", "add_round", "overlap"):
        runs = []
        for rep in range(3):
            j = Job(kind=kind, session="s0", other="s0", chi=5, precision=precision, job_id=rep)
            srv.submit(j)
            assert j.done.wait(120) and j.error is None, j.error
            runs.append(summary(j))
        results[kind] = runs
    # two at once: one replays, the other runs eagerly
    burst = [Job(kind="round", session="s0", other="s0", chi=5, precision=precision, job_id=10 + i) for i in range(2)]
    for j in burst:
        srv.submit(j)
    for j in burst:
        assert j.done.wait(120) and j.error is None
    srv.stop()
    assert srv.replayed >= 6
    for kind, runs in results.items():
        np.testing.assert_allclose(runs, [runs[0]] * 3, rtol=1e-12, atol=0, err_msg=kind)
    np.testing.assert_allclose([summary(j) for j in burst], [results["round"][0]] * 2, rtol=1e-12, atol=0)


def test_small_job_passes_a_job_waiting_for_memory():
    """Backfill: with room for one round job, a second round job waits for
    memory while a later overlap job that fits is admitted at once."""
    from syngular_gb300.serving import Job

    rng = np.random.default_rng(23)
    srv = server_with_sessions(rng, 3, slots=4)
    a = Job(kind="round", session="s0", chi=8, precision=0, job_id=0)
    b = Job(kind="round", session="s0", chi=8, precision=0, job_id=1)
    small = Job(kind="overlap", session="s1", other="s1", job_id=2)
    f_round, f_small = srv.footprint(a), srv.footprint(small)
    srv.budget = f_round + 2 * f_small  # one round job at a time, with room for the overlap
    for j in (a, b, small):
        srv.submit(j)
    srv.start()
    for j in (a, b, small):
        assert j.done.wait(120) and j.error is None, j.error
    srv.stop()
    assert small.start < b.start
