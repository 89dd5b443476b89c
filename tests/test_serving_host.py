"""The serving loop's admission logic on the host: budget rejection, backfill
past a job that waits for memory, eviction of idle captured graphs that would
otherwise keep a job out for good, error isolation and cancellation.  The
device work is replaced by events the test fires; no GPU is used."""
import threading
import time

import pytest

from syngular_gb300.serving import Job, RoundServer, _Graph


class FakeEvent:
    def __init__(self):
        self.fired = threading.Event()

    def query(self):
        return self.fired.is_set()


class HostServer(RoundServer):
    """RoundServer whose jobs' footprints come from a table (by session) and
    whose launches complete when the test fires their events."""

    def __init__(self, budget, slots, needs):
        super().__init__(budget_bytes=budget, slots=0, graphs=False)
        self.slots = slots
        self.streams = [None] * slots
        self.free_streams = list(range(slots))
        self.needs = dict(needs)
        self.events = {}
        self.order = []

    def footprint(self, job):
        return self.needs[job.session]  # KeyError for an unknown session

    def _launch(self, job, stream_idx):
        ev = FakeEvent()
        self.events[job.job_id] = ev
        self.order.append(job.job_id)
        return ("out", job.job_id), ev, None


def wait_for(cond, timeout=5.0):
    t0 = time.perf_counter()
    while not cond():
        if time.perf_counter() - t0 > timeout:
            return False
        time.sleep(0.001)
    return True


def test_budget_rejection_and_unknown_session():
    srv = HostServer(100, 2, {"big": 101, "ok": 10}).start()
    big, bad, ok = Job("round", "big", job_id=0), Job("round", "nope", job_id=1), Job("overlap", "ok", job_id=2)
    for j in (big, bad, ok):
        srv.submit(j)
    assert big.done.wait(5) and bad.done.wait(5)
    assert "budget" in big.error and "KeyError" in bad.error
    assert wait_for(lambda: 2 in srv.events)
    srv.events[2].fired.set()
    assert ok.done.wait(5) and ok.error is None and ok.result == ("out", 2)
    srv.stop()


def test_backfill_then_head_of_line():
    """B waits for memory; C, later and smaller, passes it; once A retires B
    runs.  After max_bypass_s a waiting job stops later jobs from passing."""
    srv = HostServer(100, 4, {"a": 60, "b": 60, "c": 30, "d": 10})
    srv.max_bypass_s = 0.2
    a, b, c = Job("round", "a", job_id=0), Job("round", "b", job_id=1), Job("round", "c", job_id=2)
    for j in (a, b, c):
        srv.submit(j)
    srv.start()
    assert wait_for(lambda: 0 in srv.events and 2 in srv.events)
    assert 1 not in srv.events  # b waits for memory, c passed it
    time.sleep(0.3)  # b has now waited longer than max_bypass_s
    d = srv.submit(Job("round", "d", job_id=3))
    time.sleep(0.1)
    assert 3 not in srv.events  # d fits (10 <= 100 - 90) but may no longer pass b
    srv.events[0].fired.set()  # a retires: b fits, then d
    assert wait_for(lambda: 1 in srv.events and 3 in srv.events)
    assert srv.order == [0, 2, 1, 3]
    for k in (1, 2, 3):
        srv.events[k].fired.set()
    for j in (a, b, c, d):
        assert j.done.wait(5) and j.error is None
    srv.stop()
    assert srv.used == 0


def test_idle_graphs_are_evicted_for_a_job_they_block():
    """Captured graphs hold 80 of a 100-byte budget; a job of 50 fits the
    budget but not beside them, so idle graphs are freed (oldest first, only
    as many as needed) and the job runs; a busy graph is kept until its job
    retires."""
    srv = HostServer(100, 2, {"j": 50})
    srv.graphs = {"g0": _Graph(None, None, 30), "g1": _Graph(None, None, 30, busy=True), "g2": _Graph(None, None, 20)}
    srv.graph_bytes = srv.used = 80
    j = srv.submit(Job("round", "j", job_id=0))
    srv.start()
    time.sleep(0.2)
    # freeing g0 (the oldest idle graph) leaves 50 + 50 <= 100: g1 (busy) and g2 stay
    assert wait_for(lambda: 0 in srv.events)
    assert srv.graphs["g0"] is None and srv.graphs["g1"] is not None and srv.graphs["g2"] is not None
    assert srv.graph_bytes == 50
    srv.events[0].fired.set()
    assert j.done.wait(5) and j.error is None
    srv.stop()
    assert srv.used == 50


def test_busy_graph_blocks_until_released():
    srv = HostServer(100, 2, {"j": 50})
    g = _Graph(None, None, 80, busy=True)
    srv.graphs = {"g": g}
    srv.graph_bytes = srv.used = 80
    j = srv.submit(Job("round", "j", job_id=0))
    srv.start()
    time.sleep(0.2)
    assert 0 not in srv.events
    g.busy = False  # its replay's job retired
    assert wait_for(lambda: 0 in srv.events)
    assert srv.graphs["g"] is None
    srv.events[0].fired.set()
    assert j.done.wait(5)
    srv.stop()


def test_stop_with_cancel_ends_pending_jobs():
    srv = HostServer(100, 1, {"x": 10})
    first = srv.submit(Job("round", "x", job_id=0))
    rest = [srv.submit(Job("round", "x", job_id=k)) for k in (1, 2)]
    srv.start()
    assert wait_for(lambda: 0 in srv.events)
    t = threading.Thread(target=srv.stop, kwargs={"cancel_pending": True})
    t.start()
    for j in rest:
        assert j.done.wait(5) and j.error.startswith("cancelled")
    srv.events[0].fired.set()
    t.join(5)
    assert not t.is_alive() and first.done.is_set() and first.error is None


@pytest.mark.parametrize("slots", [1, 3])
def test_every_job_completes_once(slots):
    srv = HostServer(1000, slots, {"s": 100})
    jobs = [srv.submit(Job("overlap", "s", job_id=k)) for k in range(40)]
    srv.start()

    def fire_all():
        while not all(j.done.is_set() for j in jobs):
            for ev in list(srv.events.values()):
                ev.fired.set()
            time.sleep(0.001)

    f = threading.Thread(target=fire_all)
    f.start()
    f.join(10)
    srv.stop()
    assert sorted(srv.order) == list(range(40)) and len(srv.completed) == 40
    assert srv.used == 0 and sorted(srv.free_streams) == list(range(slots))
