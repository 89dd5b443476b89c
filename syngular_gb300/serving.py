"""Continuous-batching request loop for contract / round / overlap jobs.

Jobs arrive on a queue; a scheduler thread admits them while the device
memory they need (workspace + outputs, from the library's size queries) fits
an HBM budget and a stream slot is free, launches them on their own CUDA
stream, and retires them as their completion events fire -- so requests that
arrive while others run join as soon as memory and slots free up, and their
kernels overlap on the device.  Session cores stay resident on the device
between jobs (a job references them by session id).  A job whose own
footprint exceeds the whole budget is rejected at submission.

Job kinds (the three of the serving workload):
  * "round"   : raw W @ X followed by TT-SVD rounding to chi (sgt_mpo_mps_round)
  * "add_round": X + Y (bond concatenation) followed by TT-SVD rounding to chi
  * "overlap" : <X|Y>
Every job's result is the same whether it runs alone or in the mix: each job
has its own workspace and stream, and the kernels read only its own data.
"""
from __future__ import annotations

import ctypes
import queue
import threading
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import torch

from . import _lib as L
from .tensor import _ops


@dataclass
class Job:
    kind: str
    session: str
    chi: int = 0
    precision: int = L.PREC_BF16X6
    spectra: bool = False                # rounding jobs: also return every bond's singular values
    other: Optional[str] = None          # second operand's session (add_round / overlap)
    arrival: float = 0.0                 # seconds (time.perf_counter clock)
    job_id: int = 0
    # filled in by the server
    start: float = 0.0
    end: float = 0.0
    result: object = None
    error: Optional[str] = None
    done: threading.Event = field(default_factory=threading.Event)

    @property
    def latency(self) -> float:
        return self.end - self.arrival


class RoundServer:
    """Admission by HBM budget, one CUDA stream per in-flight job."""

    def __init__(self, budget_bytes: int = 120 << 30, slots: int = 8, graphs: bool = True,
                 graph_job_bytes: int = 2 << 30, graph_budget_bytes: int = 24 << 30):
        self.budget = int(budget_bytes)
        self.slots = int(slots)
        # captured CUDA graphs, one per (kind, sessions, chi, precision): a job
        # whose graph exists and is idle replays it (one launch instead of its
        # thousands of kernel launches from this thread) and copies the graph's
        # outputs out; the graphs' memory counts against the budget for good
        self.use_graphs = bool(graphs)
        self.graph_job_bytes = int(graph_job_bytes)
        self.graph_budget = int(graph_budget_bytes)
        self.graphs: Dict[tuple, "_Graph"] = {}
        self.graph_bytes = 0
        self.replayed = 0
        # admission: pending jobs looked at per pass, and how long a job that
        # waits for memory lets later jobs pass it
        self.scan = 256
        self.max_bypass_s = 2.0
        self.sessions: Dict[str, dict] = {}
        self.inbox: "queue.Queue[Job]" = queue.Queue()
        self.streams = [torch.cuda.Stream() for _ in range(self.slots)]
        self.free_streams = list(range(self.slots))
        self.used = 0
        self.inflight: List[tuple] = []
        self.pending: List[Job] = []
        self.completed: List[Job] = []
        self.rejected: List[Job] = []
        self._stop = threading.Event()
        self._cancel = threading.Event()
        self._thread = threading.Thread(target=self._loop, daemon=True)

    # ---------------------------------------------------------------- sessions
    def add_session(self, name: str, mps=None, mpo=None):
        """Keep cores resident on the device: mps = list of (l, p, r), mpo =
        list of (l, in, out, r) float64 tensors (host or device)."""
        self.sessions[name] = {
            "mps": [L.as_device(c) for c in mps] if mps is not None else None,
            "mpo": [L.as_device(c) for c in mpo] if mpo is not None else None,
        }

    # ----------------------------------------------------------------- control
    def start(self):
        self._thread.start()
        return self

    def stop(self, cancel_pending: bool = False):
        """Stop the loop once the work it holds is done; with
        ``cancel_pending`` the jobs not yet admitted end at once with an error
        (in-flight jobs still finish)."""
        if cancel_pending:
            self._cancel.set()
        self._stop.set()
        self._thread.join()

    def submit(self, job: Job) -> Job:
        if not job.arrival:
            job.arrival = time.perf_counter()
        self.inbox.put(job)
        return job

    # ------------------------------------------------------------- accounting
    def footprint(self, job: Job) -> int:
        s = self.sessions[job.session]
        if job.kind == "round":
            W, X = s["mpo"], s["mps"]
            n = len(X)
            wsh, _a = L.i64_array([int(v) for w in W for v in w.shape])
            xsh, _b = L.shape_array([tuple(x.shape) for x in X])
            ws = L.query("sgt_mpo_mps_round_workspace_size", n, wsh, xsh, job.chi, job.precision)
            # outputs as the library sizes them: the rounded cores carry the
            # operator's out leg; plus the spectra, discarded weights and status
            psh, _p = L.shape_array([(X[k].shape[0] * W[k].shape[0], W[k].shape[2], X[k].shape[2] * W[k].shape[3])
                                     for k in range(n)])
            out_arr = (ctypes.c_int64 * (3 * n))()
            cnt_arr = (ctypes.c_int64 * max(1, n - 1))()
            L.call("sgt_svd_round_shapes", n, psh, job.chi, ctypes.cast(out_arr, L._PI64),
                   ctypes.cast(cnt_arr, L._PI64))
            out = 8 * sum(out_arr[3 * k] * out_arr[3 * k + 1] * out_arr[3 * k + 2] for k in range(n))
            out += 8 * (sum(cnt_arr[k] for k in range(n - 1)) + max(1, n - 1)) + 4
            return ws + out if ws else -1
        if job.kind == "add_round":
            X, Y = s["mps"], self.sessions[job.other]["mps"]
            cat = sum(8 * (x.shape[0] + y.shape[0]) * x.shape[1] * (x.shape[2] + y.shape[2]) for x, y in zip(X, Y))
            shp = [(x.shape[0] + (y.shape[0] if k else 0), x.shape[1],
                    x.shape[2] + (y.shape[2] if k < len(X) - 1 else 0)) for k, (x, y) in enumerate(zip(X, Y))]
            shp[0] = (1, shp[0][1], shp[0][2])
            sh, _c = L.shape_array(shp)
            ws = L.query("sgt_svd_round_workspace_size", len(X), sh, job.chi, job.precision)
            return cat + ws if ws else -1
        X, Y = s["mps"], self.sessions[job.other]["mps"]
        xs, _d = L.shape_array([tuple(x.shape) for x in X])
        ys, _e = L.shape_array([tuple(y.shape) for y in Y])
        return L.query("sgt_overlap_workspace_size", len(X), xs, ys) + 16

    # -------------------------------------------------------------- execution
    def _run(self, job: Job):
        """Enqueue the job's work on the current stream; returns its outputs."""
        s = self.sessions[job.session]
        if job.kind == "round":
            res = _ops.mpo_mps_round(s["mpo"], s["mps"], job.chi, job.precision, spectra=job.spectra)
            return (res[0], res[1], res[2], res[3], res[4])
        if job.kind == "add_round":
            S = _ops.concat(s["mps"], self.sessions[job.other]["mps"])
            return _ops.svd_round(S, job.chi, job.precision, spectra=job.spectra)
        return _ops.overlap_device(s["mps"], self.sessions[job.other]["mps"])

    @staticmethod
    def _graph_key(job: Job):
        return (job.kind, job.session, job.other, job.chi, job.precision, job.spectra)

    def _capture(self, job: Job, key) -> None:
        """Capture the job's work into a CUDA graph (no GPU execution; the
        library's one-time set-up already ran in the job's eager launch)."""
        before = torch.cuda.memory_reserved()
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        try:
            with torch.cuda.stream(side):
                with torch.cuda.graph(g, stream=side, capture_error_mode="thread_local"):
                    outputs = self._run(job)
        except Exception:  # a job that cannot be captured keeps running eagerly
            self.graphs[key] = None
            return
        nbytes = max(0, torch.cuda.memory_reserved() - before)
        self.graphs[key] = _Graph(g, outputs, nbytes)
        self.graph_bytes += nbytes
        self.used += nbytes

    def _launch(self, job: Job, stream_idx: int):
        st = self.streams[stream_idx]
        st.wait_stream(torch.cuda.current_stream())
        key = self._graph_key(job) if self.use_graphs else None
        gr = self.graphs.get(key) if key is not None else None
        with torch.cuda.stream(st):
            if gr is not None and not gr.busy:
                gr.graph.replay()
                out = _clone(gr.outputs)
                gr.busy = True
                self.replayed += 1
            else:
                gr = None
                out = self._run(job)
            ev = torch.cuda.Event()
            ev.record(st)
        if (key is not None and key not in self.graphs and job._need <= self.graph_job_bytes
                and self.graph_bytes + job._need <= self.graph_budget
                and self.used + job._need <= self.budget):
            self._capture(job, key)
        return out, ev, gr

    def _evict_idle_graphs(self, need: int) -> bool:
        """Graph memory is held for good, so a job that fits the budget could
        wait forever behind it: when the graphs alone leave too little room
        for ``need`` bytes, free idle graphs, oldest first, until they do not
        (a job that only waits for in-flight work evicts nothing).  An evicted
        key is not captured again.  Returns whether the job fits now."""
        for key in list(self.graphs):
            if self.graph_bytes + need <= self.budget:
                break
            gr = self.graphs[key]
            if gr is None or gr.busy:
                continue
            self.graphs[key] = None
            self.graph_bytes -= gr.nbytes
            self.used -= gr.nbytes
        return self.used + need <= self.budget

    def _loop(self):
        while not self._stop.is_set() or self.pending or self.inflight or not self.inbox.empty():
            # take arrivals
            try:
                while True:
                    j = self.inbox.get_nowait()
                    try:
                        need = self.footprint(j)
                    except Exception as e:  # unknown session, shape the size query rejects, ...
                        j.error = "rejected: %s: %s" % (type(e).__name__, e)
                        j.end = time.perf_counter()
                        self.rejected.append(j)
                        j.done.set()
                        continue
                    if need < 0 or need > self.budget:
                        j.error = "rejected: footprint %d bytes exceeds the HBM budget" % need
                        j.end = time.perf_counter()
                        self.rejected.append(j)
                        j.done.set()
                        continue
                    j._need = need
                    self.pending.append(j)
            except queue.Empty:
                pass
            # retire finished jobs
            still = []
            for job, ev, out, sidx, gr in self.inflight:
                if ev.query():
                    job.end = time.perf_counter()
                    job.result = out
                    self.used -= job._need
                    self.free_streams.append(sidx)
                    if gr is not None:
                        gr.busy = False
                    self.completed.append(job)
                    job.done.set()
                else:
                    still.append((job, ev, out, sidx, gr))
            self.inflight = still
            if self._cancel.is_set() and self.pending:
                now = time.perf_counter()
                for j in self.pending:
                    j.error = "cancelled: server stopped"
                    j.end = now
                    self.rejected.append(j)
                    j.done.set()
                self.pending = []
            # admit in arrival order while memory and slots allow; a job that
            # does not fit the memory left lets later, smaller jobs pass
            # (backfill) for at most max_bypass_s, then admission waits for it
            admitted = []
            now = time.perf_counter()
            for j in self.pending[: self.scan]:
                if not self.free_streams:
                    break
                if self.used + j._need > self.budget and not self._evict_idle_graphs(j._need):
                    if getattr(j, "_blocked", None) is None:
                        j._blocked = now
                    if now - j._blocked < self.max_bypass_s:
                        continue
                    break
                sidx = self.free_streams.pop()
                self.used += j._need
                j.start = time.perf_counter()
                try:
                    out, ev, gr = self._launch(j, sidx)
                    self.inflight.append((j, ev, out, sidx, gr))
                except Exception as e:  # surface the error on the job, keep serving
                    j.error = str(e)
                    j.end = time.perf_counter()
                    self.used -= j._need
                    self.free_streams.append(sidx)
                    self.rejected.append(j)
                    j.done.set()
                admitted.append(j)
            if admitted:
                gone = set(id(j) for j in admitted)
                self.pending = [j for j in self.pending if id(j) not in gone]
            if not admitted and not self.inflight:
                time.sleep(0.0002)
            else:
                time.sleep(0)


@dataclass
class _Graph:
    graph: torch.cuda.CUDAGraph
    outputs: object                      # the captured outputs (tensors the replays overwrite)
    nbytes: int                          # device memory the graph holds
    busy: bool = False                   # a replay's outputs are still being copied out


def _clone(out):
    """Fresh copies of a job's outputs (tensors cloned on the current stream)."""
    if isinstance(out, torch.Tensor):
        return out.clone()
    if isinstance(out, (list, tuple)):
        return type(out)(_clone(o) for o in out)
    return out


def latency_stats(jobs: List[Job]):
    lat = sorted(j.latency for j in jobs)
    if not lat:
        return {"p50_ms": None, "p99_ms": None, "count": 0}

    def pct(p):
        k = min(len(lat) - 1, max(0, int(round(p / 100.0 * (len(lat) - 1)))))
        return lat[k] * 1e3

    return {"p50_ms": pct(50), "p99_ms": pct(99), "count": len(lat), "mean_ms": 1e3 * sum(lat) / len(lat)}
