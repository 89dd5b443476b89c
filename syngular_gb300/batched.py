"""Many independent MPO x MPS + TT-SVD round + overlap problems of uneven size.

Instances (their own N, d, chi, D) are dealt to S CUDA streams, longest first;
each stream runs its instances one after another inside one reusable
workspace, so device memory is S x (largest workspace of a stream) plus the
outputs.  Everything is enqueued through the C ABI with preallocated buffers
(no allocation, no host synchronisation), so the whole batch can be captured
once into a CUDA graph and replayed.

The autotuner times the candidate stream counts (by graph replay) for a shape
class (bucketed largest fused bond, mean length, count) and caches the choice
in a JSON file.
"""
from __future__ import annotations

import ctypes
import json
import math
import os
from typing import Dict, List, Optional, Sequence, Tuple

import torch

from . import _lib as L

TUNE_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")


class Instance:
    def __init__(self, W: Sequence[torch.Tensor], X: Sequence[torch.Tensor], chi: int):
        self.W = [L.as_device(w) for w in W]
        self.X = [L.as_device(x) for x in X]
        self.chi = int(chi)
        self.n = len(self.X)
        self.wsh = [int(v) for w in self.W for v in w.shape]
        self.xsh = [int(v) for x in self.X for v in x.shape]
        self.pshapes = [(x.shape[0] * w.shape[0], w.shape[2], x.shape[2] * w.shape[3])
                        for w, x in zip(self.W, self.X)]
        self.rmax = max(max(p[0], p[2]) for p in self.pshapes)


def _work_estimate(inst: "Instance") -> float:
    """Leading cost of one instance's rounding: per bond the product of the
    bond matrix's side (d chi) and the squared product bond (the Gram-step and
    bond-matrix products)."""
    tot = 0.0
    for p in inst.pshapes:
        r, d, r2 = p
        tot += float(r) * float(r) * float(d) * float(min(r2, inst.chi))
    return tot


class BatchedRound:
    def __init__(self, instances: List[Instance], precision: int = L.PREC_TF32X3, streams: int = 4,
                 budget_bytes: int = 160 << 30, spectra: bool = True):
        self.instances = instances
        self.precision = precision
        # without spectra the rounding returns only the rounded cores (the
        # BF16X6 form then finds kept subspaces by purification)
        self.spectra = bool(spectra)
        dev = L.device()
        # output shapes, spectra counts, workspace sizes
        self.ws_need = []
        for inst in instances:
            n = inst.n
            psh, _p = L.shape_array(inst.pshapes)
            out = (ctypes.c_int64 * (3 * n))()
            cnt = (ctypes.c_int64 * max(1, n - 1))()
            L.call("sgt_svd_round_shapes", n, psh, inst.chi, ctypes.cast(out, L._PI64), ctypes.cast(cnt, L._PI64))
            inst.out = [torch.empty((out[3 * k], out[3 * k + 1], out[3 * k + 2]), dtype=torch.float64, device=dev)
                        for k in range(n)]
            inst.counts = [cnt[k] for k in range(n - 1)]
            inst.spectra = torch.zeros(max(1, sum(inst.counts)), dtype=torch.float64, device=dev)
            inst.disc = torch.zeros(max(1, n - 1), dtype=torch.float64, device=dev)
            inst.status = torch.zeros(1, dtype=torch.int32, device=dev)
            inst.ovl = torch.zeros(2, dtype=torch.float64, device=dev)
            wsh, _w = L.i64_array(inst.wsh)
            xsh, _x = L.i64_array(inst.xsh)
            need = L.query("sgt_mpo_mps_round_workspace_size", n, wsh, xsh, inst.chi, precision)
            if need == 0:
                raise L.SyngularError("sgt_mpo_mps_round_workspace_size", 1,
                                      L.load().sgt_last_error().decode(errors="replace"))
            outsh, _o = L.shape_array([tuple(o.shape) for o in inst.out])
            ovl_need = L.query("sgt_overlap_workspace_size", n, xsh, outsh)
            inst.ws_need = max(need, ovl_need)
        # deal instances to streams, most work first, onto the least loaded
        # stream (longest-processing-time order); the work estimate is the
        # rounding's leading term, sum over bonds of (product bond)^2 x (d chi)
        S = max(1, int(streams))
        work = [_work_estimate(inst) for inst in instances]
        order = sorted(range(len(instances)), key=lambda i: -work[i])
        self.lanes: List[List[int]] = [[] for _ in range(S)]
        load = [0.0] * S
        for i in order:
            s = min(range(S), key=lambda j: load[j])
            self.lanes[s].append(i)
            load[s] += work[i]
        self.lanes = [lane for lane in self.lanes if lane]
        lane_ws = [max(instances[i].ws_need for i in lane) for lane in self.lanes]
        if sum(lane_ws) > budget_bytes:
            raise MemoryError("batched workspaces need %d bytes > budget %d; use fewer streams"
                              % (sum(lane_ws), budget_bytes))
        self.ws = [torch.empty(b, dtype=torch.uint8, device=dev) for b in lane_ws]
        self.streams = [torch.cuda.Stream() for _ in self.lanes]
        self.graph: Optional[torch.cuda.CUDAGraph] = None
        self.graphs: List[torch.cuda.CUDAGraph] = []
        # keep the ctypes argument arrays alive for graph replays
        self._keep = []
        self._args = [self._build_args(inst) for inst in instances]

    def _build_args(self, inst: Instance):
        n = inst.n
        wp, a1 = L.ptr_array(inst.W)
        xp, a2 = L.ptr_array(inst.X)
        op, a3 = L.ptr_array(inst.out)
        wsh, a4 = L.i64_array(inst.wsh)
        xsh, a5 = L.i64_array(inst.xsh)
        osh, a6 = L.shape_array([tuple(o.shape) for o in inst.out])
        self._keep += [a1, a2, a3, a4, a5, a6]
        return (n, wp, wsh, xp, xsh, op, osh)

    def launch(self, chunk=None):
        """Enqueue every instance on its stream (no synchronisation); with
        ``chunk = (j0, j1)`` only the instances at positions j0..j1-1 of every
        lane."""
        cur = torch.cuda.current_stream()
        for lane, ws, st in zip(self.lanes, self.ws, self.streams):
            st.wait_stream(cur)
            sp = L._c_vp(st.cuda_stream)
            for i in (lane if chunk is None else lane[chunk[0]:chunk[1]]):
                inst = self.instances[i]
                n, wp, wsh, xp, xsh, op, osh = self._args[i]
                L.call("sgt_mpo_mps_round", n, wp, wsh, xp, xsh, inst.chi, self.precision, op,
                       L.ptr(inst.spectra) if self.spectra else None, L.ptr(inst.disc), L.ptr(inst.status),
                       L.ptr(ws), ws.numel(), sp)
                L.call("sgt_overlap_sweep", n, xp, xsh, op, osh, L.ptr(inst.ovl), L.ptr(ws), ws.numel(), sp)
        for st in self.streams:
            cur.wait_stream(st)

    def capture(self, per_lane: int = 0):
        """Capture launch() into CUDA graphs (run launch() eagerly first so
        every one-time set-up inside the library has happened).  ``per_lane >
        0`` splits the batch into graphs of at most that many instances per
        lane, replayed back to back: a large batch of long chains holds
        millions of kernel nodes, more than one graph should."""
        self.launch()
        torch.cuda.synchronize()
        longest = max(len(l) for l in self.lanes)
        step = longest if per_lane <= 0 else per_lane
        graphs = []
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        for j0 in range(0, longest, step):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(side):
                with torch.cuda.graph(g, stream=side):
                    self.launch((j0, j0 + step))
            graphs.append(g)
        torch.cuda.current_stream().wait_stream(side)
        self.graphs = graphs
        self.graph = graphs[0]
        return graphs

    def replay(self):
        if self.graph is None:
            self.capture()
        for g in self.graphs:
            g.replay()

    def overlaps(self) -> List[float]:
        from .tensor._ops import decode_overlap

        return [decode_overlap(inst.ovl.cpu().tolist()) for inst in self.instances]

    def statuses(self) -> List[int]:
        return [int(inst.status.item()) for inst in self.instances]


def _vp_array(items):
    arr = (ctypes.c_void_p * len(items))(*items)
    return arr


class NativePlan:
    """Host side of the library's batched plan (sgt_batched_plan_create): the
    per-instance workspace sizes, the deal of instances onto stream lanes and
    the rounded core shapes.  Needs no GPU."""

    def __init__(self, shapes, precision: int = L.PREC_TF32X3, lanes: int = 4):
        # shapes: list of (wshape list (4 n), xshape list (3 n), chi)
        self.count = len(shapes)
        self.n = [len(x) // 3 for _, x, _ in shapes]
        self._keep = []
        narr = (ctypes.c_int * self.count)(*self.n)
        warrs = [L.i64_array(w)[1] for w, _, _ in shapes]
        xarrs = [L.i64_array(x)[1] for _, x, _ in shapes]
        self._keep += [narr, warrs, xarrs]
        wp = _vp_array([ctypes.cast(a, ctypes.c_void_p).value for a in warrs])
        xp = _vp_array([ctypes.cast(a, ctypes.c_void_p).value for a in xarrs])
        chis = (ctypes.c_int64 * self.count)(*[int(c) for _, _, c in shapes])
        self._keep += [wp, xp, chis]
        self.handle = ctypes.c_void_p()
        wsb = ctypes.c_size_t()
        L.call("sgt_batched_plan_create", self.count, narr, wp, xp, chis, int(precision), int(lanes),
               ctypes.byref(self.handle), ctypes.byref(wsb))
        self.ws_bytes = int(wsb.value)
        lib = L.load()
        self.lane = [int(lib.sgt_batched_plan_lane(self.handle, i)) for i in range(self.count)]
        self.out_shapes = []
        for i in range(self.count):
            o = (ctypes.c_int64 * (3 * self.n[i]))()
            L.call("sgt_batched_plan_out_shape", self.handle, i, o)
            self.out_shapes.append([tuple(o[3 * k:3 * k + 3]) for k in range(self.n[i])])

    def __del__(self):
        try:
            if getattr(self, "handle", None) is not None and self.handle.value:
                L.load().sgt_batched_plan_destroy(self.handle)
                self.handle = ctypes.c_void_p()
        except Exception:
            pass


class NativeBatchedRound:
    """The batch run through sgt_batched_launch (one library call that forks the
    lanes off the current stream and joins them): same results as BatchedRound,
    graph-capturable."""

    def __init__(self, instances: List[Instance], precision: int = L.PREC_TF32X3, lanes: int = 4,
                 spectra: bool = True):
        self.instances = instances
        self.spectra = bool(spectra)
        self.plan = NativePlan([(i.wsh, i.xsh, i.chi) for i in instances], precision, lanes)
        dev = L.device()
        self._keep = []
        W, X, O, SP, DI, ST, OV = [], [], [], [], [], [], []
        for inst, oshape in zip(instances, self.plan.out_shapes):
            inst.out = [torch.empty(s, dtype=torch.float64, device=dev) for s in oshape]
            inst.spectra = torch.zeros(max(1, sum(self._counts(inst))), dtype=torch.float64, device=dev)
            inst.disc = torch.zeros(max(1, inst.n - 1), dtype=torch.float64, device=dev)
            inst.status = torch.zeros(1, dtype=torch.int32, device=dev)
            inst.ovl = torch.zeros(2, dtype=torch.float64, device=dev)
            for lst, ts in ((W, inst.W), (X, inst.X), (O, inst.out)):
                _p, arr = L.ptr_array(ts)
                self._keep.append(arr)
                lst.append(ctypes.cast(arr, ctypes.c_void_p).value)
            SP.append(inst.spectra.data_ptr())
            DI.append(inst.disc.data_ptr())
            ST.append(inst.status.data_ptr())
            OV.append(inst.ovl.data_ptr())
        self._arrs = [_vp_array(v) for v in (W, X, O, SP, DI, ST, OV)]
        self.ws = torch.empty(max(1, self.plan.ws_bytes), dtype=torch.uint8, device=dev)
        self.graph: Optional[torch.cuda.CUDAGraph] = None

    @staticmethod
    def _counts(inst):
        psh, _p = L.shape_array(inst.pshapes)
        out = (ctypes.c_int64 * (3 * inst.n))()
        cnt = (ctypes.c_int64 * max(1, inst.n - 1))()
        L.call("sgt_svd_round_shapes", inst.n, psh, inst.chi, ctypes.cast(out, L._PI64), ctypes.cast(cnt, L._PI64))
        return [cnt[k] for k in range(inst.n - 1)]

    def launch(self):
        W, X, O, SP, DI, ST, OV = self._arrs
        L.call("sgt_batched_launch", self.plan.handle, W, X, O, SP if self.spectra else None, DI, ST, OV,
               L.ptr(self.ws), self.ws.numel(), L.stream_ptr())

    def capture(self):
        self.launch()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            with torch.cuda.graph(g, stream=side):
                self.launch()
        torch.cuda.current_stream().wait_stream(side)
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def overlaps(self) -> List[float]:
        from .tensor._ops import decode_overlap

        return [decode_overlap(inst.ovl.cpu().tolist()) for inst in self.instances]

    def statuses(self) -> List[int]:
        return [int(inst.status.item()) for inst in self.instances]


def shape_class(instances: List[Instance]) -> str:
    r = max(i.rmax for i in instances)
    nb = int(round(sum(i.n for i in instances) / max(1, len(instances))))
    return "r%d_n%d_c%d" % (2 ** math.ceil(math.log2(max(r, 1))), 8 * ((nb + 7) // 8), len(instances))


def _time_config(instances, precision, streams, budget_bytes, reps, spectra, per_lane):
    b = BatchedRound(instances, precision, streams=streams, budget_bytes=budget_bytes, spectra=spectra)
    b.capture(per_lane=per_lane)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        b.replay()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    del b
    torch.cuda.empty_cache()
    return ms


def autotune(instances: List[Instance], precision: int = L.PREC_TF32X3,
             candidates: Sequence[int] = (2, 4, 8, 16), budget_bytes: int = 160 << 30,
             reps: int = 2, spectra: bool = True, per_lane: int = 0,
             splits: Sequence[Tuple[int, int]] = ()) -> Dict:
    """Pick, by timed graph replays of this batch, the stream-lane count and
    (when ``splits`` lists candidates) the sliced GEMM's split-K shape: the
    CTA count a product with few output tiles is spread over and the least K
    extent (in 32-wide tiles) each split keeps, i.e. the K depth of the tiles
    of the bond-sized products (the library's SGT_TUNE_SLICED_SPLIT_CTAS and
    SGT_TUNE_SLICED_SPLIT_MIN_KTILES).  Lanes are tuned first at the library's
    current split shape, then the split shape at the best lane count.  The
    choice is cached in TUNE_FILE per shape class and applied to the library
    before returning."""
    key = "%s_p%d%s%s" % (shape_class(instances), precision, "" if spectra else "_nospec",
                          "_k" + "-".join("%dx%d" % (int(a), int(b)) for a, b in splits) if splits else "")
    cache = {}
    if os.path.exists(TUNE_FILE):
        try:
            with open(TUNE_FILE) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    lib = L.load()

    def apply(split):
        L.call("sgt_set_tuning", L.TUNE_SLICED_SPLIT_CTAS, int(split[0]))
        L.call("sgt_set_tuning", L.TUNE_SLICED_SPLIT_MIN_KTILES, int(split[1]))

    if key in cache:
        res = cache[key]
        if res.get("split"):
            apply(res["split"])
        return res
    base = (int(lib.sgt_get_tuning(L.TUNE_SLICED_SPLIT_CTAS)), int(lib.sgt_get_tuning(L.TUNE_SLICED_SPLIT_MIN_KTILES)))
    best = None
    trials = {}
    for s in candidates:
        try:
            ms = _time_config(instances, precision, s, budget_bytes, reps, spectra, per_lane)
        except MemoryError:
            continue
        trials["lanes=%d" % s] = ms
        if best is None or ms < best[1]:
            best = (s, ms)
    lanes = best[0] if best else candidates[0]
    chosen = base
    try:
        for sp in splits:
            sp = (int(sp[0]), int(sp[1]))
            if sp == base and best is not None:
                continue
            apply(sp)
            try:
                ms = _time_config(instances, precision, lanes, budget_bytes, reps, spectra, per_lane)
            except MemoryError:
                continue
            trials["lanes=%d,split=%dx%d" % (lanes, sp[0], sp[1])] = ms
            if best is None or ms < best[1]:
                best = (lanes, ms)
                chosen = sp
    finally:  # a failed trial leaves the library at the best shape so far, not at the trial's
        apply(chosen)
    res = {"streams": lanes, "split": list(chosen), "ms": best[1] if best else None, "trials": trials}
    cache[key] = res
    try:
        with open(TUNE_FILE, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
    except OSError:
        pass
    return res


def shard(indices: Sequence[int], rank: int, world: int) -> List[int]:
    """Instances of this rank when a batch is spread over `world` GPUs (no
    data exchange: every instance is independent)."""
    return [i for k, i in enumerate(indices) if k % world == rank]
