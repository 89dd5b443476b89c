"""DMRG environment blocks on the device (reference: variational/dmrg.py).

``DMRG.left_blocks`` / ``DMRG.right_blocks`` return the lists that the
reference's ``DMRG.__left_blocks`` (dmrg.py:89-112) and
``DMRG.__right_blocks`` (dmrg.py:65-87) build: ``n`` entries, the left block
of site k, ``[a', b', c']``, for k = 0..n-3 and the right block ``[a, b, c]``
for k = n-1 down to 2, ``None`` elsewhere.  ``DMRG.effective_site`` is the
contraction each sweep step hands to the optimiser (dmrg.py:143-165 and
202-224): the two-site effective operator applied to the merged tensor of
sites k and k+1.  Blocks are float64 CUDA tensors; each list is one C-ABI call
(``sgt_env_blocks``), each effective site one call (``sgt_env_two_site``).
"""
from __future__ import annotations

from typing import List, Optional

import torch

from .. import _lib as L
from ..tensor import _ops


def _w_shapes(operator):
    flat = []
    for w in operator.sites:
        flat += [int(v) for v in w.shape]
    return L.i64_array(flat)


def _blocks(operator, state, side: int, bra=None) -> List[Optional[torch.Tensor]]:
    W = [L.as_device(w) for w in operator.sites]
    Y = [L.as_device(x) for x in state.sites]
    X = Y if bra is None else [L.as_device(x) for x in bra.sites]
    n = len(W)
    if len(X) != n or len(Y) != n:
        raise ValueError("operator and state have different lengths")
    count = max(0, n - 2)
    out: List[Optional[torch.Tensor]] = [None] * n
    if count == 0:
        return out
    for j in range(count):
        k = j if side == 0 else n - 1 - j
        if side == 0:
            shape = (X[k].shape[-1], W[k].shape[-1], Y[k].shape[-1])
        else:
            shape = (X[k].shape[0], W[k].shape[0], Y[k].shape[0])
        out[k] = _ops.empty(shape)
    ws_, _w = _w_shapes(operator)
    xs, _x = L.shape_array([_ops.shape3(c) for c in X])
    ys, _y = L.shape_array([_ops.shape3(c) for c in Y])
    need = L.query("sgt_env_blocks_workspace_size", n, ws_, xs, ys, side, count)
    if need == 0:
        raise L.SyngularError("sgt_env_blocks_workspace_size", L.SGT_ERR_INVALID,
                              L.load().sgt_last_error().decode(errors="replace"))
    ws = L.workspace(need)
    dummy = out[0] if out[0] is not None else out[n - 1]
    bp, _b = L.ptr_array([o if o is not None else dummy for o in out])
    wp, _wp = L.ptr_array(W)
    xp, _xp = L.ptr_array(X)
    yp, _yp = L.ptr_array(Y)
    L.call("sgt_env_blocks", n, wp, ws_, xp, xs, yp, ys, side, count, bp, L.ptr(ws), ws.numel(), L.stream_ptr())
    return out


class DMRG:
    """The reference's DMRG environment contractions (no optimiser)."""

    @staticmethod
    def left_blocks(operator, state, bra=None) -> List[Optional[torch.Tensor]]:
        """Left blocks (dmrg.py:89-112): entry k = <state|operator|state> over
        sites 0..k with legs (bra bond, operator bond, ket bond), k <= n-3.
        ``bra`` (default: ``state``) replaces the state on the operator's
        output side."""
        return _blocks(operator, state, 0, bra)

    @staticmethod
    def right_blocks(operator, state, bra=None) -> List[Optional[torch.Tensor]]:
        """Right blocks (dmrg.py:65-87): entry k = the contraction over sites
        k..n-1, legs (bra bond, operator bond, ket bond), k >= 2."""
        return _blocks(operator, state, 1, bra)

    @staticmethod
    def effective_site(operator, state, left_blocks, right_blocks, index: int) -> torch.Tensor:
        """The two-site tensor of sweep step ``index`` (dmrg.py:128-165):
        left block ``index-1`` (none at the first step), the merged sites
        ``index``/``index+1`` of ``state``, the operator's sites
        ``index``/``index+1`` and right block ``index+2`` (none at the last
        step), contracted to (bra bond, out_k, out_{k+1}, bra bond)."""
        n = operator.sites_number
        k = int(index)
        if not 0 <= k <= n - 2:
            raise Exception("site index out of range (between 0 & n-2)")
        x0, x1 = L.as_device(state.sites[k]), L.as_device(state.sites[k + 1])
        w1, w2 = L.as_device(operator.sites[k]), L.as_device(operator.sites[k + 1])
        a, p0, r = x0.shape
        _r, p1, c4 = x1.shape
        merge = _ops.empty((a, p0, p1, c4))
        # merged two-site tensor M[c, i1, i2, c4] = X_k[c, i1, m] X_{k+1}[m, i2, c4]
        L.call("sgt_gemm_f64", 0, 0, a * p0, p1 * c4, r, 1.0, L.ptr(x0), r, 0, L.ptr(x1), p1 * c4, 0, 0.0,
               L.ptr(merge), p1 * c4, 0, 1, L.stream_ptr())
        Lb = None if k == 0 else left_blocks[k - 1]
        Rb = None if k == n - 2 else right_blocks[k + 2]
        if k != 0 and Lb is None:
            raise Exception("missing left block %d" % (k - 1))
        if k != n - 2 and Rb is None:
            raise Exception("missing right block %d" % (k + 2))
        ls = L.i64_array(list(Lb.shape)) if Lb is not None else (None, None)
        rs = L.i64_array(list(Rb.shape)) if Rb is not None else (None, None)
        ms, _m = L.i64_array(list(merge.shape))
        w1s, _1 = L.i64_array(list(w1.shape))
        w2s, _2 = L.i64_array(list(w2.shape))
        A = Lb.shape[0] if Lb is not None else 1
        A4 = Rb.shape[0] if Rb is not None else 1
        out = _ops.empty((A, w1.shape[2], w2.shape[2], A4))
        need = L.query("sgt_env_two_site_workspace_size", ls[0], ms, w1s, w2s, rs[0])
        if need == 0:
            raise L.SyngularError("sgt_env_two_site_workspace_size", L.SGT_ERR_INVALID,
                                  L.load().sgt_last_error().decode(errors="replace"))
        ws = L.workspace(need)
        L.call("sgt_env_two_site", L.ptr(Lb) if Lb is not None else None, ls[0], L.ptr(merge), ms, L.ptr(w1), w1s,
               L.ptr(w2), w2s, L.ptr(Rb) if Rb is not None else None, rs[0], L.ptr(out), L.ptr(ws), ws.numel(),
               L.stream_ptr())
        return out
