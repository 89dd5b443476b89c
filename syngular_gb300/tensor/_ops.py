"""Chain-level operations on lists of device cores, each one C-ABI call.

A core is a contiguous ``torch.float64`` CUDA tensor of rank >= 3 whose first
and last axes are the bonds; the middle axes form the physical leg (an MPO core
``(l, in, out, r)`` is handled as ``(l, in*out, r)`` wherever the reference
reshapes it that way).  Every function here enqueues work on the current CUDA
stream; only the ones returning Python scalars or host arrays synchronise.
"""
from __future__ import annotations

import ctypes
import math
from typing import List, Sequence, Tuple

import numpy as np
import torch

from .. import _lib as L

Cores = List[torch.Tensor]


def shape3(t: torch.Tensor) -> Tuple[int, int, int]:
    s = tuple(t.shape)
    return int(s[0]), int(np.prod(s[1:-1], dtype=np.int64)) if len(s) > 2 else 1, int(s[-1])


def _check(cores: Sequence[torch.Tensor]):
    for c in cores:
        if not (c.is_cuda and c.dtype == torch.float64 and c.is_contiguous()):
            raise TypeError("cores must be contiguous float64 CUDA tensors")


def empty(shape) -> torch.Tensor:
    return torch.empty(tuple(int(x) for x in shape), dtype=torch.float64, device=L.device())


# ---------------------------------------------------------------------------
# site contractions
# ---------------------------------------------------------------------------

def contract_mpo_mps(W: Cores, X: Cores) -> Cores:
    """Raw per-site ``W @ X`` (matrix_product_operator.py:183-191)."""
    _check(W)
    _check(X)
    out = []
    st = L.stream_ptr()
    for w, x in zip(W, X):
        a, p, a2 = x.shape
        b, i, o, b2 = w.shape
        if p != i:
            raise ValueError("physical leg mismatch: state %d vs operator input %d" % (p, i))
        P = empty((a * b, o, a2 * b2))
        L.call("sgt_site_contract_mpo_mps", L.ptr(x), a, p, a2, L.ptr(w), b, o, b2, L.ptr(P), st)
        out.append(P)
    return out


def contract_mpo_mpo(A: Cores, B: Cores) -> Cores:
    """Raw per-site ``A @ B`` (matrix_product_operator.py:279-288), output leg
    of size ``B.out``."""
    _check(A)
    _check(B)
    out = []
    st = L.stream_ptr()
    for a_, b_ in zip(A, B):
        b, i, m, b2 = a_.shape
        c, m2, o, c2 = b_.shape
        if m != m2:
            raise ValueError("contracted leg mismatch: %d vs %d" % (m, m2))
        P = empty((b * c, i, o, b2 * c2))
        L.call("sgt_site_contract_mpo_mpo", L.ptr(a_), b, i, m, b2, L.ptr(b_), c, o, c2, L.ptr(P), st)
        out.append(P)
    return out


# ---------------------------------------------------------------------------
# direct sum
# ---------------------------------------------------------------------------

def concat(A: Cores, B: Cores) -> Cores:
    """Bond concatenation of two chains in one launch
    (matrix_product_state.py:75-100, matrix_product_operator.py:84-108)."""
    _check(A)
    _check(B)
    n = len(A)
    outs = []
    for k, (a, b) in enumerate(zip(A, B)):
        if tuple(a.shape[1:-1]) != tuple(b.shape[1:-1]):
            raise ValueError("physical legs differ at site %d" % k)
        la, ra, lb, rb = a.shape[0], a.shape[-1], b.shape[0], b.shape[-1]
        if n == 1:
            ol, orr = la, ra
        elif k == 0:
            ol, orr = la, ra + rb
        elif k == n - 1:
            ol, orr = la + lb, ra
        else:
            ol, orr = la + lb, ra + rb
        outs.append(empty((ol,) + tuple(a.shape[1:-1]) + (orr,)))
    ap, _a = L.ptr_array(A)
    bp, _b = L.ptr_array(B)
    op, _o = L.ptr_array(outs)
    ash, _as = L.shape_array([shape3(a) for a in A])
    bsh, _bs = L.shape_array([shape3(b) for b in B])
    L.call("sgt_bond_concat_chain", n, ap, ash, bp, bsh, op, None, 0, L.stream_ptr())
    return outs


# ---------------------------------------------------------------------------
# overlap
# ---------------------------------------------------------------------------

def overlap_device(X: Cores, Y: Cores, precision: int = L.PREC_F64) -> torch.Tensor:
    """Transfer sweep; returns a device tensor ``(mantissa, exponent2)`` with
    ``<X|Y> = mantissa * 2**exponent2`` (no synchronisation).  ``precision``
    PREC_BF16X6 runs the contractions on the sliced tensor-core GEMM."""
    _check(X)
    _check(Y)
    n = len(X)
    if len(Y) != n:
        raise ValueError("chains have different lengths")
    xs, _x = L.shape_array([shape3(c) for c in X])
    ys, _y = L.shape_array([shape3(c) for c in Y])
    res = torch.empty(2, dtype=torch.float64, device=L.device())
    xp, _xp = L.ptr_array(X)
    yp, _yp = L.ptr_array(Y)
    if precision == L.PREC_F64:
        ws = L.workspace(L.query("sgt_overlap_workspace_size", n, xs, ys))
        L.call("sgt_overlap_sweep", n, xp, xs, yp, ys, L.ptr(res), L.ptr(ws), ws.numel(), L.stream_ptr())
        return res
    need = L.query("sgt_overlap_prec_workspace_size", n, xs, ys, precision)
    if need == 0:
        raise L.SyngularError("sgt_overlap_prec_workspace_size", L.SGT_ERR_INVALID,
                              L.load().sgt_last_error().decode(errors="replace"))
    ws = L.workspace(need)
    L.call("sgt_overlap_sweep_prec", n, xp, xs, yp, ys, precision, L.ptr(res), L.ptr(ws), ws.numel(),
           L.stream_ptr())
    return res


def decode_overlap(res) -> float:
    m, e = (float(v) for v in res)
    try:
        return math.ldexp(m, int(e))
    except OverflowError:
        return math.copysign(math.inf, m)


def overlap(X: Cores, Y: Cores, precision: int = L.PREC_F64) -> float:
    """``X | Y`` (matrix_product_state.py:116-127), as a Python float."""
    return decode_overlap(overlap_device(X, Y, precision).cpu().tolist())


# ---------------------------------------------------------------------------
# QR truncation (reference >>) and decompose
# ---------------------------------------------------------------------------

def qr_truncate(cores: Cores, dim: int) -> Cores:
    """Left QR-column truncation to ``dim`` (matrix_product_state.py:432-468).
    Raises ValueError where the reference's reshape fails (l*p < dim)."""
    _check(cores)
    n = len(cores)
    shp = [shape3(c) for c in cores]
    sh, _s = L.shape_array(shp)
    outs = []
    for k, c in enumerate(cores):
        l = c.shape[0] if k == 0 else dim
        r = c.shape[-1] if k == n - 1 else dim
        outs.append(empty((l,) + tuple(c.shape[1:-1]) + (r,)))
    nbytes = L.query("sgt_qr_truncate_workspace_size", n, sh, dim)
    if nbytes == 0:
        # size query fails exactly when the call would: surface its message
        lib = L.load()
        msg = lib.sgt_last_error().decode(errors="replace")
        if "reshape" in msg:
            raise ValueError(msg)
        raise L.SyngularError("sgt_qr_truncate_workspace_size", 1, msg)
    ws = L.workspace(nbytes)
    cp, _c = L.ptr_array(cores)
    op, _o = L.ptr_array(outs)
    L.call("sgt_qr_truncate_sweep", n, cp, sh, dim, op, L.ptr(ws), ws.numel(), L.stream_ptr())
    return outs


def decompose(tensor: torch.Tensor, phys: Sequence[int], bonds: Sequence[int], core_shapes,
              mode: int = 0) -> Cores:
    """Dense tensor -> cores (matrix_product_state.py:296-350)."""
    t = L.as_device(tensor)
    n = len(phys)
    ph, _p = L.i64_array(phys)
    bd, _b = L.i64_array(list(bonds) if len(bonds) else [1])
    nbytes = L.query("sgt_decompose_workspace_size", n, ph, bd, mode)
    if nbytes == 0:
        msg = L.load().sgt_last_error().decode(errors="replace")
        if "reshape" in msg:
            raise ValueError(msg)
        raise L.SyngularError("sgt_decompose_workspace_size", 1, msg)
    ws = L.workspace(nbytes)
    outs = [empty(s) for s in core_shapes]
    op, _o = L.ptr_array(outs)
    L.call("sgt_decompose", L.ptr(t), n, ph, bd, mode, op, L.ptr(ws), ws.numel(), L.stream_ptr())
    return outs


# ---------------------------------------------------------------------------
# orthonormalisation / orthogonality / normalisation
# ---------------------------------------------------------------------------

def _orth(cores: Cores, fn: str):
    _check(cores)
    n = len(cores)
    sh, _s = L.shape_array([shape3(c) for c in cores])
    ws = L.workspace(L.query("sgt_orthonormalize_workspace_size", n, sh))
    cp, _c = L.ptr_array(cores)
    L.call(fn, n, cp, sh, L.ptr(ws), ws.numel(), L.stream_ptr())


def left_orthonormalize(cores: Cores):
    """In place (matrix_product_state.py:554-566)."""
    _orth(cores, "sgt_left_orthonormalize")


def right_orthonormalize(cores: Cores):
    """In place (matrix_product_state.py:568-580)."""
    _orth(cores, "sgt_right_orthonormalize")


def orthogonality(core: torch.Tensor, side: int) -> torch.Tensor:
    """``L^T L`` (side 0) or ``R R^T`` (side 1) of one core, on the device."""
    _check([core])
    l, p, r = shape3(core)
    d = r if side == 0 else l
    out = empty((d, d))
    L.call("sgt_orthogonality", L.ptr(core), l, p, r, side, L.ptr(out), L.stream_ptr())
    return out


def normalize_(core: torch.Tensor) -> torch.Tensor:
    """Divide ``core`` by its Frobenius norm in place; returns the device norm."""
    _check([core])
    norm = torch.empty(1, dtype=torch.float64, device=L.device())
    L.call("sgt_normalize", L.ptr(core), core.numel(), L.ptr(norm), L.stream_ptr())
    return norm


# ---------------------------------------------------------------------------
# TT-SVD rounding
# ---------------------------------------------------------------------------

def svd_round_shapes(cores: Cores, chi: int):
    n = len(cores)
    sh, _s = L.shape_array([shape3(c) for c in cores])
    out = (ctypes.c_int64 * (3 * n))()
    cnt = (ctypes.c_int64 * max(1, n - 1))()
    L.call("sgt_svd_round_shapes", n, sh, chi, ctypes.cast(out, L._PI64), ctypes.cast(cnt, L._PI64))
    shapes = [(out[3 * k], out[3 * k + 1], out[3 * k + 2]) for k in range(n)]
    return shapes, [cnt[k] for k in range(n - 1)]


def svd_round(cores: Cores, chi: int, precision: int = L.PREC_F64, spectra: bool = True):
    """TT-SVD rounding to ``chi``.  Returns ``(cores, spectra, counts,
    discarded, status)``: device tensors; ``spectra`` concatenates every bond's
    singular values (``counts`` gives the split), ``status`` the solver's
    outcome.  ``spectra=False`` asks for none (returned as None): the BF16X6
    form then finds each kept subspace without an eigensolve."""
    _check(cores)
    n = len(cores)
    shapes3, counts = svd_round_shapes(cores, chi)
    sh, _s = L.shape_array([shape3(c) for c in cores])
    nbytes = L.query("sgt_svd_round_workspace_size", n, sh, chi, precision)
    if nbytes == 0:
        msg = L.load().sgt_last_error().decode(errors="replace")
        raise L.SyngularError("sgt_svd_round_workspace_size", 1, msg)
    ws = L.workspace(nbytes)
    outs = []
    for k, c in enumerate(cores):
        l, p, r = shapes3[k]
        outs.append(empty((l,) + tuple(c.shape[1:-1]) + (r,)))
    dev = L.device()
    spec = torch.zeros(max(1, sum(counts)), dtype=torch.float64, device=dev) if spectra else None
    disc = torch.zeros(max(1, n - 1), dtype=torch.float64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    cp, _c = L.ptr_array(cores)
    op, _o = L.ptr_array(outs)
    L.call("sgt_svd_round", n, cp, sh, chi, precision, op, L.ptr(spec) if spectra else None, L.ptr(disc),
           L.ptr(status), L.ptr(ws), ws.numel(), L.stream_ptr())
    return outs, spec, counts, disc, status


# ---------------------------------------------------------------------------
# dense reconstruction / element retrieval (chains of GEMMs)
# ---------------------------------------------------------------------------

def _gemm(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, aoff=0, boff=0):
    L.call("sgt_gemm_f64", int(ta), int(tb), M, N, K, alpha,
           L._c_vp(A.data_ptr() + 8 * aoff), lda, 0, L._c_vp(B.data_ptr() + 8 * boff), ldb, 0,
           beta, L.ptr(C), ldc, 0, 1, L.stream_ptr())


def to_tensor_device(cores: Cores) -> torch.Tensor:
    """Contract the whole chain: ``(prod phys)`` tensor (row-major over the
    flattened physical legs), on the device."""
    _check(cores)
    l0, p0, r0 = shape3(cores[0])
    T = cores[0].reshape(l0 * p0, r0)
    rows = l0 * p0
    for c in cores[1:]:
        l, p, r = shape3(c)
        out = empty((rows, p * r))
        _gemm(False, False, rows, p * r, l, 1.0, T, l, c, p * r, 0.0, out, p * r)
        rows = rows * p
        T = out.reshape(rows, r)
    return T.reshape(-1)


def _reshape_or_raise(count: int, shape) -> None:
    """numpy's reshape rule: ``count`` elements into ``shape`` (one -1 allowed)."""
    known = 1
    for s in shape:
        if s != -1:
            known *= int(s)
    ok = (count == known) if -1 not in shape else (known > 0 and count % known == 0)
    if not ok:
        raise ValueError("cannot reshape array of size %d into shape %s" % (count, tuple(shape)))


def apply_window(cores: Cores, gate: torch.Tensor, index: int) -> Cores:
    """``MatrixProductState.apply`` (matrix_product_state.py:487-534) on the
    device: contract sites ``index .. index+m-1`` into ``T[l, in.., r]`` (GEMM
    chain), apply the dense operator (axes ``(out_1..out_m, in_1..in_m)``) as one
    batched GEMM over the left bond, then split ``T`` back left to right: the
    QR of ``L = T(l * p, rest)`` keeps the first ``r_k`` columns of the complete
    Q as core k (``r_k`` the site's original right bond; same sign convention as
    the reference's complete QR) and carries ``R[:r_k, :] = Q^T L`` reshaped,
    row-major, to ``(r_k, -1, r_{k+1})`` exactly as the reference does.  Returns
    a new list (the window replaced, other cores shared); the input is left
    unchanged.  Shapes that numpy cannot reshape raise ValueError."""
    _check(cores)
    g = L.as_device(gate)
    if not g.is_contiguous():
        g = g.contiguous()
    m = g.dim() // 2
    n = len(cores)
    if m < 1 or index < 0 or index + m > n:
        raise IndexError("list index out of range")
    shapes = [tuple(int(s) for s in c.shape) for c in cores]
    out_legs = tuple(int(s) for s in g.shape[:m])
    p_out = int(np.prod(out_legs))
    p_in = int(np.prod(g.shape[m:]))
    win = cores[index:index + m]
    lw, rw = shapes[index][0], shapes[index + m - 1][-1]
    phys_in = int(np.prod([shape3(c)[1] for c in win]))
    if phys_in != p_in:
        raise ValueError("operands could not be broadcast together: operator input %d vs sites %d"
                         % (p_in, phys_in))
    T = to_tensor_device(win) if m > 1 else win[0].reshape(-1)
    # T'[l] (p_out x r) = G (p_out x p_in) @ T[l] (p_in x r), batched over l
    Tg = empty((lw, p_out, rw))
    L.call("sgt_gemm_f64", 0, 0, p_out, rw, p_in, 1.0, L.ptr(g), p_in, 0, L.ptr(T), rw, p_in * rw,
           0.0, L.ptr(Tg), rw, p_out * rw, lw, L.stream_ptr())
    out = list(cores)
    rows, cur = lw, Tg.reshape(-1)
    first_leg = out_legs[0]
    for k in range(index, index + m - 1):
        mrows = rows * first_leg
        ncols = cur.numel() // mrows
        rank = shapes[k][2]
        keep = min(rank, mrows)
        _reshape_or_raise(mrows * keep, shapes[k])
        A = cur.reshape(mrows, ncols).clone()
        Q = empty((mrows, keep))
        tau = empty((min(mrows, ncols),))
        ws = L.workspace(L.query("sgt_qr_workspace_size", mrows, ncols, keep))
        L.call("sgt_qr", L.ptr(A), mrows, ncols, ncols, L.ptr(tau), L.ptr(Q), keep, L.ptr(ws), ws.numel(),
               L.stream_ptr())
        out[k] = Q.reshape(shapes[k])
        # R[:keep, :] = Q^T L
        Rk = empty((keep, ncols))
        _gemm(True, False, keep, ncols, mrows, 1.0, Q, keep, cur, ncols, 0.0, Rk, ncols)
        nxt_r = shapes[k + 1][2]
        _reshape_or_raise(keep * ncols, (rank, -1, nxt_r))
        mid = keep * ncols // (rank * nxt_r)
        rows, first_leg, cur = rank, mid, Rk.reshape(-1)
    _reshape_or_raise(cur.numel(), shapes[index + m - 1])
    out[index + m - 1] = cur.reshape(shapes[index + m - 1])
    return out


def retrieve(cores: Cores, indices: Sequence[int]) -> float:
    """One element (matrix_product_state.py:546-551): product of the slices
    ``core_k[:, i_k, :]``."""
    _check(cores)
    v = torch.ones((1, 1), dtype=torch.float64, device=L.device())
    for c, i in zip(cores, indices):
        l, p, r = shape3(c)
        nv = empty((1, r))
        _gemm(False, False, 1, r, l, 1.0, v, l, c, p * r, 0.0, nv, r, boff=int(i) * r)
        v = nv
    return float(v.reshape(-1)[0].item())


# ---------------------------------------------------------------------------
# fused metric operation: raw W @ X then TT-SVD round
# ---------------------------------------------------------------------------

def eig_method(method: int = 0) -> int:
    """Select the bond eigensolver of the Gram form (1: one-sided Jacobi on Z,
    2: on Z's Cholesky factor, vectors by normalisation, 3: on the factor's
    columns with accumulated rotations); 0 only queries.
    Returns the previous choice."""
    return int(L.load().sgt_eig_method(int(method)))


def mpo_mps_zipup(W: Cores, X: Cores, chi: int):
    """Zip-up of ``W @ X`` to bond ``chi`` (FP64; the library's
    sgt_mpo_mps_zipup).  Returns ``(cores, discarded, status)`` as device
    tensors; the caller chooses the gauge of X (right-orthonormal X gives the
    near-optimal truncation)."""
    _check(W)
    _check(X)
    n = len(X)
    if len(W) != n:
        raise ValueError("operator and state have different lengths")
    wsh, _w = L.i64_array([int(v) for w in W for v in w.shape])
    xsh, _x = L.shape_array([shape3(x) for x in X])
    out_arr = (ctypes.c_int64 * (3 * n))()
    L.call("sgt_mpo_mps_zipup_shapes", n, wsh, xsh, chi, ctypes.cast(out_arr, L._PI64))
    outs = [empty((out_arr[3 * k], out_arr[3 * k + 1], out_arr[3 * k + 2])) for k in range(n)]
    need = L.query("sgt_mpo_mps_zipup_workspace_size", n, wsh, xsh, chi)
    if need == 0:
        raise L.SyngularError("sgt_mpo_mps_zipup_workspace_size", L.SGT_ERR_INVALID,
                              L.load().sgt_last_error().decode(errors="replace"))
    ws = L.workspace(need)
    dev = L.device()
    disc = torch.zeros(max(1, n - 1), dtype=torch.float64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    wp, _wp = L.ptr_array(W)
    xp, _xp = L.ptr_array(X)
    op, _op = L.ptr_array(outs)
    L.call("sgt_mpo_mps_zipup", n, wp, wsh, xp, xsh, chi, op, L.ptr(disc), L.ptr(status), L.ptr(ws), ws.numel(),
           L.stream_ptr())
    return outs, disc, status


def mpo_mps_round(W: Cores, X: Cores, chi: int, precision: int = L.PREC_F64, spectra: bool = True):
    """Raw ``W @ X`` followed by TT-SVD rounding to ``chi`` in one library call.
    Returns ``(cores, spectra, counts, discarded, status)`` (device tensors);
    ``spectra=False`` asks for none (returned as None), which lets the BF16X6
    form find each kept subspace without an eigensolve."""
    _check(W)
    _check(X)
    n = len(X)
    wsh, _w = L.i64_array([int(v) for w in W for v in w.shape])
    xsh, _x = L.shape_array([tuple(x.shape) for x in X])
    pshapes = [(X[k].shape[0] * W[k].shape[0], W[k].shape[2], X[k].shape[2] * W[k].shape[3]) for k in range(n)]
    psh, _p = L.shape_array(pshapes)
    out_arr = (ctypes.c_int64 * (3 * n))()
    cnt_arr = (ctypes.c_int64 * max(1, n - 1))()
    L.call("sgt_svd_round_shapes", n, psh, chi, ctypes.cast(out_arr, L._PI64), ctypes.cast(cnt_arr, L._PI64))
    counts = [cnt_arr[k] for k in range(n - 1)]
    nbytes = L.query("sgt_mpo_mps_round_workspace_size", n, wsh, xsh, chi, precision)
    if nbytes == 0:
        msg = L.load().sgt_last_error().decode(errors="replace")
        raise L.SyngularError("sgt_mpo_mps_round_workspace_size", 1, msg)
    ws = L.workspace(nbytes)
    outs = [empty((out_arr[3 * k], out_arr[3 * k + 1], out_arr[3 * k + 2])) for k in range(n)]
    dev = L.device()
    spec = torch.zeros(max(1, sum(counts)), dtype=torch.float64, device=dev) if spectra else None
    disc = torch.zeros(max(1, n - 1), dtype=torch.float64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    wp, _wp = L.ptr_array(W)
    xp, _xp = L.ptr_array(X)
    op, _o = L.ptr_array(outs)
    L.call("sgt_mpo_mps_round", n, wp, wsh, xp, xsh, chi, precision, op, L.ptr(spec) if spectra else None,
           L.ptr(disc), L.ptr(status), L.ptr(ws), ws.numel(), L.stream_ptr())
    return outs, spec, counts, disc, status
