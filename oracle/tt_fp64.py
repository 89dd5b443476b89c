"""numpy FP64 restatement of Syngular's matrix-product hot path.

Test infrastructure only: the GPU library is checked against these functions;
nothing in the product imports them.

Conventions (as in the reference): MPS core ``(l, p, r)``, MPO core
``(l, in, out, r)``, row-major unfoldings, first/last bond of size 1.  An MPO
core is treated as an MPS core whose physical leg is ``in*out`` wherever the
reference does so (its ``left_matricization`` reshapes to ``(l*in*out, r)``,
``tensor/matrix_product_operator.py:727-742``).

Every function names the reference lines it restates.  The TT-SVD rounding
(``tt_svd_round``) has no counterpart in the reference (it only has a QR column
truncation); it follows Oseledets, "Tensor-Train Decomposition", SIAM J. Sci.
Comput. 33(5), 2011, Algorithm 2.  Neither has the zip-up (``zipup``;
Stoudenmire & White 2010).  Pinning: the functions with reference counterparts
are checked against fixtures made by running the reference itself
(tests/golden/make_golden.py, tests/test_oracle_golden.py); ``tt_svd_round``
and ``zipup`` are parity unpinned, checked by identities only
(tests/test_oracle_golden.py::test_tt_svd_round_identities,
tests/test_oracle_props.py).
"""
from __future__ import annotations

import math
from typing import List, Sequence, Tuple

import numpy as np

Cores = List[np.ndarray]


# ---------------------------------------------------------------------------
# shapes / bookkeeping
# ---------------------------------------------------------------------------

def mps_shapes(input_shape: Sequence[int], bond_shape: Sequence[int]):
    """Core shapes of an MPS (``tensor/matrix_product_state.py:53-58``,
    ``zeros`` at ``:225-230``)."""
    n = len(input_shape)
    if tuple(bond_shape) == ():
        return [(1, input_shape[0], 1)]
    shp = [(1, input_shape[0], bond_shape[0])]
    shp += [(bond_shape[i - 1], input_shape[i], bond_shape[i]) for i in range(1, n - 1)]
    shp += [(bond_shape[n - 2], input_shape[n - 1], 1)]
    return shp


def mpo_shapes(input_shape, output_shape, bond_shape):
    """Core shapes of an MPO (``tensor/matrix_product_operator.py:49-54``,
    ``zeros`` at ``:390-395``)."""
    n = len(input_shape)
    if tuple(bond_shape) == ():
        return [(1, input_shape[0], output_shape[0], 1)]
    shp = [(1, input_shape[0], output_shape[0], bond_shape[0])]
    shp += [(bond_shape[i - 1], input_shape[i], output_shape[i], bond_shape[i])
            for i in range(1, n - 1)]
    shp += [(bond_shape[n - 2], input_shape[n - 1], output_shape[n - 1], 1)]
    return shp


def bond_shape_of(cores: Cores) -> Tuple[int, ...]:
    """``bond_shape`` as ``from_sites`` recomputes it
    (``tensor/matrix_product_state.py:207-212``): the right bond of every core
    but the last."""
    return tuple(int(c.shape[-1]) for c in cores[:-1])


# ---------------------------------------------------------------------------
# construction
# ---------------------------------------------------------------------------

def _complete_qr_keep(L: np.ndarray, keep: int):
    """``np.linalg.qr(L, mode="complete")`` then ``Q[:, :keep]``, ``R[:keep, :]``
    -- the truncation step used by decompose and compress
    (``tensor/matrix_product_state.py:307-311, 443-446``)."""
    Q, R = np.linalg.qr(L, mode="complete")
    return Q[:, :keep], R[:keep, :]


def mps_decompose(tensor: np.ndarray, bond_shape) -> Cores:
    """Left truncated-QR sweep of a dense tensor
    (``tensor/matrix_product_state.py:296-322``)."""
    shp = mps_shapes(tensor.shape, bond_shape)
    n = len(shp)
    T = np.asarray(tensor, dtype=np.float64)
    cores: Cores = [None] * n
    for k in range(n - 1):
        l, p, r = shp[k]
        L = T.reshape(l * p, -1)
        Q, R = _complete_qr_keep(L, r)
        cores[k] = Q.reshape(l, p, r)
        T = R
    l, p, r = shp[-1]
    cores[-1] = T.reshape(l, p, r)
    return cores


def mpo_interleave(tensor: np.ndarray) -> np.ndarray:
    """Axis order ``(in0, out0, in1, out1, ...)`` of the dense MPO tensor
    (``tensor/matrix_product_operator.py:60``)."""
    n = tensor.ndim // 2
    axes = sum(list(zip(range(n), range(n, 2 * n))), ())
    return np.transpose(tensor, axes=axes)


def mpo_decompose(tensor: np.ndarray, bond_shape) -> Cores:
    """Left truncated-QR sweep of a dense operator
    (``tensor/matrix_product_operator.py:418-453``; a bond-less operator is a
    single reshaped core, ``:419-425``)."""
    n = tensor.ndim // 2
    ins, outs = tensor.shape[:n], tensor.shape[n:]
    shp = mpo_shapes(ins, outs, bond_shape)
    T = mpo_interleave(np.asarray(tensor, dtype=np.float64))
    if tuple(bond_shape) == ():
        return [T.reshape(shp[0])]
    cores: Cores = [None] * n
    for k in range(n - 1):
        l, i, o, r = shp[k]
        L = np.reshape(T, (l * i * o, -1))
        Q, R = _complete_qr_keep(L, r)
        cores[k] = Q.reshape(l, i, o, r)
        T = R
    cores[-1] = T.reshape(shp[-1])
    return cores


def mps_zeros(input_shape, bond_shape) -> Cores:
    """``tensor/matrix_product_state.py:221-235``."""
    return [np.zeros(s) for s in mps_shapes(input_shape, bond_shape)]


def mpo_zeros(input_shape, output_shape, bond_shape) -> Cores:
    """``tensor/matrix_product_operator.py:386-400``."""
    return [np.zeros(s) for s in mpo_shapes(input_shape, output_shape, bond_shape)]


# ---------------------------------------------------------------------------
# site contractions (the raw products, no rounding)
# ---------------------------------------------------------------------------

def mpo_mps_product(W: Cores, X: Cores) -> Cores:
    """Raw ``W @ X`` cores (``tensor/matrix_product_operator.py:183-191``):
    ``P[(a,b), o, (a',b')] = sum_i X[a,i,a'] W[b,i,o,b']`` with the fused bond
    index ``a*B + b`` (state-major)."""
    out = []
    for w, x in zip(W, X):
        a, i, a2 = x.shape
        b, i2, o, b2 = w.shape
        assert i == i2
        site = np.einsum("xiy,bioc->xboyc", x, w, optimize=True)
        out.append(site.reshape(a * b, o, a2 * b2))
    return out


def mpo_mpo_product(A: Cores, B: Cores) -> Cores:
    """Raw ``A @ B`` cores (``tensor/matrix_product_operator.py:279-288``):
    ``P[(b,c), i, o, (b',c')] = sum_m A[b,i,m,b'] B[c,m,o,c']`` with the fused
    bond index ``b*C + c`` (left-operand-major).  The reference reshapes with
    ``A.out`` where ``B.out`` is meant (``:285``), which only works when the two
    agree; this restatement uses ``B.out``."""
    out = []
    for a, bb in zip(A, B):
        b, i, m, b2 = a.shape
        c, m2, o, c2 = bb.shape
        assert m == m2
        site = np.einsum("bimx,cmoy->bcioxy", a, bb, optimize=True)
        out.append(site.reshape(b * c, i, o, b2 * c2))
    return out


# ---------------------------------------------------------------------------
# direct sum
# ---------------------------------------------------------------------------

def direct_sum(A: Cores, B: Cores) -> Cores:
    """Bond concatenation ``A + B`` for MPS or MPO cores
    (``tensor/matrix_product_state.py:75-100``,
    ``tensor/matrix_product_operator.py:84-108``): first core ``[A | B]`` along
    the right bond, last core stacked along the left bond, middle cores block
    diagonal for every physical index, zeros elsewhere."""
    n = len(A)
    out = []
    for k in range(n):
        a, b = A[k], B[k]
        if n == 1:
            out.append(a + b)
            continue
        phys = a.shape[1:-1]
        if k == 0:
            s = np.zeros((a.shape[0],) + phys + (a.shape[-1] + b.shape[-1],))
            s[..., : a.shape[-1]] = a
            s[..., a.shape[-1]:] = b
        elif k == n - 1:
            s = np.zeros((a.shape[0] + b.shape[0],) + phys + (a.shape[-1],))
            s[: a.shape[0]] = a
            s[a.shape[0]:] = b
        else:
            s = np.zeros((a.shape[0] + b.shape[0],) + phys + (a.shape[-1] + b.shape[-1],))
            s[: a.shape[0], ..., : a.shape[-1]] = a
            s[a.shape[0]:, ..., a.shape[-1]:] = b
        out.append(s)
    return out


# ---------------------------------------------------------------------------
# overlap
# ---------------------------------------------------------------------------

def overlap(X: Cores, Y: Cores) -> float:
    """``X | Y`` = ``sum prod_k X_k[a,p,a'] Y_k[c,p,c']`` without conjugation
    (``tensor/matrix_product_state.py:116-127``), evaluated as a transfer sweep
    ``E_{k+1} = sum_p X_k[:,p,:]^T E_k Y_k[:,p,:]`` from ``E_0 = [[1]]``."""
    E = np.ones((1, 1))
    for x, y in zip(X, Y):
        a, p, a2 = x.shape
        c, p2, c2 = y.shape
        assert p == p2
        T = (E @ y.reshape(c, p * c2)).reshape(a * p, c2)
        E = x.reshape(a * p, a2).T @ T
    return float(E.reshape(-1)[0])


def overlap_log(X: Cores, Y: Cores):
    """Transfer sweep with per-site rescaling: returns ``(sign*mantissa, log)``
    with ``X|Y = mantissa * exp(log)``, safe for long chains."""
    E = np.ones((1, 1))
    logscale = 0.0
    for x, y in zip(X, Y):
        a, p, a2 = x.shape
        c, p2, c2 = y.shape
        T = (E @ y.reshape(c, p * c2)).reshape(a * p, c2)
        E = x.reshape(a * p, a2).T @ T
        s = float(np.max(np.abs(E)))
        if s > 0:
            E = E / s
            logscale += math.log(s)
    return float(E.reshape(-1)[0]), logscale


# ---------------------------------------------------------------------------
# QR column truncation (the reference ``>>``) and orthonormalisation
# ---------------------------------------------------------------------------

def _phys(core: np.ndarray) -> int:
    return int(np.prod(core.shape[1:-1]))


def qr_truncate(cores: Cores, dim: int, bond_shape=None) -> Cores:
    """Reference rounding ``>> dim`` = ``compress(dim, strict=True)``
    (``tensor/matrix_product_state.py:362-368, 432-468``;
    ``tensor/matrix_product_operator.py:469-474, 544-580``).

    Early exit when ``dim >= min(bond_shape)`` (the attribute, which the caller
    passes when it is stale); otherwise for k = 0..N-2:
    ``L_k = Q S`` (complete QR), core_k <- ``Q[:, :dim]``,
    core_{k+1} <- ``S[:dim, :] @ R_{k+1}``.  A bond narrower than ``dim`` is
    padded (the extra columns of the complete ``Q`` meet zero rows of ``S``);
    ``l*p < dim`` makes the reference's reshape fail, raised here as
    ``ValueError``."""
    if bond_shape is None:
        bond_shape = bond_shape_of(cores)
    if len(bond_shape) == 0 or dim >= min(bond_shape):
        return list(cores)
    out = [c.copy() for c in cores]
    n = len(out)
    for k in range(n - 1):
        ck, cn = out[k], out[k + 1]
        lead = ck.shape[:-1]
        L = ck.reshape(-1, ck.shape[-1])
        R = cn.reshape(cn.shape[0], -1)
        if L.shape[0] < dim:
            raise ValueError(
                "cannot reshape array of size %d into shape %s"
                % (L.shape[0] * min(L.shape[0], dim), lead + (dim,)))
        Q, S = _complete_qr_keep(L, dim)
        out[k] = Q.reshape(lead + (dim,))
        out[k + 1] = (S @ R).reshape((dim,) + cn.shape[1:])
    return out


def left_orthonormalize(cores: Cores) -> Cores:
    """``left_orthonormalization`` (``tensor/matrix_product_state.py:554-566``,
    ``tensor/matrix_product_operator.py:673-694``): reduced QR ``L_k = U B``,
    core_k <- U, core_{k+1} <- ``B @ R_{k+1}``.  The reference keeps the old
    core shapes, so it needs ``l*p >= r``; the same precondition holds here."""
    out = [c.copy() for c in cores]
    for k in range(len(out) - 1):
        ck, cn = out[k], out[k + 1]
        L = ck.reshape(-1, ck.shape[-1])
        if L.shape[0] < L.shape[1]:
            raise ValueError("left_orthonormalization needs l*p >= r at site %d" % k)
        U, B = np.linalg.qr(L)
        out[k] = U.reshape(ck.shape)
        out[k + 1] = (B @ cn.reshape(cn.shape[0], -1)).reshape(cn.shape)
    return out


def right_orthonormalize(cores: Cores) -> Cores:
    """``right_orthonormalization`` (``tensor/matrix_product_state.py:568-580``,
    ``tensor/matrix_product_operator.py:696-719``): for k = N-1..1,
    ``R_k^T = V U``; core_k <- ``V^T``, core_{k-1} <- ``L_{k-1} @ U^T``."""
    out = [c.copy() for c in cores]
    for k in range(len(out) - 1, 0, -1):
        ck, cp = out[k], out[k - 1]
        R = ck.reshape(ck.shape[0], -1)
        if R.shape[1] < R.shape[0]:
            raise ValueError("right_orthonormalization needs p*r >= l at site %d" % k)
        V, U = np.linalg.qr(R.T)
        out[k] = V.T.reshape(ck.shape)
        out[k - 1] = (cp.reshape(-1, cp.shape[-1]) @ U.T).reshape(cp.shape)
    return out


def left_orthogonality(core: np.ndarray) -> np.ndarray:
    """``L^T L`` of the left unfolding (``tensor/matrix_product_state.py:624-626``)."""
    L = core.reshape(-1, core.shape[-1])
    return L.T @ L


def right_orthogonality(core: np.ndarray) -> np.ndarray:
    """``R R^T`` of the right unfolding (``tensor/matrix_product_state.py:628-630``)."""
    R = core.reshape(core.shape[0], -1)
    return R @ R.T


def normalize(cores: Cores) -> Cores:
    """Divide the last core by its Frobenius norm
    (``tensor/matrix_product_state.py:252-256``)."""
    out = list(cores)
    out[-1] = out[-1] / np.linalg.norm(out[-1].reshape(out[-1].shape[0], -1))
    return out


def dot(cores: Cores) -> float:
    """``sqrt(X | X)`` (``tensor/matrix_product_state.py:243-244``)."""
    return math.sqrt(overlap(cores, cores))


def to_tensor(cores: Cores) -> np.ndarray:
    """Dense tensor of an MPS (``tensor/matrix_product_state.py:265-273``) --
    contracted directly instead of element by element."""
    T = cores[0].reshape(-1, cores[0].shape[-1])
    phys = [cores[0].shape[1]]
    for c in cores[1:]:
        T = T @ c.reshape(c.shape[0], -1)
        T = T.reshape(-1, c.shape[-1])
        phys.append(c.shape[1])
    return T.reshape(phys)


def mps_apply(cores: Cores, gate: np.ndarray, index: int) -> Cores:
    """``MatrixProductState.apply(gate, index)`` with ``strict=True``
    (``tensor/matrix_product_state.py:487-534``): a dense operator with axes
    ``(out_1..out_m, in_1..in_m)`` acts on sites ``index .. index+m-1``; the
    contracted window ``T[l, out.., r]`` is split back left to right by complete
    QR, keeping ``Q[:, :r_k]`` (``r_k`` the site's original right bond) as core
    k and reshaping ``R[:r_k, :]`` to ``(r_k, -1, r_{k+1})`` (the reference's
    reshape, row-major, whatever the window length); the last window core is
    the remainder.  Shapes follow the reference's ``tensoricization``, so a
    window whose sizes do not fit raises numpy's ValueError as it does."""
    shapes = [tuple(c.shape) for c in cores]
    out = list(cores)
    m = gate.ndim // 2
    T = cores[index]
    for k in range(index + 1, index + m):
        T = np.tensordot(T, cores[k], axes=([T.ndim - 1], [0]))
    l, r = T.shape[0], T.shape[-1]
    p_in = int(np.prod(gate.shape[m:]))
    p_out = int(np.prod(gate.shape[:m]))
    T = np.einsum("oi,lir->lor", gate.reshape(p_out, p_in), T.reshape(l, p_in, r))
    T = T.reshape((l,) + tuple(gate.shape[:m]) + (r,))
    for k in range(index, index + m - 1):
        L_ = T.reshape(T.shape[1] * T.shape[0], -1)
        Q, R = _complete_qr_keep(L_, shapes[k][2])
        out[k] = np.reshape(Q, shapes[k])
        T = R.reshape((shapes[k][2], -1, shapes[k + 1][2]))
    out[index + m - 1] = np.reshape(T, shapes[index + m - 1])
    return out


def mul(kind1: str, cores1: Cores, kind2: str, cores2: Cores, bonds1=None, bonds2=None):
    """``syngular.mul(op1, op2, mode="standard")`` (``tensor/utils.py:8-73``);
    ``kind`` is "mps" or "mpo", ``bonds`` the objects' ``bond_shape``
    attributes (default: the cores' bonds).  MPS x MPO and MPO x MPS: the site
    product with the state-major fused bond, then ``>> min_bond``; MPS x MPS:
    the overlap; MPO x MPO: ``op2``'s output leg contracted with ``op1``'s input
    leg, ``op2``-major fused bond (utils.py:61-71), then ``>> min_bond``.
    Returns (kind, cores) or ("scalar", value)."""
    b1 = bond_shape_of(cores1) if bonds1 is None else tuple(bonds1)
    b2 = bond_shape_of(cores2) if bonds2 is None else tuple(bonds2)
    if len(cores1) != len(cores2):
        raise Exception("both operator do not have the same number of sites")
    min_bond = min(min(b1), min(b2))
    if kind1 == "mps" and kind2 == "mpo":
        return "mps", qr_truncate(mpo_mps_product(cores2, cores1), min_bond)
    if kind1 == "mpo" and kind2 == "mps":
        return "mps", qr_truncate(mpo_mps_product(cores1, cores2), min_bond)
    if kind1 == "mps" and kind2 == "mps":
        return "scalar", overlap(cores1, cores2)
    return "mpo", qr_truncate(mpo_mpo_product(cores2, cores1), min_bond)


def mpo_to_tensor(cores: Cores) -> np.ndarray:
    """Dense ``(*in, *out)`` tensor of an MPO
    (``tensor/matrix_product_operator.py:405-416``)."""
    n = len(cores)
    T = cores[0].reshape(-1, cores[0].shape[-1])
    for c in cores[1:]:
        T = (T @ c.reshape(c.shape[0], -1)).reshape(-1, c.shape[-1])
    ins = [c.shape[1] for c in cores]
    outs = [c.shape[2] for c in cores]
    T = T.reshape(sum(([i, o] for i, o in zip(ins, outs)), []))
    axes = list(range(0, 2 * n, 2)) + list(range(1, 2 * n, 2))
    return np.transpose(T, axes)


# ---------------------------------------------------------------------------
# TT-SVD rounding (no reference counterpart)
# ---------------------------------------------------------------------------

def left_qr_sweep(cores: Cores) -> Cores:
    """Left orthogonalisation with bond reduction to ``min(l*p, r)`` (step 1 of
    Oseledets Alg. 2)."""
    out = [np.array(c, dtype=np.float64) for c in cores]
    for k in range(len(out) - 1):
        ck, cn = out[k], out[k + 1]
        lead = ck.shape[:-1]
        L = ck.reshape(-1, ck.shape[-1])
        Q, R = np.linalg.qr(L)
        out[k] = Q.reshape(lead + (Q.shape[1],))
        out[k + 1] = (R @ cn.reshape(cn.shape[0], -1)).reshape((R.shape[0],) + cn.shape[1:])
    return out


def tt_svd_round(cores: Cores, chi: int, rel_tol: float = 0.0):
    """TT-SVD rounding to bond ``chi``: left QR sweep, then right-to-left
    truncated SVDs (Oseledets 2011, Alg. 2).

    Returns ``(cores, spectra, discarded)``: the rounded cores (right
    orthonormal except the first), the full singular values at every bond
    ``k = 1..N-1`` (index ``k-1``), and the discarded weight
    ``sum(dropped s^2) / sum(s^2)`` at every bond.  With ``rel_tol > 0`` a bond
    is also cut where ``s_j < rel_tol * s_0``."""
    out = left_qr_sweep(cores)
    n = len(out)
    spectra = [None] * (n - 1)
    discarded = [0.0] * (n - 1)
    for k in range(n - 1, 0, -1):
        ck = out[k]
        M = ck.reshape(ck.shape[0], -1)
        U, s, Vt = np.linalg.svd(M, full_matrices=False)
        keep = min(chi, len(s))
        if rel_tol > 0 and len(s) and s[0] > 0:
            keep = min(keep, max(1, int(np.sum(s > rel_tol * s[0]))))
        spectra[k - 1] = s.copy()
        tot = float(np.sum(s * s))
        discarded[k - 1] = float(np.sum(s[keep:] ** 2) / tot) if tot > 0 else 0.0
        out[k] = Vt[:keep].reshape((keep,) + ck.shape[1:])
        cp = out[k - 1]
        out[k - 1] = (cp.reshape(-1, cp.shape[-1]) @ (U[:, :keep] * s[:keep])).reshape(
            cp.shape[:-1] + (keep,))
    return out, spectra, discarded


# ---------------------------------------------------------------------------
# seeded workloads
# ---------------------------------------------------------------------------

def random_mps_cores(rng: np.random.Generator, n: int, d, chi, scale: bool = True) -> Cores:
    """Cores built directly (``from_sites``) with entries N(0,1)/sqrt(chi*d);
    ``d`` and ``chi`` are ints or per-site / per-bond sequences."""
    ds = [d] * n if np.isscalar(d) else list(d)
    bonds = [chi] * (n - 1) if np.isscalar(chi) else list(chi)
    dims = [1] + bonds + [1]
    out = []
    for k in range(n):
        sh = (dims[k], ds[k], dims[k + 1])
        s = 1.0 / math.sqrt(max(dims[k], dims[k + 1]) * ds[k]) if scale else 1.0
        out.append(rng.standard_normal(sh) * s)
    return out


def random_mpo_cores(rng: np.random.Generator, n: int, d, D, scale: bool = True) -> Cores:
    """MPO cores ``(D, d, d, D)`` with entries N(0,1)/sqrt(D*d)."""
    ds = [d] * n if np.isscalar(d) else list(d)
    bonds = [D] * (n - 1) if np.isscalar(D) else list(D)
    dims = [1] + bonds + [1]
    out = []
    for k in range(n):
        sh = (dims[k], ds[k], ds[k], dims[k + 1])
        s = 1.0 / math.sqrt(max(dims[k], dims[k + 1]) * ds[k]) if scale else 1.0
        out.append(rng.standard_normal(sh) * s)
    return out


def geometric_mps_cores(rng: np.random.Generator, n: int, d: int, chi: int, ratio: float = 0.98) -> Cores:
    """Cores with geometric singular spectra ``s_k ~ ratio**k``: each core is a
    random orthogonal factor times ``diag(s)`` times a random orthogonal factor,
    reshaped to ``(chi, d, chi)`` (bonds capped by the rank bound at the
    edges)."""
    dims = [1] + [min(chi, d ** min(k, n - k)) for k in range(1, n)] + [1]
    out = []
    for k in range(n):
        l, r = dims[k], dims[k + 1]
        m, c = l * d, r
        G = rng.standard_normal((m, m))
        Q1, _ = np.linalg.qr(G)
        G2 = rng.standard_normal((c, c))
        Q2, _ = np.linalg.qr(G2)
        kk = min(m, c)
        s = ratio ** np.arange(kk)
        core = (Q1[:, :kk] * s) @ Q2[:kk, :]
        out.append(core.reshape(l, d, r))
    return out


def config1_inputs(seed: int):
    """README-sized plain case: dense N(0,1) tensors from the legacy global RNG,
    in the order W (16^6), X (16^3), Y (16^3)."""
    np.random.seed(seed)
    w = np.random.normal(size=(16, 16, 16, 16, 16, 16))
    x = np.random.normal(size=(16, 16, 16))
    y = np.random.normal(size=(16, 16, 16))
    return w, x, y


def config1_flow(seed: int):
    """Config-1 flow with the reference's semantics: ``Z = (W @ X) >> 4``,
    ``Z | Y``, left orthonormalisation and the orthogonality diagonals.
    ``@`` ends with ``>> min(min(W.bond_shape), min(X.bond_shape))``
    (``tensor/matrix_product_operator.py:176, 192``)."""
    w, x, y = config1_inputs(seed)
    W = mpo_decompose(w, (8, 8))
    X = mps_decompose(x, (8, 8))
    Y = mps_decompose(y, (8, 8))
    P = mpo_mps_product(W, X)
    Z = qr_truncate(P, min(min(bond_shape_of(W)), min(bond_shape_of(X))))
    Z = qr_truncate(Z, 4)
    zy = overlap(Z, Y)
    Zo = left_orthonormalize(Z)
    return dict(W=W, X=X, Y=Y, Z=Z, zy=zy, Zo=Zo,
                diag0=np.diag(left_orthogonality(Zo[0])),
                diag1=np.diag(left_orthogonality(Zo[1])))


def sweep_fp64(W: Cores, X: Cores, chi: int):
    """One metric sweep: raw ``W @ X``, TT-SVD round back to ``chi``, overlap
    of the result with the input state."""
    P = mpo_mps_product(W, X)
    Z, spectra, disc = tt_svd_round(P, chi)
    return Z, overlap(X, Z), spectra, disc


# ---------------------------------------------------------------------------
# DMRG environment blocks (variational/dmrg.py)
# ---------------------------------------------------------------------------

def env_left_blocks(W: Cores, X: Cores, Y: Cores = None) -> list:
    """``DMRG.__left_blocks`` (``variational/dmrg.py:89-112``): for k = 0..n-3,
    ``L_k[a', b', c'] = sum L_{k-1}[a, b, c] X_k[a, o, a'] W_k[b, i, o, b']
    Y_k[c, i, c']`` (the bra X on the operator's output leg, the ket Y on its
    input leg; the reference uses one state for both), the first block without
    ``L_{-1}``.  Entries k >= n-2 are None, as in the reference."""
    Y = X if Y is None else Y
    n = len(W)
    out = [None] * n
    prev = np.ones((1, 1, 1))
    for k in range(n - 2):
        t = np.tensordot(prev, X[k], axes=([0], [0]))            # [b, c, o, a']
        t = np.tensordot(t, W[k], axes=([0, 2], [0, 2]))         # [c, a', i, b']
        t = np.tensordot(t, Y[k], axes=([0, 2], [0, 1]))         # [a', b', c']
        out[k] = t
        prev = t
    return out


def env_right_blocks(W: Cores, X: Cores, Y: Cores = None) -> list:
    """``DMRG.__right_blocks`` (``variational/dmrg.py:65-87``): for k = n-1
    down to 2, ``R_k[a, b, c] = sum X_k[a, o, a'] W_k[b, i, o, b']
    Y_k[c, i, c'] R_{k+1}[a', b', c']``, the last block without ``R_n``.
    Entries k < 2 are None."""
    Y = X if Y is None else Y
    n = len(W)
    out = [None] * n
    nxt = np.ones((1, 1, 1))
    for k in range(n - 1, 1, -1):
        t = np.tensordot(X[k], nxt, axes=([2], [0]))             # [a, o, b', c']
        t = np.tensordot(t, W[k], axes=([1, 2], [2, 3]))         # [a, c', b, i]
        t = np.tensordot(t, Y[k], axes=([3, 1], [1, 2]))         # [a, b, c]
        out[k] = t
        nxt = t
    return out


def env_two_site(Lb, merge: np.ndarray, W1: np.ndarray, W2: np.ndarray, Rb) -> np.ndarray:
    """The tensor each DMRG sweep step hands to its optimiser
    (``variational/dmrg.py:143-165``): ``out[a, o1, o2, a4] = sum L[a, b, c]
    M[c, i1, i2, c4] W1[b, i1, o1, b2] W2[b2, i2, o2, b3] R[a4, b3, c4]``, with
    L (first step) or R (last step) absent, i.e. the unit block."""
    Lb = np.ones((1, 1, 1)) if Lb is None else Lb
    Rb = np.ones((1, 1, 1)) if Rb is None else Rb
    t = np.tensordot(Lb, merge, axes=([2], [0]))                 # [a, b, i1, i2, c4]
    t = np.tensordot(t, W1, axes=([1, 2], [0, 1]))               # [a, i2, c4, o1, b2]
    t = np.tensordot(t, W2, axes=([4, 1], [0, 1]))               # [a, c4, o1, o2, b3]
    t = np.tensordot(t, Rb, axes=([4, 1], [1, 2]))               # [a, o1, o2, a4]
    return t


# ---------------------------------------------------------------------------
# zip-up MPO x MPS (no reference code: the reference's "variational" and
# "fit-up" MATMUL_MODE branches, tensor/matrix_product_operator.py:262-276, are
# empty); Stoudenmire & White, New J. Phys. 12, 055026 (2010)
# ---------------------------------------------------------------------------

def zipup(W: Cores, X: Cores, chi: int):
    """Zip-up of ``W @ X`` to bond ``chi``: a carry C[r, a, b] moves left to
    right; at site k, M[(r, o), (a', b')] = sum C[r, a, b] X_k[a, i, a']
    W_k[b, i, o, b'] is split by its SVD, the core takes the leading
    min(chi, rank bound) left singular vectors and the carry S V^T; the last
    core is M.  Returns (cores, discarded) with discarded[k] = dropped s^2 /
    total s^2 at the cut after site k."""
    n = len(X)
    C = np.ones((1, 1, 1))
    out, disc = [], []
    for k in range(n):
        T = np.tensordot(C, X[k], axes=([1], [0]))          # [r, b, i, a']
        T = np.tensordot(T, W[k], axes=([1, 2], [0, 1]))    # [r, a', o, b']
        r, a2, o, b2 = T.shape
        M = T.transpose(0, 2, 1, 3).reshape(r * o, a2 * b2)
        if k == n - 1:
            out.append(M.reshape(r, o, 1))
            break
        U, s, Vt = np.linalg.svd(M, full_matrices=False)
        q = min(chi, len(s))
        tot = float(np.sum(s * s))
        disc.append(float(np.sum(s[q:] ** 2) / tot) if tot > 0 else 0.0)
        out.append(U[:, :q].reshape(r, o, q))
        C = (s[:q, None] * Vt[:q]).reshape(q, a2, b2)
    return out, disc
