"""Generate the golden fixtures by running the unmodified Python reference.

Run in a container that holds the reference source (``SYNGULAR_REFERENCE``,
default ``/root/reference``):

    python tests/golden/make_golden.py

It writes ``tests/golden/*.npz``.  Each file holds the inputs (dense tensors or
cores built with a seeded generator) and the reference's outputs for one group
of cases.  Arrays are stored under ``<case>/<name>`` or ``<case>/<name>/<k>``
for lists of cores; scalars are 0-d arrays.  The reference prints from inside
its hot path; that output is discarded.
"""
from __future__ import annotations

import contextlib
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref_shim  # noqa: E402

syn = ref_shim.load()
from syngular.tensor import MatrixProductOperator as MPO  # noqa: E402
from syngular.tensor import MatrixProductState as MPS  # noqa: E402


def quiet():
    return contextlib.redirect_stdout(io.StringIO())


class Store:
    def __init__(self):
        self.d = {}

    def put(self, case, name, value):
        if isinstance(value, (list, tuple)) and len(value) and isinstance(value[0], np.ndarray):
            for k, v in enumerate(value):
                self.d["%s/%s/%d" % (case, name, k)] = np.asarray(v, dtype=np.float64)
            self.d["%s/%s/n" % (case, name)] = np.asarray(len(value))
        else:
            self.d["%s/%s" % (case, name)] = np.asarray(value)

    def save(self, fname):
        np.savez_compressed(os.path.join(HERE, fname), **self.d)


def cores(mp):
    return [np.array(s, dtype=np.float64) for s in mp.sites]


def rnd_mps(rng, phys, bonds):
    dims = [1] + list(bonds) + [1]
    return [rng.standard_normal((dims[k], phys[k], dims[k + 1])) for k in range(len(phys))]


def rnd_mpo(rng, ins, outs, bonds):
    dims = [1] + list(bonds) + [1]
    return [rng.standard_normal((dims[k], ins[k], outs[k], dims[k + 1])) for k in range(len(ins))]


# ---------------------------------------------------------------------------
def readme_flow(st: Store):
    """readme.md:42-73 with np.random.seed(0) before the flow."""
    np.random.seed(0)
    with quiet():
        W = MPO(np.arange(16 ** 6).reshape((16,) * 6), bond_shape=(16, 16))
        W.decompose()
        X = MPS(np.arange(16 ** 3).reshape((16,) * 3), bond_shape=(4, 4))
        X.decompose()
        T = MPO.random((16, 16, 16), (16, 16, 16), (8, 8))
        MPO.zeros((16, 16, 16), (16, 16, 16), (4, 4))
        U = MPS.random((16, 16, 16), (8, 8))
        W = W >> 4
        T = T >> 2
        TW = T + W
        TWT = TW @ T
        Z = TWT @ X
        xu = X | U
        zx = Z | X
        Z = Z >> 16
        Z.left_orthonormalization()
    st.put("readme", "xu", xu)
    st.put("readme", "zx", zx)
    st.put("readme", "diag0", np.diag(Z.left_orthogonality(0)))
    st.put("readme", "diag1", np.diag(Z.left_orthogonality(1)))
    st.put("readme", "z_shape", np.array(Z.shape))
    st.put("readme", "z_bond_shape", np.array(Z.bond_shape))
    st.put("readme", "tw_bond_shape", np.array(TW.bond_shape))
    st.put("readme", "twt_bond_shape", np.array(TWT.bond_shape))
    st.put("readme", "twt_shape", np.array(TWT.shape))


def config1(st: Store):
    """Config 1 (3 sites, 16-dim legs, bonds 8): Z=(W@X)>>4, Z|Y, orthogonality."""
    for seed in (1, 2):
        np.random.seed(seed)
        w = np.random.normal(size=(16,) * 6)
        x = np.random.normal(size=(16,) * 3)
        y = np.random.normal(size=(16,) * 3)
        with quiet():
            W = MPO(w, bond_shape=(8, 8)).decompose()
            X = MPS(x, bond_shape=(8, 8)).decompose()
            Y = MPS(y, bond_shape=(8, 8)).decompose()
            P = W @ X
            Z = P >> 4
            zy = Z | Y
            zt = Z.to_tensor()
            pt = P.to_tensor()
            Z.left_orthonormalization()
        c = "seed%d" % seed
        st.put(c, "W", cores(W))
        st.put(c, "X", cores(X))
        st.put(c, "Y", cores(Y))
        st.put(c, "P_tensor", pt)
        st.put(c, "Z_tensor", zt)
        st.put(c, "zy", zy)
        st.put(c, "xy", X | Y)
        st.put(c, "Z_shape", np.array(Z.shape))
        st.put(c, "diag0", np.diag(Z.left_orthogonality(0)))
        st.put(c, "diag1", np.diag(Z.left_orthogonality(1)))
        st.put(c, "gram0", Z.left_orthogonality(0))


def known_answers(st: Store):
    """Known answers of the reference's own scripts (deterministic inputs)."""
    # test/test_mpo.py:177-196 test_matmul
    w = np.arange(2 ** 4).reshape((2, 2, 2, 2))
    x = np.arange(2 ** 2).reshape((2, 2))
    with quiet():
        W = MPO(w, bond_shape=(2,)).decompose()
        X = MPS(x, bond_shape=(2,)).decompose()
        Z = W @ W @ X
    st.put("mpo_matmul", "out", Z.to_tensor().reshape(4))
    st.put("mpo_matmul", "exact", x.reshape(4) @ w.reshape(4, 4) @ w.reshape(4, 4))

    # test/test_mpo.py:44-64 test_decompose
    w = np.arange(2 ** 4).reshape((2, 2, 2, 2))
    z = np.arange(4 ** 3 * 3 ** 3).reshape((4, 4, 4, 3, 3, 3))
    with quiet():
        W = MPO(w, bond_shape=(4,)).decompose()
        Z = MPO(z, bond_shape=(3, 3)).decompose()
    st.put("mpo_decompose", "w1111", np.asarray(W[(1, 1), (1, 1)]).reshape(-1)[0])
    st.put("mpo_decompose", "z", np.asarray(Z[(3, 1, 0), (1, 2, 1)]).reshape(-1)[0])
    st.put("mpo_decompose", "W_cores_shape", np.array([c.shape for c in W.sites]))

    # test/test_mpo.py:256-282 test_add
    x = np.arange(1, 17).reshape((2, 2, 2, 2))
    y = np.arange(18, 34).reshape((2, 2, 2, 2))
    with quiet():
        X = MPO(x, bond_shape=(3,)).decompose()
        Y = MPO(y, bond_shape=(3,)).decompose()
        Z = X + Y + Y + Y + Y + Y + Y + Y + Y + Y
    st.put("mpo_add", "z1111", np.asarray(Z[(1, 1), (1, 1)]).reshape(-1)[0])
    st.put("mpo_add", "z_tensor", Z.to_tensor())
    st.put("mpo_add", "z_shape", np.array(Z.shape))

    # test/test_mps.py:51-70 test_add
    x = np.arange(8).reshape((2, 2, 2))
    with quiet():
        X = MPS(x, bond_shape=(2, 2)).decompose()
        Y = MPS(x.copy(), bond_shape=(2, 2)).decompose()
        Z = X + Y
    st.put("mps_add", "z_tensor", Z.to_tensor())
    st.put("mps_add", "z_shape", np.array(Z.shape))

    # test/test_mps.py:22-38 test_augment
    with quiet():
        X = MPS(np.arange(8).reshape((2, 2, 2)), bond_shape=(2, 2)).decompose()
        Y = MPS.zeros((2, 2, 2), (2, 2))
        Z = X
        for _ in range(31):
            Z = Z + Y
        Zc = Z >> 2
    st.put("mps_augment", "z_shape", np.array(Z.shape))
    st.put("mps_augment", "z_tensor", Z.to_tensor())
    st.put("mps_augment", "zc_tensor", Zc.to_tensor())
    st.put("mps_augment", "zc_shape", np.array(Zc.shape))

    # test/test_mps.py:100-126 test_dot / test_normalize
    x = np.arange(4 ** 3).reshape((4, 4, 4))
    with quiet():
        X = MPS(x, bond_shape=(4, 4)).decompose()
        d = X.dot()
        X.normalize()
        d2 = X.dot()
    st.put("mps_dot", "dot", d)
    st.put("mps_dot", "norm2", np.linalg.norm(x) ** 2)
    st.put("mps_dot", "dot_after_normalize", d2)

    # test/test_mps.py:72-84 test_compress
    with quiet():
        X = MPS(np.arange(64).reshape((4, 4, 4)), bond_shape=(4, 4)).decompose()
        Z = X >> 2
    st.put("mps_compress", "z_shape", np.array(Z.shape))
    st.put("mps_compress", "z_tensor", Z.to_tensor())

    # test/test_mps.py:129-157 left/right canonical decompose
    x = np.arange(64).reshape((4, 4, 4))
    with quiet():
        XL = MPS(x, bond_shape=(2, 2))
        XL.decompose(mode="left")
        XR = MPS(x, bond_shape=(2, 2))
        XR.decompose(mode="right")
    st.put("mps_canonical", "left_tensor", XL.to_tensor())
    st.put("mps_canonical", "right_tensor", XR.to_tensor())

    # test/test_mpo.py:66-112 test_orthogonality
    w = np.arange(4 ** 6).reshape((4,) * 6)
    with quiet():
        W = MPO(w, bond_shape=(2, 2))
        W.decompose()
        W.left_orthonormalization()
        l0 = np.diag(W.left_orthogonality(0))
        l1 = np.diag(W.left_orthogonality(1))
        W.right_orthonormalization()
        r1 = np.diag(W.right_orthogonality(1))
        r2 = np.diag(W.right_orthogonality(2))
        v = np.asarray(W[(1, 0, 0), (1, 0, 0)]).reshape(-1)[0]
    st.put("mpo_orth", "l0", l0)
    st.put("mpo_orth", "l1", l1)
    st.put("mpo_orth", "r1", r1)
    st.put("mpo_orth", "r2", r2)
    st.put("mpo_orth", "w100100", v)
    st.put("mpo_orth", "w_exact", w[1, 0, 0, 1, 0, 0])
    st.put("mpo_orth", "params", np.array([W.parameters_number, W.real_parameters_number]))

    # test/test_mpo.py:115-158 test_compress (non-strict in-place compress, then >>)
    w = np.arange(16 ** 4).reshape((16, 16, 16, 16))
    with quiet():
        W = MPO(w, bond_shape=(8,)).decompose()
        p0 = W.parameters_number
        W.compress(4, mode="left")
        p1 = W.parameters_number
        s1 = np.array(W.shape)
        Z = W >> 2
    st.put("mpo_compress", "params", np.array([p0, p1, W.parameters_number]))
    st.put("mpo_compress", "w_shape", s1)
    st.put("mpo_compress", "z_shape", np.array(Z.shape))
    st.put("mpo_compress", "z_tensor", Z.to_tensor())
    st.put("mpo_compress", "w_bond_shape", np.array(W.bond_shape))

    # test/test_mpo.py:296-330 test_compare
    y = np.zeros(2 ** 4).reshape((4, 4))
    np.fill_diagonal(y, list(range(1, 5)))
    y = y.reshape((2, 2, 2, 2))
    with quiet():
        Y = MPO(y, bond_shape=(4,)).decompose().right_orthonormalization()
    st.put("mpo_compare", "y", y)
    st.put("mpo_compare", "y_tensor", Y.to_tensor())


def random_cases(st: Store):
    """Seeded random cases for every hot-path operation."""
    rng = np.random.default_rng(20240611)

    # MPO @ MPS with the auto-round (>> min bond), several shapes
    specs = [((3, 2, 4), (3, 2, 4), (2, 3), (3, 2)),
             ((2, 2, 2, 2), (3, 2, 2, 3), (2, 2, 2), (3, 3, 3)),
             ((4, 3, 2), (2, 3, 4), (3, 5), (4, 2))]
    for n, (ins, outs, xb, wb) in enumerate(specs):
        X = rnd_mps(rng, ins, xb)
        W = rnd_mpo(rng, ins, outs, wb)
        with quiet():
            Xo = MPS.from_sites(X)
            Wo = MPO.from_sites(W)
            Z = Wo @ Xo
        c = "matmul_mps%d" % n
        st.put(c, "X", X)
        st.put(c, "W", W)
        st.put(c, "Z_tensor", Z.to_tensor())
        st.put(c, "Z_shape", np.array(Z.shape))
        st.put(c, "Z_bond_shape", np.array(Z.bond_shape))

    # MPO @ MPO (A.out == B.out so the reference's reshape holds)
    for n, (ins, mids, outs, ab, bb) in enumerate([
            ((2, 3, 2), (3, 2, 2), (3, 2, 2), (2, 3), (3, 2)),
            ((2, 2), (2, 3), (2, 3), (3,), (2,))]):
        A = rnd_mpo(rng, ins, mids, ab)
        B = rnd_mpo(rng, mids, outs, bb)
        with quiet():
            Z = MPO.from_sites(list(A)) @ MPO.from_sites(list(B))
        c = "matmul_mpo%d" % n
        st.put(c, "A", A)
        st.put(c, "B", B)
        st.put(c, "Z_tensor", Z.to_tensor())
        st.put(c, "Z_shape", np.array(Z.shape))

    # MPS + MPS (no rounding) and MPO + MPO (rounds to the min bond)
    X = rnd_mps(rng, (3, 2, 2, 3), (2, 3, 2))
    Y = rnd_mps(rng, (3, 2, 2, 3), (3, 1, 2))
    with quiet():
        Z = MPS.from_sites(X) + MPS.from_sites(Y)
    st.put("add_mps", "X", X)
    st.put("add_mps", "Y", Y)
    st.put("add_mps", "Z", cores(Z))
    A = rnd_mpo(rng, (2, 2, 3), (2, 3, 2), (2, 3))
    B = rnd_mpo(rng, (2, 2, 3), (2, 3, 2), (3, 2))
    with quiet():
        Z = MPO.from_sites(list(A)) + MPO.from_sites(list(B))
    st.put("add_mpo", "A", A)
    st.put("add_mpo", "B", B)
    st.put("add_mpo", "Z_tensor", Z.to_tensor())
    st.put("add_mpo", "Z_shape", np.array(Z.shape))

    # overlaps
    for n, (phys, xb, yb) in enumerate([((2, 3, 2), (2, 2), (2, 3)),
                                        ((4, 4, 4, 4, 4), (4, 8, 8, 4), (3, 5, 7, 2)),
                                        ((5,), (), ())]):
        X = rnd_mps(rng, phys, xb)
        Y = rnd_mps(rng, phys, yb)
        with quiet():
            v = MPS.from_sites(X) | MPS.from_sites(Y)
        c = "overlap%d" % n
        st.put(c, "X", X)
        st.put(c, "Y", Y)
        st.put(c, "value", v)

    # QR truncation >>: plain, padding (dim > r), early exit, MPO
    X = rnd_mps(rng, (4, 4, 4, 4), (4, 8, 4))
    for dim in (2, 3):
        with quiet():
            Z = MPS.from_sites(X) >> dim
        c = "rshift_mps_d%d" % dim
        st.put(c, "X", X)
        st.put(c, "Z_tensor", Z.to_tensor())
        st.put(c, "Z_shape", np.array(Z.shape))
        st.put(c, "Z_bond_shape", np.array(Z.bond_shape))
    X = rnd_mps(rng, (4, 4, 4), (2, 6))
    with quiet():
        Zo = MPS.from_sites(X)
        Z = Zo.compress(4, strict=True)
    st.put("rshift_pad", "X", X)
    st.put("rshift_pad", "Z_tensor", Z.to_tensor())
    st.put("rshift_pad", "Z_shape", np.array(Z.shape))
    st.put("rshift_pad", "Z_gram0", Z.left_orthogonality(0))
    W = rnd_mpo(rng, (2, 2, 2), (2, 2, 2), (4, 5))
    with quiet():
        Wo = MPO.from_sites(list(W))
        Z = Wo >> 2
    st.put("rshift_mpo", "W", W)
    st.put("rshift_mpo", "Z_tensor", Z.to_tensor())
    st.put("rshift_mpo", "Z_shape", np.array(Z.shape))
    st.put("rshift_mpo", "src_bond_shape", np.array(Wo.bond_shape))

    # left / right orthonormalisation and orthogonality
    X = rnd_mps(rng, (3, 3, 3, 3), (3, 4, 3))
    with quiet():
        Xo = MPS.from_sites(X)
        Xo.left_orthonormalization()
        L = cores(Xo)
        Xr = MPS.from_sites(X)
        Xr.right_orthonormalization()
        Rr = cores(Xr)
    st.put("orth_mps", "X", X)
    st.put("orth_mps", "left", L)
    st.put("orth_mps", "right", Rr)
    st.put("orth_mps", "left_gram", [Xo.left_orthogonality(k) for k in range(3)])
    st.put("orth_mps", "right_gram", [Xr.right_orthogonality(k) for k in range(1, 4)])

    # decompose of dense random tensors
    t = rng.standard_normal((3, 4, 5, 2))
    with quiet():
        D = MPS(t, bond_shape=(3, 6, 2)).decompose()
    st.put("decompose_mps", "t", t)
    st.put("decompose_mps", "bonds", np.array([3, 6, 2]))
    st.put("decompose_mps", "Z_tensor", D.to_tensor())
    st.put("decompose_mps", "Z_shape", np.array(D.shape))
    t = rng.standard_normal((2, 3, 3, 2, 2, 3))
    with quiet():
        D = MPO(t, bond_shape=(3, 5)).decompose()
    st.put("decompose_mpo", "t", t)
    st.put("decompose_mpo", "bonds", np.array([3, 5]))
    st.put("decompose_mpo", "Z_tensor", D.to_tensor())
    st.put("decompose_mpo", "Z_shape", np.array(D.shape))


def apply_cases(st: Store):
    """``MatrixProductState.apply`` (tensor/matrix_product_state.py:487-534)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "syngular_gate", os.path.join(ref_shim.REFERENCE_ROOT, "quantum", "gate.py"))
    gate = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gate)  # numpy-only module (the quantum package needs matplotlib)

    # test/test_mps.py:9-19 test_apply: CX on sites 1, 2 of arange(8)
    x = np.arange(8).reshape((2, 2, 2))
    with quiet():
        X = MPS(x, bond_shape=(2, 2)).decompose()
        g = np.asarray(gate.CX, dtype=np.float64).reshape((2, 2, 2, 2))
        Y = X.apply(g, 1)
    st.put("test_apply", "x", cores(X))
    st.put("test_apply", "gate", g)
    st.put("test_apply", "index", 1)
    st.put("test_apply", "out", cores(Y))
    st.put("test_apply", "x_after", cores(X))  # strict: the input is unchanged

    # seeded cores, one- and two-site operators (gates and general matrices)
    rng = np.random.default_rng(2024)
    cases = [
        ("h_site0", (2, 2, 2, 2, 2), (2, 4, 4, 2), np.asarray(gate.H, dtype=np.float64), 0),
        ("x_site4", (2, 2, 2, 2, 2), (2, 4, 4, 2), np.asarray(gate.X, dtype=np.float64), 4),
        ("cx_site1", (2, 2, 2, 2, 2), (2, 4, 4, 2), np.asarray(gate.CX, dtype=np.float64).reshape(2, 2, 2, 2), 1),
        ("swap_site3", (2, 2, 2, 2, 2), (2, 4, 4, 2), np.asarray(gate.SWAP, dtype=np.float64).reshape(2, 2, 2, 2), 3),
        ("rand2_d3", (3, 3, 3, 3), (3, 9, 3), rng.standard_normal((3, 3, 3, 3)), 1),
        ("rand1_d4", (4, 4, 4), (4, 4), rng.standard_normal((4, 4)), 1),
        ("rand2_d2_wide", (2, 2, 2, 2, 2, 2), (2, 4, 8, 4, 2), rng.standard_normal((2, 2, 2, 2)), 2),
    ]
    for name, phys, bonds, g, idx in cases:
        xs = rnd_mps(rng, phys, bonds)
        with quiet():
            X = MPS.from_sites([c.copy() for c in xs])
            Y = X.apply(g, idx)
        st.put(name, "x", xs)
        st.put(name, "gate", g)
        st.put(name, "index", idx)
        st.put(name, "out", cores(Y))


def mul_cases(st: Store):
    """``syngular.mul`` (tensor/utils.py:8-73) on decomposed seeded operands."""
    from syngular.tensor.utils import mul

    rng = np.random.default_rng(77)
    x = rng.standard_normal((2, 3, 2))
    y = rng.standard_normal((2, 3, 2))
    w = rng.standard_normal((2, 3, 2, 2, 3, 2))
    v = rng.standard_normal((2, 3, 2, 2, 3, 2))
    with quiet():
        X = MPS(x, bond_shape=(2, 3)).decompose()
        Y = MPS(y, bond_shape=(2, 3)).decompose()
        W = MPO(w, bond_shape=(2, 2)).decompose()
        V = MPO(v, bond_shape=(3, 2)).decompose()
        xw = mul(X, W)
        wx = mul(W, X)
        xy = mul(X, Y)
        wv = mul(W, V)
    st.put("mul", "X", cores(X))
    st.put("mul", "Y", cores(Y))
    st.put("mul", "W", cores(W))
    st.put("mul", "V", cores(V))
    st.put("mul", "XW", cores(xw))
    st.put("mul", "XW_tensor", xw.to_tensor())
    st.put("mul", "WX", cores(wx))
    st.put("mul", "XY", float(xy))
    st.put("mul", "WV", cores(wv))
    st.put("mul", "WV_tensor", wv.to_tensor())

    # test/test_syn.py:10-26 test_mul: arange operands, both argument orders and MPS . MPS
    x = np.arange(2 ** 2)
    w = np.arange(2 ** 4).reshape((4, 4))
    with quiet():
        X = MPS(x.reshape((2, 2)), bond_shape=(2,)).decompose()
        W = MPO(w.reshape((2, 2, 2, 2)), bond_shape=(2,)).decompose()
        wx = mul(W, X, mode="standard")
        xw = mul(X, W, mode="standard")
        xx = mul(X, X, mode="standard")
    st.put("syn", "X", cores(X))
    st.put("syn", "W", cores(W))
    st.put("syn", "WX_tensor", wx.to_tensor())
    st.put("syn", "XW_tensor", xw.to_tensor())
    st.put("syn", "XX", float(xx))
    st.put("syn", "exact_xw", np.matmul(x, w).astype(np.float64))


def dmrg_cases(st: Store):
    """DMRG environment blocks (variational/dmrg.py:65-112) and the two-site
    tensors a sweep hands to its optimiser (dmrg.py:128-165), from the
    reference's own private methods.  The right sweep runs with a stand-in
    optimiser that records each step's input and returns it normalised (a
    power-iteration step), so the state changes from step to step as in a real
    sweep; every record keeps the state's two sites at that moment."""
    from syngular.variational.dmrg import DMRG as RefDMRG

    cases = [("dmrg_a", (3, 3, 3, 3), (4, 4, 4), (3, 3, 3), 5),
             ("dmrg_b", (2, 2, 2, 2, 2), (3, 5, 5, 3), (2, 4, 4, 2), 6)]
    for case, phys, wb, xb, seed in cases:
        np.random.seed(seed)
        with quiet():
            op = MPO.random(input_shape=phys, output_shape=phys, bond_shape=wb)
            state = MPS.random(input_shape=phys, bond_shape=xb)
            left = RefDMRG._DMRG__left_blocks(operator=op, state=state)
            right = RefDMRG._DMRG__right_blocks(operator=op, state=state)
        st.put(case, "W", cores(op))
        st.put(case, "X", cores(state))
        n = len(phys)
        for k in range(n):
            if left[k] is not None:
                st.put(case, "left/%d" % k, np.asarray(left[k], dtype=np.float64))
            if right[k] is not None:
                st.put(case, "right/%d" % k, np.asarray(right[k], dtype=np.float64))
        records = []

        class Recorder:
            @staticmethod
            def fit(site, init_vec=None):
                k = len(records)
                records.append((np.array(state.sites[k]), np.array(state.sites[k + 1]), np.array(site)))
                v = np.asarray(site).reshape(-1)
                return 0.0, v / np.linalg.norm(v)

        with quiet():
            RefDMRG._DMRG__right_sweep(operator=op, state=state, left_blocks=left, right_blocks=right,
                                       optimizer=Recorder)
        for k, (s0, s1, site) in enumerate(records):
            st.put(case, "step/%d/x0" % k, s0)
            st.put(case, "step/%d/x1" % k, s1)
            st.put(case, "step/%d/site" % k, site)
        st.put(case, "steps", len(records))


GROUPS = {
    "readme_flow": readme_flow,
    "config1": config1,
    "known_answers": known_answers,
    "random_cases": random_cases,
    "apply_cases": apply_cases,
    "mul_cases": mul_cases,
    "dmrg_cases": dmrg_cases,
}


def main():
    """``python make_golden.py [group ...]``: every group, or the ones named."""
    import time
    t0 = time.time()
    for name in (sys.argv[1:] or list(GROUPS)):
        st = Store()
        GROUPS[name](st)
        st.save(name + ".npz")
    print("golden fixtures written to", HERE, "in %.1f s" % (time.time() - t0))


if __name__ == "__main__":
    main()
