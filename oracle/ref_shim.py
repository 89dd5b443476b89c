"""Import the unmodified Python reference as ``syngular`` (development container only).

Test infrastructure: used by ``tests/golden/make_golden.py`` to run the
reference on seeded inputs and write the golden fixtures.  It never runs on a
GPU host and the product never imports it.

The reference source is not edited.  What this shim supplies:
  * stub modules for imports the hot path never uses: ``cv2`` and
    ``django.forms`` (``tensor/matrix_product_operator.py:7-8``) and ``turtle``
    (``tensor/differential_matrix_product_operator.py:1``);
  * numpy-2 compatibility: ``np.reshape(..., newshape=...)`` (used by the
    matricization helpers, ``tensor/matrix_product_state.py:589-622``) and
    ``np.complex`` (``tensor/matrix_product_state.py:266``);
  * ``to_tensor`` for MPS/MPO re-expressed so that the (1,1)-shaped values of
    ``retrieve`` are stored as scalars (the original assignment fails on numpy 2).
"""
from __future__ import annotations

import itertools
import os
import sys
import tempfile
import types

import numpy as np

REFERENCE_ROOT = os.environ.get("SYNGULAR_REFERENCE", "/root/reference")

_loaded = None


def _install_stubs():
    if "cv2" not in sys.modules:
        cv2 = types.ModuleType("cv2")
        cv2.eigen = None
        sys.modules["cv2"] = cv2
    if "django" not in sys.modules:
        dj = types.ModuleType("django")
        forms = types.ModuleType("django.forms")
        forms.PasswordInput = object
        dj.forms = forms
        sys.modules["django"] = dj
        sys.modules["django.forms"] = forms
    if "turtle" not in sys.modules:
        t = types.ModuleType("turtle")
        t.right = None
        sys.modules["turtle"] = t


def _patch_numpy():
    if getattr(np.reshape, "_syngular_shim", False):
        return
    orig = np.reshape

    def reshape(a, *args, newshape=None, **kw):
        if newshape is not None:
            return orig(a, newshape, **kw)
        return orig(a, *args, **kw)

    reshape._syngular_shim = True
    np.reshape = reshape
    if not hasattr(np, "complex"):
        np.complex = complex


def load():
    """Return the reference package imported as ``syngular``."""
    global _loaded
    if _loaded is not None:
        return _loaded
    if not os.path.isdir(REFERENCE_ROOT):
        raise RuntimeError("reference source not found at %s" % REFERENCE_ROOT)
    _install_stubs()
    _patch_numpy()
    tmp = tempfile.mkdtemp(prefix="syngular_ref_")
    os.symlink(REFERENCE_ROOT, os.path.join(tmp, "syngular"))
    sys.path.insert(0, tmp)
    sys.dont_write_bytecode = True
    import syngular  # noqa: F401
    from syngular.tensor import MatrixProductOperator, MatrixProductState

    def mps_to_tensor(self):
        out = np.zeros(shape=self.input_shape)
        for inp in itertools.product(*[range(i) for i in self.input_shape]):
            out[inp] = np.asarray(self[inp]).reshape(-1)[0]
        return out

    def mpo_to_tensor(self):
        out = np.zeros(shape=(*self.input_shape, *self.output_shape))
        for inp in itertools.product(*[range(i) for i in self.input_shape]):
            for o in itertools.product(*[range(i) for i in self.output_shape]):
                out[(*inp, *o)] = np.asarray(self[inp, o]).reshape(-1)[0]
        return out

    MatrixProductState.to_tensor = mps_to_tensor
    MatrixProductOperator.to_tensor = mpo_to_tensor
    _loaded = syngular
    return syngular
