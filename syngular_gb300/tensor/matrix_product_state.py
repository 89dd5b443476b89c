"""MatrixProductState with device-resident cores (drop-in for
``syngular.tensor.MatrixProductState``, tensor/matrix_product_state.py).

Attributes, operators, error messages and bookkeeping follow the reference:
``sites`` (list of ``(l, p, r)`` cores -- here float64 CUDA tensors),
``sites_number``, ``shape``, ``bond_shape``, ``input_shape``, ``decomposed``,
``orthonormalized``, ``parameters_number``, ``real_parameters_number``.  The
arithmetic runs in the sm_103a library through its C ABI; there is no CPU path.

Deliberate deviations, all on inputs where the reference fails: ``to_tensor``
returns a real array (the reference uses the removed ``np.complex``), and the
hot path prints nothing (the reference prints from
``left_orthonormalization``, mps:556).
"""
from __future__ import annotations

from typing import List, Tuple, Union

import numpy as np
import torch

from .. import _lib as L
from . import _ops


PRECISIONS = {"f64": L.PREC_F64, "tf32": L.PREC_TF32, "tf32x3": L.PREC_TF32X3, "bf16x6": L.PREC_BF16X6}


def precision_code(name: str) -> int:
    """Library code of a precision policy name ("f64", "tf32", "tf32x3",
    "bf16x6"; see include/syngular_gb300.h SGT_PREC_*)."""
    try:
        return PRECISIONS[name]
    except KeyError:
        raise ValueError("unknown precision %r (one of %s)" % (name, ", ".join(sorted(PRECISIONS)))) from None


class MatrixProductState:
    """Matrix product state ``sum prod_k X_k[a_k, i_k, a_{k+1}]``."""

    # Rounding used by ``>>``: "qr" is the reference's QR-column truncation
    # (mps:432-468); "svd" the TT-SVD rounding to the same bond.
    ROUNDING = "qr"
    # Arithmetic of the "svd" rounding: "f64" (plain FP64), "bf16x6" (FP64-class
    # sliced bf16 tensor-core products), "tf32x3" / "tf32" (split / plain TF32).
    PRECISION = "f64"

    def __init__(self, tensor=None, bond_shape: Union[Tuple, List] = (), verbose=0) -> None:
        """mps:30-61."""
        self.parameters_number = 0
        self.real_parameters_number = 0
        self.orthonormalized = None
        if tensor is not None:
            self.tensor = tensor
            self.tensor_shape = tuple(int(s) for s in tensor.shape)
            self.bond_shape = bond_shape
            self.order = len(self.tensor_shape)
            self.real_parameters_number = int(np.prod(self.tensor_shape))
            self.input_shape = self.tensor_shape
            self.sites_number = len(self.bond_shape) + 1
            self.sites = [None] * self.sites_number
            self.norm = None
            if self.order != self.sites_number:
                raise Exception("dimensions of bond indices do not match order - 1")
            if tuple(self.bond_shape) != ():
                n = self.sites_number
                self.shape = [(1, self.tensor_shape[0], self.bond_shape[0])]
                self.shape += [(self.bond_shape[i - 1], self.tensor_shape[i], self.bond_shape[i])
                               for i in range(1, n - 1)]
                self.shape += [(self.bond_shape[n - 2], self.tensor_shape[n - 1], 1)]
            else:
                self.shape = [(1, self.tensor_shape[0], 1)]
        self.verbose = verbose
        self.decomposed = False

    # A raw MPO x MPS product (``W @ X`` with AUTO_ROUND off) keeps its two
    # factors and forms its cores only when they are read: ``>>`` with the
    # "svd" rounding sends the factors to the fused product-and-round call
    # instead, which never stores the product (17 GB in FP64 at chi=256, D=16,
    # 64 sites).
    _lazy = None
    _sites = None

    @property
    def sites(self):
        if self._sites is None and self._lazy is not None:
            W, X, _prec = self._lazy
            self._sites = _ops.contract_mpo_mps(W, X)
        return self._sites

    @sites.setter
    def sites(self, value):
        self._sites = value

    @staticmethod
    def lazy_product(W_sites, X_sites, precision: str):
        """The raw product ``W @ X`` as a state whose cores are formed on first
        read (shapes and bonds as the product's: fused bond a*b)."""
        mp = MatrixProductState()
        mp._lazy = (list(W_sites), list(X_sites), precision)
        mp.sites_number = len(X_sites)
        mp.decomposed = True
        mp.orthonormalized = None
        mp.real_parameters_number = None
        mp.shape = [(int(x.shape[0]) * int(w.shape[0]), int(w.shape[2]), int(x.shape[2]) * int(w.shape[3]))
                    for w, x in zip(W_sites, X_sites)]
        mp.parameters_number = int(sum(a * b * c for a, b, c in mp.shape))
        mp.input_shape = tuple(s[1] for s in mp.shape)
        mp.bond_shape = tuple(s[2] for s in mp.shape[:-1])
        return mp

    # ------------------------------------------------------------------ ops
    def __add__(self, mps):
        """Direct sum, no rounding (mps:75-102)."""
        if self.decomposed and mps.decomposed:
            return MatrixProductState.from_sites(_ops.concat(self.sites, mps.sites))
        raise Exception("Both Matrix Product Operator must be in canonical form (use .decompose()")

    def __or__(self, mp):
        """Inner product without conjugation (mps:116-129)."""
        if isinstance(mp, MatrixProductState):
            # "bf16x6" runs the transfer sweep's contractions on the sliced
            # tensor-core GEMM; the TF32 forms have no overlap of their own
            prec = precision_code(type(self).PRECISION)
            prec = prec if prec == L.PREC_BF16X6 else L.PREC_F64
            return np.float64(_ops.overlap(self.sites, mp.sites, prec))
        raise Exception("right-hand site must be a MatrixProductState")

    def __rshift__(self, dim: int):
        """mps:139-143."""
        if isinstance(dim, int):
            return self.compress(dim, strict=True)
        raise Exception("dimension should be an integer")

    def __getitem__(self, key):
        """mps:157-161."""
        if len(key) != self.sites_number:
            raise Exception("input indices do not match the number of sites")
        return self.retrieve(key)

    def __repr__(self) -> str:
        r = "<Matrix Product State> \n> Sites shape" + str(self.shape) + "\n"
        r += "\t" + "|   " * self.sites_number + "\n"
        r += "\t" + ("O---" * (self.sites_number - 1)) + "O" + "\n"
        return r

    # --------------------------------------------------------- constructors
    @staticmethod
    def random(input_shape, bond_shape):
        """Dense N(0,1) draw from numpy's global RNG (mps:175-178), decomposed on
        the device."""
        tensor = np.random.normal(size=input_shape)
        return MatrixProductState(tensor, bond_shape=bond_shape).decompose()

    @staticmethod
    def from_sites(sites, orthogonality=None, real_parameters_number=None):
        """mps:191-214 (the site list is copied, the cores are not)."""
        mp = MatrixProductState()
        mp.sites = [s if _is_dev(s) else L.as_device(s) for s in list(sites)]
        mp.sites_number = len(mp.sites)
        mp.decomposed = True
        mp.orthonormalized = orthogonality
        mp.parameters_number = int(sum(int(np.prod(s.shape)) for s in mp.sites))
        mp.real_parameters_number = real_parameters_number
        mp.input_shape, mp.bond_shape = (), ()
        mp.shape = [None] * mp.sites_number
        for idx, site in enumerate(mp.sites):
            shp = tuple(int(x) for x in site.shape)
            mp.shape[idx] = shp
            mp.input_shape += (shp[1],)
            if idx != mp.sites_number - 1:
                mp.bond_shape += (shp[2],)
        return mp

    @staticmethod
    def empty():
        return MatrixProductState()

    @staticmethod
    def zeros(input_shape, bond_shape):
        """mps:221-235."""
        n = len(input_shape)
        if tuple(bond_shape) != ():
            shape = [(1, input_shape[0], bond_shape[0])]
            shape += [(bond_shape[i - 1], input_shape[i], bond_shape[i]) for i in range(1, n - 1)]
            shape += [(bond_shape[n - 2], input_shape[n - 1], 1)]
        else:
            shape = [(1, input_shape[0], 1)]
        dev = L.device()
        return MatrixProductState.from_sites(
            [torch.zeros(s, dtype=torch.float64, device=dev) for s in shape])

    # ------------------------------------------------------------- methods
    def dot(self):
        """mps:243-244."""
        return np.sqrt(self | self)

    def normalize(self):
        """Divide the last core by its Frobenius norm (mps:252-256)."""
        _ops.normalize_(self.sites[-1])
        return self

    def to_tensor(self):
        """Dense tensor (mps:265-273), contracted on the device and copied to
        the host."""
        return _ops.to_tensor_device(self.sites).cpu().numpy().reshape(self.input_shape)

    def copy(self):
        """mps:282."""
        return MatrixProductState.from_sites(self.sites)

    def decompose(self, mode="left"):
        """Truncated-QR sweep of the dense tensor (mps:296-350)."""
        if not self.decomposed:
            if mode not in ("left", "right"):
                self.decomposed = True
                return self
            bonds = [int(b) for b in self.bond_shape]
            cores = _ops.decompose(self.tensor, self.tensor_shape, bonds, self.shape,
                                   0 if mode == "left" else 1)
            self.sites = cores
            self.parameters_number += int(sum(int(np.prod(c.shape)) for c in cores))
            del self.tensor
            self.decomposed = True
        return self

    def compress(self, dim: int, mode="left", strict=False):
        """Rounding to ``dim`` (mps:362-468).  ``strict`` returns a new state
        (the ``>>`` path), otherwise the state is rounded in place after a
        left orthonormalisation."""
        if dim >= min(self.bond_shape):
            return self
        if not strict:
            if mode == "left":
                if self.orthonormalized != "left":
                    self.left_orthonormalization()
                new = self._round(self.sites, dim)
                self.sites = new
                self.shape = [tuple(int(x) for x in c.shape) for c in new]
                self.parameters_number = int(sum(int(np.prod(c.shape)) for c in new))
                return None
            if mode == "right":
                raise NotImplementedError("compress(mode='right', strict=False) is not provided")
            return None
        if (self._lazy is not None and self._sites is None and mode == "left"
                and type(self).ROUNDING == "svd"):
            # fused raw product + TT-SVD round: the product is never stored
            W, X, prec = self._lazy
            out, _spec, _cnt, _disc, _st = _ops.mpo_mps_round(W, X, dim, precision_code(prec), spectra=False)
            return MatrixProductState.from_sites(out)
        that = self.copy()
        if mode == "left":
            new = self._round(that.sites, dim)
            that.sites = new
            that.shape = [tuple(int(x) for x in c.shape) for c in new]
            that.parameters_number = int(sum(int(np.prod(c.shape)) for c in new))
        return that

    def _round(self, cores, dim):
        if type(self).ROUNDING == "svd":
            out, _spec, _cnt, _disc, _st = _ops.svd_round(cores, dim, precision_code(type(self).PRECISION),
                                                          spectra=False)
            return out
        return _ops.qr_truncate(cores, dim)

    def apply(self, operator, index, strict=True, mode="compress"):
        """A dense operator (axes ``(out_1..out_m, in_1..in_m)``, numpy or
        torch) on sites ``index .. index+m-1``, split back into cores of the
        original shapes by truncated QR (mps:487-534), on the device.  With
        ``strict`` it works on a copy and returns it.  The reference has no
        working copy when ``strict`` is False and raises NameError; so does this.
        ``mode`` is accepted and unused, as in the reference."""
        if not strict:
            raise NameError("name 'that' is not defined")
        that = self.copy()
        that.sites = _ops.apply_window(that.sites, operator, int(index))
        return that

    def retrieve(self, indices):
        """One tensor element (mps:546-551)."""
        return np.float64(_ops.retrieve(self.sites, indices))

    def left_orthonormalization(self, bond_shape=()):
        """In-place left orthonormalisation (mps:554-566).  Returns None like
        the reference."""
        _ops.left_orthonormalize(self.sites)
        self.orthonormalized = "left"

    def right_orthonormalization(self, bond_shape=()):
        """In-place right orthonormalisation (mps:568-580)."""
        _ops.right_orthonormalize(self.sites)
        self.orthonormalized = "right"

    # matricization helpers (mps:583-622), as device views
    def left_site_matricization(self, index):
        return self.left_matricization(self.sites[index], index)

    def right_site_matricization(self, index):
        return self.right_matricization(self.sites[index], index)

    def left_matricization(self, matrix=None, index: int = 0):
        lrank, input_shape = self.shape[index][0], self.shape[index][1]
        if matrix is None:
            return self.sites[index].reshape(input_shape * lrank, self.shape[index][2])
        return matrix.reshape(input_shape * lrank, -1)

    def right_matricization(self, matrix=None, index: int = 0):
        rrank, input_shape = self.shape[index][2], self.shape[index][1]
        if matrix is None:
            return self.sites[index].reshape(self.shape[index][0], input_shape * rrank)
        return matrix.reshape(-1, input_shape * rrank)

    def tensoricization(self, matrix, index):
        return matrix.reshape(self.shape[index][0], self.shape[index][1], self.shape[index][2])

    def left_orthogonality(self, index):
        """``L^T L`` of core ``index`` (mps:624-626), as a host array."""
        return _ops.orthogonality(self.sites[index], 0).cpu().numpy()

    def right_orthogonality(self, index):
        """``R R^T`` of core ``index`` (mps:628-630), as a host array."""
        return _ops.orthogonality(self.sites[index], 1).cpu().numpy()

    def grad(self, index):
        """mps:632-633."""
        return self.sites[:index] + self.sites[index + 2:]


def _is_dev(t) -> bool:
    return isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()
