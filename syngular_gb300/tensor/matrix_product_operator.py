"""MatrixProductOperator with device-resident cores (drop-in for
``syngular.tensor.MatrixProductOperator``, tensor/matrix_product_operator.py).

Cores are ``(l, in, out, r)`` float64 CUDA tensors.  ``@`` (MPO x MPS and
MPO x MPO) and ``+`` end with ``>> min(min(A.bond_shape), min(B.bond_shape))``
computed from the ``bond_shape`` attributes, which can be stale exactly as in
the reference (mpo:110, 176, 192, 289); ``>>`` sets the source's
``bond_shape`` to ``(dim,) * (n-1)`` (mpo:477).

Deliberate deviations, on inputs where the reference misbehaves:
  * ``>>`` does not overwrite the source's cores (the reference's ``copy``
    aliases the site list, mpo:360/403, so its truncation mutates the source);
  * MPO x MPO uses the second operand's output dimension (mpo:285 reshapes with
    the first operand's, which only works when the two agree);
  * ``decompose`` prints nothing (mpo:442).
``MATMUL_MODE`` "opti" (the reference's unfinished density-matrix compression,
mpo:193-273) is the fused product + TT-SVD round to the min bond; "zip-up" (not
a reference mode) is the zip-up compression of Stoudenmire & White 2010;
"variational" and "fit-up" are empty in the reference and return None here as
there.
"""
from __future__ import annotations

from typing import List, Tuple, Union

import numpy as np
import torch

from .. import _lib as L
from . import _ops
from .matrix_product_state import MatrixProductState, _is_dev, precision_code


class MatrixProductOperator:
    COMPRESS = True
    DECOMPOSE = False
    MATMUL_MODE = "standard"
    # "qr": reference QR-column truncation; "svd": TT-SVD rounding
    ROUNDING = "qr"
    # False: `@` and `+` return the raw (unrounded) product / sum; an MPO x MPS
    # product is then formed lazily, and `>>` on it with ROUNDING = "svd" runs
    # the fused product + TT-SVD round in PRECISION without storing the product
    AUTO_ROUND = True
    # Arithmetic of the "svd" rounding of `@` / `+` / `>>`: "f64" (plain FP64),
    # "bf16x6" (FP64-class sliced bf16 tensor-core products, FP32-pair
    # elementwise work, refined FP32 Jacobi), "tf32x3" / "tf32" (split / plain TF32)
    PRECISION = "f64"

    def __init__(self, tensor=None, bond_shape: Union[Tuple, List] = (), verbose=0) -> None:
        """mpo:25-64."""
        self.parameters_number = 0
        self.real_parameters_number = 0
        if tensor is not None:
            self.tensor = tensor
            self.tensor_shape = tuple(int(s) for s in tensor.shape)
            self.bond_shape = tuple(bond_shape)
            self.real_parameters_number = int(np.prod(self.tensor_shape))
            self.sites_number = len(self.bond_shape) + 1
            self.sites = [None] * self.sites_number
            n = self.sites_number
            self.input_shape = tuple(self.tensor_shape[:n])
            self.output_shape = tuple(self.tensor_shape[n:])
            if len(self.input_shape) != len(self.output_shape):
                raise Exception("input_shape and output_shape of the tensor must have the same length")
            if len(self.input_shape) != len(self.bond_shape) + 1:
                raise Exception("dimensions of bond indices do not match input dimension - 1")
            ts = self.tensor_shape
            if self.bond_shape != ():
                self.shape = [(1, ts[0], ts[n], self.bond_shape[0])]
                self.shape += [(self.bond_shape[i - 1], ts[i], ts[n + i], self.bond_shape[i])
                               for i in range(1, n - 1)]
                self.shape += [(self.bond_shape[n - 2], ts[n - 1], ts[2 * n - 1], 1)]
            else:
                self.shape = [(1, ts[0], ts[1], 1)]
            self.shape_indices = [(2 * n + i, i, n + i, 2 * n + i + 1) for i in range(n)]
            # interleave (in0, out0, in1, out1, ...) (mpo:60); done on the device
            axes = sum(list(zip(range(n), range(n, 2 * n))), ())
            t = L.as_device(tensor)
            self.tensor = t.permute(*axes).contiguous()
        self.verbose = verbose
        self.decomposed = False
        self.orthonormalized = None

    # ------------------------------------------------------------------ ops
    def __add__(self, mpo):
        """Direct sum then ``>> min_bond`` (mpo:78-112)."""
        min_bond = min(min(self.bond_shape), min(mpo.bond_shape))
        if self.decomposed and mpo.decomposed:
            s = MatrixProductOperator.from_sites(_ops.concat(self.sites, mpo.sites))
            return s >> min_bond if type(self).AUTO_ROUND else s
        raise Exception("Both Matrix Product Operator must be in canonical form (use .decompose()")

    def __matmul__(self, mp):
        """MPO x MPS (mpo:181-192) or MPO x MPO (mpo:278-289), then
        ``>> min_bond``."""
        min_bond = min(min(self.bond_shape), min(mp.bond_shape))
        auto = type(self).AUTO_ROUND
        if isinstance(mp, MatrixProductState):
            if MatrixProductOperator.MATMUL_MODE == "standard":
                s = MatrixProductState.lazy_product(self.sites, mp.sites, type(self).PRECISION)
                if auto and type(self).ROUNDING == "svd":
                    # fused product + round (the rounding this operator class asks for)
                    if min_bond >= min(s.bond_shape):
                        return s
                    out, _sp, _c, _d, _st = _ops.mpo_mps_round(self.sites, mp.sites, min_bond,
                                                               precision_code(type(self).PRECISION),
                                                               spectra=False)
                    return MatrixProductState.from_sites(out)
                return s >> min_bond if auto else s
            if MatrixProductOperator.MATMUL_MODE == "opti":
                # The reference's unfinished density-matrix mode (mpo:193-273):
                # left blocks of <WX|WX>, then from the right the dominant
                # eigenvectors of each bond's reduced density matrix, kept to
                # min_bond.  That is the Gram-form TT-SVD of the fused
                # product + round (the optimal truncation; "f64" computes the
                # same state by QR + SVD), in this class's PRECISION.
                s = MatrixProductState.lazy_product(self.sites, mp.sites, type(self).PRECISION)
                if min_bond >= min(s.bond_shape):
                    return s
                out, _sp, _c, _d, _st = _ops.mpo_mps_round(self.sites, mp.sites, min_bond,
                                                           precision_code(type(self).PRECISION), spectra=False)
                return MatrixProductState.from_sites(out)
            if MatrixProductOperator.MATMUL_MODE == "zip-up":
                # Zip-up (Stoudenmire & White 2010) to min_bond: the state is
                # first brought to right-orthonormal form (an exact FP64
                # TT-SVD at its own bonds), then W X is compressed site by
                # site from the left without forming the product
                xs = [L.as_device(x) for x in mp.sites]
                big = max(int(x.shape[0]) for x in xs) * max(int(x.shape[1]) for x in xs) + 1
                xr, _sp, _c, _d, _st = _ops.svd_round(xs, big, L.PREC_F64, spectra=False)
                out, _disc, _st2 = _ops.mpo_mps_zipup([L.as_device(w) for w in self.sites], xr, min_bond)
                return MatrixProductState.from_sites(out)
            return None
        if isinstance(mp, MatrixProductOperator):
            s = MatrixProductOperator.from_sites(_ops.contract_mpo_mpo(self.sites, mp.sites))
            return s >> min_bond if auto else s
        return None

    def __rshift__(self, dim: int):
        """mpo:327-331."""
        if isinstance(dim, int):
            return self.compress(dim, strict=True)
        raise Exception("dimension should be an integer")

    def __getitem__(self, key):
        """mpo:333-342."""
        key_inp, key_out = key[0], key[1]
        if len(key_inp) != self.sites_number:
            raise Exception("input indices do not match the number of sites")
        if len(key_out) != self.sites_number:
            raise Exception("output indices do not match the number of sites")
        return self.retrieve(key_inp, key_out)

    def __repr__(self) -> str:
        r = "<Matrix Product Operator> \n> Sites shape" + str(self.shape) + "\n"
        r += "\t" + "|   " * self.sites_number + "\n"
        r += "\t" + ("O---" * (self.sites_number - 1)) + "O" + "\n"
        r += "\t" + "|   " * self.sites_number + "\n"
        return r

    # --------------------------------------------------------- constructors
    @staticmethod
    def random(input_shape, output_shape, bond_shape):
        """mpo:352-355: dense N(0,1) draw from numpy's global RNG, decomposed on
        the device."""
        tensor = np.random.normal(size=(*input_shape, *output_shape))
        return MatrixProductOperator(tensor, bond_shape=bond_shape).decompose()

    @staticmethod
    def from_sites(sites, orthogonality=None, real_parameters_number=None):
        """mpo:357-380."""
        mp = MatrixProductOperator()
        mp.sites = [s if _is_dev(s) else L.as_device(s) for s in list(sites)]
        mp.sites_number = len(mp.sites)
        mp.decomposed = True
        mp.orthonormalized = orthogonality
        mp.parameters_number = int(sum(int(np.prod(s.shape)) for s in mp.sites))
        mp.real_parameters_number = real_parameters_number
        mp.input_shape, mp.output_shape, mp.bond_shape = (), (), ()
        mp.shape = [None] * mp.sites_number
        for idx, site in enumerate(mp.sites):
            shp = tuple(int(x) for x in site.shape)
            mp.shape[idx] = shp
            mp.input_shape += (shp[1],)
            mp.output_shape += (shp[2],)
            if idx != mp.sites_number - 1:
                mp.bond_shape += (shp[3],)
        return mp

    @staticmethod
    def empty():
        return MatrixProductOperator()

    @staticmethod
    def zeros(input_shape, output_shape, bond_shape):
        """mpo:386-400."""
        n = len(input_shape)
        if tuple(bond_shape) != ():
            shape = [(1, input_shape[0], output_shape[0], bond_shape[0])]
            shape += [(bond_shape[i - 1], input_shape[i], output_shape[i], bond_shape[i])
                      for i in range(1, n - 1)]
            shape += [(bond_shape[n - 2], input_shape[n - 1], output_shape[n - 1], 1)]
        else:
            shape = [(1, input_shape[0], output_shape[0], 1)]
        dev = L.device()
        return MatrixProductOperator.from_sites(
            [torch.zeros(s, dtype=torch.float64, device=dev) for s in shape])

    def copy(self):
        """mpo:402-403 (a new site list: the cores themselves are shared)."""
        return MatrixProductOperator.from_sites(list(self.sites))

    def to_tensor(self):
        """Dense ``(*in, *out)`` tensor (mpo:405-416), contracted on the device
        and copied to the host."""
        n = self.sites_number
        flat = _ops.to_tensor_device(self.sites).cpu().numpy()
        inter = []
        for i, o in zip(self.input_shape, self.output_shape):
            inter += [i, o]
        t = flat.reshape(inter)
        axes = list(range(0, 2 * n, 2)) + list(range(1, 2 * n, 2))
        return np.ascontiguousarray(np.transpose(t, axes))

    def decompose(self, mode="left"):
        """Truncated-QR sweep of the interleaved dense tensor (mpo:418-467).
        ``mode="right"`` decomposes from the left and reverses the site list,
        as the reference does (mpo:455-463)."""
        if self.bond_shape == ():
            self.sites = [self.tensor.reshape(1, self.tensor_shape[0], self.tensor_shape[1], 1)
                          .contiguous()]
            self.decomposed = True
            del self.tensor
        if not self.decomposed:
            n = self.sites_number
            phys = [self.shape[k][1] * self.shape[k][2] for k in range(n)]
            shapes3 = [(s[0], s[1] * s[2], s[3]) for s in self.shape]
            cores = _ops.decompose(self.tensor, phys, list(self.bond_shape), shapes3, 0)
            self.sites = [c.reshape(self.shape[k]) for k, c in enumerate(cores)]
            self.parameters_number += int(sum(int(np.prod(c.shape)) for c in cores))
            del self.tensor
            if mode == "right":
                self.sites = self.sites[::-1]
            self.decomposed = True
        return self

    def compress(self, dim, mode="left", strict=False):
        """Rounding to ``dim`` (mpo:469-580)."""
        if dim >= min(self.bond_shape):
            return self
        self.bond_shape = (dim,) * (self.sites_number - 1)
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
        that = self.copy()
        if mode == "left":
            new = self._round(that.sites, dim)
            that.sites = new
            that.shape = [tuple(int(x) for x in c.shape) for c in new]
            that.parameters_number = int(sum(int(np.prod(c.shape)) for c in new))
        return that

    def _round(self, cores, dim):
        flat = [c.reshape(c.shape[0], c.shape[1] * c.shape[2], c.shape[3]) for c in cores]
        if type(self).ROUNDING == "svd":
            out, _spec, _cnt, _disc, _st = _ops.svd_round(flat, dim, precision_code(type(self).PRECISION),
                                                          spectra=False)
        else:
            out = _ops.qr_truncate(flat, dim)
        return [o.reshape(o.shape[0], c.shape[1], c.shape[2], o.shape[2]) for o, c in zip(out, cores)]

    def retrieve(self, input_indices, output_indices):
        """One element (mpo:663-670)."""
        flat = [c.reshape(c.shape[0], c.shape[1] * c.shape[2], c.shape[3]) for c in self.sites]
        idx = [int(i) * int(c.shape[2]) + int(o)
               for i, o, c in zip(input_indices, output_indices, self.sites)]
        return np.float64(_ops.retrieve(flat, idx))

    def left_orthonormalization(self, bond_shape=()):
        """mpo:673-694."""
        if self.decomposed:
            flat = [c.view(c.shape[0], c.shape[1] * c.shape[2], c.shape[3]) for c in self.sites]
            _ops.left_orthonormalize(flat)
            self.orthonormalized = "left"
        else:
            raise Exception("Cannot orthonormalize an undecomposed MatrixProductOperator")
        return self

    def right_orthonormalization(self, bond_shape=()):
        """mpo:696-719."""
        if self.decomposed:
            flat = [c.view(c.shape[0], c.shape[1] * c.shape[2], c.shape[3]) for c in self.sites]
            _ops.right_orthonormalize(flat)
            self.orthonormalized = "right"
        else:
            raise Exception("Cannot orthonormalize an undecomposed MatrixProductOperator")
        return self

    # matricization helpers (mpo:721-769), as device views
    def left_site_matricization(self, index):
        return self.left_matricization(self.sites[index], index)

    def right_site_matricization(self, index):
        return self.right_matricization(self.sites[index], index)

    def left_matricization(self, matrix=None, index: int = 0):
        l, i, o, r = self.shape[index]
        if matrix is None:
            return self.sites[index].reshape(i * o * l, r)
        return matrix.reshape(i * o * l, -1)

    def right_matricization(self, matrix=None, index: int = 0):
        l, i, o, r = self.shape[index]
        if matrix is None:
            return self.sites[index].reshape(l, i * o * r)
        return matrix.reshape(-1, i * o * r)

    def tensoricization(self, matrix, index):
        return matrix.reshape(*self.shape[index])

    def left_orthogonality(self, index):
        """mpo:771-773."""
        c = self.sites[index]
        return _ops.orthogonality(c.reshape(c.shape[0], -1, c.shape[-1]), 0).cpu().numpy()

    def right_orthogonality(self, index):
        """mpo:775-777."""
        c = self.sites[index]
        return _ops.orthogonality(c.reshape(c.shape[0], -1, c.shape[-1]), 1).cpu().numpy()
