"""``syngular.mul`` (tensor/utils.py:8-99): standard-mode products of MPS / MPO
objects through the device site contractions, each ending with
``>> min_bond`` as in the reference."""
from __future__ import annotations

from . import _ops
from .matrix_product_operator import MatrixProductOperator
from .matrix_product_state import MatrixProductState


def mul(op1, op2, mode="standard"):
    n = op1.sites_number
    m = op2.sites_number
    min_bond = min(min(op1.bond_shape), min(op2.bond_shape))
    if n != m:
        raise Exception("both operator do not have the same number of sites")
    if mode != "standard":
        return None  # the other modes are empty in the reference (utils.py:82-99)
    if isinstance(op1, MatrixProductState) and isinstance(op2, MatrixProductOperator):
        if not op1.decomposed or not op2.decomposed:
            raise Exception("Operators and States must be decomposed")
        return MatrixProductState.from_sites(_ops.contract_mpo_mps(op2.sites, op1.sites)) >> min_bond
    if isinstance(op1, MatrixProductOperator) and isinstance(op2, MatrixProductState):
        if not op1.decomposed or not op2.decomposed:
            raise Exception("Operators and States must be decomposed")
        return MatrixProductState.from_sites(_ops.contract_mpo_mps(op1.sites, op2.sites)) >> min_bond
    if isinstance(op1, MatrixProductState) and isinstance(op2, MatrixProductState):
        return op1 | op2
    if isinstance(op1, MatrixProductOperator) and isinstance(op2, MatrixProductOperator):
        # utils.py:61-71 contracts op2's output leg with op1's input leg, op2-major bond
        return MatrixProductOperator.from_sites(_ops.contract_mpo_mpo(op2.sites, op1.sites)) >> min_bond
    raise Exception("`syn.mul` should be provided MatrixProductState or MatrixProductOperator objects only")
