"""syngular_gb300 -- GB300 (sm_103a) implementation of Syngular's matrix-product
hot path behind the same API (``syngular.tensor`` and ``syngular.mul``).

    import syngular_gb300 as syn
    from syngular_gb300.tensor import MatrixProductState, MatrixProductOperator

The arithmetic runs in ``lib/libsyngular_gb300.so`` (C ABI:
``include/syngular_gb300.h``); build it with ``syngular_gb300.build.build()``.
"""
from . import tensor
from .tensor.utils import mul

__all__ = ["tensor", "mul"]
__version__ = "0.1.0"
