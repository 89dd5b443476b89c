"""Drop-in for ``syngular.tensor`` (tensor/__init__.py:1-2): MatrixProductState
and MatrixProductOperator with site cores on the GPU."""
from .matrix_product_operator import MatrixProductOperator
from .matrix_product_state import MatrixProductState

__all__ = ["MatrixProductState", "MatrixProductOperator"]
