"""API misuse raises the reference's own exceptions with its own messages
(bare ``Exception``), before any device work, so these run on the host.
Messages: tensor/matrix_product_state.py:51, 102, 129, 143, 159,
tensor/matrix_product_operator.py:44, 112, 331, 338, 340, 693, 717 and
tensor/utils.py:16, 32, 46, 73."""
import numpy as np
import pytest

from syngular_gb300.tensor import MatrixProductOperator, MatrixProductState


def raises_exactly(msg, fn):
    with pytest.raises(Exception) as e:
        fn()
    assert type(e.value) is Exception and str(e.value) == msg


def test_mps_messages():
    raises_exactly("dimensions of bond indices do not match order - 1",
                   lambda: MatrixProductState(np.zeros((2, 2, 2)), (2,)))
    X = MatrixProductState(np.zeros((2, 2)), (2,))  # not decomposed
    raises_exactly("Both Matrix Product Operator must be in canonical form (use .decompose()", lambda: X + X)
    raises_exactly("right-hand site must be a MatrixProductState", lambda: X | 3)
    raises_exactly("dimension should be an integer", lambda: X >> 2.5)
    raises_exactly("dimension should be an integer", lambda: X >> "4")
    raises_exactly("input indices do not match the number of sites", lambda: X[(0,)])


def test_mpo_messages():
    raises_exactly("input_shape and output_shape of the tensor must have the same length",
                   lambda: MatrixProductOperator(np.zeros((2, 2, 2)), ()))
    W = MatrixProductOperator()
    W.sites_number = 2
    W.bond_shape = (2,)
    raises_exactly("Both Matrix Product Operator must be in canonical form (use .decompose()", lambda: W + W)
    raises_exactly("dimension should be an integer", lambda: W >> 1.0)
    raises_exactly("input indices do not match the number of sites", lambda: W[(0,), (0, 0)])
    raises_exactly("output indices do not match the number of sites", lambda: W[(0, 0), (0,)])
    raises_exactly("Cannot orthonormalize an undecomposed MatrixProductOperator", W.left_orthonormalization)
    raises_exactly("Cannot orthonormalize an undecomposed MatrixProductOperator", W.right_orthonormalization)


def test_mul_messages():
    from syngular_gb300.tensor.utils import mul

    X = MatrixProductState(np.zeros((2, 2)), (2,))
    X3 = MatrixProductState(np.zeros((2, 2, 2)), (2, 2))
    W = MatrixProductOperator()
    W.sites_number, W.bond_shape, W.decomposed = 2, (2,), False

    class Other:
        sites_number, bond_shape = 2, (2,)

    raises_exactly("both operator do not have the same number of sites", lambda: mul(X, X3))
    raises_exactly("Operators and States must be decomposed", lambda: mul(X, W))
    raises_exactly("Operators and States must be decomposed", lambda: mul(W, X))
    raises_exactly("`syn.mul` should be provided MatrixProductState or MatrixProductOperator objects only",
                   lambda: mul(X, Other()))
    assert mul(X, W, mode="variational") is None
