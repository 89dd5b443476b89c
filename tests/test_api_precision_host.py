"""Host-side part of the precision policy (no GPU): names map to the library
codes, unknown names are rejected, and a lazy MPO x MPS product reports the
product's shapes without touching a device."""
import pytest
import torch


def test_precision_codes():
    from syngular_gb300 import _lib as L
    from syngular_gb300.tensor.matrix_product_state import precision_code

    assert precision_code("f64") == L.PREC_F64 == 0
    assert precision_code("bf16x6") == L.PREC_BF16X6 == 5
    assert precision_code("tf32x3") == L.PREC_TF32X3
    with pytest.raises(ValueError):
        precision_code("fp8")


def test_lazy_product_shapes_on_host():
    from syngular_gb300.tensor import MatrixProductState

    X = [torch.zeros(1, 2, 4), torch.zeros(4, 2, 4), torch.zeros(4, 2, 1)]
    W = [torch.zeros(1, 2, 3, 5), torch.zeros(5, 2, 3, 5), torch.zeros(5, 2, 3, 1)]
    P = MatrixProductState.lazy_product(W, X, "bf16x6")
    assert P.shape == [(1, 3, 20), (20, 3, 20), (20, 3, 1)]
    assert P.bond_shape == (20, 20) and P.input_shape == (3, 3, 3) and P.sites_number == 3
    assert P._sites is None and P.decomposed
