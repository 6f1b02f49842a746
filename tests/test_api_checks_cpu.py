"""Argument checks of the Python mirror (no GPU): operands the C ABI would
read or write past their end are refused in Python with TypeError /
ValueError before any pointer reaches the library."""
import numpy as np
import pytest
import torch

from conftest import pkg


@pytest.fixture(scope="module")
def api():
    return pkg("api")


def test_device_entries_refuse_host_tensors(api):
    A = torch.zeros((2, 3, 4), dtype=torch.float64)
    B = torch.zeros((3, 5, 4), dtype=torch.float64)
    for call in (lambda: api.gemm(A, B), lambda: api.gemm_ex(A, B),
                 lambda: api.gemm_batched([(A, B)]), lambda: api.slice_conv(A, B),
                 lambda: api.scale_exponents(A, B),
                 lambda: api.plane_conv(A, torch.zeros((2, 3, 5), dtype=torch.float64))):
        with pytest.raises(TypeError, match="CUDA tensor"):
            call()


def test_operand_checks(api):
    A = torch.zeros((2, 3, 4), dtype=torch.float64)
    with pytest.raises(TypeError, match="CUDA tensor"):
        api._device_pd(A, "A")
    with pytest.raises(TypeError, match="CUDA tensor"):
        api._device_pd(np.zeros((2, 3, 4)), "A")


def test_host_entry_shapes(api):
    A = np.zeros((2, 3, 4))
    with pytest.raises(ValueError, match="do not chain"):
        api.gemm_host(A, np.zeros((4, 5, 4)))  # k 3 vs 4
    with pytest.raises(ValueError, match="do not chain"):
        api.gemm_host(A, np.zeros((3, 5, 2)))  # P 4 vs 2
    with pytest.raises(ValueError, match=r"\(rows, cols, P\)"):
        api.gemm_host(A.reshape(6, 4), np.zeros((3, 5, 4)))


def test_leading_dimension_of_views(api):
    base = torch.zeros((6, 10, 4), dtype=torch.float64)
    assert api._ld(base, 4) == 10
    assert api._ld(base[:, :7], 4) == 10  # padded rows: the row stride
    assert api._ld(base[:1, :7], 4) == 7
    with pytest.raises(ValueError, match="not dense"):
        api._ld(base[:, ::2], 4)  # entries of a row are not adjacent
    with pytest.raises(ValueError, match="not dense"):
        api._ld(base[:, :, :2], 2)  # limbs of an entry are not the whole row step
    with pytest.raises(ValueError, match="not dense"):
        api._ld(torch.zeros((1, 10, 4), dtype=torch.float64).expand(6, 10, 4), 4)  # rows alias
