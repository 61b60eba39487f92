"""Compact material copies for the staged passes (host side, no GPU).

``compact_material`` turns an inverse-material array into a table of its
distinct value triples and a one-byte index per cell, or one triple for a
uniform material; the staged kernels then read the index (or nothing) instead
of three values per cell.  The table must reproduce every cell bit for bit.
"""

import numpy as np
import pytest
import torch

from fdtd_gb300.engine import compact_material


def _expand(enc, shape):
    table, index = enc
    if index is None:
        return table[0].expand(shape)
    return table[index.long()]


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_round_trip_few_triples(dtype):
    rng = np.random.default_rng(3)
    levels = rng.uniform(0.2, 1.0, size=(7, 3))
    pick = rng.integers(0, 7, size=(9, 10, 16))
    x = torch.tensor(levels[pick], dtype=dtype)
    x[2:4, 1:3, :] = 0.0  # cells inside objects
    x[0, 0, 0, 1] = -0.0
    table, index = compact_material(x, chunk=97)
    assert index.dtype == torch.uint8 and index.shape == (9, 10, 16)
    assert table.dtype == dtype and table.shape[1] == 3 and table.shape[0] <= 256
    assert torch.unique(index).numel() <= 9
    back = _expand((table, index), x.shape)
    itype = torch.int32 if dtype == torch.float32 else torch.int64
    assert torch.equal(back.view(itype), x.view(itype))  # bit patterns, -0.0 included


def test_uniform():
    x = torch.full((4, 5, 16, 3), 0.25, dtype=torch.float32)
    table, index = compact_material(x)
    assert index is None and table.shape == (1, 3) and torch.all(table == 0.25)


def test_signed_zero_is_its_own_row():
    x = torch.zeros((2, 2, 16, 3), dtype=torch.float64)
    x[1, 1, 3, 2] = -0.0
    table, index = compact_material(x)
    assert index is not None and table.shape[0] == 2
    back = table[index.long()]
    assert torch.equal(back.view(torch.int64), x.view(torch.int64))


def test_too_many_triples():
    x = torch.rand((8, 8, 16, 3), dtype=torch.float32)
    assert compact_material(x) is None
    # every component has few values but their combinations exceed 256
    rng = np.random.default_rng(0)
    y = torch.tensor(rng.integers(0, 9, size=(16, 16, 16, 3)).astype(np.float32))
    assert compact_material(y, chunk=1000) is None


def test_table_limit_exact():
    v = torch.arange(256, dtype=torch.float32)
    x = torch.stack([v, v * 2, v * 3], dim=1).reshape(4, 4, 16, 3)
    table, index = compact_material(x)
    assert table.shape == (256, 3) and int(index.max()) == 255
    assert torch.equal(table[index.long()], x)


def test_index_not_allowed():
    x = torch.zeros((2, 2, 8, 3), dtype=torch.float32)
    assert compact_material(x, index_ok=False)[1] is None
    x[0, 0, 0, 0] = 1.0
    assert compact_material(x, index_ok=False) is None


def test_values_the_sample_misses():
    """A value present in only a few cells (missed by the strided sample)
    still gets its own table row."""
    x = torch.full((64, 64, 32, 3), 0.5, dtype=torch.float32)
    x[::2] = 0.25
    x[17, 33, 5, 1] = 0.125
    x[63, 63, 31, 2] = -0.0
    table, index = compact_material(x, chunk=5000)
    assert torch.equal(table[index.long()].view(torch.int32), x.view(torch.int32))
    assert torch.unique(index).numel() == 4


def test_every_combination_table():
    """Few values per component: the table lists every combination of them
    (here 2 x 2 x 1) and the index is the combination's number."""
    x = torch.zeros((4, 4, 16, 3), dtype=torch.float32)
    x[..., 0] = 1.0
    x[:2, ..., 0] = 2.0
    x[:, :2, :, 1] = 5.0
    table, index = compact_material(x)
    assert table.shape == (4, 3)
    assert torch.equal(table[index.long()], x)
