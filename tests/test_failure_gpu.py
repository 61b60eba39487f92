"""Failure detection on the GPU without a fault.

The staged passes give up a pipeline wait after a bounded number of polls,
record bit 0 in a status word and return; ``Grid.run`` reads the word and
raises.  ``fdtd_selftest_bounded_wait`` runs that same bounded wait on an
mbarrier that nothing arrives at: the wait must expire, the status word must
reach the host, and the context must stay usable for the next time step.
"""

import ctypes

import pytest
import torch

from helpers import rel_l2
from oracle import fdtd_oracle as fo

pytestmark = pytest.mark.gpu


def _selftest(lib, polls):
    st = ctypes.c_int32(-1)
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.fdtd_selftest_bounded_wait(polls, ctypes.byref(st), ctypes.c_void_p(stream)) == 0
    return st.value


def test_wait_on_nothing_expires_and_reports(fd):
    from fdtd_gb300 import _native

    lib = _native.load()
    assert _selftest(lib, 0) == 1
    assert _selftest(lib, 4096) == 1
    assert lib.fdtd_selftest_bounded_wait(16, None, None) == 1  # argument error


def test_context_usable_after_expired_waits(fd):
    from fdtd_gb300 import _native

    lib = _native.load()
    for _ in range(3):
        assert _selftest(lib, 1024) == 1
    fd.set_backend("gb300.float64")
    g = fd.Grid((12, 10, 16), grid_spacing=100e-9)
    g[6, 5, 8] = fd.PointSource(period=10)
    o = fo.Grid((12, 10, 16), grid_spacing=100e-9)
    o[6, 5, 8] = fo.PointSource(period=10)
    g.run(12, progress_bar=False)
    o.run(12)
    g._engine.check_status()
    assert rel_l2(g.E, o.E) <= 1e-12
