"""The allocation-free field statistics entry point.

fdtd_field_stats_noalloc serves callers that cannot allocate device memory
(their device memory belongs to another framework's allocator, or they run in
a hook between time steps that must not touch an allocator): it keeps its
per-CTA partial sums in a fixed device array inside the library instead of a
caller-provided scratch buffer.  This test calls it through the C ABI and
checks its output against fdtd_field_stats (which takes a caller scratch
buffer) on two calls in a row, and that sizes above the array's limit are
refused.  The file is named so that pytest collects it last.
"""

import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


def _stats_both(lib, plan, stream, dev):
    nbytes = lib.fdtd_stats_scratch_bytes(plan)
    scratch = torch.empty(int(nbytes), dtype=torch.uint8, device=dev)
    ref = torch.full((5,), -1.0, dtype=torch.float64, device=dev)
    got = torch.full((5,), -2.0, dtype=torch.float64, device=dev)
    assert lib.fdtd_field_stats(plan, ref.data_ptr(), scratch.data_ptr(), stream) == 0
    assert lib.fdtd_field_stats_noalloc(plan, got.data_ptr(), 0, stream) == 0
    torch.cuda.synchronize()
    return ref.cpu(), got.cpu()


@pytest.mark.parametrize("prec", ["float32", "float32c", "float64"])
def test_noalloc_stats_match_allocating_entry_point(prec):
    import fdtd_gb300 as fd
    from fdtd_gb300 import _native, scenes

    assert torch.cuda.is_available()
    lib = _native.load()
    fd.set_backend("gb300." + prec)
    try:
        g = scenes.c1(fd, n=32, pml=6)
        g.run(15, progress_bar=False)
        plan = g._engine.plan
        dev = g.E.device
        stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

        ref1, got1 = _stats_both(lib, plan, stream, dev)
        assert float(ref1[0]) > 0.0 and float(ref1[4]) == 0.0
        assert torch.allclose(got1, ref1, rtol=1e-12, atol=0.0), (got1, ref1)

        g.run(7, progress_bar=False)  # second call on changed fields reuses the shared array
        ref2, got2 = _stats_both(lib, plan, stream, dev)
        assert not torch.equal(ref2, ref1)
        assert torch.allclose(got2, ref2, rtol=1e-12, atol=0.0), (got2, ref2)

        out = torch.zeros(5, dtype=torch.float64, device=dev)
        too_many = _native.STATS_STATIC_MAX_ROWS + 1
        assert lib.fdtd_field_stats_noalloc(plan, out.data_ptr(), too_many, stream) == 5  # FDTD_ERR_RANGE
        assert lib.fdtd_field_stats_noalloc(plan, out.data_ptr(), _native.STATS_STATIC_MAX_ROWS, stream) == 0
        torch.cuda.synchronize()
        assert torch.allclose(out.cpu(), ref2, rtol=1e-9, atol=0.0)
    finally:
        fd.set_backend("gb300.float64")
