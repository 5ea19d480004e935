"""The device-allocator hook (phs_set_device_allocator) on the GPU: every buffer the library
needs comes from the caller's allocator -- here PyTorch's caching allocator, as a framework
that owns the device heap would route it -- the outputs equal the default allocator's bit
for bit, and destroying the handle hands every buffer back."""
import ctypes as C

import numpy as np
import pytest

from gpu_phs_gb300 import processes as P
from gpu_phs_gb300.philox import uniform_x

pytestmark = pytest.mark.gpu

ALLOC_FN = C.CFUNCTYPE(C.c_int, C.POINTER(C.c_void_p), C.c_size_t, C.c_void_p)
FREE_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p)


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _same(a, b):
    return all(bool((u == w).all()) for u, w in ((a.p, b.p), (a.factor, b.factor),
                                                  (a.volume, b.volume), (a.ok, b.ok)))


def test_library_buffers_from_the_callers_allocator(torch):
    from gpu_phs_gb300 import _lib
    from gpu_phs_gb300.api import PRECISION_F32X2, PhaseSpace
    lib = _lib.load()
    proc = P.tt()
    n = 300_000                      # above the autotuner's 2^18: its scratch is used too
    x = torch.from_numpy(uniform_x(41, n, proc.n_x)).cuda()
    refs = {}
    for prec in (0, 1):              # default allocator
        ps = PhaseSpace(proc, 500.0, 500.0)
        ps.set_precision(prec)
        refs[prec] = ps.generate(x)
        torch.cuda.synchronize()
        ps.close()

    pool, sizes, calls = {}, [], {"free": 0}

    @ALLOC_FN
    def alloc(ptr, nbytes, user):
        t = torch.empty(int(nbytes), dtype=torch.uint8, device="cuda")
        pool[t.data_ptr()] = t
        sizes.append(int(nbytes))
        ptr[0] = t.data_ptr()
        return 0

    @FREE_FN
    def free(ptr, user):
        pool.pop(ptr)
        calls["free"] += 1

    assert lib.phs_set_device_allocator(alloc, free, None) == 0
    try:
        for prec in (0, 1):
            ps = PhaseSpace(proc, 500.0, 500.0)
            ps.set_precision(prec)
            got = ps.generate(x)
            torch.cuda.synchronize()
            assert _same(got, refs[prec]), f"precision {prec}: outputs differ"
            # the host path's chunk buffers and streams, through the same allocator
            xh = x.cpu()
            host = ps.generate_host(xh)
            assert torch.equal(host.p, refs[prec].p.cpu()) and torch.equal(host.ok, refs[prec].ok.cpu())
            assert len(pool) > 0
            ps.close()
            assert not pool, f"{len(pool)} buffers not handed back"
        assert len(sizes) == calls["free"] and min(sizes) > 0
    finally:
        assert lib.phs_set_device_allocator(None, None, None) == 0
