"""phs_generate_device_noalloc: forward generation for callers that cannot allocate device
memory (a host program that owns the device heap through its own allocator, or a plug-in
host that denies cudaMalloc).  It keeps the channel programs and the event segments in
the library's static device array instead of allocating buffers.

Each check calls it twice in a row through the C ABI and compares with the regular entry
point phs_generate_device; both run the same kernel on the same programs, so the outputs
must agree bit for bit (inside the parity bar the other GPU tests use).  This file is
collected last so that a failure here cannot hide the other tests' results.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import counts_of, golden, load_process
from gpu_phs_gb300 import processes as P
from gpu_phs_gb300.philox import uniform_x

pytestmark = pytest.mark.gpu

PHS_ERR_UNSUPPORTED = -7


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _noalloc(lib, ps, E, x, counts, out, torch, E2=None):
    c = None if counts is None else np.ascontiguousarray(counts, np.int64)
    rc = lib.phs_generate_device_noalloc(
        ps.h, E, E if E2 is None else E2, x.shape[0], None if c is None else c.ctypes.data,
        x.data_ptr(), out.p.data_ptr(), out.factor.data_ptr(), out.volume.data_ptr(),
        out.ok.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.phs_last_error().decode()


def _cases():
    rng = np.random.default_rng(8)
    bw = golden("whizard_bwbw")
    many = P.random_process(rng, 5, 150, 1000.0)       # > 64 channels: device segment table
    return [
        (P.tt(), 500.0, None, 100_003),
        (load_process(bw), 500.0, rng.integers(0, 90, 61).astype(np.int64), None),
        (many, 500.0, rng.integers(1, 40, 150).astype(np.int64), None),
    ]


def _same(a, b):
    return all(bool((u == w).all()) for u, w in ((a.p, b.p), (a.factor, b.factor),
                                                  (a.volume, b.volume), (a.ok, b.ok)))


def test_noalloc_matches_regular_entry_point(torch):
    from gpu_phs_gb300 import _lib
    from gpu_phs_gb300.api import PhaseSpace
    lib = _lib.load()
    runs = []
    for proc, E, counts, n in _cases():
        n = int(counts.sum()) if counts is not None else n
        x = torch.from_numpy(uniform_x(31, n, proc.n_x)).cuda()
        ps = PhaseSpace(proc, E, E)
        ref = ps.generate(x, counts)
        runs.append((ps, E, counts, x, ref))
    # two calls in a row per process, interleaved across processes so that each call
    # must fully replace what the previous one left in the shared scratch array
    for rep in range(2):
        for ps, E, counts, x, ref in runs:
            out = ps.alloc(x.shape[0])
            _noalloc(lib, ps, E, x, counts, out, torch)
            torch.cuda.synchronize()
            assert _same(out, ref), f"call {rep + 1} differs from phs_generate_device"


def test_noalloc_allocates_no_device_memory(torch):
    from gpu_phs_gb300 import _lib
    from gpu_phs_gb300.api import PhaseSpace
    lib = _lib.load()
    proc = P.tt()
    x = torch.from_numpy(uniform_x(32, 50_000, proc.n_x)).cuda()
    ps = PhaseSpace(proc)                  # no set_beams: the no-alloc call needs none
    outs = [ps.alloc(x.shape[0]) for _ in range(3)]
    _noalloc(lib, ps, 500.0, x, None, outs[0], torch)   # first call: resolves the scratch address
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    _noalloc(lib, ps, 500.0, x, None, outs[1], torch)
    _noalloc(lib, ps, 500.0, x, None, outs[2], torch)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert _same(outs[1], outs[0]) and _same(outs[2], outs[0])


def test_noalloc_unequal_beams_match_set_beams(torch):
    """E1 != E2: the call compiles the constants at sqrt(s) = 2 sqrt(E1 E2) and the lab boost
    itself; two calls in a row equal set_beams(E1, E2) + phs_generate_device bit for bit."""
    from gpu_phs_gb300 import _lib
    from gpu_phs_gb300.api import PhaseSpace
    lib = _lib.load()
    for proc, n in ((P.tt(), 100_003), (P.ww(), 40_000)):
        x = torch.from_numpy(uniform_x(33, n, proc.n_x)).cuda()
        ref = PhaseSpace(proc, 600.0, 400.0).generate(x)
        ps = PhaseSpace(proc)
        for rep in range(2):
            out = ps.alloc(n)
            _noalloc(lib, ps, 600.0, x, None, out, torch, E2=400.0)
            torch.cuda.synchronize()
            assert _same(out, ref), f"{proc.name}: call {rep + 1} differs from phs_generate_device"
        # the lab boost moved the momenta: the unboosted run differs
        sym = PhaseSpace(proc, 500.0, 500.0).generate(x)
        assert not torch.equal(sym.p, ref.p)


def test_noalloc_refuses_a_capturing_stream(torch):
    """Its uploads read host memory that is gone when the call returns, so a call on a
    stream under capture is refused before it enqueues anything; the next plain call works."""
    from gpu_phs_gb300 import _lib
    from gpu_phs_gb300.api import PhaseSpace
    lib = _lib.load()
    proc = P.tt()
    n = 4096
    x = torch.from_numpy(uniform_x(34, n, proc.n_x)).cuda()
    ps = PhaseSpace(proc)
    out = ps.alloc(n)
    _noalloc(lib, ps, 500.0, x, None, out, torch)      # set-up outside capture
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    rc = None
    with torch.cuda.graph(g, stream=s):
        rc = lib.phs_generate_device_noalloc(
            ps.h, 500.0, 500.0, n, None, x.data_ptr(), out.p.data_ptr(), out.factor.data_ptr(),
            out.volume.data_ptr(), out.ok.data_ptr(), s.cuda_stream)
        msg = lib.phs_last_error().decode()
    assert rc == PHS_ERR_UNSUPPORTED
    assert "captured" in msg
    del g
    again = ps.alloc(n)
    _noalloc(lib, ps, 500.0, x, None, again, torch)
    torch.cuda.synchronize()
    assert _same(again, out)


def test_noalloc_rejects_more_channels_than_its_scratch_holds(torch):
    from gpu_phs_gb300 import _lib
    from gpu_phs_gb300.api import PhaseSpace
    lib = _lib.load()
    proc = P.random_process(np.random.default_rng(9), 3, 257, 1000.0)
    ps = PhaseSpace(proc)
    x = torch.zeros((257, proc.n_x), dtype=torch.float64, device="cuda")
    out = ps.alloc(257)
    counts = np.ones(257, np.int64)
    rc = lib.phs_generate_device_noalloc(ps.h, 500.0, 500.0, 257, counts.ctypes.data,
                                         x.data_ptr(), out.p.data_ptr(), out.factor.data_ptr(),
                                         out.volume.data_ptr(), out.ok.data_ptr(), None)
    assert rc == PHS_ERR_UNSUPPORTED
    assert "at most 256 channels" in lib.phs_last_error().decode()
