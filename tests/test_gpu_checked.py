"""The bounds-checked build (libgpuphs_checked.so, -DPHS_CHECKED) on small cases of every
kernel family: each index the kernels compute from run-time data is checked against the
extent of its array before the access (gpu_phs_gb300/csrc/phs_check.h).  This is the
memory-safety check of the library on the GPU in place of compute-sanitizer, which is not
available on the GPU pool.

Every case runs through both libraries on the same inputs: the checked build must record
no out-of-range index (phs_check_status; every skipped access records its site) and give
the regular build's outputs -- bit for bit for the forward, inverse and grid kernels, and
within 1e-10 of each row's largest entry for the adjoint, whose file is compiled with FMA
contraction: the checks' branches change which multiply-adds the compiler fuses.  Cases: FP64 one pass, compacting and split forms and the FP32-pair one pass,
compacting and split forms (with their exact FP64 path) on tt, the 13 TeV tree, a batch
of random trees with more than 64 segments, Whizard's bwbw channels (friend boosts) with
uniform, boosted and per-event beams; the adjoint in both storage forms; the inverse map
(outgoing momenta from p, staged with a lab boost, per-event beams); the warm-up grid; the
no-allocation entry point.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden, load_process
from gpu_phs_gb300 import processes as P
from gpu_phs_gb300.philox import uniform_x

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def libs():
    from gpu_phs_gb300 import _lib
    reg, chk = _lib.load(), _lib.load_checked()
    assert reg.phs_is_checked_build() == 0 and chk.phs_is_checked_build() == 1
    w = C.c_uint64()
    assert reg.phs_check_status(C.byref(w), None) == -7       # PHS_ERR_UNSUPPORTED
    assert chk.phs_check_status(C.byref(w), None) == 0        # clears the words
    return reg, chk


def run_both(libs, torch, fn):
    """fn() under each library -> list of tensors; returns (regular, checked) and asserts
    the checked build recorded nothing."""
    from gpu_phs_gb300 import _lib
    reg, chk = libs
    outs = []
    for lib in (reg, chk):
        with _lib.using(lib):
            outs.append([t.clone() for t in fn()])
            torch.cuda.synchronize()
    w, first = C.c_uint64(), C.c_int64()
    assert chk.phs_check_status(C.byref(w), C.byref(first)) == 0, chk.phs_last_error()
    assert w.value == 0, f"checked build: sites {w.value:#x}, first index {first.value}"
    return outs


def assert_same(outs, what, rtol=0.0):
    """Bit for bit (rtol 0), or floating outputs within rtol of each row's largest entry."""
    a, b = outs
    for i, (u, v) in enumerate(zip(a, b)):
        assert u.shape == v.shape, f"{what}: output {i} shape"
        if rtol == 0.0 or not v.is_floating_point():
            assert bool((u == v).all()), f"{what}: output {i} differs"
            continue
        scale = v.abs().reshape(v.shape[0], -1).amax(dim=1).clamp(min=1e-300)
        rel = ((u - v).abs().reshape(v.shape[0], -1).amax(dim=1) / scale).max().item()
        assert rel <= rtol, f"{what}: output {i} differs by {rel:.2e} of its row scale"


def forward_forms(torch, proc, counts, n, E=(500.0, 500.0)):
    from gpu_phs_gb300.api import PhaseSpace
    x = torch.from_numpy(uniform_x(77, n, proc.n_x)).cuda()
    res = []
    for prec, variants in ((0, (-1, 0)), (0, (-1, 2)), (0, (-1, 6)), (0, (-1, 8)),
                           (1, (0, -1)), (1, (3, -1)), (1, (5, -1))):
        ps = PhaseSpace(proc, *E)
        ps.set_precision(prec)
        ps.set_variants(*variants)
        ev = ps.generate(x, counts)
        res += [ev.p, ev.factor, ev.volume, ev.ok]
        ps.close()
    return res


def test_forward_forms_tt(torch, libs):
    assert_same(run_both(libs, torch, lambda: forward_forms(torch, P.tt(), None, 20_003)), "tt")


def test_forward_forms_13tev(torch, libs):
    proc = P.precision()
    assert_same(run_both(libs, torch, lambda: forward_forms(torch, proc, None, 40_000)), "13 TeV")


def test_forward_forms_batch_of_random_trees(torch, libs):
    """150 channels of 3-8 outgoing particles (more than the 64 segments the kernel
    parameters hold), some channels empty, through the batch API."""
    from gpu_phs_gb300.api import Batch, PhaseSpace, philox_fill
    rng = np.random.default_rng(5)
    procs = [P.random_process(rng, int(rng.integers(3, 9)), 1, 1000.0) for _ in range(150)]
    counts = rng.integers(0, 300, 150).astype(np.int64)
    counts[::7] = 0

    def fn():
        spaces = [PhaseSpace(p, 500.0, 500.0) for p in procs]
        res = []
        for prec, variants in ((0, (-1, 0)), (0, (-1, 2)), (0, (-1, 6)), (1, (1, -1)),
                               (1, (5, -1))):
            b = Batch(spaces)
            b.set_precision(prec)
            b.set_variants(*variants)
            xo, _ = b.offsets(counts)
            x = torch.empty(int(xo[-1]), dtype=torch.float64, device="cuda")
            philox_fill(x, int(xo[-1]), 1, 9)
            res += list(b.generate(x, counts))
            b.close()
        for s in spaces:
            s.close()
        return res
    assert_same(run_both(libs, torch, fn), "batch")


def test_bwbw_friends_boosted_and_per_event_beams(torch, libs):
    proc = load_process(golden("whizard_bwbw"))
    rng = np.random.default_rng(6)
    counts = rng.integers(50, 400, proc.n_channels).astype(np.int64)
    n = int(counts.sum())
    assert_same(run_both(libs, torch, lambda: forward_forms(torch, proc, counts, n)), "bwbw")
    assert_same(run_both(libs, torch, lambda: forward_forms(torch, proc, counts, n, (600.0, 400.0))),
                "bwbw boosted")

    def per_event():
        from gpu_phs_gb300.api import PhaseSpace
        x = torch.from_numpy(uniform_x(78, n, proc.n_x)).cuda()
        g = torch.Generator(device="cuda").manual_seed(3)
        E1 = 300 + 400 * torch.rand(n, generator=g, device="cuda", dtype=torch.float64)
        E2 = 300 + 400 * torch.rand(n, generator=g, device="cuda", dtype=torch.float64)
        res = []
        for prec in (0, 1):
            ps = PhaseSpace(proc)
            ps.set_precision(prec)
            ev = ps.generate_beams(x, E1, E2, counts)
            res += [ev.p, ev.factor, ev.volume, ev.ok]
            ps.close()
        return res
    assert_same(run_both(libs, torch, per_event), "bwbw per-event beams")


def test_adjoint_both_storage_forms(torch, libs):
    from gpu_phs_gb300.api import ADJOINT_STORED, PhaseSpace
    bw = load_process(golden("whizard_bwbw"))
    friend = [c for c in range(bw.n_channels) if np.any(bw.friends[c] != 0)][0]
    for proc in (P.tt(), bw.subset([friend])):
        n = 10_000

        def fn():
            x = torch.from_numpy(uniform_x(79, n, proc.n_x)).cuda()
            g = torch.Generator(device="cuda").manual_seed(4)
            pbar = torch.randn((n, proc.n_out, 4), generator=g, device="cuda", dtype=torch.float64)
            jbar = torch.randn(n, generator=g, device="cuda", dtype=torch.float64)
            res = []
            for stored in (False, True):
                ps = PhaseSpace(proc, 500.0, 500.0)
                if stored:
                    ps.set_adjoint_storage(ADJOINT_STORED)
                res += list(ps.vjp(x, pbar, jbar))
                ps.close()
            return res
        assert_same(run_both(libs, torch, fn), f"adjoint {proc.name}", rtol=1e-10)


def test_inverse_map(torch, libs):
    from gpu_phs_gb300.api import PhaseSpace
    proc = load_process(golden("whizard_bwbw"))
    counts = np.full(proc.n_channels, 300, np.int64)
    n = int(counts.sum())
    for E in ((500.0, 500.0), (600.0, 400.0), None):
        def fn():
            x = torch.from_numpy(uniform_x(80, n, proc.n_x)).cuda()
            if E is None:
                g = torch.Generator(device="cuda").manual_seed(5)
                E1 = 300 + 400 * torch.rand(n, generator=g, device="cuda", dtype=torch.float64)
                E2 = 300 + 400 * torch.rand(n, generator=g, device="cuda", dtype=torch.float64)
                ps = PhaseSpace(proc)
                ev = ps.generate_beams(x, E1, E2, counts)
                fac, xo = ps.inverse(ev.p, counts, ev.ok, x, ev.factor, E1=E1, E2=E2)
            else:
                ps = PhaseSpace(proc, *E)
                ev = ps.generate(x, counts)
                fac, xo = ps.inverse(ev.p, counts, ev.ok, x, ev.factor)
            ps.close()
            return [fac, xo]
        assert_same(run_both(libs, torch, fn), f"inverse {E}")


def test_grid_and_noalloc(torch, libs):
    from gpu_phs_gb300 import _lib
    from gpu_phs_gb300.api import Grid, PhaseSpace, precondition
    proc = P.precision()
    counts = np.array([5000], np.int64)

    def grid():
        ps = PhaseSpace(proc, 6500.0, 6500.0)
        g = Grid(1, proc.n_x)
        precondition(ps, g, 3, 5000, seed=3)
        w = torch.from_numpy(g.weights())
        x = g.sample(5000, counts, seed=4)
        g.close()
        ps.close()
        return [w, x]
    assert_same(run_both(libs, torch, grid), "grid")

    def noalloc():
        lib = _lib.load()
        tt = P.tt()
        x = torch.from_numpy(uniform_x(81, 7000, tt.n_x)).cuda()
        ps = PhaseSpace(tt)
        out = ps.alloc(7000)
        rc = lib.phs_generate_device_noalloc(ps.h, 600.0, 400.0, 7000, None, x.data_ptr(),
                                             out.p.data_ptr(), out.factor.data_ptr(),
                                             out.volume.data_ptr(), out.ok.data_ptr(), None)
        assert rc == 0, lib.phs_last_error()
        torch.cuda.synchronize()
        ps.close()
        return [out.p, out.factor, out.volume, out.ok]
    assert_same(run_both(libs, torch, noalloc), "noalloc")
