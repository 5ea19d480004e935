"""Parity of the CUDA inverse map (phs_inverse_device) with the oracle's inverse and with
Whizard's all_factors, its round trip through the forward map, and the Whizard ABI's
all-channel outputs.

Bar (FP64).  The kernel keeps the oracle's (the reference's) operation order and is
compiled without contraction, except that it divides by a few constants (2 pi for x_phi,
m w and a1 - a0 in the Breit-Wigner inverse) as products with their reciprocals, so the
two differ through the ulps of the transcendental functions (CUDA's vs glibc's atan2, sin,
cos, log, atan) and of those products.  The reference's
algorithm amplifies such ulps on some elements: near the poles of a decay (1 - cos(theta)
cancels in the collinear map), for light combinations (msq = E^2 - |p|^2 cancels), and
through boosts of rounded rotations (a one-ulp change of one sin(phi) in the reference's
own arithmetic moves a factor by 6e-11 on one of these events).  So:
  * element-wise: |d factor| <= 1e-9 |factor| and |d x| <= 1e-9, each plus 64 times the
    oracle's own change under one-ulp perturbations of its input momenta (with per-event
    beams also of its transcendental values, assert_inverse_parity); inf and NaN (the
    reference's maps outside their domains) in the same places;
  * in distribution: median relative factor difference below 1e-14, 99th percentile
    below 1e-12 (not over four decades of beam energy: there the per-event constants'
    ulps move more than 1 % of the factors, test_inverse_per_event_beams_wide_energy_range);
  * against the truth: on the generating channel (whose x and factor are known), the GPU's
    round-trip error is at most that of the oracle (x4, plus 1e-15)."""
import ctypes as C

import numpy as np
import pytest

from conftest import all_maps_process, counts_of, golden, load_process, wide_beams
from gpu_phs_gb300 import processes as P
from gpu_phs_gb300.philox import uniform_x
from oracle import oracle

pytestmark = pytest.mark.gpu


def assert_inverse_parity(o, fac, xo, p, ch, ok, x_own=None, factor_own=None, E1=None, E2=None,
                          q99=1e-12):
    """GPU (fac, xo) against the oracle's inverse of the same momenta p.  The reference's
    inverse maps return inf or NaN outside their domains (a step map's logarithm of zero, a
    square root of a negative): those entries must be non-finite in the same places and
    with the same signs; the finite ones meet the bar of the module docstring.  With
    per-event beams the sensitivity also covers every transcendental value on the mapping
    path moved by one and two ulps (Oracle.inverse(nudge=...)): the device forms the
    per-event constants (a Breit-Wigner map's bound a1 = atan(u)) with its own library.
    q99: the bar on the 99th percentile of the relative factor difference (None: none)."""
    kw = dict(x_own=x_own, factor_own=factor_own, n_x=xo.shape[2], E1=E1, E2=E2)
    rf, rx = o.inverse(p, ch, ok, **kw)
    for g, r, name in ((fac, rf, "factor"), (xo, rx, "x")):
        for test in (np.isnan, np.isposinf, np.isneginf):
            assert np.array_equal(test(g), test(r)), f"{name}: non-finite entries differ"
    rng = np.random.default_rng(1)
    sf = np.zeros_like(rf)
    sx = np.zeros_like(rx)
    runs = [dict(p=p * (1 + rng.choice([-1.0, 1.0], p.shape) * 2.0 ** -52)) for _ in range(2)]
    if E1 is not None:
        runs += [dict(p=p, nudge=k * sign) for k in (1, 2) for sign in (1, -1)]
    with np.errstate(invalid="ignore"):
        for run in runs:
            pf, px = o.inverse(run.pop("p"), ch, ok, **kw, **run)
            sf = np.maximum(sf, np.where(np.isfinite(pf) & np.isfinite(rf), np.abs(pf - rf), np.inf))
            sx = np.maximum(sx, np.where(np.isfinite(px) & np.isfinite(rx), np.abs(px - rx), np.inf))
    finite_f, finite_x = np.isfinite(rf), np.isfinite(rx)
    df = np.where(finite_f, np.abs(fac - np.where(finite_f, rf, 0.0)), 0.0)
    dx = np.where(finite_x, np.abs(xo - np.where(finite_x, rx, 0.0)), 0.0)
    bf = 1e-9 * np.abs(np.where(finite_f, rf, 0.0)) + 64 * sf
    bx = 1e-9 + 64 * sx
    assert np.all(df <= bf), f"factor: {np.max(df / (bf + 1e-300)):.3g} x the bound"
    assert np.all(dx <= bx), f"x: {np.max(dx / bx):.3g} x the bound"
    live = np.broadcast_to(np.asarray(ok, bool)[:, None], fac.shape) & finite_f & (rf != 0)
    rel = (df / np.maximum(np.abs(np.where(finite_f, rf, 1.0)), 1e-300))[live]
    assert np.median(rel) < 1e-14
    if q99 is not None:
        assert np.quantile(rel, 0.99) < q99
    return rf, rx


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def gpu_forward_inverse(torch, proc, x, counts, E=(500.0, 500.0), own=True, Eev=None):
    from gpu_phs_gb300.api import PhaseSpace
    ps = PhaseSpace(proc, *E)
    xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    if Eev is None:
        ev = ps.generate(xd, counts)
        E1 = E2 = None
    else:
        E1 = torch.from_numpy(Eev[0]).cuda()
        E2 = torch.from_numpy(Eev[1]).cuda()
        ev = ps.generate_beams(xd, E1, E2, counts)
    fac, xo = ps.inverse(ev.p, counts, ev.ok, xd if own else None, ev.factor if own else None,
                         E1, E2)
    torch.cuda.synchronize()
    return (ev.p.cpu().numpy(), ev.factor.cpu().numpy(), ev.ok.cpu().numpy(),
            fac.cpu().numpy(), xo.cpu().numpy())


@pytest.mark.parametrize("name", ["ttH", "bwbw"])
def test_inverse_vs_oracle_and_whizard(torch, name):
    z = golden(f"whizard_{name}")
    proc = load_process(z)
    counts = counts_of(z["channel"], proc.n_channels)
    p, f, ok, fac, xo = gpu_forward_inverse(torch, proc, z["x"], counts)
    o = oracle.Oracle(proc, 1000.0)
    assert_inverse_parity(o, fac, xo, p, z["channel"], ok, x_own=z["x"], factor_own=f)
    n = len(z["channel"])
    assert np.array_equal(xo[z["channel"], np.arange(n)], z["x"])
    g = z["all_factors"]
    dec = 4 if name == "ttH" else 7
    assert np.all(np.abs(fac - g) <= 0.5 * 10.0 ** -dec + 2e-3 * np.abs(g))


@pytest.mark.parametrize("builder", [P.ww, P.tt, P.precision])
def test_round_trip(torch, builder):
    proc = builder()
    n = 100_003
    x = uniform_x(404, n, proc.n_x)
    p, f, ok, fac, xo = gpu_forward_inverse(torch, proc, x, None, E=(proc.sqrts / 2,) * 2,
                                            own=False)
    okb = ok == 1
    nu = 3 * proc.n_out - 4
    dx = np.abs(xo[0][okb, :nu] - x[okb, :nu])
    assert np.median(dx) < 1e-13 and dx.max() < 1e-6
    rel = np.abs(fac[okb, 0] / f[okb] - 1)
    assert np.median(rel) < 1e-11 and rel.max() < 1e-5
    assert np.all(fac[~okb] == 0) and np.all(xo[0][~okb, :nu] == 0)
    # against the oracle's inverse of the same momenta
    sl = slice(0, 20000)
    assert_inverse_parity(oracle.Oracle(proc, proc.sqrts), fac[sl], xo[:, sl], p[sl], None,
                          ok[sl])


@pytest.mark.parametrize("builder", [P.tt, P.precision])
def test_round_trip_at_least_as_accurate_as_oracle(torch, builder):
    """Against the known truth (the generating channel's x and forward factor): the GPU's
    inverse errs no more than the oracle's."""
    proc = builder()
    n = 50_000
    x = uniform_x(505, n, proc.n_x)
    p, f, ok, fac, xo = gpu_forward_inverse(torch, proc, x, None, E=(proc.sqrts / 2,) * 2,
                                            own=False)
    okb = ok == 1
    nu = 3 * proc.n_out - 4
    rf, rx = oracle.Oracle(proc, proc.sqrts).inverse(p, None, ok, n_x=proc.n_x)
    err_gpu = np.abs(xo[0][okb, :nu] - x[okb, :nu])
    err_ora = np.abs(rx[0][okb, :nu] - x[okb, :nu])
    assert err_gpu.max() <= 4 * err_ora.max() + 1e-15
    assert np.quantile(err_gpu, 0.999) <= 4 * np.quantile(err_ora, 0.999) + 1e-15
    ferr_gpu = np.abs(fac[okb, 0] / f[okb] - 1)
    ferr_ora = np.abs(rf[okb, 0] / f[okb] - 1)
    assert ferr_gpu.max() <= 4 * ferr_ora.max() + 1e-15
    assert np.quantile(ferr_gpu, 0.999) <= 4 * np.quantile(ferr_ora, 0.999) + 1e-15


def test_round_trip_random_trees_and_lab_frame(torch):
    rng = np.random.default_rng(12)
    for n_out in range(3, 9):
        proc = P.random_process(rng, n_out, 5, 1000.0, name=f"inv{n_out}")
        n = 20000
        counts = np.full(proc.n_channels, n // proc.n_channels, np.int64)
        counts[0] += n - counts.sum()
        x = uniform_x(50 + n_out, n, proc.n_x)
        E1 = np.full(n, 600.0)
        E2 = np.linspace(300.0, 700.0, n)
        p, f, ok, fac, xo = gpu_forward_inverse(torch, proc, x, counts, own=False, Eev=(E1, E2))
        ch = np.repeat(np.arange(proc.n_channels), counts)
        okb = ok == 1
        nu = 3 * n_out - 4
        own = xo[ch, np.arange(n)]
        assert np.median(np.abs(own[okb, :nu] - x[okb, :nu])) < 1e-12
        ownf = fac[np.arange(n), ch]
        assert np.median(np.abs(ownf[okb] / f[okb] - 1)) < 1e-11
        assert_inverse_parity(oracle.Oracle(proc, 1000.0), fac, xo, p, ch.astype(np.int32), ok,
                              E1=E1, E2=E2)


@pytest.mark.parametrize("case", ["ww", "tt", "all_maps_5", "all_maps_7"])
def test_inverse_per_event_beams_wide_energy_range(torch, case):
    """All-channel inverse of forward events with beam energies log-uniform in
    [1e-4, 0.7] sqrt(s) each (wide_beams): Breit-Wigner ranges below the pole, whose bounds
    the device forms per event, lab boosts up to gamma ~ 40, every mapping kind (random
    channels of all_maps_process).  Against the oracle's inverse of the same momenta at the
    inverse's element-wise bar (assert_inverse_parity) and median, and each event's own
    channel gives back its x.  No bar on the 99th percentile: at these energies more than
    1 % of the factors sit on Breit-Wigner ranges far below the pole, where the device's
    per-event bound a1, one ulp from glibc's, moves a factor by up to 1e-8 (the oracle's
    own factor moves as much when its a1 moves by an ulp, which the element-wise bar
    measures)."""
    if case in ("ww", "tt"):
        proc = getattr(P, case)()
        counts = None
        n = 50_000
    else:
        proc = all_maps_process(300 + int(case[-1]), int(case[-1]), 6)
        n = 30_000
        counts = np.full(proc.n_channels, n // proc.n_channels, np.int64)
    x = uniform_x(606, n, proc.n_x)
    E1, E2 = wide_beams(n, proc.sqrts, 11)
    p, f, ok, fac, xo = gpu_forward_inverse(torch, proc, x, counts, own=False, Eev=(E1, E2))
    ch = (np.repeat(np.arange(proc.n_channels), counts) if counts is not None
          else np.zeros(n, np.int64))
    okb = ok == 1
    assert okb.any()
    nu = 3 * proc.n_out - 4
    own = xo[ch, np.arange(n)]
    assert np.median(np.abs(own[okb, :nu] - x[okb, :nu])) < 1e-12
    assert_inverse_parity(oracle.Oracle(proc, proc.sqrts), fac, xo, p,
                          ch.astype(np.int32) if counts is not None else None, ok, E1=E1, E2=E2,
                          q99=None)


def test_full_size_bwbw(torch):
    """2^21 events over the 61 bwbw channels (1.28e8 channel inversions): the generating
    channel's round trip for every event and the oracle on a slice."""
    from gpu_phs_gb300.api import PhaseSpace, philox_x
    z = golden("whizard_bwbw")
    proc = load_process(z)
    n = 1 << 21
    counts = np.full(proc.n_channels, n // proc.n_channels, np.int64)
    counts[: n - counts.sum()] += 1
    ps = PhaseSpace(proc, 500.0, 500.0)
    x = philox_x(n, proc.n_x, seed=77)
    ev = ps.generate(x, counts)
    fac, xo = ps.inverse(ev.p, counts, ev.ok)
    ch = torch.repeat_interleave(torch.arange(proc.n_channels, device="cuda"),
                                 torch.from_numpy(counts).cuda())
    idx = torch.arange(n, device="cuda")
    okb = ev.ok.bool()
    own_x = xo[ch, idx][okb]
    dx = (own_x - x[okb]).abs()
    assert dx.median().item() < 1e-12
    own_f = fac[idx, ch][okb]
    assert ((own_f / ev.factor[okb] - 1).abs().median().item()) < 1e-11
    assert torch.isfinite(fac[okb]).all().item()
    sl = slice(1_000_000, 1_004_000)
    assert_inverse_parity(oracle.Oracle(proc, 1000.0), fac[sl].cpu().numpy(),
                          xo[:, sl].cpu().numpy(), ev.p[sl].cpu().numpy(),
                          ch[sl].cpu().numpy().astype(np.int32), ev.ok[sl].cpu().numpy())


def test_whizard_abi_all_channels(torch):
    from gpu_phs_gb300 import _lib
    lib = _lib.load()
    z = golden("whizard_bwbw")
    proc = load_process(z)
    ip = lambda v: C.byref(C.c_int(v))
    nch, n_x = proc.n_channels, proc.n_x
    lib.c_whizard_set_particle_structure(ip(nch), ip(nch), ip(nch), ip(n_x), ip(2), ip(proc.n_out))
    fm = np.ascontiguousarray(proc.flv_masses)
    fw = np.ascontiguousarray(proc.flv_widths)
    lib.c_whizard_set_flavors(fm.ctypes.data, fw.ctypes.data)
    lib.c_whizard_init_mappings()
    keep = []
    for c in range(nch):
        a = [np.ascontiguousarray(proc.map_ids[c], np.int32), np.ascontiguousarray(proc.map_masses[c]),
             np.ascontiguousarray(proc.map_widths[c])]
        keep += a
        lib.c_whizard_fill_mapping(ip(c + 1), *[t.ctypes.data for t in a])
    lib.c_whizard_init_tree_structures()
    for c in range(nch):
        a = [np.ascontiguousarray(t[c], np.int32) for t in (proc.d1, proc.d2, proc.has_children, proc.friends)]
        keep += a
        lib.c_whizard_fill_tree_structure(ip(c + 1), *[t.ctypes.data for t in a])
    lib.c_whizard_set_threads(ip(512), ip(512), ip(512))
    lib.c_whizard_init_gpu_phs()
    counts = counts_of(z["channel"], nch)
    n = int(counts.sum())
    limits = np.ascontiguousarray(np.cumsum(counts), np.int32)
    lib.c_whizard_init_channel_ids(ip(n), ip(nch), limits.ctypes.data)
    x = np.ascontiguousarray(z["x"])
    E1 = np.full(n, 500.0)
    E2 = np.full(n, 500.0)
    factors = np.zeros(n * nch)
    volumes = np.zeros(n)
    oks = np.zeros(n, np.uint8)
    p = np.zeros(n * proc.n_out * 4)
    x_out = np.zeros(n * n_x * nch)
    flag = C.c_bool(False)
    lib.c_whizard_gen_phs_from_x_gpu(E1.ctypes.data, E2.ctypes.data, C.byref(flag), ip(n), ip(nch),
                                     ip(n_x), x.ctypes.data, factors.ctypes.data,
                                     volumes.ctypes.data, oks.ctypes.data, p.ctypes.data,
                                     x_out.ctypes.data)
    assert lib.phs_last_error().decode() == ""
    o = oracle.Oracle(proc, 1000.0)
    fac = factors.reshape(n, nch)
    own = fac[np.arange(n), z["channel"]]
    assert_inverse_parity(o, fac, x_out.reshape(nch, n, n_x), p.reshape(n, proc.n_out, 4),
                          z["channel"], oks, x_own=x, factor_own=own)
    g = z["all_factors"]
    assert np.all(np.abs(fac - g) <= 0.5e-7 + 2e-3 * np.abs(g))
    lib.c_whizard_reset_generator()
    lib.c_whizard_finalize_gpu_phs()


def whizard_setup(lib, proc):
    """The Whizard ABI's set-up calls for proc, up to c_whizard_init_gpu_phs."""
    ip = lambda v: C.byref(C.c_int(v))
    nch, n_x, n_out = proc.n_channels, proc.n_x, proc.n_out
    lib.c_whizard_set_particle_structure(ip(nch), ip(nch), ip(nch), ip(n_x), ip(2), ip(n_out))
    fm = np.ascontiguousarray(proc.flv_masses)
    fw = np.ascontiguousarray(proc.flv_widths)
    lib.c_whizard_set_flavors(fm.ctypes.data, fw.ctypes.data)
    lib.c_whizard_init_mappings()
    for c in range(nch):
        a = [np.ascontiguousarray(proc.map_ids[c], np.int32), np.ascontiguousarray(proc.map_masses[c]),
             np.ascontiguousarray(proc.map_widths[c])]
        lib.c_whizard_fill_mapping(ip(c + 1), *[t.ctypes.data for t in a])
    lib.c_whizard_init_tree_structures()
    for c in range(nch):
        a = [np.ascontiguousarray(t[c], np.int32) for t in (proc.d1, proc.d2, proc.has_children, proc.friends)]
        lib.c_whizard_fill_tree_structure(ip(c + 1), *[t.ctypes.data for t in a])
    lib.c_whizard_init_gpu_phs()


def whizard_call_vs_handle_api(torch, name, n, counts, beams, calls=None):
    """n events of the process `name` (a sample file's, or a builder of processes.py;
    events per channel `counts`) through c_whizard_gen_phs_from_x_gpu and through the
    handle API's forward and inverse calls on the whole batch: every output equal bit for
    bit.  calls: several (n, counts) in turn after one set-up, instead."""
    from gpu_phs_gb300 import _lib
    from gpu_phs_gb300.api import PhaseSpace
    lib = _lib.load()
    proc = getattr(P, name)() if hasattr(P, name) else load_process(golden(f"whizard_{name}"))
    ip = lambda v: C.byref(C.c_int(v))
    nch, n_x, n_out = proc.n_channels, proc.n_x, proc.n_out
    whizard_setup(lib, proc)
    ps = PhaseSpace(proc, 500.0, 500.0)
    rng = np.random.default_rng(17)
    for k, (n, counts) in enumerate(calls or [(n, counts)]):
        assert int(counts.sum()) == n
        limits = np.ascontiguousarray(np.cumsum(counts), np.int32)
        lib.c_whizard_init_channel_ids(ip(n), ip(nch), limits.ctypes.data)
        x = np.ascontiguousarray(uniform_x(18 + k, n, n_x))
        if beams == "uniform":
            E1, E2 = np.full(n, 500.0), np.full(n, 500.0)
        else:
            E1, E2 = rng.uniform(400, 600, n), rng.uniform(400, 600, n)
        factors, volumes = np.zeros(n * nch), np.zeros(n)
        oks = np.zeros(n, np.uint8)
        p = np.zeros(n * n_out * 4)
        x_out = np.zeros(n * n_x * nch)
        lib.c_whizard_gen_phs_from_x_gpu(E1.ctypes.data, E2.ctypes.data, C.byref(C.c_bool(False)),
                                         ip(n), ip(nch), ip(n_x), x.ctypes.data, factors.ctypes.data,
                                         volumes.ctypes.data, oks.ctypes.data, p.ctypes.data,
                                         x_out.ctypes.data)
        assert lib.phs_last_error().decode() == ""
        xd = torch.from_numpy(x).cuda()
        if beams == "uniform":
            ev = ps.generate(xd, counts)
            fa, xo = ps.inverse(ev.p, counts, ev.ok, xd, ev.factor)
        else:
            e1, e2 = torch.from_numpy(E1).cuda(), torch.from_numpy(E2).cuda()
            ev = ps.generate_beams(xd, e1, e2, counts)
            fa, xo = ps.inverse(ev.p, counts, ev.ok, xd, ev.factor, E1=e1, E2=e2)
        assert np.array_equal(p.reshape(n, n_out, 4), ev.p.cpu().numpy())
        assert np.array_equal(volumes, ev.volume.cpu().numpy())
        assert np.array_equal(oks, ev.ok.cpu().numpy())
        assert np.array_equal(factors.reshape(n, nch), fa.cpu().numpy())
        assert np.array_equal(x_out.reshape(nch, n, n_x), xo.cpu().numpy())
    lib.c_whizard_reset_generator()
    lib.c_whizard_finalize_gpu_phs()


@pytest.mark.parametrize("beams", ["uniform", "per_event"])
def test_whizard_abi_pipelined_call_equals_handle_api(torch, beams):
    """100 000 bwbw events (61 channels, one of them empty) through
    c_whizard_gen_phs_from_x_gpu, which runs the inverse map in launches over slices of the
    channels (the last slice in chunks of events) beside the copies of the finished ones:
    momenta, every channel's factors and x, volumes and ok flags equal the handle API's
    forward and inverse calls on the whole batch (one inverse launch), bit for bit."""
    n, nch = 100_000, 61
    counts = np.random.default_rng(17).multinomial(n, np.full(nch, 1.0 / nch)).astype(np.int64)
    counts[5] = 0                                      # an empty channel inside
    counts[0] += n - int(counts.sum())
    whizard_call_vs_handle_api(torch, "bwbw", n, counts, beams)


@pytest.mark.parametrize("beams", ["uniform", "per_event"])
def test_whizard_abi_one_channel_chunked(torch, beams):
    """The tt tree alone (one channel), 600 001 events: the forward map runs in chunks of
    events with the copies in and back beside the kernels, x and factors of the one channel
    come from the input and the forward map; equal to the handle API bit for bit."""
    whizard_call_vs_handle_api(torch, "tt", 600_001, np.array([600_001], np.int64), beams)


def test_whizard_abi_pipelined_call_few_channels(torch):
    """ttH (3 channels, fewer than the call's slices), 400 000 events with the first channel
    empty: one slice per channel, the last one in chunks of uneven events; equal to the
    handle API bit for bit."""
    whizard_call_vs_handle_api(torch, "ttH", 400_000, np.array([0, 300_001, 99_999], np.int64),
                               "uniform")


@pytest.mark.parametrize("beams", ["uniform", "per_event"])
def test_whizard_abi_calls_of_changing_size(torch, beams):
    """Calls of 700 000, 3 000 and 300 000 ttH events after one set-up (buffers grown,
    then reused with shorter rows; chunked and unchunked forward maps, sliced and single
    inverse launches), each equal to the handle API bit for bit."""
    calls = [(700_000, np.array([200_000, 0, 500_000], np.int64)),
             (3_000, np.array([1_000, 1_500, 500], np.int64)),
             (300_000, np.array([100_000, 150_000, 50_000], np.int64))]
    whizard_call_vs_handle_api(torch, "ttH", 0, None, beams, calls=calls)


def test_whizard_abi_rejects_bad_calls(torch):
    """A negative event count, a channel count or n_x other than the set-up's and event
    counts that differ from c_whizard_init_channel_ids are refused with a message (the call
    returns nothing); a valid call afterwards succeeds."""
    from gpu_phs_gb300 import _lib
    lib = _lib.load()
    proc = load_process(golden("whizard_ttH"))
    ip = lambda v: C.byref(C.c_int(v))
    nch, n_x, n_out = proc.n_channels, proc.n_x, proc.n_out
    whizard_setup(lib, proc)
    n = 30
    limits = np.ascontiguousarray(np.cumsum([10, 10, 10]), np.int32)
    lib.c_whizard_init_channel_ids(ip(n), ip(nch), limits.ctypes.data)
    x = np.ascontiguousarray(uniform_x(3, n, n_x))
    E = np.full(n, 500.0)
    f, v, ok, p, xo = np.zeros(n * nch), np.zeros(n), np.zeros(n, np.uint8), np.zeros(n * n_out * 4), np.zeros(n * n_x * nch)

    def call(n_ev, n_ch, nx):
        lib.c_whizard_gen_phs_from_x_gpu(E.ctypes.data, E.ctypes.data, C.byref(C.c_bool(False)),
                                         ip(n_ev), ip(n_ch), ip(nx), x.ctypes.data, f.ctypes.data,
                                         v.ctypes.data, ok.ctypes.data, p.ctypes.data, xo.ctypes.data)
        return lib.phs_last_error().decode()
    try:
        assert "< 0" in call(-5, nch, n_x)
        assert "n_channels/n_x" in call(n, nch + 1, n_x)
        assert "n_channels/n_x" in call(n, nch, n_x + 1)
        assert "cover" in call(n - 1, nch, n_x)
        assert call(n, nch, n_x) == ""
        assert ok.sum() > 0
    finally:
        lib.c_whizard_reset_generator()
        lib.c_whizard_finalize_gpu_phs()
