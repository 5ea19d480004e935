"""Parity of the CUDA path (through the C ABI) with the CPU oracle, the reference CPU
fixtures and the Whizard golden vectors.

Bar: ok flags bit-exact; momenta within 1e-12 of max(particle energy, 1e-3 sqrt(s))
(conftest.momentum_rel_err), factors within 1e-12 relative (FP64; the transcendental
functions of CUDA and glibc may differ by an ulp); volumes within 1e-15 relative.
Channels with a friend (beam-axis) boost: momenta within 1e-10, because the rotation onto
the friend axis divides by 1 + cos(angle of the axis to z) (Rodrigues), so two FP64
evaluations in different operation order drift apart as that axis nears -z.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import (REFCPU_FIXTURES, all_maps_process, assert_within_conditioning, counts_of,
                      golden, load_process, momentum_rel_err, wide_beams)
from gpu_phs_gb300 import processes as P
from gpu_phs_gb300.philox import uniform_x
from oracle import oracle

pytestmark = pytest.mark.gpu

MOM_TOL = 1e-12
MOM_TOL_FRIEND = 1e-10
FAC_TOL = 1e-12


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def run_gpu(torch, proc, x, sqrts, counts=None, E=None, precision=0, variants=(-1, -1)):
    from gpu_phs_gb300.api import PhaseSpace
    ps = PhaseSpace(proc)
    ps.set_beams(*(E if E else (sqrts / 2, sqrts / 2)))
    ps.set_precision(precision)
    ps.set_variants(*variants)
    xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    ev = ps.generate(xd, counts)
    torch.cuda.synchronize()
    out = (ev.p.cpu().numpy(), ev.factor.cpu().numpy(), ev.volume.cpu().numpy(), ev.ok.cpu().numpy())
    ps.close()
    return out


def assert_parity(got, ref_p, ref_f, ref_v, ref_ok, vol_all=False, sqrts=1000.0, friend=None):
    """friend: per-event mask of events generated by a channel with a friend boost."""
    p, f, v, ok = got
    mism = int(np.count_nonzero(ok != ref_ok))
    assert mism == 0, f"{mism} ok-flag mismatches"
    sel = ref_ok == 1
    if sel.any():
        tol = np.full(len(ok), MOM_TOL)
        if friend is not None:
            tol[friend] = MOM_TOL_FRIEND
        err = momentum_rel_err(p[sel], ref_p[sel], sqrts).max(axis=-1)
        worst = (err / tol[sel]).max()
        assert worst <= 1.0, f"momentum error {worst:.3e} x the tolerance"
        ferr = (np.abs(f[sel] - ref_f[sel]) / np.abs(ref_f[sel])).max()
        assert ferr <= FAC_TOL, f"factor error {ferr:.3e}"
    vs = slice(None) if vol_all else sel
    if np.any(vs if not isinstance(vs, slice) else True):
        verr = (np.abs(v[vs] - ref_v[vs]) / np.abs(ref_v[vs])).max()
        assert verr <= 1e-15, f"volume error {verr:.3e}"
    assert np.all(p[~sel] == 0) and np.all(f[~sel] == 0)


def test_philox_device_matches_numpy(torch):
    from gpu_phs_gb300.api import philox_x
    for n, nx, e0 in [(1000, 14, 0), (777, 5, 123), (1, 3, 9)]:
        x = philox_x(n, nx, seed=42, first_event=e0).cpu().numpy()
        assert np.array_equal(x, uniform_x(42, n, nx, first_event=e0))


@pytest.mark.parametrize("builder", [P.ww, P.tt, P.precision])
def test_forward_vs_oracle(torch, builder):
    proc = builder()
    n = 200_003
    x = uniform_x(2024, n, proc.n_x)
    r = oracle.Oracle(proc, proc.sqrts).generate(x)
    got = run_gpu(torch, proc, x, proc.sqrts)
    assert_parity(got, r.p, r.factor, r.volume, r.ok, vol_all=True, sqrts=proc.sqrts)


@pytest.mark.parametrize("name", REFCPU_FIXTURES)
def test_forward_vs_reference_fixture(torch, name):
    z = golden(f"refcpu_{name}")
    proc = load_process(z)
    x = uniform_x(int(z["seed"][0]), len(z["ok"]), proc.n_x)
    counts = counts_of(z["channel"], proc.n_channels)
    got = run_gpu(torch, proc, x, float(z["sqrts"][0]), counts)
    assert_parity(got, z["p"], z["factor"], z["volume"], z["ok"], sqrts=float(z["sqrts"][0]))


@pytest.mark.parametrize("name", ["ttH", "bwbw"])
def test_forward_vs_whizard_golden(torch, name):
    z = golden(f"whizard_{name}")
    proc = load_process(z)
    counts = counts_of(z["channel"], proc.n_channels)
    p, f, v, ok = run_gpu(torch, proc, z["x"], 1000.0, counts)
    assert np.array_equal(ok, z["ok"].astype(np.uint8))
    # all channels, the 16 friend-boost trees of bwbw included
    assert np.abs(p - z["p_out"]).max() < 1e-3
    assert np.allclose(v, z["volume"], rtol=1e-14, atol=0)
    r = oracle.Oracle(proc, 1000.0).generate(z["x"], z["channel"])
    assert_parity((p, f, v, ok), r.p, r.factor, r.volume, r.ok,
                  friend=z["hasfriends"][z["channel"]] == 1)


@pytest.mark.parametrize("n", [0, 1, 31, 32, 33, 1025])
def test_edge_sizes(torch, n):
    proc = P.tt()
    x = uniform_x(5, max(n, 1), proc.n_x)[:n]
    r = oracle.Oracle(proc, 1000.0).generate(x) if n else None
    got = run_gpu(torch, proc, x, 1000.0)
    if n:
        assert_parity(got, r.p, r.factor, r.volume, r.ok)
    else:
        assert got[0].shape == (0, 6, 4)


# (precision, (FP32-pair variant, FP64 variant)): the split forms and a non-default shape
SPLIT_FORMS = [(0, (-1, 6)), (0, (-1, 8)), (1, (5, -1)), (1, (3, -1))]


@pytest.mark.parametrize("form", SPLIT_FORMS)
@pytest.mark.parametrize("n", [0, 1, 31, 33, 1025])
def test_edge_sizes_compacting_and_split_forms(torch, n, form):
    """Partial and single tiles, one-tile segments and no events at all through the
    pre-test, scan and walk kernels (and the fused compacting FP32-pair form)."""
    prec, variants = form
    proc = P.tt()
    x = uniform_x(15, max(n, 1), proc.n_x)[:n]
    got = run_gpu(torch, proc, x, 1000.0, precision=prec, variants=variants)
    if not n:
        assert got[0].shape == (0, 6, 4)
        return
    r = oracle.Oracle(proc, 1000.0).generate(x)
    if prec == 0:
        assert_parity(got, r.p, r.factor, r.volume, r.ok)
    else:
        p, f, v, ok = got
        assert np.array_equal(ok, r.ok)
        sel = r.ok == 1
        assert momentum_rel_err(p[sel], r.p[sel], 1000.0).max() <= 1e-7
        assert np.all(p[~sel] == 0) and np.all(f[~sel] == 0)


@pytest.mark.parametrize("n_out", [10, 12])
def test_largest_trees(torch, n_out):
    """The API's largest trees (up to 12 outgoing particles, 11 visits, 32 x per event):
    balanced and caterpillar channels of nested resonances, FP64 against the oracle, FP32
    pairs at their bar, and the inverse map's round trip."""
    from gpu_phs_gb300.api import PhaseSpace
    proc = P.nested_resonances(n_out)
    counts = np.array([3000, 1, 2999], np.int64)
    chan = np.repeat(np.arange(3), counts).astype(np.int32)
    x = uniform_x(41, int(counts.sum()), proc.n_x)
    r = oracle.Oracle(proc, 1000.0).generate(x, chan)
    got = run_gpu(torch, proc, x, 1000.0, counts)
    assert_parity(got, r.p, r.factor, r.volume, r.ok)
    assert r.ok.mean() > 0.1
    ff = run_gpu(torch, proc, x, 1000.0, counts, precision=1)
    assert np.array_equal(ff[3], r.ok)
    sel = r.ok == 1
    assert momentum_rel_err(ff[0][sel], r.p[sel], 1000.0).max() <= 1e-7
    # inverse map: the generating channel's own x comes back
    ps = PhaseSpace(proc, 500.0, 500.0)
    xd = torch.from_numpy(x).cuda()
    ev = ps.generate(xd, counts)
    fa, xo = ps.inverse(ev.p, counts, ev.ok)
    xo = xo.cpu().numpy()
    own = xo[chan, np.arange(x.shape[0])]
    okb = ev.ok.cpu().numpy() == 1
    assert np.abs(own[okb] - x[okb]).max() < 1e-6


def test_multichannel_uneven_counts(torch):
    z = golden("whizard_bwbw")
    proc = load_process(z)
    rng = np.random.default_rng(3)
    counts = rng.integers(0, 70, proc.n_channels).astype(np.int64)
    counts[[0, 5, 17]] = 0
    n = int(counts.sum())
    channels = np.repeat(np.arange(proc.n_channels), counts).astype(np.int32)
    x = uniform_x(6, n, proc.n_x)
    r = oracle.Oracle(proc, 1000.0).generate(x, channels)
    got = run_gpu(torch, proc, x, 1000.0, counts)
    assert_parity(got, r.p, r.factor, r.volume, r.ok, friend=z["hasfriends"][channels] == 1)


def test_many_channels_device_segment_table(torch):
    # more channels with events than fit the launch parameters: the segment table goes
    # through device memory
    rng = np.random.default_rng(8)
    proc = P.random_process(rng, 5, 150, 1000.0)
    counts = rng.integers(1, 40, proc.n_channels).astype(np.int64)
    channels = np.repeat(np.arange(proc.n_channels), counts).astype(np.int32)
    x = uniform_x(7, int(counts.sum()), proc.n_x)
    r = oracle.Oracle(proc, 1000.0).generate(x, channels)
    got = run_gpu(torch, proc, x, 1000.0, counts)
    assert_parity(got, r.p, r.factor, r.volume, r.ok)


def test_host_path_matches_device(torch):
    from gpu_phs_gb300.api import PhaseSpace
    proc = P.tt()
    n = 2_500_000           # more than two pipeline chunks
    x = uniform_x(11, n, proc.n_x)
    ps = PhaseSpace(proc, 500.0, 500.0)
    xh = torch.from_numpy(x).pin_memory()
    h = ps.generate_host(xh)
    d = ps.generate(xh.cuda())
    torch.cuda.synchronize()
    assert torch.equal(h.p, d.p.cpu()) and torch.equal(h.ok, d.ok.cpu())
    assert torch.equal(h.factor, d.factor.cpu()) and torch.equal(h.volume, d.volume.cpu())


@pytest.mark.parametrize("precision", [0, 1])
def test_host_path_matches_device_many_channels(torch, precision):
    """40 channels with uneven counts through the pipelined host call (the volumes are
    written on the host per channel, the rest copied back per chunk): the device path's bits,
    in FP64 and in FP32 pairs."""
    from gpu_phs_gb300.api import PhaseSpace
    rng = np.random.default_rng(21)
    proc = P.random_process(rng, 6, 40, 1000.0)
    counts = rng.integers(0, 60_000, proc.n_channels).astype(np.int64)
    counts[::9] = 0
    n = int(counts.sum())
    x = uniform_x(23, n, proc.n_x)
    ps = PhaseSpace(proc, 500.0, 500.0)
    ps.set_precision(precision)
    xh = torch.from_numpy(x).pin_memory()
    h = ps.generate_host(xh, counts)
    d = ps.generate(xh.cuda(), counts)
    torch.cuda.synchronize()
    assert torch.equal(h.p, d.p.cpu()) and torch.equal(h.ok, d.ok.cpu())
    assert torch.equal(h.factor, d.factor.cpu()) and torch.equal(h.volume, d.volume.cpu())


@pytest.mark.parametrize("beams", ["uniform", "asymmetric", "random"])
def test_per_event_beams(torch, beams):
    from gpu_phs_gb300.api import PhaseSpace
    proc = P.tt()
    n = 50_000
    x = uniform_x(12, n, proc.n_x)
    rng = np.random.default_rng(1)
    if beams == "uniform":
        E1 = E2 = np.full(n, 500.0)
    elif beams == "asymmetric":
        E1, E2 = np.full(n, 600.0), np.full(n, 420.0)
    else:
        E1, E2 = rng.uniform(300, 700, n), rng.uniform(300, 700, n)
    r = oracle.Oracle(proc, 1000.0).generate(x, E1=E1, E2=E2)
    ps = PhaseSpace(proc)
    ev = ps.generate_beams(torch.from_numpy(x).cuda(), torch.from_numpy(E1).cuda(),
                           torch.from_numpy(E2).cuda())
    got = (ev.p.cpu().numpy(), ev.factor.cpu().numpy(), ev.volume.cpu().numpy(), ev.ok.cpu().numpy())
    # per-event constants go through CUDA's atan/log, so allow a few more ulps
    p, f, v, ok = got
    assert int(np.count_nonzero(ok != r.ok)) == 0
    sel = r.ok == 1
    assert momentum_rel_err(p[sel], r.p[sel], 1000.0).max() < 1e-11
    assert (np.abs(f[sel] - r.factor[sel]) / np.abs(r.factor[sel])).max() < 1e-11
    assert (np.abs(v - r.volume) / r.volume).max() < 1e-15
    if beams != "uniform":
        tot = p[sel].sum(axis=1)
        assert np.allclose(tot[:, 0], (E1 + E2)[sel], rtol=1e-12)
        assert np.allclose(tot[:, 3], (E1 - E2)[sel], atol=1e-8)


@pytest.mark.parametrize("builder", [P.ww, P.tt, P.precision])
def test_per_event_beams_wide_energy_range(torch, builder):
    """Per-event beams over four decades of energy (wide_beams).  The device evaluates the
    constants that depend on sqrt(s), and the maps' tan/exp/log, within a few ulps of the
    oracle's (CUDA's library against glibc's, the Breit-Wigner bound's series, products
    with 1/s).  Far below a resonance the reference's Breit-Wigner map is ill-conditioned
    in exactly these values (one ulp of a1 moves tan(z) by (1 + u^2) ulps, and
    msq = m (m + w tan z) cancels), and many events sit near a threshold, where the Kallen
    function amplifies that into momenta: the oracle itself moves by up to 1e-7 when they
    move by two ulps.  Bar: ok flags bit-exact; momenta and factors within 1e-11, or 64
    times the oracle's own change under such perturbations (assert_within_conditioning,
    oracle_sensitivity); volumes within 1e-15."""
    from gpu_phs_gb300.api import PhaseSpace
    proc = builder()
    n = 50_000
    x = uniform_x(14, n, proc.n_x)
    E1, E2 = wide_beams(n, proc.sqrts, 4)
    sq = 2.0 * np.sqrt(E1 * E2)
    o = oracle.Oracle(proc, proc.sqrts)
    r = o.generate(x, E1=E1, E2=E2)
    ps = PhaseSpace(proc)
    ev = ps.generate_beams(torch.from_numpy(x).cuda(), torch.from_numpy(E1).cuda(),
                           torch.from_numpy(E2).cuda())
    p, f, v, ok = (ev.p.cpu().numpy(), ev.factor.cpu().numpy(), ev.volume.cpu().numpy(),
                   ev.ok.cpu().numpy())
    assert_within_conditioning(p, f, ok, o, x, r, sq, E1, E2, 1e-11, 64)
    assert (np.abs(v - r.volume) / r.volume).max() < 1e-15


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("n_out", [3, 4, 5, 6, 7, 8])
def test_every_mapping_uniform_beams(torch, n_out, precision):
    """8 random channels of n_out particles with every mapping kind (all_maps_process) at
    sqrt(s) = 1 TeV, FP64 and FP32 pairs: ok flags bit-exact with the oracle; momenta and
    factors within 1e-12 (FP32 pairs 1e-7) or 64 (1024) times the oracle's own change when
    x and the maps' tan/exp/log values move by an ulp or two (the constants are the host's
    bits here; CUDA's and glibc's functions differ by an ulp, which a Breit-Wigner map
    far below its pole, msq = m (m + w tan z), and the Kallen function near a threshold
    amplify); volumes within 1e-15."""
    from gpu_phs_gb300.api import PhaseSpace
    proc = all_maps_process(100 + n_out, n_out, 8)
    n = 20_000
    counts = np.full(8, n // 8, np.int64)
    ch = np.repeat(np.arange(8), counts).astype(np.int32)
    x = uniform_x(700 + n_out, n, proc.n_x)
    o = oracle.Oracle(proc, 1000.0)
    r = o.generate(x, ch)
    p, f, v, ok = run_gpu(torch, proc, x, 1000.0, counts, precision=precision)
    bar, ulps = (1e-12, 64) if precision == 0 else (1e-7, 1024)
    assert_within_conditioning(p, f, ok, o, x, r, np.full(n, 1000.0), None, None, bar, ulps,
                               channels=ch)
    assert (np.abs(v - r.volume) / r.volume).max() < 1e-15


@pytest.mark.parametrize("beams", ["mid", "wide"])
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("n_out", [3, 4, 5, 6, 7, 8])
def test_per_event_beams_every_mapping(torch, n_out, precision, beams):
    """Per-event beams on 8 random channels of n_out particles with every mapping kind
    (all_maps_process), beam energies uniform in [0.3, 0.7] sqrt(s) ("mid") or over four
    decades (wide_beams), FP64 and FP32 pairs (whose step-map channels take the exact
    path per event).  Bar as test_per_event_beams_wide_energy_range: ok flags bit-exact,
    momenta and factors within 1e-11 (FP32 pairs 1e-7) or 64 (1024) times the oracle's own
    change under perturbations of the device's rounding size, volumes within 1e-15."""
    from gpu_phs_gb300.api import PhaseSpace
    proc = all_maps_process(100 + n_out, n_out, 8)
    n = 20_000
    counts = np.full(8, n // 8, np.int64)
    ch = np.repeat(np.arange(8), counts).astype(np.int32)
    x = uniform_x(200 + n_out, n, proc.n_x)
    if beams == "wide":
        E1, E2 = wide_beams(n, 1000.0, 7)
    else:
        rng = np.random.default_rng(n_out)
        E1, E2 = rng.uniform(300.0, 700.0, n), rng.uniform(300.0, 700.0, n)
    sq = 2.0 * np.sqrt(E1 * E2)
    o = oracle.Oracle(proc, 1000.0)
    r = o.generate(x, ch, E1=E1, E2=E2)
    ps = PhaseSpace(proc)
    ps.set_precision(precision)
    ev = ps.generate_beams(torch.from_numpy(x).cuda(), torch.from_numpy(E1).cuda(),
                           torch.from_numpy(E2).cuda(), counts)
    torch.cuda.synchronize()
    p, f, v, ok = (ev.p.cpu().numpy(), ev.factor.cpu().numpy(), ev.volume.cpu().numpy(),
                   ev.ok.cpu().numpy())
    bar, ulps = (1e-11, 64) if precision == 0 else (1e-7, 1024)
    assert_within_conditioning(p, f, ok, o, x, r, sq, E1, E2, bar, ulps, channels=ch)
    assert (np.abs(v - r.volume) / r.volume).max() < 1e-15


def test_batch_matches_single_process_runs(torch):
    from gpu_phs_gb300.api import Batch, PhaseSpace
    rng = np.random.default_rng(21)
    procs = [P.random_process(rng, n_out, 1, 1000.0) for n_out in (3, 8, 5, 4, 7, 6, 3, 8)]
    procs[3].n_x = 11            # padding x columns beyond the 8 the tree consumes
    spaces = [PhaseSpace(p, 500.0, 500.0) for p in procs]
    batch = Batch(spaces)
    counts = np.array([37, 1000, 0, 64, 333, 95, 1, 2048], np.int64)
    xo, po = batch.offsets(counts)
    xs = [uniform_x(30 + i, int(c), p.n_x) for i, (p, c) in enumerate(zip(procs, counts))]
    xflat = torch.from_numpy(np.concatenate([a.reshape(-1) for a in xs])).cuda()
    p, f, v, ok = batch.generate(xflat, counts)
    p, f, v, ok = p.cpu().numpy(), f.cpu().numpy(), v.cpu().numpy(), ok.cpu().numpy()
    e = 0
    for i, (proc, c) in enumerate(zip(procs, counts)):
        c = int(c)
        r = oracle.Oracle(proc, 1000.0).generate(xs[i]) if c else None
        if c:
            pp = p[po[i]:po[i + 1]].reshape(c, proc.n_out, 4)
            assert_parity((pp, f[e:e + c], v[e:e + c], ok[e:e + c]), r.p, r.factor, r.volume, r.ok)
        e += c


def test_whizard_binding_end_to_end(torch):
    """Drives the 14 c_whizard_* entry points as Whizard does (whizard_gpu_phs.cpp)."""
    from gpu_phs_gb300 import _lib
    lib = _lib.load()
    z = golden("whizard_ttH")
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
    assert lib.phs_whizard_momentum_device_pointer()
    r = oracle.Oracle(proc, 1000.0).generate(x, z["channel"])
    own = factors.reshape(n, nch)[np.arange(n), z["channel"]]
    assert_parity((p.reshape(n, proc.n_out, 4), own, volumes, oks), r.p, r.factor, r.volume, r.ok,
                  friend=z["hasfriends"][z["channel"]] == 1)
    xo = x_out.reshape(nch, n, n_x)
    assert np.array_equal(xo[z["channel"], np.arange(n)], x)
    lib.c_whizard_reset_generator()
    lib.c_whizard_finalize_gpu_phs()


class _DeviceArray:
    """A device pointer the library returned, seen by torch (CUDA array interface)."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr,
                                         "data": (ptr, False), "version": 3, "strides": None}


@pytest.mark.parametrize("beams", [(500.0, 500.0), (600.0, 420.0)])
def test_whizard_device_handoff(torch, beams):
    """The reference's transfer_to_whizard.h functions after a Whizard call: momenta in the
    sparse [event][2^(n_in+n_out)-1][4] layout (outgoing codes in the lab frame, internal
    codes of any channel as centre-of-mass sums, all else 0), the beams [E1; E2] and the ok
    flags, all in device memory."""
    from gpu_phs_gb300 import _lib
    lib = _lib.load()
    z = golden("whizard_ttH")
    proc = load_process(z)
    ip = lambda v: C.byref(C.c_int(v))
    nch, n_x, n_out = proc.n_channels, proc.n_x, proc.n_out
    lib.c_whizard_set_particle_structure(ip(nch), ip(nch), ip(nch), ip(n_x), ip(2), ip(n_out))
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
    lib.c_whizard_init_gpu_phs()
    counts = counts_of(z["channel"], nch)
    n = int(counts.sum())
    limits = np.ascontiguousarray(np.cumsum(counts), np.int32)
    lib.c_whizard_init_channel_ids(ip(n), ip(nch), limits.ctypes.data)
    x = np.ascontiguousarray(z["x"])
    E1, E2 = np.full(n, beams[0]), np.full(n, beams[1])
    factors, volumes = np.zeros(n * nch), np.zeros(n)
    oks = np.zeros(n, np.uint8)
    p = np.zeros(n * n_out * 4)
    x_out = np.zeros(n * n_x * nch)
    lib.c_whizard_gen_phs_from_x_gpu(E1.ctypes.data, E2.ctypes.data, C.byref(C.c_bool(False)), ip(n),
                                     ip(nch), ip(n_x), x.ctypes.data, factors.ctypes.data,
                                     volumes.ctypes.data, oks.ctypes.data, p.ctypes.data,
                                     x_out.ctypes.data)
    assert lib.phs_last_error().decode() == ""
    getters = {}
    for name, res in (("get_momentum_device_pointer", C.c_void_p),
                      ("get_in_momentum_device_pointer", C.c_void_p),
                      ("get_ok_device_pointer", C.c_void_p)):
        f = getattr(lib, f"_Z{len(name)}{name}v")
        f.restype = res
        getters[name] = f
    n_prt = 2 ** (2 + n_out) - 1
    sp = torch.as_tensor(_DeviceArray(getters["get_momentum_device_pointer"](), (n, n_prt, 4), "<f8"),
                         device="cuda").cpu().numpy()
    pin = torch.as_tensor(_DeviceArray(getters["get_in_momentum_device_pointer"](), (2 * n,), "<f8"),
                          device="cuda").cpu().numpy()
    okd = torch.as_tensor(_DeviceArray(getters["get_ok_device_pointer"](), (n,), "|u1"),
                          device="cuda").cpu().numpy()
    assert np.array_equal(pin, np.concatenate([E1, E2]))
    assert np.array_equal(okd, oks)
    pl = p.reshape(n, n_out, 4)
    # centre-of-mass frame: the inverse of the lab boost along z
    bg = (E1 - E2) / (2 * np.sqrt(E1 * E2))
    ga = np.sqrt(1 + bg * bg)
    pcm = pl.copy()
    pcm[..., 0] = ga[:, None] * pl[..., 0] - bg[:, None] * pl[..., 3]
    pcm[..., 3] = ga[:, None] * pl[..., 3] - bg[:, None] * pl[..., 0]
    internal = {code for c in range(nch) for code in range(1, 2 ** n_out)
                if proc.has_children[c][code - 1]}
    assert (2 ** n_out - 1) in internal
    sqrts = 2 * np.sqrt(beams[0] * beams[1])
    for code in range(1, n_prt + 1):
        slot = sp[:, code - 1]
        if code < 2 ** n_out and code & (code - 1) == 0:
            assert np.array_equal(slot, pl[:, code.bit_length() - 1])
        elif code in internal:
            want = sum(pcm[:, k] for k in range(n_out) if code >> k & 1)
            assert np.abs(slot - want).max() <= 1e-12 * sqrts
        else:
            assert not slot.any(), code
    root = sp[oks == 1, 2 ** n_out - 2]
    assert np.abs(root - np.array([sqrts, 0, 0, 0])).max() <= 1e-9
    lib.c_whizard_reset_generator()
    assert not getters["get_momentum_device_pointer"]()
    lib.c_whizard_finalize_gpu_phs()


def test_full_size_invariants_tt(torch):
    """1e7 tt events: the sizes the benchmark runs, checked through properties that do not
    need the oracle: momentum conservation, on-shell masses, a stable ok fraction."""
    from gpu_phs_gb300.api import PhaseSpace, philox_x
    proc = P.tt()
    n = 10_000_000
    ps = PhaseSpace(proc, 500.0, 500.0)
    x = philox_x(n, proc.n_x, seed=99)
    ev = ps.generate(x)
    ok = ev.ok.bool()
    frac = ok.double().mean().item()
    assert 0.98 < frac < 0.999
    pk = ev.p[ok]
    tot = pk.sum(dim=1)
    assert (tot[:, 0] - 1000.0).abs().max().item() < 1e-9
    assert tot[:, 1:].abs().max().item() < 1e-9
    m2 = pk[..., 0] ** 2 - (pk[..., 1:] ** 2).sum(-1)
    want = torch.tensor(proc.flv_masses[2:] ** 2, device="cuda")
    assert (m2 - want).abs().max().item() < 1e-6
    # the oracle on a slice of the same stream
    sl = slice(4_000_000, 4_020_000)
    r = oracle.Oracle(proc, 1000.0).generate(x[sl].cpu().numpy())
    assert_parity((ev.p[sl].cpu().numpy(), ev.factor[sl].cpu().numpy(),
                   ev.volume[sl].cpu().numpy(), ev.ok[sl].cpu().numpy()),
                  r.p, r.factor, r.volume, r.ok)
