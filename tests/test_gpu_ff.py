"""The FP32-pair (float-float) forward kernel: ok flags bit-exact with the oracle and the
FP64 kernel, momenta (to max(E, 1e-3 sqrt(s))) and factors within 1e-7 relative -- the
requirement on this path is 1e-6; the float-float functions carry ~1e-11, and events
within 1e-5 of a kinematic limit, where the Kallen function amplifies msq errors, are
recomputed in FP64 -- and that exact fallback itself."""
import numpy as np
import pytest

from conftest import (REFCPU_FIXTURES, assert_within_conditioning, counts_of, golden, load_process,
                      momentum_rel_err, wide_beams)
from gpu_phs_gb300 import processes as P
from gpu_phs_gb300.philox import uniform_x
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-7


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


# FP32-pair kernel variants: one pass, fused compacting, split (pre-test kernel + walk)
FF_FORMS = [0, 3, 5]


def run(torch, proc, x, sqrts, counts=None, precision=1, variant=-1):
    from gpu_phs_gb300.api import PhaseSpace
    ps = PhaseSpace(proc, sqrts / 2, sqrts / 2)
    ps.set_precision(precision)
    if precision == 1:
        ps.set_variants(variant, -1)
    ev = ps.generate(torch.from_numpy(np.ascontiguousarray(x)).cuda(), counts)
    torch.cuda.synchronize()
    return ev.p.cpu().numpy(), ev.factor.cpu().numpy(), ev.volume.cpu().numpy(), ev.ok.cpu().numpy()


def check(got, ref_p, ref_f, ref_v, ref_ok, sqrts, tol=TOL):
    p, f, v, ok = got
    assert int(np.count_nonzero(ok != ref_ok)) == 0
    sel = ref_ok == 1
    if sel.any():
        err = momentum_rel_err(p[sel], ref_p[sel], sqrts).max()
        assert err <= tol, f"momentum error {err:.3e}"
        ferr = (np.abs(f[sel] - ref_f[sel]) / np.abs(ref_f[sel])).max()
        assert ferr <= tol, f"factor error {ferr:.3e}"
        assert np.allclose(v[sel], ref_v[sel], rtol=1e-15, atol=0)
    assert np.all(p[~sel] == 0) and np.all(f[~sel] == 0)


@pytest.mark.parametrize("builder", [P.ww, P.tt, P.precision])
def test_ff_vs_oracle(torch, builder):
    proc = builder()
    x = uniform_x(4242, 300_001, proc.n_x)
    r = oracle.Oracle(proc, proc.sqrts).generate(x)
    check(run(torch, proc, x, proc.sqrts), r.p, r.factor, r.volume, r.ok, proc.sqrts)


@pytest.mark.parametrize("name", REFCPU_FIXTURES)
def test_ff_vs_reference_fixture(torch, name):
    z = golden(f"refcpu_{name}")
    proc = load_process(z)
    sq = float(z["sqrts"][0])
    x = uniform_x(int(z["seed"][0]), len(z["ok"]), proc.n_x)
    got = run(torch, proc, x, sq, counts_of(z["channel"], proc.n_channels))
    check(got, z["p"], z["factor"], z["volume"], z["ok"], sq)


@pytest.mark.parametrize("variant", FF_FORMS)
def test_ff_whizard_golden_bwbw(torch, variant):
    """Whizard's 61 bwbw channels, 16 of them with friend boosts (exact path only)."""
    z = golden("whizard_bwbw")
    proc = load_process(z)
    counts = counts_of(z["channel"], proc.n_channels)
    r = oracle.Oracle(proc, 1000.0).generate(z["x"], z["channel"])
    check(run(torch, proc, z["x"], 1000.0, counts, variant=variant), r.p, r.factor, r.volume,
          r.ok, 1000.0)


@pytest.mark.parametrize("variant", FF_FORMS)
def test_ff_fallback_at_kinematic_limits(torch, variant):
    """x = 0 on an unmapped branch gives msq = msq_min exactly: m = m1 + m2, a tie the
    reference decides as not ok.  Those events must take the exact path."""
    rng = np.random.default_rng(5)
    proc = P.random_process(rng, 4, 1, 1000.0)
    proc.map_ids = proc.map_ids.copy()
    proc.map_ids[:] = 0                                       # every branch unmapped
    x = uniform_x(6, 20_000, proc.n_x)
    x[::3, :proc.n_out - 2] = 0.0                            # msq at the lower limit
    x[1::7, :proc.n_out - 2] = 1.0 - 2.0 ** -53              # msq just below the upper limit
    r = oracle.Oracle(proc, 1000.0).generate(x)
    check(run(torch, proc, x, 1000.0, variant=variant), r.p, r.factor, r.volume, r.ok, 1000.0)
    f64 = run(torch, proc, x, 1000.0, precision=0)
    assert np.array_equal(f64[3], r.ok)


def test_ff_matches_f64_kernel_at_scale(torch):
    """2^22 events of the 13 TeV caterpillar, the hardest tree for boosts (gamma ~ 1e3)."""
    from gpu_phs_gb300.api import PhaseSpace, philox_x
    proc = P.precision()
    n = 1 << 22
    x = philox_x(n, proc.n_x, seed=77)
    a = PhaseSpace(proc, 6500.0, 6500.0)
    b = PhaseSpace(proc, 6500.0, 6500.0)
    b.set_precision(1)
    ea, eb = a.generate(x), b.generate(x)
    assert torch.equal(ea.ok, eb.ok)
    sel = ea.ok.bool()
    pa, pb = ea.p[sel], eb.p[sel]
    floor = torch.clamp(pa[..., 0].abs(), min=13.0)
    err = ((pb - pa).abs().amax(-1) / floor).max().item()
    assert err < 1e-7, err
    ferr = ((eb.factor[sel] - ea.factor[sel]).abs() / ea.factor[sel].abs()).max().item()
    assert ferr < 1e-7, ferr


def test_ff_batch(torch):
    from gpu_phs_gb300.api import Batch, PhaseSpace
    rng = np.random.default_rng(21)
    procs = [P.random_process(rng, n_out, 1, 1000.0) for n_out in (3, 8, 5, 4, 7, 6)]
    spaces = [PhaseSpace(p, 500.0, 500.0) for p in procs]
    batch = Batch(spaces)
    batch.set_precision(1)
    counts = np.array([37, 1000, 64, 333, 95, 2048], np.int64)
    xo, po = batch.offsets(counts)
    xs = [uniform_x(30 + i, int(c), p.n_x) for i, (p, c) in enumerate(zip(procs, counts))]
    xflat = torch.from_numpy(np.concatenate([a.reshape(-1) for a in xs])).cuda()
    p, f, v, ok = (t.cpu().numpy() for t in batch.generate(xflat, counts))
    e = 0
    for i, (proc, c) in enumerate(zip(procs, counts)):
        c = int(c)
        r = oracle.Oracle(proc, 1000.0).generate(xs[i])
        pp = p[po[i]:po[i + 1]].reshape(c, proc.n_out, 4)
        check((pp, f[e:e + c], v[e:e + c], ok[e:e + c]), r.p, r.factor, r.volume, r.ok, 1000.0)
        e += c


@pytest.mark.parametrize("variant", FF_FORMS)
def test_ff_exact_path_beside_ff_warps(torch, variant):
    """Channels alternate between trees the float-float path handles and trees with a STEP
    mapping (exact path only), so blocks run both paths at once; the paths share the
    frame stack memory and must not disturb each other."""
    base = P.tt()
    n_ch = 64
    proc = base.subset([0] * n_ch)
    proc.map_ids = proc.map_ids.copy()
    for c in range(1, n_ch, 2):
        proc.map_ids[c, 0b000110 - 1] = P.MAP_STEP_H      # W+ -> STEP_H on odd channels
    counts = np.full(n_ch, 257, np.int64)
    channels = np.repeat(np.arange(n_ch), counts).astype(np.int32)
    x = uniform_x(91, int(counts.sum()), proc.n_x)
    r = oracle.Oracle(proc, 1000.0).generate(x, channels)
    check(run(torch, proc, x, 1000.0, counts, variant=variant), r.p, r.factor, r.volume, r.ok,
          1000.0)


def test_ff_matches_f64_kernel_tt_full_size(torch):
    """1e7 tt events (the benchmark size): identical ok flags, momenta and factors within
    1e-7 of the FP64 kernel."""
    from gpu_phs_gb300.api import PhaseSpace, philox_x
    proc = P.tt()
    n = 10_000_000
    x = philox_x(n, proc.n_x, seed=1234)
    a = PhaseSpace(proc, 500.0, 500.0)
    b = PhaseSpace(proc, 500.0, 500.0)
    b.set_precision(1)
    ea, eb = a.generate(x), b.generate(x)
    assert torch.equal(ea.ok, eb.ok)
    sel = ea.ok.bool()
    floor = torch.clamp(ea.p[sel][..., 0].abs(), min=1.0)
    err = ((eb.p[sel] - ea.p[sel]).abs().amax(-1) / floor).max().item()
    assert err < 1e-7, err
    ferr = ((eb.factor[sel] - ea.factor[sel]).abs() / ea.factor[sel].abs()).max().item()
    assert ferr < 1e-7, ferr
    assert torch.equal(ea.volume, eb.volume)


@pytest.mark.parametrize("beams", ["asymmetric", "random"])
@pytest.mark.parametrize("builder", [P.tt, P.precision])
def test_ff_per_event_beams(torch, builder, beams):
    """Per-event beam energies in FP32-pair arithmetic: the beams and the uniform and
    Breit-Wigner constants in float-float (the others, sqrt(s) and the volume in FP64), the
    walk in float-float; against the oracle at the same bar."""
    from gpu_phs_gb300.api import PhaseSpace
    proc = builder()
    n = 50_000
    sq = proc.sqrts
    x = uniform_x(13, n, proc.n_x)
    rng = np.random.default_rng(3)
    if beams == "asymmetric":
        E1, E2 = np.full(n, 0.6 * sq), np.full(n, 0.42 * sq)
    else:
        E1, E2 = rng.uniform(0.3, 0.7, n) * sq, rng.uniform(0.3, 0.7, n) * sq
    r = oracle.Oracle(proc, sq).generate(x, E1=E1, E2=E2)
    ps = PhaseSpace(proc)
    ps.set_precision(1)
    ev = ps.generate_beams(torch.from_numpy(x).cuda(), torch.from_numpy(E1).cuda(),
                           torch.from_numpy(E2).cuda())
    torch.cuda.synchronize()
    got = (ev.p.cpu().numpy(), ev.factor.cpu().numpy(), ev.volume.cpu().numpy(), ev.ok.cpu().numpy())
    check(got, r.p, r.factor, r.volume, r.ok, sq)


@pytest.mark.parametrize("builder", [P.ww, P.tt, P.precision])
def test_ff_per_event_beams_wide_energy_range(torch, builder):
    """FP32 pairs with beam energies log-uniform in [1e-4, 0.7] sqrt(s) each (wide_beams:
    negative Breit-Wigner ranges, the float-float series and its FP64 fallback, tiny s).
    Bar: ok flags bit-exact with the oracle; momenta (against the event's own sqrt(s)) and
    factors within 1e-7, or 1024 times the oracle's own change under perturbations of the
    FP64 rounding size (oracle_sensitivity; float-float carries about 2^-48, 16 FP64 ulps,
    times the FP64 test's 64) on the events near a threshold that the walk decides in
    float-float (margins above 1e-5)."""
    from gpu_phs_gb300.api import PhaseSpace
    proc = builder()
    n = 50_000
    x = uniform_x(15, n, proc.n_x)
    E1, E2 = wide_beams(n, proc.sqrts, 5)
    sq = 2.0 * np.sqrt(E1 * E2)
    o = oracle.Oracle(proc, proc.sqrts)
    r = o.generate(x, E1=E1, E2=E2)
    ps = PhaseSpace(proc)
    ps.set_precision(1)
    ev = ps.generate_beams(torch.from_numpy(x).cuda(), torch.from_numpy(E1).cuda(),
                           torch.from_numpy(E2).cuda())
    torch.cuda.synchronize()
    p, f, v, ok = (ev.p.cpu().numpy(), ev.factor.cpu().numpy(), ev.volume.cpu().numpy(),
                   ev.ok.cpu().numpy())
    assert_within_conditioning(p, f, ok, o, x, r, sq, E1, E2, TOL, 1024)
    assert np.allclose(v, r.volume, rtol=1e-15, atol=0)


def test_ff_per_event_beams_exact_path(torch):
    """bwbw's 61 channels with per-event beams in FP32-pair arithmetic: its 16 friend
    channels and the events near kinematic limits go through the exact path per event."""
    from gpu_phs_gb300.api import PhaseSpace
    z = golden("whizard_bwbw")
    proc = load_process(z)
    x = np.ascontiguousarray(z["x"])
    n = x.shape[0]
    rng = np.random.default_rng(8)
    E1, E2 = rng.uniform(350, 650, n), rng.uniform(350, 650, n)
    counts = counts_of(z["channel"], proc.n_channels)
    r = oracle.Oracle(proc, 1000.0).generate(x, z["channel"], E1=E1, E2=E2)
    ps = PhaseSpace(proc)
    ps.set_precision(1)
    ev = ps.generate_beams(torch.from_numpy(x).cuda(), torch.from_numpy(E1).cuda(),
                           torch.from_numpy(E2).cuda(), counts)
    torch.cuda.synchronize()
    got = (ev.p.cpu().numpy(), ev.factor.cpu().numpy(), ev.volume.cpu().numpy(), ev.ok.cpu().numpy())
    check(got, r.p, r.factor, r.volume, r.ok, 1000.0)


def test_ff_per_event_beams_fp64_candidates(torch):
    """With per-event beams the FP32-pair autotuner may pick the FP64 compacting kernel
    (variants 2 and 3 there): pinned, it gives the FP64 path's bits."""
    from gpu_phs_gb300.api import PhaseSpace, philox_x
    proc = P.precision()
    n = 100_000
    x = philox_x(n, proc.n_x, seed=21)
    g = torch.Generator(device="cuda").manual_seed(6)
    E1 = proc.sqrts * (0.3 + 0.4 * torch.rand(n, generator=g, device="cuda", dtype=torch.float64))
    E2 = proc.sqrts * (0.3 + 0.4 * torch.rand(n, generator=g, device="cuda", dtype=torch.float64))
    ref = PhaseSpace(proc)
    ref.set_variants(-1, 0)
    r = ref.generate_beams(x, E1, E2)
    for v in (2, 3):
        ps = PhaseSpace(proc)
        ps.set_precision(1)
        ps.set_variants(v, -1)
        ev = ps.generate_beams(x, E1, E2)
        torch.cuda.synchronize()
        for a, b in ((r.p, ev.p), (r.factor, ev.factor), (r.volume, ev.volume), (r.ok, ev.ok)):
            assert torch.equal(a, b)
