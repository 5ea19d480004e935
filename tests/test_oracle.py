"""The CPU oracle (oracle/phs_oracle.c) pinned against the reference's golden vectors
(the Whizard sample files) and against outputs of the reference's own phs_cpu.cpp."""
import os

import numpy as np
import pytest

from conftest import REFCPU_FIXTURES, golden, load_process, momentum_rel_err
from gpu_phs_gb300 import processes as P
from gpu_phs_gb300.philox import philox4x32_10, uniform_x
from oracle import oracle


def test_philox_known_answers():
    # Random123 kat_vectors for philox4x32_10
    cases = [([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
             ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
             ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
              [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1])]
    for ctr, key, want in cases:
        got = philox4x32_10(np.array([ctr], np.uint32), np.array(key, np.uint32))[0]
        assert [int(v) for v in got] == want


def test_philox_stream_windows():
    a = uniform_x(5, 40, 7)
    assert np.array_equal(a[13:29], uniform_x(5, 16, 7, first_event=13))
    assert a.min() >= 0 and a.max() < 1


@pytest.mark.parametrize("name", ["ttH", "bwbw"])
def test_oracle_vs_whizard_golden(name):
    z = golden(f"whizard_{name}")
    proc = load_process(z)
    r = oracle.Oracle(proc, 1000.0).generate(z["x"], z["channel"])
    assert np.array_equal(r.ok, z["ok"].astype(np.uint8))
    # x is printed with 9 decimals, which limits momentum agreement to ~1e-4 GeV; the
    # friend-boost channels of bwbw (16 of 61) are included
    dp = np.abs(r.p - z["p_out"])
    assert dp.max() < 1e-3
    assert np.allclose(r.volume, z["volume"], rtol=1e-14, atol=0)
    # factors are printed with a fixed number of decimals (4 for ttH, 7 for bwbw)
    f, g = r.factor, z["factor"]
    dec = 4 if name == "ttH" else 7
    assert np.all(np.abs(f - g) <= 2e-3 * np.abs(g) + 0.5 * 10.0 ** -dec)


def test_friend_channels_need_the_friend_boost():
    """Without the friend table the flagged bwbw trees miss Whizard's momenta by far: the
    golden events pin the friend boost itself, not just the friend-free channels."""
    z = golden("whizard_bwbw")
    proc = load_process(z)
    assert proc.friends.any()
    flagged = z["hasfriends"][z["channel"]] == 1
    assert flagged.sum() == 149
    proc.friends = np.zeros_like(proc.friends)
    r = oracle.Oracle(proc, 1000.0).generate(z["x"], z["channel"])
    assert np.abs(r.p - z["p_out"])[flagged].max() > 10.0


@pytest.mark.parametrize("name", REFCPU_FIXTURES)
def test_oracle_bitexact_vs_reference_fixture(name):
    z = golden(f"refcpu_{name}")
    proc = load_process(z)
    x = uniform_x(int(z["seed"][0]), len(z["ok"]), proc.n_x)
    assert x.sum() == z["x_checksum"][0]
    r = oracle.Oracle(proc, float(z["sqrts"][0])).generate(x, z["channel"])
    assert np.array_equal(r.ok, z["ok"])
    ok = r.ok == 1
    assert np.array_equal(r.p[ok], z["p"][ok])
    assert np.array_equal(r.factor[ok], z["factor"][ok])
    assert np.array_equal(r.volume[ok], z["volume"][ok])
    assert np.all(r.p[~ok] == 0) and np.all(r.factor[~ok] == 0)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference CPU path not built here")
@pytest.mark.parametrize("case", ["nested_10", "nested_12", "all_maps_5", "all_maps_8"])
def test_oracle_bitexact_vs_live_reference_largest_and_every_mapping(case):
    """The API's largest trees (10 and 12 outgoing particles, nested resonances) and random
    channels with every mapping kind (step, radiation and u-channel maps swapped in),
    several channels per process: the oracle against the reference build, bit for bit."""
    from conftest import all_maps_process
    k = int(case.split("_")[-1])
    proc = P.nested_resonances(k) if case.startswith("nested") else all_maps_process(k + 2, k, 6)
    n = 6000
    ch = np.repeat(np.arange(proc.n_channels, dtype=np.int32), n // proc.n_channels)
    x = uniform_x(99, ch.size, proc.n_x)
    r = oracle.Oracle(proc, 1000.0).generate(x, ch)
    q = oracle.RefCPU(proc, 1000.0).generate(x, ch)
    assert np.array_equal(r.ok, q.ok)
    ok = r.ok == 1
    assert ok.sum() > 200
    assert np.array_equal(r.p[ok], q.p[ok])
    assert np.array_equal(r.factor[ok], q.factor[ok])
    assert np.array_equal(r.volume[ok], q.volume[ok])


@pytest.mark.skipif(not oracle.ref_available(), reason="reference CPU path not built here")
@pytest.mark.parametrize("builder", [P.ww, P.tt, P.precision])
def test_oracle_bitexact_vs_live_reference(builder):
    proc = builder()
    x = uniform_x(77, 20000, proc.n_x)
    r = oracle.Oracle(proc, proc.sqrts).generate(x)
    q = oracle.RefCPU(proc, proc.sqrts).generate(x)
    assert np.array_equal(r.ok, q.ok)
    ok = r.ok == 1
    assert np.array_equal(r.p[ok], q.p[ok])
    assert np.array_equal(r.factor[ok], q.factor[ok])
    assert np.array_equal(r.volume[ok], q.volume[ok])


def test_oracle_invariants_tt():
    proc = P.tt()
    x = uniform_x(3, 5000, proc.n_x)
    r = oracle.Oracle(proc, 1000.0).generate(x)
    ok = r.ok == 1
    assert 0.9 < ok.mean() < 1.0          # some events fall outside the kinematic limits
    tot = r.p[ok].sum(axis=1)
    assert np.allclose(tot[:, 0], 1000.0, rtol=1e-12)
    assert np.abs(tot[:, 1:]).max() < 1e-9
    m2 = r.p[ok, :, 0] ** 2 - (r.p[ok, :, 1:] ** 2).sum(-1)
    masses = proc.flv_masses[2:] ** 2
    assert np.abs(m2 - masses).max() < 1e-6


def test_oracle_beams_uniform_matches_scalar():
    proc = P.ww()
    x = uniform_x(9, 1000, proc.n_x)
    o = oracle.Oracle(proc, 500.0)
    a = o.generate(x)
    b = o.generate(x, E1=np.full(1000, 250.0), E2=np.full(1000, 250.0))
    assert np.array_equal(a.ok, b.ok)
    assert np.array_equal(a.p, b.p)
    assert np.array_equal(a.factor, b.factor)


def test_oracle_lab_boost_conserves_beam_momentum():
    proc = P.ww()
    x = uniform_x(10, 2000, proc.n_x)
    E1, E2 = 300.0, 200.0
    r = oracle.Oracle(proc, 500.0).generate(x, E1=np.full(2000, E1), E2=np.full(2000, E2))
    ok = r.ok == 1
    tot = r.p[ok].sum(axis=1)
    assert np.allclose(tot[:, 0], E1 + E2, rtol=1e-12)
    assert np.allclose(tot[:, 3], E1 - E2, atol=1e-9)


def test_oracle_rejects_bad_trees():
    proc = P.ww()
    bad = proc.subset([0])
    bad.d1 = bad.d1.copy()
    bad.d1[0, 2] = 1
    bad.d2 = bad.d2.copy()
    bad.d2[0, 2] = 4            # code 3 -> (1, 4): does not OR to 3
    with pytest.raises(ValueError):
        oracle.Oracle(bad, 500.0)
    bad = proc.subset([0])
    bad.map_ids = bad.map_ids.copy()
    bad.map_ids[0, 2] = 99      # ONSHELL has no implementation
    with pytest.raises(ValueError):
        oracle.Oracle(bad, 500.0)


SAMPLES = os.path.join(oracle.reference_dir(), "samples")


@pytest.mark.skipif(not os.path.isdir(SAMPLES), reason="reference samples absent")
def test_ref_reader_matches_fixture():
    from gpu_phs_gb300.refformat import read_ref
    proc, fr, ev = read_ref(os.path.join(SAMPLES, "ttH.ref"))
    z = golden("whizard_ttH")
    assert np.array_equal(proc.d1, z["d1"]) and np.array_equal(proc.map_ids, z["map_ids"])
    assert len(ev.ok) == 999 and ev.x.shape == (999, 5)


def test_oracle_philox_matches_numpy_stream():
    """The threaded C Philox of the oracle library (used for full-size comparisons) gives
    the stream of gpu_phs_gb300.philox.uniform_x, at odd offsets and 64-bit seeds too."""
    for n, nx, e0, seed in [(1000, 14, 0, 42), (777, 5, 123, 7), (1, 3, 9, 1234),
                            (50_001, 16, 3, 2**40 + 5), (0, 8, 0, 1)]:
        a = oracle.uniform_x(seed, n, nx, e0, threads=4)
        assert np.array_equal(a, uniform_x(seed, n, nx, first_event=e0)), (n, nx, e0)


def test_oracle_condition_output_leaves_results_unchanged():
    """generate(condition=True) returns the same bits plus the Kallen condition kappa:
    >= 1 for every ok event of the tt tree (each branch has a sum of three terms over lda,
    one of them >= lda), and largest for the events closest to a threshold."""
    proc = P.tt()
    x = uniform_x(77, 20_000, proc.n_x)
    o = oracle.Oracle(proc, proc.sqrts)
    a, b = o.generate(x), o.generate(x, condition=True)
    for f in ("p", "factor", "volume", "ok"):
        assert np.array_equal(getattr(a, f), getattr(b, f))
    k = b.kappa[b.ok == 1]
    assert (k >= 1.0).all() and np.isfinite(k).all()
    assert (b.kappa[b.ok == 0] >= 0).all()


def test_oracle_nudge_is_a_probe_that_resets():
    """generate(nudge=k) (a sensitivity probe) moves the transcendental values on the
    mapping path by k ulps: nudge=0 is the reference's arithmetic bit for bit, a nudge
    changes some momenta by a little and is reset after the call; with uniform beams it
    moves the maps' own values and leaves the constants (and so the volumes) alone."""
    proc = P.ww()
    n = 20_000
    x = uniform_x(78, n, proc.n_x)
    rng = np.random.default_rng(9)
    E1, E2 = rng.uniform(100, 350, n), rng.uniform(100, 350, n)
    o = oracle.Oracle(proc, proc.sqrts)
    a = o.generate(x, E1=E1, E2=E2)
    b = o.generate(x, E1=E1, E2=E2, nudge=0)
    for f in ("p", "factor", "volume", "ok"):
        assert np.array_equal(getattr(a, f), getattr(b, f))
    c = o.generate(x, E1=E1, E2=E2, nudge=2)
    sel = (a.ok == 1) & (c.ok == 1)
    sq = 2.0 * np.sqrt(E1 * E2)
    d = momentum_rel_err(c.p[sel], a.p[sel], sq[sel][:, None]).max(axis=1)
    assert d.max() > 0 and np.median(d) < 1e-13
    assert np.array_equal(a.volume, c.volume)
    again = o.generate(x, E1=E1, E2=E2)
    assert np.array_equal(again.p, a.p)
    u0, u1 = o.generate(x), o.generate(x, nudge=1)
    sel = (u0.ok == 1) & (u1.ok == 1)
    du = momentum_rel_err(u1.p[sel], u0.p[sel], proc.sqrts).max(axis=1)
    assert du.max() > 0 and np.median(du) < 1e-13
    assert np.array_equal(u0.volume, u1.volume)
    assert np.array_equal(o.generate(x).p, u0.p)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference CPU path not built here")
@pytest.mark.parametrize("case", ["ww", "tt", "precision", "all_maps_4", "all_maps_6"])
def test_oracle_per_event_constants_bitexact_vs_live_reference(case):
    """The oracle's per-event path (constants formed for each event's sqrt(s), as with
    per-event beams) against the reference's phs_cpu.cpp set up at that sqrt(s), over three
    decades of energy: bit for bit.  E1 = E2 = sqrt(s)/2 gives each event exactly that
    sqrt(s) (sqrt of a correctly rounded square is the number itself)."""
    from conftest import all_maps_process
    if case.startswith("all_maps"):
        proc = all_maps_process(500 + int(case[-1]), int(case[-1]), 4)
    else:
        proc = getattr(P, case)()
    n = 4000
    ch = np.repeat(np.arange(proc.n_channels, dtype=np.int32), n // proc.n_channels)
    x = uniform_x(88, ch.size, proc.n_x)
    o = oracle.Oracle(proc, proc.sqrts)
    for f in (1e-3, 1e-2, 0.05, 0.2, 0.6, 1.0, 1.4):
        sq = proc.sqrts * f
        E = np.full(ch.size, sq / 2)
        assert np.all(2.0 * np.sqrt(E * E) == sq)
        r = o.generate(x, ch, E1=E, E2=E)
        q = oracle.RefCPU(proc, sq).generate(x, ch)
        assert np.array_equal(r.ok, q.ok), f"sqrt(s) = {sq}"
        ok = r.ok == 1
        assert np.array_equal(r.p[ok], q.p[ok]), f"sqrt(s) = {sq}"
        assert np.array_equal(r.factor[ok], q.factor[ok]), f"sqrt(s) = {sq}"
        assert np.array_equal(r.volume[ok], q.volume[ok]), f"sqrt(s) = {sq}"
