import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built_oracles():
    """The CPU oracle is a few ms of gcc; build it if this checkout has no copy yet."""
    so = os.path.join(ROOT, "oracle", "_build", "libphsoracle.so")
    if not os.path.exists(so):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)


def load_process(z, prefix=""):
    from gpu_phs_gb300.processes import Process
    meta = z[prefix + "meta"]
    return Process(int(meta[0]), int(meta[1]), z[prefix + "d1"], z[prefix + "d2"],
                   z[prefix + "has_children"], z[prefix + "friends"], z[prefix + "map_ids"],
                   z[prefix + "map_masses"], z[prefix + "map_widths"], z[prefix + "flv_masses"],
                   z[prefix + "flv_widths"], n_x=int(meta[2]),
                   sqrts=float(z[prefix + "sqrts_nominal"][0]))


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


REFCPU_FIXTURES = ["ww", "tt", "precision"] + [f"random_n{n}" for n in range(3, 9)]


def momentum_rel_err(p, q, sqrts=None):
    """Per event and particle: max_mu |p - q| / max(E_q, 1e-3 sqrt(s)).

    The floor keeps the measure meaningful for soft particles in strongly boosted frames,
    whose components are differences of terms of order gamma^2 E: there two correct FP64
    evaluations that differ only in rounding order (e.g. FMA contraction of the reference
    CPU path itself) disagree by ~1e-12 of the particle's energy but ~1e-15 of sqrt(s)."""
    floor = 1e-3 * sqrts if sqrts is not None else 0.0
    e = np.maximum(np.maximum(np.abs(q[..., 0]), floor), 1e-300)
    return (np.abs(p - q).max(axis=-1) / e)


def wide_beams(n, sqrts, seed):
    """Beam energies log-uniform in [1e-4, 0.7] sqrt(s) each: collision energies from far
    below the resonances' masses (negative Breit-Wigner ranges) up to where the range in
    widths passes 1024 (the three-term atan series), lab boosts up to gamma ~ 40, tiny s."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(1e-4), np.log(0.7)
    return (sqrts * np.exp(rng.uniform(lo, hi, n)), sqrts * np.exp(rng.uniform(lo, hi, n)))


def oracle_sensitivity(o, x, r, sq, E1=None, E2=None, trials=2, seed=2, nudge=2, channels=None):
    """The oracle's own change under perturbations of the size a device's rounding makes:
    one-ulp perturbations of its x inputs (each entry times 1 +- 2^-52, `trials` draws)
    and every value a transcendental function returns on the mapping path moved by
    +-1 ... +-`nudge` ulps (Oracle.generate(nudge=...): the maps' own tan, exp and log and,
    with per-event beams, the constants formed per event such as the Breit-Wigner bound
    a1 = atan(u), which a device evaluates with its own library within a few ulps of
    glibc's).  The
    reference's Breit-Wigner map is ill-conditioned in both far below its pole: one ulp of
    a1 moves z and tan(z) by (1 + u^2) ulps, and msq = m (m + w tan z) cancels.  Per event
    the largest momentum change (the measure of momentum_rel_err against the event's
    sqrt(s) `sq`) and relative factor change; infinite where the ok flag moved.  Near a
    kinematic threshold the Kallen function amplifies all of these.  Every step from 1 to
    `nudge` runs: the response is not monotonic (a2 = (a1 - a0) m w / s and tan z move
    with a1 and can cancel at one step and not at the next)."""
    rng = np.random.default_rng(seed)
    n = x.shape[0]
    sp = np.zeros(n)
    sf = np.zeros(n)
    flips = np.zeros(n, bool)
    runs = [dict(x=x * (1 + rng.choice([-1.0, 1.0], x.shape) * 2.0 ** -52))
            for _ in range(trials)]
    runs += [dict(x=x, nudge=k * sign) for k in range(1, nudge + 1) for sign in (1, -1)]
    for kw in runs:
        q = o.generate(kw.pop("x"), channels, E1=E1, E2=E2, **kw)
        flips |= q.ok != r.ok
        both = (q.ok == 1) & (r.ok == 1)
        sp[both] = np.maximum(sp[both], momentum_rel_err(q.p[both], r.p[both],
                                                         sq[both][:, None]).max(axis=1))
        sf[both] = np.maximum(sf[both], np.abs(q.factor[both] - r.factor[both]) /
                              np.abs(r.factor[both]))
    sp[flips] = np.inf
    sf[flips] = np.inf
    return sp, sf


def assert_within_conditioning(p, f, ok, o, x, r, sq, E1, E2, bar, ulps, channels=None):
    """ok flags bit-exact with the oracle; per event, momenta (against the event's own
    sqrt(s)) and factors within max(bar, ulps x the oracle's own change under perturbations
    of the device's rounding size, oracle_sensitivity); zero momenta and factor where
    ok = 0."""
    assert int(np.count_nonzero(ok != r.ok)) == 0
    sel = r.ok == 1
    assert sel.sum() > 0
    sp, sf = oracle_sensitivity(o, x, r, sq, E1, E2, channels=channels)
    ep = momentum_rel_err(p[sel], r.p[sel], sq[sel][:, None]).max(axis=1)
    ef = np.abs(f[sel] - r.factor[sel]) / np.abs(r.factor[sel])
    tp = np.maximum(bar, ulps * sp[sel])
    tf = np.maximum(bar, ulps * sf[sel])
    wide = (ep > bar) | (ef > bar)
    print(f"max momentum error {ep.max():.3g}, factor {ef.max():.3g}; {int(wide.sum())} of "
          f"{int(sel.sum())} ok events above {bar:g}; worst error / bound: momentum "
          f"{np.max(ep / tp):.3g}, factor {np.max(ef / tf):.3g}")
    ev = np.flatnonzero(sel)
    i, j = int(np.argmax(ep / tp)), int(np.argmax(ef / tf))
    assert np.all(ep <= tp), (f"momentum: {ep[i] / tp[i]:.3g} x the bound at event {ev[i]} "
                              f"(sqrt(s) {sq[ev[i]]:.4g}, error {ep[i]:.3g})")
    assert np.all(ef <= tf), (f"factor: {ef[j] / tf[j]:.3g} x the bound at event {ev[j]} "
                              f"(sqrt(s) {sq[ev[j]]:.4g}, error {ef[j]:.3g})")
    assert np.all(p[~sel] == 0) and np.all(f[~sel] == 0)


def all_maps_process(seed, n_out, n_channels):
    """random_process trees with some of their mappings swapped for the kinds it does not
    draw: Breit-Wigner -> STEP_E or STEP_H, collinear -> RADIATION, t- -> u-channel, so
    that every mapping's per-event constants run (n_out >= 4 draws all nine kinds)."""
    rng = np.random.default_rng(seed)
    from gpu_phs_gb300 import processes as P
    proc = P.random_process(rng, n_out, n_channels, 1000.0)
    ids = proc.map_ids.copy()
    for c in range(ids.shape[0]):
        for j in range(ids.shape[1]):
            t = ids[c, j]
            if t == P.MAP_SCHANNEL and rng.random() < 0.5:
                ids[c, j] = P.MAP_STEP_E if rng.random() < 0.5 else P.MAP_STEP_H
            elif t == P.MAP_COLLINEAR and rng.random() < 0.5:
                ids[c, j] = P.MAP_RADIATION
            elif t == P.MAP_TCHANNEL and rng.random() < 0.5:
                ids[c, j] = P.MAP_UCHANNEL
    proc.map_ids = ids
    return proc


def counts_of(channels, n_channels):
    return np.bincount(channels, minlength=n_channels).astype(np.int64)
