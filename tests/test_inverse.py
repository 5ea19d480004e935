"""The inverse map in the CPU oracle: all-channel factors and x of generated events
(phs.cu:1499-1554), pinned against Whizard's own all_factors in the sample files, and its
round trip through the forward map."""
import numpy as np
import pytest

from conftest import golden, load_process
from gpu_phs_gb300 import processes as P
from gpu_phs_gb300.philox import uniform_x
from oracle import oracle


def _decimals(name):
    return 4 if name == "ttH" else 7


@pytest.mark.parametrize("name", ["ttH", "bwbw"])
def test_oracle_inverse_vs_whizard_all_factors(name):
    z = golden(f"whizard_{name}")
    proc = load_process(z)
    o = oracle.Oracle(proc, 1000.0)
    r = o.generate(z["x"], z["channel"])
    fac, xo = o.inverse(r.p, z["channel"], r.ok, x_own=z["x"], factor_own=r.factor)
    g = z["all_factors"]
    assert fac.shape == g.shape
    # printed to a fixed number of decimals; x (9 decimals) moves the momenta by ~1e-4 GeV
    tol = 0.5 * 10.0 ** -_decimals(name) + 2e-3 * np.abs(g)
    assert np.all(np.abs(fac - g) <= tol)
    big = np.abs(g) > 2e4 * 10.0 ** -_decimals(name)  # print rounding below 2.5e-5
    if name == "bwbw":
        assert big.sum() > 30000
        assert (np.abs(fac - g)[big] / np.abs(g[big])).max() < 1e-4
    n = len(z["channel"])
    assert np.array_equal(xo[z["channel"], np.arange(n)], z["x"])


def test_bwbw_all_factors_pin_the_friend_inverse():
    z = golden("whizard_bwbw")
    proc = load_process(z)
    r = oracle.Oracle(proc, 1000.0).generate(z["x"], z["channel"])
    bare = load_process(z)
    bare.friends = np.zeros_like(bare.friends)
    fac, _ = oracle.Oracle(bare, 1000.0).inverse(r.p, z["channel"], r.ok, x_own=z["x"],
                                                 factor_own=r.factor)
    g = z["all_factors"]
    flagged = z["hasfriends"].astype(bool)
    off = np.abs(fac - g) > 0.5e-7 + 2e-3 * np.abs(g)
    assert off[:, flagged].sum() > 1000 and off[:, ~flagged].sum() == 0


@pytest.mark.parametrize("builder", [P.ww, P.tt, P.precision])
def test_oracle_round_trip(builder):
    """Inverting the generating channel gives back its x and factor."""
    proc = builder()
    x = uniform_x(21, 3000, proc.n_x)
    o = oracle.Oracle(proc, proc.sqrts)
    r = o.generate(x)
    fac, xo = o.inverse(r.p, None, r.ok)
    ok = r.ok == 1
    nu = 3 * proc.n_out - 4
    assert np.abs(xo[0][ok, :nu] - x[ok, :nu]).max() < 1e-7
    rel = np.abs(fac[ok, 0] / r.factor[ok] - 1)
    assert np.median(rel) < 1e-12 and rel.max() < 1e-5
    assert np.all(fac[~ok] == 0) and np.all(xo[0][~ok, :nu] == 0)


def test_oracle_round_trip_random_trees():
    rng = np.random.default_rng(8)
    for n_out in range(3, 9):
        proc = P.random_process(rng, n_out, 3, 1000.0, name=f"inv{n_out}")
        x = uniform_x(30 + n_out, 2000, proc.n_x)
        ch = np.arange(2000, dtype=np.int32) * proc.n_channels // 2000
        o = oracle.Oracle(proc, 1000.0)
        r = o.generate(x, ch)
        fac, xo = o.inverse(r.p, ch, r.ok)
        ok = r.ok == 1
        nu = 3 * n_out - 4
        own = xo[ch, np.arange(2000)]
        assert np.median(np.abs(own[ok, :nu] - x[ok, :nu])) < 1e-12
        ownf = fac[np.arange(2000), ch]
        assert np.median(np.abs(ownf[ok] / r.factor[ok] - 1)) < 1e-12


def test_oracle_inverse_lab_frame():
    """Asymmetric beams: the inverse boosts the lab momenta back to the CM frame."""
    proc = P.tt()
    x = uniform_x(9, 2000, proc.n_x)
    o = oracle.Oracle(proc, proc.sqrts)
    E1, E2 = np.full(2000, 700.0), np.full(2000, 400.0)
    r = o.generate(x, E1=E1, E2=E2)
    fac, xo = o.inverse(r.p, None, r.ok, E1=E1, E2=E2)
    ok = r.ok == 1
    nu = 3 * proc.n_out - 4
    assert np.median(np.abs(xo[0][ok, :nu] - x[ok, :nu])) < 1e-12
    assert np.median(np.abs(fac[ok, 0] / r.factor[ok] - 1)) < 1e-12
