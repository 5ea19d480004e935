"""The device x grid of the warm-up (rng.cpp): weight updates against the restated
update_weights, samples against the restated inverse distribution function, the sampled
density against the weights, and the warm-up raising the ok fraction."""
import numpy as np
import pytest

from gpu_phs_gb300 import processes as P
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_update_and_sample_match_restatement(torch):
    from gpu_phs_gb300.api import Grid, philox_x
    proc = P.tt()
    n_ch, n_x = 3, proc.n_x
    counts = np.array([4000, 0, 2500], np.int64)
    n = int(counts.sum())
    g = Grid(n_ch, n_x)
    w0 = g.weights()
    assert np.all(w0 == 0.1)
    x = philox_x(n, n_x, seed=5)
    ok = (torch.rand(n, device="cuda", generator=torch.Generator(device="cuda").manual_seed(1)) < 0.7).to(torch.uint8)
    g.update(x, ok, counts)
    w = g.weights()
    ref = oracle.grid_update(w0, x.cpu().numpy(), counts, ok.cpu().numpy())
    assert np.array_equal(w, ref)
    assert np.all(w[1] == 0.1)                     # no events: weights kept
    xs = g.sample(n, counts, seed=9)
    u = philox_x(n, n_x, seed=9).cpu().numpy()
    sel = slice(0, 300)
    assert np.array_equal(xs.cpu().numpy()[sel], oracle.grid_sample(w, u, counts)[sel])
    assert xs.min().item() >= 0.0 and xs.max().item() < 1.0


def test_sampled_density_follows_weights(torch):
    from gpu_phs_gb300.api import Grid
    g = Grid(1, 2)
    x = torch.empty((1 << 20, 2), dtype=torch.float64, device="cuda")
    # a grid with an empty bin and a heavy one, set through an update from chosen x
    xs = np.zeros((1000, 2))
    xs[:500, :] = 0.05
    xs[500:800, :] = 0.35
    xs[800:, :] = 0.95
    g.update(torch.from_numpy(xs).cuda(), torch.ones(1000, dtype=torch.uint8, device="cuda"))
    w = g.weights()[0, 0]
    assert np.allclose(w, [0.5, 0, 0, 0.3, 0, 0, 0, 0, 0, 0.2])
    g.sample(1 << 20, None, seed=2, out=x)
    b = np.clip((x.cpu().numpy() * 10).astype(int), 0, 9)
    freq = np.bincount(b[:, 0], minlength=10) / (1 << 20)
    assert np.abs(freq - w).max() < 3e-3
    assert freq[1] == 0 and freq[8] == 0


def test_warm_up_raises_ok_fraction(torch):
    from gpu_phs_gb300.api import Grid, PhaseSpace, precondition
    # the precision configuration: ~4 % of uniform x pass the kinematic test
    proc = P.precision()
    ps = PhaseSpace(proc, proc.sqrts / 2, proc.sqrts / 2)
    g = Grid(1, proc.n_x)
    fr = precondition(ps, g, n_trials=4, n_per_channel=1 << 18, seed=11)
    assert fr[0] < 0.06 and fr[-1] > 2 * fr[0]
