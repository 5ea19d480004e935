"""The adjoint kernel against FP64 central finite differences (h = 1e-6) of the forward
kernel, on the tt tree, excluding events within 1e-4 of a kinematic limit."""
import numpy as np
import pytest

from gpu_phs_gb300 import processes as P
from gpu_phs_gb300.philox import uniform_x

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def margins(p, proc):
    """Smallest relative distance of each event to a kinematic limit, from its momenta:
    (m - m1 - m2)/m and (m_max - m)/m_max over the internal branches."""
    R = (1 << proc.n_out) - 1
    d1, d2, hc = proc.d1[0], proc.d2[0], proc.has_children[0]
    sqrts = proc.sqrts
    m_tot = proc.flv_masses[2:].sum()
    out = np.full(p.shape[0], np.inf)

    def leaves(code):
        return [j for j in range(proc.n_out) if code >> j & 1]

    def mass(code):
        q = p[:, leaves(code)].sum(axis=1)
        return np.sqrt(np.maximum(q[:, 0] ** 2 - (q[:, 1:] ** 2).sum(-1), 0))

    for code in range(1, R + 1):
        if not hc[code - 1]:
            continue
        m = mass(code)
        m1, m2 = mass(int(d1[code - 1])), mass(int(d2[code - 1]))
        # a massless branch (m = 0) sits on its threshold: margin 0
        rel = np.divide(m - m1 - m2, m, out=np.zeros_like(m), where=m > 0)
        out = np.minimum(out, rel)
        if code != R:
            m_min = proc.flv_masses[2:][leaves(code)].sum()
            m_max = sqrts - m_tot + m_min
            out = np.minimum(out, (m_max - m) / m_max)
    return out


def loss(torch, ps, x, pbar, jbar):
    ev = ps.generate(x)
    ok = ev.ok.bool()
    lj = torch.where(ok, torch.log(torch.where(ok, ev.factor, torch.ones_like(ev.factor))), 0.0)
    return (pbar * ev.p).sum(dim=(1, 2)) + jbar * lj, ok


def test_adjoint_x_against_finite_differences(torch):
    from gpu_phs_gb300.api import PhaseSpace
    proc = P.tt()
    n, h = 10_000, 1e-6
    x = torch.from_numpy(uniform_x(404, n, proc.n_x)).cuda()
    ps = PhaseSpace(proc, 500.0, 500.0)
    g = torch.Generator(device="cuda").manual_seed(1)
    pbar = torch.randn((n, proc.n_out, 4), generator=g, device="cuda", dtype=torch.float64)
    jbar = torch.randn(n, generator=g, device="cuda", dtype=torch.float64)
    xbar, _ = ps.vjp(x, pbar, jbar)
    ev = ps.generate(x)
    keep = ev.ok.bool().cpu().numpy() & (margins(ev.p.cpu().numpy(), proc) > 1e-4)
    keep &= ((x > 2 * h) & (x < 1 - 2 * h)).all(dim=1).cpu().numpy()
    fd = torch.zeros_like(x)
    for k in range(proc.n_x):
        xp, xm = x.clone(), x.clone()
        xp[:, k] += h
        xm[:, k] -= h
        lp, okp = loss(torch, ps, xp, pbar, jbar)
        lm, okm = loss(torch, ps, xm, pbar, jbar)
        fd[:, k] = (lp - lm) / (2 * h)
        keep &= (okp & okm).cpu().numpy()
    a, b = xbar.cpu().numpy()[keep], fd.cpu().numpy()[keep]
    scale = np.abs(b).max(axis=1, keepdims=True) + 1.0
    rel = np.abs(a - b) / scale
    assert keep.sum() > 0.9 * n
    assert np.median(rel) < 1e-7
    assert np.quantile(rel, 0.999) < 1e-4, np.quantile(rel, [0.5, 0.99, 0.999, 1.0])


def test_adjoint_parameters_against_finite_differences(torch):
    """d/d(m_t, Gamma_t, m_W, Gamma_W): the t and tbar (W+ and W-) branches share them."""
    from gpu_phs_gb300.api import PhaseSpace
    base = P.tt()
    n = 10_000
    x = torch.from_numpy(uniform_x(405, n, base.n_x)).cuda()
    ps = PhaseSpace(base, 500.0, 500.0)
    g = torch.Generator(device="cuda").manual_seed(2)
    pbar = torch.randn((n, base.n_out, 4), generator=g, device="cuda", dtype=torch.float64)
    jbar = torch.randn(n, generator=g, device="cuda", dtype=torch.float64)
    _, thbar = ps.vjp(x, pbar, jbar)
    ev = ps.generate(x)
    keep = ev.ok.bool().cpu().numpy() & (margins(ev.p.cpu().numpy(), base) > 1e-4)
    codes = {"m_t": ([0b000111, 0b111000], 0), "G_t": ([0b000111, 0b111000], 1),
             "m_W": ([0b000110, 0b110000], 0), "G_W": ([0b000110, 0b110000], 1)}
    # msq x index of each branch (post-order over non-root internals): W+, t, W-, tbar
    slot = {0b000110: 0, 0b000111: 1, 0b110000: 2, 0b111000: 3}
    for name, (branch_codes, col) in codes.items():
        ad = sum(thbar[:, slot[c], col] for c in branch_codes)
        val = base.map_masses[0, branch_codes[0] - 1] if col == 0 else base.map_widths[0, branch_codes[0] - 1]
        h = 1e-6 * val
        ls = []
        oks = []
        for sgn in (1, -1):
            proc = base.subset([0])
            arr = proc.map_masses if col == 0 else proc.map_widths
            arr = arr.copy()
            for c in branch_codes:
                arr[0, c - 1] += sgn * h
            if col == 0:
                proc.map_masses = arr
            else:
                proc.map_widths = arr
            l_, ok_ = loss(torch, PhaseSpace(proc, 500.0, 500.0), x, pbar, jbar)
            ls.append(l_)
            oks.append(ok_.cpu().numpy())
        fd = ((ls[0] - ls[1]) / (2 * h)).cpu().numpy()
        k = keep & oks[0] & oks[1]
        a, b = ad.cpu().numpy()[k], fd[k]
        rel = np.abs(a - b) / (np.abs(b) + np.abs(b).mean())
        assert np.median(rel) < 1e-6, (name, np.quantile(rel, [0.5, 0.99, 1.0]))
        assert np.quantile(rel, 0.99) < 1e-3, (name, np.quantile(rel, [0.5, 0.99, 1.0]))


def test_autograd_binding(torch):
    from gpu_phs_gb300.api import PhaseSpace
    from gpu_phs_gb300.autograd import mapping_parameters, phase_space
    proc = P.tt()
    ps = PhaseSpace(proc, 500.0, 500.0)
    x = torch.from_numpy(uniform_x(406, 2000, proc.n_x)).cuda().requires_grad_(True)
    theta = mapping_parameters(ps).requires_grad_(True)
    p, logj, ok = phase_space(ps, x, theta)
    w = torch.linspace(-1, 1, 24, device="cuda", dtype=torch.float64).view(1, 6, 4)
    (w * p).sum().add(logj.sum()).backward()
    xbar, thbar = ps.vjp(x.detach(), w.expand_as(p).contiguous(),
                         torch.ones(2000, device="cuda", dtype=torch.float64))
    assert torch.equal(x.grad, xbar)
    assert torch.allclose(theta.grad, thbar.sum(0).cpu())
    assert theta.grad[1, 0] != 0      # d/dm of the t branch


@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_adjoint_friend_channels_against_finite_differences(torch, k):
    """Channels of Whizard's bwbw process whose decays are measured from a beam axis (friend
    boosts; t-channel mappings and collinear angles too), one at a time, against FP64
    central finite differences as above."""
    from conftest import golden, load_process
    from gpu_phs_gb300.api import PhaseSpace
    z = golden("whizard_bwbw")
    full = load_process(z)
    friends = [c for c in range(full.n_channels) if np.any(full.friends[c] != 0)]
    assert len(friends) >= 4
    proc = full.subset([friends[4 * k]])
    proc.sqrts = 1000.0
    n, h = 4000, 1e-6
    x = torch.from_numpy(uniform_x(700 + k, n, proc.n_x)).cuda()
    ps = PhaseSpace(proc, 500.0, 500.0)
    g = torch.Generator(device="cuda").manual_seed(10 + k)
    pbar = torch.randn((n, proc.n_out, 4), generator=g, device="cuda", dtype=torch.float64)
    jbar = torch.randn(n, generator=g, device="cuda", dtype=torch.float64)
    xbar, _ = ps.vjp(x, pbar, jbar)
    ev = ps.generate(x)
    keep = ev.ok.bool().cpu().numpy() & (margins(ev.p.cpu().numpy(), proc) > 1e-4)
    keep &= ((x > 2 * h) & (x < 1 - 2 * h)).all(dim=1).cpu().numpy()
    fd = torch.zeros_like(x)
    for i in range(proc.n_x):
        xp, xm = x.clone(), x.clone()
        xp[:, i] += h
        xm[:, i] -= h
        lp, okp = loss(torch, ps, xp, pbar, jbar)
        lm, okm = loss(torch, ps, xm, pbar, jbar)
        fd[:, i] = (lp - lm) / (2 * h)
        keep &= (okp & okm).cpu().numpy()
    a, b = xbar.cpu().numpy()[keep], fd.cpu().numpy()[keep]
    scale = np.abs(b).max(axis=1, keepdims=True) + 1.0
    rel = np.abs(a - b) / scale
    assert keep.sum() > 0.3 * n
    assert np.median(rel) < 1e-7, np.quantile(rel, [0.5, 0.99, 0.999, 1.0])
    assert np.quantile(rel, 0.99) < 1e-4, np.quantile(rel, [0.5, 0.99, 0.999, 1.0])


@pytest.mark.parametrize("channel", [0, 1])
def test_adjoint_largest_trees_against_finite_differences(torch, channel):
    """12 outgoing particles (11 visits, 32 x, a two-deep frame stack): the balanced tree
    and the caterpillar of nested resonances, against finite differences as above."""
    from gpu_phs_gb300.api import PhaseSpace
    proc = P.nested_resonances(12).subset([channel])
    n, h = 3000, 1e-6
    x = torch.from_numpy(uniform_x(900 + channel, n, proc.n_x)).cuda()
    ps = PhaseSpace(proc, 500.0, 500.0)
    g = torch.Generator(device="cuda").manual_seed(20 + channel)
    pbar = torch.randn((n, proc.n_out, 4), generator=g, device="cuda", dtype=torch.float64)
    jbar = torch.randn(n, generator=g, device="cuda", dtype=torch.float64)
    xbar, _ = ps.vjp(x, pbar, jbar)
    ev = ps.generate(x)
    keep = ev.ok.bool().cpu().numpy() & (margins(ev.p.cpu().numpy(), proc) > 1e-4)
    keep &= ((x > 2 * h) & (x < 1 - 2 * h)).all(dim=1).cpu().numpy()
    fd = torch.zeros_like(x)
    for i in range(proc.n_x):
        xp, xm = x.clone(), x.clone()
        xp[:, i] += h
        xm[:, i] -= h
        lp, okp = loss(torch, ps, xp, pbar, jbar)
        lm, okm = loss(torch, ps, xm, pbar, jbar)
        fd[:, i] = (lp - lm) / (2 * h)
        keep &= (okp & okm).cpu().numpy()
    a, b = xbar.cpu().numpy()[keep], fd.cpu().numpy()[keep]
    scale = np.abs(b).max(axis=1, keepdims=True) + 1.0
    rel = np.abs(a - b) / scale
    assert keep.sum() > 0.05 * n
    assert np.median(rel) < 1e-7, np.quantile(rel, [0.5, 0.99, 0.999, 1.0])
    assert np.quantile(rel, 0.99) < 1e-4, np.quantile(rel, [0.5, 0.99, 0.999, 1.0])
