"""The adjoint kernel against FP64 central finite differences (h = 1e-6) of the forward
kernel, on the tt tree, Whizard's friend channels and the 12-particle trees.

Every kept derivative is checked against a bound, not a quantile:

    |adjoint - FD(h)| <= 1e-7 * scale + 2 |FD(h) - FD(2h)| + 4e-15 * |loss| / h

scale: the event's largest derivative + 1 (x), or |FD| + its mean over the events
(mapping parameters).  FD(2h) - FD(h) is three times the h^2 truncation error of FD(h), so
the second term bounds the difference quotient's own error where the map curves strongly
(Breit-Wigner tails near +-pi/2); the third is the rounding of two loss evaluations
divided by 2h.  Events are excluded only by stated criteria: ok = 0, within 1e-4 of a
kinematic limit (relative margin of a mass to its threshold or upper bound), an ok flag
that changes at x +- h or x +- 2h, an x within 2h of 0 or 1, or within 2h of 0.5 (where
the two-sided exponential maps switch branches and the derivative jumps).
"""
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


TOL = 1e-7        # relative to the event's derivative scale
ROUND = 4e-15     # relative rounding of one loss evaluation (FP64 forward map and the sum)


def loss(torch, ps, x, pbar, jbar):
    """sum pbar . p + jbar log(factor) per event, its ok flag and its magnitude
    sum |pbar| |p| + |jbar log(factor)| (the scale of its rounding error)."""
    ev = ps.generate(x)
    ok = ev.ok.bool()
    lj = torch.where(ok, torch.log(torch.where(ok, ev.factor, torch.ones_like(ev.factor))), 0.0)
    mag = (pbar.abs() * ev.p.abs()).sum(dim=(1, 2)) + (jbar * lj).abs()
    return (pbar * ev.p).sum(dim=(1, 2)) + jbar * lj, ok, mag


def x_finite_differences(torch, ps, x, pbar, jbar, h):
    """Central differences of the loss in every x at steps h and 2h, whether the event is
    ok at all of x +- h, x +- 2h, and the largest loss magnitude seen."""
    fd1, fd2 = torch.zeros_like(x), torch.zeros_like(x)
    ok_all = torch.ones(x.shape[0], dtype=torch.bool, device=x.device)
    mag = torch.zeros(x.shape[0], dtype=torch.float64, device=x.device)
    for k in range(x.shape[1]):
        val = {}
        for m in (1, -1, 2, -2):
            xs = x.clone()
            xs[:, k] += m * h
            val[m], ok, mg = loss(torch, ps, xs, pbar, jbar)
            ok_all &= ok
            mag = torch.maximum(mag, mg)
        fd1[:, k] = (val[1] - val[-1]) / (2 * h)
        fd2[:, k] = (val[2] - val[-2]) / (4 * h)
    return fd1, fd2, ok_all, mag


def x_keep(torch, ev, x, proc, h):
    """The stated exclusions that need no finite differences: ok = 0, within 1e-4 of a
    kinematic limit, an x within 2h of 0, 1 or 0.5."""
    keep = ev.ok.bool().cpu().numpy() & (margins(ev.p.cpu().numpy(), proc) > 1e-4)
    keep &= ((x > 2 * h) & (x < 1 - 2 * h)).all(dim=1).cpu().numpy()
    keep &= ((x - 0.5).abs() > 2 * h).all(dim=1).cpu().numpy()
    return keep


def assert_bound(a, fd1, fd2, mag, h, scale, what):
    """|a - fd1| <= TOL scale + 2 |fd1 - fd2| + ROUND mag / h, element by element."""
    bound = TOL * scale + 2 * np.abs(fd1 - fd2) + ROUND * mag / h
    ratio = np.abs(a - fd1) / bound
    q = np.quantile(np.abs(a - fd1) / scale, [0.5, 0.99, 1.0])
    worst = ratio.max() if ratio.size else 0.0
    print(f"{what}: {a.shape[0]} events, worst |adjoint - FD| / bound {worst:.3g}, "
          f"|adjoint - FD| / scale median {q[0]:.2e} 99% {q[1]:.2e} max {q[2]:.2e}")
    assert worst <= 1.0, (what, worst, np.unravel_index(np.argmax(ratio), ratio.shape))


def check_x_derivatives(torch, ps, proc, x, pbar, jbar, h, min_kept, what):
    xbar, _ = ps.vjp(x, pbar, jbar)
    ev = ps.generate(x)
    keep = x_keep(torch, ev, x, proc, h)
    fd1, fd2, ok_all, mag = x_finite_differences(torch, ps, x, pbar, jbar, h)
    keep &= ok_all.cpu().numpy()
    assert keep.sum() > min_kept * x.shape[0], keep.sum()
    a, b, b2 = (t.cpu().numpy()[keep] for t in (xbar, fd1, fd2))
    scale = np.abs(b).max(axis=1, keepdims=True) + 1.0
    assert_bound(a, b, b2, mag.cpu().numpy()[keep][:, None], h, scale, what)


def test_adjoint_x_against_finite_differences(torch):
    from gpu_phs_gb300.api import PhaseSpace
    proc = P.tt()
    n, h = 10_000, 1e-6
    x = torch.from_numpy(uniform_x(404, n, proc.n_x)).cuda()
    ps = PhaseSpace(proc, 500.0, 500.0)
    g = torch.Generator(device="cuda").manual_seed(1)
    pbar = torch.randn((n, proc.n_out, 4), generator=g, device="cuda", dtype=torch.float64)
    jbar = torch.randn(n, generator=g, device="cuda", dtype=torch.float64)
    check_x_derivatives(torch, ps, proc, x, pbar, jbar, h, 0.9, "tt dx")


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
        ls, k, mag = {}, keep.copy(), np.zeros(n)
        for m in (1, -1, 2, -2):
            proc = base.subset([0])
            arr = (proc.map_masses if col == 0 else proc.map_widths).copy()
            for c in branch_codes:
                arr[0, c - 1] += m * h
            if col == 0:
                proc.map_masses = arr
            else:
                proc.map_widths = arr
            ls[m], ok_, mg = loss(torch, PhaseSpace(proc, 500.0, 500.0), x, pbar, jbar)
            k &= ok_.cpu().numpy()
            mag = np.maximum(mag, mg.cpu().numpy())
        fd1 = ((ls[1] - ls[-1]) / (2 * h)).cpu().numpy()[k]
        fd2 = ((ls[2] - ls[-2]) / (4 * h)).cpu().numpy()[k]
        a = ad.cpu().numpy()[k]
        assert k.sum() > 0.9 * n
        assert_bound(a, fd1, fd2, mag[k], h, np.abs(fd1) + np.abs(fd1).mean(), f"tt d/d{name}")


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
    check_x_derivatives(torch, ps, proc, x, pbar, jbar, h, 0.3, f"bwbw friend channel {k} dx")


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
    check_x_derivatives(torch, ps, proc, x, pbar, jbar, h, 0.05, f"12-particle tree {channel} dx")


def test_stored_matrix_form_against_finite_differences_and_recompute(torch):
    """The stored-matrix adjoint (every visit's parent frame kept in a device buffer, read
    back in the reverse walk) on the tt tree: within the finite-difference bound above, close
    to the recompute form, and holding n x max visits x 128 bytes of device memory exactly
    while it is selected."""
    from gpu_phs_gb300.api import ADJOINT_RECOMPUTE, ADJOINT_STORED, PhaseSpace
    proc = P.tt()
    n, h = 10_000, 1e-6
    x = torch.from_numpy(uniform_x(407, n, proc.n_x)).cuda()
    ps = PhaseSpace(proc, 500.0, 500.0)
    g = torch.Generator(device="cuda").manual_seed(3)
    pbar = torch.randn((n, proc.n_out, 4), generator=g, device="cuda", dtype=torch.float64)
    jbar = torch.randn(n, generator=g, device="cuda", dtype=torch.float64)
    xr, tr = ps.vjp(x, pbar, jbar)
    ps.set_adjoint_storage(ADJOINT_STORED)
    xs, ts = ps.vjp(x, pbar, jbar)
    torch.cuda.synchronize()
    scale = xr.abs().amax(dim=1, keepdim=True) + 1.0
    assert ((xs - xr).abs() / scale).max().item() < 1e-9
    assert ((ts - tr).abs() / (tr.abs().amax(dim=(1, 2), keepdim=True) + 1.0)).max().item() < 1e-9
    # the buffer the handle holds: released on the switch back (nothing else allocates here)
    free_a = torch.cuda.mem_get_info()[0]
    ps.set_adjoint_storage(ADJOINT_RECOMPUTE)
    torch.cuda.synchronize()
    held = torch.cuda.mem_get_info()[0] - free_a
    want = n * (proc.n_out - 1) * 16 * 8
    assert want <= held <= want + (2 << 20), (held, want)   # cudaMalloc's 2 MiB pages
    ps.set_adjoint_storage(ADJOINT_STORED)
    check_x_derivatives(torch, ps, proc, x, pbar, jbar, h, 0.9, "tt dx, stored-matrix form")


@pytest.mark.parametrize("builder,E1,E2", [(P.ww, 250.0, 250.0), (P.ww, 300.0, 200.0),
                                           (P.tt, 600.0, 400.0)])
def test_adjoint_lab_boost_and_leaf_pairs_against_finite_differences(torch, builder, E1, E2):
    """WW's root daughters each decay to two leaves (their frames are kept from the root's
    in the forward pass, which is also the frame the root-daughter shortcuts assume), and
    unequal beams (E1 = 1.2 E2) put the lab boost into the root's frame, where those
    shortcuts do not apply; against finite differences as above."""
    from gpu_phs_gb300.api import PhaseSpace
    proc = builder()
    proc.sqrts = 2.0 * np.sqrt(E1 * E2)        # the margins' upper bounds
    n, h = 4000, 1e-6
    x = torch.from_numpy(uniform_x(950 + proc.n_out + int(E1), n, proc.n_x)).cuda()
    ps = PhaseSpace(proc, E1, E2)
    g = torch.Generator(device="cuda").manual_seed(30 + proc.n_out)
    pbar = torch.randn((n, proc.n_out, 4), generator=g, device="cuda", dtype=torch.float64)
    jbar = torch.randn(n, generator=g, device="cuda", dtype=torch.float64)
    check_x_derivatives(torch, ps, proc, x, pbar, jbar, h, 0.7,
                        f"{proc.name} E1 {E1:g} E2 {E2:g} dx")
