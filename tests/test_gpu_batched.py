"""The batched workload: 64 channel trees with 3-8 outgoing particles and power-law event
counts in one persistent launch, replayed from a CUDA graph.  ok flags must equal those of
per-channel plain runs bit for bit, in FP64 and in FP32-pair arithmetic."""
import numpy as np
import pytest

from gpu_phs_gb300 import processes as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_batched_graph_matches_direct_and_per_channel(torch):
    from gpu_phs_gb300.api import Batch, PhaseSpace, batch_graph, philox_fill
    procs, counts = P.batched(seed=2024, n_channels=64, total_events=1 << 20)
    spaces = [PhaseSpace(p, 500.0, 500.0) for p in procs]
    results = {}
    for prec in (0, 1):
        batch = Batch(spaces)
        batch.set_precision(prec)
        xo, po = batch.offsets(counts)
        x = torch.empty(int(xo[-1]), dtype=torch.float64, device="cuda")
        philox_fill(x, int(xo[-1]), 1, seed=5)
        n = int(counts.sum())
        direct = batch.generate(x, counts)
        bufs = (torch.empty(int(po[-1]), dtype=torch.float64, device="cuda"),
                torch.empty(n, dtype=torch.float64, device="cuda"),
                torch.empty(n, dtype=torch.float64, device="cuda"),
                torch.empty(n, dtype=torch.uint8, device="cuda"))
        g = batch_graph(batch, x, counts, *bufs)
        for t in bufs:
            t.zero_()
        g.launch()
        g.launch()
        torch.cuda.synchronize()
        for a, b in zip(direct, bufs):
            assert torch.equal(a, b)
        results[prec] = (x, xo, po, direct)
    # FP32 pairs decide ok exactly as FP64 does
    assert torch.equal(results[0][3][3], results[1][3][3])
    # ... and FP64 batched equals per-channel plain runs
    x, xo, po, (p, f, v, ok) = results[0]
    e = 0
    for i, (ps, c) in enumerate(zip(spaces, counts)):
        c = int(c)
        ev = ps.generate(x[xo[i]:xo[i + 1]].view(c, ps.proc.n_x))
        assert torch.equal(ev.ok, ok[e:e + c])
        assert torch.equal(ev.p.reshape(-1), p[po[i]:po[i + 1]])
        e += c
    assert 0.01 < ok.double().mean().item() < 1.0


def test_process_graph_replay(torch):
    from gpu_phs_gb300.api import PhaseSpace, philox_x, process_graph
    proc = P.tt()
    ps = PhaseSpace(proc, 500.0, 500.0)
    x = philox_x(300_000, proc.n_x, seed=8)
    ref = ps.generate(x)
    out = ps.alloc(300_000)
    g = process_graph(ps, x, out)
    out.p.zero_()
    g.launch()
    torch.cuda.synchronize()
    assert torch.equal(out.p, ref.p) and torch.equal(out.ok, ref.ok)


@pytest.mark.parametrize("prec,variant", [(0, 5), (0, 8), (1, 5), (1, 4)])
def test_split_forms_in_cuda_graphs(torch, prec, variant):
    """A split variant pinned before capture (so the graph holds its pre-test, scan, walk,
    and for FP32 pairs the exact path, with their counter resets): replays equal the
    one-pass kernel's outputs, twice in a row."""
    from gpu_phs_gb300.api import Batch, PhaseSpace, batch_graph, philox_fill
    procs, counts = P.batched(seed=77, n_channels=64, total_events=1 << 19)
    spaces = [PhaseSpace(p, 500.0, 500.0) for p in procs]
    ref = None
    xo = po = None
    for v in (0, variant):
        batch = Batch(spaces)
        batch.set_precision(prec)
        batch.set_variants(v if prec else -1, -1 if prec else v)
        xo, po = batch.offsets(counts)
        if ref is None:
            x = torch.empty(int(xo[-1]), dtype=torch.float64, device="cuda")
            philox_fill(x, int(xo[-1]), 1, seed=9)
        n = int(counts.sum())
        bufs = (torch.empty(int(po[-1]), dtype=torch.float64, device="cuda"),
                torch.empty(n, dtype=torch.float64, device="cuda"),
                torch.empty(n, dtype=torch.float64, device="cuda"),
                torch.empty(n, dtype=torch.uint8, device="cuda"))
        g = batch_graph(batch, x, counts, *bufs)
        outs = []
        for _ in range(2):
            for t in bufs:
                t.fill_(7)
            g.launch()
            torch.cuda.synchronize()
            outs.append([t.clone() for t in bufs])
        if ref is None:
            ref = outs[0]
        for o in outs:
            for a, b in zip(ref, o):
                assert torch.equal(a, b)


def _gen_batch(torch, spaces, counts, x, prec, ff_v=-1, f64_v=-1):
    from gpu_phs_gb300.api import Batch
    batch = Batch(spaces)
    batch.set_precision(prec)
    batch.set_variants(ff_v, f64_v)
    out = batch.generate(x, counts)
    torch.cuda.synchronize()
    return [t.clone() for t in out]


@pytest.mark.parametrize("prec,n_var", [(0, 9), (1, 6)])
def test_kernel_variants_identical_bits(torch, prec, n_var):
    """Every kernel variant (block shapes, register budgets, one-pass, compacting or split)
    computes the same bits: the compacting and split forms run the same event code on the events that
    pass their pre-test, and the pre-test writes the outputs of failing events exactly as
    the one-pass form does."""
    from gpu_phs_gb300.api import Batch, PhaseSpace, philox_fill
    procs, counts = P.batched(seed=2024, n_channels=64, total_events=1 << 19)
    spaces = [PhaseSpace(p, 500.0, 500.0) for p in procs]
    xo, _ = Batch(spaces).offsets(counts)
    x = torch.empty(int(xo[-1]), dtype=torch.float64, device="cuda")
    philox_fill(x, int(xo[-1]), 1, seed=6)
    kw = (lambda v: dict(ff_v=v)) if prec else (lambda v: dict(f64_v=v))
    ref = _gen_batch(torch, spaces, counts, x, prec, **kw(0))
    assert 0.1 < ref[3].double().mean().item() < 0.5   # many events fail: compaction matters
    for v in range(1, n_var):
        got = _gen_batch(torch, spaces, counts, x, prec, **kw(v))
        for a, b in zip(ref, got):
            assert torch.equal(a, b), f"variant {v} differs from variant 0"


@pytest.mark.parametrize("f64_v", [1, 2, 3, 4, 5, 6, 7, 8])
def test_compacting_fp64_vs_oracle_low_ok_fraction(torch, f64_v):
    """The 13 TeV configuration (about 4% of events pass) through every FP64 variant but the
    default one pass (block shapes, compacting, split), against the oracle."""
    from conftest import momentum_rel_err
    from gpu_phs_gb300.api import PhaseSpace
    from gpu_phs_gb300.philox import uniform_x
    from oracle import oracle
    proc = P.precision()
    n = 100_000
    x = uniform_x(77, n, proc.n_x)
    ps = PhaseSpace(proc, proc.sqrts / 2, proc.sqrts / 2)
    ps.set_variants(-1, f64_v)
    ev = ps.generate(torch.from_numpy(x).cuda())
    p, f, v, ok = (t.cpu().numpy() for t in (ev.p, ev.factor, ev.volume, ev.ok))
    r = oracle.Oracle(proc, proc.sqrts).generate(x)
    assert np.array_equal(ok, r.ok)
    sel = r.ok == 1
    assert 0.01 < sel.mean() < 0.1
    assert momentum_rel_err(p[sel], r.p[sel], proc.sqrts).max() <= 1e-12
    assert (np.abs(f[sel] / r.factor[sel] - 1)).max() <= 1e-12
    assert np.all(p[~sel] == 0) and np.all(f[~sel] == 0)
    assert np.allclose(v, r.volume, rtol=1e-15, atol=0)


def test_split_form_many_segments_and_empty_channels(torch):
    """The FP32-pair split form with more segments than the launch parameters hold inline
    (a device segment table) and with empty channels between full ones (the scan gives
    them no claims): identical bits to the one-pass form."""
    from gpu_phs_gb300.api import Batch, PhaseSpace, philox_fill
    procs, counts = P.batched(seed=11, n_channels=100, total_events=1 << 18)
    counts = counts.copy()
    counts[[0, 7, 50, 99]] = 0
    spaces = [PhaseSpace(p, 500.0, 500.0) for p in procs]
    xo, _ = Batch(spaces).offsets(counts)
    x = torch.empty(int(xo[-1]), dtype=torch.float64, device="cuda")
    philox_fill(x, int(xo[-1]), 1, seed=12)
    ref = _gen_batch(torch, spaces, counts, x, 1, ff_v=0)
    for v in (4, 5):
        got = _gen_batch(torch, spaces, counts, x, 1, ff_v=v)
        for a, b in zip(ref, got):
            assert torch.equal(a, b), f"variant {v} differs from variant 0"


def test_per_event_beams_with_a_split_variant_pinned(torch):
    """The FP32 pre-test needs uniform beams: with per-event beams a pinned split variant
    runs as the compacting or one-pass variant of its block shape, with the same bits as
    the default one-pass kernel."""
    from gpu_phs_gb300.api import PhaseSpace, philox_x
    proc = P.tt()
    n = 100_000
    x = philox_x(n, proc.n_x, seed=31)
    g = torch.Generator(device="cuda").manual_seed(3)
    E1 = 300 + 400 * torch.rand(n, generator=g, device="cuda", dtype=torch.float64)
    E2 = 300 + 400 * torch.rand(n, generator=g, device="cuda", dtype=torch.float64)
    outs = []
    for v in (0, 3, 4, 5, 6, 7, 8):
        ps = PhaseSpace(proc)
        ps.set_variants(-1, v)
        ev = ps.generate_beams(x, E1, E2)
        torch.cuda.synchronize()
        outs.append((ev.p.clone(), ev.factor.clone(), ev.volume.clone(), ev.ok.clone()))
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            assert torch.equal(a, b)
