"""Benchmark: events/s of the fused phase-space kernel on GB300.

Default workload (one GPU): e+e- -> t tbar -> b l nu bbar q q' at sqrt(s) = 1 TeV, plain
FP64, 1e7 events per step, 14 Philox4x32-10 x per event resident in HBM.  A step is one
forward generation of all events (one kernel launch).  x (1.12 GB) and the outputs
(2.1 GB) are far larger than L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

For N > 1 (torchrun) every rank generates its own event range on its own GPU (replicas,
no collective on the data path); value is the events of all ranks / the slowest rank's
time.  --impl reference times the reference CPU path on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "events/s on 1 GB300: FP32-mixed batched vs plain FP64 at stated momentum error"
SEED = 1234


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload(name: str):
    from gpu_phs_gb300 import processes as P
    if name == "tt":
        return P.tt(), 10_000_000
    if name == "ww":
        return P.ww(), 1_000_000
    if name == "precision":
        return P.precision(), 1 << 24
    raise ValueError(name)


def bytes_per_event(proc) -> int:
    """Algorithmic HBM bytes per event: x row read + momenta, factor, volume, ok written."""
    return 8 * proc.n_x + 32 * proc.n_out + 8 + 8 + 1


def hbm_roofline(total_bytes: float, ms: float, what: str) -> dict:
    """HBM view of a form: algorithmic bytes of the whole step / its CUDA-event time, against
    the measured copy bandwidth."""
    peak, kind = peaks()
    gbs = total_bytes / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
            "peak_kind": kind, "algorithmic_bytes_per_step": total_bytes, "what": what}


def flops_per_event(proc) -> float:
    """FP64 operations of the minimal algorithm per event, one convention for all
    workloads: add/sub/mul/div/sqrt = 1, FMA = 2, each transcendental call = 1.  It
    undercounts library math (tan, exp, sincos expand to tens of operations), so the
    FP64-pipe fraction is also measured directly with ncu."""
    from gpu_phs_gb300.processes import MAP_NO, MAP_SCHANNEL, MAP_STEP_E, MAP_STEP_H
    R = (1 << proc.n_out) - 1
    d1, d2, hc, mid = proc.d1[0], proc.d2[0], proc.has_children[0], proc.map_ids[0]
    msq_cost = {MAP_NO: 5, MAP_SCHANNEL: 11, MAP_STEP_E: 12, MAP_STEP_H: 12}
    total = 0.0

    def internal(code):
        return hc[code - 1] != 0

    def walk(code, root):
        nonlocal total
        k = (d1[code - 1], d2[code - 1])
        if not root:
            total += msq_cost.get(int(mid[code - 1]), 7) + 1       # mapping + sqrt(msq)
        total += 12                                                  # Kallen, p_decay, factor
        total += 21                                                  # bg, gamma, sincos, ct, L1
        if not root:
            total += 80 if any(internal(c) for c in k) else 40       # L0 * L1 (structured)
        for c in k:
            if internal(c):
                walk(c, False)
            else:
                total += 15                                          # E and L * (E,0,0,p)

    walk(R, True)
    return total


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-i", str(self.device), "-lms", "200"], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        self.tmp.flush()
        self.tmp.seek(0)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.tmp.read().splitlines():
            f = [t.strip() for t in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.tmp.name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _time_calls(torch, fn, steps: int, warmup: int, stream) -> float:
    """Mean ms per call from CUDA events on `stream` after `warmup` untimed calls."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def _errors(torch, ref, got, sqrts):
    """FP32-pair outputs against the FP64 kernel's on the same x (the FP64 kernel equals the
    CPU oracle to 1e-12; tests/test_gpu_parity.py)."""
    ok_mism = int((ref.ok != got.ok).sum().item())
    sel = ref.ok.bool() & got.ok.bool()
    a, b = ref.p[sel], got.p[sel]
    d = (b - a).abs().amax(-1)
    floored = d / a[..., 0].abs().clamp(min=1e-3 * sqrts)
    unfloored = d / a[..., 0].abs().clamp(min=1e-300)
    fr = (got.factor[sel] - ref.factor[sel]).abs() / ref.factor[sel].abs()
    return {"ok_mismatches": ok_mism,
            "momentum_max_rel": floored.max().item(),
            "momentum_rms_rel": floored.pow(2).mean().sqrt().item(),
            "momentum_max_rel_unfloored": unfloored.max().item(),
            "factor_max_rel": fr.max().item(),
            "factor_rms_rel": fr.pow(2).mean().sqrt().item(),
            "definition": "per particle max_mu |dp^mu| / max(E, 1e-3 sqrt(s)); unfloored: / E"}


def measure_variants(torch, steps: int, warmup: int, x_tt, out_tt, ms_tt64, pin=(-1, -1)):
    """FP32-pair arithmetic on the tt workload, the 13 TeV configuration and the batched
    64-channel workload (CUDA-graph replay), each beside FP64 on the same x."""
    import ctypes as C
    from gpu_phs_gb300 import _lib
    from gpu_phs_gb300 import processes as P
    from gpu_phs_gb300.api import (PRECISION_F32X2, Batch, PhaseSpace, batch_graph, philox_fill)
    stream = torch.cuda.current_stream()
    steps = max(3, min(steps, 20))
    res = {}

    proc = P.tt()
    n = x_tt.shape[0]
    ps = PhaseSpace(proc, proc.sqrts / 2, proc.sqrts / 2)
    ps.set_precision(PRECISION_F32X2)
    o = ps.alloc(n)
    ms = _time_calls(torch, lambda: ps.generate(x_tt, out=o), steps, warmup, stream)
    v = C.c_int()
    _lib.load().phs_process_tuning(ps.h, C.byref(v), None)
    res["fp32_mixed_tt"] = {"value": n / ms * 1e3, "unit": "events/s", "ms_per_step": ms,
                            "speedup_vs_fp64": ms_tt64 / ms, "n_events": n,
                            "autotuned_variant": v.value,
                            "error_vs_fp64": _errors(torch, out_tt, o, proc.sqrts)}
    del o

    # per-event beam energies on the same tt x (E1, E2 uniform in [0.3, 0.7] sqrt(s)): FP64
    # and FP32 pairs (constants per event in FP64, the walk in float-float)
    g = torch.Generator(device="cuda").manual_seed(SEED)
    E1 = proc.sqrts * (0.3 + 0.4 * torch.rand(n, generator=g, device="cuda", dtype=torch.float64))
    E2 = proc.sqrts * (0.3 + 0.4 * torch.rand(n, generator=g, device="cuda", dtype=torch.float64))
    pe = {}
    for prec in (0, 1):
        ps = PhaseSpace(proc)
        ps.set_precision(prec)
        o = ps.alloc(n)
        pe[prec] = (_time_calls(torch, lambda: ps.generate_beams(x_tt, E1, E2, out=o), steps,
                                warmup, stream), o)
    res["per_event_beams_tt"] = {
        "n_events": n, "beams": "E1, E2 uniform in [0.3, 0.7] sqrt(s) per event",
        "fp64_events_per_s": n / pe[0][0] * 1e3, "fp32_mixed_events_per_s": n / pe[1][0] * 1e3,
        "speedup": pe[0][0] / pe[1][0],
        "error_vs_fp64": _errors(torch, pe[0][1], pe[1][1], proc.sqrts)}
    # the CPU path beside it on all n events with the same beams, checked event by event.
    # The reference's phs_cpu.cpp takes one sqrt(s) per call, so its C restatement (which
    # forms the constants per event as the reference's GPU path does) runs here.
    from oracle import oracle as _oracle
    threads = os.cpu_count() or 1
    beams = (E1.cpu().numpy(), E2.cpu().numpy())
    rate, passes, ref = cpu_time(_PerEventBeams(_oracle.Oracle(proc, proc.sqrts), *beams),
                                 x_tt.cpu().numpy(), 2.0, threads)
    rows = torch.full((n,), proc.n_out, dtype=torch.int64, device="cuda")
    res["per_event_beams_tt"]["cpu_baseline"] = {
        "value": rate, "unit": "events/s", "cores": threads, "kind": "port",
        "sample": f"all {n} events (the GPU's x and beams), {passes} passes, all host threads"}
    for prec, k in ((0, "fp64"), (1, "fp32_mixed")):
        o = pe[prec][1]
        res["per_event_beams_tt"][f"{k}_parity_vs_cpu"] = parity_vs_cpu(
            torch, ref, o.p.view(-1), o.factor, o.volume, o.ok, rows, proc.sqrts)
    del pe, E1, E2, ref, rows

    # Four forms per workload, three of them FP64 with identical output bits: the plain FP64
    # kernel (one pass: every event walked in full), FP64 compacting (an FP64 pass tests
    # every event first, only those that pass are walked), FP64 split (an FP32 pre-test with
    # error bounds settles only the events that fail for certain, the FP64 walk computes
    # the rest), and the FP32 pair form autotuned (register budgets x one pass / compacting
    # / split).  (name, precision, kernel variant of that precision); pin: the (FP32 pair,
    # FP64 split) variants (-1: the autotuner picks / the 128 x 3 split walk; a profiler
    # distorts the autotuner's timings, so a profiled run pins what the plain run picked)
    forms = (("fp64_one_pass", 0, 0), ("fp64_compacting", 0, 2),
             ("fp64_split", 0, pin[1] if pin[1] >= 0 else 6), ("fp32_mixed", 1, pin[0]))

    proc = P.precision()
    n = 1 << 24
    x = torch.empty((n, proc.n_x), dtype=torch.float64, device="cuda")
    philox_fill(x, n, proc.n_x, SEED)
    outs, t, tuned = {}, {}, {}
    for name, prec, var in forms:
        ps = PhaseSpace(proc, proc.sqrts / 2, proc.sqrts / 2)
        ps.set_precision(prec)
        ps.set_variants(var if prec else -1, -1 if prec else var)
        outs[name] = ps.alloc(n)
        t[name] = _time_calls(torch, lambda: ps.generate(x, out=outs[name]), steps, warmup, stream)
        tuned[name] = ps.tuning()[prec == 0]
    res["precision_13TeV"] = {
        "workload": proc.name, "n_events": n, "n_x": proc.n_x,
        **{f"{k}_events_per_s": n / t[k] * 1e3 for k, _, _ in forms},
        "kernel_variants": tuned,
        "speedup_vs_plain_fp64": t["fp64_one_pass"] / t["fp32_mixed"],
        "speedup_vs_fp64_compacting": t["fp64_compacting"] / t["fp32_mixed"],
        "speedup_vs_fp64_split": t["fp64_split"] / t["fp32_mixed"],
        "roofline": {k: hbm_roofline(n * bytes_per_event(proc), t[k],
                                     "x rows read, momenta, factor, volume, ok written "
                                     f"({bytes_per_event(proc)} B/event)")
                     for k in ("fp64_split", "fp32_mixed")},
        "ok_fraction": outs["fp64_one_pass"].ok.double().mean().item(),
        "fp64_forms_identical_bits": all(
            torch.equal(getattr(outs["fp64_one_pass"], f), getattr(outs[k], f))
            for k in ("fp64_compacting", "fp64_split") for f in ("p", "factor", "volume", "ok")),
        "error_vs_fp64": _errors(torch, outs["fp64_one_pass"], outs["fp32_mixed"], proc.sqrts)}
    # the reference CPU path beside it, on all n events (the GPU's x), checked event by event
    # against the FP64 split form and the FP32-pair form
    threads = os.cpu_count() or 1
    gen, kind = cpu_generator(proc, proc.sqrts)
    rate, passes, ref = cpu_time(gen, x.cpu().numpy(), 2.0, threads)
    rows = torch.full((n,), proc.n_out, dtype=torch.int64, device="cuda")
    res["precision_13TeV"]["cpu_baseline"] = {
        "value": rate, "unit": "events/s", "cores": threads, "kind": kind,
        "sample": f"all {n} events (the GPU's x), {passes} passes, all host threads"}
    for k in ("fp64_split", "fp32_mixed"):
        o = outs[k]
        res["precision_13TeV"][f"{k}_parity_vs_cpu"] = parity_vs_cpu(
            torch, ref, o.p.view(-1), o.factor, o.volume, o.ok, rows, proc.sqrts)
    del outs, x, ref, gen

    procs, counts = P.batched(seed=2024, n_channels=64, total_events=1 << 24)
    spaces = [PhaseSpace(p, 500.0, 500.0) for p in procs]
    n = int(counts.sum())
    bres, bufs, tuned = {}, {}, {}
    for name, prec, var in forms:
        batch = Batch(spaces)
        batch.set_precision(prec)
        batch.set_variants(var if prec else -1, -1 if prec else var)
        xo, po = batch.offsets(counts)
        if name == "fp64_one_pass":
            xb = torch.empty(int(xo[-1]), dtype=torch.float64, device="cuda")
            philox_fill(xb, int(xo[-1]), 1, SEED)
        bufs[name] = (torch.empty(int(po[-1]), dtype=torch.float64, device="cuda"),
                      torch.empty(n, dtype=torch.float64, device="cuda"),
                      torch.empty(n, dtype=torch.float64, device="cuda"),
                      torch.empty(n, dtype=torch.uint8, device="cuda"))
        g = batch_graph(batch, xb, counts, *bufs[name])   # tunes on its untimed first run
        bres[name] = _time_calls(torch, lambda: g.launch(), steps, warmup, stream)
        tuned[name] = batch.tuning()[prec == 0]
        del g
    # ok flags of the FP64 batch against per-channel plain runs
    per_channel_mism = 0
    e = 0
    for i, (sp, c) in enumerate(zip(spaces, counts)):
        c = int(c)
        ev = sp.generate(xb[xo[i]:xo[i + 1]].view(c, sp.proc.n_x))
        per_channel_mism += int((ev.ok != bufs["fp64_split"][3][e:e + c]).sum().item())
        e += c
    ok64 = bufs["fp64_one_pass"][3]
    batch_bytes = float(sum(int(c) * bytes_per_event(sp.proc) for sp, c in zip(spaces, counts)))
    res["batched_64ch"] = {
        "n_channels": 64, "n_events": n, "n_out_range": [3, 8],
        "counts": "power law, exponent 1.5, seed 2024",
        "launch": "one CUDA-graph replay per step: one pass and compacting are one "
                  "persistent kernel; the split forms replay the FP32 pre-test, a scan, the "
                  "walk and (FP32 pairs) the exact FP64 path's scan and kernel",
        **{f"{k}_events_per_s": n / bres[k] * 1e3 for k, _, _ in forms},
        "kernel_variants": tuned,
        "speedup_vs_plain_fp64": bres["fp64_one_pass"] / bres["fp32_mixed"],
        "speedup_vs_fp64_compacting": bres["fp64_compacting"] / bres["fp32_mixed"],
        "speedup_vs_fp64_split": bres["fp64_split"] / bres["fp32_mixed"],
        "roofline": {k: hbm_roofline(batch_bytes, bres[k],
                                     "per channel: x rows read, momenta, factor, volume, ok "
                                     "written, summed over the 64 channels' events")
                     for k in ("fp64_split", "fp32_mixed")},
        "ok_fraction": ok64.double().mean().item(),
        "ok_mismatches_fp32_mixed_vs_fp64": int((ok64 != bufs["fp32_mixed"][3]).sum().item()),
        "fp64_forms_identical_bits": all(
            torch.equal(a, b) for k in ("fp64_compacting", "fp64_split")
            for a, b in zip(bufs["fp64_one_pass"], bufs[k])),
        "ok_mismatches_vs_per_channel_runs": per_channel_mism}
    # momentum / factor error of the FP32-pair batch against FP64 (ok events)
    sel = ok64.bool()
    pf, p6 = bufs["fp32_mixed"][0], bufs["fp64_one_pass"][0]
    dp = (pf - p6).abs().max().item()
    res["batched_64ch"]["max_abs_momentum_diff_gev"] = dp
    res["batched_64ch"]["factor_max_rel"] = (
        (bufs["fp32_mixed"][1][sel] / bufs["fp64_one_pass"][1][sel] - 1).abs().max().item())
    # the per-particle relative momentum error of the other workloads, channel by channel
    # (flat momenta, each channel's events [count][n_out][4] from its offset)
    mx, sq, n_p, e = 0.0, 0.0, 0, 0
    okf = bufs["fp32_mixed"][3].bool()
    for i, (sp, c) in enumerate(zip(spaces, counts)):
        c, no = int(c), sp.proc.n_out
        both = (sel & okf)[e:e + c]
        a = p6[int(po[i]):int(po[i + 1])].view(c, no, 4)[both]
        b = pf[int(po[i]):int(po[i + 1])].view(c, no, 4)[both]
        if a.numel():
            r = (b - a).abs().amax(-1) / a[..., 0].abs().clamp(min=1e-3 * sp.proc.sqrts)
            mx = max(mx, r.max().item())
            sq += r.pow(2).sum().item()
            n_p += r.numel()
        e += c
    res["batched_64ch"]["momentum_max_rel"] = mx
    res["batched_64ch"]["momentum_rms_rel"] = (sq / max(n_p, 1)) ** 0.5
    res["batched_64ch"]["momentum_rel_definition"] = \
        "per particle max_mu |dp^mu| / max(E, 1e-3 sqrt(s)), events ok in both"
    # the reference CPU path beside it: every channel's events through its own process on
    # all host threads, timed over the whole batch and checked event by event
    threads = os.cpu_count() or 1
    xh = xb.cpu().numpy()
    flat = FlatResult(int(po[-1]), n)
    el, kinds, e = 0.0, set(), 0
    for i, (sp, c) in enumerate(zip(spaces, counts)):
        c = int(c)
        if c:
            gen, kind = cpu_generator(sp.proc, sp.proc.sqrts)
            kinds.add(kind)
            xc = xh[xo[i]:xo[i + 1]].reshape(c, sp.proc.n_x)
            t0 = time.perf_counter()
            r = gen.generate(xc, threads=threads)
            el += time.perf_counter() - t0
            flat.p[po[i]:po[i + 1]] = r.p.reshape(-1)
            flat.factor[e:e + c], flat.volume[e:e + c], flat.ok[e:e + c] = r.factor, r.volume, r.ok
        e += c
    rows = torch.from_numpy(np.repeat([sp.proc.n_out for sp in spaces], counts)).to("cuda")
    res["batched_64ch"]["cpu_baseline"] = {
        "value": n / el, "unit": "events/s", "cores": threads, "kind": "/".join(sorted(kinds)),
        "sample": f"all {n} events of the batch (the GPU's x), one pass per channel, all host "
                  "threads"}
    for k in ("fp64_split", "fp32_mixed"):
        bp, bf, bv, bo = bufs[k]
        res["batched_64ch"][f"{k}_parity_vs_cpu"] = parity_vs_cpu(
            torch, flat, bp, bf, bv, bo, rows, 1000.0)
    del flat, xh
    del bufs, xb, spaces

    # adjoint: forward + reverse on 1e6 tt events with random cotangents, in the recompute
    # form (parent frames recovered with inverse boosts) and the stored-matrix form (every
    # visit's parent frame written to a device buffer and read back, as the reference keeps
    # its boost chain in device memory)
    from gpu_phs_gb300.api import ADJOINT_RECOMPUTE, ADJOINT_STORED
    proc = P.tt()
    n = 1_000_000
    ps = PhaseSpace(proc, proc.sqrts / 2, proc.sqrts / 2)
    x = torch.empty((n, proc.n_x), dtype=torch.float64, device="cuda")
    philox_fill(x, n, proc.n_x, SEED)
    g = torch.Generator(device="cuda").manual_seed(SEED)
    pbar = torch.randn((n, proc.n_out, 4), dtype=torch.float64, device="cuda", generator=g)
    jbar = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
    o = ps.alloc(n)
    t_fwd = _time_calls(torch, lambda: ps.generate(x, out=o), steps, warmup, stream)
    in_bytes = (x.numel() + pbar.numel() + jbar.numel()) * 8

    def adjoint_memory(storage):
        """Device bytes of one vjp call in this storage form: the inputs, what torch
        allocates for the outputs (peak allocated during the call), and what the library
        holds after the call (cudaMemGetInfo minus torch's reserved growth)."""
        ps.set_adjoint_storage(ADJOINT_RECOMPUTE)       # releases a stored-matrix buffer
        ps.set_adjoint_storage(storage)
        torch.cuda.synchronize()
        free0, res0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_reserved()
        torch.cuda.reset_peak_memory_stats()
        alloc0 = torch.cuda.memory_allocated()
        xb, tb = ps.vjp(x, pbar, jbar)
        torch.cuda.synchronize()
        lib_held = (free0 - torch.cuda.mem_get_info()[0]) - (torch.cuda.memory_reserved() - res0)
        out_peak = torch.cuda.max_memory_allocated() - alloc0
        del xb, tb
        return {"inputs_bytes_per_event": in_bytes / n, "outputs_bytes_per_event": out_peak / n,
                "library_scratch_bytes_per_event": lib_held / n,
                "peak_device_bytes_per_event": (in_bytes + out_peak + lib_held) / n}

    forms = {}
    for name, storage in (("recompute", ADJOINT_RECOMPUTE), ("stored_matrix", ADJOINT_STORED)):
        mem = adjoint_memory(storage)
        t_adj = _time_calls(torch, lambda: ps.vjp(x, pbar, jbar), steps, warmup, stream)
        forms[name] = {"adjoint_ms": t_adj, "adjoint_over_forward": t_adj / t_fwd,
                       "fwd_plus_bwd_events_per_s": n / (t_fwd + t_adj) * 1e3, **mem}
    ps.set_adjoint_storage(ADJOINT_RECOMPUTE)
    rc = forms["recompute"]
    res["adjoint_tt"] = {
        "n_events": n, "n_x": proc.n_x, "forward_ms": t_fwd,
        "adjoint_ms": rc["adjoint_ms"], "adjoint_over_forward": rc["adjoint_over_forward"],
        "fwd_plus_bwd_events_per_s": rc["fwd_plus_bwd_events_per_s"],
        "outputs": "d(momenta, log factor)/dx and d/d(m, Gamma) of every Breit-Wigner branch",
        "forms": forms,
        "memory": "measured per call: inputs + torch's peak allocation for the outputs + the "
                  "library's device buffer (cudaMemGetInfo change net of torch's reserve)",
        "default": "recompute: parent frames recovered with inverse boosts, per-visit state in "
                   "shared memory, no device scratch"}
    del x, pbar, jbar, o

    # inverse map: Whizard's bwbw process (61 channels, 16 with friend boosts), every
    # event inverted in every channel, as the Whizard ABI does
    proc = whizard_process("bwbw")
    n = 1 << 20
    counts = np.full(proc.n_channels, n // proc.n_channels, np.int64)
    counts[: n - int(counts.sum())] += 1
    ps = PhaseSpace(proc, 500.0, 500.0)
    x = torch.empty((n, proc.n_x), dtype=torch.float64, device="cuda")
    philox_fill(x, n, proc.n_x, SEED)
    ev = ps.generate(x, counts)
    fac = torch.empty((n, proc.n_channels), dtype=torch.float64, device="cuda")
    xo = torch.empty((proc.n_channels, n, proc.n_x), dtype=torch.float64, device="cuda")
    lib = _lib.load()

    def inv():
        _lib.check(lib.phs_inverse_device(ps.h, n, counts.ctypes.data, None, None,
                                          ev.p.data_ptr(), ev.ok.data_ptr(), x.data_ptr(),
                                          ev.factor.data_ptr(), fac.data_ptr(), xo.data_ptr(),
                                          stream.cuda_stream))

    t_inv = _time_calls(torch, inv, steps, warmup, stream)
    pairs = n * proc.n_channels
    wbytes = pairs * 8 * (proc.n_x + 1)
    rbytes = n * (32 * proc.n_out + 1 + 8 * proc.n_x + 8)
    res["inverse_bwbw_61ch"] = {
        "n_events": n, "n_channels": proc.n_channels, "ms_per_step": t_inv,
        "events_per_s": n / t_inv * 1e3, "channel_inversions_per_s": pairs / t_inv * 1e3,
        "hbm_gbs": (wbytes + rbytes) / t_inv * 1e-6,
        "algorithmic_bytes_per_step": wbytes + rbytes,
        "ok_fraction": ev.ok.double().mean().item(),
        "launch": "one persistent kernel: 64 events per block at a time, every channel per event"}
    # the CPU path beside it: the reference has no CPU inverse (its inverse is GPU code,
    # phs.cu:1499-1554), so the oracle's restatement of that algorithm runs, on the first
    # ns events (each channel's first ns / n_channels), checked element by element
    from oracle import oracle as _oracle
    threads = os.cpu_count() or 1
    ns = 1 << 17
    first = np.concatenate([[0], np.cumsum(counts)[:-1]])
    sel = np.concatenate([np.arange(first[c], first[c] + ns // proc.n_channels)
                          for c in range(proc.n_channels)])
    ch = np.repeat(np.arange(proc.n_channels, dtype=np.int32), ns // proc.n_channels)
    idx = torch.from_numpy(sel).cuda()
    ph, okh = ev.p[idx].cpu().numpy(), ev.ok[idx].cpu().numpy()
    xh, fh = x[idx].cpu().numpy(), ev.factor[idx].cpu().numpy()
    o_inv = _oracle.Oracle(proc, 1000.0)
    t0, passes = time.perf_counter(), 0
    while True:
        rf, rx = o_inv.inverse(ph, ch, okh, x_own=xh, factor_own=fh, threads=threads)
        passes += 1
        if time.perf_counter() - t0 >= 2.0:
            break
    el = time.perf_counter() - t0
    gf, gx = fac[idx].cpu().numpy(), xo[:, idx].cpu().numpy()
    fin = np.isfinite(rf) & np.isfinite(gf) & (rf != 0)
    finx = np.isfinite(rx) & np.isfinite(gx)
    df = np.abs(gf[fin] - rf[fin]) / np.abs(rf[fin])
    res["inverse_bwbw_61ch"]["cpu_baseline"] = {
        "value": passes * sel.size * proc.n_channels / el, "unit": "channel inversions/s",
        "cores": threads, "kind": "port",
        "sample": f"{sel.size} events ({sel.size // proc.n_channels} of each channel) x "
                  f"{proc.n_channels} channels, {passes} passes, all host threads"}
    res["inverse_bwbw_61ch"]["parity_vs_cpu"] = {
        "events": int(sel.size),
        "non_finite_entries_differ": int((np.isfinite(gf) != np.isfinite(rf)).sum() +
                                         (np.isfinite(gx) != np.isfinite(rx)).sum()),
        "factor_max_rel_vs_cpu": float(df.max()),
        "factor_median_rel_vs_cpu": float(np.median(df)),
        "x_max_abs_vs_cpu": float(np.abs(gx[finx] - rx[finx]).max()),
        "definition": "every (event, channel) factor and x against the CPU inverse of the "
                      "GPU's momenta; relative factor error over finite non-zero entries"}
    del fac, xo, ev, x, ps, idx, gf, gx, rf, rx, df
    res["whizard_abi_bwbw_61ch"] = whizard_abi_rate(proc, 1 << 17, max(2, min(steps, 5)))
    return res


def whizard_abi_rate(proc, n: int, steps: int, x_host=None) -> dict:
    """The drop-in call as Whizard makes it: the 14-symbol C ABI set up for the process,
    then c_whizard_gen_phs_from_x_gpu on host arrays (x in, x_host or Philox seed SEED;
    momenta, every channel's factor and x, volumes and ok flags out), host wall clock per
    call."""
    import ctypes as C
    from gpu_phs_gb300 import _lib
    from gpu_phs_gb300.philox import uniform_x
    lib = _lib.load()
    ip = lambda v: C.byref(C.c_int(v))
    nch, n_x, n_out = proc.n_channels, proc.n_x, proc.n_out
    lib.c_whizard_set_particle_structure(ip(nch), ip(nch), ip(nch), ip(n_x), ip(proc.n_in), ip(n_out))
    keep = [np.ascontiguousarray(proc.flv_masses), np.ascontiguousarray(proc.flv_widths)]
    lib.c_whizard_set_flavors(keep[0].ctypes.data, keep[1].ctypes.data)
    lib.c_whizard_init_mappings()
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
    counts = np.full(nch, n // nch, np.int64)
    counts[: n - int(counts.sum())] += 1
    limits = np.ascontiguousarray(np.cumsum(counts), np.int32)
    lib.c_whizard_init_channel_ids(ip(n), ip(nch), limits.ctypes.data)
    x = np.ascontiguousarray(uniform_x(SEED, n, n_x) if x_host is None else x_host)
    E1, E2 = np.full(n, proc.sqrts / 2), np.full(n, proc.sqrts / 2)
    factors, volumes = np.zeros(n * nch), np.zeros(n)
    oks = np.zeros(n, np.uint8)
    p = np.zeros(n * n_out * 4)
    x_out = np.zeros(n * n_x * nch)
    flag = C.c_bool(False)

    def call():
        lib.c_whizard_gen_phs_from_x_gpu(E1.ctypes.data, E2.ctypes.data, C.byref(flag), ip(n),
                                         ip(nch), ip(n_x), x.ctypes.data, factors.ctypes.data,
                                         volumes.ctypes.data, oks.ctypes.data, p.ctypes.data,
                                         x_out.ctypes.data)
    call()
    err = lib.phs_last_error().decode()
    t0 = time.perf_counter()
    for _ in range(steps):
        call()
    dt = (time.perf_counter() - t0) / steps
    lib.c_whizard_reset_generator()
    lib.c_whizard_finalize_gpu_phs()
    out_bytes = n * (32 * n_out + 8 * nch + 8 + 1 + 8 * n_x * nch)
    return {"n_events": n, "n_channels": nch, "ms_per_call": dt * 1e3,
            "events_per_s": n / dt, "channel_inversions_per_s": n * nch / dt,
            "h2d_bytes_per_call": n * 8 * n_x, "d2h_bytes_per_call": out_bytes,
            "error": err or None,
            "path": "c_whizard_gen_phs_from_x_gpu (host arrays): forward, all-channel inverse, "
                    "copies back of momenta, factors [n][61], x [61][n][n_x], volumes, ok"}


def whizard_process(name: str):
    """A Whizard process from the sample-file fixtures committed under tests/golden."""
    z = np.load(os.path.join(ROOT, "tests", "golden", f"whizard_{name}.npz"))
    from gpu_phs_gb300.processes import Process
    meta = z["meta"]
    return Process(int(meta[0]), int(meta[1]), z["d1"], z["d2"], z["has_children"], z["friends"],
                   z["map_ids"], z["map_masses"], z["map_widths"], z["flv_masses"],
                   z["flv_widths"], n_x=int(meta[2]), name=f"whizard_{name}", sqrts=1000.0)


def cpu_generator(proc, sqrts):
    """The reference CPU path for one process: the reference's own phs_cpu.cpp (oracle/_ref)
    where it was built on this machine, else its C restatement.  Returns (generator, kind)."""
    from oracle import oracle
    if oracle.ref_available():
        try:
            return oracle.RefCPU(proc, sqrts), "reference"
        except OSError:
            pass
    return oracle.Oracle(proc, sqrts), "port"


class _PerEventBeams:
    """An oracle generator with fixed per-event beam energies, for cpu_time."""

    def __init__(self, gen, E1, E2):
        self.gen, self.E1, self.E2 = gen, E1, E2

    def generate(self, x, threads: int = 0):
        return self.gen.generate(x, threads=threads, E1=self.E1, E2=self.E2)


def cpu_time(gen, x, min_seconds: float, threads: int):
    """Events/s of gen over x (all host threads), repeated until min_seconds have passed
    (at least once); returns (rate, passes, the last pass's outputs)."""
    done, passes, t0 = 0, 0, time.perf_counter()
    while True:
        r = gen.generate(x, threads=threads)
        done += x.shape[0]
        passes += 1
        el = time.perf_counter() - t0
        if el >= min_seconds:
            return done / el, passes, r


def parity_vs_cpu(torch, ref, p, factor, volume, ok, n_out_rows, sqrts):
    """The GPU outputs (device tensors; p flat) against the CPU path's on the same events:
    ok-flag mismatches; over the events ok on both sides, the largest per-particle momentum
    error max_mu |dp| / max(E, 1e-3 sqrt(s)) and the largest relative factor error; the
    largest relative volume error over all events."""
    dev = p.device
    rok = torch.from_numpy(ref.ok).to(dev)
    res = {"events": int(rok.numel()), "ok_mismatches_vs_cpu": int((ok != rok).sum().item())}
    both = rok.bool() & ok.bool()
    rf = torch.from_numpy(ref.factor).to(dev)
    fr = (factor[both] - rf[both]).abs() / rf[both].abs()
    res["factor_max_rel_vs_cpu"] = fr.max().item() if fr.numel() else 0.0
    del rf
    rv = torch.from_numpy(ref.volume).to(dev)
    res["volume_max_rel_vs_cpu"] = ((volume - rv).abs() / rv.abs()).max().item()
    del rv
    rows = torch.repeat_interleave(both, n_out_rows)
    rp = torch.from_numpy(ref.p.reshape(-1)).to(dev).view(-1, 4)[rows]
    d = (p.view(-1, 4)[rows] - rp).abs().amax(-1) / rp[:, 0].abs().clamp(min=1e-3 * sqrts)
    res["momentum_max_rel_vs_cpu"] = d.max().item() if d.numel() else 0.0
    res["definition"] = "per particle max_mu |dp^mu| / max(E, 1e-3 sqrt(s)), events ok on both"
    return res


class FlatResult:
    """CPU outputs of a batch, flat in the batch's layout."""

    def __init__(self, n_p, n):
        self.p = np.zeros(n_p)
        self.factor = np.zeros(n)
        self.volume = np.zeros(n)
        self.ok = np.zeros(n, np.uint8)


def run_reference(args):
    """The reference CPU path on this machine's host cores, all threads, on the same
    workload as our arm: every step generates all n events of the workload (the first n
    events of the same Philox stream)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle
    proc, n = workload(args.config)
    if args.events:
        n = args.events
    threads = os.cpu_count() or 1
    gen, kind = cpu_generator(proc, proc.sqrts)
    x = oracle.uniform_x(SEED, n, proc.n_x, threads=threads)
    for _ in range(args.warmup):
        gen.generate(x, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gen.generate(x, threads=threads)
    el = time.perf_counter() - t0
    value = n * args.steps / el
    sample = (f"all {n} events of the {proc.name} workload per step (the GPU arm's events), "
              f"{args.steps} steps")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "events/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (Philox4x32-10 x, seed 1234)",
        "config": {"workload": proc.name, "n_events_per_step": n, "n_x": proc.n_x,
                   "n_out": proc.n_out, "sqrts_gev": proc.sqrts, "same_config": True,
                   "path": "reference phs_cpu.cpp set_msq_cpu + set_angles_cpu" if kind == "reference"
                   else "C restatement of phs_cpu.cpp (oracle/phs_oracle.c)"},
        "cpu_baseline": {"value": value, "unit": "events/s", "cores": threads, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()

    from gpu_phs_gb300 import _lib
    from gpu_phs_gb300.api import PhaseSpace, philox_fill
    from gpu_phs_gb300.replicas import event_window, max_over_ranks

    proc, n = workload(args.config)
    if args.events:
        n = args.events
    ps = PhaseSpace(proc, proc.sqrts / 2, proc.sqrts / 2)
    # the plain FP64 kernel: one pass, 128 threads x 4 blocks per SM (the variant the ncu
    # profile covers; the other block shapes differ by under 0.5 % on this workload)
    ps.set_variants(-1, 0)
    x = torch.empty((n, proc.n_x), dtype=torch.float64, device="cuda")
    # weak scaling: n events per rank, rank r's window of one Philox stream
    first, _ = event_window(rank, world, n * world)
    philox_fill(x, n, proc.n_x, SEED, first_event=first)
    out = ps.alloc(n)
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            dist.barrier()

    for _ in range(args.warmup):
        ps.generate(x, out=out)
    torch.cuda.synchronize()
    ok_frac = out.ok.double().mean().item()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    with Clocks(dev) as clk:
        t_all0 = torch.cuda.Event(enable_timing=True)
        t_all1 = torch.cuda.Event(enable_timing=True)
        t_all0.record(stream)
        for k in range(args.steps):
            starts[k].record(stream)
            ps.generate(x, out=out)
            ends[k].record(stream)
        t_all1.record(stream)
        torch.cuda.synchronize()
    barrier()
    total_ms = t_all0.elapsed_time(t_all1)
    kern_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms_per_step = max_over_ranks(total_ms) / args.steps
    value = world * n / (ms_per_step * 1e-3)
    clocks = clk.summary()

    # roofline of the forward kernel (one launch per step)
    hbm_peak, peak_kind = peaks()
    launch_ms = statistics.mean(kern_ms)
    bpe = bytes_per_event(proc)
    achieved_gbs = bpe * n / (launch_ms * 1e-3) / 1e9
    fpe = flops_per_event(proc)
    lib = _lib.load()
    import ctypes as C
    g64 = C.c_double()
    _lib.check(lib.phs_measure_fma_peak(1, C.byref(g64)))
    fp64_peak = g64.value
    fp64_achieved = fpe * n / (launch_ms * 1e-3) / 1e9
    traffic, pipe_pct = None, None
    prof = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(prof):
        with open(prof) as fh:
            tj = json.load(fh).get(proc.name, {})
        if tj.get("dram_bytes_per_event"):
            traffic = tj["dram_bytes_per_event"] * n
        pipe_pct = tj.get("fp64_pipe_pct_of_peak")

    # end to end through the host-pointer C entry point (pinned buffers)
    e2e = None
    if not args.no_e2e:
        xh = torch.empty((n, proc.n_x), dtype=torch.float64).pin_memory()
        xh.copy_(x.cpu())
        outh = type(out)(torch.empty((n, proc.n_out, 4), dtype=torch.float64).pin_memory(),
                         torch.empty(n, dtype=torch.float64).pin_memory(),
                         torch.empty(n, dtype=torch.float64).pin_memory(),
                         torch.empty(n, dtype=torch.uint8).pin_memory())
        e2e_steps = max(1, min(args.steps, 10))
        for _ in range(max(1, min(args.warmup, 3))):
            ps.generate_host(xh, out=outh)
        # three equal windows, the median reported: the host link's bandwidth varies from
        # one moment to the next on shared hosts, and the call is bound by it
        windows = []
        for _ in range(3):
            barrier()
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                ps.generate_host(xh, out=outh)
            el = max_over_ranks(time.perf_counter() - t0)
            windows.append(world * n * e2e_steps / el)
        e2e = {"value": statistics.median(windows), "unit": "events/s",
               "h2d_bytes_per_step": n * proc.n_x * 8,
               "d2h_bytes_per_step": n * (32 * proc.n_out + 8 + 1),
               "path": "phs_generate_host (C ABI), pinned host buffers, 512 Ki-event chunks on 3 "
                       "streams; volumes (one constant per channel) written on the host",
               "steps": e2e_steps, "windows": windows,
               "windowing": "median of three windows of `steps` calls each"}
        if world == 1:
            # the same call with the FP32-mixed form (information: there the host copies,
            # not the kernel, bound the call)
            from gpu_phs_gb300.api import PRECISION_F32X2
            ps_ff = PhaseSpace(proc, proc.sqrts / 2, proc.sqrts / 2)
            ps_ff.set_precision(PRECISION_F32X2)
            for _ in range(max(1, min(args.warmup, 3))):
                ps_ff.generate_host(xh, out=outh)
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                ps_ff.generate_host(xh, out=outh)
            el_ff = time.perf_counter() - t0
            e2e["fp32_mixed"] = {"value": n * e2e_steps / el_ff, "unit": "events/s",
                                 "path": "phs_generate_host, FP32-mixed precision, same buffers"}
            ps_ff.close()

    # the drop-in call, c_whizard_gen_phs_from_x_gpu, on the same workload with the host
    # arrays Whizard passes (pageable): x in; momenta, volumes, ok flags and, as its forced
    # inverse mapping adds, every channel's x and factor (one channel: the input x and the
    # forward factor) out
    e2e_abi = None
    if not args.no_e2e and world == 1:
        r = whizard_abi_rate(proc, n, max(2, min(args.steps, 5)), x.cpu().numpy())
        e2e_abi = {"value": r["events_per_s"], "unit": "events/s",
                   "h2d_bytes_per_step": r["h2d_bytes_per_call"],
                   "d2h_bytes_per_step": r["d2h_bytes_per_call"], "ms_per_call": r["ms_per_call"],
                   "error": r["error"],
                   "path": "c_whizard_gen_phs_from_x_gpu (the reference's C ABI), pageable host "
                           "arrays, equal beams (read on the host, not copied)"}

    variants = None
    if not args.no_variants and world == 1:
        variants = measure_variants(torch, args.steps, args.warmup, x, out, ms_per_step,
                                    tuple(int(v) for v in args.pin.split(",")))
        # the precision target compares the FP32-pair batched form with the plain FP64
        # kernel; the compacting and split FP64 forms are listed beside it
        bv = variants["batched_64ch"]
        variants["fp32_mixed_over_plain_fp64_batched"] = bv["speedup_vs_plain_fp64"]
        variants["fp32_mixed_over_fp64_compacting_batched"] = bv["speedup_vs_fp64_compacting"]
        variants["fp32_mixed_over_fp64_split_batched"] = bv["speedup_vs_fp64_split"]

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        # the reference CPU path on the same n events (x copied from the device), repeated
        # for about --cpu-seconds on all host threads; its outputs of the last pass are
        # checked against the GPU's of the timed run, event by event
        threads = os.cpu_count() or 1
        gen, kind = cpu_generator(proc, proc.sqrts)
        xh = x.cpu().numpy()
        rate, passes, ref = cpu_time(gen, xh, args.cpu_seconds, threads)
        rows = torch.full((n,), proc.n_out, dtype=torch.int64, device=x.device)
        cpu = {"value": rate, "unit": "events/s", "cores": threads, "kind": kind,
               "sample": f"all {n} events of the workload (the GPU's x), {passes} passes, "
                         f"all host threads",
               "parity_vs_gpu": parity_vs_cpu(torch, ref, out.p.view(-1), out.factor, out.volume,
                                              out.ok, rows, proc.sqrts)}
        del ref, xh, gen

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (Philox4x32-10 x, seed 1234, in HBM)",
            "config": {"workload": proc.name, "variant": "plain FP64, fused persistent kernel",
                       "n_events_per_gpu": n, "n_x": proc.n_x, "n_out": proc.n_out,
                       "sqrts_gev": proc.sqrts, "parallelism": f"replicas x{world}",
                       "l2": "inputs (x 1.12 GB) and outputs larger than L2; no flush"},
            "ok_fraction": ok_frac,
            # the binding roof is the FP64 pipe: achieved = the flops model's operations
            # per event x events per launch / the launch's CUDA-event time, against the
            # measured DFMA peak; HBM (a few percent) beside it
            "roofline": {"bound": "fp64", "achieved": fp64_achieved / 1e3,
                         "peak": fp64_peak / 1e3, "unit": "TFLOP/s",
                         "frac": fp64_achieved / fp64_peak, "traffic": traffic,
                         "peak_kind": "measured (phs_measure_fma_peak: DFMA chains on every SM)",
                         "flops_per_event": fpe, "kernel_ms": launch_ms,
                         "pipe_utilization_ncu": pipe_pct / 100 if pipe_pct else None,
                         "note": "frac counts each transcendental call as one operation; the "
                                 "ncu FP64-pipe utilisation counts the instructions the "
                                 "library math expands into",
                         "hbm": {"achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                                 "frac": achieved_gbs / hbm_peak, "peak_kind": peak_kind,
                                 "bytes_per_event": bpe}},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "e2e_whizard_abi": e2e_abi,
            "variants": variants,
            "gpu_launches": args.steps,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


PROFILE_CASES = ("f64_tt", "ff_tt", "f64_tt_beams", "ff_tt_beams", "f64_batched", "f64_split_batched",
                 "ff_batched", "inverse_bwbw", "adjoint_tt", "adjoint_tt_stored")


def run_case(name: str) -> None:
    """Small workloads for ncu captures of one kernel each (a few hundred MB on the device,
    inputs still larger than L2): two launches of the kernel, the second is the one to
    capture (ncu -k <kernel> -s 1 -c 1)."""
    import torch
    from gpu_phs_gb300 import processes as P
    from gpu_phs_gb300.api import Batch, PhaseSpace, philox_fill, philox_x
    if name in ("f64_tt", "ff_tt"):   # 2^21 tt events, FP64 or FP32-pair one pass
        proc = P.tt()
        n = 1 << 21
        ps = PhaseSpace(proc, 500.0, 500.0)
        if name == "ff_tt":
            ps.set_precision(1)
            ps.set_variants(1, -1)
        else:
            ps.set_variants(-1, 0)
        x = philox_x(n, proc.n_x, SEED)
        o = ps.alloc(n)
        for _ in range(2):
            ps.generate(x, out=o)
    elif name in ("f64_tt_beams", "ff_tt_beams"):   # 2^21 tt events, per-event beam energies
        proc = P.tt()
        n = 1 << 21
        ps = PhaseSpace(proc)
        if name == "ff_tt_beams":
            ps.set_precision(1)
            ps.set_variants(1, -1)
        else:
            ps.set_variants(-1, 0)
        x = philox_x(n, proc.n_x, SEED)
        g = torch.Generator(device="cuda").manual_seed(SEED)
        E1 = proc.sqrts * (0.3 + 0.4 * torch.rand(n, generator=g, device="cuda", dtype=torch.float64))
        E2 = proc.sqrts * (0.3 + 0.4 * torch.rand(n, generator=g, device="cuda", dtype=torch.float64))
        o = ps.alloc(n)
        for _ in range(2):
            ps.generate_beams(x, E1, E2, out=o)
    elif name in ("f64_batched", "f64_split_batched", "ff_batched"):   # 2^22 batched events
        procs, counts = P.batched(seed=2024, n_channels=64, total_events=1 << 22)
        b = Batch([PhaseSpace(p, 500.0, 500.0) for p in procs])
        if name == "ff_batched":          # split: FP32 pre-test, float-float walk
            b.set_precision(1)
            b.set_variants(5, -1)
        elif name == "f64_split_batched":  # split: FP32 pre-test, FP64 walk (128 x 3)
            b.set_variants(-1, 6)
        else:                              # compacting, FP64 pre-test
            b.set_variants(-1, 2)
        xo, _ = b.offsets(counts)
        x = torch.empty(int(xo[-1]), dtype=torch.float64, device="cuda")
        philox_fill(x, int(xo[-1]), 1, SEED)
        for _ in range(2):
            b.generate(x, counts)
    elif name == "inverse_bwbw":      # 2^17 bwbw events x 61 channels
        proc = whizard_process("bwbw")
        n = 1 << 17
        counts = np.full(proc.n_channels, n // proc.n_channels, np.int64)
        counts[: n - int(counts.sum())] += 1
        ps = PhaseSpace(proc, 500.0, 500.0)
        ps.set_variants(-1, 0)
        x = philox_x(n, proc.n_x, SEED)
        ev = ps.generate(x, counts)
        for _ in range(2):
            ps.inverse(ev.p, counts, ev.ok, x, ev.factor)
    elif name in ("adjoint_tt", "adjoint_tt_stored"):   # 2^20 tt events, recompute / stored
        from gpu_phs_gb300.api import ADJOINT_STORED
        proc = P.tt()
        n = 1 << 20
        ps = PhaseSpace(proc, 500.0, 500.0)
        if name == "adjoint_tt_stored":
            ps.set_adjoint_storage(ADJOINT_STORED)
        x = philox_x(n, proc.n_x, SEED)
        g = torch.Generator(device="cuda").manual_seed(SEED)
        pbar = torch.randn((n, proc.n_out, 4), dtype=torch.float64, device="cuda", generator=g)
        jbar = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
        for _ in range(2):
            ps.vjp(x, pbar, jbar)
    torch.cuda.synchronize()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=["tt", "ww", "precision"], default="tt")
    ap.add_argument("--events", type=int, default=0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--pin", default="-1,-1",
                    help="kernel variants of the fp32_mixed form (-1: autotune) and of the "
                         "fp64_split form (-1: 6) in the 13 TeV and batched measurements; for "
                         "profiled runs")
    ap.add_argument("--case", choices=PROFILE_CASES, default=None,
                    help="run one small profiling workload instead of the benchmark")
    args = ap.parse_args()
    if args.case:
        run_case(args.case)
        return
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
