"""Regenerates the golden fixtures in tests/golden/ (run where the reference sources are:
the directory oracle.reference_dir() names, $GPU_PHS_REFERENCE_DIR or oracle/Makefile's
REF; the fixtures themselves travel without it).

Two kinds of fixture, each a compressed .npz:

* ``whizard_<name>.npz`` -- a subset of the reference's own Whizard sample files
  (samples/ttH.ref, samples/bwbw.ref): the process tables, the per-channel
  ``hasfriends`` flag with the friend table derived from it
  (gpu_phs_gb300.refformat.friends_from_trees), and per event the channel, x (9
  printed decimals), the outgoing momenta, volume, ok, the event's own-channel
  factor and the factors of all channels (``all_factors``, Whizard's inverse
  mapping; printed to a fixed number of decimals).  These are the golden vectors the
  reference's test.sh checks against.
* ``refcpu_<name>.npz`` -- outputs of the reference's own phs_cpu.cpp (compiled
  from the reference sources by ``make -C oracle ref``) on seeded Philox x for
  the benchmark processes: the process tables, the Philox seed, sqrt(s) and the
  per-event p, factor, volume, ok (p/factor/volume are defined only where ok).

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gpu_phs_gb300 import processes as P  # noqa: E402
from gpu_phs_gb300.philox import uniform_x  # noqa: E402
from gpu_phs_gb300.refformat import read_ref  # noqa: E402
from oracle import oracle  # noqa: E402

SAMPLES = os.path.join(oracle.reference_dir(), "samples")


def proc_arrays(proc, prefix=""):
    return {prefix + k: getattr(proc, k) for k in
            ("d1", "d2", "has_children", "friends", "map_ids", "map_masses", "map_widths",
             "flv_masses", "flv_widths")} | {
        prefix + "meta": np.array([proc.n_in, proc.n_out, proc.n_x], np.int64),
        prefix + "sqrts_nominal": np.array([proc.sqrts]),
    }


def whizard_fixture(name: str, per_channel: int) -> None:
    proc, friends_flag, ev = read_ref(os.path.join(SAMPLES, f"{name}.ref"))
    keep = []
    seen = {}
    for i, c in enumerate(ev.channel):
        if seen.get(int(c), 0) < per_channel:
            keep.append(i)
            seen[int(c)] = seen.get(int(c), 0) + 1
    keep = np.array(keep)
    own = ev.all_factors[np.arange(len(ev.ok)), ev.channel]
    out = proc_arrays(proc) | {
        "hasfriends": friends_flag,
        "channel": ev.channel[keep], "x": ev.x[keep], "p_out": ev.p_out[keep],
        "p_in": ev.p_in[keep], "volume": ev.volume[keep], "ok": ev.ok[keep],
        "factor": own[keep], "all_factors": ev.all_factors[keep],
    }
    path = os.path.join(HERE, f"whizard_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {len(keep)} events, {proc.n_channels} channels")


def refcpu_fixture(name: str, proc, n_events: int, seed: int, sqrts: float) -> None:
    x = uniform_x(seed, n_events, proc.n_x)
    ref = oracle.RefCPU(proc, sqrts)
    channels = np.arange(n_events, dtype=np.int32) * proc.n_channels // n_events
    r = ref.generate(x, channels)
    out = proc_arrays(proc) | {
        "seed": np.array([seed], np.int64), "sqrts": np.array([sqrts]),
        "channel": channels, "x_checksum": np.array([x.sum()]),
        "p": r.p, "factor": r.factor, "volume": r.volume, "ok": r.ok,
    }
    path = os.path.join(HERE, f"refcpu_{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {n_events} events, ok fraction {r.ok.mean():.4f}")


def main() -> None:
    oracle.build(ref=True)
    whizard_fixture("ttH", per_channel=100)
    whizard_fixture("bwbw", per_channel=1000)
    refcpu_fixture("ww", P.ww(), 256, seed=11, sqrts=500.0)
    refcpu_fixture("tt", P.tt(), 512, seed=12, sqrts=1000.0)
    refcpu_fixture("precision", P.precision(), 512, seed=13, sqrts=13000.0)
    rng = np.random.default_rng(14)
    for n_out in range(3, 9):
        proc = P.random_process(rng, n_out, 4, 1000.0, name=f"random_n{n_out}")
        n_ev = 256 if n_out < 5 else 2048
        refcpu_fixture(f"random_n{n_out}", proc, n_ev, seed=100 + n_out, sqrts=1000.0)


if __name__ == "__main__":
    main()
