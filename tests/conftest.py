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


def counts_of(channels, n_channels):
    return np.bincount(channels, minlength=n_channels).astype(np.int64)
