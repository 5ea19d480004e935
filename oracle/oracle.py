"""ctypes front end for the CPU oracles.  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module.  Two oracles, both built by oracle/Makefile:

* ``Oracle``    -- the C restatement in phs_oracle.c (_build/libphsoracle.so).
* ``RefCPU``    -- the reference's own phs_cpu.cpp driven by ref_harness.cpp
                   (_ref/libphsref.so); present only where the reference sources
                   were available to compile it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libphsoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libphsref.so")


def reference_dir() -> str:
    """Directory of the reference sources: $GPU_PHS_REFERENCE_DIR, else the default of
    oracle/Makefile (REF).  It need not exist: the GPU machine has no reference sources."""
    env = os.environ.get("GPU_PHS_REFERENCE_DIR")
    if env:
        return env
    r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
    return r.stdout.strip()


_pd = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_pi = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_pu8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def build(ref: bool = True) -> None:
    """Compile the restatement, and the reference harness when the reference sources exist."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    src = reference_dir()
    if ref and os.path.exists(os.path.join(src, "phs_cpu.cpp")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={src}"], check=True)


def _load(path: str) -> C.CDLL:
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is not built; run `make -C oracle`")
    return C.CDLL(path)


def _tables(proc):
    return (np.ascontiguousarray(proc.d1, np.int32), np.ascontiguousarray(proc.d2, np.int32),
            np.ascontiguousarray(proc.has_children, np.int32),
            np.ascontiguousarray(proc.map_ids, np.int32),
            np.ascontiguousarray(proc.map_masses, np.float64),
            np.ascontiguousarray(proc.map_widths, np.float64))


class Result:
    def __init__(self, n: int, n_out: int):
        self.p = np.zeros((n, n_out, 4))
        self.factor = np.zeros(n)
        self.volume = np.zeros(n)
        self.ok = np.zeros(n, np.uint8)


class Oracle:
    """The C restatement of the reference CPU path for one process."""

    _lib: Optional[C.CDLL] = None

    @classmethod
    def lib(cls) -> C.CDLL:
        if cls._lib is None:
            L = _load(ORACLE_SO)
            L.oracle_create.restype = C.c_void_p
            L.oracle_create.argtypes = [C.c_int, C.c_int, C.c_int, _pi, _pi, _pi, _pi, _pd, _pd, _pd]
            L.oracle_destroy.argtypes = [C.c_void_p]
            L.oracle_set_sqrts.argtypes = [C.c_void_p, C.c_double]
            L.oracle_get_constants.argtypes = [C.c_void_p, C.c_int, _pd, _pd]
            L.oracle_mass_sum.restype = C.c_double
            L.oracle_mass_sum.argtypes = [C.c_void_p, C.c_int, C.c_int]
            L.oracle_generate.argtypes = [C.c_void_p, C.c_long, C.c_int, _pd, C.c_void_p,
                                          _pd, _pd, _pd, _pu8, C.c_int]
            L.oracle_generate_beams.argtypes = [C.c_void_p, C.c_long, C.c_int, _pd, C.c_void_p,
                                                _pd, _pd, _pd, _pd, _pd, _pu8, C.c_int]
            L.oracle_generate_cond.argtypes = [C.c_void_p, C.c_long, C.c_int, _pd, C.c_void_p,
                                               _pd, _pd, _pd, _pu8, _pd, C.c_int]
            L.oracle_set_nudge.argtypes = [C.c_void_p, C.c_int]
            L.oracle_set_friends.restype = C.c_int
            L.oracle_set_friends.argtypes = [C.c_void_p, _pi]
            L.oracle_inverse.restype = C.c_int
            L.oracle_inverse.argtypes = [C.c_void_p, C.c_long, C.c_int, _pd, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, _pd, _pd, C.c_int]
            cls._lib = L
        return cls._lib

    def __init__(self, proc, sqrts: float):
        L = self.lib()
        self.proc = proc
        t = _tables(proc)
        self.h = L.oracle_create(proc.n_in, proc.n_out, proc.n_channels, *t,
                                 np.ascontiguousarray(proc.flv_masses, np.float64))
        if not self.h:
            raise ValueError("oracle rejected the process tables")
        fr = np.ascontiguousarray(proc.friends, np.int32)
        if fr.any() and L.oracle_set_friends(self.h, fr) != 0:
            raise ValueError("oracle rejected the friend table")
        L.oracle_set_sqrts(self.h, float(sqrts))
        self.sqrts = float(sqrts)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib().oracle_destroy(self.h)
            self.h = None

    def constants(self, channel: int):
        n = 1 << self.proc.n_out
        a = np.zeros(3 * n)
        b = np.zeros(3 * n)
        self.lib().oracle_get_constants(self.h, channel, a, b)
        return a.reshape(n, 3), b.reshape(n, 3)

    def mass_sum(self, channel: int, code: int) -> float:
        return self.lib().oracle_mass_sum(self.h, channel, code)

    def generate(self, x: np.ndarray, channels: Optional[np.ndarray] = None,
                 threads: int = 0, E1: Optional[np.ndarray] = None,
                 E2: Optional[np.ndarray] = None, condition: bool = False,
                 nudge: int = 0) -> Result:
        """condition=True (uniform beams) also returns r.kappa, the per-event condition of
        the Kallen functions (oracle_generate_cond in phs_oracle.c).  nudge != 0: a
        sensitivity probe for tests (oracle_set_nudge) -- every value a transcendental
        function returns on the mapping path moved by that many ulps: the maps' tan, exp and
        log, and with per-event beams the constants formed per event; the uniform-beam
        constants stay the reference's."""
        x = np.ascontiguousarray(x, np.float64)
        n, n_x = x.shape
        r = Result(n, self.proc.n_out)
        chp = None
        if channels is not None:
            channels = np.ascontiguousarray(channels, np.int32)
            chp = channels.ctypes.data_as(C.c_void_p)
        threads = threads or os.cpu_count() or 1
        if condition and E1 is not None:
            raise ValueError("condition numbers are computed for uniform beams")
        self.lib().oracle_set_nudge(self.h, int(nudge))
        try:
            if condition:
                r.kappa = np.zeros(n)
                self.lib().oracle_generate_cond(self.h, n, n_x, x.reshape(-1), chp,
                                                r.p.reshape(-1), r.factor, r.volume, r.ok,
                                                r.kappa, threads)
            elif E1 is None:
                self.lib().oracle_generate(self.h, n, n_x, x.reshape(-1), chp, r.p.reshape(-1),
                                           r.factor, r.volume, r.ok, threads)
            else:
                E1 = np.ascontiguousarray(np.broadcast_to(E1, (n,)), np.float64)
                E2 = np.ascontiguousarray(np.broadcast_to(E2, (n,)), np.float64)
                self.lib().oracle_generate_beams(self.h, n, n_x, x.reshape(-1), chp, E1, E2,
                                                 r.p.reshape(-1), r.factor, r.volume, r.ok,
                                                 threads)
        finally:
            self.lib().oracle_set_nudge(self.h, 0)
        return r

    def inverse(self, p: np.ndarray, channels: Optional[np.ndarray] = None,
                ok: Optional[np.ndarray] = None, x_own: Optional[np.ndarray] = None,
                factor_own: Optional[np.ndarray] = None, n_x: Optional[int] = None,
                E1: Optional[np.ndarray] = None, E2: Optional[np.ndarray] = None,
                threads: int = 0, nudge: int = 0):
        """All-channel factors [n, n_channels] and x [n_channels, n, n_x] of events with
        lab momenta p [n, n_out, 4] (phs.cu:1499-1554).  With x_own/factor_own the
        generating channel's row is copied, otherwise inverted like the others.  nudge != 0:
        the sensitivity probe of generate(nudge=...), on the inverse maps' atan, exp and
        log too."""
        p = np.ascontiguousarray(p, np.float64)
        n = p.shape[0]
        n_x = n_x or (x_own.shape[1] if x_own is not None else self.proc.n_x)
        keep = []

        def vp(a, dt):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dt)
            keep.append(a)
            return a.ctypes.data_as(C.c_void_p)

        if E1 is not None:
            E1 = np.broadcast_to(E1, (n,))
            E2 = np.broadcast_to(E2, (n,))
        fac = np.zeros((n, self.proc.n_channels))
        xo = np.zeros((self.proc.n_channels, n, n_x))
        threads = threads or os.cpu_count() or 1
        self.lib().oracle_set_nudge(self.h, int(nudge))
        try:
            self.lib().oracle_inverse(self.h, n, n_x, p.reshape(-1), vp(channels, np.int32),
                                      vp(ok, np.uint8), vp(E1, np.float64), vp(E2, np.float64),
                                      vp(x_own, np.float64), vp(factor_own, np.float64),
                                      fac.reshape(-1), xo.reshape(-1), threads)
        finally:
            self.lib().oracle_set_nudge(self.h, 0)
        return fac, xo


def uniform_x(seed: int, n_events: int, n_x: int, first_event: int = 0,
              threads: int = 0) -> np.ndarray:
    """The Philox stream of gpu_phs_gb300.philox.uniform_x (the same values), computed by
    the oracle library on all host threads: for full-size workloads."""
    L = Oracle.lib()
    if not hasattr(L, "_ux"):
        L.oracle_uniform_x.restype = C.c_int
        L.oracle_uniform_x.argtypes = [C.c_uint64, C.c_long, C.c_long, C.c_int, _pd, C.c_int]
        L._ux = True
    x = np.empty((n_events, n_x), np.float64)
    if n_events:
        rc = L.oracle_uniform_x(seed, first_event, n_events, n_x, x.reshape(-1),
                                threads or os.cpu_count() or 1)
        if rc != 0:
            raise ValueError("bad sizes")
    return x


def ref_available() -> bool:
    return os.path.exists(REF_SO)


class RefCPU:
    """The reference's own phs_cpu.cpp (process-global state: one process at a time)."""

    _lib: Optional[C.CDLL] = None

    @classmethod
    def lib(cls) -> C.CDLL:
        if cls._lib is None:
            L = _load(REF_SO)
            L.ref_setup.restype = C.c_int
            L.ref_setup.argtypes = [C.c_int, C.c_int, C.c_int, _pi, _pi, _pi, _pi, _pd, _pd,
                                    _pd, _pd, C.c_double]
            L.ref_generate.restype = C.c_int
            L.ref_generate.argtypes = [C.c_long, C.c_int, _pd, C.c_void_p, C.c_double, _pd, _pd,
                                       _pd, _pu8, C.c_int]
            L.ref_teardown.argtypes = []
            cls._lib = L
        return cls._lib

    def __init__(self, proc, sqrts: float):
        self.proc = proc
        self.sqrts = float(sqrts)
        t = _tables(proc)
        self.lib().ref_setup(proc.n_in, proc.n_out, proc.n_channels, *t,
                             np.ascontiguousarray(proc.flv_masses, np.float64),
                             np.ascontiguousarray(proc.flv_widths, np.float64), self.sqrts)

    def generate(self, x: np.ndarray, channels: Optional[np.ndarray] = None,
                 threads: int = 0) -> Result:
        x = np.ascontiguousarray(x, np.float64)
        n, n_x = x.shape
        r = Result(n, self.proc.n_out)
        chp = None
        if channels is not None:
            channels = np.ascontiguousarray(channels, np.int32)
            chp = channels.ctypes.data_as(C.c_void_p)
        threads = threads or os.cpu_count() or 1
        rc = self.lib().ref_generate(n, n_x, x.reshape(-1), chp, self.sqrts, r.p.reshape(-1),
                                     r.factor, r.volume, r.ok, threads)
        if rc != 0:
            raise RuntimeError("reference harness not set up")
        return r


# --------------------------------------------------------------------------- x grids
GRID_BINS = 10


def grid_update(weights, x, counts, ok):
    """update_weights (rng.cpp:34-67) restated: per channel and dimension, the fraction of
    the channel's ok events whose x falls into each of the 10 bins.  Channels without ok
    events keep their weights (the reference divides by zero there)."""
    w = np.array(weights, dtype=np.float64, copy=True)
    ch = np.repeat(np.arange(len(counts)), counts)
    ok = np.asarray(ok).astype(bool)
    for c in range(len(counts)):
        sel = (ch == c) & ok
        n_ok = int(sel.sum())
        if n_ok == 0:
            continue
        b = np.clip((x[sel] * GRID_BINS).astype(np.int64), 0, GRID_BINS - 1)
        for d in range(x.shape[1]):
            cnt = np.bincount(b[:, d], minlength=GRID_BINS).astype(np.float64)
            w[c, d] = cnt / n_ok
    return w


def grid_sample(weights, u, counts):
    """The inverse distribution function of the piecewise-constant density (the device
    sampler's formula): bin b with C[b] <= u among bins of positive weight, x = (b + (u -
    C[b]) / w[b]) / 10, the offset kept inside [0, 1)."""
    ch = np.repeat(np.arange(len(counts)), counts)
    x = np.empty_like(u)
    for i in range(u.shape[0]):
        for d in range(u.shape[1]):
            w = weights[ch[i], d]
            c, b = 0.0, 0
            for k in range(GRID_BINS):
                if w[k] > 0.0 and c <= u[i, d]:
                    b = k
                c += w[k]
            cb = 0.0
            for k in range(b):
                cb += w[k]
            t = (u[i, d] - cb) / w[b]
            t = 0.0 if t < 0.0 else (np.nextafter(1.0, 0.0) if t >= 1.0 else t)
            x[i, d] = (b + t) / GRID_BINS
    return x