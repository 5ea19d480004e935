"""Python front end of libgpuphs, over its C ABI (include/gpu_phs.h).

PyTorch supplies device memory and streams only; every computation runs in the CUDA
library.  ``PhaseSpace`` mirrors the reference's generate call gen_phs_from_x_gpu
(phs.cu:1333) for one process, ``Batch`` runs many processes in one launch.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from ._lib import check, load
from .processes import Process


def _ptr(t) -> Optional[int]:
    if t is None:
        return None
    if isinstance(t, np.ndarray):
        return t.ctypes.data
    return t.data_ptr()


def _stream(stream) -> Optional[int]:
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


@dataclass
class Events:
    p: "object"       # [n, n_out, 4] float64
    factor: "object"  # [n] float64
    volume: "object"  # [n] float64
    ok: "object"      # [n] uint8


PRECISION_F64 = 0     # IEEE FP64 throughout
PRECISION_F32X2 = 1   # float-float pairs on the FP32 pipe, FP64 next to kinematic limits
ADJOINT_RECOMPUTE = 0  # vjp recovers parent frames with inverse boosts (no scratch)
ADJOINT_STORED = 1     # vjp keeps every visit's parent frame in a device buffer


class _Handle:
    """A library handle: its calls report errors from the library that made it."""

    _L = None

    def _check(self, rc: int) -> None:
        check(rc, self._L)


class PhaseSpace(_Handle):
    """One process on the current CUDA device."""

    def __init__(self, proc: Process, E1: Optional[float] = None, E2: Optional[float] = None):
        lib = self._L = load()   # the library this handle belongs to (_lib.using)
        self.proc = proc
        self._keep = [np.ascontiguousarray(a, dt) for a, dt in (
            (proc.d1, np.int32), (proc.d2, np.int32), (proc.has_children, np.int32),
            (proc.friends, np.int32), (proc.map_ids, np.int32), (proc.map_masses, np.float64),
            (proc.map_widths, np.float64), (proc.flv_masses, np.float64),
            (proc.flv_widths, np.float64))]
        h = C.c_void_p()
        check(lib.phs_process_create(C.byref(h), proc.n_in, proc.n_out, proc.n_channels,
                                     proc.n_x, *[_ptr(a) for a in self._keep]), lib)
        self.h = h
        if E1 is not None:
            self.set_beams(E1, E2 if E2 is not None else E1)

    def set_beams(self, E1: float, E2: float) -> None:
        self._check(self._L.phs_process_set_beams(self.h, float(E1), float(E2)))

    def set_precision(self, precision: int) -> None:
        """PRECISION_F64 (default) or PRECISION_F32X2 for the uniform-beam generate calls."""
        self._check(self._L.phs_process_set_precision(self.h, int(precision)))

    def set_adjoint_storage(self, storage: int) -> None:
        """ADJOINT_RECOMPUTE (default) or ADJOINT_STORED for vjp (the stored-matrix form,
        kept for comparison: a device buffer of n x max visits x 128 bytes)."""
        self._check(self._L.phs_process_set_adjoint_storage(self.h, int(storage)))

    def tuning(self):
        """(ff_variant, f64_variant) the autotuner chose (-1: not tuned yet)."""
        f, d = C.c_int(), C.c_int()
        self._check(self._L.phs_process_tuning(self.h, C.byref(f), C.byref(d)))
        return f.value, d.value

    def set_variants(self, ff_variant: int = -1, f64_variant: int = -1) -> None:
        """Pins the kernel variants (-1: autotune)."""
        self._check(self._L.phs_process_set_variants(self.h, int(ff_variant), int(f64_variant)))

    def close(self) -> None:
        if getattr(self, "h", None):
            self._L.phs_process_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        v = [C.c_int() for _ in range(5)]
        self._check(self._L.phs_process_info(self.h, *[C.byref(i) for i in v]))
        return dict(zip(("n_in", "n_out", "n_channels", "n_x", "stack_depth"), [i.value for i in v]))

    def alloc(self, n: int, device="cuda") -> Events:
        import torch
        return Events(torch.empty((n, self.proc.n_out, 4), dtype=torch.float64, device=device),
                      torch.empty(n, dtype=torch.float64, device=device),
                      torch.empty(n, dtype=torch.float64, device=device),
                      torch.empty(n, dtype=torch.uint8, device=device))

    @staticmethod
    def _counts(counts, n_channels: int, n: int) -> Optional[np.ndarray]:
        if counts is None:
            if n_channels != 1:
                raise ValueError("counts are required for a multi-channel process")
            return None
        c = np.ascontiguousarray(counts, np.int64)
        if c.shape != (n_channels,):
            raise ValueError(f"counts must have shape ({n_channels},)")
        return c

    def generate(self, x, counts=None, out: Optional[Events] = None, stream=None) -> Events:
        """x: CUDA float64 [n, n_x]; events grouped by channel with ``counts`` per channel."""
        n = int(x.shape[0])
        if x.dtype.itemsize != 8 or not x.is_cuda or not x.is_contiguous():
            raise ValueError("x must be a contiguous CUDA float64 tensor")
        if x.dim() != 2 or x.shape[1] != self.proc.n_x:
            raise ValueError(f"x must be [n, {self.proc.n_x}]")
        out = out or self.alloc(n, x.device)
        c = self._counts(counts, self.proc.n_channels, n)
        self._check(self._L.phs_generate_device(self.h, n, _ptr(c), _ptr(x), _ptr(out.p),
                                         _ptr(out.factor), _ptr(out.volume), _ptr(out.ok),
                                         _stream(stream)))
        return out

    def generate_beams(self, x, E1, E2, counts=None, out: Optional[Events] = None,
                       stream=None) -> Events:
        """Per-event beam energies E1[n], E2[n] (CUDA float64)."""
        n = int(x.shape[0])
        out = out or self.alloc(n, x.device)
        c = self._counts(counts, self.proc.n_channels, n)
        self._check(self._L.phs_generate_beams_device(self.h, n, _ptr(c), _ptr(E1), _ptr(E2), _ptr(x),
                                               _ptr(out.p), _ptr(out.factor), _ptr(out.volume),
                                               _ptr(out.ok), _stream(stream)))
        return out

    def vjp(self, x, pbar, jbar=None, counts=None, stream=None):
        """Reverse-mode derivatives (FP64): for cotangents pbar [n, n_out, 4] of the momenta
        and jbar [n] of log(factor), returns xbar [n, n_x] and thbar [n, n_out - 2, 2]
        (d/dm, d/dGamma of the Breit-Wigner branch at each msq x index)."""
        import torch
        n = int(x.shape[0])
        xbar = torch.empty_like(x)
        thbar = torch.empty((n, max(1, self.proc.n_out - 2), 2), dtype=torch.float64, device=x.device)
        c = self._counts(counts, self.proc.n_channels, n)
        pbar = pbar.contiguous()
        jbar = jbar.contiguous() if jbar is not None else None
        self._check(self._L.phs_adjoint_device(self.h, n, _ptr(c), _ptr(x), _ptr(pbar), _ptr(jbar),
                                        _ptr(xbar), _ptr(thbar), _stream(stream)))
        return xbar, thbar

    def inverse(self, p, counts=None, ok=None, x=None, factor=None, E1=None, E2=None,
                stream=None):
        """All-channel factors [n, n_channels] and x [n_channels, n, n_x] of events with lab
        momenta p [n, n_out, 4] (CUDA float64), events grouped by generating channel.  With
        x (and factor) the generating channel's row is copied from them, as the reference
        does; without, it is inverted like the others (a round trip of the forward map)."""
        import torch
        n = int(p.shape[0])
        if p.dtype != torch.float64 or not p.is_cuda or not p.is_contiguous():
            raise ValueError("p must be a contiguous CUDA float64 tensor")
        nch = self.proc.n_channels
        fac = torch.empty((n, nch), dtype=torch.float64, device=p.device)
        xo = torch.empty((nch, n, self.proc.n_x), dtype=torch.float64, device=p.device)
        c = self._counts(counts, nch, n)
        self._check(self._L.phs_inverse_device(self.h, n, _ptr(c), _ptr(E1), _ptr(E2), _ptr(p), _ptr(ok),
                                        _ptr(x), _ptr(factor), _ptr(fac), _ptr(xo),
                                        _stream(stream)))
        return fac, xo

    def generate_host(self, x, counts=None, out: Optional[Events] = None) -> Events:
        """Host (ideally pinned) tensors or arrays in and out; synchronous."""
        import torch
        n = int(x.shape[0])
        if out is None:
            out = Events(torch.empty((n, self.proc.n_out, 4), dtype=torch.float64),
                         torch.empty(n, dtype=torch.float64), torch.empty(n, dtype=torch.float64),
                         torch.empty(n, dtype=torch.uint8))
        c = self._counts(counts, self.proc.n_channels, n)
        self._check(self._L.phs_generate_host(self.h, n, _ptr(c), _ptr(x), _ptr(out.p), _ptr(out.factor),
                                       _ptr(out.volume), _ptr(out.ok)))
        return out


class Batch(_Handle):
    """Many processes (uneven n_out, n_x and counts) in one persistent launch."""

    def __init__(self, spaces: Sequence[PhaseSpace]):
        self.spaces = list(spaces)
        self._L = self.spaces[0]._L if self.spaces else load()
        arr = (C.c_void_p * len(self.spaces))(*[s.h.value for s in self.spaces])
        h = C.c_void_p()
        self._check(self._L.phs_batch_create(C.byref(h), len(self.spaces), C.cast(arr, C.c_void_p)))
        self.h = h
        self.n_outs: List[int] = []
        self.n_xs: List[int] = []
        for s in self.spaces:
            self.n_outs += [s.proc.n_out] * s.proc.n_channels
            self.n_xs += [s.proc.n_x] * s.proc.n_channels

    def close(self) -> None:
        if getattr(self, "h", None):
            self._L.phs_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_channels(self) -> int:
        return len(self.n_outs)

    def set_precision(self, precision: int) -> None:
        self._check(self._L.phs_batch_set_precision(self.h, int(precision)))

    def tuning(self):
        f, d = C.c_int(), C.c_int()
        self._check(self._L.phs_batch_tuning(self.h, C.byref(f), C.byref(d)))
        return f.value, d.value

    def set_variants(self, ff_variant: int = -1, f64_variant: int = -1) -> None:
        self._check(self._L.phs_batch_set_variants(self.h, int(ff_variant), int(f64_variant)))

    def offsets(self, counts):
        c = np.ascontiguousarray(counts, np.int64)
        xo = np.zeros(self.n_channels + 1, np.int64)
        po = np.zeros(self.n_channels + 1, np.int64)
        self._check(self._L.phs_batch_offsets(self.h, _ptr(c), _ptr(xo), _ptr(po)))
        return xo, po

    def generate(self, x, counts, p=None, factor=None, volume=None, ok=None, stream=None):
        """x: flat CUDA float64 of all channels' x rows; returns flat p and per-event arrays."""
        import torch
        c = np.ascontiguousarray(counts, np.int64)
        n = int(c.sum())
        xo, po = self.offsets(c)
        dev = x.device
        p = p if p is not None else torch.empty(int(po[-1]), dtype=torch.float64, device=dev)
        factor = factor if factor is not None else torch.empty(n, dtype=torch.float64, device=dev)
        volume = volume if volume is not None else torch.empty(n, dtype=torch.float64, device=dev)
        ok = ok if ok is not None else torch.empty(n, dtype=torch.uint8, device=dev)
        self._check(self._L.phs_batch_generate_device(self.h, _ptr(c), _ptr(x), _ptr(p), _ptr(factor),
                                               _ptr(volume), _ptr(ok), _stream(stream)))
        return p, factor, volume, ok


class Graph(_Handle):
    """A captured generate call (fixed pointers and counts); launch() replays it."""

    def __init__(self, handle, lib=None):
        self.h = handle
        self._L = lib or load()

    def launch(self, stream=None) -> None:
        self._check(self._L.phs_graph_launch(self.h, _stream(stream)))

    def close(self) -> None:
        if getattr(self, "h", None):
            self._L.phs_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_graph(batch: "Batch", x, counts, p, factor, volume, ok) -> Graph:
    c = np.ascontiguousarray(counts, np.int64)
    h = C.c_void_p()
    check(batch._L.phs_batch_graph_create(C.byref(h), batch.h, _ptr(c), _ptr(x), _ptr(p),
                                          _ptr(factor), _ptr(volume), _ptr(ok)), batch._L)
    g = Graph(h, batch._L)
    g._keep = (batch, x, c, p, factor, volume, ok)
    return g


def process_graph(ps: PhaseSpace, x, out: Events, counts=None) -> Graph:
    n = int(x.shape[0])
    c = ps._counts(counts, ps.proc.n_channels, n)
    h = C.c_void_p()
    check(ps._L.phs_process_graph_create(C.byref(h), ps.h, n, _ptr(c), _ptr(x), _ptr(out.p),
                                         _ptr(out.factor), _ptr(out.volume), _ptr(out.ok)), ps._L)
    g = Graph(h, ps._L)
    g._keep = (ps, x, c, out)
    return g


GRID_BINS = 10


class Grid(_Handle):
    """Per-channel x grid of the warm-up (rng.cpp): weights [n_channels, n_x, 10] on the
    device, uniform at first."""

    def __init__(self, n_channels: int, n_x: int):
        h = C.c_void_p()
        self._L = load()
        self._check(self._L.phs_grid_create(C.byref(h), int(n_channels), int(n_x)))
        self.h, self.n_channels, self.n_x = h, int(n_channels), int(n_x)

    def close(self) -> None:
        if getattr(self, "h", None):
            self._L.phs_grid_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _counts(self, counts, n):
        if counts is None:
            if self.n_channels != 1:
                raise ValueError("counts are required for a multi-channel grid")
            return None
        return np.ascontiguousarray(counts, np.int64)

    def sample(self, n_events: int, counts=None, seed: int = 0, first_event: int = 0,
               out=None, stream=None):
        """x [n_events, n_x] (CUDA float64) drawn from each channel's grid."""
        import torch
        x = out if out is not None else torch.empty((n_events, self.n_x), dtype=torch.float64,
                                                    device="cuda")
        c = self._counts(counts, n_events)
        self._check(self._L.phs_grid_sample_device(self.h, int(n_events), _ptr(c), int(seed),
                                            int(first_event), _ptr(x), _stream(stream)))
        return x

    def update(self, x, ok, counts=None, stream=None) -> None:
        """Weights from the ok events' x (rng.cpp:34-67)."""
        c = self._counts(counts, int(x.shape[0]))
        self._check(self._L.phs_grid_update_device(self.h, int(x.shape[0]), _ptr(c), _ptr(x), _ptr(ok),
                                            _stream(stream)))

    def weights(self) -> np.ndarray:
        w = np.zeros((self.n_channels, self.n_x, GRID_BINS))
        self._check(self._L.phs_grid_weights(self.h, w.ctypes.data))
        return w


def precondition(ps: "PhaseSpace", grid: Grid, n_trials: int, n_per_channel: int,
                 seed: int = 0):
    """The reference's grid warm-up (main.cpp:145-157): n_trials rounds of sampling
    n_per_channel events per channel, generating them, and updating the grid from their
    ok flags.  Returns the ok fraction of each round."""
    counts = np.full(ps.proc.n_channels, int(n_per_channel), np.int64)
    n = int(counts.sum())
    fractions = []
    for t in range(int(n_trials)):
        x = grid.sample(n, counts, seed=seed, first_event=t * n)
        ev = ps.generate(x, counts)
        grid.update(x, ev.ok, counts)
        fractions.append(ev.ok.double().mean().item())
    return fractions


def philox_fill(x, n_events: int, n_x: int, seed: int, first_event: int = 0, stream=None):
    """Fills CUDA float64 x[n_events * n_x] with the Philox stream (gpu_phs_gb300/philox.py)."""
    check(load().phs_philox_fill(_ptr(x), n_events, n_x, seed, first_event, _stream(stream)))
    return x


def philox_x(n_events: int, n_x: int, seed: int, first_event: int = 0, device="cuda"):
    import torch
    x = torch.empty((n_events, n_x), dtype=torch.float64, device=device)
    return philox_fill(x, n_events, n_x, seed, first_event)
