"""ctypes loader for libgpuphs.so (the CUDA library).  There is no fallback: if the
library is missing or fails to load, importing the generator raises."""
from __future__ import annotations

import ctypes as C
import os
import re
from typing import List

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgpuphs.so")
# the bounds-checked build of the same library (csrc/phs_check.h), for tests
CHECKED_PATH = os.path.join(HERE, "libgpuphs_checked.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "gpu_phs.h")

_lib = None

P = C.c_void_p
I = C.c_int
I64 = C.c_int64
D = C.c_double

_SIGS = {
    "phs_last_error": (C.c_char_p, []),
    "phs_version": (C.c_char_p, []),
    "phs_set_device_allocator": (I, [P, P, P]),
    "phs_is_checked_build": (I, []),
    "phs_check_status": (I, [P, P]),
    "phs_process_create": (I, [C.POINTER(P), I, I, I, I, P, P, P, P, P, P, P, P, P]),
    "phs_process_destroy": (I, [P]),
    "phs_process_set_beams": (I, [P, D, D]),
    "phs_process_info": (I, [P, P, P, P, P, P]),
    "phs_process_set_precision": (I, [P, I]),
    "phs_process_set_adjoint_storage": (I, [P, I]),
    "phs_process_tuning": (I, [P, P, P]),
    "phs_process_set_variants": (I, [P, I, I]),
    "phs_batch_tuning": (I, [P, P, P]),
    "phs_batch_set_variants": (I, [P, I, I]),
    "phs_batch_set_precision": (I, [P, I]),
    "phs_generate_device": (I, [P, I64, P, P, P, P, P, P, P]),
    "phs_generate_beams_device": (I, [P, I64, P, P, P, P, P, P, P, P, P]),
    "phs_generate_host": (I, [P, I64, P, P, P, P, P, P]),
    "phs_adjoint_device": (I, [P, I64, P, P, P, P, P, P, P]),
    "phs_inverse_device": (I, [P, I64, P, P, P, P, P, P, P, P, P, P]),
    "phs_grid_create": (I, [C.POINTER(P), I, I]),
    "phs_grid_destroy": (I, [P]),
    "phs_grid_sample_device": (I, [P, I64, P, C.c_uint64, I64, P, P]),
    "phs_grid_update_device": (I, [P, I64, P, P, P, P]),
    "phs_grid_weights": (I, [P, P]),
    "phs_generate_device_noalloc": (I, [P, D, D, I64, P, P, P, P, P, P, P]),
    "phs_batch_create": (I, [C.POINTER(P), I, P]),
    "phs_batch_destroy": (I, [P]),
    "phs_batch_info": (I, [P, P, P, P]),
    "phs_batch_generate_device": (I, [P, P, P, P, P, P, P, P]),
    "phs_batch_offsets": (I, [P, P, P, P]),
    "phs_philox_fill": (I, [P, I64, I, C.c_uint64, I64, P]),
    "phs_batch_graph_create": (I, [C.POINTER(P), P, P, P, P, P, P, P]),
    "phs_process_graph_create": (I, [C.POINTER(P), P, I64, P, P, P, P, P, P]),
    "phs_graph_launch": (I, [P, P]),
    "phs_graph_destroy": (I, [P]),
    "phs_whizard_momentum_device_pointer": (P, []),
    "phs_measure_fma_peak": (I, [I, P]),
    "c_whizard_set_particle_structure": (None, [P] * 6),
    "c_whizard_set_flavors": (None, [P, P]),
    "c_whizard_init_mappings": (None, []),
    "c_whizard_fill_mapping": (None, [P, P, P, P]),
    "c_whizard_init_tree_structures": (None, []),
    "c_whizard_fill_tree_structure": (None, [P] * 5),
    "c_whizard_init_channel_ids": (None, [P, P, P]),
    "c_whizard_set_threads": (None, [P, P, P]),
    "c_whizard_init_gpu_phs": (None, []),
    "c_whizard_finalize_gpu_phs": (None, []),
    "c_whizard_gen_phs_from_x_gpu": (None, [P] * 12),
    "c_whizard_get_momentum_device_pointer": (None, [P]),
    "c_whizard_reset_generator": (None, []),
    "c_whizard_show_module": (None, []),
}


class PhsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gpu_phs error {code}: {msg}")
        self.code = code


def header_symbols() -> List[str]:
    """Function names declared in include/gpu_phs.h."""
    with open(HEADER) as fh:
        text = fh.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b((?:phs|c_whizard)_\w+)\s*\(", text)))


def _open(path: str) -> C.CDLL:
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def load() -> C.CDLL:
    """Loads libgpuphs.so (built by gpu_phs_gb300.build).  Inside `using(lib)` it returns
    that library instead."""
    global _lib
    if _active is not None:
        return _active
    if _lib is None:
        _lib = _open(LIB_PATH)
    return _lib


_checked = None
_active = None


def load_checked() -> C.CDLL:
    """Loads libgpuphs_checked.so, the bounds-checked build, beside the regular one (its
    own symbols and kernels: ctypes opens each library with local symbol binding)."""
    global _checked
    if _checked is None:
        _checked = _open(CHECKED_PATH)
    return _checked


class using:
    """with using(lib): the Python API (PhaseSpace, Batch, ...) calls `lib` instead of
    libgpuphs.so.  Handles made inside belong to that library: close them inside."""

    def __init__(self, lib: C.CDLL):
        self.lib = lib

    def __enter__(self):
        global _active
        self.prev, _active = _active, self.lib
        return self.lib

    def __exit__(self, *exc):
        global _active
        _active = self.prev


def check(rc: int, lib: C.CDLL = None) -> None:
    """Raises PhsError for a non-zero status, with the message of `lib` (the library that
    made the call; default: load())."""
    if rc != 0:
        raise PhsError(rc, (lib or load()).phs_last_error().decode())
