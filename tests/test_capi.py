"""The C ABI: the library loads, exports every symbol include/gpu_phs.h declares, and
rejects malformed input with status codes (host-side only; no kernel launches)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from gpu_phs_gb300 import _lib
from gpu_phs_gb300 import processes as P

REF_SYMBOLS = [  # whizard_gpu_phs.cpp:12-132
    "c_whizard_set_particle_structure", "c_whizard_set_flavors", "c_whizard_init_mappings",
    "c_whizard_fill_mapping", "c_whizard_init_tree_structures", "c_whizard_fill_tree_structure",
    "c_whizard_init_channel_ids", "c_whizard_set_threads", "c_whizard_init_gpu_phs",
    "c_whizard_finalize_gpu_phs", "c_whizard_gen_phs_from_x_gpu",
    "c_whizard_get_momentum_device_pointer", "c_whizard_reset_generator",
    "c_whizard_show_module"]


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from gpu_phs_gb300 import build
        build.build()
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    declared = _lib.header_symbols()
    assert set(REF_SYMBOLS) <= set(declared)
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    for s in declared:
        assert getattr(lib, s) is not None


def test_every_declared_function_has_a_prototype():
    """The loader declares argument and result types for every function of the header:
    without them ctypes would pass 64-bit pointers as 32-bit ints."""
    declared = _lib.header_symbols()
    missing = [s for s in declared if s not in _lib._SIGS]
    assert not missing, missing


def test_exports_the_device_handoff_with_cpp_linkage(lib):
    """include/gpu_phs_transfer.h declares the reference's transfer_to_whizard.h functions
    with C++ linkage: the library exports them under their Itanium-mangled names."""
    import re
    hdr = os.path.join(os.path.dirname(_lib.HEADER), "gpu_phs_transfer.h")
    text = re.sub(r"/\*.*?\*/", "", open(hdr).read(), flags=re.S)
    names = re.findall(r"\b(get_\w+_device_pointer)\s*\(\s*\)", text)
    assert sorted(names) == ["get_in_momentum_device_pointer", "get_momentum_device_pointer",
                             "get_ok_device_pointer"]
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    for nm in names:
        mangled = f"_Z{len(nm)}{nm}v"
        assert mangled in exported, mangled
        assert getattr(lib, mangled) is not None


def _create(lib, proc, **over):
    t = dict(d1=proc.d1, d2=proc.d2, hc=proc.has_children, fr=proc.friends, mid=proc.map_ids,
             mm=proc.map_masses, mw=proc.map_widths, fm=proc.flv_masses, fw=proc.flv_widths)
    t.update(over)
    arrs = [np.ascontiguousarray(t[k], np.int32 if k in ("d1", "d2", "hc", "fr", "mid") else np.float64)
            for k in ("d1", "d2", "hc", "fr", "mid", "mm", "mw", "fm", "fw")]
    h = C.c_void_p()
    rc = lib.phs_process_create(C.byref(h), over.get("n_in", proc.n_in), over.get("n_out", proc.n_out),
                                proc.n_channels, over.get("n_x", proc.n_x),
                                *[a.ctypes.data for a in arrs])
    if rc == 0:
        lib.phs_process_destroy(h)
    return rc, lib.phs_last_error().decode()


def test_create_accepts_benchmark_processes(lib):
    for proc in (P.ww(), P.tt(), P.precision()):
        rc, msg = _create(lib, proc)
        assert rc == 0, msg


def test_create_rejects_malformed_trees(lib):
    proc = P.ww()
    d2 = proc.d2.copy()
    d2[0, 2] = 4                     # branch 3 -> (1, 4)
    rc, msg = _create(lib, proc, d2=d2)
    assert rc == -2 and "do not split" in msg
    hc = proc.has_children.copy()
    hc[0, 14] = 0                    # root without daughters
    rc, msg = _create(lib, proc, hc=hc)
    assert rc == -2
    hc = proc.has_children.copy()
    hc[0, 2] = 0                     # composite branch 3 left without daughters
    rc, msg = _create(lib, proc, hc=hc)
    assert rc == -2 and "composite" in msg


def test_create_rejects_unimplemented_mapping(lib):
    proc = P.ww()
    mid = proc.map_ids.copy()
    mid[0, 2] = 99                   # MAP_ONSHELL (phs.h:17) has no implementation
    rc, msg = _create(lib, proc, mid=mid)
    assert rc == -3 and "99" in msg


def test_create_rejects_bad_sizes(lib):
    proc = P.tt()
    rc, msg = _create(lib, proc, n_x=13)    # the tt tree consumes 14 x
    assert rc == -1 and "n_x" in msg
    rc, _ = _create(lib, proc, n_in=3)
    assert rc == -1
    h = C.c_void_p()
    assert lib.phs_process_create(C.byref(h), 2, 4, 1, 8, *([None] * 9)) == -1


def test_null_handles_are_errors(lib):
    assert lib.phs_process_set_beams(None, 250.0, 250.0) == -1
    assert lib.phs_generate_device(None, 0, None, None, None, None, None, None, None) == -1
    assert lib.phs_batch_generate_device(None, None, None, None, None, None, None, None) == -1
    assert lib.phs_process_destroy(None) == 0


ALLOC_FN = C.CFUNCTYPE(C.c_int, C.POINTER(C.c_void_p), C.c_size_t, C.c_void_p)
FREE_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p)


def test_device_allocator_failure_is_reported(lib):
    """An allocation failure injected through the device-allocator hook surfaces as
    PHS_ERR_ALLOC with the size in the message, and nothing is freed that was not made
    (host only: set_beams fails at its first device buffer, before any copy)."""
    from gpu_phs_gb300.api import _ptr
    asked, freed = [], []

    @ALLOC_FN
    def failing_alloc(ptr, nbytes, user):
        asked.append(nbytes)
        return 7

    @FREE_FN
    def record_free(ptr, user):
        freed.append(ptr)

    assert lib.phs_set_device_allocator(failing_alloc, None, None) == -1   # both or neither
    assert lib.phs_set_device_allocator(failing_alloc, record_free, None) == 0
    try:
        proc = P.ww()
        keep = [np.ascontiguousarray(a, dt) for a, dt in (
            (proc.d1, np.int32), (proc.d2, np.int32), (proc.has_children, np.int32),
            (proc.friends, np.int32), (proc.map_ids, np.int32), (proc.map_masses, np.float64),
            (proc.map_widths, np.float64), (proc.flv_masses, np.float64),
            (proc.flv_widths, np.float64))]
        h = C.c_void_p()
        assert lib.phs_process_create(C.byref(h), proc.n_in, proc.n_out, proc.n_channels,
                                      proc.n_x, *[_ptr(a) for a in keep]) == 0
        rc = lib.phs_process_set_beams(h, 250.0, 250.0)
        assert rc == -6                      # PHS_ERR_ALLOC
        msg = lib.phs_last_error().decode()
        assert "device allocator failed" in msg and str(asked[0]) in msg
        assert len(asked) == 1 and asked[0] > 0
        assert lib.phs_process_destroy(h) == 0
        assert freed == []
    finally:
        assert lib.phs_set_device_allocator(None, None, None) == 0
