"""CPU checks of the C-ABI library: it loads and exports every symbol that
include/mrsph_relax.h declares (no compute calls without a GPU)."""
import ctypes
import os
import re

from mrsph import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            syms |= set(re.findall(r"^\s*int\s+(mrsph_\w+)\s*\(", txt, flags=re.M))
    return syms


def test_library_exports_every_declared_symbol():
    lib = L.load()
    syms = declared_symbols()
    assert len(syms) >= 18
    for s in sorted(syms):
        assert hasattr(lib, s), s
    assert set(L.EXPORTS) >= syms


def test_version_and_create_errors_without_gpu():
    lib = L.load()
    assert lib.mrsph_version() == 1
    # invalid parameters are rejected before any device call
    p = L.Params()
    p.dim = 5
    h = ctypes.c_void_p()
    rc = lib.mrsph_create(ctypes.byref(p), ctypes.byref(h))
    assert rc == -1
    buf = ctypes.create_string_buffer(256)
    lib.mrsph_last_error(None, buf, 256)
    assert b"dim" in buf.value


def test_level_plan_rejects_bad_domain():
    lib = L.load()
    p = L.Params()
    p.dim = 2
    p.kernel = 2
    p.precision = 0
    p.cell_ratio = 2.6
    p.cutoff = 2.0
    p.min_dl = p.max_dl = 0.5
    p.box_l[0] = p.box_l[1] = 0.0
    p.box_r[0] = p.box_r[1] = 1.0
    h = ctypes.c_void_p()
    rc = lib.mrsph_create(ctypes.byref(p), ctypes.byref(h))
    assert rc == -1  # coarsest cell (1.3) larger than the domain


def test_null_arguments_rejected_without_gpu():
    """Entry points check their handle and output pointers before any device
    call (mrsph_volume_mass, the stats and step entry points)."""
    lib = L.load()
    st = L.VolumeMassStats()
    assert lib.mrsph_volume_mass(None, -1, ctypes.byref(st), None, None) == -1
    assert lib.mrsph_step(None, 1) < 0
    assert lib.mrsph_get_stats(None, None) < 0
