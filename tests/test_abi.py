"""CPU tests of the C ABI boundary and the host logic (no GPU calls)."""
import ctypes as C
import os
import re

import numpy as np

from sde_gb300 import _abi
from sde_gb300.imaging import Geom, crdshift, fftpwr2

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "sde_gpu.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", txt)
    skip = {"if", "sizeof", "defined"}
    return sorted({n for n in names if n not in skip and not n.startswith("__")})


def test_library_loads_and_exports_every_declared_symbol():
    L = _abi.lib()
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(L, n), "missing export " + n
    for n in _abi.DATA_SYMBOLS:
        assert C.c_int.in_dll(L, n) is not None
    declared = {s[0] for s in _abi.SIGNATURES}
    assert set(names) <= declared, set(names) - declared


def test_error_common_block_is_exported_and_clean():
    s = _abi.sysi()
    assert s.error == 0


def test_fortran_error_flag_short_circuits_without_gpu():
    # With ERROR set every drop-in entry point returns at once (the reference's
    # IF (ERROR) GO TO 999 convention), so this runs on a machine without a GPU.
    L = _abi.lib()
    s = _abi.sysi()
    s.error = 1
    try:
        n = C.c_int(4)
        a = (C.c_float * 4)(1, -5, 3, 5)
        i = C.c_int(7)
        assert L.pixisama_(C.byref(n), a, C.byref(i)) == 7
    finally:
        s.error = 0


def test_geometry_matches_oracle(orc):
    for n, cell, dec, sh in [(512, 1.0, 40.0, (0, 0)), (4096, 0.5, 40.0, (0, 0)),
                             (128, 12.0, 63.8666666, (0, 0)), (100, 3.0, 55.0, (30.0, -20.0))]:
        p = orc.params(n, cell, vdec=dec, shift=sh)
        g = orc.geom(p)
        h = Geom(n, cell, vdec=dec, shift=sh)
        assert (h.nu, h.nv, h.fnu) == (g.nu, g.nv, g.fnu)
        assert np.float32(h.uscale) == np.float32(g.uscale)
        assert np.float32(h.vscale) == np.float32(g.vscale)
        assert (h.uorigin, h.vorigin) == (g.uorigin, g.vorigin)
        assert np.array_equal(h.shift, np.array(list(g.shift)))


def test_crdshift_matches_oracle(orc):
    for args in [(10.0, 40.0, 10.0, 40.0), (5.6, 63.9, 5.61, 63.88), (200.0, -30.0, 200.2, -29.5)]:
        assert np.array_equal(crdshift(*args), orc.crdshift(*args))


def test_fftpwr2():
    assert [fftpwr2(i) for i in (1, 2, 3, 5, 6, 12, 100, 4096, 4097)] == \
        [1, 2, 4, 8, 8, 16, 128, 4096, 8192]


def test_window_is_crdnhalf():
    g = Geom(512, 1.0)
    lo, hi = g.window()
    assert (lo, hi - lo) == (128, 255)
    g = Geom(4096, 0.5)
    lo, hi = g.window()
    assert (lo, hi - lo) == (1024, 2047)
