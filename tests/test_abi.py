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


def _oracle_cf(orc, code_sf):
    cf = np.zeros(1 + 8 * 129, np.float32)
    s, o = C.c_int(), C.c_int()
    orc.lib().orc_grdcf(code_sf, cf, C.byref(s), C.byref(o))
    return cf, s.value, o.value


def test_library_gridding_tables_equal_the_oracle(orc):
    """The library's host-side GRDCF ('SF' and 'BOX'), GRDCCF ('SF' and 'BOX') and GRDSF
    (grd/grdcf.f:41-90, grd/grdccf.f:42-52, grd/grdsf.f:46-73) -- the tables a caller of the
    drop-ins builds -- equal the oracle's restatement bit for bit; an unknown code reports
    through ERRREPOR and leaves ERROR set."""
    L = _abi.lib()
    P = C.c_void_p
    for code, code_sf, supp_ref in ((b"SF", 1, 3), (b"BOX", 0, 1)):
        ref, rs, ro = _oracle_cf(orc, code_sf)
        cf = np.full(1 + 8 * 129, np.nan, np.float32)
        cfs, cfo = C.c_int(-1), C.c_int(-1)
        # only the table's used span is written: (SUPP+1)*OSAMP on each side of the centre
        L.grdcf_(code, cf.ctypes.data_as(P), C.byref(cfs), C.byref(cfo), len(code))
        assert (cfs.value, cfo.value) == (rs, ro) == (supp_ref, 128)
        n = 2 * (supp_ref + 1) * 128 + 1
        assert np.array_equal(cf[:n].view(np.uint32), ref[:n].view(np.uint32)), code
    for ccflen in (33, 257, 2049, 4097):
        for code, code_sf in ((b"SF", 1), (b"BOX", 0)):
            ref = np.zeros(ccflen, np.float32)
            orc.lib().orc_grdccf(code_sf, ref, ccflen)
            got = np.zeros(ccflen, np.float32)
            L.grdccf_(code, got.ctypes.data_as(P), C.byref(C.c_int(ccflen)), len(code))
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (code, ccflen)
    for nu in np.linspace(-0.1, 1.1, 1201):
        x = C.c_double(float(nu))
        assert L.grdsf_(C.byref(x)) == orc.lib().orc_grdsf(float(nu))
    s = _abi.sysi()
    try:
        cf = np.zeros(1 + 8 * 129, np.float32)
        L.grdcf_(b"XYZ", cf.ctypes.data_as(P), C.byref(C.c_int()), C.byref(C.c_int()), 3)
        assert s.error != 0
    finally:
        s.error = 0
