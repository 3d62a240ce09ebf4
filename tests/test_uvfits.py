"""Visibility loading from FITS random-groups files (VISGET's FTS branch: fts/ftsgrpre.f,
fts/fti.c, vis/visstd.f, vis/visconvs.f, visconv2.f, visconvp.f).

CPU: the oracle restatement (oracle/uvfits.py) pinned on the reference's own reqdata/3C10UV.FTS
(when the reference tree is present) and on its committed 300-group head
(tests/golden/3c10uv_head.fts) against tests/golden/3c10.npz; the header checks of
sde_uvfits_open (host code, no CUDA call) against the reference's messages.
GPU: sde_uvfits_read bit for bit against the oracle over every data form the reference reads
(16/32-bit integers and IEEE words, AIPS and pipeline layouts, 4/2/1 Stokes, RR/LL/RL/LR and
IQUV, every Stokes parameter), host and device outputs, a file shorter than GCOUNT, a file of
many chunks; and uvmap of 3C10 on the GPU against the reference's golden map."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import uvfits as OU

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "3c10.npz")
HEAD = os.path.join(HERE, "golden", "3c10uv_head.fts")


def _reference_uv():
    """reqdata/3C10UV.FTS of the reference tree named by $SDE_REFERENCE, else /root/reference
    (a path that does not exist skips the test that reads it)."""
    root = os.environ.get("SDE_REFERENCE") or "/root/reference"
    return os.path.join(root, "reqdata", "3C10UV.FTS")


REF_UV = _reference_uv()
KEYS = ("u", "v", "w", "vis", "wt")


# ---------------------------------------------------------------------------------------
# A writer of random-groups files with chosen words (the decoding is defined on the words).
def _card(key, val=None, comment=""):
    if val is None:
        s = key.ljust(80)
    elif isinstance(val, bool):
        s = "%-8s= %20s /%s" % (key, "T" if val else "F", comment)
    elif isinstance(val, str):
        s = "%-8s= '%-8s' /%s" % (key, val, comment)
    elif isinstance(val, int):
        s = "%-8s= %20d /%s" % (key, val, comment)
    else:
        s = "%-8s= %20.12E /%s" % (key, val, comment)
    return s[:80].ljust(80).encode()


def write_groups(path, *, ngroups, bitpix=32, ptypes=("UU", "VV", "WW", "BASELINE", "DATE"),
                 pscal=None, pzero=None, ncomplex=3, nstokes=4, stokes_crval=-1.0,
                 freq=(1.4e9, 1.0e6, 1.0), bscale=1.0, bzero=0.0, axes=None, seed=0,
                 groups=True, first_axis="COMPLEX", truncate_to=None, extra_cards=()):
    rng = np.random.default_rng(seed)
    npar = len(ptypes)
    pscal = pscal or [1.0] * npar
    pzero = pzero or [0.0] * npar
    axes = axes or [(first_axis, ncomplex, 1.0, 1.0, 1.0), ("STOKES", nstokes, stokes_crval, -1.0, 1.0),
                    ("FREQ", 1, freq[0], freq[1], freq[2]), ("RA", 1, 12.5, 1.0, 1.0),
                    ("DEC", 1, 45.25, 1.0, 1.0)]
    cards = [_card("SIMPLE", True), _card("BITPIX", bitpix), _card("NAXIS", len(axes) + 1),
             _card("NAXIS1", 0)]
    cards += [_card("NAXIS%d" % (k + 2), a[1]) for k, a in enumerate(axes)]
    cards += [_card("BSCALE", bscale), _card("BZERO", bzero)]
    for k, (ct, n, crval, cdelt, crpix) in enumerate(axes):
        cards += [_card("CTYPE%d" % (k + 2), ct), _card("CRVAL%d" % (k + 2), crval),
                  _card("CDELT%d" % (k + 2), cdelt), _card("CRPIX%d" % (k + 2), crpix)]
    cards += [_card("GROUPS", groups), _card("GCOUNT", ngroups), _card("PCOUNT", npar)]
    for k, nm in enumerate(ptypes):
        cards += [_card("PTYPE%d" % (k + 1), nm), _card("PSCAL%d" % (k + 1), pscal[k]),
                  _card("PZERO%d" % (k + 1), pzero[k])]
    cards += [_card(*c) for c in extra_cards]
    cards.append(_card("END"))
    head = b"".join(cards)
    head += b" " * ((-len(head)) % 2880)
    nreg = int(np.prod([a[1] for a in axes]))
    lgrp = npar + nreg
    if bitpix == 16:
        words = rng.integers(-32768, 32768, size=(ngroups, lgrp)).astype(">i2")
    elif bitpix == 32:
        words = rng.integers(-2 ** 31, 2 ** 31, size=(ngroups, lgrp), dtype=np.int64).astype(">i4")
    else:
        words = rng.standard_normal((ngroups, lgrp)).astype(">f4")
        words[::7, npar:] = np.float32(-0.0)
    if bitpix != -32 and ncomplex == 3:
        # weights: mostly positive, some zero or negative (flagged)
        for s in range(nreg // 3):
            col = npar + 3 * s + 2
            wv = np.abs(words[:, col].astype(np.int64)) // 2 + 1
            wv[::5] = 0
            wv[::11] = -wv[::11]
            words[:, col] = wv.astype(words.dtype)
    if "WEIGHT" in ptypes and bitpix != -32:
        col = list(ptypes).index("WEIGHT")
        wv = np.abs(words[:, col].astype(np.int64)) // 2 + 1
        wv[::4] = -wv[::4]
        words[:, col] = wv.astype(words.dtype)
    data = words.tobytes()
    data += b"\0" * ((-len(data)) % 2880)
    blob = head + data
    if truncate_to is not None:
        blob = blob[:len(head) + truncate_to]
    open(path, "wb").write(blob)
    return path


# ---------------------------------------------------------------------------------------
# CPU
@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _same(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b))


@pytest.mark.skipif(not os.path.exists(REF_UV), reason="reference tree not present")
def test_oracle_reads_reference_3c10_file(gold):
    r = OU.read(REF_UV, "I")
    assert r["nread"] == 8832
    for k in KEYS:
        assert _same(r[k], gold[k]), k
    assert r["desc"]["freq"] == float(gold["freq"])


def test_oracle_head_fixture_matches_golden(gold):
    r = OU.read(HEAD, "I")
    assert r["nread"] == 300
    for k in KEYS:
        assert _same(r[k], gold[k][:300]), k


def test_oracle_stokes_conversions(tmp_path):
    """VISCONVS, VISCONV2 and VISCONVP by their formulas on decoded words."""
    p = write_groups(str(tmp_path / "a.fts"), ngroups=64, bitpix=-32, seed=3)
    raw = open(p, "rb").read()
    d = OU.describe(raw)
    rec = np.frombuffer(raw, ">f4", count=64 * (5 + 12), offset=d["off"]).reshape(64, 17)
    a = rec[:, 5:].astype(np.float32)
    rr, ll = a[:, 0] + 1j * a[:, 1], a[:, 3] + 1j * a[:, 4]
    rl, lr = a[:, 6] + 1j * a[:, 7], a[:, 9] + 1j * a[:, 10]
    good_iv = (a[:, 2] > 0) & (a[:, 5] > 0)
    good_qu = (a[:, 8] > 0) & (a[:, 11] > 0)
    exp = {"I": 0.5 * (rr + ll), "V": 0.5 * (rr - ll), "Q": 0.5 * (rl + lr), "U": -0.5j * (rl - lr)}
    for s, good in (("I", good_iv), ("V", good_iv), ("Q", good_qu), ("U", good_qu)):
        r = OU.read(p, s)
        assert np.allclose(r["vis"][good], exp[s][good], rtol=1e-6, atol=0)
        assert np.all(r["vis"][~good] == 0) and np.all(r["wt"][~good] == -1.0)
    pipe = write_groups(str(tmp_path / "p.fts"), ngroups=40, bitpix=32, ncomplex=2,
                        ptypes=("UU", "VV", "WW", "WEIGHT"), seed=4)
    r = OU.read(pipe, "I")
    wp = r["desc"]["par"]["WEIGHT"]
    raw = open(pipe, "rb").read()
    rec = np.frombuffer(raw, ">i4", count=40 * 12, offset=OU.describe(raw)["off"]).reshape(40, 12)
    assert _same(r["wt"], rec[:, wp].astype(np.float32))  # the WEIGHT parameter as read
    assert np.all(r["vis"][rec[:, wp] <= 0] == 0)


def _lib():
    from sde_gb300 import _abi
    return _abi.lib(), _abi


def test_open_describes_3c10_head_without_gpu(gold):
    L, A = _lib()
    h = C.c_void_p()
    assert L.sde_uvfits_open(HEAD.encode(), C.byref(h)) == 0
    d = A.UvfitsDesc()
    assert L.sde_uvfits_describe(h, C.byref(d)) == 0
    L.sde_uvfits_close(h)
    assert (d.ngroups, d.ngroups_in_file, d.npar, d.bitpix, d.ncomplex, d.nstokes) == (300, 300, 6, 32, 3, 4)
    assert (d.iquv, d.uvw_scaled) == (0, 1)
    assert d.freq == float(gold["freq"]) and d.ra == float(gold["ra"]) and d.dec == float(gold["dec"])


@pytest.mark.parametrize("kw,msg", [
    (dict(groups=False), "Not a groups file"),
    (dict(ngroups=0), "No groups!"),
    (dict(bitpix=-64), "Cannot read -64-bit files"),
    (dict(first_axis="STOKES"), "First axis not COMPLEX"),
    (dict(axes=[("COMPLEX", 3, 1.0, 1.0, 1.0), ("FREQ", 1, 1.4e9, 1e6, 1.0)]), "No stokes axes"),
    (dict(axes=[("COMPLEX", 3, 1.0, 1.0, 1.0), ("STOKES", 4, -1.0, -1.0, 1.0)]), "No frequency"),
    (dict(ptypes=("VV", "WW", "DATE")), "PTYPE=UU not in header"),
    (dict(ncomplex=4), "Unable to read such data"),
    (dict(axes=[("COMPLEX", 3, 1.0, 1.0, 1.0), ("STOKES", 4, -1.0, -1.0, 1.0),
                ("FREQ", 2, 1.4e9, 1e6, 1.0)]), "more than one frequency channel"),
])
def test_open_rejects_what_the_reference_rejects(tmp_path, kw, msg):
    L, A = _lib()
    args = dict(ngroups=kw.pop("ngroups", 8))
    p = write_groups(str(tmp_path / "bad.fts"), **args, **kw)
    with pytest.raises(OU.UvfitsError, match=msg):
        OU.read(p, "I")
    h = C.c_void_p()
    assert L.sde_uvfits_open(p.encode(), C.byref(h)) != 0
    assert msg in A.last_error()


# ---------------------------------------------------------------------------------------
# GPU
FORMS = {
    "aips4_i32": dict(bitpix=32, pscal=[2.7e-15, 2.8e-15, 1.9e-15, 1.0, 0.25],
                      pzero=[0.0, 0.0, 0.0, 0.0, 2445538.5], bscale=3.06e-8),
    "aips4_i16": dict(bitpix=16, pscal=[1e-9, 2e-9, 3e-9, 1.0, 1.0], bscale=1e-3, bzero=0.5),
    "aips4_ieee": dict(bitpix=-32),
    "aips4_ieee_scaled": dict(bitpix=-32, bscale=2.0, bzero=-0.25, pscal=[3.0, 3.0, 3.0, 1.0, 1.0]),
    "aips2_i32": dict(bitpix=32, nstokes=2, bscale=1e-6),
    "pipe4_i32": dict(bitpix=32, ncomplex=2, ptypes=("UU", "VV", "WW", "WEIGHT"), bscale=1e-6),
    "iquv_i32": dict(bitpix=32, stokes_crval=1.0, bscale=1e-6),
    "one_stokes": dict(bitpix=32, nstokes=1, bscale=1e-6),
    "uvw_wavelengths": dict(bitpix=32, ptypes=("UU-L", "VV-L", "WW-L", "DATE"), bscale=1e-6),
    "uvw_sin": dict(bitpix=32, ptypes=("UU---SIN", "VV---SIN", "WW---SIN"), bscale=1e-6,
                    freq=(1.4e9, 2.5e7, 0.5)),
}


def _read_gpu(ctx, path, stokes, device):
    from sde_gb300.uvfits import UVFits
    with UVFits(path) as f:
        out = f.read(ctx, stokes, device=device)
    ctx.sync()
    if device:
        out = {k: (v.cpu().numpy() if hasattr(v, "cpu") else v) for k, v in out.items()}
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("form", sorted(FORMS))
def test_gpu_loader_matches_oracle(gpu_ctx, tmp_path, form):
    kw = FORMS[form]
    p = write_groups(str(tmp_path / (form + ".fts")), ngroups=1000, seed=sum(map(ord, form)), **kw)
    ns = kw.get("nstokes", 4)
    for i, s in enumerate("IVQU"[:ns]):
        ref = OU.read(p, s)
        got = _read_gpu(gpu_ctx, p, s, device=(i % 2 == 0))
        assert got["nread"] == ref["nread"] == 1000
        for k in KEYS:
            assert _same(got[k], ref[k]), (form, s, k)


@pytest.mark.gpu
def test_gpu_loader_3c10_head(gpu_ctx, gold):
    for device in (True, False):
        got = _read_gpu(gpu_ctx, HEAD, "I", device)
        assert got["nread"] == 300
        for k in KEYS:
            assert _same(got[k], gold[k][:300]), k


@pytest.mark.gpu
def test_gpu_loader_short_file(gpu_ctx, tmp_path):
    lgrp_bytes = (5 + 12) * 4
    p = write_groups(str(tmp_path / "short.fts"), ngroups=500, seed=9, bscale=1e-6,
                     truncate_to=321 * lgrp_bytes + 17)
    ref = OU.read(p, "I")
    got = _read_gpu(gpu_ctx, p, "I", True)
    assert got["nread"] == ref["nread"] == 321
    for k in KEYS:
        assert _same(got[k], ref[k]), k


@pytest.mark.gpu
def test_gpu_loader_many_chunks(gpu_ctx, tmp_path):
    """1.2 M groups of 72 bytes: three 32 MB chunks through both pinned buffers."""
    p = write_groups(str(tmp_path / "big.fts"), ngroups=1_200_000, seed=11, bscale=3e-8,
                     pscal=[2.7e-15, 2.8e-15, 1.9e-15, 1.0, 0.25])
    ref = OU.read(p, "Q")
    got = _read_gpu(gpu_ctx, p, "Q", True)
    assert got["nread"] == 1_200_000
    for k in KEYS:
        assert _same(got[k], ref[k]), k


@pytest.mark.gpu
def test_gpu_uvmap_3c10_matches_golden_map(gpu_ctx, orc, gold):
    """The reference's 3C10 data through the GPU uvmap (uniform weighting, FOV 1, 128^2 at
    12"): the golden map's statistics (test/timer:32-34) and the oracle's image within the
    parity bar."""
    from sde_gb300.imaging import Geom, uvmap
    ctx = gpu_ctx
    d = gold
    g = Geom(128, 12.0, vra=float(d["ra"]), vdec=float(d["dec"]), fov=1.0)
    t = {k: ctx.tensor(d[k]) for k in KEYS}
    res = uvmap(ctx, g, t["u"], t["v"], t["w"], t["vis"], t["wt"], rmode="UNIFORM")
    ctx.sync()
    dirty = res["dirty"].cpu().numpy()
    p = orc.params(128, 12.0, fov=1.0, rmode="NONE", vra=float(d["ra"]), vdec=float(d["dec"]))
    rd, rp, rwt, rmax, rsw, rc = orc.uvmap(p, d["u"], d["v"], d["w"], d["vis"], d["wt"])
    assert rc == 0
    assert np.array_equal(t["wt"].cpu().numpy(), rwt)
    # the image bars of the uvmap parity tests: 1e-5 of the peak inside CRDNHALF's window,
    # 5e-3 over the image (the grid correction amplifies FP32 rounding towards the corners)
    w = slice(32, 95)
    pk = np.abs(rd).max()
    assert np.abs(dirty - rd)[w, w].max() / pk < 1e-5
    assert np.abs(dirty - rd).max() / pk < 5e-3
    rms = float(np.sqrt((dirty.astype(np.float64) ** 2).mean()))
    assert abs(rms - 0.1402) < 2e-4
    assert abs(float(dirty.max()) - 0.6791) < 1e-4
    assert np.abs(dirty - d["map"])[w, w].max() < 2e-3
    res["plan"].close()
