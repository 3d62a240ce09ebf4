"""CPU restatement of SDE's visibility load from a FITS random-groups file (the FTS branch of
VISGET, vis/visget.f:60-68: FILGRPGE -> FTSGRPRE, then VISSTD), in numpy.

TEST INFRASTRUCTURE: only tests/ import this module.  The product (sde_gb300, libsdegpu's
sde_uvfits_*) never imports or calls it.

Steps and the reference lines they follow:
  * header cards, GROUPS/GCOUNT/PCOUNT/BITPIX checks        fts/ftsgrpre.f:62-90, 191-200
  * words -> REAL: big-endian 16/32-bit integers or IEEE,
    value = SCALE * word + ZERO in DOUBLE, stored REAL;
    IEEE with the identity scaling copied as is              fts/fti.c:69-168
    (random parameters with PSCALn/PZEROn,
     the regular array with BSCALE/BZERO)                    fts/ftsgrpre.f:229-243
  * COMPLEX first axis, STOKES axis, ISIQUV = CRVAL > 0      vis/visstd.f:102-118
  * FREQ = CRVAL + (1.0 - CRPIX) * CDELT (CRPIX, CDELT REAL) vis/visstd.f:122-131
  * UU/VV/WW (seconds) -> ARRSCALE(x, SNGL(FREQ), 0.0);
    UU-L/UU-L-SIN taken as wavelengths                       vis/visstd.f:135-202,
                                                            pix/pixrscal.f
  * RR,LL,RL,LR -> I,V,Q,U                                   vis/visconvs.f:43-82 (4 Stokes),
                                                            vis/visconv2.f:40-60 (2),
                                                            vis/visconvp.f:44-80 (pipeline)
  * one Stokes plane's VIS and WT (by position I,V,Q,U)      vis/visstd.f:260-314
  * a short file: the groups read so far                     fts/ftsgrpre.f:254-258

Deliberate differences, mirrored by the GPU loader: GCOUNT is read as an integer (the
reference rounds it through REAL, exact only below 2^24 groups); groups holding more than one
COMPLEX x STOKES block are refused (the reference's conversions would misread them); a Stokes
position beyond the file's planes is refused (the reference reads past the group).
"""
import numpy as np

STOKES_ORDER = "IVQU"  # vis/visstd.f:51 STKTYPE


class UvfitsError(ValueError):
    pass


def parse_header(raw):
    """Cards up to END -> (dict keyword -> value, byte offset of the data)."""
    hdr, i = {}, 0
    while True:
        if i + 80 > len(raw):
            raise UvfitsError("no END card")
        card = raw[i:i + 80].decode("ascii", "replace")
        i += 80
        key = card[:8].strip()
        if key == "END":
            break
        if card[8:10] != "= " or not key or key in hdr:
            continue
        v = card[10:]
        s = v.lstrip()
        if s.startswith("'"):
            out, k = [], 1
            while k < len(s):
                if s[k] == "'":
                    if k + 1 < len(s) and s[k + 1] == "'":
                        out.append("'")
                        k += 2
                        continue
                    break
                out.append(s[k])
                k += 1
            hdr[key] = "".join(out).rstrip(" ")
        else:
            tok = s.split("/")[0].strip()
            if tok in ("T", "F"):
                hdr[key] = tok == "T"
            else:
                try:
                    hdr[key] = float(tok.replace("D", "E").replace("d", "E"))
                except ValueError:
                    hdr[key] = tok
    return hdr, (i + 2879) // 2880 * 2880


def _num(h, k, dflt=None):
    x = h.get(k, dflt)
    return x if isinstance(x, float) and not isinstance(x, bool) else dflt


def describe(raw):
    """The header checks of FTSGRPRE and VISSTD; returns the decoding parameters."""
    h, off = parse_header(raw)
    if h.get("GROUPS") is not True:
        raise UvfitsError("Not a groups file")
    gc = _num(h, "GCOUNT", 0.0)
    if gc < 1:
        raise UvfitsError("No groups!")
    npar = int(_num(h, "PCOUNT", 0.0))
    bitpix = int(_num(h, "BITPIX", 0.0))
    if bitpix not in (16, 32, -32):
        raise UvfitsError("Cannot read %d-bit files" % bitpix)
    nax = int(_num(h, "NAXIS", 0.0))
    nreg, nstokes, iquv, freq, ncomplex = 1, None, False, None, None
    for k in range(2, nax + 1):
        n = int(_num(h, "NAXIS%d" % k, 0.0))
        nreg *= n
        ct = h.get("CTYPE%d" % k, "")
        if k == 2:
            if ct != "COMPLEX":
                raise UvfitsError("First axis not COMPLEX")
            ncomplex = n
        if ct == "STOKES" and nstokes is None:
            nstokes = n
            iquv = _num(h, "CRVAL%d" % k, 0.0) > 0.0
        if ct == "FREQ":
            rpix = np.float32(_num(h, "CRPIX%d" % k, 0.0))
            delt = np.float32(_num(h, "CDELT%d" % k, 0.0))
            freq = _num(h, "CRVAL%d" % k, 0.0) + float((np.float32(1.0) - rpix) * delt)
    if nstokes is None:
        raise UvfitsError("No stokes axes")
    if not freq:
        raise UvfitsError("No frequency")
    names = [h.get("PTYPE%d" % (k + 1), "") for k in range(npar)]
    pscal = [_num(h, "PSCAL%d" % (k + 1), 1.0) for k in range(npar)]
    pzero = [_num(h, "PZERO%d" % (k + 1), 0.0) for k in range(npar)]
    par, kinds = {}, []
    for ax in ("UU", "VV", "WW"):
        idx, kind = None, None
        for sfx, sc in (("", 1), ("--", 1), ("---SIN", 1), ("  -SIN", 1), ("-L-SIN", 0), ("-L", 0)):
            if ax + sfx in names:
                idx, kind = names.index(ax + sfx), sc
                break
        if idx is None:
            raise UvfitsError("PTYPE=%s not in header" % ax)
        par[ax] = idx
        kinds.append(kind)
    if len(set(kinds)) != 1:
        raise UvfitsError("UU, VV and WW in different units")
    if ncomplex not in (2, 3):
        raise UvfitsError("Unable to read such data")
    if ncomplex == 2:
        if "WEIGHT" not in names:
            raise UvfitsError("pipeline-form data without a WEIGHT parameter")
        par["WEIGHT"] = names.index("WEIGHT")
    if nreg != ncomplex * nstokes:
        raise UvfitsError("more than one frequency channel, IF or position per group")
    return dict(off=off, ngroups=int(gc), npar=npar, bitpix=bitpix, nreg=nreg, ncomplex=ncomplex,
                nstokes=nstokes, iquv=iquv, freq=freq, uvw_scaled=kinds[0], par=par,
                pscal=pscal, pzero=pzero, bscale=_num(h, "BSCALE", 1.0),
                bzero=_num(h, "BZERO", 0.0))


def _to_real(words, bitpix, scale, zero):
    """fticr_: SCALE * word + ZERO in double, stored REAL; IEEE words with the identity
    scaling copied (signed zeros kept)."""
    if bitpix == -32:
        f = words.astype(np.float32)
        if scale == 1.0 and zero == 0.0:
            return f
        return (f.astype(np.float64) * scale + zero).astype(np.float32)
    return (words.astype(np.float64) * scale + zero).astype(np.float32)


def _half(a):
    return (np.float32(0.5) * a.real.astype(np.float32)
            + 1j * (np.float32(0.5) * a.imag.astype(np.float32))).astype(np.complex64)


def _mjhalf(d):
    """-0.5 * J * d: the complex product (-0.0, -0.5) * d in REAL arithmetic."""
    a, b = np.float32(-0.0), np.float32(-0.5)
    dr, di = d.real.astype(np.float32), d.imag.astype(np.float32)
    re = (a * dr) - (b * di)
    im = (a * di) + (b * dr)
    return (re + 1j * im).astype(np.complex64)


def read(path, stokes="I"):
    """dict(u, v, w, vis, wt, nread, desc) as VISGET leaves them for one Stokes parameter."""
    raw = open(path, "rb").read()
    d = describe(raw)
    if stokes not in STOKES_ORDER:
        raise UvfitsError("Stokes must be one of I, V, Q, U")
    pos = STOKES_ORDER.index(stokes)
    if pos >= d["nstokes"]:
        raise UvfitsError("Stokes %s not in the file" % stokes)
    ws = 2 if d["bitpix"] == 16 else 4
    lgrp = d["npar"] + d["nreg"]
    avail = max(0, (len(raw) - d["off"]) // (lgrp * ws))
    n = min(d["ngroups"], avail)
    dt = {16: ">i2", 32: ">i4", -32: ">f4"}[d["bitpix"]]
    rec = np.frombuffer(raw, dt, count=n * lgrp, offset=d["off"]).reshape(n, lgrp)

    def par(name):
        k = d["par"][name]
        return _to_real(rec[:, k], d["bitpix"], d["pscal"][k], d["pzero"][k])

    arr = _to_real(rec[:, d["npar"]:], d["bitpix"], d["bscale"], d["bzero"])
    uvw = []
    for ax in ("UU", "VV", "WW"):
        x = par(ax)
        if d["uvw_scaled"]:
            x = (np.float32(d["freq"]) * x + np.float32(0.0)).astype(np.float32)
        uvw.append(x)
    inc, ns = d["ncomplex"], d["nstokes"]
    cplx = lambda k: (arr[:, k] + 1j * arr[:, k + 1]).astype(np.complex64)  # noqa: E731
    zero = np.zeros(n, np.complex64)
    if inc == 3 and ns in (4, 2) and not d["iquv"]:
        b = 0 if pos < 2 else 6
        s1, s2 = cplx(b), cplx(b + 3)
        w1, w2 = np.maximum(arr[:, b + 2], np.float32(0)), np.maximum(arr[:, b + 5], np.float32(0))
        good = (w1 > 0) & (w2 > 0)
        out = [_half(s1 + s2), _half(s1 - s2), _half(s1 + s2), _mjhalf(s1 - s2)][pos]
        vis = np.where(good, out, zero)
        wt = np.where(good, (w1 + w2) / np.float32(2.0), np.float32(-1.0)).astype(np.float32)
    elif inc == 2 and ns == 4:
        wp = par("WEIGHT")
        b = 0 if pos < 2 else 4
        s1, s2 = cplx(b), cplx(b + 2)
        good = np.maximum(wp, np.float32(0)) > 0
        out = [_half(s1 + s2), _half(s1 - s2), _half(s1 + s2), _mjhalf(s1 - s2)][pos]
        vis = np.where(good, out, zero)
        wt = wp
    else:
        b = inc * pos
        vis = cplx(b)
        wt = arr[:, b + 2] if inc == 3 else par("WEIGHT")
    return dict(u=uvw[0], v=uvw[1], w=uvw[2], vis=vis.astype(np.complex64),
                wt=np.asarray(wt, np.float32), nread=n, desc=d)
