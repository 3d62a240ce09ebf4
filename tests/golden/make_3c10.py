"""Generate tests/golden/3c10.npz from the reference's shipped golden FITS files.

Inputs (timcornwell/sde reqdata/): 3C10UV.FTS (VLA random-groups uv data, 8832 groups x
4 Stokes RR,LL,RL,LR), 3C10MAP.FTS and 3C10BEAM.FTS (the 128^2 dirty image and PSF that
uvmap made from it: 12" cells, SF kernel, FOV=1 uniform weighting, per their HISTORY cards).

The uv data are reduced exactly the way SDE's VISGET/VISSTD do before imaging:
  * group parameters UU, VV, WW (seconds) -> wavelengths by ARRSCALE(x, SNGL(FREQ), 0.0)
    with FREQ = CRVAL + (1 - CRPIX) * CDELT of the FREQ axis (vis/visstd.f:123-148);
  * Stokes I = 0.5 (RR + LL) with weight (WRR + WLL)/2, or weight -1 when either is
    non-positive (vis/visconvs.f:43-61).
Usage: python tests/golden/make_3c10.py [path/to/reqdata]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_header(raw):
    cards, i = [], 0
    while True:
        card = raw[i:i + 80].decode("ascii", "replace")
        i += 80
        cards.append(card)
        if card.startswith("END"):
            break
    hdr = {}
    for c in cards:
        if "=" in c[:10]:
            key = c[:8].strip()
            val = c[10:].split("/")[0].strip()
            if val.startswith("'"):
                val = val.strip("'").strip()
            else:
                try:
                    val = float(val) if any(ch in val for ch in ".E") else int(val)
                except ValueError:
                    pass
            hdr[key] = val
    data_start = ((i + 2879) // 2880) * 2880
    return hdr, data_start


def read_image(path):
    raw = open(path, "rb").read()
    h, off = read_header(raw)
    nx, ny = h["NAXIS1"], h["NAXIS2"]
    assert h["BITPIX"] == -32
    img = np.frombuffer(raw, ">f4", count=nx * ny, offset=off).astype(np.float32)
    return img.reshape(ny, nx), h


def read_uv(path):
    raw = open(path, "rb").read()
    h, off = read_header(raw)
    assert h["GROUPS"] and h["BITPIX"] == 32
    ng, npar = h["GCOUNT"], h["PCOUNT"]
    ncplx, nstk = h["NAXIS2"], h["NAXIS3"]
    nd = ncplx * nstk * h["NAXIS4"] * h["NAXIS5"] * h["NAXIS6"]
    rec = np.frombuffer(raw, ">i4", count=ng * (npar + nd), offset=off).reshape(ng, npar + nd)
    par = rec[:, :npar].astype(np.float64)
    scal = [h.get("PSCAL%d" % (k + 1), 1.0) for k in range(npar)]
    zero = [h.get("PZERO%d" % (k + 1), 0.0) for k in range(npar)]
    par = par * np.array(scal) + np.array(zero)
    data = (rec[:, npar:].astype(np.float64) * h["BSCALE"] + h["BZERO"]).astype(np.float32)
    data = data.reshape(ng, nstk, ncplx)  # axis2 (complex) fastest, then stokes
    freq = h["CRVAL4"] + (1.0 - h["CRPIX4"]) * h["CDELT4"]
    f32 = np.float32(freq)
    uvw = [(np.float32(f32) * par[:, k].astype(np.float32) + np.float32(0.0)).astype(np.float32)
           for k in range(3)]
    rr = data[:, 0, 0] + 1j * data[:, 0, 1]
    ll = data[:, 1, 0] + 1j * data[:, 1, 1]
    wrr = np.maximum(data[:, 0, 2], np.float32(0))
    wll = np.maximum(data[:, 1, 2], np.float32(0))
    good = (wrr > 0) & (wll > 0)
    si = np.where(good, np.float32(0.5) * (rr.astype(np.complex64) + ll.astype(np.complex64)), 0)
    wiv = np.where(good, (wrr + wll) / np.float32(2.0), np.float32(-1.0)).astype(np.float32)
    return dict(u=uvw[0], v=uvw[1], w=uvw[2], vis=si.astype(np.complex64), wt=wiv,
                ra=np.float64(h["CRVAL5"]), dec=np.float64(h["CRVAL6"]), freq=np.float64(freq))



def reference_root():
    """The reference tree: $SDE_REFERENCE, else /root/reference (None if that is not an
    existing directory)."""
    root = os.environ.get("SDE_REFERENCE") or "/root/reference"
    return root if os.path.isdir(root) else None

def main(reqdata):
    uv = read_uv(os.path.join(reqdata, "3C10UV.FTS"))
    dmap, hm = read_image(os.path.join(reqdata, "3C10MAP.FTS"))
    beam, _ = read_image(os.path.join(reqdata, "3C10BEAM.FTS"))
    out = os.path.join(HERE, "3c10.npz")
    np.savez_compressed(out, map=dmap, beam=beam, cellsize=np.float32(12.0), imsize=128, **uv)
    print("wrote", out, "nvis", len(uv["wt"]), "map max %.4f min %.4f rms %.4f" % (
        dmap.max(), dmap.min(), np.sqrt((dmap.astype(np.float64) ** 2).mean())))


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main(sys.argv[1])
    else:
        root = reference_root()
        if root is None:
            sys.exit("no reference tree: pass path/to/reqdata or set SDE_REFERENCE")
        main(os.path.join(root, "reqdata"))
