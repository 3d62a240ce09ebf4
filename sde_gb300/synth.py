"""Seeded synthetic interferometer observations for the imaging benchmarks and tests.

The reference's own simulator (sim/simuv.f, SIMUV) generates Earth-rotation uv tracks from
antenna positions; this module follows the same physics with numpy:
  * antennas at seeded random distances along the three arms of a Y (azimuths 0, 120,
    240 deg, VLA-like latitude 34.08 deg);
  * baseline vectors rotated to equatorial (X, Y, Z) and projected to (u, v, w) for each
    hour angle H and declination dec:  u = sinH X + cosH Y,
    v = -sin(dec) cosH X + sin(dec) sinH Y + cos(dec) Z,
    w =  cos(dec) cosH X - cos(dec) sinH Y + sin(dec) Z, in wavelengths;
  * visibilities of point (and Gaussian) sources
    V = sum_k S_k exp(+2 pi i (u l_k + v m_k)) (times the Gaussian's transform), plus
    complex Gaussian noise -- SDE's sign: its direct-transform imaging applies
    exp(-2 pi i u l) with l = CDELT (I - CRPIX), CDELT < 0 in RA (vis/visdftp2.f:101-107),
    so a source east of the centre (l > 0) appears left of the centre pixel.
Visibilities are ordered channel-major, then time, then baseline (AIPS 'TB' order within a
channel).  Coordinates are float32 wavelengths, visibilities complex64, weights float32,
matching the reference's SoA layout (Vis/UU, Vis/VV, Vis/WW, Vis/OBS/I/VIS, .../WT).
"""
import math

import numpy as np

C_LIGHT = 299792458.0
LAT_DEG = 34.0784
SEED_BASE = 20261203


def y_array(n_ant, arm_m, seed):
    """Antenna positions (east, north, up) in metres on a Y of arms of length arm_m."""
    rng = np.random.default_rng(seed)
    az = np.deg2rad(np.array([0.0, 120.0, 240.0]))
    arm = np.arange(n_ant) % 3
    r = rng.uniform(0.02, 1.0, n_ant) ** 1.5 * arm_m
    east = r * np.sin(az[arm])
    north = r * np.cos(az[arm])
    up = rng.normal(0.0, 2.0, n_ant)
    return np.stack([east, north, up], axis=1)


def baselines(pos):
    n = len(pos)
    i, j = np.triu_indices(n, 1)
    return pos[j] - pos[i]


def uvw_tracks(pos, dec_deg, hours, dt_s, freqs_hz, lat_deg=LAT_DEG):
    """(u, v, w) float32 arrays ordered [channel][time][baseline]."""
    b = baselines(pos)
    lat = math.radians(lat_deg)
    e, n, up = b[:, 0], b[:, 1], b[:, 2]
    X = -math.sin(lat) * n + math.cos(lat) * up
    Y = e
    Z = math.cos(lat) * n + math.sin(lat) * up
    nt = int(round(hours * 3600.0 / dt_s))
    ha = (np.arange(nt) + 0.5) * dt_s / 3600.0 - hours / 2.0
    H = np.deg2rad(ha * 15.0)[:, None]
    d = math.radians(dec_deg)
    sH, cH = np.sin(H), np.cos(H)
    u_m = sH * X + cH * Y
    v_m = -math.sin(d) * cH * X + math.sin(d) * sH * Y + math.cos(d) * Z
    w_m = math.cos(d) * cH * X - math.cos(d) * sH * Y + math.sin(d) * Z
    out = []
    for arr in (u_m, v_m, w_m):
        lam = np.asarray(freqs_hz, np.float64)[:, None, None] / C_LIGHT
        out.append((arr[None, :, :] * lam).astype(np.float32).reshape(-1))
    return out[0], out[1], out[2]


def point_sky(n_src, field_arcsec, seed, s_min=1e-4, s_max=1.0, index=-1.5):
    """Power-law fluxes N(>S) ~ S^index between s_min and s_max, uniform positions."""
    rng = np.random.default_rng(seed + 1)
    a = index
    x = rng.uniform(0, 1, n_src)
    s = (s_min ** a + x * (s_max ** a - s_min ** a)) ** (1.0 / a)
    half = math.radians(field_arcsec / 3600.0) * 0.4
    l = rng.uniform(-half, half, n_src)
    m = rng.uniform(-half, half, n_src)
    return s, l, m


def visibilities(u, v, flux, l, m, noise_sigma, seed, gauss=None, chunk=1 << 20):
    """Complex64 visibilities of point sources (+ optional Gaussians (S, l, m, fwhm_rad)),
    SDE's sign convention (module docstring)."""
    n = len(u)
    out = np.empty(n, np.complex64)
    rng = np.random.default_rng(seed + 2)
    for s0 in range(0, n, chunk):
        uu = u[s0:s0 + chunk].astype(np.float64)
        vv = v[s0:s0 + chunk].astype(np.float64)
        acc = np.zeros(len(uu), np.complex128)
        for S, ll, mm in zip(flux, l, m):
            acc += S * np.exp(2j * np.pi * (uu * ll + vv * mm))
        if gauss is not None:
            for S, ll, mm, fw in gauss:
                sig = fw / (2.0 * math.sqrt(2.0 * math.log(2.0)))
                amp = np.exp(-2.0 * np.pi ** 2 * sig ** 2 * (uu ** 2 + vv ** 2))
                acc += S * amp * np.exp(2j * np.pi * (uu * ll + vv * mm))
        out[s0:s0 + chunk] = acc
    if noise_sigma > 0:
        out += (rng.normal(0, noise_sigma, n) + 1j * rng.normal(0, noise_sigma, n)).astype(
            np.complex64)
    return out


def config1():
    """Plain single field: 27 antennas, Y of 21 km arms, 240 x 120 s, 1 channel at
    1.4 GHz, dec +40; 3 points (1, 0.3, 0.1 Jy) + one 20" Gaussian, sigma 1 mJy;
    512^2 grid at 1" cells, uniform weighting, Hogbom 1000 iterations gain 0.1."""
    seed = SEED_BASE + 1
    pos = y_array(27, 21000.0, seed)
    u, v, w = uvw_tracks(pos, 40.0, 8.0, 120.0, [1.4e9])
    as2r = math.radians(1.0 / 3600.0)
    flux = np.array([1.0, 0.3, 0.1])
    l = np.array([0.0, 40.0, -75.0]) * as2r
    m = np.array([0.0, -30.0, 55.0]) * as2r
    gauss = [(0.2, -20.0 * as2r, -60.0 * as2r, 20.0 * as2r)]
    vis = visibilities(u, v, flux, l, m, 1e-3, seed, gauss=gauss)
    wt = np.ones(len(u), np.float32)
    return dict(u=u, v=v, w=w, vis=vis, wt=wt, imsize=512, cellsize=1.0, vra=0.0, vdec=40.0,
                fov=1.0, rmode="NONE", robust=(0.0, 0.0, 0.0), niter=1000, gain=0.1)


def config2_uvw(n_chan=64, dt_s=10.0):
    """Large single field uv coverage: 27 antennas, 8 h at 10 s x 64 channels over
    1.2-1.6 GHz (64,696,320 visibilities), dec +40."""
    seed = SEED_BASE + 2
    pos = y_array(27, 21000.0, seed)
    freqs = 1.2e9 + (np.arange(n_chan) + 0.5) * (0.4e9 / n_chan)
    return uvw_tracks(pos, 40.0, 8.0, dt_s, freqs), seed


CONFIG2 = dict(imsize=4096, cellsize=0.5, vra=0.0, vdec=40.0, fov=1.0, rmode="NORM",
               robust=(0.0, 0.0, 0.0), n_src=200, noise=1e-3)


def config3_uvw(n_ant=64, n_time=8640, dt_s=5.0, n_chan=32):
    """Precision case uv coverage: 64 antennas (2016 baselines) on a Y of 21 km arms,
    8640 x 5 s (12 h) x 32 channels over 1.2-1.6 GHz = 557,383,680 visibilities, dec +40."""
    seed = SEED_BASE + 3
    pos = y_array(n_ant, 21000.0, seed)
    freqs = 1.2e9 + (np.arange(n_chan) + 0.5) * (0.4e9 / n_chan)
    return uvw_tracks(pos, 40.0, n_time * dt_s / 3600.0, dt_s, freqs), seed


CONFIG3 = dict(imsize=8192, cellsize=0.5, vdec=40.0, n_src=20, noise=1e-3)


# ---- config 4: a mosaic of uneven pointings -----------------------------------------------
CONFIG4 = dict(n_point=49, fwhm_arcmin=30.0, spacing_arcmin=15.0, cell_arcsec=2.0,
               nvis_range=(2e3, 2e6), size_range=(256, 2048), n_src=40, noise=1e-3, dec=40.0,
               arm_m=5000.0, freq_hz=1.4e9, hours=8.0)


def hex_pointings(n, spacing):
    """n pointing offsets (l, m) on a hexagonal lattice (rows offset by half a spacing,
    row pitch spacing*sqrt(3)/2), centred on (0, 0)."""
    side = int(math.ceil(math.sqrt(n)))
    pts = []
    for r in range(side):
        for c in range(side):
            if len(pts) < n:
                pts.append(((c + 0.5 * (r % 2)) * spacing, r * spacing * math.sqrt(3.0) / 2.0))
    pts = np.array(pts)
    return pts - pts.mean(axis=0)


def config4(n_point=None, seed=SEED_BASE + 4, nvis_range=None, size_range=None, vis_fn=None):
    """Seeded mosaic: per pointing a dict(u, v, w, vis, wt, imsize, l0, m0, pb_fwhm_rad).
    Pointing i sees the sky through a Gaussian primary beam centred on (l0, m0); its
    visibilities are phased to its own centre.  vis_fn(u, v, flux, l, m, noise, seed) may
    replace the numpy visibility sum (e.g. a device version); default: visibilities()."""
    c = dict(CONFIG4)
    n_point = c["n_point"] if n_point is None else n_point
    nvis_range = c["nvis_range"] if nvis_range is None else nvis_range
    size_range = c["size_range"] if size_range is None else size_range
    rng = np.random.default_rng(seed)
    a2r = math.radians(1.0 / 3600.0)
    fwhm = c["fwhm_arcmin"] * 60.0 * a2r
    centres = hex_pointings(n_point, c["spacing_arcmin"] * 60.0 * a2r)
    pos = y_array(27, c["arm_m"], seed)
    # sky: power-law point sources over the mosaic area (+ one FWHM margin)
    ext = np.abs(centres).max(axis=0) + fwhm
    a = -1.5
    x = rng.uniform(0, 1, c["n_src"])
    flux = (1e-3 ** a + x * (1.0 ** a - 1e-3 ** a)) ** (1.0 / a)
    sl = rng.uniform(-ext[0], ext[0], c["n_src"])
    sm = rng.uniform(-ext[1], ext[1], c["n_src"])
    lo, hi = math.log(nvis_range[0]), math.log(nvis_range[1])
    e_lo, e_hi = int(round(math.log2(size_range[0]))), int(round(math.log2(size_range[1])))
    nbl = 27 * 26 // 2
    out = []
    for i, (l0, m0) in enumerate(centres):
        nvis = int(math.exp(rng.uniform(lo, hi)))
        imsize = 2 ** int(rng.integers(e_lo, e_hi + 1))
        nt = max(1, -(-nvis // nbl))
        u, v, w = uvw_tracks(pos, c["dec"], c["hours"], c["hours"] * 3600.0 / nt, [c["freq_hz"]])
        u, v, w = u[:nvis], v[:nvis], w[:nvis]
        dl, dm = sl - l0, sm - m0
        pb = np.exp(-4.0 * math.log(2.0) * (dl ** 2 + dm ** 2) / fwhm ** 2)
        keep = pb > 1e-3
        fn = vis_fn or visibilities
        vis = fn(u, v, flux[keep] * pb[keep], dl[keep], dm[keep], c["noise"], seed + 100 + i)
        out.append(dict(u=u, v=v, w=w, vis=np.asarray(vis, np.complex64),
                        wt=np.ones(len(u), np.float32), imsize=imsize, l0=float(l0),
                        m0=float(m0), pb_fwhm_rad=fwhm))
    return out, c
