"""Seeded synthetic interferometer data for the w-gridder workloads.

There are no measurement sets in this environment, so the workloads are built
from first principles: antenna positions on a local east-north-up grid, rotated
to equatorial baseline coordinates at a fixed site latitude, tracked with
earth-rotation uvw over the requested time steps, point-source sky models, and
complex Gaussian noise.  Model visibilities use the convention
V = sum_s S_s exp(+2 pi i (u l_s + v m_s + w (n_s - 1))), which places flux S_s
at (l_s, m_s) in the image of gridding/directmsgridder.cpp:92-132.

Samples whose |u| dl or |v| dm reach 0.5 lie beyond the image's Nyquist limit;
they are set to zero (WSClean's gridder skips zero visibilities,
wgridder/gridder_simple.h:111) and their fraction is reported.
"""
import math

import numpy as np

C_LIGHT = 299792458.0
ARCSEC = math.pi / (180.0 * 3600.0)
SITE_LATITUDE_DEG = 34.0784  # fixed site latitude used for every array
OMEGA_EARTH = 7.2921150e-5  # rad/s (sidereal)

# Workload definitions (image, pixel size, array, time and frequency sampling,
# sky model).  "wide" etc. name the workloads by what they are.
WORKLOADS = {
    # 1024^2 Stokes I, 10" pixels; 64 antennas uniform in a 3 km disk; 2016
    # baselines x 60 x 10 s; 16 channels 120-180 MHz; 20 sources; eps 1e-4.
    "plain1024": dict(npix=1024, pix_arcsec=10.0, n_ant=64, layout="disk", radius_m=1500.0,
                      n_t=60, dt=10.0, n_chan=16, f0=120e6, f1=180e6, n_src=20,
                      flux="loguniform", fmin=0.01, fmax=1.0, noise=0.01, weights="unit",
                      dec_deg=45.0, epsilon=1e-4),
    # 8192^2, 3" pixels; 256 antennas log-radial to 20 km; 32640 baselines x
    # 300 x 8 s; 64 channels 0.9-1.7 GHz; 500 sources, power law; eps 1e-5.
    "wide8192": dict(npix=8192, pix_arcsec=3.0, n_ant=256, layout="lograd", radius_m=20000.0,
                     n_t=300, dt=8.0, n_chan=64, f0=0.9e9, f1=1.7e9, n_src=500,
                     flux="powerlaw", fmin=1e-3, fmax=5.0, noise=0.01, weights="uniform",
                     dec_deg=45.0, epsilon=1e-5),
    # Profiling-size wide field: the 8192^2 workload's array, pixels and band
    # on a 2048^2 image over 8 time steps; each 16x16-cell x 16-plane gridding
    # unit reads about as many visibilities (~190) as in the full workload
    # (~180), within a few GB of device memory.
    "wide2048": dict(npix=2048, pix_arcsec=3.0, n_ant=256, layout="lograd", radius_m=20000.0,
                     n_t=8, dt=8.0, n_chan=64, f0=0.9e9, f1=1.7e9, n_src=500,
                     flux="powerlaw", fmin=1e-3, fmax=5.0, noise=0.01, weights="uniform",
                     dec_deg=45.0, epsilon=1e-5),
    # 4096^2 full polarisation with the 3 km array, 32 channels.
    "fullpol4096": dict(npix=4096, pix_arcsec=10.0, n_ant=64, layout="disk", radius_m=1500.0,
                        n_t=60, dt=10.0, n_chan=32, f0=120e6, f1=180e6, n_src=20,
                        flux="loguniform", fmin=0.01, fmax=1.0, noise=0.01, weights="unit",
                        dec_deg=45.0, epsilon=1e-4),
}


def antenna_enu(n_ant, layout, radius_m, rng):
    if layout == "disk":
        r = radius_m * np.sqrt(rng.uniform(0.0, 1.0, n_ant))
    elif layout == "lograd":
        r = np.exp(rng.uniform(np.log(25.0), np.log(radius_m), n_ant))
    else:
        raise ValueError(layout)
    phi = rng.uniform(0.0, 2 * np.pi, n_ant)
    e = r * np.cos(phi)
    n = r * np.sin(phi)
    u = rng.normal(0.0, 2.0, n_ant)  # a few metres of height scatter
    return np.stack([e, n, u], axis=1)


def baselines_xyz(enu, lat_deg=SITE_LATITUDE_DEG):
    """Baseline vectors (i < j) in the equatorial frame (X toward H=0, Y east, Z pole)."""
    lat = np.radians(lat_deg)
    e, n, u = enu[:, 0], enu[:, 1], enu[:, 2]
    x = -np.sin(lat) * n + np.cos(lat) * u
    y = e
    z = np.cos(lat) * n + np.sin(lat) * u
    xyz = np.stack([x, y, z], axis=1)
    i, j = np.triu_indices(len(enu), k=1)
    return xyz[j] - xyz[i], i, j


def uvw_tracks(bxyz, n_t, dt, dec_deg):
    """Earth-rotation uvw (metres), rows ordered time-major: row = t*n_bl + bl."""
    dec = np.radians(dec_deg)
    h = (np.arange(n_t) - 0.5 * (n_t - 1)) * dt * OMEGA_EARTH
    sh, ch = np.sin(h)[:, None], np.cos(h)[:, None]
    X, Y, Z = bxyz[None, :, 0], bxyz[None, :, 1], bxyz[None, :, 2]
    u = sh * X + ch * Y
    v = -np.sin(dec) * ch * X + np.sin(dec) * sh * Y + np.cos(dec) * Z
    w = np.cos(dec) * ch * X - np.cos(dec) * sh * Y + np.sin(dec) * Z
    return np.stack([u, v, w], axis=-1).reshape(-1, 3)


def sky_model(cfg, rng, dl):
    n = cfg["n_src"]
    half = 0.5 * cfg["npix"] * dl * 0.95
    l = rng.uniform(-half, half, n)
    m = rng.uniform(-half, half, n)
    if cfg["flux"] == "loguniform":
        s = np.exp(rng.uniform(np.log(cfg["fmin"]), np.log(cfg["fmax"]), n))
    else:
        # power law dN/dS ~ S^-1.8 between fmin and fmax (inverse CDF)
        a = 1.0 - 1.8
        u = rng.uniform(0.0, 1.0, n)
        s = (cfg["fmin"] ** a + u * (cfg["fmax"] ** a - cfg["fmin"] ** a)) ** (1.0 / a)
    return np.stack([l, m, s], axis=1)


def nm1(l, m):
    r2 = l * l + m * m
    return np.where(r2 >= 1.0, 0.0, -r2 / (np.sqrt(np.maximum(1.0 - r2, 0.0)) + 1.0))


def model_vis_numpy(uvw, freq, sources):
    """sum_s S exp(+2 pi i (u l + v m + w (n-1))), FP64 phases (small cases)."""
    inv_lambda = freq / C_LIGHT
    out = np.zeros((uvw.shape[0], freq.size), np.complex128)
    for l, m, s in sources:
        t = (uvw[:, 0:1] * l + uvw[:, 1:2] * m + uvw[:, 2:3] * nm1(l, m)) * inv_lambda[None, :]
        t -= np.rint(t)
        out += s * np.exp(2j * np.pi * t)
    return out


def model_vis_torch(uvw, freq, sources, device, chunk_rows=1 << 16):
    """Same model on a CUDA device with torch (large cases; FP32 phases after an
    FP64 row-wise reduction).  Used only to make input data."""
    import torch
    fl = torch.tensor(freq / C_LIGHT, dtype=torch.float64, device=device)
    src = torch.tensor(np.stack([sources[:, 0], sources[:, 1], nm1(sources[:, 0], sources[:, 1]),
                                 sources[:, 2]], 1), dtype=torch.float64, device=device)
    out = torch.empty((uvw.shape[0], freq.size), dtype=torch.complex64, device=device)
    for r0 in range(0, uvw.shape[0], chunk_rows):
        u = torch.as_tensor(uvw[r0:r0 + chunk_rows], device=device)
        # turns per unit frequency factor, per row and source (FP64), then per channel
        base = u @ src[:, :3].T  # rows x src, metres * direction
        acc = torch.zeros((u.shape[0], freq.size), dtype=torch.complex64, device=device)
        for c in range(freq.size):
            t = base * fl[c]
            t = (t - torch.round(t)).float()
            acc[:, c] = (src[:, 3].float()[None, :] * torch.exp(2j * math.pi * t)).sum(1)
        out[r0:r0 + u.shape[0]] = acc
    return out


def make_workload(name, seed=1, max_rows=None, with_model=True, device=None,
                  n_src=None, n_t=None):
    """Builds the named workload.  Returns a dict with uvw [rows,3] f64, freq f64,
    vis [rows, chan] complex64 (weighted, Nyquist-guarded), image/pixel geometry,
    the sources and the sum of weights (ImageWeight).  max_rows keeps a
    leading subset of rows (all baselines of the first time steps); n_t
    overrides the number of time steps."""
    cfg = dict(WORKLOADS[name])
    if n_src is not None:
        cfg["n_src"] = n_src
    if n_t is not None:
        cfg["n_t"] = int(n_t)
    rng = np.random.default_rng(seed)
    enu = antenna_enu(cfg["n_ant"], cfg["layout"], cfg["radius_m"], rng)
    bxyz, a1, a2 = baselines_xyz(enu)
    uvw = uvw_tracks(bxyz, cfg["n_t"], cfg["dt"], cfg["dec_deg"])
    n_bl = bxyz.shape[0]
    ant1 = np.tile(a1, cfg["n_t"])
    ant2 = np.tile(a2, cfg["n_t"])
    tidx = np.repeat(np.arange(cfg["n_t"]), n_bl)
    if max_rows is not None:
        uvw, ant1, ant2, tidx = uvw[:max_rows], ant1[:max_rows], ant2[:max_rows], tidx[:max_rows]
    freq = np.linspace(cfg["f0"], cfg["f1"], cfg["n_chan"])
    dl = cfg["pix_arcsec"] * ARCSEC
    sources = sky_model(cfg, rng, dl)
    n_rows = uvw.shape[0]
    out = dict(name=name, uvw=np.ascontiguousarray(uvw), freq=freq, width=cfg["npix"],
               height=cfg["npix"], dl=dl, dm=dl, epsilon=cfg["epsilon"], sources=sources,
               ant1=ant1, ant2=ant2, time_index=tidx, n_ant=cfg["n_ant"], n_t=cfg["n_t"])
    inv_lambda = freq / C_LIGHT
    ul = np.abs(uvw[:, 0:1]) * inv_lambda[None, :] * dl
    vl = np.abs(uvw[:, 1:2]) * inv_lambda[None, :] * dl
    keep = (ul < 0.5) & (vl < 0.5)
    out["flagged_fraction"] = float(1.0 - keep.mean())
    if cfg["weights"] == "unit":
        wts = np.ones((n_rows, freq.size), np.float32)
    else:
        wts = rng.uniform(0.5, 1.5, (n_rows, freq.size)).astype(np.float32)
    wts[~keep] = 0.0
    out["image_weight"] = float(wts.sum(dtype=np.float64))
    if not with_model:
        out["weights"] = wts
        return out
    if device is None:
        v = model_vis_numpy(uvw, freq, sources)
        noise = cfg["noise"] * (rng.standard_normal(v.shape) + 1j * rng.standard_normal(v.shape))
        vis = ((v + noise) * wts).astype(np.complex64)
    else:
        import torch
        v = model_vis_torch(uvw, freq, sources, device)
        g = torch.Generator(device=device)
        g.manual_seed(seed)
        noise = torch.randn(v.shape, generator=g, dtype=torch.complex64, device=device)
        vis = ((v + cfg["noise"] * (2 ** 0.5) * noise) *
               torch.as_tensor(wts, device=device)).cpu().numpy()
    out["vis"] = np.ascontiguousarray(vis)
    return out


def random_points(n_rows, n_chan, width, dl, seed, w_scale=1.0, f0=1e8, f1=2e8,
                  frac_zero=0.0):
    """Small random test sets: uvw uniform within the grid's Nyquist range and
    random complex visibilities."""
    rng = np.random.default_rng(seed)
    freq = np.linspace(f0, f1, n_chan)
    umax = 0.45 / dl * C_LIGHT / f1
    uvw = np.empty((n_rows, 3))
    uvw[:, 0] = rng.uniform(-umax, umax, n_rows)
    uvw[:, 1] = rng.uniform(-umax, umax, n_rows)
    uvw[:, 2] = rng.uniform(-umax, umax, n_rows) * w_scale
    vis = (rng.standard_normal((n_rows, n_chan)) + 1j * rng.standard_normal((n_rows, n_chan)))
    vis = vis.astype(np.complex64)
    if frac_zero > 0:
        vis[rng.uniform(size=vis.shape) < frac_zero] = 0
    return uvw, freq, vis


def full_polarisation(d, device, seed=3, pol_fraction=0.3, gain_scatter=0.1, n_times=None):
    """Four-correlation visibilities (XX, XY, YX, YY) of the workload's sources
    with random Stokes Q, U, V (|pol fraction| <= pol_fraction) for linear
    feeds: XX = I + Q, XY = U + iV, YX = U - iV, YY = I - Q; plus per-antenna
    full-Jones solutions (identity + complex Gaussian scatter) per time step and
    channel, indexed ((t * n_chan + ch) * n_ant + ant) * 4 + parm.  Returns
    (vis [rows, chan, 4] complex64 on the host, antennas [rows, 2] u64, time
    offsets [rows] u64, solutions, n_times)."""
    import torch
    rng = np.random.default_rng(seed)
    src = d["sources"]
    n = src.shape[0]
    frac = rng.uniform(-pol_fraction, pol_fraction, (n, 3)) / np.sqrt(3.0)
    stokes = {"I": src[:, 2], "Q": src[:, 2] * frac[:, 0], "U": src[:, 2] * frac[:, 1],
              "V": src[:, 2] * frac[:, 2]}
    parts = {}
    for k, s in stokes.items():
        srck = src.copy()
        srck[:, 2] = s
        parts[k] = model_vis_torch(d["uvw"], d["freq"], srck, device)
    vis = torch.stack([parts["I"] + parts["Q"], parts["U"] + 1j * parts["V"],
                       parts["U"] - 1j * parts["V"], parts["I"] - parts["Q"]], dim=-1)
    del parts
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    vis = vis + 0.01 * np.sqrt(2.0) * torch.randn(vis.shape, generator=g, dtype=vis.dtype,
                                                  device=device)
    vis = vis.cpu().numpy().astype(np.complex64)
    n_t = int(d["n_t"]) if n_times is None else int(n_times)
    n_ant, n_chan = int(d["n_ant"]), d["freq"].size
    eye = np.array([1, 0, 0, 1], np.complex64)
    sol = (eye[None, None, None, :] + gain_scatter * (
        rng.standard_normal((n_t, n_chan, n_ant, 4)) +
        1j * rng.standard_normal((n_t, n_chan, n_ant, 4)))).astype(np.complex64)
    ant = np.stack([d["ant1"], d["ant2"]], axis=1).astype(np.uint64)
    tof = (d["time_index"] % n_t).astype(np.uint64)
    return np.ascontiguousarray(vis), ant, tof, sol, n_t
