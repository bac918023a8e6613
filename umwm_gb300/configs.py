"""Seeded synthetic workloads (numpy only).

Each builder returns a Case: a main.nml text plus the inputs the reference
would read from files (grid/topography, forcing snapshots per time key,
a restart spectrum), ready to be staged into the GPU library (umwm_gb300)
or into any object with the same put_* methods.

Workloads (sizes are parameters so tests can run reduced versions):
  fetch_limited  100x100, dx=5 km, 1000 m, 10 m/s along +x, JONSWAP Hs 0.1 m
                 fp 0.3 Hz + 1 % noise, 6 h, constant forcing
  random_field   1000x1000, dx=2 km, ~20 % land from a smoothed Gaussian
                 field, log-Gaussian depth 10-5000 m (50 km correlation),
                 smooth wind 0-25 m/s (200 km), currents 0-1 m/s, 3 h
  hurricane      800x800, dx=2 km, linear shelf 20->3000 m over 300 km with
                 +-5 % roughness, translating Holland vortex (Vmax 50 m/s,
                 Rmax 30 km, B 1.5, 5 m/s), 0.5 m/s background current,
                 600 s forcing snapshots, 12 h
"""
import numpy as np

from .namelist import DEFAULTS, make_namelist

G = 9.80665


def _time_str(t0, seconds):
    """'YYYY-MM-DD hh:mm:ss' of t0 + seconds."""
    base = np.datetime64(t0.replace(" ", "T"), "s") + np.timedelta64(int(seconds), "s")
    return str(base).replace("T", " ")


def spectral_grid(om=37, pm=36, fmin=0.0313, fmax=2.0):
    dlnf = (np.log(fmax) - np.log(fmin)) / (om - 1)
    f = np.exp(np.log(fmin) + np.arange(om) * dlnf)
    dth = 2 * np.pi / pm
    th = (np.arange(1, pm + 1) - 0.5 * (pm + 1)) * dth
    return f, th, dlnf, dth


def wavenumber(f, d, sfct=0.07, rhow=1030.0):
    """Linear dispersion with surface tension, solved to convergence in fp64."""
    f = np.asarray(f, dtype=np.float64)
    d = np.asarray(d, dtype=np.float64)
    fnd = 2 * np.pi * np.sqrt(d / G) * f
    b = sfct / (rhow * G * d * d)
    k = fnd * fnd + 0 * b
    for _ in range(60):
        t = np.tanh(k)
        dk = -(fnd * fnd - k * t * (1 + b * k * k)) / (3 * b * k * k * t + t + k * (1 + b * k * k) * (1 - t * t))
        k = k - dk
    return np.abs(k) / d


def kdk_table(depth, f, dlnf):
    """k*dk(o, i) for each depth (dk = 2 pi f dlnf / cg), interpolated in log depth."""
    depth = np.asarray(depth, dtype=np.float64)
    grid = np.exp(np.linspace(np.log(max(depth.min(), 1e-3)), np.log(depth.max() * 1.0001 + 1e-3), 2048))
    k = wavenumber(f[None, :], grid[:, None])
    kd = np.minimum(k * grid[:, None], 20.0)
    cp = 2 * np.pi * f[None, :] / k
    cg = cp * (0.5 + k * grid[:, None] / np.sinh(2 * kd) + 0.07 * k * k / (1030.0 * G + 0.07 * k * k))
    kdk = k * (2 * np.pi * dlnf * f[None, :]) / np.abs(cg)
    x = np.log(grid)
    xi = np.log(depth)
    out = np.empty((depth.size, f.size))
    for o in range(f.size):
        out[:, o] = np.interp(xi, x, np.log(kdk[:, o]))
    return np.exp(out)


def jonswap_state(depth, wdir, hs, fp, om=37, pm=36, fmin=0.0313, fmax=2.0, gamma=3.3, noise=0.01, seed=1):
    """Restart spectrum F as an (im, pm, om) float32 array: JONSWAP(f) x cos^2
    spreading about wdir, scaled per point so 4 sqrt(sum F kdk dth) = hs, times
    (1 + noise U(-1,1)) from a seeded Philox stream."""
    f, th, dlnf, dth = spectral_grid(om, pm, fmin, fmax)
    depth = np.asarray(depth, dtype=np.float64)
    im = depth.size
    sig = np.where(f <= fp, 0.07, 0.09)
    S = f ** -5 * np.exp(-1.25 * (fp / f) ** 4) * gamma ** np.exp(-((f - fp) ** 2) / (2 * sig ** 2 * fp ** 2))
    wd = np.broadcast_to(np.asarray(wdir, dtype=np.float64), (im,))
    ang = th[None, :] - wd[:, None]
    D = np.where(np.cos(ang) > 0, np.cos(ang) ** 2, 0.0)  # (im, pm)
    kdk = kdk_table(depth, f, dlnf)                        # (im, om)
    m0_unit = (S * f * dlnf)[None, :].sum(1) * D.sum(1) * dth  # per point, before 1/kdk
    scale = (hs / 4.0) ** 2 / m0_unit                          # (im,)
    out = np.empty((im, pm, om), dtype=np.float32)
    rng = np.random.Generator(np.random.Philox(seed))
    chunk = max(1, 4_000_000 // (pm * om))
    Sf = (S * f * dlnf)[None, None, :]
    for a in range(0, im, chunk):
        b = min(im, a + chunk)
        base = scale[a:b, None, None] * D[a:b, :, None] * Sf / kdk[a:b, None, :]
        u = rng.random((b - a, pm, om), dtype=np.float32) * 2 - 1
        out[a:b] = (base * (1 + noise * u)).astype(np.float32)
    return out


def unroll(mask):
    """Wet points in the reference's serial unrolling order (m outer, n inner)."""
    ms, ns = np.nonzero(np.asarray(mask).astype(bool))   # row-major over (m, n) = m outer, n inner
    return ms + 1, ns + 1


def sea_mask_from_z(z, isglobal=False):
    """Mask rule of umwm_init.F90:581-605 without the optional fills."""
    mask = (np.asarray(z) < 0).astype(np.int32)
    mask[:, 0] = 0
    mask[:, -1] = 0
    if not isglobal:
        mask[0, :] = 0
        mask[-1, :] = 0
    return mask


def smooth_field(shape, sigma_cells, rng):
    """Zero-mean, unit-variance Gaussian random field with a Gaussian kernel of
    sigma_cells, made with FFTs (periodic)."""
    noise = rng.standard_normal(shape)
    kx = np.fft.fftfreq(shape[0])[:, None]
    ky = np.fft.rfftfreq(shape[1])[None, :]
    filt = np.exp(-2 * (np.pi * sigma_cells) ** 2 * (kx ** 2 + ky ** 2))
    fld = np.fft.irfft2(np.fft.rfft2(noise) * filt, s=shape)
    fld -= fld.mean()
    fld /= fld.std() + 1e-30
    return fld


class Case:
    """A namelist plus staged inputs."""

    def __init__(self, name, nml, start, stop, gridtopo=None, forcing=None, restart=None, meta=None):
        self.name = name
        self.nml = nml
        self.start = start
        self.stop = stop
        self.gridtopo = gridtopo or {}
        self.forcing = forcing or {}
        self.restart = restart  # (time, F(im,pm,om), ust(im)) or None
        self.meta = meta or {}

    def stage(self, api):
        """api: module or object with put_gridtopo / put_forcing / put_restart."""
        for var, fld in self.gridtopo.items():
            api.put_gridtopo(var, fld)
        for t, vars_ in self.forcing.items():
            for var, fld in vars_.items():
                api.put_forcing(t, var, fld)
        if self.restart is not None:
            t, F, u = self.restart
            api.put_restart(t, F, u)


def _ustar_guess(w):
    cd = np.where(w > 11, (0.49 + 0.065 * w) * 1e-3, 1.2e-3)
    return (np.sqrt(cd) * w).astype(np.float32)


def fetch_limited(mm=100, nm=100, hours=6, dx=5000.0, depth=1000.0, wspd=10.0, hs=0.1, fp=0.3, seed=1,
                  restart=True, **nml):
    """Idealised fetch-limited wind sea (constant forcing, uniform depth)."""
    start = "2012-01-01 00:00:00"
    stop = _time_str(start, hours * 3600)
    kw = dict(mm=mm, nm=nm, delx=dx, dely=dx, dpt=depth, wspd0=wspd, wdir0=0.0, startTimeStr=start,
              stopTimeStr=stop, restart=restart, xpl=mm // 2, ypl=nm // 2, dtg=3600)
    kw.update(nml)
    text = make_namelist(**kw)
    rs = None
    if restart:
        im = (mm - 2) * (nm - 2)
        F = jonswap_state(np.full(im, depth), 0.0, hs, fp, om=kw.get("om", 37), pm=kw.get("pm", 36), seed=seed)
        rs = (start, F, np.full(im, _ustar_guess(np.float32(wspd)), dtype=np.float32))
    return Case("fetch_limited_%dx%d" % (mm, nm), text, start, stop, restart=rs,
                meta=dict(mm=mm, nm=nm, hours=hours))


def random_field(mm=1000, nm=1000, hours=3, dx=2000.0, seed=2, hs=0.2, fp=0.3, land_frac=0.2, **nml):
    """Large domain with land, variable depth, winds and currents (constant in time)."""
    rng = np.random.Generator(np.random.Philox(seed))
    scale = dx / 2000.0
    land = smooth_field((mm, nm), 25.0 / scale, rng)
    depth_f = smooth_field((mm, nm), 25.0 / scale, rng)
    u = smooth_field((mm, nm), 100.0 / scale, rng)
    v = smooth_field((mm, nm), 100.0 / scale, rng)
    cu = smooth_field((mm, nm), 25.0 / scale, rng)
    cv = smooth_field((mm, nm), 25.0 / scale, rng)
    thr = np.quantile(land, land_frac)
    depth = np.clip(np.exp(np.log(300.0) + 1.3 * depth_f), 10.0, 5000.0)
    z = np.where(land < thr, np.maximum(1.0, 10 * (thr - land)), -depth).astype(np.float32)
    sp = np.hypot(u, v)
    uw = (u * 25.0 / sp.max()).astype(np.float32)
    vw = (v * 25.0 / sp.max()).astype(np.float32)
    cs = np.hypot(cu, cv)
    uc = (cu / cs.max()).astype(np.float32)
    vc = (cv / cs.max()).astype(np.float32)
    start = "2012-01-01 00:00:00"
    stop = _time_str(start, hours * 3600)
    # a global (periodic in m) domain keeps its m = 1 and m = mm rows wet
    isglobal = bool({k.lower(): v for k, v in nml.items()}.get("isglobal", False))
    mask = sea_mask_from_z(z, isglobal)
    wm, wn = unroll(mask)
    if len(wm) == 0:
        raise ValueError("random_field: no wet point")
    xm, yn = int(wm[len(wm) // 2]), int(wn[len(wn) // 2])
    kw = dict(mm=mm, nm=nm, delx=dx, dely=dx, topoFromFile=True, winds=True, currents=True, restart=True,
              startTimeStr=start, stopTimeStr=stop, xpl=xm, ypl=yn, dtg=3600)
    kw.update(nml)
    text = make_namelist(**kw)
    forcing = {}
    for h in range(hours + 1):
        forcing[_time_str(start, h * 3600)] = {"uw": uw, "vw": vw, "uc": uc, "vc": vc}
    dwet = -z[wm - 1, wn - 1].astype(np.float64)
    wdir = np.arctan2(vw[wm - 1, wn - 1], uw[wm - 1, wn - 1]).astype(np.float64)
    F = jonswap_state(dwet, wdir, hs, fp, om=kw.get("om", 37), pm=kw.get("pm", 36), seed=seed + 100)
    ust = _ustar_guess(np.hypot(uw, vw)[wm - 1, wn - 1])
    return Case("random_field_%dx%d" % (mm, nm), text, start, stop, gridtopo={"z": z}, forcing=forcing,
                restart=(start, F, ust), meta=dict(mm=mm, nm=nm, hours=hours, im=len(wm)))


def holland_wind(X, Y, xc, yc, vmax=50.0, rmax=30e3, B=1.5, heading=0.0, vt=5.0, inflow=np.deg2rad(20.0)):
    """Holland (1980) gradient-wind profile V = Vmax sqrt((Rmax/r)^B exp(1-(Rmax/r)^B)),
    counter-clockwise with inflow, plus half the translation velocity."""
    dx, dy = X - xc, Y - yc
    r = np.hypot(dx, dy) + 1.0
    a = (rmax / r) ** B
    V = vmax * np.sqrt(a * np.exp(1 - a))
    ang = np.arctan2(dy, dx) + 0.5 * np.pi + inflow
    u = V * np.cos(ang) + 0.5 * vt * np.cos(heading)
    v = V * np.sin(ang) + 0.5 * vt * np.sin(heading)
    return u.astype(np.float32), v.astype(np.float32)


def hurricane(mm=800, nm=800, hours=12, dx=2000.0, seed=3, dtg=600, vmax=50.0, rmax=30e3, B=1.5, hs=0.2, fp=0.3,
              heading_scale=1.0, warm=True, **nml):
    """Translating Holland vortex over a linear shelf.  heading_scale scales
    the seeded heading (ensemble perturbations); warm=False starts cold
    (restart=.false.: the model's own initial spectrum, no restart staged)."""
    rng = np.random.Generator(np.random.Philox(seed))
    x = (np.arange(mm) * dx)[:, None] * np.ones((1, nm))
    y = (np.arange(nm) * dx)[None, :] * np.ones((mm, 1))
    shelf = np.minimum(x / 300e3, 1.0)
    depth = 20.0 + (3000.0 - 20.0) * shelf
    rough = smooth_field((mm, nm), 5.0, rng)
    depth = depth * (1 + 0.05 * np.clip(rough / 3.0, -1, 1))
    z = (-depth).astype(np.float32)
    heading = rng.uniform(0, 2 * np.pi) * heading_scale
    cur_dir = rng.uniform(0, 2 * np.pi)
    vt = 5.0
    Lx, Ly = mm * dx, nm * dx
    travel = vt * hours * 3600
    xc0 = 0.5 * Lx - 0.5 * travel * np.cos(heading)
    yc0 = 0.5 * Ly - 0.5 * travel * np.sin(heading)
    start = "2012-01-01 00:00:00"
    stop = _time_str(start, hours * 3600)
    nsnap = int(hours * 3600 // dtg)
    forcing = {}
    ucf = np.full((mm, nm), 0.5 * np.cos(cur_dir), dtype=np.float32)
    vcf = np.full((mm, nm), 0.5 * np.sin(cur_dir), dtype=np.float32)
    for s in range(nsnap + 1):
        t = s * dtg
        xc = xc0 + vt * t * np.cos(heading)
        yc = yc0 + vt * t * np.sin(heading)
        uw, vw = holland_wind(x, y, xc, yc, vmax, rmax, B, heading, vt)
        forcing[_time_str(start, t)] = {"uw": uw, "vw": vw, "uc": ucf, "vc": vcf}
    mask = sea_mask_from_z(z)
    wm, wn = unroll(mask)
    kw = dict(mm=mm, nm=nm, delx=dx, dely=dx, topoFromFile=True, winds=True, currents=True, restart=warm,
              startTimeStr=start, stopTimeStr=stop, xpl=mm // 2, ypl=nm // 2, dtg=dtg)
    kw.update(nml)
    text = make_namelist(**kw)
    meta = dict(mm=mm, nm=nm, hours=hours, im=len(wm), heading=heading, vmax=vmax, rmax=rmax)
    if not warm:
        return Case("hurricane_%dx%d" % (mm, nm), text, start, stop, gridtopo={"z": z}, forcing=forcing, meta=meta)
    f0 = forcing[start]
    wdir = np.arctan2(f0["vw"][wm - 1, wn - 1], f0["uw"][wm - 1, wn - 1]).astype(np.float64)
    F = jonswap_state(depth[wm - 1, wn - 1], wdir, hs, fp, om=kw.get("om", 37), pm=kw.get("pm", 36), seed=seed + 100)
    ust = _ustar_guess(np.hypot(f0["uw"], f0["vw"])[wm - 1, wn - 1])
    return Case("hurricane_%dx%d" % (mm, nm), text, start, stop, gridtopo={"z": z}, forcing=forcing,
                restart=(start, F, ust), meta=meta)


def ensemble_members(n=64, seed=11, size_lo=(200, 200), size_hi=(1000, 600), hours=12, dx=2000.0, dtg=600,
                     warm=True, **kw):
    """n hurricane members: grid sizes uniform in [size_lo, size_hi] and Vmax,
    Rmax and heading scaled by seeded factors in [0.85, 1.15]; member m uses
    seed + m for its bathymetry roughness and base heading."""
    rng = np.random.Generator(np.random.Philox(seed))
    out = []
    for m in range(n):
        mm = int(rng.integers(size_lo[0], size_hi[0] + 1))
        nm = int(rng.integers(size_lo[1], size_hi[1] + 1))
        fv, fr, fh = rng.uniform(0.85, 1.15, size=3)
        out.append(hurricane(mm=mm, nm=nm, hours=hours, dx=dx, seed=seed + m, dtg=dtg, vmax=50.0 * fv,
                             rmax=30e3 * fr, heading_scale=fh, warm=warm, **kw))
    return out


__all__ = ["Case", "fetch_limited", "random_field", "hurricane", "ensemble_members", "jonswap_state", "unroll", "sea_mask_from_z",
           "spectral_grid", "wavenumber", "DEFAULTS"]
