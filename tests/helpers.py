"""Shared helpers of the parity tests: run a Case on the GPU library and on
the oracle with the same inputs and compare fields."""
import numpy as np


def run_gpu(U, case, max_substeps=-1, start=None, stop=None, groups=None):
    """Run the GPU library on a case; groups (2 or 4) fixes the direction
    mapping of the spectral kernels instead of the size-based default."""
    U.clear_inputs()
    case.stage(U)
    U.umwm_initialize(nml_text=case.nml)
    if groups is not None:
        U.set_option("direction_groups", groups)
    U.set_option("max_substeps", max_substeps)
    U.umwm_run(start or case.start, stop or case.stop)


def run_oracle(pyoracle, case, prec=32, max_substeps=-1, start=None, stop=None):
    o = pyoracle.Oracle(case.nml, prec)
    case.stage(o)
    o.initialize()
    o.set_option("max_substeps", max_substeps)
    o.run(start or case.start, stop or case.stop)
    return o


def rel_err(a, b, floor_frac=1e-6):
    """Max relative error of a vs b where |b| > floor_frac * max|b|."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    m = np.abs(b) > floor_frac * np.abs(b).max() if b.size and np.abs(b).max() > 0 else np.zeros(b.shape, bool)
    if not m.any():
        return float(np.abs(a - b).max()) if a.size else 0.0
    return float((np.abs(a[m] - b[m]) / np.abs(b[m])).max())


def vec_err(ax, ay, bx, by):
    """Max |a - b| of a 2-vector field relative to the largest |b|."""
    ax, ay, bx, by = (np.asarray(v, dtype=np.float64) for v in (ax, ay, bx, by))
    scale = np.hypot(bx, by).max()
    if scale == 0:
        return float(max(np.abs(ax).max(), np.abs(ay).max()))
    return float(max(np.abs(ax - bx).max(), np.abs(ay - by).max()) / scale)


def spec_stats(a, b, floor_frac=1e-6):
    """Relative L2 norm, 99.9th percentile and max of the bin-wise relative
    error of spectrum a against b (bins of b above floor_frac * max b)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    l2 = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    m = np.abs(b) > floor_frac * np.abs(b).max()
    r = np.abs(a[m] - b[m]) / np.abs(b[m])
    return l2, float(np.percentile(r, 99.9)), float(r.max())


def lonlat_grid(mm, nm, lon0=-80.0, lat0=20.0, dlon=0.05, dlat=0.05, skew=0.002):
    """A skewed longitude/latitude grid (mm, nm) for gridFromFile cases."""
    m = np.arange(mm)[:, None]
    n = np.arange(nm)[None, :]
    lon = lon0 + dlon * m + skew * n
    lat = lat0 + dlat * n + 0.5 * skew * m
    return lon.astype(np.float32), lat.astype(np.float32)
