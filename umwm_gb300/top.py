"""Python mirror of the reference's umwm_top module (umwm_top.F90:7-204).

    umwm_initialize()            -> umwm_top.F90:7-29
    umwm_run(start, stop)        -> umwm_top.F90:32-196
    umwm_finalize()              -> umwm_top.F90:199-204

plus the input staging that replaces the reference's netCDF files and the
field getters.  Every call goes through the C ABI of libumwm_gb300.so and
raises UmwmError on a non-zero status.
"""
import ctypes

import numpy as np

from ._lib import check, lib

_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _fortran(field_mn):
    """(mm, nm) array -> flat Fortran order (m fastest)."""
    return _f32(np.asarray(field_mn, dtype=np.float32).ravel(order="F"))


# ---- inputs standing in for files ------------------------------------------

def put_gridtopo(var, field_mn):
    """input/umwm.gridtopo variable 'lon', 'lat' or 'z' as an (mm, nm) array."""
    a = np.asarray(field_mn)
    f = _fortran(a)
    check(lib().umwm_gpu_put_gridtopo(var.encode(), f.ctypes.data_as(_fp), a.shape[0], a.shape[1]))


def put_exclude(pairs):
    """namelists/exclude.nml lake seeds [(m, n), ...] (1-based)."""
    a = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).ravel())
    check(lib().umwm_gpu_put_exclude(a.ctypes.data_as(_ip), len(a) // 2))


def put_forcing(time19, var, field_mn):
    """input/umwmin_<time>.nc variable (uw, vw, uc, vc, rhoa, rhow, fice)."""
    a = np.asarray(field_mn)
    f = _fortran(a)
    check(lib().umwm_gpu_put_forcing(time19.encode(), var.encode(), f.ctypes.data_as(_fp), a.shape[0], a.shape[1]))


def put_restart(time19, e_ipo, ust):
    """restart/umwmrst_<time>.nc: F as an (im, pm, om) array (== Fortran F(om,pm,im)) and ust(im)."""
    e = _f32(e_ipo).ravel()
    u = _f32(ust).ravel()
    check(lib().umwm_gpu_put_restart(time19.encode(), e.ctypes.data_as(_fp), e.size, u.ctypes.data_as(_fp), u.size))


def clear_inputs():
    check(lib().umwm_gpu_clear_inputs())


# ---- umwm_top ---------------------------------------------------------------

def umwm_initialize(nml_path=None, nml_text=None):
    """umwm_initialize: namelist from a path (default namelists/main.nml) or text."""
    if nml_text is not None:
        check(lib().umwm_gpu_initialize_text(nml_text.encode()))
    else:
        check(lib().umwm_gpu_initialize(nml_path.encode() if nml_path else None))


def umwm_run(starttimestr, stoptimestr):
    check(lib().umwm_gpu_run(starttimestr.encode(), stoptimestr.encode()))


def umwm_finalize():
    check(lib().umwm_gpu_finalize())


def ensemble_add(nml_text):
    """Add an ensemble member: this namelist plus the inputs staged so far."""
    check(lib().umwm_gpu_ensemble_add(nml_text.encode()))


def ensemble_initialize():
    """umwm_initialize for every added member, as one model."""
    check(lib().umwm_gpu_ensemble_initialize())


def select_member(m):
    """Member that get_field / get_state / set_state act on."""
    check(lib().umwm_gpu_select_member(int(m)))


def setup_host(nml_text):
    """Host part of umwm_initialize only (no GPU needed)."""
    check(lib().umwm_gpu_setup_host(nml_text.encode()))


# ---- state and fields -------------------------------------------------------

def dims():
    d = (ctypes.c_int * 8)()
    check(lib().umwm_gpu_get_dims(d))
    keys = ("mm", "nm", "om", "pm", "im", "imm", "lm", "substeps")
    return dict(zip(keys, list(d)))


def set_option(name, value):
    check(lib().umwm_gpu_set_option(name.encode(), float(value)))


def stat(name):
    return lib().umwm_gpu_get_stat(name.encode())


_WET = {"ustar", "cd", "taux", "tauy", "taux_form", "tauy_form", "taux_skin", "tauy_skin", "taux_diag",
        "tauy_diag", "tailatmx", "tailatmy", "shelt", "fcutoff", "physics_time_step", "ds", "ht", "mwp", "mwd",
        "mss", "mwl", "dwd", "dwl", "dwp", "dcp0", "dcp", "dcg0", "dcg", "momx", "momy", "cgmxx", "cgmxy", "cgmyy",
        "ar", "oneovar", "oneovdx", "oneovdy", "dxn", "dxs", "dye", "dyw",
        "taux_ocntop", "tauy_ocntop", "taux_ocnbot", "tauy_ocnbot", "taux_snl", "tauy_snl", "epsx_ocn", "epsy_ocn",
        "epsx_atm", "epsy_atm", "tailocnx", "tailocny", "taux1", "tauy1", "taux2", "tauy2", "taux3", "tauy3"}
_IMM = {"wspd", "wdir", "uc", "vc", "rhoa", "rhow", "rhorat", "fice", "d", "dx", "dy"}
_TABLES = {"k", "logl2overz", "fkovg", "k4", "k3dk", "kdk", "cothkd", "sbf", "sdv", "bf1_renorm", "bf2_renorm"}
_SCALARS = {"dts", "dta", "dtr", "dtr_temp", "sumt", "dtamin", "cgmax", "dth"}


def get_field(name):
    """A named field as a numpy array (wet points first axis where applicable)."""
    d = dims()
    om, pm, im, imm, lm, mm, nm = d["om"], d["pm"], d["im"], d["imm"], d["lm"], d["mm"], d["nm"]
    if name in _WET:
        shape = (im,)
    elif name in _IMM:
        shape = (imm,)
    elif name in _TABLES:
        shape = (im, om)
    elif name in ("cp0", "cg0"):
        shape = (im + 1, om)
    elif name in ("ssin", "sds", "snl"):
        shape = (im, pm, om)  # the source terms a stress('ocn') step kept
    elif name in ("us", "vs"):
        shape = (lm, im)
    elif name == "f":
        shape = (om,)
    elif name == "th":
        shape = (pm,)
    elif name == "depth":
        shape = (lm,)
    elif name in ("d_2d", "dx_2d", "dy_2d", "curv", "lon", "lat"):
        out = np.zeros(mm * nm, dtype=np.float32)
        check(lib().umwm_gpu_get_field(name.encode(), out.ctypes.data_as(_fp), out.size))
        return out.reshape(nm, mm).T
    elif name in _SCALARS:
        out = np.zeros(1, dtype=np.float32)
        check(lib().umwm_gpu_get_field(name.encode(), out.ctypes.data_as(_fp), 1))
        return float(out[0])
    else:
        raise KeyError(name)
    out = np.zeros(int(np.prod(shape)), dtype=np.float32)
    if out.size:
        check(lib().umwm_gpu_get_field(name.encode(), out.ctypes.data_as(_fp), out.size))
    return out.reshape(shape)


def get_field_i(name):
    d = dims()
    if name in ("mask", "ii"):
        out = np.zeros(d["mm"] * d["nm"], dtype=np.int32)
        check(lib().umwm_gpu_get_field_i(name.encode(), out.ctypes.data_as(_ip), out.size))
        return out.reshape(d["nm"], d["mm"]).T
    if name in ("im", "imm", "iip", "members", "substeps"):
        out = np.zeros(1, dtype=np.int32)
        check(lib().umwm_gpu_get_field_i(name.encode(), out.ctypes.data_as(_ip), 1))
        return int(out[0])
    n = d["im"] if name == "oc" else d["imm"]
    out = np.zeros(n, dtype=np.int32)
    check(lib().umwm_gpu_get_field_i(name.encode(), out.ctypes.data_as(_ip), n))
    return out


def get_state():
    """(F as an (im, pm, om) array == Fortran F(om,pm,im), ust(im))."""
    d = dims()
    F = np.zeros((d["im"], d["pm"], d["om"]), dtype=np.float32)
    u = np.zeros(d["im"], dtype=np.float32)
    check(lib().umwm_gpu_get_state(F.ctypes.data_as(_fp), u.ctypes.data_as(_fp)))
    return F, u


def get_state_noalloc():
    """get_state without device allocation: the spectrum goes to the host
    through the library's fixed 16 MiB scratch (see umwm_gpu_get_state_noalloc)."""
    d = dims()
    F = np.zeros((d["im"], d["pm"], d["om"]), dtype=np.float32)
    u = np.zeros(d["im"], dtype=np.float32)
    check(lib().umwm_gpu_get_state_noalloc(F.ctypes.data_as(_fp), u.ctypes.data_as(_fp)))
    return F, u


def write_restart(path):
    """restart_write: the selected member's state as a netCDF restart file."""
    check(lib().umwm_gpu_write_restart(str(path).encode()))


def write_output(path):
    """output_grid_nc: the gridded output of the last outer step as a netCDF
    file (needs set_option("stress_ocn", 1) before the run)."""
    check(lib().umwm_gpu_write_output(str(path).encode()))


def set_state(F=None, ust=None):
    Fp = _f32(F).ravel() if F is not None else None
    up = _f32(ust).ravel() if ust is not None else None
    check(lib().umwm_gpu_set_state(Fp.ctypes.data_as(_fp) if Fp is not None else None,
                                   up.ctypes.data_as(_fp) if up is not None else None))


def get_screen():
    """Screen lines so far: (rows, 8) = sumt/dtg, dts, wspd, wdir, swh, mwp, cd*1e3, f(oc)."""
    rows = ctypes.c_long(0)
    check(lib().umwm_gpu_get_screen(None, 0, ctypes.byref(rows)))
    out = np.zeros(rows.value * 8, dtype=np.float64)
    if rows.value:
        check(lib().umwm_gpu_get_screen(out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.size,
                                        ctypes.byref(rows)))
    return out.reshape(-1, 8)


# ---- learned source-term surrogate -------------------------------------------

SURROGATE_WIDTH = 1344


def surrogate_init(om=37, pm=36, seed=0):
    check(lib().umwm_gpu_surrogate_init(int(om), int(pm), int(seed)))


def surrogate_nparams():
    return int(stat("surrogate_nparams"))


def surrogate_get_params():
    out = np.zeros(surrogate_nparams(), dtype=np.float32)
    check(lib().umwm_gpu_surrogate_get_params(out.ctypes.data_as(_fp), out.size))
    return out


def surrogate_set_params(w):
    a = _f32(w).ravel()
    check(lib().umwm_gpu_surrogate_set_params(a.ctypes.data_as(_fp), a.size))


def surrogate_capture(capacity, points_per_substep):
    check(lib().umwm_gpu_surrogate_capture(int(capacity), int(points_per_substep)))


def surrogate_train(steps, batch=4096, lr=1e-3, seed=0):
    """Adam steps on the captured pairs; returns the loss of each step."""
    losses = np.zeros(int(steps), dtype=np.float32)
    check(lib().umwm_gpu_surrogate_train(int(steps), int(batch), float(lr), int(seed), losses.ctypes.data_as(_fp)))
    return losses


def surrogate_eval(first, count):
    """Mean-squared-error loss of the network over stored pairs [first, first+count)."""
    out = ctypes.c_double(0)
    check(lib().umwm_gpu_surrogate_eval(int(first), int(count), ctypes.byref(out)))
    return out.value


def surrogate_forward(X):
    X = _f32(X)
    n = X.shape[0]
    Y = np.zeros((n, SURROGATE_WIDTH), dtype=np.float32)
    check(lib().umwm_gpu_surrogate_forward(X.ctypes.data_as(_fp), n, Y.ctypes.data_as(_fp)))
    return Y


def surrogate_grad(X, T):
    X, T = _f32(X), _f32(T)
    loss = np.zeros(1, dtype=np.float32)
    g = np.zeros(surrogate_nparams(), dtype=np.float32)
    check(lib().umwm_gpu_surrogate_grad(X.ctypes.data_as(_fp), T.ctypes.data_as(_fp), X.shape[0],
                                        loss.ctypes.data_as(_fp), g.ctypes.data_as(_fp)))
    return float(loss[0]), g


def surrogate_features():
    """Surrogate input rows (im, 1344) of the selected member's current state."""
    n = dims()["im"]
    X = np.zeros((n, SURROGATE_WIDTH), dtype=np.float32)
    check(lib().umwm_gpu_surrogate_features(X.ctypes.data_as(_fp), X.size))
    return X


def gemm_bf16(A_bits, B_bits):
    """C = A B^T on the tensor cores; A (M, K), B (N, K) as uint16 bf16 bit patterns."""
    A = np.ascontiguousarray(A_bits, dtype=np.uint16)
    B = np.ascontiguousarray(B_bits, dtype=np.uint16)
    M, K = A.shape
    N = B.shape[0]
    C = np.zeros((M, N), dtype=np.float32)
    up = ctypes.POINTER(ctypes.c_uint16)
    check(lib().umwm_gpu_gemm_bf16(A.ctypes.data_as(up), B.ctypes.data_as(up), C.ctypes.data_as(_fp), M, N, K))
    return C
