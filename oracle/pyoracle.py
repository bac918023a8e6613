"""ctypes wrapper of the oracle (CPU restatement of the reference path).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline legs, never by the umwm_gb300 package.

Parity unpinned: the reference ships no golden vectors; the oracle follows
its source line by line (see oracle/umwm_oracle.cpp).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {}


def build(quiet=True):
    """Compile oracle/_build/liboracle.so (and the timing-only
    liboracle_fast.so) with the committed Makefile."""
    out = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return os.path.join(_HERE, "_build", "liboracle.so")


def lib(fast=False):
    """The strict oracle, or (fast=True) the same source built with the
    reference's production flags, for timing only."""
    if fast not in _LIBS:
        path = os.path.join(_HERE, "_build", "liboracle_fast.so" if fast else "liboracle.so")
        src = os.path.join(_HERE, "umwm_oracle.cpp")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        L = ctypes.CDLL(path)
        L.oracle_new.restype = ctypes.c_void_p
        L.oracle_new.argtypes = [ctypes.c_int, ctypes.c_char_p]
        L.oracle_free.argtypes = [ctypes.c_void_p]
        L.oracle_error.restype = ctypes.c_char_p
        L.oracle_error.argtypes = [ctypes.c_void_p]
        fp = ctypes.POINTER(ctypes.c_float)
        L.oracle_put_gridtopo.argtypes = [ctypes.c_void_p, ctypes.c_char_p, fp, ctypes.c_long]
        L.oracle_put_exclude.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int]
        L.oracle_put_forcing.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, fp, ctypes.c_long]
        L.oracle_put_restart.argtypes = [ctypes.c_void_p, ctypes.c_char_p, fp, ctypes.c_long, fp, ctypes.c_long]
        L.oracle_set_option.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_double]
        L.oracle_initialize.argtypes = [ctypes.c_void_p]
        L.oracle_run.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p]
        L.oracle_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double), ctypes.c_long]
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_set_threads.restype = ctypes.c_int
        _LIBS[fast] = L
    return _LIBS[fast]


def set_threads(n, fast=False):
    return lib(fast).oracle_set_threads(int(n))


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _fortran_2d(field_mn):
    """(mm, nm) array -> flat Fortran order (m fastest)."""
    a = np.asarray(field_mn, dtype=np.float32)
    return _f32(a.ravel(order="F"))


class Oracle:
    """One model instance of the oracle; prec is 32 or 64.  fast=True loads
    the timing-only build (the reference's production flags)."""

    def __init__(self, nml_text, prec=32, fast=False):
        self.L = lib(fast)
        self.prec = prec
        self.h = self.L.oracle_new(int(prec), nml_text.encode())

    def __del__(self):
        try:
            if self.h:
                self.L.oracle_free(self.h)
                self.h = None
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("oracle %s failed: %s" % (what, self.L.oracle_error(self.h).decode()))

    def put_gridtopo(self, var, field_mn):
        a = _fortran_2d(field_mn)
        self.L.oracle_put_gridtopo(self.h, var.encode(), a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), a.size)

    def put_exclude(self, pairs):
        a = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).ravel())
        self.L.oracle_put_exclude(self.h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(a) // 2)

    def put_forcing(self, time19, var, field_mn):
        a = _fortran_2d(field_mn)
        self.L.oracle_put_forcing(self.h, time19.encode(), var.encode(),
                                  a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), a.size)

    def put_restart(self, time19, e_ipo, ust):
        """e_ipo: array (im, pm, om) in C order == reference F(om, pm, im)."""
        e = _f32(e_ipo).ravel()
        u = _f32(ust).ravel()
        fp = ctypes.POINTER(ctypes.c_float)
        self.L.oracle_put_restart(self.h, time19.encode(), e.ctypes.data_as(fp), e.size, u.ctypes.data_as(fp), u.size)

    def set_option(self, name, value):
        self._check(self.L.oracle_set_option(self.h, name.encode(), float(value)), "set_option")

    def initialize(self):
        self._check(self.L.oracle_initialize(self.h), "initialize")

    def run(self, start, stop):
        self._check(self.L.oracle_run(self.h, start.encode(), stop.encode()), "run")

    def scalar(self, name):
        out = np.zeros(1, dtype=np.float64)
        self._check(self.L.oracle_get(self.h, name.encode(), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1),
                    "get " + name)
        return float(out[0])

    def dims(self):
        return {k: int(self.scalar(k)) for k in ("mm", "nm", "om", "pm", "im", "imm", "lm")}

    _WET = {"ar", "cd", "dxn", "dxs", "dye", "dyw", "fcutoff", "oneovar", "oneovdx", "oneovdy", "shelt",
            "physics_time_step", "ustar", "taux", "tauy", "taux_form", "tauy_form", "taux_skin", "tauy_skin",
            "taux_diag", "tauy_diag", "tailatmx", "tailatmy", "ht", "mss", "mwd", "mwl", "mwp", "dwd", "dwl",
            "dwp", "dcp0", "dcp", "dcg0", "dcg", "momx", "momy", "cgmxx", "cgmxy", "cgmyy", "ds", "oc",
            "taux_ocntop", "tauy_ocntop", "taux_ocnbot", "tauy_ocnbot", "taux_snl", "tauy_snl", "epsx_ocn",
            "epsy_ocn", "epsx_atm", "epsy_atm", "tailocnx", "tailocny", "taux1", "tauy1", "taux2", "tauy2",
            "taux3", "tauy3"}
    _IMM = {"mi", "ni", "iw", "ie", "is", "in", "iiw", "iie", "iis", "iin", "d", "dx", "dy", "wspd", "wdir",
            "uc", "vc", "rhoa", "rhow", "rhorat", "fice"}
    _TWOD = {"ii", "mask", "d_2d", "dx_2d", "dy_2d", "curv"}
    _OI = {"k", "bf1_renorm", "bf2_renorm", "cothkd", "dwn", "fkovg", "invcp0", "k4", "kdk", "k3dk",
           "oneoverk4", "sbf", "sdt", "sdv", "snl_arg", "l2", "logl2overz", "sice"}
    _OI_GHOST = {"cp0", "cg0"}
    _OPI = {"e", "ef", "dummy", "rotl", "rotr", "sds", "snl", "ssin"}

    def get(self, name):
        d = self.dims()
        om, pm, im, imm, lm, mm, nm = d["om"], d["pm"], d["im"], d["imm"], d["lm"], d["mm"], d["nm"]
        if name in self._WET:
            shape = (im,)
        elif name in self._IMM:
            shape = (imm,)
        elif name in self._TWOD:
            shape = (nm, mm)  # Fortran (mm, nm) -> C (nm, mm)
        elif name in self._OI:
            shape = (im, om)
        elif name in self._OI_GHOST:
            shape = (im + 1, om)
        elif name in self._OPI:
            shape = (im, pm, om)
        elif name in ("us", "vs"):
            shape = (lm, im)
        elif name == "f":
            shape = (om,)
        elif name == "th":
            shape = (pm,)
        elif name == "depth":
            shape = (lm,)
        elif name == "screen":
            shape = (int(self.scalar("substeps")), 8)
        else:
            return self.scalar(name)
        out = np.zeros(int(np.prod(shape)) if shape else 1, dtype=np.float64)
        if out.size == 0:
            return out.reshape(shape)
        self._check(self.L.oracle_get(self.h, name.encode(), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                      out.size), "get " + name)
        out = out.reshape(shape)
        if name in self._TWOD:
            out = out.T  # back to (mm, nm)
        return out
