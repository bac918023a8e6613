"""Writer of main.nml text (the namelist format read by umwm_init.F90:56-193
and umwm_stokes.F90:25-34) from a dict of values.

DEFAULTS are the values of the namelist shipped with the reference
(namelists/main.nml); any key can be overridden.
"""

GROUPS = {
    "DOMAIN": ["isGlobal", "mm", "nm", "om", "pm", "fmin", "fmax", "fprog", "startTimeStr", "stopTimeStr", "dtg",
               "restart"],
    "PHYSICS": ["g", "nu_air", "nu_water", "sfct", "kappa", "z", "gustiness", "dmin", "explim", "sin_fac",
                "sin_diss1", "sin_diss2", "sds_fac", "sds_power", "mss_fac", "snl_fac", "sdt_fac", "sbf_fac",
                "sbp_fac"],
    "GRID": ["gridFromFile", "delx", "dely", "topoFromFile", "dpt", "fillEstuaries", "fillLakes"],
    "FORCING": ["winds", "currents", "air_density", "water_density", "seaice"],
    "FORCING_CONSTANT": ["wspd0", "wdir0", "uc0", "vc0", "rhoa0", "rhow0", "fice0", "fice_lth", "fice_uth"],
    "OUTPUT": ["outgrid", "outspec", "outrst", "xpl", "ypl", "stokes"],
    "STOKES": ["depths"],
}

DEFAULTS = {
    "isGlobal": False, "mm": 21, "nm": 11, "om": 37, "pm": 36, "fmin": 0.0313, "fmax": 2.0, "fprog": 2.0,
    "startTimeStr": "2012-01-01 00:00:00", "stopTimeStr": "2012-01-01 06:00:00", "dtg": 3600, "restart": False,
    "g": 9.80665, "nu_air": 1.56e-5, "nu_water": 0.90e-6, "sfct": 0.07, "kappa": 0.4, "z": 10.0,
    "gustiness": 0.0, "dmin": 10.0, "explim": 0.9, "sin_fac": 0.11, "sin_diss1": 0.10, "sin_diss2": 0.001,
    "sds_fac": 42.0, "sds_power": 2.4, "mss_fac": 360, "snl_fac": 5.0, "sdt_fac": 0.002, "sbf_fac": 0.003,
    "sbp_fac": 0.003,
    "gridFromFile": False, "delx": 10000, "dely": 10000, "topoFromFile": False, "dpt": 1000,
    "fillEstuaries": False, "fillLakes": False,
    "winds": False, "currents": False, "air_density": False, "water_density": False, "seaice": False,
    "wspd0": 10, "wdir0": 0, "uc0": 0, "vc0": 0, "rhoa0": 1.2, "rhow0": 1030, "fice0": 0.0, "fice_lth": 0.30,
    "fice_uth": 0.75,
    "outgrid": 1, "outspec": 0, "outrst": 6, "xpl": 20, "ypl": 6, "stokes": True,
    "depths": [0.1, 0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 1.0, 1.2, 1.4, 1.6, 1.8, 2.0, 2.4, 2.8, 3.2, 3.6, 4.0,
               4.5, 5.0, 6, 7, 8, 9, 10, 12, 14, 16, 18, 20, 24, 28, 32, 40, 50, 60, 70, 80, 90, 100],
}


def _fmt(v):
    if isinstance(v, bool):
        return ".T." if v else ".F."
    if isinstance(v, str):
        return "'%s'" % v
    if isinstance(v, (list, tuple)):
        return " ".join(_fmt(x) for x in v)
    if isinstance(v, float):
        return repr(v)
    return str(v)


def make_namelist(**overrides):
    vals = dict(DEFAULTS)
    lower = {k.lower(): k for k in vals}
    for k, v in overrides.items():
        vals[lower.get(k.lower(), k)] = v
    lines = []
    for g, keys in GROUPS.items():
        lines.append("&" + g)
        for k in keys:
            lines.append("  %-14s = %s" % (k, _fmt(vals[k])))
        lines.append("/")
    return "\n".join(lines) + "\n"
