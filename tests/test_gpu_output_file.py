"""Gridded output in the reference's netCDF layout (umwm_io.F90:317-854).

The files the library writes are read back with scipy's netCDF-3 reader, an
implementation independent of the library's writer.  Each wet cell of a
variable must equal the wet-point field read through the C ABI at that
cell, land cells are NaN, and the variables come in the reference's order
with its descriptions and units.
"""
import datetime
import os
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# the reference's variable order after the Stokes drift (umwm_io.F90:360-633)
VARIABLES = [
    "frequency", "theta", "lon", "lat", "seamask", "depth", "wspd", "wdir", "uc", "vc", "rhoa", "rhow", "fice",
    "psim", "momx", "momy", "cgmxx", "cgmxy", "cgmyy", "shelt", "epsx_atm", "epsy_atm", "epsx_ocn", "epsy_ocn",
    "taux_form", "tauy_form", "taux_form_1", "tauy_form_1", "taux_form_2", "tauy_form_2", "taux_form_3",
    "tauy_form_3", "taux_skin", "tauy_skin", "taux_diag", "tauy_diag", "taux_ocn", "tauy_ocn", "taux_bot",
    "tauy_bot", "taux_snl", "tauy_snl", "tailatmx", "tailatmy", "tailocnx", "tailocny", "cd", "ust", "swh",
    "mss", "mwp", "mwl", "mwd", "dwp", "dwl", "dwd", "dcp0", "dcg0", "dcp", "dcg", "physics_time_step"]

# output variable -> wet-point field of the C ABI
WET = {"swh": "ht", "ust": "ustar", "cd": "cd", "mss": "mss", "mwp": "mwp", "mwd": "mwd", "dwp": "dwp",
       "momx": "momx", "cgmxy": "cgmxy", "taux_form": "taux_form", "taux_skin": "taux_skin",
       "taux_ocn": "taux_ocntop", "tauy_bot": "tauy_ocnbot", "taux_snl": "taux_snl", "epsx_atm": "epsx_atm",
       "epsy_ocn": "epsy_ocn", "taux_form_2": "taux2", "tailocnx": "tailocnx", "dcg": "dcg", "shelt": "shelt"}


def _case():
    from umwm_gb300 import configs

    case = configs.hurricane(mm=40, nm=36, hours=2, dx=4000.0, dtg=600, seed=3)
    nml = re.sub(r"outgrid\s*=\s*-?\d+", "outgrid = 1", case.nml)
    assert "outgrid = 1" in nml
    return case, nml


def test_output_grid_files(lib_built, tmp_path, monkeypatch):
    scipy_io = pytest.importorskip("scipy.io")
    U = lib_built
    monkeypatch.chdir(tmp_path)
    os.makedirs("output")
    case, nml = _case()
    U.clear_inputs()
    case.stage(U)
    U.umwm_initialize(nml_text=nml)
    U.umwm_run(case.start, case.stop)
    got = {v: U.get_field(w) for v, w in WET.items()}
    mask = U.get_field_i("mask")  # (mm, nm)
    ii = U.get_field_i("ii").T  # point number (1-based) of each cell, 0 on land, (nm, mm)
    d = U.dims()
    freq, theta = U.get_field("f"), U.get_field("th")
    stokes_u = U.get_field("us")  # (lm, im)
    U.write_output("explicit.nc")
    U.umwm_finalize()

    t0 = datetime.datetime.strptime(case.start, "%Y-%m-%d %H:%M:%S")
    keys = [(t0 + datetime.timedelta(hours=h)).strftime("%Y-%m-%d_%H:%M:%S") for h in range(3)]
    start_key, stop_key = keys[0], keys[-1]
    assert stop_key == case.stop.replace(" ", "_")
    # the start time (first substep) and each full hour of the 2-hour run
    assert sorted(os.listdir("output")) == ["umwmout_%s.nc" % k for k in keys]

    for path in ("output/umwmout_%s.nc" % stop_key, "explicit.nc"):
        with scipy_io.netcdf_file(path, "r", mmap=False) as f:
            assert f.dimensions["x"] == d["mm"] and f.dimensions["y"] == d["nm"]
            assert f.dimensions["f"] == d["om"] and f.dimensions["th"] == d["pm"]
            assert f.dimensions["time"] is None  # the record dimension
            sea = f.variables["seamask"][0]
            np.testing.assert_array_equal(sea, mask.T)
            wet = sea == 1
            # wet points are 1..im; boundary cells im+1..imm are not written
            np.testing.assert_array_equal(wet, (ii > 0) & (ii <= d["im"]))
            # the hurricane case has the Stokes drift on: z and its fields first
            assert f.dimensions["z"] == d["lm"] > 0
            assert list(f.variables) == ["z", "u_stokes", "v_stokes", "d_stokes"] + VARIABLES
            assert f.variables["u_stokes"].dimensions == ("time", "z", "y", "x")
            us = f.variables["u_stokes"][0]
            for lev in range(d["lm"]):
                np.testing.assert_array_equal(us[lev][wet], stokes_u[lev][ii[wet] - 1])
            assert f.variables["swh"].description == b"significant wave height"
            assert f.variables["swh"].units == b"m"
            assert f.variables["swh"].dimensions == ("time", "y", "x")
            assert f.variables["seamask"].typecode() == "i"
            for v, ref in got.items():
                a = f.variables[v][0]
                assert a.shape == (d["nm"], d["mm"])
                assert np.isnan(a[~wet]).all(), v
                np.testing.assert_array_equal(a[wet], ref[ii[wet] - 1], err_msg=v)
            np.testing.assert_array_equal(f.variables["frequency"][:], freq)
            np.testing.assert_array_equal(f.variables["theta"][:], theta)
            assert np.isfinite(f.variables["depth"][0][wet]).all()

    # the file written at the start time carries zero stress('ocn') fields
    with scipy_io.netcdf_file("output/umwmout_%s.nc" % start_key, "r", mmap=False) as f:
        sea = f.variables["seamask"][0] == 1
        assert (f.variables["taux_ocn"][0][sea] == 0).all()
        assert np.isfinite(f.variables["swh"][0][sea]).all()


def test_output_grid_needs_directory(lib_built, tmp_path, monkeypatch):
    """Without an output directory the run writes nothing and goes on, as
    the reference's failed nf90_create does."""
    U = lib_built
    monkeypatch.chdir(tmp_path)
    case, nml = _case()
    U.clear_inputs()
    case.stage(U)
    U.umwm_initialize(nml_text=nml)
    U.umwm_run(case.start, case.stop)
    ht = U.get_field("ht")
    U.umwm_finalize()
    assert not os.path.exists("output")
    assert np.isfinite(ht).all()


def test_output_spectrum_files(lib_built, tmp_path, monkeypatch):
    """output_spectrum_nc (umwm_io.F90:150-314): for each wet point listed in
    namelists/spectrum.nml a file output/umwmspc_<id>_<start>.nc gets one
    record at the start time and one per outspec hour: the spectrum and the
    last substep's Sin, Sds, Snl and Sdt at that point, equal to what the C
    ABI returns.  Points given by longitude/latitude take the nearest cell;
    land cells write nothing."""
    scipy_io = pytest.importorskip("scipy.io")
    from umwm_gb300 import configs

    U = lib_built
    monkeypatch.chdir(tmp_path)
    os.makedirs("output")
    os.makedirs("namelists")
    case = configs.hurricane(mm=40, nm=36, hours=2, dx=4000.0, dtg=600, seed=3, outspec=1, outgrid=0)
    U.clear_inputs()
    case.stage(U)
    U.umwm_initialize(nml_text=case.nml)
    d = U.dims()
    ii = U.get_field_i("ii")  # (mm, nm), point number or 0
    cells = [(m, n) for n in range(2, d["nm"]) for m in range(2, d["mm"])
             if 1 <= ii[m - 1, n - 1] <= d["im"]]
    wet1, wet2 = cells[len(cells) // 3], cells[2 * len(cells) // 3]
    land = [(m, n) for n in range(2, d["nm"]) for m in range(2, d["mm"]) if ii[m - 1, n - 1] == 0]
    lines = ["XY", "%d %d p1" % wet1, "%d %d p2" % wet2] + (["%d %d dry" % land[0]] if land else [])
    with open("namelists/spectrum.nml", "w") as f:
        f.write("\n".join(lines) + "\n")
    U.umwm_run(case.start, case.stop)
    lon, lat = U.get_field("lon"), U.get_field("lat")  # (mm, nm)
    F, _ = U.get_state()
    src = {v: U.get_field(v) for v in ("ssin", "sds", "snl")}
    k, sdv, sbf = U.get_field("k"), U.get_field("sdv"), U.get_field("sbf")
    wspd, wdir = U.get_field("wspd"), U.get_field("wdir")
    U.umwm_finalize()

    key = case.start.replace(" ", "_")
    assert sorted(os.listdir("output")) == ["umwmspc_p1_%s.nc" % key, "umwmspc_p2_%s.nc" % key]
    for pid, (m, n) in (("p1", wet1), ("p2", wet2)):
        i = ii[m - 1, n - 1] - 1
        with scipy_io.netcdf_file("output/umwmspc_%s_%s.nc" % (pid, key), "r", mmap=False) as f:
            assert list(f.variables) == ["frequency", "wavenumber", "direction", "longitude", "latitude", "wspd",
                                         "wdir", "F", "Sin", "Sds", "Sdt", "Sdv", "Sbf", "Snl"]
            assert f.dimensions["time"] is None and f.variables["F"].shape == (3, d["pm"], d["om"])
            np.testing.assert_array_equal(f.variables["F"][-1], F[i])
            np.testing.assert_array_equal(f.variables["Sin"][-1], src["ssin"][i])
            np.testing.assert_array_equal(f.variables["Sds"][-1], src["sds"][i])
            np.testing.assert_array_equal(f.variables["Snl"][-1], src["snl"][i])
            np.testing.assert_array_equal(f.variables["wavenumber"][:], k[i])
            np.testing.assert_array_equal(f.variables["Sdv"][:], sdv[i])
            np.testing.assert_array_equal(f.variables["Sbf"][:], sbf[i])
            np.testing.assert_array_equal(f.variables["wspd"][-1], [wspd[i]])
            np.testing.assert_array_equal(f.variables["wdir"][-1], [wdir[i]])
            sdt = f.variables["Sdt"][:]  # sdt_fac sqrt(rhorat) u* k: proportional to k
            r = sdt / k[i][None, :]
            assert np.all(r > 0) and np.allclose(r, r[:, :1], rtol=1e-6)
            # the records differ in time: the start, +1 h, +2 h
            assert not np.array_equal(f.variables["F"][0], f.variables["F"][2])

    # on this Cartesian grid lon = lat = 0 (umwm_init.F90:524), so a point
    # given by longitude/latitude falls on the first cell, a boundary cell:
    # no file, as in the reference
    os.remove("output/umwmspc_p1_%s.nc" % key)
    os.remove("output/umwmspc_p2_%s.nc" % key)
    with open("namelists/spectrum.nml", "w") as f:
        f.write("LL\n%.6f %.6f q0\n" % (0.0, 0.0))
    U.clear_inputs()
    case.stage(U)
    U.umwm_initialize(nml_text=case.nml)
    U.set_option("max_substeps", 1)
    U.umwm_run(case.start, case.stop)
    U.umwm_finalize()
    assert os.listdir("output") == []

    # on a lon/lat grid the nearest cell
    from helpers import lonlat_grid

    case = configs.random_field(mm=40, nm=36, hours=1, gridFromFile=True, outspec=1, outgrid=0)
    lon, lat = lonlat_grid(40, 36)
    case.gridtopo["lon"] = lon
    case.gridtopo["lat"] = lat
    U.clear_inputs()
    case.stage(U)
    U.umwm_initialize(nml_text=case.nml)
    ii = U.get_field_i("ii")
    m, n = next((m, n) for n in range(10, 30) for m in range(10, 30) if 1 <= ii[m - 1, n - 1] <= U.dims()["im"])
    glon, glat = U.get_field("lon"), U.get_field("lat")
    with open("namelists/spectrum.nml", "w") as f:
        f.write("LL\n%.6f %.6f q1\n" % (glon[m - 1, n - 1] + 1e-4, glat[m - 1, n - 1] - 1e-4))
    U.set_option("max_substeps", 1)
    U.umwm_run(case.start, case.stop)
    U.umwm_finalize()
    key = case.start.replace(" ", "_")
    with scipy_io.netcdf_file("output/umwmspc_q1_%s.nc" % key, "r", mmap=False) as f:
        assert f.variables["longitude"][0] == glon[m - 1, n - 1]
        assert f.variables["latitude"][0] == glat[m - 1, n - 1]
        assert f.variables["F"].shape[0] == 1
