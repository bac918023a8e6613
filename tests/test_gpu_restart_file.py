"""Restart files in the reference's netCDF layout (umwm_restart.F90:19-154).

The file the library writes is read back with scipy's netCDF-3 reader, an
implementation independent of the library's writer, and compared with the
state read through the C ABI.  A second model then starts from that file
(restart = .true., nothing staged) and must hold the same state.  The
namelist's outrst makes umwm_run write the file at full hours.
"""
import os
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_restart_file_roundtrip(lib_built, tmp_path, monkeypatch):
    scipy_io = pytest.importorskip("scipy.io")
    from umwm_gb300 import configs

    U = lib_built
    monkeypatch.chdir(tmp_path)
    os.makedirs("restart")
    case = configs.fetch_limited(mm=24, nm=14, hours=2)
    U.clear_inputs()
    case.stage(U)
    nml = re.sub(r"outrst\s*=\s*\d+", "outrst = 1", case.nml)
    U.umwm_initialize(nml_text=nml)
    U.umwm_run(case.start, case.stop)
    F, ust = U.get_state()
    k = U.get_field("k")
    U.write_restart("restart/explicit.nc")
    U.umwm_finalize()

    with scipy_io.netcdf_file("restart/explicit.nc", "r", mmap=False) as f:
        assert f.dimensions["x"] == F.shape[0] and f.dimensions["f"] == 37 and f.dimensions["th"] == 36
        np.testing.assert_array_equal(f.variables["F"][:], F)
        np.testing.assert_array_equal(f.variables["ust"][:], ust)
        np.testing.assert_array_equal(f.variables["wavenumber"][:], k)
        assert f.variables["F"].units == b"m^4 rad^-1"
        assert f.variables["ust"].description == b"friction velocity"

    # namelist-driven output at the full hours of the run
    stop_key = case.stop.replace(" ", "_")
    assert os.path.exists("restart/umwmrst_%s.nc" % stop_key)

    # a new model restarting from the file at the stop time
    os.replace("restart/explicit.nc", "restart/umwmrst_%s.nc" % stop_key)
    U.clear_inputs()
    case.stage(U)
    U.clear_inputs()  # drop the staged restart: the file must be read
    for t, vars_ in case.forcing.items():
        for var, fld in vars_.items():
            U.put_forcing(t, var, fld)
    for var, fld in (case.gridtopo or {}).items():
        U.put_gridtopo(var, fld)
    U.umwm_initialize(nml_text=nml)
    U.set_option("max_substeps", 0)
    U.umwm_run(case.stop, case.stop)
    F2, ust2 = U.get_state()
    U.umwm_finalize()
    np.testing.assert_array_equal(F2, F)
    np.testing.assert_array_equal(ust2, ust)


def test_input_files_match_staged_inputs(lib_built, tmp_path, monkeypatch):
    """Inputs not staged are read from the reference's files
    (input/umwm.gridtopo, input/umwmin_<time>.nc), written here with scipy's
    netCDF-3 writer: the run equals the run with the same fields staged."""
    scipy_io = pytest.importorskip("scipy.io")
    from umwm_gb300 import configs

    U = lib_built
    monkeypatch.chdir(tmp_path)
    os.makedirs("input")
    case = configs.hurricane(mm=40, nm=36, hours=1, dx=4000.0, dtg=600, seed=3)

    def staged():
        U.clear_inputs()
        case.stage(U)
        U.umwm_initialize(nml_text=case.nml)
        U.umwm_run(case.start, case.stop)
        out = U.get_field("ht"), U.get_state()[0]
        U.umwm_finalize()
        return out

    ht0, F0 = staged()
    mm, nm = case.meta["mm"], case.meta["nm"]
    with scipy_io.netcdf_file("input/umwm.gridtopo", "w") as f:
        f.createDimension("y", nm)
        f.createDimension("x", mm)
        v = f.createVariable("z", "f4", ("y", "x"))
        v[:] = case.gridtopo["z"].T
    for t, fields in case.forcing.items():
        with scipy_io.netcdf_file("input/umwmin_%s.nc" % t.replace(" ", "_"), "w") as f:
            f.createDimension("y", nm)
            f.createDimension("x", mm)
            for name, fld in fields.items():
                v = f.createVariable(name, "f4", ("y", "x"))
                v[:] = np.asarray(fld, np.float32).T
    U.clear_inputs()
    start, F, ust = case.restart
    U.put_restart(start, F, ust)  # the spectrum still staged; grid, depth and forcing from the files
    U.umwm_initialize(nml_text=case.nml)
    U.umwm_run(case.start, case.stop)
    ht1, F1 = U.get_field("ht"), U.get_state()[0]
    U.umwm_finalize()
    np.testing.assert_array_equal(ht1, ht0)
    np.testing.assert_array_equal(F1, F0)
