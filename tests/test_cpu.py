"""CPU tests: the oracle, the host set-up of the library (no GPU needed),
the C ABI surface, the namelist rules and the workload generators."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# ---------------------------------------------------------------------------
# Known answers for the wet-point unrolling (umwm_init.F90:897-1014, serial
# remap_dir = 'v': m outer, n inner, sea points first, then land points),
# worked out by hand for a 5 x 4 regional grid whose edges are land.
# ---------------------------------------------------------------------------
KA_II = np.array([  # ii(m, n), m = 1..5 (rows), n = 1..4 (columns)
    [7, 8, 9, 10],
    [11, 1, 2, 12],
    [13, 3, 4, 14],
    [15, 5, 6, 16],
    [17, 18, 19, 20]])
# neighbours of the wet points i = 1..6: true (iis, iin, iiw, iie) and
# aliased to the ghost 0 when the neighbour is land (is, in, iw, ie)
KA_TRUE = {"iis": [11, 1, 13, 3, 15, 5], "iin": [2, 12, 4, 14, 6, 16],
           "iiw": [8, 9, 1, 2, 3, 4], "iie": [3, 4, 5, 6, 18, 19]}
KA_ALIAS = {"is": [0, 1, 0, 3, 0, 5], "in": [2, 0, 4, 0, 6, 0], "iw": [0, 0, 1, 2, 3, 4],
            "ie": [3, 4, 5, 6, 0, 0]}


def _ka_namelist():
    from umwm_gb300.namelist import make_namelist

    return make_namelist(mm=5, nm=4, xpl=2, ypl=2)


def test_known_answer_unrolling_oracle(oracle_mod):
    o = oracle_mod.Oracle(_ka_namelist(), 32)
    o.initialize()
    assert int(o.scalar("im")) == 6
    assert np.array_equal(o.get("ii"), KA_II)
    for k, v in KA_TRUE.items():
        assert list(o.get(k)[:6].astype(int)) == v, k
    for k, v in KA_ALIAS.items():
        assert list(o.get(k)[:6].astype(int)) == v, k


def test_known_answer_unrolling_library(lib_built):
    U = lib_built
    U.clear_inputs()
    U.setup_host(_ka_namelist())
    assert U.dims()["im"] == 6
    assert np.array_equal(U.get_field_i("ii"), KA_II)
    for k, v in KA_TRUE.items():
        assert list(U.get_field_i(k)[:6]) == v, k
    for k, v in KA_ALIAS.items():
        assert list(U.get_field_i(k)[:6]) == v, k


def _lake_case():
    """A basin with an enclosed lake (seeded fill) and a one-cell estuary."""
    from umwm_gb300 import configs
    from umwm_gb300.namelist import make_namelist

    mm, nm = 30, 24
    z = -np.full((mm, nm), 50.0, dtype=np.float32)
    z[10:20, 8:16] = 5.0        # island ...
    z[13:17, 11:13] = -20.0     # ... with a lake inside
    z[25:27, 5:19] = 3.0        # a two-cell wall with a one-cell dead-end inlet
    z[25, 12] = -15.0
    nml = make_namelist(mm=mm, nm=nm, topoFromFile=True, fillLakes=True, fillEstuaries=True, xpl=5, ypl=5)
    return configs.Case("lake", nml, "2012-01-01 00:00:00", "2012-01-01 01:00:00", gridtopo={"z": z}), [(14, 12)]


SETUP_INT = ["mask", "ii", "mi", "ni", "iw", "ie", "is", "in", "iiw", "iie", "iis", "iin"]
SETUP_FLT = ["ar", "dxn", "dxs", "dye", "dyw", "d", "k", "cp0", "cg0", "kdk", "k3dk", "k4", "cothkd", "sbf", "sdv",
             "logl2overz", "fkovg", "bf1_renorm", "bf2_renorm"]


def _setup_cases():
    from umwm_gb300 import configs

    lon = (-80 + 0.05 * np.arange(40)[:, None] + 0.002 * np.arange(36)[None, :]).astype(np.float32)
    lat = (20 + 0.05 * np.arange(36)[None, :] + 0.001 * np.arange(40)[:, None]).astype(np.float32)
    curv = configs.random_field(mm=40, nm=36, hours=1, gridFromFile=True)
    curv.gridtopo.update(lon=lon, lat=lat)
    lake, seeds = _lake_case()
    return {
        "reference_namelist": (configs.Case("ci", __import__("umwm_gb300.namelist", fromlist=["x"]).make_namelist(),
                                            "2012-01-01 00:00:00", "2012-01-01 06:00:00"), None),
        "random_field": (configs.random_field(mm=60, nm=50, hours=1), None),
        "global": (configs.random_field(mm=48, nm=40, hours=1, isGlobal=True), None),
        "estuaries": (configs.random_field(mm=48, nm=40, hours=1, fillEstuaries=True), None),
        "curvilinear": (curv, None),
        "lake": (lake, seeds),
    }


@pytest.mark.parametrize("name", ["reference_namelist", "random_field", "global", "estuaries", "curvilinear", "lake"])
def test_setup_bit_exact_vs_oracle(lib_built, oracle_mod, name):
    """Masks, unrolling, neighbours (bit-exact) and the spectral tables of the
    library's host set-up against the oracle on the same inputs."""
    U = lib_built
    case, seeds = _setup_cases()[name]
    U.clear_inputs()
    case.stage(U)
    if seeds:
        U.put_exclude(seeds)
    U.setup_host(case.nml)
    o = oracle_mod.Oracle(case.nml, 32)
    case.stage(o)
    if seeds:
        o.put_exclude(seeds)
    o.initialize()
    assert U.dims()["im"] == int(o.scalar("im"))
    for n in SETUP_INT:
        assert np.array_equal(U.get_field_i(n), o.get(n).astype(np.int32)), n
    for n in SETUP_FLT:
        assert np.array_equal(U.get_field(n), o.get(n).astype(np.float32)), n
    for n in ("dtamin", "cgmax", "dth"):
        assert U.get_field(n) == np.float32(o.scalar(n)), n
    assert np.array_equal(U.get_field("curv"), o.get("curv").astype(np.float32))


def test_lake_and_estuary_fill_applied(oracle_mod):
    case, seeds = _lake_case()
    o = oracle_mod.Oracle(case.nml, 32)
    case.stage(o)
    o.put_exclude(seeds)
    o.initialize()
    mask = o.get("mask")
    assert mask[13:17, 11:13].sum() == 0      # lake filled
    assert mask[25, 12] == 0                  # estuary cell filled
    assert mask[5, 5] == 1


# ---------------------------------------------------------------------------
# namelist rules, umwm_init.F90:94-185
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("kw,msg", [
    (dict(pm=30), "pm must be divisible by 4"),
    (dict(mm=2), "mm and nm must be > 2"),
    (dict(fmin=2.0, fmax=1.0), "fmin must be < fmax"),
    (dict(dtg=0), "dtg must be > 0"),
    (dict(outgrid=5), "outgrid"),
    (dict(dmin=-1), "dmin must be > 0"),
    (dict(gustiness=-0.1), "gustiness must be positive"),
])
def test_namelist_errors(lib_built, kw, msg):
    from umwm_gb300 import UmwmError
    from umwm_gb300.namelist import make_namelist

    with pytest.raises(UmwmError) as ei:
        lib_built.setup_host(make_namelist(**kw))
    assert ei.value.code == 1 and msg in str(ei.value)


def test_namelist_syntax_variants(lib_built):
    """Comments, upper/lower case, .TRUE./T logicals, Fortran d-exponents,
    comma-separated lists and a missing name (static storage zero)."""
    text = """! comment line
&domain
  ISGLOBAL = .false., MM = 12, nm=10 ! trailing comment
  om = 25, pm = 24, fmin = 3.13d-2, fmax = 2.0, fprog = 2.0
  startTimeStr = '2012-01-01 00:00:00', stopTimeStr = "2012-01-01 01:00:00"
  dtg = 3600, restart = F
/
&PHYSICS g=9.80665, nu_air=1.56E-5, nu_water=0.90E-6, sfct=0.07, kappa=0.4, z=10., gustiness=0.0,
  dmin=10., explim=0.9, sin_fac=0.11, sin_diss1=0.10, sin_diss2=0.001, sds_fac=42., sds_power=2.4,
  mss_fac=360, snl_fac=5.0, sdt_fac=0.002, sbf_fac=0.003, sbp_fac=0.003 /
&GRID gridFromFile=.F., delx=5000, dely=5000, topoFromFile=.F., dpt=200, fillEstuaries=.F., fillLakes=.F. /
&FORCING winds=.F., currents=.F., air_density=.F., water_density=.F., seaice=.F. /
&FORCING_CONSTANT wspd0=10, wdir0=0, uc0=0, vc0=0, rhoa0=1.2, rhow0=1030, fice0=0, fice_lth=0.3, fice_uth=0.75 /
&OUTPUT outgrid=0, outspec=0, outrst=0, xpl=4, ypl=4, stokes=.TRUE. /
&STOKES depths = 0.5, 1, 2,4 8 /
"""
    U = lib_built
    U.setup_host(text)
    d = U.dims()
    assert (d["mm"], d["nm"], d["om"], d["pm"], d["im"], d["lm"]) == (12, 10, 25, 24, 80, 5)
    f = U.get_field("f")
    assert abs(f[0] - 3.13e-2) < 1e-8 and abs(f[-1] - 2.0) < 1e-6
    assert np.allclose(U.get_field("depth"), [-0.5, -1, -2, -4, -8])
    assert abs(U.get_field("dth") - 2 * np.pi / 24) < 1e-6


def test_missing_group(lib_built):
    from umwm_gb300 import UmwmError
    from umwm_gb300.namelist import make_namelist

    text = make_namelist().replace("&STOKES", "&NOTSTOKES")
    with pytest.raises(UmwmError) as ei:
        lib_built.setup_host(text)
    assert ei.value.code == 1 and "stokes" in str(ei.value)


def test_input_argument_errors(lib_built):
    from umwm_gb300 import UmwmError

    U = lib_built
    with pytest.raises(UmwmError) as ei:
        U.put_forcing("2012-13-01 00:00:00", "uw", np.zeros((4, 4)))
    assert ei.value.code == 7
    with pytest.raises(UmwmError):
        U.put_forcing("2012-01-01 00:00:00", "wind", np.zeros((4, 4)))
    with pytest.raises(UmwmError):
        U.put_gridtopo("depth", np.zeros((4, 4)))
    # topoFromFile without a staged 'z' is an input error, like a missing file
    from umwm_gb300.namelist import make_namelist

    U.clear_inputs()
    with pytest.raises(UmwmError) as ei:
        U.setup_host(make_namelist(topoFromFile=True))
    assert ei.value.code == 2


# ---------------------------------------------------------------------------
# C ABI surface
# ---------------------------------------------------------------------------
def test_c_abi_exports(lib_built):
    """Every entry point declared in include/umwm_gpu.h is exported by the
    library and bound by the Python package."""
    import umwm_gb300

    hdr = open(os.path.join(ROOT, "include", "umwm_gpu.h")).read()
    declared = sorted(set(re.findall(r"\b(umwm_gpu_\w+)\s*\(", hdr)))
    assert declared == sorted(umwm_gb300.EXPORTS)
    L = umwm_gb300.lib()
    for name in declared:
        assert hasattr(L, name), name
    assert L.umwm_gpu_last_error() is not None


def test_run_before_initialize(lib_built):
    from umwm_gb300 import UmwmError

    lib_built.umwm_finalize()
    with pytest.raises(UmwmError) as ei:
        lib_built.umwm_run("2012-01-01 00:00:00", "2012-01-01 01:00:00")
    assert ei.value.code == 6


# ---------------------------------------------------------------------------
# oracle
# ---------------------------------------------------------------------------
def test_oracle_fp32_vs_fp64_reference_namelist(oracle_mod):
    """The shipped namelist over 6 h: the fp32 and fp64 restatements agree."""
    from umwm_gb300.namelist import make_namelist

    nml = make_namelist()
    r = {}
    for prec in (32, 64):
        o = oracle_mod.Oracle(nml, prec)
        o.initialize()
        o.run("2012-01-01 00:00:00", "2012-01-01 06:00:00")
        r[prec] = o
    a, b = r[32].get("screen"), r[64].get("screen")
    assert a.shape == b.shape and a.shape[0] == 223
    assert np.abs(a[:, 4] - b[:, 4]).max() / b[:, 4].max() < 1e-5       # Hs at the print point
    hs32, hs64 = r[32].get("ht"), r[64].get("ht")
    assert np.abs(hs32 - hs64).max() / hs64.max() < 1e-5
    assert (r[32].get("e") >= 0).all()


def test_oracle_first_step_is_zero_without_restart(oracle_mod):
    """Without a restart the first substep integrates with dts = 0
    (umwm_physics.F90:53); with one it does not."""
    from umwm_gb300 import configs
    from umwm_gb300.namelist import make_namelist

    o = oracle_mod.Oracle(make_namelist(), 32)
    o.initialize()
    o.set_option("max_substeps", 1)
    o.run("2012-01-01 00:00:00", "2012-01-01 06:00:00")
    assert o.scalar("dts") == 0.0
    case = configs.fetch_limited(mm=12, nm=10, hours=1)
    o = oracle_mod.Oracle(case.nml, 32)
    case.stage(o)
    o.initialize()
    o.set_option("max_substeps", 1)
    o.run(case.start, case.stop)
    assert o.scalar("dts") > 0.0


def test_oracle_uniform_depth_no_refraction(oracle_mod):
    """Uniform depth and no currents: the rotation rate is zero everywhere,
    so refraction leaves the spectrum unchanged (dtr falls back to dts)."""
    from umwm_gb300 import configs

    case = configs.fetch_limited(mm=16, nm=12, hours=1)
    o = oracle_mod.Oracle(case.nml, 32)
    case.stage(o)
    o.initialize()
    o.set_option("max_substeps", 2)
    o.run(case.start, case.stop)
    assert np.abs(o.get("rotl")).max() == 0.0 and np.abs(o.get("rotr")).max() == 0.0
    assert o.scalar("dtr_temp") == o.scalar("dts") or o.scalar("substeps") >= 1


def test_oracle_gustiness_draws(oracle_mod):
    """Wind gustiness in the oracle (umwm_forcing.F90:49-61): the seeded
    gust draws repeat for the same seed, change with it, and perturb the
    wind within the gustiness bound."""
    from umwm_gb300 import configs

    # gusts apply to forcing winds (winds = .true.), as in the reference
    case = configs.random_field(mm=48, nm=40, hours=1, dx=2000.0, gustiness=0.1)

    def run(seed, gust=True):
        c = case if gust else configs.random_field(mm=48, nm=40, hours=1, dx=2000.0)
        o = oracle_mod.Oracle(c.nml, 32)
        c.stage(o)
        o.initialize()
        o.set_option("gust_seed", seed)
        o.set_option("max_substeps", 2)
        o.run(c.start, c.stop)
        return o.get("wspd"), o.get("e")

    w7, e7 = run(7)
    w7b, e7b = run(7)
    w8, e8 = run(8)
    w0, _ = run(7, gust=False)
    assert np.array_equal(w7, w7b) and np.array_equal(e7, e7b)
    assert not np.array_equal(w7, w8) and not np.array_equal(e7, e8)
    ratio = w7 / w0
    assert np.abs(ratio - 1).max() <= 0.1 * np.sqrt(2) + 1e-6  # |1 + gu|, |1 + gv| within 1 +- 0.1
    assert np.abs(ratio - 1).max() > 0.02


def test_oracle_restart_roundtrip(oracle_mod):
    """A restart staged at the start time is read into e and ustar."""
    from umwm_gb300 import configs

    case = configs.fetch_limited(mm=12, nm=10, hours=1)
    o = oracle_mod.Oracle(case.nml, 32)
    case.stage(o)
    o.initialize()
    o.set_option("max_substeps", 0)
    o.run(case.start, case.stop)
    assert np.array_equal(o.get("e").astype(np.float32), case.restart[1])
    assert np.array_equal(o.get("ustar").astype(np.float32), case.restart[2])


# ---------------------------------------------------------------------------
# workload generators
# ---------------------------------------------------------------------------
def test_jonswap_normalisation(oracle_mod):
    """The restart spectrum gives the requested Hs with the reference's Hs
    formula 4 sqrt(sum e kdk dth) (umwm_physics.F90:148-154)."""
    from umwm_gb300 import configs

    case = configs.fetch_limited(mm=12, nm=10, hours=1, hs=0.1)
    o = oracle_mod.Oracle(case.nml, 64)
    case.stage(o)
    o.initialize()
    kdk = o.get("kdk")  # (im, om)
    F = case.restart[1].astype(np.float64)  # (im, pm, om)
    hs = 4 * np.sqrt((F * kdk[:, None, :]).sum(axis=(1, 2)) * o.scalar("dth"))
    assert np.abs(hs - 0.1).max() < 0.002  # 1 % noise on the bins


def test_random_field_statistics():
    from umwm_gb300 import configs

    c = configs.random_field(mm=200, nm=200, hours=1)
    z = c.gridtopo["z"]
    land = (z >= 0).mean()
    assert 0.15 < land < 0.3
    d = -z[z < 0]
    assert d.min() >= 10.0 and d.max() <= 5000.0
    f = c.forcing[c.start]
    sp = np.hypot(f["uw"], f["vw"])
    assert sp.max() <= 25.0 + 1e-4 and sp.min() >= 0.0
    assert np.hypot(f["uc"], f["vc"]).max() <= 1.0 + 1e-6
    assert c.restart[1].shape == (c.meta["im"], 36, 37)


def test_hurricane_forcing():
    from umwm_gb300 import configs

    c = configs.hurricane(mm=80, nm=80, hours=1, dx=4000.0, dtg=600)
    assert len(c.forcing) == 7
    sp = max(np.hypot(v["uw"], v["vw"]).max() for v in c.forcing.values())
    assert 45.0 < sp < 56.0
    z = c.gridtopo["z"]
    assert -z.min() < 3000 * 1.06 and -z.max() > 20 * 0.94
