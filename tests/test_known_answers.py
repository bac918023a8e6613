"""Known answers that pin the oracle (and the library) to the mathematics of
the reference's formulas, with expected values worked out here independently
of the restatement in oracle/umwm_oracle.cpp:

* linear dispersion with surface tension, omega^2 = (g k + sfct/rhow k^3)
  tanh(k d) (umwm_init.F90:1436-1476): the exact root (bracketing solve in
  float64) and the group velocity d omega / d k by central differences;
* the COARE 3.5 sheltering fit (umwm_sheltering.F90:49-79) from its
  construction: a line from the intercept through (x1, y1), a parabola with
  the same value and slope at x1 whose curvature is 0.65 of the change of
  secant slopes over [x1, x2], and exponential decay from its value at x2;
* Sds of a two-bin spectrum (umwm_source_functions.F90:85-105, :174-176): the
  mean-square-slope factor of the upper bin is (1 + mss_fac E1 cos^2(dtheta)
  dth k^3 dk)^2 from the lower bin alone; and its Snl (:156-171): each bin
  loses snl_fac Sds e and hands the renormalised bf1, bf2 shares one and two
  levels down;
* the monochromatic deep-water Stokes drift u_s(z) = omega k a^2 e^{2kz}
  (umwm_stokes.F90:55-101) summed over the bins of the spectrum, with a^2
  twice each bin's variance, and the e-folding depth 1/(2k) below the first
  level (umwm_stokes.F90:104-128);
* the unrolling of a periodic (global) grid worked out by hand
  (umwm_init.F90:897-1007);
* one first-order upwind step of a step function in x: the front cell gets
  CFL times the upstream energy (umwm_advection.F90:30-97).

CPU tests run the oracle and the library's host set-up; the GPU tests
(marked gpu) run the same cases through the CUDA path."""
import numpy as np
import pytest
from scipy.optimize import brentq

G = 9.80665
SFCT, RHOW = 0.07, 1030.0


# ---------------------------------------------------------------------------
# independent dispersion relation
# ---------------------------------------------------------------------------
def omega_of_k(k, d):
    return np.sqrt((G * k + SFCT / RHOW * k ** 3) * np.tanh(k * d))


def exact_k(f, d):
    """Root of omega(k) = 2 pi f (float64, bracketed)."""
    w = 2 * np.pi * f
    lo = 1e-12
    hi = 2.0 * max(w * w / G, w / np.sqrt(G * d)) + 1.0
    return brentq(lambda k: omega_of_k(k, d) - w, lo, hi, xtol=1e-15, rtol=1e-15, maxiter=500)


def exact_cg(k, d):
    h = 1e-6 * k
    return (omega_of_k(k + h, d) - omega_of_k(k - h, d)) / (2 * h)


def freqs(om=37, fmin=0.0313, fmax=2.0):
    dlnf = (np.log(fmax) - np.log(fmin)) / (om - 1)
    return np.exp(np.log(fmin) + np.arange(om) * dlnf), dlnf


def _uniform_case(depth, wspd=10.0, mm=6, nm=5, **kw):
    from umwm_gb300 import configs

    return configs.fetch_limited(mm=mm, nm=nm, hours=1, depth=depth, wspd=wspd, **kw)


DEPTHS = [10.0, 50.0, 1000.0, 5000.0]


def _check_dispersion(k, cp0, cg0, d):
    """k, cp0, cg0: (om,) of one wet point at depth d."""
    f, _ = freqs(len(k))
    ke = np.array([exact_k(x, d) for x in f])
    # the reference's Newton iteration stops once its step in k d is below
    # 1e-2; the error left is second order in that step
    assert np.all(np.abs(k - ke) * d <= 2e-4 + 2e-6 * ke * d), np.max(np.abs(k - ke) * d)
    np.testing.assert_allclose(cp0, 2 * np.pi * f / k, rtol=2e-6)
    # group velocity d omega / d k of the exact curve; the stopped Newton
    # iteration's error in k carries over to cg at most about one for one
    cge = np.array([exact_cg(x, d) for x in ke])
    rk = np.abs(k - ke) / ke
    assert np.all(np.abs(cg0 - cge) / cge <= 2 * rk + 2e-5), np.max(np.abs(cg0 - cge) / cge)


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("depth", DEPTHS)
def test_dispersion_oracle(oracle_mod, depth, prec):
    o = oracle_mod.Oracle(_uniform_case(depth).nml, prec)
    o.initialize()
    _check_dispersion(o.get("k")[0], o.get("cp0")[1], o.get("cg0")[1], depth)


@pytest.mark.parametrize("depth", DEPTHS)
def test_dispersion_library(lib_built, depth):
    U = lib_built
    U.clear_inputs()
    U.setup_host(_uniform_case(depth).nml)
    _check_dispersion(U.get_field("k")[0].astype(np.float64), U.get_field("cp0")[1].astype(np.float64),
                      U.get_field("cg0")[1].astype(np.float64), depth)


# ---------------------------------------------------------------------------
# sheltering coefficient from the construction of the fit
# ---------------------------------------------------------------------------
def shelter_expected(w):
    x1, x2, y1, y2, x3, y3 = 15.0, 33.0, 0.10, 0.09, 60.0, 0.06
    intercept, curvature, decay = 0.04, 0.65, 1.6
    s_lo = (y1 - intercept) / x1                # line from the intercept through (x1, y1)
    s_hi = (y3 - y2) / (x3 - x2)                # secant slope of the upper range
    c = curvature * (s_hi - s_lo) / (x2 - x1)   # curvature of the middle parabola
    par = lambda x: y1 + s_lo * (x - x1) + c * (x - x1) ** 2  # value and slope of the line at x1
    if w <= x1:
        return intercept + s_lo * w
    if w <= x2:
        return par(w)
    return par(x2) * np.exp(-(w - x2) / (decay * w))


# wind speeds at the fit's joints and inside each range (0 m/s is clamped to
# 0.01 by sin_d12, umwm_source_functions.F90:22)
WINDS = [0.0, 10.0, 15.0, 24.0, 33.0, 45.0, 60.0]


def test_shelter_known_values():
    assert shelter_expected(15.0) == pytest.approx(0.10, abs=1e-15)
    assert shelter_expected(33.0) == pytest.approx(0.10 + 18 * (0.004 + 0.65 * (-0.03 / 27 - 0.004)), abs=1e-15)


@pytest.mark.parametrize("wspd", WINDS)
def test_shelter_oracle(oracle_mod, wspd):
    case = _uniform_case(1000.0, wspd=wspd)
    o = oracle_mod.Oracle(case.nml, 32)
    case.stage(o)
    o.initialize()
    o.set_option("max_substeps", 1)
    o.run(case.start, case.stop)
    np.testing.assert_allclose(o.get("shelt"), shelter_expected(max(wspd, 0.01)), rtol=2e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("wspd", WINDS)
def test_shelter_gpu(lib_built, wspd):
    from helpers import run_gpu

    U = lib_built
    run_gpu(U, _uniform_case(1000.0, wspd=wspd), max_substeps=1)
    np.testing.assert_allclose(U.get_field("shelt"), shelter_expected(max(wspd, 0.01)), rtol=2e-6)
    U.umwm_finalize()


# ---------------------------------------------------------------------------
# Sds of a two-bin spectrum
# ---------------------------------------------------------------------------
O1, P1, E1 = 9, 17, 2.0e4    # lower bin (0-based o, p) and its energy
O2, P2, E2 = 19, 20, 0.1     # upper bin: three directions (30 degrees) away
SDS_DEPTH = 1000.0


def _two_bin_case():
    from umwm_gb300 import configs

    case = configs.fetch_limited(mm=6, nm=5, hours=1, depth=SDS_DEPTH, wspd=5.0)
    t, F, u = case.restart
    F = np.full_like(F, np.finfo(np.float32).tiny)   # tiny(e) elsewhere, as the reference's init
    F[:, P1, O1] = E1
    F[:, P2, O2] = E2
    case.restart = (t, F, u)
    return case


def sds_expected(om=37, pm=36):
    """Sds after the coth(0.2 kd) factor at the two bins (float64)."""
    f, dlnf = freqs(om)
    dth = 2 * np.pi / pm
    k1, k2 = exact_k(f[O1], SDS_DEPTH), exact_k(f[O2], SDS_DEPTH)
    dk1 = 2 * np.pi * f[O1] * dlnf / exact_cg(k1, SDS_DEPTH)   # bin width in k: d omega / cg
    mss = E1 * np.cos((P2 - P1) * dth) ** 2 * dth * k1 ** 3 * dk1  # mean-square slope below the upper bin
    # coth(0.2 kd) with kd capped at 20 against overflow (umwm_init.F90:1484)
    coth = lambda k: 1.0 / np.tanh(0.2 * min(k * SDS_DEPTH, 20.0))
    s_lo = 2 * np.pi * 42.0 * f[O1] * (E1 * k1 ** 4) ** 2.4 * coth(k1)
    s_hi = 2 * np.pi * 42.0 * f[O2] * (1 + 360.0 * mss) ** 2 * (E2 * k2 ** 4) ** 2.4 * coth(k2)
    return s_lo, s_hi, mss


def test_sds_two_bins_oracle(oracle_mod):
    s_lo, s_hi, mss = sds_expected()
    assert 0.05 < 360 * mss < 2  # the slope factor matters
    case = _two_bin_case()
    for prec in (32, 64):
        o = oracle_mod.Oracle(case.nml, prec)
        case.stage(o)
        o.initialize()
        o.set_option("max_substeps", 1)
        o.run(case.start, case.stop)
        sds = o.get("sds")   # (im, pm, om), after the coth factor
        np.testing.assert_allclose(sds[:, P1, O1], s_lo, rtol=1e-4)
        np.testing.assert_allclose(sds[:, P2, O2], s_hi, rtol=1e-4)


@pytest.mark.gpu
def test_sds_two_bins_gpu(lib_built):
    s_lo, s_hi, _ = sds_expected()
    U = lib_built
    case = _two_bin_case()
    U.clear_inputs()
    case.stage(U)
    U.umwm_initialize(nml_text=case.nml)
    U.set_option("stress_ocn", 1)        # keep the substep's source terms
    U.set_option("max_substeps", 1)
    U.umwm_run(case.start, case.stop)
    sds = U.get_field("sds")
    U.umwm_finalize()
    np.testing.assert_allclose(sds[:, P1, O1], s_lo, rtol=1e-4)
    np.testing.assert_allclose(sds[:, P2, O2], s_hi, rtol=1e-4)


def snl_expected(om=37):
    """Snl of the two-bin spectrum (umwm_source_functions.F90:156-171): each
    energetic bin o loses snl_fac Sds(o) e(o) and passes the shares bf1 and
    bf2 of it, times kdk(o)/kdk(o-1) and kdk(o)/kdk(o-2), down one and two
    levels, with bf1 : bf2 = exp(-16 dlnf^2) : exp(-64 dlnf^2) normalised to
    a sum of 1 (umwm_init.F90:1290-1294), so the energy sum(kdk Snl) is
    conserved; Sds before the coth factor.  Returns ({(o, p): Snl}, kdk)."""
    f, dlnf = freqs(om)
    s_lo, s_hi, _ = sds_expected(om)
    coth = lambda k: 1.0 / np.tanh(0.2 * min(k * SDS_DEPTH, 20.0))
    k = np.array([exact_k(x, SDS_DEPTH) for x in f])
    kdk = k * 2 * np.pi * f * dlnf / np.array([exact_cg(x, SDS_DEPTH) for x in k])
    b1, b2 = np.exp(-16 * dlnf ** 2), np.exp(-64 * dlnf ** 2)
    bf1, bf2 = b1 / (b1 + b2), b2 / (b1 + b2)
    out = {}
    for o, p, e, sds in ((O1, P1, E1, s_lo / coth(k[O1])), (O2, P2, E2, s_hi / coth(k[O2]))):
        loss = 5.0 * sds * e  # snl_fac = 5
        out[(o, p)] = out.get((o, p), 0.0) - loss
        out[(o - 1, p)] = out.get((o - 1, p), 0.0) + bf1 * kdk[o] / kdk[o - 1] * loss
        out[(o - 2, p)] = out.get((o - 2, p), 0.0) + bf2 * kdk[o] / kdk[o - 2] * loss
    return out, kdk


def _check_snl(snl):
    exp, kdk = snl_expected()
    top = max(abs(v) for v in exp.values())
    for (o, p), v in exp.items():
        np.testing.assert_allclose(snl[:, p, o], v, rtol=2e-4, atol=1e-6 * top)
    # the downshifting conserves energy: sum over o of kdk Snl is zero
    for p in (P1, P2):
        cons = np.abs((snl[:, p, :] * kdk[None, :]).sum(axis=1))
        assert cons.max() <= 1e-4 * max(abs(v) * kdk[o] for (o, pp), v in exp.items() if pp == p)
    # no other bin of the two directions sees the downshifting
    for p in (P1, P2):
        others = [o for o in range(37) if (o, p) not in exp]
        assert np.abs(snl[:, p, others]).max() <= 1e-6 * top


def test_snl_two_bins_oracle(oracle_mod):
    case = _two_bin_case()
    for prec in (32, 64):
        o = oracle_mod.Oracle(case.nml, prec)
        case.stage(o)
        o.initialize()
        o.set_option("max_substeps", 1)
        o.run(case.start, case.stop)
        _check_snl(o.get("snl"))


@pytest.mark.gpu
def test_snl_two_bins_gpu(lib_built):
    U = lib_built
    case = _two_bin_case()
    U.clear_inputs()
    case.stage(U)
    U.umwm_initialize(nml_text=case.nml)
    U.set_option("stress_ocn", 1)        # keep the substep's source terms
    U.set_option("max_substeps", 1)
    U.umwm_run(case.start, case.stop)
    snl = U.get_field("snl")
    U.umwm_finalize()
    _check_snl(snl)


# ---------------------------------------------------------------------------
# deep-water Stokes drift
# ---------------------------------------------------------------------------
ST_DEPTH = 5000.0
# f ~ 0.315 Hz, 1/(2k) ~ 1.25 m; the bin is gentle enough (Sds ~ E^2.4) that
# the substep's downshifting moves less than 1e-3 of its energy
O_ST, P_ST, E_ST = 20, 22, 0.02


def _stokes_case():
    """One energetic bin in deep water under a light wind; dtg = 60 s so that
    the Stokes drift is computed after a single substep."""
    from umwm_gb300 import configs

    case = configs.fetch_limited(mm=12, nm=10, hours=1, depth=ST_DEPTH, wspd=1.0, dtg=60)
    t, F, u = case.restart
    F = np.full_like(F, np.finfo(np.float32).tiny)
    F[:, P_ST, O_ST] = E_ST
    case.restart = (t, F, u * 0.1)
    case.stop = "2012-01-01 00:01:00"
    return case


def stokes_expected(F, depths, om=37, pm=36):
    """u_s(z) = sum over bins of omega k a^2 exp(2 k z) (cos, sin) theta with
    a^2 = 2 F k dk dth (the bin's variance times 2), deep water; and the
    depth below z1 where |u_s| falls to |u_s(z1)|/e, by linear interpolation
    between levels as the reference does."""
    f, dlnf = freqs(om)
    dth = 2 * np.pi / pm
    th = (np.arange(1, pm + 1) - 0.5 * (pm + 1)) * dth
    k = np.array([exact_k(x, ST_DEPTH) for x in f])
    dk = 2 * np.pi * f * dlnf / np.array([exact_cg(x, ST_DEPTH) for x in k])
    a2 = 2 * F * (k * dk)[None, None, :] * dth            # (im, pm, om)
    z = -np.asarray(depths, dtype=np.float64)
    prof = (2 * np.pi * f * k)[None, :] * np.exp(2 * k[None, :] * z[:, None])   # (lm, om)
    us = np.einsum("lo,ipo,p->li", prof, a2, np.cos(th))
    vs = np.einsum("lo,ipo,p->li", prof, a2, np.sin(th))
    return us, vs


def _efold(mag, depths):
    ue = mag[0] / np.e
    for l in range(1, len(depths)):
        if mag[l] < ue:
            return (abs(mag[l - 1] - ue) * depths[l] + abs(mag[l] - ue) * depths[l - 1]) / (mag[l - 1] - mag[l])
    return 0.0


def _check_stokes(F, us, vs, ds, depths):
    ue, ve = stokes_expected(F.astype(np.float64), depths)
    scale = np.hypot(ue, ve).max()
    assert scale > 1e-5
    assert np.abs(us - ue).max() <= 2e-4 * scale, np.abs(us - ue).max() / scale
    assert np.abs(vs - ve).max() <= 2e-4 * scale, np.abs(vs - ve).max() / scale
    # monochromatic: |u_s| ~ exp(2 k z), e-folding 1/(2k) below the first level
    k = exact_k(freqs()[0][O_ST], ST_DEPTH)
    mag = np.hypot(ue, ve)
    for i in range(0, len(ds), 7):
        assert ds[i] == pytest.approx(_efold(mag[:, i], depths), abs=2e-3)
        assert ds[i] == pytest.approx(depths[0] + 1 / (2 * k), abs=0.02)


def test_stokes_deep_water_oracle(oracle_mod):
    from umwm_gb300.namelist import DEFAULTS

    case = _stokes_case()
    for prec in (32, 64):
        o = oracle_mod.Oracle(case.nml, prec)
        case.stage(o)
        o.initialize()
        o.run(case.start, case.stop)
        _check_stokes(o.get("e"), o.get("us"), o.get("vs"), o.get("ds"), DEFAULTS["depths"])


@pytest.mark.gpu
def test_stokes_deep_water_gpu(lib_built):
    from helpers import run_gpu
    from umwm_gb300.namelist import DEFAULTS

    U = lib_built
    run_gpu(U, _stokes_case())
    F, _ = U.get_state()
    _check_stokes(F, U.get_field("us"), U.get_field("vs"), U.get_field("ds"), DEFAULTS["depths"])
    U.umwm_finalize()


# ---------------------------------------------------------------------------
# unrolling of a periodic (global) grid, worked out by hand
# ---------------------------------------------------------------------------
# mm = nm = 4, isGlobal: only the n = 1 and n = nm rows are land
# (umwm_init.F90:659-667); sea points m outer, n inner, then land points
KG_II = np.array([[9, 1, 2, 10], [11, 3, 4, 12], [13, 5, 6, 14], [15, 7, 8, 16]])
# the west neighbour of m = 1 is m = mm and the east neighbour of m = mm is
# m = 1 (umwm_init.F90:993-1007)
KG_TRUE = {"iis": [9, 1, 11, 3, 13, 5, 15, 7], "iin": [2, 10, 4, 12, 6, 14, 8, 16],
           "iiw": [7, 8, 1, 2, 3, 4, 5, 6], "iie": [3, 4, 5, 6, 7, 8, 1, 2]}
KG_ALIAS = {"is": [0, 1, 0, 3, 0, 5, 0, 7], "in": [2, 0, 4, 0, 6, 0, 8, 0],
            "iw": [7, 8, 1, 2, 3, 4, 5, 6], "ie": [3, 4, 5, 6, 7, 8, 1, 2]}


def _kg_namelist():
    from umwm_gb300.namelist import make_namelist

    return make_namelist(mm=4, nm=4, isGlobal=True, xpl=2, ypl=2)


def test_known_answer_global_unrolling_oracle(oracle_mod):
    o = oracle_mod.Oracle(_kg_namelist(), 32)
    o.initialize()
    assert int(o.scalar("im")) == 8
    assert np.array_equal(o.get("ii"), KG_II)
    for k, v in list(KG_TRUE.items()) + list(KG_ALIAS.items()):
        assert list(o.get(k)[:8].astype(int)) == v, k


def test_known_answer_global_unrolling_library(lib_built):
    U = lib_built
    U.clear_inputs()
    U.setup_host(_kg_namelist())
    assert U.dims()["im"] == 8
    assert np.array_equal(U.get_field_i("ii"), KG_II)
    for k, v in list(KG_TRUE.items()) + list(KG_ALIAS.items()):
        assert list(U.get_field_i(k)[:8]) == v, k


# ---------------------------------------------------------------------------
# first-order upwind propagation of a step in x
# ---------------------------------------------------------------------------
PR_MM, PR_NM, PR_DX, PR_DEPTH = 20, 8, 5000.0, 1000.0
PR_O, PR_P, PR_E0, PR_M0 = 2, 17, 1.0, 10  # f ~ 0.039 Hz, theta = -5 degrees


def _step_case():
    """Energy E0 in one bin (deep water, theta = -5 deg) for m <= M0 and
    tiny(e) elsewhere; no wind (wspd clamped to 0.01), no currents, uniform
    depth: the sources change the bin by about 1e-6 in a substep and the
    rotation is zero, so one substep is the textbook upwind step
    e'(m) = e(m) - dts cg cos(theta) / dx (e(m) - e(m-1))
    (umwm_advection.F90:30-97 with cge = (cg0_i + cg0_ie) cos th, summed as
    0.25 dta / ar times the face fluxes)."""
    from umwm_gb300 import configs

    case = configs.fetch_limited(mm=PR_MM, nm=PR_NM, hours=1, dx=PR_DX, depth=PR_DEPTH, wspd=0.0)
    t, F, u = case.restart
    F = np.full_like(F, np.finfo(np.float32).tiny)
    nw = PR_NM - 2
    for m in range(2, PR_M0 + 1):
        F[(m - 2) * nw:(m - 1) * nw, PR_P, PR_O] = PR_E0
    case.restart = (t, F, np.full_like(u, 1e-3))
    return case


def _check_step(F, dts):
    f, _ = freqs()
    th = (PR_P + 1 - 0.5 * 37) * (2 * np.pi / 36)
    cfl = dts * exact_cg(exact_k(f[PR_O], PR_DEPTH), PR_DEPTH) * np.cos(th) / PR_DX
    assert 0.3 < cfl < 1.0
    nw = PR_NM - 2
    col = lambda m: F[(m - 2) * nw + 2:(m - 1) * nw - 2, PR_P, PR_O]  # interior rows
    np.testing.assert_allclose(col(PR_M0), PR_E0, rtol=1e-4)          # upstream: unchanged
    np.testing.assert_allclose(col(PR_M0 + 1), cfl * PR_E0, rtol=1e-4)  # the front advances by CFL
    assert col(PR_M0 + 2).max() < 1e-30                                 # nothing beyond it


def test_upwind_step_oracle(oracle_mod):
    case = _step_case()
    for prec in (32, 64):
        o = oracle_mod.Oracle(case.nml, prec)
        case.stage(o)
        o.initialize()
        o.set_option("max_substeps", 1)
        o.run(case.start, case.stop)
        _check_step(o.get("e"), o.scalar("dts"))


@pytest.mark.gpu
def test_upwind_step_gpu(lib_built):
    from helpers import run_gpu

    U = lib_built
    run_gpu(U, _step_case(), max_substeps=1)
    F, _ = U.get_state()
    dts = U.get_field("dts")
    U.umwm_finalize()
    _check_step(F, dts)
