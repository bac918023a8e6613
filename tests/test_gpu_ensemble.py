"""Ensemble (batched) form: members of different sizes advanced as one model.

Each member of an ensemble must give exactly what it gives when run alone:
the kernels are the same, every per-point quantity depends only on the
member's own points, and the only cross-point operations (the dts minimum,
the rotation-rate maximum) are order-independent min/max per member.  So the
comparison is bit-exact.  One member is also checked against the oracle.
"""
import numpy as np
import pytest

from helpers import run_oracle, spec_stats

pytestmark = pytest.mark.gpu


def _members():
    from umwm_gb300 import configs

    return [configs.hurricane(mm=40, nm=36, hours=1, dx=4000.0, dtg=600, seed=3),
            configs.hurricane(mm=56, nm=48, hours=1, dx=3000.0, dtg=600, seed=5),
            configs.hurricane(mm=30, nm=44, hours=1, dx=5000.0, dtg=600, seed=7)]


def _run_alone(U, case):
    U.clear_inputs()
    case.stage(U)
    U.umwm_initialize(nml_text=case.nml)
    U.set_option("max_substeps", -1)
    U.umwm_run(case.start, case.stop)
    F, u = U.get_state()
    out = {"F": F, "ust": u, "ht": U.get_field("ht"), "taux": U.get_field("taux"),
           "screen": U.get_screen()}
    U.umwm_finalize()
    return out


def test_ensemble_members_match_single_runs(lib_built):
    U = lib_built
    members = _members()
    alone = [_run_alone(U, c) for c in members]
    U.clear_inputs()
    for c in members:
        c.stage(U)
        U.ensemble_add(c.nml)
    U.ensemble_initialize()
    assert U.get_field_i("members") == len(members)
    U.umwm_run(members[0].start, members[0].stop)
    for m, ref in enumerate(alone):
        U.select_member(m)
        F, u = U.get_state()
        np.testing.assert_array_equal(F, ref["F"])
        np.testing.assert_array_equal(u, ref["ust"])
        np.testing.assert_array_equal(U.get_field("ht"), ref["ht"])
        np.testing.assert_array_equal(U.get_field("taux"), ref["taux"])
        np.testing.assert_array_equal(U.get_screen(), ref["screen"])
    U.umwm_finalize()


def test_ensemble_member_vs_oracle(lib_built, oracle_mod):
    U = lib_built
    members = _members()
    U.clear_inputs()
    for c in members:
        c.stage(U)
        U.ensemble_add(c.nml)
    U.ensemble_initialize()
    U.set_option("max_substeps", 6)
    U.umwm_run(members[0].start, members[0].stop)
    U.select_member(1)
    o = run_oracle(oracle_mod, members[1], 32, max_substeps=6)
    l2, p999, mx = spec_stats(U.get_state()[0], o.get("e"))
    assert l2 < 1e-4 and p999 < 1e-3, (l2, p999, mx)
    U.umwm_finalize()
