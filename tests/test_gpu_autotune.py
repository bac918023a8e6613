"""The online autotuner of the spectral kernels' launch configuration
(option "autotune").

Mode 1 tunes the register budget (resident CTAs per SM) and the L2 prefetch
distance of the dts pre-pass, the integration and the propagation while the
model's own substeps run, round-robin over the candidates, five samples each.  Neither knob
changes any arithmetic, so a tuned run is compared bit for bit with an untuned
one, also across the substeps during which the candidates rotate (the
candidates include the forms of the propagation and the dts pre-pass that
stage their own rows with bulk copies).  Mode 2
also tunes the direction mapping, which changes summation order only: its run
meets the oracle's parity bar.  The choice is cached per domain signature, so
a second model of the same shape starts tuned.
"""
import numpy as np
import pytest

from helpers import run_oracle, spec_stats

pytestmark = pytest.mark.gpu


def _run(U, case, autotune, nsub, graph=True):
    U.clear_inputs()
    case.stage(U)
    U.umwm_initialize(nml_text=case.nml)
    U.set_option("use_graph", 1 if graph else 0)
    if autotune:
        U.set_option("autotune", autotune)
    U.set_option("max_substeps", nsub)
    U.umwm_run(case.start, case.stop)
    F, u = U.get_state()
    info = {"done": U.stat("autotune_done"), "active": U.stat("autotune_active"),
            "measured": U.stat("autotune_substeps"),
            "config": [U.stat("config:" + k) for k in ("phys", "integ", "advect")]}
    U.umwm_finalize()
    return F, u, info


def test_autotune_bit_identical(lib_built):
    from umwm_gb300 import configs

    U = lib_built
    case = configs.random_field(mm=64, nm=56, hours=1, dx=2000.0)
    F0, u0, _ = _run(U, case, 0, 50)
    F1, u1, info = _run(U, case, 1, 50)
    np.testing.assert_array_equal(F1, F0)
    np.testing.assert_array_equal(u1, u0)
    # 9 pre-pass candidates x 5 samples after the first substep: tuning done
    assert info["done"] == 1 and info["active"] == 0 and info["measured"] == 45
    for c in info["config"]:
        assert (int(c) // 100) % 10 in (2, 4) and 1 <= int(c) % 10 <= 3
    # the same shape again starts from the cached choice
    F2, u2, info2 = _run(U, case, 1, 50)
    assert info2["done"] == 1 and info2["measured"] == 0 and info2["config"] == info["config"]
    np.testing.assert_array_equal(F2, F0)


def test_autotune_direction_mapping_parity(lib_built, oracle_mod):
    from umwm_gb300 import configs

    U = lib_built
    case = configs.random_field(mm=48, nm=40, hours=2, dx=2000.0)
    # 20 pre-pass candidates (two mappings, two with staged rows) x 5 samples
    # after the first substep
    F, _, info = _run(U, case, 2, 110)
    assert info["done"] == 1 and info["measured"] == 100
    o = run_oracle(oracle_mod, case, 32, max_substeps=110)
    l2, p999, _ = spec_stats(F, o.get("e"))
    assert l2 < 1e-4 and p999 < 1e-3, (l2, p999)


@pytest.mark.parametrize("option,value", [("advect_tma", 1), ("advect_tma", 2), ("phys_tma", 1)])
def test_tma_forms_bit_identical(lib_built, option, value):
    """The propagation and the dts pre-pass with their own rows staged in
    shared memory by bulk copies (options advect_tma 1: E* and e, 2: E*
    only; phys_tma; candidates of the tuner) read the same values as the
    kernels that load them from global memory, so the run is bit-identical."""
    from umwm_gb300 import configs

    U = lib_built
    case = configs.random_field(mm=96, nm=80, hours=1, dx=2000.0)

    def run(tma):
        U.clear_inputs()
        case.stage(U)
        U.umwm_initialize(nml_text=case.nml)
        U.set_option("direction_groups", 2)  # the TMA form is the two-group form
        U.set_option(option, tma)
        U.set_option("max_substeps", 12)
        U.umwm_run(case.start, case.stop)
        F, u = U.get_state()
        cfg = U.stat("config:advect" if option == "advect_tma" else "config:phys")
        U.umwm_finalize()
        return F, u, cfg

    F0, u0, c0 = run(0)
    F1, u1, c1 = run(value)
    assert c0 < 1000 and c1 // 1000 == value
    np.testing.assert_array_equal(F1, F0)
    np.testing.assert_array_equal(u1, u0)
