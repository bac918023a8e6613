"""The inner loop of umwm_run as a CUDA graph (option "use_graph") and the
finite-state check (option "check_finite").

The graph runs the same kernels with the same arguments as the host-driven
loop, so the two are compared bit for bit: spectrum, friction velocity,
significant wave height, the per-substep screen lines and the substep count,
also when the run is cut short by "max_substeps" inside a dtg.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(U, case, graph, max_substeps=-1, ensemble=None):
    U.clear_inputs()
    if ensemble:
        for c in ensemble:
            c.stage(U)
            U.ensemble_add(c.nml)
        U.ensemble_initialize()
    else:
        case.stage(U)
        U.umwm_initialize(nml_text=case.nml)
    U.set_option("use_graph", 1 if graph else 0)
    U.set_option("max_substeps", max_substeps)
    U.umwm_run(case.start, case.stop)
    out = []
    for m in range(len(ensemble) if ensemble else 1):
        U.select_member(m)
        F, u = U.get_state()
        out.append({"F": F, "ust": u, "ht": U.get_field("ht"), "screen": U.get_screen(),
                    "substeps": U.dims()["substeps"]})
    U.umwm_finalize()
    return out


def _same(a, b):
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x["F"], y["F"])
        np.testing.assert_array_equal(x["ust"], y["ust"])
        np.testing.assert_array_equal(x["ht"], y["ht"])
        np.testing.assert_array_equal(x["screen"], y["screen"])
        assert x["substeps"] == y["substeps"]


@pytest.mark.parametrize("max_substeps", [-1, 7])
def test_graph_loop_matches_host_loop(lib_built, max_substeps):
    from umwm_gb300 import configs

    U = lib_built
    case = configs.random_field(mm=48, nm=40, hours=2, dx=2000.0)
    host = _run(U, case, False, max_substeps)
    graph = _run(U, case, True, max_substeps)
    _same(host, graph)
    if max_substeps > 0:
        assert graph[0]["screen"].shape[0] == max_substeps


def test_graph_loop_ensemble(lib_built):
    from umwm_gb300 import configs

    U = lib_built
    members = [configs.hurricane(mm=40, nm=36, hours=1, dx=4000.0, dtg=600, seed=3),
               configs.hurricane(mm=30, nm=44, hours=1, dx=5000.0, dtg=600, seed=7)]
    _same(_run(U, members[0], False, ensemble=members), _run(U, members[0], True, ensemble=members))


def test_check_finite(lib_built):
    from umwm_gb300 import configs

    U = lib_built
    case = configs.fetch_limited(mm=24, nm=14, hours=1)
    U.clear_inputs()
    case.stage(U)
    U.umwm_initialize(nml_text=case.nml)
    U.set_option("check_finite", 1)
    U.umwm_run(case.start, case.stop)  # a finite run passes the check
    F, u = U.get_state()
    F[F.shape[0] // 2, 3, 5] = np.nan  # a non-finite bin planted from the host
    U.set_state(F, None)
    with pytest.raises(U.UmwmError) as exc:
        U.umwm_run(case.stop, configs._time_str(case.stop, 3600))
    assert exc.value.code == 4  # UMWM_ERR_NONFINITE
    U.umwm_finalize()
