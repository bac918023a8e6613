"""The persistent substep kernel (option "persistent"): the whole inner
dynamic-dts loop of a dtg, every member, in one cooperative launch with
grid-wide barriers between the stages.

It runs the stage bodies of the per-stage kernels with the same launch
parameters, so it is compared bit for bit with the graph-driven loop: the
spectrum, ustar, Hs, the screen lines and the substep count, for one domain
and for an ensemble whose members end the dtg after different numbers of
substeps.

Its barrier waits are bounded.  The stall test arms one launch whose barrier
expects one CTA more than were launched, so every wait runs out (after
20 ms): umwm_run must report UMWM_ERR_TIMEOUT, the GPU context must stay
usable, and running on must give the same state as a run that never stalled
(the stalled launch changed nothing but the forcing fields of a substep that
is then redone).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

UMWM_ERR_TIMEOUT = 5  # include/umwm_gpu.h


def _state(U, nmem=1):
    out = []
    for m in range(nmem):
        U.select_member(m)
        F, u = U.get_state()
        out.append((F, u, U.get_field("ht"), U.get_screen(), U.dims()["substeps"]))
    return out


def _same(a, b):
    for x, y in zip(a, b):
        for p, q in zip(x[:4], y[:4]):
            np.testing.assert_array_equal(p, q)
        assert x[4] == y[4]


def _run(U, cases, persistent, stop=None):
    U.clear_inputs()
    if len(cases) > 1:
        for c in cases:
            c.stage(U)
            U.ensemble_add(c.nml)
        U.ensemble_initialize()
    else:
        cases[0].stage(U)
        U.umwm_initialize(nml_text=cases[0].nml)
    U.set_option("use_graph", 1)
    U.set_option("persistent", 1 if persistent else 0)
    U.umwm_run(cases[0].start, stop or cases[0].stop)
    out = _state(U, len(cases))
    graph_state = U.stat("persistent_graph")
    U.umwm_finalize()
    return out, graph_state


def test_persistent_matches_graph_loop(lib_built):
    from umwm_gb300 import configs

    U = lib_built
    case = configs.random_field(mm=64, nm=56, hours=1, dx=2000.0)
    a, _ = _run(U, [case], False)
    b, gs = _run(U, [case], True)
    _same(a, b)
    assert gs in (1, -1)  # the launch ran (captured in a graph, or directly)


def test_persistent_ensemble_matches_graph_loop(lib_built):
    from umwm_gb300 import configs

    U = lib_built
    members = [configs.hurricane(mm=40 + 8 * k, nm=36 + 4 * k, hours=1, dx=4000.0, dtg=600, seed=3 + k)
               for k in range(3)]
    stop = configs._time_str(members[0].start, 1800)
    a, _ = _run(U, members, False, stop)
    b, _ = _run(U, members, True, stop)
    _same(a, b)


def test_persistent_barrier_timeout(lib_built):
    """A barrier wait that runs out: UMWM_ERR_TIMEOUT, then the run goes on."""
    from umwm_gb300 import configs

    U = lib_built
    case = configs.random_field(mm=48, nm=40, hours=1, dx=2000.0)

    def start():
        U.clear_inputs()
        case.stage(U)
        U.umwm_initialize(nml_text=case.nml)
        U.set_option("persistent", 1)
        U.set_option("max_substeps", 1)  # the first substep runs host-driven
        U.umwm_run(case.start, case.stop)

    start()
    U.set_option("max_substeps", 6)
    U.umwm_run(case.start, case.stop)
    ref = _state(U)
    U.umwm_finalize()

    start()
    U.set_option("max_substeps", 6)
    U.set_option("persistent_stall_test", 1)
    with pytest.raises(U.UmwmError) as err:
        U.umwm_run(case.start, case.stop)
    assert err.value.code == UMWM_ERR_TIMEOUT and "barrier" in str(err.value)
    assert U.dims()["substeps"] == 1
    U.umwm_run(case.start, case.stop)  # the context is usable and the run goes on
    _same(_state(U), ref)
    U.umwm_finalize()
