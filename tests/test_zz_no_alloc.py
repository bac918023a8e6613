"""umwm_gpu_get_state_noalloc against umwm_gpu_get_state.

The no-allocation read-back exists for callers that cannot allocate device
memory at the moment they save the state: a job whose GPU memory is fully
committed to an ensemble or to another model's pool allocator, or a coupling
loop that must not pay cudaFree's device-wide synchronisation.  It streams the
spectrum through the library's fixed 16 MiB scratch array instead of a
temporary buffer as large as the spectrum.  It must return exactly what the
allocating entry point returns (both are copies of the same state), on two
calls in a row, which reuse the same scratch, and the device's free memory
must be the same after the second call as after the first (a call that left
a buffer behind would show there).  The 100x100 case has 9604
wet points, more than one scratch chunk (3149 points), so the chunking is
exercised.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_get_state_noalloc_matches_get_state(lib_built):
    from umwm_gb300 import configs

    U = lib_built
    case = configs.fetch_limited(mm=100, nm=100, hours=1)
    U.clear_inputs()
    case.stage(U)
    U.umwm_initialize(nml_text=case.nml)
    U.set_option("max_substeps", 3)
    U.umwm_run(case.start, case.stop)
    F_ref, u_ref = U.get_state()
    assert np.isfinite(F_ref).all() and F_ref.max() > 0
    free0 = None
    for call in range(2):  # two calls in a row share the scratch
        F, u = U.get_state_noalloc()
        assert F.shape == F_ref.shape
        np.testing.assert_array_equal(F, F_ref)
        np.testing.assert_array_equal(u, u_ref)
        free = U.stat("device_free_bytes")
        assert free > 0
        if free0 is None:
            free0 = free  # after the first call: the scratch address is resolved
        else:
            assert free == free0, "device free memory changed across a call: %d -> %d" % (free0, free)
    U.umwm_finalize()
