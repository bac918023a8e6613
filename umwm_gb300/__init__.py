"""GB300 (sm_103a) implementation of the UMWM per-time-step path.

The compute path is libumwm_gb300.so (CUDA kernels + C ABI, include/umwm_gpu.h);
this package is its Python binding, a mirror of the reference's umwm_top
module, and the synthetic-workload generators.
"""
from ._lib import EXPORTS, LIB_PATH, UmwmError, lib  # noqa: F401
from .top import (clear_inputs, dims, ensemble_add, ensemble_initialize, get_field, get_field_i,  # noqa: F401
                  get_screen, get_state, get_state_noalloc, put_exclude, put_forcing, put_gridtopo, put_restart,
                  select_member, set_option, set_state, setup_host, stat, umwm_finalize, umwm_initialize, umwm_run,
                  write_restart, write_output)
from .top import (SURROGATE_WIDTH, gemm_bf16, surrogate_capture, surrogate_eval, surrogate_forward, surrogate_get_params,  # noqa: F401
                  surrogate_features, surrogate_grad, surrogate_init, surrogate_nparams, surrogate_set_params, surrogate_train)
