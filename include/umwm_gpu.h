/*
 * umwm_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the UMWM
 * per-time-step path: source terms and their exponential integration,
 * upwind propagation, refraction, wind stress and Stokes drift.
 *
 * Plain pointers and sizes only.  Every call returns UMWM_OK (0) or one of
 * the UMWM_ERR_* codes; umwm_gpu_last_error() returns the message of the
 * last failure.  The library never calls exit().
 *
 * One process-wide model, like the reference's module-global memory pool
 * (umwm_module.F90:98-207).  Calls are not re-entrant; use one host thread.
 *
 * Arrays follow the reference's Fortran layouts, given as flat C arrays:
 *   2-d fields (mm, nm)      : m fastest, index (m-1) + (n-1)*mm
 *   spectrum F(om, pm, im)   : o fastest, then p, then the wet index i
 *   wet-point fields (im)    : unrolled wet index i = 1..im, at offset i-1
 *
 * Inputs the reference reads from netCDF files are staged in memory under
 * the same names and time keys (there is no netCDF library on this
 * platform); umwm_gpu_initialize / umwm_gpu_run read them where the
 * reference opens the file.  An input that was not staged is read from the
 * reference's own file when that file is a netCDF classic or 64-bit-offset
 * file: input/umwm.gridtopo (lon, lat, z), input/umwmin_<time>.nc (uw, vw,
 * uc, vc, rhoa, rhow, fice) and restart/umwmrst_<time>.nc (F, ust), paths
 * relative to the working directory as in the reference.
 */
#ifndef UMWM_GPU_H
#define UMWM_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define UMWM_OK 0
#define UMWM_ERR_NAMELIST 1    /* bad or missing namelist value (umwm_init.F90:94-185) */
#define UMWM_ERR_INPUT 2       /* staged input missing or mis-sized (stands in for nc_check, umwm_io.F90:904-915) */
#define UMWM_ERR_CUDA 3        /* a CUDA call failed */
#define UMWM_ERR_NONFINITE 4   /* the finite-state check found NaN/Inf in the state */
#define UMWM_ERR_TIMEOUT 5     /* a bounded device-side wait gave up */
#define UMWM_ERR_STATE 6       /* call out of order (e.g. run before initialize) */
#define UMWM_ERR_ARG 7         /* bad argument (null pointer, wrong size, unknown name) */
#define UMWM_ERR_UNSUPPORTED 8 /* configuration outside what this build supports */

/* ---- input staging (stand-ins for the files the reference opens) ------- */

/* input/umwm.gridtopo variables 'lon', 'lat' (gridFromFile) and 'z'
 * (topoFromFile); replaces umwm_init.F90:397-427 and :541-546. */
int umwm_gpu_put_gridtopo(const char* var, const float* field_mn, int mm, int nm);

/* namelists/exclude.nml seed points (m, n) for fillLakes; replaces
 * umwm_init.F90:640-651.  mn holds npairs pairs. */
int umwm_gpu_put_exclude(const int* mn, int npairs);

/* input/umwmin_<time>.nc variable 'uw','vw','uc','vc','rhoa','rhow' or
 * 'fice' for the 19-character time key 'YYYY-MM-DD hh:mm:ss' (or with '_'
 * between date and time); replaces the reads of umwm_io.F90:13-93. */
int umwm_gpu_put_forcing(const char* time19, const char* var, const float* field_mn, int mm, int nm);

/* restart/umwmrst_<time>.nc variables 'F' (om*pm*im floats) and 'ust'
 * (im floats); replaces restart_read, umwm_restart.F90:19-56. */
int umwm_gpu_put_restart(const char* time19, const float* F, long nF, const float* ust, long nust);

/* Drop every staged input. */
int umwm_gpu_clear_inputs(void);

/* ---- umwm_top entry points --------------------------------------------- */

/* umwm_initialize, umwm_top.F90:7-29.  nml_path NULL means
 * "namelists/main.nml" relative to the working directory, as the
 * reference opens it (umwm_init.F90:84). */
int umwm_gpu_initialize(const char* nml_path);

/* Same as umwm_gpu_initialize with the namelist given as text. */
int umwm_gpu_initialize_text(const char* nml_text);

/* umwm_run(starttimestr, stoptimestr), umwm_top.F90:32-196.  Times are
 * 'YYYY-MM-DD hh:mm:ss'. */
int umwm_gpu_run(const char* start19, const char* stop19);

/* umwm_finalize, umwm_top.F90:199-204: frees every device and host
 * buffer of the model.  Staged inputs are kept. */
int umwm_gpu_finalize(void);

/* The host part of umwm_initialize only (namelist, grid, masks,
 * partition, remap, spectral tables), without touching the GPU, so that
 * the unrolled grid and tables can be inspected with the getters below. */
int umwm_gpu_setup_host(const char* nml_text);

/* ---- ensembles: many domains advanced together ---------------------------
 * An ensemble is one model over several domains ("members") that share the
 * spectral grid, physics, forcing switches, dtg and start time; each has its
 * own grid, depth, forcing, restart and dynamic time step.  Kernels run over
 * the concatenated wet points of all members, one launch per stage per
 * substep for the whole ensemble; a member that has reached the end of the
 * current dtg sits out the remaining substeps of that dtg.  Each member runs
 * exactly the computation it runs alone (no extension of the reference; it
 * replaces running the reference once per member). */

/* Add a member: its namelist text, and the inputs staged so far with the
 * put_* calls (the staging is then cleared for the next member). */
int umwm_gpu_ensemble_add(const char* nml_text);

/* Initialize every added member as one model (umwm_initialize for each). */
int umwm_gpu_ensemble_initialize(void);

/* Select the member the state and field getters/setters act on (default 0). */
int umwm_gpu_select_member(int member);

/* ---- state and fields ---------------------------------------------------- */

/* dims[0..7] = mm, nm, om, pm, im, imm, lm, substeps-so-far */
int umwm_gpu_get_dims(int* dims);

/* Spectrum F(om,pm,im) and friction velocity ust(im): what restart_write
 * stores, umwm_restart.F90:59-154.  Either pointer may be NULL. */
int umwm_gpu_get_state(float* F, float* ust);

/* Overwrite the spectrum and friction velocity (the restart_read
 * assignment, umwm_restart.F90:46-49).  Either pointer may be NULL. */
int umwm_gpu_set_state(const float* F, const float* ust);

/* Same output as umwm_gpu_get_state, for callers that cannot allocate device
 * memory at that moment: a job whose GPU memory is fully committed to an
 * ensemble or a pool allocator, or a coupling loop that must not pay
 * cudaFree's device-wide synchronisation.  umwm_gpu_get_state allocates a
 * temporary device buffer as large as the spectrum (om*pm*im floats); this
 * variant allocates nothing and streams the spectrum to F through a fixed
 * 16 MiB scratch array compiled into the library (held on every GPU that
 * loads the library until the process exits), in chunks of whole wet points,
 * all on the model's stream.  A point's spectrum larger than the scratch
 * (om*pm > 4 Mi floats) is rejected with UMWM_ERR_ARG.  The first call on a
 * device looks up the scratch address there; make it before any stream
 * capture.  All calls share the scratch: calls that overlap on the GPU race.
 * This entry point has no counterpart in the reference. */
int umwm_gpu_get_state_noalloc(float* F, float* ust);

/* restart_write, umwm_restart.F90:59-154: write the selected member's
 * state to a netCDF file (64-bit-offset classic format) in the reference's
 * layout: dimensions x, f, th; variables lon, lat, frequency, theta, ust,
 * wavenumber(x,f), F(x,th,f).  umwm_gpu_run also writes
 * restart/umwmrst_<time>.nc at the times the namelist's outrst asks for
 * (umwm_top.F90:183-190), and at a restart initialize reads that file when
 * no restart was staged for the start time (umwm_restart.F90:19-56).
 * Ensemble members use restart/umwmrst_<time>_m<member>.nc. */
int umwm_gpu_write_restart(const char* path);

/* output_grid_nc, umwm_io.F90:317-854: write the gridded output of the
 * last outer step (one-member models) to a netCDF file in the reference's
 * layout: dimensions x, y, f, th, time (record) and z with the Stokes
 * drift; the reference's variables in its order (frequency, theta, lon,
 * lat, seamask, depth, forcing, momentum, stresses with the stress('ocn')
 * parts, tails, cd, ust, swh and the mean and dominant wave fields,
 * physics_time_step), each with its description and units; land cells
 * NaN.  Needs the stress('ocn') fields (option stress_ocn, or a run that
 * wrote output).  umwm_gpu_run also writes output/umwmout_<time>.nc at
 * the times the namelist's outgrid asks for when the directory output
 * exists, computing stress('ocn') for those steps (umwm_top.F90:165-177);
 * it writes nothing otherwise, as the reference's failed nf90_create
 * does. */
int umwm_gpu_write_output(const char* path);

/* output_spectrum_nc (umwm_io.F90:150-314) has no entry point of its own:
 * with the namelist's outspec set, umwm_gpu_run appends a record per output
 * time (and one at the start) to output/umwmspc_<id>_<time>.nc for each
 * point of namelists/spectrum.nml, when the directory output exists. */

/* Copy a named field into out (n floats).  Names are the reference's
 * variable names: wet-point fields (ht, mwp, mwd, mss, mwl, dwd, dwl, dwp,
 * dcp0, dcp, dcg0, dcg, momx, momy, cgmxx, cgmxy, cgmyy, ustar, cd, taux,
 * tauy, taux_form, tauy_form, taux_skin, tauy_skin, taux_diag, tauy_diag,
 * tailatmx, tailatmy, shelt, fcutoff, physics_time_step, ds, ar, dxn, dxs,
 * dye, dyw, oneovar, oneovdx, oneovdy), all-point fields over imm (wspd,
 * wdir, uc, vc, rhoa, rhow, rhorat, fice, d, dx, dy), Stokes drift 'us',
 * 'vs' (lm*im, level-major), spectral tables (om*im: k, kdk, k3dk, ...;
 * cp0, cg0 as om*(im+1) with the ghost point first), 'f' (om), 'th' (pm),
 * 'depth' (lm), the 2-d grid fields d_2d, dx_2d, dy_2d, curv, lon, lat
 * (mm*nm, m fastest) and the scalars dts, dta, dtr, dtamin, sumt, cgmax, dth.
 * The outputs of stress('ocn') (umwm_stress.F90:34-214), over wet points,
 * once it has run (option "stress_ocn", or an outer step with gridded
 * output due): taux_ocntop, tauy_ocntop, taux_ocnbot, tauy_ocnbot, taux_snl,
 * tauy_snl, epsx_ocn, epsy_ocn, epsx_atm, epsy_atm, tailocnx, tailocny,
 * taux1, tauy1, taux2, tauy2, taux3, tauy3; and the source terms its last
 * substep kept, in get_state's (om, pm, im) layout: ssin, sds (after the
 * cothkd factor) and snl (umwm_source_functions.F90:16-183). */
int umwm_gpu_get_field(const char* name, float* out, long n);

/* Integer fields: mask, ii (mm*nm); mi, ni, iw, ie, is, in, iiw, iie,
 * iis, iin (imm); oc (im); and scalars im, imm, iip. */
int umwm_gpu_get_field_i(const char* name, int* out, long n);

/* The per-substep screen line of umwm_top.F90:143-148 (sumt/dtg, dts,
 * wspd, wdir, swh, mwp, cd*1e3, f(oc) at the print point), 8 doubles per
 * substep since initialize; returns the number of rows in *rows. */
int umwm_gpu_get_screen(double* out, long n, long* rows);

/* Options: "verbose" (print the screen lines), "max_substeps" (stop a run
 * after that many substeps in total; -1 = off), "check_finite" (after each
 * outer step, check that the significant wave height and friction velocity
 * of every wet point are finite -- a NaN/Inf bin makes its point's wave
 * height non-finite -- and fail with UMWM_ERR_NONFINITE otherwise),
 * "use_graph" (run the inner loop as a CUDA graph with a device-side while
 * node: one host synchronisation per outer step instead of one per
 * substep; results are bit-identical), "kernel_timing" (CUDA-event time of
 * each kernel, read with umwm_gpu_get_stat "ms:<kernel>"; the inner loop
 * then runs host-driven), "device" (CUDA device of the next initialize),
 * "stress_ocn" (run stress('ocn') after every outer step: the last substep
 * of each step keeps its source terms, three more spectrum-sized arrays),
 * "direction_groups" (2: each point's directions in two half-turn groups
 * per warp lane pair; 4: four quarter-turn groups, twice the CTAs; needs
 * pm % 4 == 0 and pm/4 in {4, 6, 8, 9, 12}; initialize picks 4 below 3
 * 64-point tiles per SM and 2 above; results differ by summation order
 * only), "advect_groups" (the same for the propagation kernel alone), "gust_seed" (seed of the wind gust draws when
 * the namelist's gustiness > 0, umwm_forcing.F90:49-61; default 1: the
 * draws are a function of seed, substep, grid cell and component, so a run
 * repeats with its seed), "phys_groups" / "integ_groups" (the mapping of the
 * dts pre-pass or the integration alone), "minb_phys" / "minb_integ" /
 * "minb_advect" (resident CTAs per SM the kernel's register budget is sized
 * for; 0 or a budget without a compiled instance: the default) and
 * "pf_phys" / "pf_integ" / "pf_advect" (frequency levels each kernel
 * prefetches into L2 ahead), "advect_tma" / "phys_tma" (the propagation /
 * dts pre-pass of the two-group 36-direction mapping stage each level's own
 * rows in shared memory with bulk copies: advect_tma 1 the E* and e rows,
 * 2 the E* rows only; phys_tma 1 the e rows; results do not change),
 * "autotune" (0 off; 1: from the next substep
 * on, time the register budgets and prefetch distances of the three
 * spectral kernels on the model's own substeps, round-robin, and keep the
 * fastest of each; results do not change; 2: also the direction mappings,
 * which changes results by rounding only; choices are cached per domain
 * shape for the life of the process), "count_cut" (1: count the bins
 * whose negative ef the propagation cuts to 0 before e = ef, read with
 * umwm_gpu_get_stat "cut_count"; pm = 36 only), "persistent" (1: each
 * dtg's inner loop, every member, runs as one cooperative launch of the
 * persistent substep kernel with grid barriers between the stages; each
 * barrier wait is bounded (2 s) and one that runs out ends the run with
 * UMWM_ERR_TIMEOUT; pm = 36 and one direction mapping for all kernels;
 * results are bit-identical to the other loops), "persistent_stall_test"
 * (1: the next persistent launch's barrier expects one CTA more than
 * launched, so its waits run out after 20 ms: for testing the time-out
 * path).  This library's own options have no counterpart in the
 * reference. */
int umwm_gpu_set_option(const char* name, double value);

/* Run statistics: "substeps", "gpu_ms" (device time of the last run),
 * "bin_updates" (wet bins x substeps of the last run), "launches",
 * "device_free_bytes" (cudaMemGetInfo's free memory of the current device),
 * "cut_count" (bins the non-negativity cut changed since option
 * "count_cut" was set), "autotune_active", "autotune_done",
 * "autotune_substeps" (substeps measured),
 * "config:phys" / "config:integ" / "config:advect" (launch configuration in
 * use: direction groups * 100 + CTAs per SM * 10 + prefetch levels),
 * "tune_n:<kernel>", "tune_cfg:<kernel>:<i>", "tune_ms:<kernel>:<i>" (the
 * autotuner's candidates, their configurations and median times),
 * "persistent_graph" (1: the persistent launch is captured in a CUDA graph,
 * -1: launched directly, 0: not run yet). */
double umwm_gpu_get_stat(const char* name);

/* Message of the last failure ("" if none). */
const char* umwm_gpu_last_error(void);

/* ---- learned source-term surrogate --------------------------------------
 * No counterpart in the reference: an MLP (om*pm + 9 inputs padded to 1344
 * -> 512 -> 512 -> 1344, GELU; bf16 operands, f32 accumulation on the tensor
 * cores) that replaces the source-term integration of a substep
 * (umwm_physics.F90:61-84) when the option "surrogate" is 1.  Inputs of a
 * point: its log-spectrum rotated so the wind lies along the first
 * direction, wind speed, the wind's offset from that direction, friction
 * velocity, log depth, dts, currents along/across the wind, rhoa/rhow and
 * ice fraction.  Output: the step's log-tendency, ef = (e+eps) exp(2 y) - eps.
 * A per-point energy-budget monitor (|ln(sum ef kdk / sum e kdk)| <=
 * "surrogate_tol", default 0.02 per substep), and the same for the energy of
 * every frequency level holding more than 1e-4 of the point's largest
 * ("surrogate_tol_level", default 0.1), sends a point that fails back to the
 * plain integration.  A bin's growth is capped by its wind input,
 * dts max(Sin, 0) + 0.02 in ln.  get_stat "surrogate_points" / "surrogate_fallback" count
 * point-substeps since the surrogate buffers were created. */

/* Create the network for om x pm spectra with seeded random weights (and
 * fresh Adam state).  Parameters persist across initialize/finalize. */
int umwm_gpu_surrogate_init(int om, int pm, unsigned long long seed);

/* Parameters as f32 in the order W1 (512 x 1344), b1 (512), W2 (512 x 512),
 * b2 (512), W3 (1344 x 512), b3 (1344); n must be get_stat
 * "surrogate_nparams". */
int umwm_gpu_surrogate_get_params(float* out, long n);
int umwm_gpu_surrogate_set_params(const float* in, long n);

/* Capture training pairs during subsequent plain runs: each substep, the
 * inputs of points_per_substep random wet points and the log-tendency the
 * plain integration gives them, into a device store of `capacity` pairs
 * (a new capacity empties the store; capacity 0 stops capturing). */
int umwm_gpu_surrogate_capture(long capacity, int points_per_substep);

/* Train on the captured pairs: `steps` Adam steps (learning rate lr) on
 * mini-batches of `batch` pairs drawn with the seed; losses[steps] (may be
 * NULL) receives the mean-squared error of each step.  batch % 128 == 0. */
int umwm_gpu_surrogate_train(int steps, int batch, double lr, unsigned long long seed, float* losses);

/* Mean-squared-error loss of the current network over the stored pairs
 * [first, first + count) (no training).  Option "surrogate_holdout" keeps
 * that many trailing stored pairs out of umwm_gpu_surrogate_train. */
int umwm_gpu_surrogate_eval(long first, long count, double* loss);

/* Network output (n x 1344 f32) for input rows X (n x 1344 f32; rounded
 * to bf16 like every input). */
int umwm_gpu_surrogate_forward(const float* X, int n, float* Y);

/* Mean-squared-error loss and its gradient (get_stat "surrogate_nparams"
 * floats, parameter order) for one batch X, T (n x 1344 f32, n % 64 == 0),
 * without updating the parameters. */
int umwm_gpu_surrogate_grad(const float* X, const float* T, int n, float* loss, float* grad);

/* Input rows of the surrogate (im x 1344 f32) for the selected member's
 * wet points in the current state, with the dts of the last substep. */
int umwm_gpu_surrogate_features(float* X, long n);

/* C = A B^T on the tensor cores: A (M x K) and B (N x K) bf16 bit
 * patterns, C (M x N) f32.  K % 64 == 0, N % 32 == 0.  The GEMM the
 * surrogate's layers use. */
int umwm_gpu_gemm_bf16(const unsigned short* A, const unsigned short* B, float* C, int M, int N, int K);

#ifdef __cplusplus
}
#endif

#endif /* UMWM_GPU_H */
