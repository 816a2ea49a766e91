/*
 * gs_abi.h -- C ABI of the GB300 UPPE z-step core (gsolver_solid_qdht hot path).
 *
 * Plain pointers and sizes only.  Every entry point returns an int status (GS_OK = 0);
 * gs_last_error() gives the message, which for physics errors is the reference's own
 * exception string.  A handle owns one CUDA stream on one device and is not
 * thread-safe: one host thread drives it.
 *
 * Complex arrays are interleaved (re, im) doubles.  Field arrays are row-major
 * [n_r][n_t] with omega contiguous and omega in the reference's own order
 * (omega0 + k*dw for k < n_t/2, then the negative offsets), i.e. the layout of the
 * reference's FIELD / BIGBUFFER1 / BIGBUFFER2 (propagator.cu:380, 593).
 *
 * Reference interfaces replaced (paths within the reference project):
 *   gs_create + gs_upload_tables  <- initialize_variables()/cuda_load_const()
 *                                    (solver_main.cpp:265-398, propagator.cu:999-1108)
 *   gs_set_field / gs_get_field   <- the host FIELD / BIGBUFFER2 globals (solver.h:169)
 *   gs_nl_step                    <- calculate_NLstep(float_type*, float_type*)
 *                                    (propagator.cu:121, 268-426)
 *   gs_lstep                      <- ht_run(BIGBUFFER1) + calculate_Lstep() + ht_run(FIELD)
 *                                    (propagator.cu:179-213, 516-626)
 *   gs_qdht                       <- ht_run(f_complex*, f_complex*) (solver.h:337-346)
 *                                    -> qdht_plan::run_many (fhatha.cpp:218-230)
 *   gs_step                       <- propagator() (solver.h:269, propagator.cu:125-266)
 *   gs_step_host                  <- propagator() on the host FIELD / BIGBUFFER2 globals (the copies in
 *                                    and out the call makes, overlapped with its first NL attempt)
 *   gs_advance                    <- the z-loop's propagator() calls between ZNET points
 *                                    (solver_main.cpp:202-225), the controller on the device
 *   gs_destroy                    <- destroy_variables()/cuda_free_const()
 *                                    (solver_main.cpp:415-440)
 *   gs_energy                     <- dump_type_average_spectrum_class (dump_types.cpp:427-457)
 *   gs_checkpoint_save / _load    <- dump_type_full_class (dump_types.cpp:77-97) and the
 *                                    DUMP_FINAL_FIELD restart (solver_main.cpp:226-229)
 */
#ifndef GS_ABI_H
#define GS_ABI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GS_ABI_VERSION 2   /* 2: gs_params gained ion_levels / ion_potentials */

typedef struct gs_handle gs_handle;

enum gs_status {
    GS_OK = 0,
    GS_ERR_ARG = 1,         /* bad argument / size */
    GS_ERR_CUDA = 2,        /* CUDA runtime error (message in gs_last_error) */
    GS_ERR_BLAST = 3,       /* "Attention!!!! Intensity is too big! Keep away, blast is possible." */
    GS_ERR_NAN = 4,         /* "float_type photoionization_function(...): Intensity is nan!" */
    GS_ERR_COLLAPSE = 5,    /* "Minimum Z step size reached, collapse is possible!" */
    GS_ERR_STATE = 6,       /* call out of order (tables / field not set) */
    GS_ERR_UNSUPPORTED = 7, /* grid not supported by this build */
    GS_ERR_NOMEM = 8        /* device allocation failed */
};

enum gs_precision {
    GS_PREC_FP64 = 0,       /* plain FP64 GPU path: the parity path against the FP64 reference */
    GS_PREC_MIXED = 1       /* FP32 elementwise/FFT; QDHT on tcgen05 with FP32 accumulation over split
                               operands: FP16 hi/lo pairs of power-of-two-scaled values where
                               2 n_t is a multiple of 256, 3xTF32 hi/lo parts for other widths */
};

/* Scalars of the hot path, in the reference's scaled units
 * (solver_main.cpp:385-393, process_input.cpp:58, ionization.cpp:11). */
typedef struct gs_params {
    int n_r, n_t;                 /* N_R (QDHT points), N_T (power of two, >= 64) */
    int precision;                /* enum gs_precision */
    int nonlinear;                /* 1: NONLINEARITY_ON; 0: zero NL response (shipped build) */
    int device;                   /* CUDA device ordinal */
    int gas;                      /* 0: the solid build (gsolver_solid_qdht: Keldysh, avalanche,
                                     recombination); 1: the gas build (gsolver_gas_qdht,
                                     Makefile:19: PPT rate tables, ionization with neutral
                                     depletion over ion_levels levels, third harmonic,
                                     IONRATE_DENOM 1e10) */
    double tstep, tmin, tmax, omega0;
    double ionrate_denom;         /* IONRATE_DENOM (1e20 for the solid build) */
    double neutral_density;       /* NEUTRAL_DENSITY */
    double rho0;                  /* start carrier density of each plasma recurrence */
    double ionization_potential;  /* U_i * IONRATE_DENOM / INTENSITY_DENOM */
    double ponderomotive;         /* PONDEROMOTIVE_COEFFICIENT * IONRATE_DENOM */
    double avalanche_cs;          /* AVALANCHE_CROSSSECTION */
    double recombination_tau;     /* RECOMBINATION_TAU * IONRATE_DENOM */
    double raman_fraction;        /* RAMAN_FRACTION */
    double n2;                    /* NONLIN_REFRINDEX * INTENSITY_DENOM */
    double omega_min, omega_max;  /* spectral window of the linear step */
    double max_tolerance;         /* MAX_TOLERANCE of the step controller */
    double raman_tau, raman_omega; /* TAU_RAMAN, OMEGA_RAMAN: when both > 0 the delayed Kerr
                                      response is computed from this oscillator by an exact
                                      recurrence instead of the RAMAN_FUNCTION FFT pair */
    double th_coeff;              /* gas build: KERR_TH_PROFILE / KERR_PROFILE = (1 - fR)/3
                                     TH_FACTOR (process_input.cpp:1020); 0: no third harmonic */
    int ion_levels;               /* gas build: IONIZATION_LEVEL_N (0 or 1: one level, with
                                     ionization_potential; up to GS_MAX_ION_LEVELS: the
                                     MULTI_LEVEL_IONIZATION branch, ionization.cpp:45-84) */
    double ion_potentials[8];     /* gas build with ion_levels > 1: IONIZATION_POTENTIALn of level
                                     n - 1, scaled as ionization_potential */
} gs_params;

#define GS_MAX_ION_LEVELS 8

/* Per-omega / per-k tables (host pointers, FP64, reference omega order). */
typedef struct gs_tables {
    const double* rate_ln;        /* IONIZATION_RATE_LN[8192]; gas build with ion_levels > 1:
                                     [ion_levels][8192], level n's row (ionization.cpp:313-331) */
    const double* plasma_func;    /* PLASMA_FUNC, complex [n_t] */
    const double* raman_func;     /* RAMAN_FUNCTION, complex [n_t] */
    const double* kerr;           /* KERR_PROFILE [n_t] */
    const double* omega;          /* OMEGA [n_t] */
    const double* wavenum;        /* WAVENUMBER, complex [n_t] */
    const double* ho_disp;        /* HO_DISPERSION [n_t] */
    const double* kt2;            /* transverse wavenumber squared per QDHT point [n_r] */
    const double* qdht_c;         /* qdht_plan::C, [n_r*n_r], element (i,j) at C[i + n_r*j] */
    const double* qdht_m1;        /* qdht_plan::m1 [n_r] */
} gs_tables;

/* Create a handle: allocates device state for one pulse on params->device. */
int gs_create(const gs_params* params, gs_handle** out);

/* Upload the tables (cuda_load_const).  Required before any step. */
int gs_upload_tables(gs_handle* h, const gs_tables* tables);

/* Set FIELD (r,omega) and BIGBUFFER2 (k,omega).  spec_k_omega may be NULL, in which case
 * BIGBUFFER2 = ht_run(FIELD), as process_input.cpp:68-73 does at start-up. */
int gs_set_field(gs_handle* h, const double* field_r_omega, const double* spec_k_omega);

/* Copy FIELD and/or BIGBUFFER2 back to the host (either pointer may be NULL). */
int gs_get_field(gs_handle* h, double* field_r_omega, double* spec_k_omega);

/* calculate_NLstep: BIGBUFFER1 = RK4 increment of the NL response with step zstep;
 * returns max |FIELD|^2 and max |BIGBUFFER1|^2. */
int gs_nl_step(gs_handle* h, double zstep, double* max_a2, double* max_nl2);

/* Copy BIGBUFFER1 (the last NL increment, (r,omega)) to the host: after gs_nl_step.  The
 * propagator() paths (gs_step, gs_advance, gs_step_host, batches) may keep only the window columns
 * the linear step reads; gs_get_nl then returns GS_ERR_STATE. */
int gs_get_nl(gs_handle* h, double* bb1_r_omega);

/* ht_run(BIGBUFFER1) -> calculate_Lstep(zstep) -> ht_run(FIELD). */
int gs_lstep(gs_handle* h, double zstep);

/* ht_run on a host array [n_r][n_t] complex, in place. */
int gs_qdht(gs_handle* h, double* data_r_omega);

/* One propagator() call: repeats NL attempts until the controller accepts.
 * current_z = CURRENT_Z, znet_cur = ZNET[n_Z], znet_prev = ZNET[n_Z-1];
 * zstep_inout = ZSTEP, step_n_inout = STEP_N (incremented per rejected attempt, as the
 * reference does); max_a2 / max_nl2 (may be NULL) of the accepted attempt. */
int gs_step(gs_handle* h, double current_z, double znet_cur, double znet_prev,
            double* zstep_inout, unsigned* step_n_inout, double* max_a2, double* max_nl2);

/* gs_step on host-resident state: the reference's propagator() works on the host globals FIELD
 * and BIGBUFFER2 (solver.h:169), so a drop-in call takes them in, steps, and gives them back.
 * Equivalent to gs_set_field(field, spec) + gs_step(...) + gs_get_field(field, spec), bit for
 * bit; FIELD goes in first and BIGBUFFER2's copy in (on a copy stream) overlaps the first NL
 * attempt, which reads FIELD only.  field / spec: [n_r][n_t] complex, in and out (pinned
 * memory for the full host-link rate). */
int gs_step_host(gs_handle* h, double* field_r_omega, double* spec_k_omega, double current_z, double znet_cur,
                 double znet_prev, double* zstep_inout, unsigned* step_n_inout, double* max_a2, double* max_nl2);

/* The z-loop of solver_main.cpp:202-225 advanced by up to max_calls propagator() calls without
 * a host round trip per call: each attempt's controller (propagator.cu:147-164: the error test,
 * the new ZSTEP, the collapse and ZNET-clamp rules) and the loop's STEP_N / CURRENT_Z update run
 * in a one-thread kernel between the NL step and the linear step, which take their step sizes
 * from device memory.  Starts from CURRENT_Z = *current_z below ZNET[n_z] (the caller has done the
 * dump test at the loop's top), ZSTEP = *zstep, STEP_N = *step_n; stops after the call that brings
 * CURRENT_Z to ZNET[n_z] or beyond (*reached = 1: the caller dumps, advances n_z, calls again), or
 * after max_calls calls (*reached = 0).  Results are those of the same calls through gs_step, bit
 * for bit.  Grids whose NL step or linear step needs the host (other than the 16384-point FP32
 * rows with the compact tensor-core plan; a photon-number tolerance; apertures) take gs_step call
 * by call.  *calls_done = accepted calls; on GS_ERR_COLLAPSE *zstep is the collapsed proposal. */
int gs_advance(gs_handle* h, const double* znet, int nz, int n_z, double* current_z, double* zstep,
               unsigned* step_n, int max_calls, int* calls_done, int* reached);

/* The handle's CUDA stream (a cudaStream_t), for callers that time or order work on it. */
void* gs_stream(const gs_handle* h);

/* Number of kernel launches issued on the handle's stream since creation. */
long long gs_launch_count(const gs_handle* h);

/* CUDA-event timing of the fused QDHT + linear-step kernels (the pair launched by each
 * accepted gs_step / gs_lstep), on the handle's stream.  Returns the milliseconds and
 * launch count accumulated since the previous call, then resets them; enable != 0 keeps
 * timing on.  No extra synchronisation: the step's own final sync is reused. */
int gs_qdht_timing(gs_handle* h, int enable, double* ms_total, int* launches);

/* The same for the fused RK4-stage kernels of gs_nl_step / gs_step (rows that fit one CTA;
 * no counterpart in the reference, which has no kernels to time): milliseconds of their
 * launches, the number of RK4 stages and of launches timed since the previous call (a launch
 * runs one stage, or all four on large grids), by CUDA events around each launch on the
 * handle's stream; enable != 0 keeps timing on.  Any output may be NULL. */
int gs_nl_timing(gs_handle* h, int enable, double* ms, int* stages, int* launches);

/* Reductions of the current FIELD behind the reference's .udf dumps (dump_types.cpp,
 * FILTER_TYPE NO), computed on the device; any output may be NULL:
 *   max_I[n_r], flux[n_r]   dump_type_maxI_class / dump_type_flux_class (104-165)
 *   plasma_max[n_r]         dump_type_plasma_max_class (535-555)
 *   field_axis[n_t]         complex E(t) at r = 0, dump_type_field_axis_class (404-417)
 *   avg_spectrum[n_t]       dump_type_average_spectrum_class (427-457); needs qdht_x (the
 *                           QDHT points x_n) and r_max */
int gs_dump_reductions(gs_handle* h, const double* qdht_x, double r_max, double* max_I, double* flux,
                       double* plasma_max, double* field_axis, double* avg_spectrum);

/* The time-domain field BW-FFT(FIELD)/N_T, [n_r][n_t] complex: dump_type_full_class (77-97). */
int gs_get_time_field(gs_handle* h, double* e_r_t);

/* Autotuning (no counterpart in the reference): times the launch shapes of the fused
 * RK4-stage kernels (threads per radial row, which also sets the recurrences' chunk length)
 * on this handle's grid and field and keeps the fastest; the choice is cached per
 * (precision, n_r, n_t) for the process.  Needs tables and field; leaves FIELD and
 * BIGBUFFER2 unchanged.  Results stay within the parity bounds for every shape (the chunking
 * of the recurrences only reorders roundings). */
int gs_autotune(gs_handle* h, int* threads, double* ms_per_stage);
/* Set (0: the default) or read the fused kernels' threads per row for this handle. */
int gs_set_nl_threads(gs_handle* h, int threads);
int gs_get_nl_threads(const gs_handle* h);

/* ---- Gradients (no counterpart in the reference: it has no adjoint) ----------------------
 * A run of n_steps propagator() calls with the step sizes given instead of chosen by the
 * controller: step n uses dz_rk[n] in its RK4 stages and dz_lin[n] in its linear step (the
 * old and the new ZSTEP of propagator.cu:139-194), so that a controller-driven run can be
 * replayed and differentiated exactly.  The objective is
 *   J = sum_{r, omega} weights[r][omega] |FIELD(r, omega)|^2   after the last step
 * (weights [n_r][n_t] doubles: e.g. the average_spectrum radial weights inside a spectral
 * band, dump_types.cpp:427-457).  Fields are [n_r][n_t] complex (interleaved doubles) on the
 * host; on return the handle holds the final state of the forward run. */
int gs_forward_fixed(gs_handle* h, const double* field_in, int n_steps, const double* dz_rk, const double* dz_lin,
                     const double* weights, double* objective, double* field_out);
/* J as above and grad_field = dJ/dRe(FIELD_0) + i dJ/dIm(FIELD_0) by the hand-written adjoint,
 * with checkpoints every checkpoint_stride steps and the steps of each segment but the last
 * re-run from its checkpoint.  checkpoint_stride 0: every step recorded during the forward
 * (no re-run) when the record fits in half of the free device memory, else the largest
 * stride that fits, at least ceil(sqrt(n_steps)); gs_adjoint_stride reports the one used.  Needs rows that fit one CTA (n_t <= 8192 mixed,
 * <= 4096 FP64) and, with Raman on, the oscillator parameters (raman_tau, raman_omega). */
int gs_gradient(gs_handle* h, const double* field_in, int n_steps, const double* dz_rk, const double* dz_lin,
                const double* weights, int checkpoint_stride, double* objective, double* grad_field);
/* The checkpoint stride of the last gs_gradient call on the handle (0 before the first; no
 * counterpart in the reference). */
int gs_adjoint_stride(gs_handle* h, int* stride);
/* One step of the adjoint from the handle's current state (FIELD_n, BIGBUFFER2_n): the step
 * is run forward (the handle then holds state n+1) and the cotangents of FIELD (r,omega) and
 * BIGBUFFER2 (k,omega) after it, field_bar and spec_bar, are replaced by those before it. */
int gs_adjoint_step(gs_handle* h, double dz_rk, double dz_lin, double* field_bar, double* spec_bar);

/* ---- Batches of independent pulses (no counterpart in the reference: one pulse per job) ----
 * A batch advances n pulses (each its own handle, grid, tables and stream, all on one
 * device) together: one z-step of the batch is every pulse's propagator() work with a
 * fixed step size dz[i] (RK4 stages and linear step), issued concurrently.  With use_graph
 * the z-step is captured once into a CUDA graph and replayed (one launch per z-step); a
 * different dz array captures a new graph.  Blast / NaN / tensor-core wait errors are
 * checked after the n_steps and name the pulse.  The pulses' handles stay owned by the
 * caller and must outlive the batch; gs_batch_advance runs the adaptive controller. */
typedef struct gs_batch gs_batch;
int gs_batch_create(int n, gs_handle* const* pulses, gs_batch** out);
int gs_batch_step(gs_batch* b, int n_steps, const double* dz, int use_graph);
/* The batch's cudaStream_t (the graph launches on it; it joins every pulse's stream). */
void* gs_batch_stream(const gs_batch* b);
/* Kernels issued by the batch (a graph replay counts its kernel nodes). */
long long gs_batch_launch_count(const gs_batch* b);
const char* gs_batch_last_error(const gs_batch* b);
/* Chooses, for the batch as a whole, between the default launch shapes and each pulse's own
 * gs_autotune shape by timing one graph z-step each way from the same state (the pulses'
 * FIELD and BIGBUFFER2 are restored afterwards); keeps the faster. */
int gs_batch_autotune(gs_batch* b, const double* dz, double* ms_default, double* ms_tuned, int* chose_tuned);
/* The z-loops of all pulses advanced together with the adaptive controller: gs_advance for
 * every pulse (propagator()'s controller and the loop's bookkeeping on the device,
 * solver_main.cpp:202-225, propagator.cu:139-164), one graph launch per attempt of all pulses.
 * Per pulse i: its ZNET (znet[i], nz[i] points), the next dump index n_z[i], CURRENT_Z, ZSTEP
 * and STEP_N in and out, at most max_calls accepted calls; calls_done[i] and reached[i]
 * (CURRENT_Z >= ZNET[n_z[i]]) out.  A pulse that reaches its ZNET point or its call budget
 * stops while the others go on; each pulse's results are bit for bit those of gs_advance on
 * it alone.  Mixed pulses whose NL kernels take their step size from the device (the fused
 * stage kernels: rows that fit one CTA with the Raman recurrence, one ionization level), no
 * photon-number check, no aperture; others give GS_ERR_UNSUPPORTED. */
int gs_batch_advance(gs_batch* b, const double* const* znet, const int* nz, const int* n_z, double* current_z,
                     double* zstep, unsigned* step_n, int max_calls, int* calls_done, int* reached);
int gs_batch_destroy(gs_batch* b);

/* Carrier-density maxima without any device allocation.  No counterpart in the reference:
 * it is an addition for host code that cannot allocate device memory where it needs this
 * result (for example an application whose own allocator has reserved the GPU's memory and
 * refuses further cudaMalloc calls from the libraries it links).  It runs the FP64 Heun
 * recurrence of the carrier density (photoionization from the rate table, avalanche,
 * recombination), then takes each row's maximum over time, on caller-owned device buffers:
 *   e_r_t_dev[rows][n_t]  complex time-domain field (interleaved doubles)
 *   rate_ln_dev[8192]     the log photoionization-rate table
 *   plasma_max_dev[rows]  output: max over t of the carrier density per row
 * with the scalars of *params (n_t and the plasma constants), on `stream` (a cudaStream_t,
 * NULL for the default stream); it synchronises that stream before returning.  Its scratch
 * is one fixed 16 MiB array inside the library, held on every GPU that loads the library
 * until the process exits; rows * n_t may not exceed gs_noalloc_max_samples() (524,280) —
 * larger requests are refused with GS_ERR_ARG.  Each call looks up the array's device address
 * on the current device (no allocation); the first call on a device also loads the library's
 * device code there, so make that first call before any stream capture begins.  All calls
 * share the array, so calls that overlap on the GPU (other streams, other host threads) race. */
int gs_plasma_max_noalloc(const gs_params* params, const double* rate_ln_dev, const double* e_r_t_dev, int rows,
                          double* plasma_max_dev, void* stream);
/* Largest rows * n_t accepted by gs_plasma_max_noalloc. */
size_t gs_noalloc_max_samples(void);
/* Message of the last failed gs_plasma_max_noalloc call. */
const char* gs_noalloc_last_error(void);

/* Energy and photon number of FIELD, FP64 reductions on the device: energy is the sum over
 * omega of the reference's average spectrum (dump_type_average_spectrum_class,
 * dump_types.cpp:427-457: R_MAX^2/2 sum_r w_r |FIELD(r, omega)|^2, w_0 = x_0 (x_1 - x_0),
 * w_r = x_r (x_r - x_{r-1}), x the QDHT points qdht_x[n_r]); photons weights each omega > 0 by
 * 1 / omega.  Units are the reference's scaled field units.  Either output may be NULL. */
int gs_energy(gs_handle* h, const double* qdht_x, double r_max, double* energy, double* photons);
/* Optional photon-number check of gs_step (no counterpart in the reference, whose controller is
 * the max-ratio rule of propagator.cu:147-150; 0, the default, keeps it that way): after each
 * accepted attempt's linear step, while |N_after / N_before - 1| > tol (N the photon number of
 * gs_energy) BIGBUFFER2 is restored and the linear step repeated with half the step (the NL
 * increment, taken with the previous step size as propagator() does, is reused); the step taken
 * is returned in zstep_inout.  A step below 1e-10 of the ZNET interval fails with
 * GS_ERR_COLLAPSE.  Plasma absorption and the absorbing layer remove photons; Kerr, Raman and
 * dispersion conserve them, so the check bounds the loss per step. */
int gs_set_energy_tolerance(gs_handle* h, double tol, const double* qdht_x, double r_max);
/* |N_after / N_before - 1| of the last step accepted by the check, and the rejections so far. */
int gs_energy_stats(const gs_handle* h, double* last_rel_change, long long* rejections);

/* Checkpoints of a handle's state (the reference restarts from its full-field dump,
 * dump_type_full_class, dump_types.cpp:77-97, and DUMP_FINAL_FIELD, solver_main.cpp:226-229):
 * FIELD, BIGBUFFER2 (with the mixed plan's double-float window columns) as stored on the device,
 * and the z-loop's CURRENT_Z, ZSTEP, n_Z and STEP_N, in a binary file.  Loading into a handle of
 * the same grid, precision and tables continues exactly where the saved one was. */
int gs_checkpoint_save(gs_handle* h, const char* path, double current_z, double zstep, int n_z, unsigned step_n);
int gs_checkpoint_load(gs_handle* h, const char* path, double* current_z, double* zstep, int* n_z, unsigned* step_n);

/* Self-test of the tensor-core kernels' bounded waits (no counterpart in the reference): a
 * kernel waits limit_s (at most 1 s) on a barrier that nothing completes, using the same bounded
 * wait and expiry record as the QDHT GEMM, and returns; the call then reports the record as a
 * GEMM's expired wait is reported: GS_ERR_CUDA with "wait expired" in gs_last_error.  The handle
 * stays usable.  Mixed handles only. */
int gs_selftest_bounded_wait(gs_handle* h, double limit_s);

/* 1 when the library was built with GS_CHECK (`python -m gsolver_gb300.build --check`): the hot
 * kernels test the indices they take from index tables (compact-column maps, rate-table rows)
 * before each access, skip a failing access and report it as GS_ERR_CUDA "index out of bounds
 * (GS_CHECK build)" from the call; else 0. */
int gs_check_build(void);

/* Self-test of the GS_CHECK index test (no counterpart in the reference): a kernel tests an index
 * one past the length it declares for a buffer that is larger (so the access could not fault
 * either way); the test fails, the access is skipped, and the call returns GS_ERR_CUDA with the
 * bounds message, the handle usable.  Builds without GS_CHECK return GS_ERR_UNSUPPORTED and
 * launch nothing. */
int gs_selftest_bounds(gs_handle* h);

/* Apertures (propagator.cu:232-261, process_input.cpp:176-179): n entries in the reference's
 * array order (z[n-1], r[n-1] is the first applied).  gs_step then applies them as
 * propagator() does: after an accepted step, when current_z (the z before the step) has
 * reached z[k-1] of the next aperture k, FIELD rows with qdht_x[row] * r_max > r[k-1] are
 * zeroed, BIGBUFFER2 = QDHT(FIELD), and the aperture is used up.  Calling again resets them. */
int gs_set_apertures(gs_handle* h, int n, const double* z, const double* r, const double* qdht_x, double r_max);

/* Release all device state. */
int gs_destroy(gs_handle* h);

/* Message of the last failed call on h (or of the last gs_create failure if h is NULL). */
const char* gs_last_error(const gs_handle* h);

/* Fixed string for a status code. */
const char* gs_status_string(int status);

#ifdef __cplusplus
}
#endif
#endif
