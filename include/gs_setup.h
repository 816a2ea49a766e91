/*
 * gs_setup.h -- host set-up of one pulse from a reference-format config (C ABI).
 *
 * Builds, in FP64 on the host, everything the z-step core needs before its loop: the
 * gs_params scalars, the gs_tables arrays, the start field and the z net.  Reference
 * start-up replaced (paths within the reference project):
 *   gs_setup_from_config  <- process_input() (process_input.cpp:33-95): load_info,
 *                            load_nonlindata, initialize_variables (solver_main.cpp:265-398),
 *                            calc_ionization_rate (ionization.cpp:313-355),
 *                            calc_raman_function (solver_main.cpp:401-413),
 *                            load_kerr_th_profiles (process_input.cpp:966-975),
 *                            create_gg (pulse_gg.cpp:6-124), init_zstep_kerr (734-753)
 *   overrides             <- the argv "KEY value" pairs every load_named* consults first
 * The config's DISPERSION_FILE is resolved relative to the config file's directory.
 * Start-field noise: noise_sigma != 0 multiplies the carrier by (1 + sigma (n1 + i n2))
 * with seeded normals n1, n2 (splitmix64 + Box-Muller) in place of the reference's
 * unseeded uniform NOISE_LEVEL draw.
 */
#ifndef GS_SETUP_H
#define GS_SETUP_H

#include "gs_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gs_setup gs_setup;

int gs_setup_from_config(const char* config_path, int n_overrides, const char* const* keys,
                         const char* const* values, unsigned long long noise_seed, double noise_sigma,
                         gs_setup** out);
/* The same set-up with its FP64 builds on GPU `device` (no counterpart in the reference, whose
   initialisation is host code): the ionization-rate table (Keldysh or PPT series), the QDHT
   matrix C (N_r^2 Bessel J0 values) and create_gg's start field (envelope, seeded noise, an
   FFT per row) with the maximum intensity of init_zstep_kerr; the per-omega tables stay on
   the host.  Results agree with gs_setup_from_config to the roundings of the two math
   libraries (relative 1e-13 or better), so batched scans can skip the host's O(N_r N_T) work. */
int gs_setup_from_config_dev(const char* path, int n_over, const char* const* keys, const char* const* vals,
                             unsigned long long noise_seed, double noise_sigma, int device, gs_setup** out);
const char* gs_setup_last_error(void);
int gs_setup_grid(const gs_setup* s, int* n_r, int* n_t, int* n_z);
/* scalars; the caller sets precision, nonlinear and device before gs_create */
/* Apertures (process_input.cpp:176-179, propagator.cu:232-261): *n entries in the
   reference's array order (entry n-1, APERTURE_Z0/R0, is applied first); z, r may be NULL. */
int gs_setup_apertures(const gs_setup* s, int* n, double* z, double* r);
int gs_setup_params(const gs_setup* s, gs_params* out);
/* pointers into memory owned by s (valid until gs_setup_destroy) */
int gs_setup_tables(const gs_setup* s, gs_tables* out);
/* start FIELD (r, omega), n_r*n_t interleaved complex, already divided by FIELD_DENOM */
int gs_setup_field(const gs_setup* s, double* field_r_omega);
/* ZNET[n_z], the first ZSTEP, R_MAX and the QDHT points x_n (r = x_n * R_MAX); any may be NULL */
int gs_setup_znet(const gs_setup* s, double* znet, double* init_zstep, double* r_max, double* qdht_x);
int gs_setup_destroy(gs_setup* s);

/* Outcome of gs_run_config. */
typedef struct gs_run_stats {
    long long calls;      /* propagator() calls */
    unsigned step_n;      /* STEP_N (accepted + rejected attempts, as the reference counts) */
    int n_z;              /* last ZNET index reached */
    double z, zstep;      /* CURRENT_Z, ZSTEP at exit */
    double seconds;       /* wall time of the z-loop */
} gs_run_stats;

/* The whole run of one config on one GPU: main() of the reference (solver_main.cpp:151-251)
 * with the z-loop (202-225) and the .udf dumps (dumps.cpp, dump_types.cpp: flux, maxI,
 * field_axis, plasma_max, average_spectrum, full; FILTER_TYPE NO) written under out_dir with
 * the reference's file layout.  max_calls < 0 runs to the last ZNET point. */
int gs_run_config(const char* config_path, const char* out_dir, int n_overrides, const char* const* keys,
                  const char* const* values, int precision, int device, unsigned long long noise_seed,
                  double noise_sigma, long long max_calls, gs_run_stats* stats);
const char* gs_run_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
