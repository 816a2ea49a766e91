/*
 * gs_oracle.h -- CPU oracle for the gsolver_solid_qdht z-step (TEST INFRASTRUCTURE).
 *
 * This is a plain-C FP64 restatement of the reference's hot path, used only by
 * tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm as
 * the checker.  It is never linked into the product library.
 *
 * Reference build flags restated: KELDYSH_IONIZATION, _ODE_RK4, PLASMA_DISPERSION,
 * QDHT, _UNIAXIAL, TRANSVERSE_DIMENSIONS=1, plus NONLINEARITY_ON (switchable through
 * gso_ctx.nonlinear so that the shipped linear-only build can be restated too).
 *
 * Complex arrays are interleaved (re, im) doubles, row-major [n_r][n_t], omega
 * contiguous -- the layout of FIELD/BIGBUFFER1/BIGBUFFER2 (propagator.cu:380,593).
 */
#ifndef GS_ORACLE_H
#define GS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    GSO_OK = 0,
    GSO_ERR_BLAST = 1,     /* ionization.cpp:114-118 "Intensity is too big" */
    GSO_ERR_NAN = 2,       /* ionization.cpp:104-105 "Intensity is nan" */
    GSO_ERR_COLLAPSE = 3,  /* propagator.cu:159-163 "Minimum Z step size reached" */
    GSO_ERR_ARG = 4
};

typedef struct gso_ctx {
    int n_r, n_t;
    int nonlinear;        /* 1: NONLINEARITY_ON defined; 0: the shipped build (zero NL response) */
    int nthreads;         /* OpenMP threads for the row / column loops (<=0: library default) */

    /* NL response scalars, already in the reference's scaled units
       (solver_main.cpp:385-393, ionization.cpp:11) */
    double tstep;             /* TSTEP [s] */
    double tmin, tmax, omega0;
    double ionrate_denom;     /* IONRATE_DENOM (1e20 for solids) */
    double neutral_density;
    double rho0;              /* AMBIENT_CARRIER_DENSITY*2*frand() restated as a fixed value */
    double ionization_potential;   /* U_i * IONRATE_DENOM/INTENSITY_DENOM */
    double ponderomotive;          /* PONDEROMOTIVE_COEFFICIENT * IONRATE_DENOM */
    double avalanche_cs;           /* AVALANCHE_CROSSSECTION */
    double recombination_tau;      /* RECOMBINATION_TAU * IONRATE_DENOM */
    double raman_fraction;
    double n2;                     /* NONLIN_REFRINDEX * INTENSITY_DENOM */
    const double* rate_ln;         /* IONIZATION_RATE_LN[8192] */
    const double* plasma_func;     /* complex [n_t] */
    const double* raman_func;      /* complex [n_t] */
    const double* kerr;            /* [n_t] */

    /* linear step (propagator.cu:570-625) */
    const double* omega;           /* [n_t] */
    const double* wavenum;         /* complex [n_t] */
    const double* ho_disp;         /* [n_t] */
    double omega_min, omega_max;
    const double* kt2;             /* [n_r]  (2*pi*x_n*V/R_MAX)^2 */

    /* QDHT (fhatha.cpp:177-230): C[i + N*j], m1[i] */
    const double* qdht_c;
    const double* qdht_m1;

    /* z-step controller */
    double max_tolerance;

    /* gas build (gsolver_gas_qdht, Makefile:19: PPT_IONIZATION, MULTI_LEVEL_IONIZATION,
       THIRD_HARMONICS; IONRATE_DENOM 1e10): gas != 0 selects the multi-level ionization of
       ionization.cpp:45-84 with `levels` rate tables (rate_ln holds levels x 8192) and
       potentials[levels] (scaled as IONIZATION_POTENTIAL); th_coeff = (1 - fR)/3 TH_FACTOR
       (KERR_TH_PROFILE = KERR_PROFILE th_coeff, process_input.cpp:1020), 0 = no third
       harmonic. */
    int gas;
    int levels;
    const double* potentials;
    double th_coeff;
} gso_ctx;

/* FFTW-convention unnormalised DFT: sign=-1 FFTW_FORWARD, sign=+1 FFTW_BACKWARD. */
int gso_fft(int n, const double* in, double* out, int sign);

/* qdht_plan::run_many (fhatha.cpp:218-230). */
int gso_qdht_run_many(const gso_ctx* c, double* data, long nN, long stride, long dist);

/* calculate_plasmadensity_losses_small (ionization.cpp:9-95), single-level branch.
   pro may be NULL; loss may be NULL. */
int gso_plasma_losses(const gso_ctx* c, const double* field, double* pro, int stride, double* loss);

/* calculate_NLresponse (propagator.cu:629-783) for one radial row. */
int gso_nl_response(const gso_ctx* c, const double* in, double* out);

/* calculate_NLstep CPU branch (propagator.cu:375-425): RK4 over all rows. */
int gso_nl_step(const gso_ctx* c, const double* field, double* bb1, double zstep,
                double* max_a2, double* max_nl2);

/* calculate_Lstep CPU branch (propagator.cu:570-625). */
int gso_lstep(const gso_ctx* c, double* field, const double* bb1, double* bb2, double zstep);

/* propagator() (propagator.cu:125-266) without apertures: repeats attempts until accepted.
   zstep, step_n are in/out; znet_cur = ZNET[n_Z], znet_prev = ZNET[n_Z-1]. */
int gso_propagator(const gso_ctx* c, double* field, double* bb1, double* bb2,
                   double* zstep, double current_z, double znet_cur, double znet_prev,
                   unsigned* step_n, double* max_a2_out, double* max_nl2_out);

/* Per-row time-domain reductions used by the .udf dumps (dump_types.cpp:104-165, 535-555):
   out_maxI[r], out_flux[r] (times tstep), out_pmax[r]; any may be NULL. */
int gso_row_reductions(const gso_ctx* c, const double* field, double* out_maxI,
                       double* out_flux, double* out_pmax);

/* ---- adjoint (gs_oracle_adj.c): cotangents g = dJ/dRe + i dJ/dIm of a real objective ---- */

/* (dN/dY)^H kbar for calculate_NLresponse at the spectral row Y. */
int gso_nl_response_vjp(const gso_ctx* c, const double* Y, const double* kbar, double* ybar);

/* Adjoint of calculate_NLstep's RK4 increment at FIELD = field with stage step zstep:
   abar = (dR/dA)^H rbar over all rows. */
int gso_nl_step_vjp(const gso_ctx* c, const double* field, double zstep, const double* rbar, double* abar);

/* Adjoint of calculate_Lstep: fbar = cotangent of FIELD (k,omega) after the step, sbar
   in: of BIGBUFFER2 after, out: before; b1bar out: of BIGBUFFER1 (k,omega). */
int gso_lstep_vjp(const gso_ctx* c, const double* fbar, double* sbar, double* b1bar, double zstep);

/* Transposed QDHT in place: per column x *= m1; y = C x; y /= m1 (H^T, C symmetric). */
int gso_qdht_transposed(const gso_ctx* c, double* data);

#ifdef __cplusplus
}
#endif
#endif
