/*
 * gs_oracle.c -- CPU oracle for the gsolver_solid_qdht z-step (TEST INFRASTRUCTURE).
 *
 * FP64 restatement of the reference algorithm, function by function, with the
 * reference's order of floating-point operations kept wherever it is visible in the
 * source.  Used only as the checker by tests/, smoke() and bench.py's CPU legs.
 * Compile with -ffp-contract=off so that x86 and aarch64 round identically.
 *
 * Third-party arithmetic the reference pulls in and that is restated here:
 *   FFTW3 (version unpinned by the reference Makefile:45): an unnormalised complex DFT
 *   with FFTW's sign convention, computed here by a radix-4 Stockham autosort FFT (a final
 *   radix-2 pass for odd powers of two).
 */
#include "gs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#else
static int omp_get_max_threads(void) { return 1; }
#endif

#define IONIZATION_I_LN_TOLERANCE 0.003304003148325   /* solver.h:63 */
#define IONIZATION_MIN_I_LN 29.933606208922594        /* solver.h:64 */
#define IONIZATION_MIN_I 1e13                         /* solver.h:65 */
#define IONIZATION_N 8192                             /* solver.h:67 */
#define INTENSITY_DENOM 1e16                          /* solver.h:72 */
#define INTENSITY_DENOM_LN 36.841361487904734         /* solver.h:74 */
#define MINSTEP_RATIO 1e-10                           /* solver.h:55 */
#define MAX_KT2 0.25                                  /* solver.h:107 */

/* ------------------------------------------------------------------ FFT -- */

typedef struct { int n; double* tw; } fft_tab;
static fft_tab g_tabs[16];
static int g_ntabs = 0;

/* tw[j] = (cos, sin)(2 pi j / n), j < n, each rounded once from the libm value */
static const fft_tab* get_tab(int n)
{
    const fft_tab* found = NULL;
#pragma omp critical(gso_fft_tab)
    {
        for (int i = 0; i < g_ntabs; i++) if (g_tabs[i].n == n) found = &g_tabs[i];
        if (!found && g_ntabs < 16) {
            fft_tab* t = &g_tabs[g_ntabs];
            t->n = n;
            t->tw = (double*)malloc(sizeof(double) * 2 * (size_t)n);
            for (int j = 0; j < n; j++) {
                double a = 2.0 * M_PI * (double)j / (double)n;
                t->tw[2 * j] = cos(a);
                t->tw[2 * j + 1] = sin(a);
            }
            g_ntabs++;
            found = t;
        }
    }
    return found;
}

/* One radix-4 pass of the Stockham autosort FFT (the published self-sorting formulation:
 * no bit reversal, the output of each pass in natural order of its sub-transforms): x holds
 * s interleaved sequences of length m = 4 m1, y receives them transformed by one radix-4
 * step with the twiddles w_m^{p}, w_m^{2p}, w_m^{3p} (w_m = exp(sign 2 pi i / m) = tw[N/m]). */
static void stockham4(int m, int s, int sign, const double* tw, int tstride, const double* x, double* y)
{
    const int m1 = m / 4;
    for (int p = 0; p < m1; p++) {
        const double* w1 = tw + 2 * (size_t)(p * tstride);
        const double* w2 = tw + 2 * (size_t)(2 * p * tstride);
        const double* w3 = tw + 2 * (size_t)(3 * p * tstride);
        const double w1r = w1[0], w1i = sign * w1[1], w2r = w2[0], w2i = sign * w2[1];
        const double w3r = w3[0], w3i = sign * w3[1];
        for (int q = 0; q < s; q++) {
            const double* a = x + 2 * ((size_t)q + (size_t)s * p);
            const double* b = x + 2 * ((size_t)q + (size_t)s * (p + m1));
            const double* c = x + 2 * ((size_t)q + (size_t)s * (p + 2 * m1));
            const double* d = x + 2 * ((size_t)q + (size_t)s * (p + 3 * m1));
            const double apcr = a[0] + c[0], apci = a[1] + c[1];
            const double amcr = a[0] - c[0], amci = a[1] - c[1];
            const double bpdr = b[0] + d[0], bpdi = b[1] + d[1];
            /* sign i (b - d) */
            const double jr = -sign * (b[1] - d[1]), ji = sign * (b[0] - d[0]);
            double* o = y + 2 * ((size_t)q + (size_t)s * 4 * p);
            const double r1 = amcr + jr, i1 = amci + ji;
            const double r2 = apcr - bpdr, i2 = apci - bpdi;
            const double r3 = amcr - jr, i3 = amci - ji;
            o[0] = apcr + bpdr;
            o[1] = apci + bpdi;
            o[2 * s] = r1 * w1r - i1 * w1i;
            o[2 * s + 1] = r1 * w1i + i1 * w1r;
            o[4 * s] = r2 * w2r - i2 * w2i;
            o[4 * s + 1] = r2 * w2i + i2 * w2r;
            o[6 * s] = r3 * w3r - i3 * w3i;
            o[6 * s + 1] = r3 * w3i + i3 * w3r;
        }
    }
}

int gso_fft(int n, const double* in, double* out, int sign)
{
    if (n <= 0) return GSO_ERR_ARG;
    if (n & (n - 1)) {
        /* plain DFT for lengths that are not powers of two */
        double* tmp = (double*)malloc(sizeof(double) * 2 * (size_t)n);
        for (int k = 0; k < n; k++) {
            double sr = 0, si = 0;
            for (int j = 0; j < n; j++) {
                double a = sign * 2.0 * M_PI * (double)(((long)j * k) % n) / (double)n;
                double c = cos(a), s = sin(a);
                sr += in[2 * j] * c - in[2 * j + 1] * s;
                si += in[2 * j] * s + in[2 * j + 1] * c;
            }
            tmp[2 * k] = sr; tmp[2 * k + 1] = si;
        }
        memcpy(out, tmp, sizeof(double) * 2 * (size_t)n);
        free(tmp);
        return GSO_OK;
    }
    if (n == 1) {
        out[0] = in[0];
        out[1] = in[1];
        return GSO_OK;
    }
    const fft_tab* t = get_tab(n);
    if (!t) return GSO_ERR_ARG;
    /* radix-4 Stockham passes, then one radix-2 pass when log2 n is odd; the first pass reads
     * `in`, the last writes `out`, the ones between alternate over two per-thread scratch rows
     * (so in == out is allowed) */
    static _Thread_local double* scratch = NULL;
    static _Thread_local size_t scratch_n = 0;
    if (scratch_n < (size_t)n) {
        free(scratch);
        scratch = (double*)malloc(sizeof(double) * 4 * (size_t)n);
        scratch_n = scratch ? (size_t)n : 0;
        if (!scratch) return GSO_ERR_ARG;
    }
    int passes = 0, lg = 0;
    while ((1 << lg) < n) lg++;
    passes = lg / 2 + (lg & 1);
    double* bufs[2] = {scratch, scratch + 2 * (size_t)n};
    const double* x = in;
    int m = n, s = 1;
    for (int k = 0; k < passes; k++) {
        /* pass k writes buffer (passes - 1 - k) % 2 of the scratch, the last one `out`; with a
         * single pass and in == out it goes through the scratch */
        double* y = (k == passes - 1 && !(passes == 1 && in == out)) ? out : bufs[(passes - 1 - k) & 1];
        if (m >= 4) {
            stockham4(m, s, sign, t->tw, n / m, x, y);
            m /= 4;
            s *= 4;
        } else {   /* m == 2 */
            for (int q = 0; q < s; q++) {
                const double* a = x + 2 * (size_t)q;
                const double* b = x + 2 * ((size_t)q + (size_t)s);
                double* o = y + 2 * (size_t)q;
                o[0] = a[0] + b[0];
                o[1] = a[1] + b[1];
                o[2 * s] = a[0] - b[0];
                o[2 * s + 1] = a[1] - b[1];
            }
            m = 1;
        }
        x = y;
    }
    if (x != out) memcpy(out, x, sizeof(double) * 2 * (size_t)n);
    return GSO_OK;
}

/* ----------------------------------------------------------------- QDHT -- */

int gso_qdht_run_many(const gso_ctx* c, double* data, long nN, long stride, long dist)
{
    const long N = c->n_r;
    const double* C = c->qdht_c;
    const double* m1 = c->qdht_m1;
    /* fhatha.cpp:218-230: per column n: x/=m1; y_i = sum_j C[i+N*j] x_j (j ascending);
       x = y*m1.  Columns are processed in blocks so that the strided gathers stay in
       cache; the per-output summation order is the reference's. */
    const long B = 16;
#pragma omp parallel for schedule(dynamic) num_threads(c->nthreads > 0 ? c->nthreads : omp_get_max_threads())
    for (long n0 = 0; n0 < nN; n0 += B) {
        long nb = (nN - n0 < B) ? (nN - n0) : B;
        double* x = (double*)malloc(sizeof(double) * 2 * (size_t)(N * B));
        double* y = (double*)malloc(sizeof(double) * 2 * (size_t)B);
        for (long j = 0; j < N; j++)
            for (long b = 0; b < nb; b++) {
                const double* s = data + 2 * ((n0 + b) * dist + j * stride);
                x[2 * (j * B + b)] = s[0] / m1[j];
                x[2 * (j * B + b) + 1] = s[1] / m1[j];
            }
        for (long i = 0; i < N; i++) {
            for (long b = 0; b < nb; b++) { y[2 * b] = 0; y[2 * b + 1] = 0; }
            for (long j = 0; j < N; j++) {
                double cij = C[i + N * j];
                const double* xj = x + 2 * j * B;
                for (long b = 0; b < nb; b++) {
                    y[2 * b] += cij * xj[2 * b];
                    y[2 * b + 1] += cij * xj[2 * b + 1];
                }
            }
            for (long b = 0; b < nb; b++) {
                double* d = data + 2 * ((n0 + b) * dist + i * stride);
                d[0] = y[2 * b] * m1[i];
                d[1] = y[2 * b + 1] * m1[i];
            }
        }
        free(x); free(y);
    }
    return GSO_OK;
}

/* ------------------------------------------------------------- ionization -- */

/* photoionization_function (ionization.cpp:98-147), KELDYSH solid branch.
   Returns the rate; *err set on NaN / table overflow. */
static double photoionization(const gso_ctx* c, double I, double ro, int* err)
{
    if (I < (IONIZATION_MIN_I / INTENSITY_DENOM)) return 0;
    if (ro > c->neutral_density) return 0;
    double lnI = log(I) + INTENSITY_DENOM_LN;
    if (isnan(lnI)) { *err = GSO_ERR_NAN; return 0; }
    int n = (int)floor((lnI - IONIZATION_MIN_I_LN) / IONIZATION_I_LN_TOLERANCE);
    if (n > IONIZATION_N - 2) { *err = GSO_ERR_BLAST; return 0; }
    if (n < 0) return 0;
    double lnIn = IONIZATION_MIN_I_LN + n * IONIZATION_I_LN_TOLERANCE;
    double lnWn = c->rate_ln[n];
    double lnWnp = c->rate_ln[n + 1];
    double lnW = lnWn + (lnI - lnIn) * (lnWnp - lnWn) / IONIZATION_I_LN_TOLERANCE;
    return exp(lnW);
}

/* avalanche_ionization_function (ionization.h:77-83) */
static double avalanche(const gso_ctx* c, double I, double ro)
{
    if (ro < 0 || ro > c->neutral_density) return 0;
    return c->avalanche_cs / (c->ionization_potential + c->ponderomotive * I) * I * ro *
           (1 - ro / c->neutral_density);
}

/* recombination_function (ionization.h:84-87) */
static double recombination(const gso_ctx* c, double ro)
{
    return (ro > 0) ? (ro / c->recombination_tau) : 0;
}

/* photoionization_functionsN (ionization.cpp:150-199), PPT, no Yudin-Ivanov correction:
   W[i] = exp(lnW_i(I)) per level, 0 below IONIZATION_MIN_I; the reference's CPU branch
   throws for n < 0 (an intensity a rounding below the table), its GPU branch returns 0:
   the GPU behaviour is kept. */
static void gas_rates(const gso_ctx* c, double I, double* W, int* err)
{
    for (int i = 0; i < c->levels; i++) W[i] = 0;
    if (I < IONIZATION_MIN_I / INTENSITY_DENOM) return;
    double lnI = log(I) + INTENSITY_DENOM_LN;
    if (isnan(lnI)) { *err = GSO_ERR_NAN; return; }
    int n = (int)floor((lnI - IONIZATION_MIN_I_LN) / IONIZATION_I_LN_TOLERANCE);
    if (n > IONIZATION_N - 2) { *err = GSO_ERR_BLAST; return; }
    if (n < 0) return;
    for (int i = 0; i < c->levels; i++) {
        double lnIn = IONIZATION_MIN_I_LN + n * IONIZATION_I_LN_TOLERANCE;
        double lnWn = c->rate_ln[IONIZATION_N * i + n];
        double lnWnp = c->rate_ln[IONIZATION_N * i + n + 1];
        double lnW = lnWn + (lnI - lnIn) * (lnWnp - lnWn) / IONIZATION_I_LN_TOLERANCE;
        W[i] = exp(lnW);
    }
}

/* calculate_plasmadensity_losses_small, MULTI_LEVEL_IONIZATION branch (ionization.cpp:
   19-24, 45-84): per level Heun steps on the ion densities (no avalanche, no
   recombination), taken only where the previous sample's intensity exceeds
   IONIZATION_MIN_I; pro = sum of the levels; loss[nt-1] = tl E[nt-1]. */
static int plasma_losses_gas(const gso_ctx* c, const double* field, double* pro, int stride, double* loss)
{
    const int N = c->n_t, L = c->levels;
    const double tstep = c->tstep * c->ionrate_denom, ND = c->neutral_density, Pc = c->ponderomotive;
    double ro[16] = {0}, W[32];
    int err = GSO_OK;
    if (L < 1 || L > 16) return GSO_ERR_ARG;
    if (loss) { loss[0] = 0; loss[1] = 0; }
    if (pro) pro[0] = 0;
    double I0 = 0;
    for (int nt = 1; nt < N; nt++) {
        double ph = -c->omega0 * (c->tmin + nt * (c->tmax - c->tmin) / N);
        double pr = cos(ph), pi = sin(ph);
        double er = field[2 * nt], ei = field[2 * nt + 1];
        double reE1 = er * pr - ei * pi, imE1 = er * pi + ei * pr;
        double I1 = reE1 * reE1 + imE1 * imE1;
        if (pro) pro[(long)nt * stride] = pro[(long)(nt - 1) * stride];
        double tl = 0;
        if (I0 > IONIZATION_MIN_I / INTENSITY_DENOM) {
            gas_rates(c, I0, W, &err);
            gas_rates(c, I1, W + L, &err);
            double k1 = tstep * W[0] * (ND - ro[0]);
            double k2 = tstep * W[L] * (ND - ro[0] - k1);
            if (k1 < 0) k1 = 0;
            if (k2 < 0) k2 = 0;
            ro[0] += 0.5 * (k1 + k2);
            if (ro[0] > ND) ro[0] = ND;
            if (pro) pro[(long)nt * stride] = ro[0];
            tl = -0.5 * k1 / tstep * (c->potentials[0] + Pc * I0) / I0;
            for (int n = 1; n < L; n++) {
                k1 = tstep * W[n] * (ro[n - 1] - ro[n]);
                k2 = tstep * W[L + n] * (ro[n - 1] - ro[n] - k1);
                if (k1 < 0) k1 = 0;
                if (k2 < 0) k2 = 0;
                ro[n] = ro[n] + 0.5 * (k1 + k2);
                if (ro[n] > ro[n - 1]) ro[n] = ro[n - 1];
                if (pro) pro[(long)nt * stride] += ro[n];
                tl -= 0.5 * k1 / tstep * (c->potentials[n] + Pc * I0) / I0;
            }
        }
        if (loss) {
            loss[2 * (nt - 1)] = tl * field[2 * (nt - 1)];
            loss[2 * (nt - 1) + 1] = tl * field[2 * (nt - 1) + 1];
        }
        I0 = I1;
        if (err) return err;
    }
    if (loss) { loss[2 * (N - 1)] = 0; loss[2 * (N - 1) + 1] = 0; }
    return err;
}

int gso_plasma_losses(const gso_ctx* c, const double* field, double* pro, int stride, double* loss)
{
    if (c->gas) return plasma_losses_gas(c, field, pro, stride, loss);
    const int N = c->n_t;
    const double tstep = c->tstep * c->ionrate_denom;
    int err = GSO_OK;
    if (loss) { loss[0] = 0; loss[1] = 0; }
    double ro1 = c->rho0;
    double k1, k2;
    if (pro) pro[0] = ro1;
    double I0 = 0;
    for (int nt = 1; nt < N; nt++) {
        /* pfactor = exp(-j*OMEGA0*t); only |E*pfactor|^2 enters the solid-state rates */
        double ph = -c->omega0 * (c->tmin + nt * (c->tmax - c->tmin) / N);
        double pr = cos(ph), pi = sin(ph);
        double er = field[2 * nt], ei = field[2 * nt + 1];
        double reE1 = er * pr - ei * pi, imE1 = er * pi + ei * pr;
        double I1 = reE1 * reE1 + imE1 * imE1;

        double W01 = photoionization(c, I0, ro1, &err);
        k1 = tstep * (W01 + avalanche(c, I0, ro1) - recombination(c, ro1));
        double W11 = photoionization(c, I1, ro1 + k1, &err);
        k2 = tstep * (W11 + avalanche(c, I1, ro1 + k1) - recombination(c, ro1 + k1));

        ro1 += 0.5 * (k1 + k2);
        if (ro1 > c->neutral_density) ro1 = c->neutral_density;
        if (pro) pro[(long)nt * stride] = ro1;
        if (loss) {
            /* the reference compares the intensity against the log threshold (ionization.cpp:43) */
            if (I0 > IONIZATION_MIN_I_LN) {
                double s = -0.5 * (W01) * (c->ionization_potential + c->ponderomotive * I0) / I0;
                loss[2 * (nt - 1)] = s * field[2 * (nt - 1)];
                loss[2 * (nt - 1) + 1] = s * field[2 * (nt - 1) + 1];
            } else {
                loss[2 * (nt - 1)] = 0; loss[2 * (nt - 1) + 1] = 0;
            }
        }
        I0 = I1;
        if (err) return err;
    }
    if (loss) { loss[2 * (N - 1)] = 0; loss[2 * (N - 1) + 1] = 0; }
    return err;
}

/* ------------------------------------------------------------ NL response -- */

static inline void cmul(double ar, double ai, double br, double bi, double* r, double* i)
{
    *r = ar * br - ai * bi;
    *i = ar * bi + ai * br;
}

static int nl_response_ws(const gso_ctx* c, const double* in, double* out, double* ws)
{
    const int N = c->n_t;
    double* E = ws;            /* FIELD_REAL_SMALL */
    double* B1 = ws + 2 * N;   /* NL_SMALLBUFFER1 */
    double* B2 = ws + 4 * N;   /* NL_SMALLBUFFER2 */
    double* B3 = ws + 6 * N;   /* NL_SMALLBUFFER3 */
    int err;

    if (!c->nonlinear) {       /* propagator.cu:634-637 */
        memset(out, 0, sizeof(double) * 2 * (size_t)N);
        return GSO_OK;
    }
    gso_fft(N, in, E, +1);
    for (int i = 0; i < 2 * N; i++) E[i] /= N;

    err = gso_plasma_losses(c, E, B3, 2, B1);
    if (err) return err;
    for (int nt = 0; nt < N; nt++) {
        double ro = B3[2 * nt];
        B3[2 * nt] = ro * E[2 * nt];
        B3[2 * nt + 1] = ro * E[2 * nt + 1];
    }
    gso_fft(N, B1, B2, -1);      /* FFT(loss) */
    gso_fft(N, B3, B1, -1);      /* FFT(rho E) */
    for (int w = 0; w < N; w++) {
        double r, i;
        cmul(B1[2 * w], B1[2 * w + 1], c->plasma_func[2 * w], c->plasma_func[2 * w + 1], &r, &i);
        B2[2 * w] += r;
        B2[2 * w + 1] += i;
    }

    if (c->n2 != 0) {
        for (int nt = 0; nt < N; nt++) {
            B3[2 * nt] = E[2 * nt] * E[2 * nt] + E[2 * nt + 1] * E[2 * nt + 1];
            B3[2 * nt + 1] = 0;
        }
        if (c->raman_fraction > 0.001) {
            gso_fft(N, B3, B1, -1);
            for (int w = 0; w < N; w++) {
                double r, i;
                cmul(B1[2 * w], B1[2 * w + 1], c->raman_func[2 * w], c->raman_func[2 * w + 1], &r, &i);
                B1[2 * w] = r; B1[2 * w + 1] = i;
            }
            gso_fft(N, B1, B3, +1);
            for (int i = 0; i < 2 * N; i++) B3[i] /= N;
        }
        for (int nt = 0; nt < N; nt++) {
            double r, i;
            cmul(B3[2 * nt], B3[2 * nt + 1], E[2 * nt], E[2 * nt + 1], &r, &i);
            B3[2 * nt] = r; B3[2 * nt + 1] = i;
        }
        gso_fft(N, B3, B1, -1);
        for (int w = 0; w < N; w++) {
            /* += -j*K*B1 */
            double K = c->kerr[w];
            B2[2 * w] += K * B1[2 * w + 1];
            B2[2 * w + 1] += -K * B1[2 * w];
        }
        /* THIRD_HARMONICS (propagator.cu:712-720): E^3 exp(j phi_t), phi_t =
           -2 OMEGA0 (TMIN + nt (TMIN - TMAX)/N_T) (the reference's sign of the step), then
           += -j KERR_TH_PROFILE FFT(.), KERR_TH_PROFILE = KERR_PROFILE th_coeff */
        if (c->th_coeff != 0) {
            for (int nt = 0; nt < N; nt++) {
                double er = E[2 * nt], ei = E[2 * nt + 1];
                double e2r = er * er - ei * ei, e2i = 2 * er * ei;
                double e3r = e2r * er - e2i * ei, e3i = e2r * ei + e2i * er;
                double ph = -2.0 * c->omega0 * (c->tmin + nt * (c->tmin - c->tmax) / N);
                double cr = cos(ph), ci = sin(ph);
                B3[2 * nt] = e3r * cr - e3i * ci;
                B3[2 * nt + 1] = e3r * ci + e3i * cr;
            }
            gso_fft(N, B3, B1, -1);
            for (int w = 0; w < N; w++) {
                double K = c->kerr[w] * c->th_coeff;
                B2[2 * w] += K * B1[2 * w + 1];
                B2[2 * w + 1] += -K * B1[2 * w];
            }
        }
    }
    memcpy(out, B2, sizeof(double) * 2 * (size_t)N);
    return GSO_OK;
}

int gso_nl_response(const gso_ctx* c, const double* in, double* out)
{
    double* ws = (double*)malloc(sizeof(double) * 8 * (size_t)c->n_t);
    int err = nl_response_ws(c, in, out, ws);
    free(ws);
    return err;
}

int gso_nl_step(const gso_ctx* c, const double* field, double* bb1, double zstep,
                double* max_a2, double* max_nl2)
{
    const int N = c->n_t;
    double mA = 0, mN = 0;
    int err = GSO_OK;
#pragma omp parallel num_threads(c->nthreads > 0 ? c->nthreads : omp_get_max_threads())
    {
        double* ws = (double*)malloc(sizeof(double) * 8 * (size_t)N);
        double* o1 = (double*)malloc(sizeof(double) * 2 * (size_t)N * 5);
        double* o2 = o1 + 2 * N; double* o3 = o2 + 2 * N; double* o4 = o3 + 2 * N; double* xin = o4 + 2 * N;
        double lA = 0, lN = 0;
        int lerr = 0;
#pragma omp for schedule(dynamic)
        for (int r = 0; r < c->n_r; r++) {
            const double* A = field + 2 * (size_t)N * r;
            double* out = bb1 + 2 * (size_t)N * r;
            if (c->nonlinear) {
                int e = 0;
                e |= nl_response_ws(c, A, o1, ws);
                for (int i = 0; i < 2 * N; i++) xin[i] = A[i] + zstep * 0.5 * o1[i];
                e |= nl_response_ws(c, xin, o2, ws);
                for (int i = 0; i < 2 * N; i++) xin[i] = A[i] + zstep * 0.5 * o2[i];
                e |= nl_response_ws(c, xin, o3, ws);
                for (int i = 0; i < 2 * N; i++) xin[i] = A[i] + zstep * o3[i];
                e |= nl_response_ws(c, xin, o4, ws);
                if (e) lerr = e;
                for (int i = 0; i < 2 * N; i++)
                    out[i] = (o1[i] + 2.0 * o2[i] + 2.0 * o3[i] + o4[i]) / 6.0;
            } else {
                memset(out, 0, sizeof(double) * 2 * (size_t)N);
            }
            for (int nt = 0; nt < N; nt++) {
                double n2 = out[2 * nt] * out[2 * nt] + out[2 * nt + 1] * out[2 * nt + 1];
                double a2 = A[2 * nt] * A[2 * nt] + A[2 * nt + 1] * A[2 * nt + 1];
                if (n2 > lN) lN = n2;
                if (a2 > lA) lA = a2;
            }
        }
#pragma omp critical(gso_nl_red)
        {
            if (lA > mA) mA = lA;
            if (lN > mN) mN = lN;
            if (lerr && !err) err = lerr;
        }
        free(ws); free(o1);
    }
    *max_a2 = mA; *max_nl2 = mN;
    return err;
}

/* --------------------------------------------------------------- L step -- */

/* sqrtHO (extmath.h:234-256): 20-term Taylor series of sqrt(1+x)-1, coefficients
   binom(1/2, n) for n = 1..20 (the reference lists them rounded to 15 digits). */
static double sqrt_ho(double x)
{
    static double k[20];
    static int init = 0;
    if (!init) {
        double b = 1.0;
        for (int n = 1; n <= 20; n++) { b *= (0.5 - (n - 1)) / n; k[n - 1] = b; }
        init = 1;
    }
    double r = 0, xn = x;
    for (int j = 0; j < 20; j++) { r += k[j] * xn; xn *= x; }
    return r;
}

int gso_lstep(const gso_ctx* c, double* field, const double* bb1, double* bb2, double zstep)
{
    const int N = c->n_t;
    sqrt_ho(0.0);
#pragma omp parallel for schedule(static) num_threads(c->nthreads > 0 ? c->nthreads : omp_get_max_threads())
    for (int nx = 0; nx < c->n_r; nx++) {
        double kt2 = c->kt2[nx];
        for (int nw = 0; nw < N; nw++) {
            size_t ofs = 2 * ((size_t)nw + (size_t)N * nx);
            double w = c->omega[nw];
            double kr = c->wavenum[2 * nw], ki = c->wavenum[2 * nw + 1];
            if (w < c->omega_min || w > c->omega_max) { field[ofs] = 0; field[ofs + 1] = 0; continue; }
            if (kt2 > MAX_KT2 * (kr * kr - ki * ki)) { field[ofs] = 0; field[ofs + 1] = 0; continue; }
            double sq = sqrt_ho(-kt2 / kr / kr);
            bb2[ofs] += zstep * bb1[ofs] / (1 + sq);
            bb2[ofs + 1] += zstep * bb1[ofs + 1] / (1 + sq);
            double er = zstep * ki, ei = zstep * (-c->ho_disp[nw] - sq * kr);
            double m = exp(er), pr = m * cos(ei), pi = m * sin(ei);
            double fr, fi;
            cmul(bb2[ofs], bb2[ofs + 1], pr, pi, &fr, &fi);
            field[ofs] = fr; field[ofs + 1] = fi;
            bb2[ofs] = fr; bb2[ofs + 1] = fi;
        }
    }
    return GSO_OK;
}

/* ----------------------------------------------------------- propagator -- */

int gso_propagator(const gso_ctx* c, double* field, double* bb1, double* bb2,
                   double* zstep, double current_z, double znet_cur, double znet_prev,
                   unsigned* step_n, double* max_a2_out, double* max_nl2_out)
{
    const double tol = c->max_tolerance;
    for (;;) {
        double max_nl2 = 0, max_a2 = 0;
        int err = gso_nl_step(c, field, bb1, *zstep, &max_a2, &max_nl2);
        if (err) return err;
        int repeat = 0;
        if ((*zstep) * (*zstep) * max_nl2 > tol * tol * max_a2) { repeat = 1; (*step_n)++; }
        *zstep = 0.5 * tol * sqrt(max_a2 / max_nl2);
        if (*zstep < MINSTEP_RATIO * (znet_cur - znet_prev) || !(*zstep > 0)) return GSO_ERR_COLLAPSE;
        double lim = znet_cur - current_z;
        if (lim < *zstep) *zstep = lim;
        if (max_a2_out) *max_a2_out = max_a2;
        if (max_nl2_out) *max_nl2_out = max_nl2;
        if (!repeat) {
            gso_qdht_run_many(c, bb1, c->n_t, c->n_t, 1);
            gso_lstep(c, field, bb1, bb2, *zstep);
            gso_qdht_run_many(c, field, c->n_t, c->n_t, 1);
            return GSO_OK;
        }
    }
}

/* -------------------------------------------------------- dump reductions -- */

int gso_row_reductions(const gso_ctx* c, const double* field, double* out_maxI,
                       double* out_flux, double* out_pmax)
{
    const int N = c->n_t;
    int err = GSO_OK;
#pragma omp parallel num_threads(c->nthreads > 0 ? c->nthreads : omp_get_max_threads())
    {
        double* buf = (double*)malloc(sizeof(double) * 2 * (size_t)N);
        double* e = (double*)malloc(sizeof(double) * 2 * (size_t)N);
        double* ro = (double*)malloc(sizeof(double) * (size_t)N);
#pragma omp for schedule(dynamic)
        for (int r = 0; r < c->n_r; r++) {
            const double* F = field + 2 * (size_t)N * r;
            /* dump_type_maxI_class / flux: BW FFT of FIELD*wfilter/N_T (wfilter = 1) */
            for (int i = 0; i < 2 * N; i++) buf[i] = F[i] / (double)N;
            gso_fft(N, buf, e, +1);
            double mI = 0, fl = 0;
            for (int t = 0; t < N; t++) {
                double I = e[2 * t] * e[2 * t] + e[2 * t + 1] * e[2 * t + 1];
                if (I > mI) mI = I;
                fl += I;
            }
            if (out_maxI) out_maxI[r] = mI;
            if (out_flux) out_flux[r] = fl * c->tstep;
            if (out_pmax) {
                /* dump_type_plasma_max_class: BW FFT then Nnormalize, then the recurrence */
                gso_fft(N, F, e, +1);
                for (int i = 0; i < 2 * N; i++) e[i] /= N;
                int le = gso_plasma_losses(c, e, ro, 1, NULL);
                double m = 0;
                for (int t = 0; t < N; t++) if (ro[t] > m) m = ro[t];
                out_pmax[r] = m;
                if (le) {
#pragma omp critical(gso_red_err)
                    err = le;
                }
            }
        }
        free(buf); free(e); free(ro);
    }
    return err;
}
