/*
 * gs_oracle_adj.c -- FP64 adjoint of the z-step (TEST INFRASTRUCTURE).
 *
 * The reference has no adjoint.  This file differentiates, by hand and in plain FP64
 * loops, exactly the discrete forward map restated in gs_oracle.c for one accepted
 * propagator() call with a given step size (propagator.cu:125-266 with the controller's
 * dz fixed):
 *   R = RK4 increment of calculate_NLstep at A_n        (propagator.cu:375-425)
 *   S_{n+1} = (S_n + dz N(H R)/(1+s)) P  inside the window, S_n outside
 *   A_{n+1} = H (window ? S_{n+1} : 0)                   (calculate_Lstep, ht_run)
 * with H = diag(m1) C diag(1/m1) the QDHT of fhatha.cpp:218-230.  Cotangents follow the
 * convention g = dJ/dRe + i dJ/dIm of a real objective J, so that for a complex-linear
 * map y = M x the rule is x_bar = M^H y_bar.  It is checked against central finite
 * differences of the oracle's own forward (tests/test_oracle_adjoint.py) and is the FP64
 * reference for the GPU adjoint.
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

static int nthreads(const gso_ctx* c) { return c->nthreads > 0 ? c->nthreads : omp_get_max_threads(); }

/* photoionization_function (ionization.cpp:98-147) and dW/dI (the table is linear in
   ln I between nodes: dW/dI = W * slope / I). */
static double photo_d(const gso_ctx* c, double I, double ro, double* dW)
{
    *dW = 0;
    if (I < IONIZATION_MIN_I / INTENSITY_DENOM) return 0;
    if (ro > c->neutral_density) return 0;
    double lnI = log(I) + INTENSITY_DENOM_LN;
    int n = (int)floor((lnI - IONIZATION_MIN_I_LN) / IONIZATION_I_LN_TOLERANCE);
    if (n > IONIZATION_N - 2 || n < 0) return 0;
    double lnIn = IONIZATION_MIN_I_LN + n * IONIZATION_I_LN_TOLERANCE;
    double w0 = c->rate_ln[n], w1 = c->rate_ln[n + 1];
    double slope = (w1 - w0) / IONIZATION_I_LN_TOLERANCE;
    double W = exp(w0 + (lnI - lnIn) * (w1 - w0) / IONIZATION_I_LN_TOLERANCE);
    *dW = W * slope / I;
    return W;
}

/* avalanche_ionization_function (ionization.h:77-83) with d/dI and d/drho */
static double aval_d(const gso_ctx* c, double I, double ro, double* dI, double* dro)
{
    *dI = 0; *dro = 0;
    if (ro < 0 || ro > c->neutral_density) return 0;
    const double U = c->ionization_potential, P = c->ponderomotive, AV = c->avalanche_cs, ND = c->neutral_density;
    const double den = U + P * I;
    const double f = ro * (1 - ro / ND);
    *dI = AV * U / (den * den) * f;
    *dro = AV / den * I * (1 - 2 * ro / ND);
    return AV / den * I * f;
}

/* recombination_function (ionization.h:84-87) with d/drho */
static double recomb_d(const gso_ctx* c, double ro, double* dro)
{
    *dro = (ro > 0) ? 1 / c->recombination_tau : 0;
    return (ro > 0) ? ro / c->recombination_tau : 0;
}

/* Partial derivatives of one Heun step rho_t = Phi(rho_{t-1}, I0, I1) of
   gso_plasma_losses (ionization.cpp:29-40): d = dPhi/drho, a = dPhi/dI0, b = dPhi/dI1. */
static void heun_partials(const gso_ctx* c, double ro, double I0, double I1, double* d, double* a, double* b)
{
    const double dt = c->tstep * c->ionrate_denom;
    double dW0, dI0, dr0, drc0, dW1, dI1, dr1, drc1;
    double W0 = photo_d(c, I0, ro, &dW0);
    double av0 = aval_d(c, I0, ro, &dI0, &dr0);
    double rc0 = recomb_d(c, ro, &drc0);
    double k1 = dt * (W0 + av0 - rc0);
    double k1r = dt * (dr0 - drc0), k1I = dt * (dW0 + dI0);
    double r2 = ro + k1;
    double W1 = photo_d(c, I1, r2, &dW1);
    double av1 = aval_d(c, I1, r2, &dI1, &dr1);
    double rc1 = recomb_d(c, r2, &drc1);
    double k2 = dt * (W1 + av1 - rc1);
    double k2r = dt * (dr1 - drc1), k2I = dt * (dW1 + dI1);
    double rn = ro + 0.5 * (k1 + k2);
    if (rn > c->neutral_density) { *d = 0; *a = 0; *b = 0; return; }
    *d = 1 + 0.5 * (k1r + k2r * (1 + k1r));
    *a = 0.5 * k1I * (1 + k2r);
    *b = 0.5 * k2I;
}

static inline void cmulc(double ar, double ai, double br, double bi, double* r, double* i)
{
    *r = ar * br - ai * bi;
    *i = ar * bi + ai * br;
}

/* Vector-Jacobian product of calculate_NLresponse (propagator.cu:629-783) for one row:
   given the spectral stage input Y and the cotangent kbar of N(Y), ybar = (dN/dY)^H kbar. */
static int nl_vjp_row(const gso_ctx* c, const double* Y, const double* kbar, double* ybar, double* ws)
{
    const int N = c->n_t;
    if (!c->nonlinear) { memset(ybar, 0, sizeof(double) * 2 * (size_t)N); return GSO_OK; }
    if (c->gas || c->th_coeff != 0) return GSO_ERR_ARG;   /* the adjoint covers the solid build */
    double* E = ws;                 /* 2N */
    double* rho = E + 2 * N;        /* N  */
    double* Q = rho + N;            /* N  */
    double* I = Q + N;              /* N  */
    double* Eb = I + N;             /* 2N */
    double* t1 = Eb + 2 * N;        /* 2N */
    double* t2 = t1 + 2 * N;        /* 2N */
    double* Ib = t2 + 2 * N;        /* N  */
    double* rb = Ib + N;            /* N  */
    double* Qb = rb + N;            /* N  */
    const double U = c->ionization_potential, Pc = c->ponderomotive;
    const int kerr_on = c->n2 != 0;
    const int raman = c->raman_fraction > 0.001;

    /* forward recompute: E = IFFT(Y)/N, rho(t), Q = (1-fR) I + Raman (the FFT form) */
    gso_fft(N, Y, E, +1);
    for (int i = 0; i < 2 * N; i++) E[i] /= N;
    int err = gso_plasma_losses(c, E, rho, 1, NULL);
    if (err) return err;
    for (int t = 0; t < N; t++) I[t] = E[2 * t] * E[2 * t] + E[2 * t + 1] * E[2 * t + 1];
    if (kerr_on) {
        if (raman) {
            for (int t = 0; t < N; t++) { t1[2 * t] = I[t]; t1[2 * t + 1] = 0; }
            gso_fft(N, t1, t2, -1);
            for (int w = 0; w < N; w++) {
                double r, i;
                cmulc(t2[2 * w], t2[2 * w + 1], c->raman_func[2 * w], c->raman_func[2 * w + 1], &r, &i);
                t2[2 * w] = r; t2[2 * w + 1] = i;
            }
            gso_fft(N, t2, t1, +1);
            for (int t = 0; t < N; t++) Q[t] = t1[2 * t] / N;
        } else {
            for (int t = 0; t < N; t++) Q[t] = I[t];
        }
    }

    /* loss term: l = F^H kbar, E_bar += s l, I_bar += s'(I) Re(conj(E) l) */
    gso_fft(N, kbar, t1, +1);
    for (int t = 0; t < N; t++) {
        Eb[2 * t] = 0; Eb[2 * t + 1] = 0; Ib[t] = 0;
        if (t >= 1 && t <= N - 2 && I[t] > IONIZATION_MIN_I_LN) {
            double dW;
            const double W = photo_d(c, I[t], rho[t], &dW);
            const double s = -0.5 * W * (U + Pc * I[t]) / I[t];
            const double ds = -0.5 * (dW * (U + Pc * I[t]) / I[t] - W * U / (I[t] * I[t]));
            Eb[2 * t] += s * t1[2 * t];
            Eb[2 * t + 1] += s * t1[2 * t + 1];
            Ib[t] += ds * (E[2 * t] * t1[2 * t] + E[2 * t + 1] * t1[2 * t + 1]);
        }
    }
    /* plasma term: p = F^H (conj(PLASMA_FUNC) kbar), E_bar += rho p, rho_bar = Re(conj(E) p) */
    for (int w = 0; w < N; w++) {
        double r, i;
        cmulc(kbar[2 * w], kbar[2 * w + 1], c->plasma_func[2 * w], -c->plasma_func[2 * w + 1], &r, &i);
        t2[2 * w] = r; t2[2 * w + 1] = i;
    }
    gso_fft(N, t2, t1, +1);
    for (int t = 0; t < N; t++) {
        Eb[2 * t] += rho[t] * t1[2 * t];
        Eb[2 * t + 1] += rho[t] * t1[2 * t + 1];
        rb[t] = E[2 * t] * t1[2 * t] + E[2 * t + 1] * t1[2 * t + 1];
    }
    /* Kerr term: q = F^H (j KERR kbar), E_bar += Q q, Q_bar = Re(conj(E) q) */
    if (kerr_on) {
        for (int w = 0; w < N; w++) {
            const double K = c->kerr[w];
            t2[2 * w] = -K * kbar[2 * w + 1];
            t2[2 * w + 1] = K * kbar[2 * w];
        }
        gso_fft(N, t2, t1, +1);
        for (int t = 0; t < N; t++) {
            Eb[2 * t] += Q[t] * t1[2 * t];
            Eb[2 * t + 1] += Q[t] * t1[2 * t + 1];
            Qb[t] = E[2 * t] * t1[2 * t] + E[2 * t + 1] * t1[2 * t + 1];
        }
        /* Q = IFFT(R FFT(I))/N  ->  I_bar += Re(IFFT(conj(R) FFT(Q_bar))/N) */
        if (raman) {
            for (int t = 0; t < N; t++) { t1[2 * t] = Qb[t]; t1[2 * t + 1] = 0; }
            gso_fft(N, t1, t2, -1);
            for (int w = 0; w < N; w++) {
                double r, i;
                cmulc(t2[2 * w], t2[2 * w + 1], c->raman_func[2 * w], -c->raman_func[2 * w + 1], &r, &i);
                t2[2 * w] = r; t2[2 * w + 1] = i;
            }
            gso_fft(N, t2, t1, +1);
            for (int t = 0; t < N; t++) Ib[t] += t1[2 * t] / N;
        } else {
            for (int t = 0; t < N; t++) Ib[t] += Qb[t];
        }
    }
    /* the density recurrence backwards: lam_{t-1} = rho_bar_{t-1} + dPhi_t/drho lam_t;
       I_{t-1} and I_t receive lam_t times the step's partials (I_0 enters as 0: no term) */
    double lam = rb[N - 1];
    for (int t = N - 1; t >= 1; t--) {
        double d, a, b;
        heun_partials(c, rho[t - 1], (t - 1 == 0) ? 0.0 : I[t - 1], I[t], &d, &a, &b);
        Ib[t] += lam * b;
        if (t - 1 >= 1) Ib[t - 1] += lam * a;
        lam = rb[t - 1] + d * lam;
    }
    /* I = |E|^2 */
    for (int t = 0; t < N; t++) {
        Eb[2 * t] += 2 * Ib[t] * E[2 * t];
        Eb[2 * t + 1] += 2 * Ib[t] * E[2 * t + 1];
    }
    /* E = F^{-1}[Y]/N  ->  ybar = F[E_bar]/N */
    gso_fft(N, Eb, ybar, -1);
    for (int i = 0; i < 2 * N; i++) ybar[i] /= N;
    return GSO_OK;
}

int gso_nl_response_vjp(const gso_ctx* c, const double* Y, const double* kbar, double* ybar)
{
    double* ws = (double*)malloc(sizeof(double) * 16 * (size_t)c->n_t);
    int err = nl_vjp_row(c, Y, kbar, ybar, ws);
    free(ws);
    return err;
}

int gso_nl_step_vjp(const gso_ctx* c, const double* field, double zstep, const double* rbar, double* abar)
{
    const int N = c->n_t;
    int err = GSO_OK;
#pragma omp parallel num_threads(nthreads(c))
    {
        double* ws = (double*)malloc(sizeof(double) * 16 * (size_t)N);
        double* b = (double*)malloc(sizeof(double) * 2 * (size_t)N * 8);
        double* o1 = b; double* o2 = o1 + 2 * N; double* o3 = o2 + 2 * N;
        double* y2 = o3 + 2 * N; double* y3 = y2 + 2 * N; double* y4 = y3 + 2 * N;
        double* kb = y4 + 2 * N; double* yb = kb + 2 * N;
        int lerr = 0;
#pragma omp for schedule(dynamic)
        for (int r = 0; r < c->n_r; r++) {
            const double* A = field + 2 * (size_t)N * r;
            const double* Rb = rbar + 2 * (size_t)N * r;
            double* Ab = abar + 2 * (size_t)N * r;
            if (!c->nonlinear) { memset(Ab, 0, sizeof(double) * 2 * (size_t)N); continue; }
            /* the forward stages (gso_nl_step) */
            double* w8 = ws;
            lerr |= gso_nl_response(c, A, o1);
            for (int i = 0; i < 2 * N; i++) y2[i] = A[i] + zstep * 0.5 * o1[i];
            lerr |= gso_nl_response(c, y2, o2);
            for (int i = 0; i < 2 * N; i++) y3[i] = A[i] + zstep * 0.5 * o2[i];
            lerr |= gso_nl_response(c, y3, o3);
            for (int i = 0; i < 2 * N; i++) y4[i] = A[i] + zstep * o3[i];
            /* R = (k1 + 2 k2 + 2 k3 + k4)/6 backwards through the stages */
            for (int i = 0; i < 2 * N; i++) kb[i] = Rb[i] / 6.0;
            lerr |= nl_vjp_row(c, y4, kb, yb, w8);
            for (int i = 0; i < 2 * N; i++) { Ab[i] = yb[i]; kb[i] = Rb[i] / 3.0 + zstep * yb[i]; }
            lerr |= nl_vjp_row(c, y3, kb, yb, w8);
            for (int i = 0; i < 2 * N; i++) { Ab[i] += yb[i]; kb[i] = Rb[i] / 3.0 + zstep * 0.5 * yb[i]; }
            lerr |= nl_vjp_row(c, y2, kb, yb, w8);
            for (int i = 0; i < 2 * N; i++) { Ab[i] += yb[i]; kb[i] = Rb[i] / 6.0 + zstep * 0.5 * yb[i]; }
            lerr |= nl_vjp_row(c, A, kb, yb, w8);
            for (int i = 0; i < 2 * N; i++) Ab[i] += yb[i];
        }
#pragma omp critical(gso_adj_err)
        {
            if (lerr && !err) err = lerr;
        }
        free(ws); free(b);
    }
    return err;
}

/* sqrtHO (extmath.h:234-256): coefficients binom(1/2, n), n = 1..20 */
static double sqrt_ho_adj(double x)
{
    double r = 0, xn = x, b = 1;
    for (int n = 1; n <= 20; n++) {
        b *= (0.5 - (n - 1)) / n;
        r += b * xn;
        xn *= x;
    }
    return r;
}

int gso_lstep_vjp(const gso_ctx* c, const double* fbar, double* sbar, double* b1bar, double zstep)
{
    const int N = c->n_t;
#pragma omp parallel for schedule(static) num_threads(nthreads(c))
    for (int nx = 0; nx < c->n_r; nx++) {
        const double kt2 = c->kt2[nx];
        for (int nw = 0; nw < N; nw++) {
            const size_t o = 2 * ((size_t)nw + (size_t)N * nx);
            const double w = c->omega[nw];
            const double kr = c->wavenum[2 * nw], ki = c->wavenum[2 * nw + 1];
            if (w < c->omega_min || w > c->omega_max || kt2 > 0.25 * (kr * kr - ki * ki)) {
                b1bar[o] = 0; b1bar[o + 1] = 0;   /* FIELD = 0 there, BIGBUFFER2 unchanged */
                continue;
            }
            const double sq = sqrt_ho_adj(-kt2 / kr / kr);
            const double er = zstep * ki, ei = zstep * (-c->ho_disp[nw] - sq * kr);
            const double m = exp(er), pr = m * cos(ei), pi = m * sin(ei);
            const double gr = fbar[o] + sbar[o], gi = fbar[o + 1] + sbar[o + 1];
            const double tr = pr * gr + pi * gi, ti = pr * gi - pi * gr;   /* conj(P) g */
            sbar[o] = tr; sbar[o + 1] = ti;
            b1bar[o] = zstep * tr / (1 + sq);
            b1bar[o + 1] = zstep * ti / (1 + sq);
        }
    }
    return GSO_OK;
}

int gso_qdht_transposed(const gso_ctx* c, double* data)
{
    const long N = c->n_r, nt = c->n_t;
    const double* C = c->qdht_c;
    const double* m1 = c->qdht_m1;
#pragma omp parallel for schedule(dynamic) num_threads(nthreads(c))
    for (long w = 0; w < nt; w++) {
        double* x = (double*)malloc(sizeof(double) * 2 * (size_t)N);
        for (long j = 0; j < N; j++) {
            x[2 * j] = data[2 * (j * nt + w)] * m1[j];
            x[2 * j + 1] = data[2 * (j * nt + w) + 1] * m1[j];
        }
        for (long i = 0; i < N; i++) {
            double yr = 0, yi = 0;
            for (long j = 0; j < N; j++) {
                const double cij = C[i + N * j];
                yr += cij * x[2 * j];
                yi += cij * x[2 * j + 1];
            }
            data[2 * (i * nt + w)] = yr / m1[i];
            data[2 * (i * nt + w) + 1] = yi / m1[i];
        }
        free(x);
    }
    return GSO_OK;
}
