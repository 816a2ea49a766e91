// shim.cpp -- implementations behind the stand-in headers of oracle/ref_shim (TEST
// INFRASTRUCTURE: linked only into oracle/_ref, the reference solver built for comparison).
//
// FFT: iterative radix-2 decimation in time over a power-of-two length with twiddles
// exp(sign 2 pi i k / n) taken from cos / sin of the exact angle, a direct DFT for any other
// length; unnormalised, FFTW's sign convention.  Bessel: the C library's j0 / j1, zeros of J0
// by McMahon's expansion and Newton's method.  Gamma: tgamma.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fftw3-mpi.h"
#include "fftw3.h"
#include "gsl/gsl_errno.h"
#include "gsl/gsl_roots.h"
#include "gsl/gsl_sf_bessel.h"
#include "gsl/gsl_sf_gamma.h"

struct gsref_fftw_plan_s {
    int n = 0, howmany = 1, istride = 1, idist = 0, ostride = 1, odist = 0, sign = -1;
    fftw_complex* in = nullptr;
    fftw_complex* out = nullptr;
    bool pow2 = false;
    std::vector<double> wr, wi;   // twiddles for k < n/2 (pow2) or k < n (direct DFT)
    std::vector<int> rev;         // bit reversal (pow2)
};

static void plan_tables(gsref_fftw_plan_s* p) {
    const int n = p->n;
    p->pow2 = n > 0 && (n & (n - 1)) == 0;
    const int nw = p->pow2 ? n / 2 : n;
    p->wr.resize(nw > 0 ? nw : 1);
    p->wi.resize(nw > 0 ? nw : 1);
    for (int k = 0; k < nw; k++) {
        const double a = 2.0 * M_PI * (double)k / (double)n;
        p->wr[k] = std::cos(a);
        p->wi[k] = (double)p->sign * std::sin(a);
    }
    if (p->pow2) {
        int lg = 0;
        while ((1 << lg) < n) lg++;
        p->rev.resize(n);
        for (int j = 0; j < n; j++) {
            int r = 0;
            for (int b = 0; b < lg; b++) r |= ((j >> b) & 1) << (lg - 1 - b);
            p->rev[j] = r;
        }
    }
}

static void transform_one(const gsref_fftw_plan_s* p, std::vector<double>& re, std::vector<double>& im) {
    const int n = p->n;
    if (p->pow2) {
        for (int j = 0; j < n; j++) {
            const int r = p->rev[j];
            if (r > j) {
                std::swap(re[j], re[r]);
                std::swap(im[j], im[r]);
            }
        }
        for (int len = 2; len <= n; len <<= 1) {
            const int half = len / 2, step = n / len;
            for (int s = 0; s < n; s += len)
                for (int k = 0; k < half; k++) {
                    const double cr = p->wr[(size_t)k * step], ci = p->wi[(size_t)k * step];
                    const int a = s + k, b = a + half;
                    const double tr = re[b] * cr - im[b] * ci;
                    const double ti = re[b] * ci + im[b] * cr;
                    re[b] = re[a] - tr;
                    im[b] = im[a] - ti;
                    re[a] += tr;
                    im[a] += ti;
                }
        }
        return;
    }
    std::vector<double> orr(n), oi(n);
    for (int k = 0; k < n; k++) {
        double sr = 0, si = 0;
        for (int j = 0; j < n; j++) {
            const int e = (int)(((long long)j * k) % n);
            sr += re[j] * p->wr[e] - im[j] * p->wi[e];
            si += re[j] * p->wi[e] + im[j] * p->wr[e];
        }
        orr[k] = sr;
        oi[k] = si;
    }
    re.swap(orr);
    im.swap(oi);
}

extern "C" {

fftw_plan fftw_plan_many_dft(int rank, const int* n, int howmany, fftw_complex* in, const int* inembed, int istride,
                             int idist, fftw_complex* out, const int* onembed, int ostride, int odist, int sign,
                             unsigned flags) {
    (void)inembed; (void)onembed; (void)flags;
    if (rank != 1) {
        fprintf(stderr, "fftw shim: only rank-1 transforms\n");
        exit(3);
    }
    gsref_fftw_plan_s* p = new gsref_fftw_plan_s();
    p->n = n[0];
    p->howmany = howmany;
    p->istride = istride;
    p->idist = idist;
    p->ostride = ostride;
    p->odist = odist;
    p->sign = sign;
    p->in = in;
    p->out = out;
    plan_tables(p);
    return p;
}

fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags) {
    return fftw_plan_many_dft(1, &n, 1, in, nullptr, 1, n, out, nullptr, 1, n, sign, flags);
}

void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out) {
    std::vector<double> re(p->n), im(p->n);
    for (int t = 0; t < p->howmany; t++) {
        const fftw_complex* x = in + (size_t)t * p->idist;
        for (int j = 0; j < p->n; j++) {
            re[j] = x[(size_t)j * p->istride][0];
            im[j] = x[(size_t)j * p->istride][1];
        }
        transform_one(p, re, im);
        fftw_complex* y = out + (size_t)t * p->odist;
        for (int j = 0; j < p->n; j++) {
            y[(size_t)j * p->ostride][0] = re[j];
            y[(size_t)j * p->ostride][1] = im[j];
        }
    }
}

void fftw_execute(const fftw_plan p) { fftw_execute_dft(p, p->in, p->out); }

void fftw_destroy_plan(fftw_plan p) { delete p; }

void* fftw_malloc(size_t n) {
    void* q = nullptr;
    if (posix_memalign(&q, 64, n ? n : 1) != 0) return nullptr;
    return q;
}

void fftw_free(void* q) { free(q); }

void fftw_mpi_init(void) {}

ptrdiff_t fftw_mpi_local_size_many_transposed(int, const ptrdiff_t*, ptrdiff_t, ptrdiff_t, ptrdiff_t, MPI_Comm,
                                              ptrdiff_t*, ptrdiff_t*, ptrdiff_t*, ptrdiff_t*) {
    fprintf(stderr, "fftw shim: the MPI transforms of the 2-D transverse build are not provided\n");
    exit(3);
}

fftw_plan fftw_mpi_plan_many_dft(int, const ptrdiff_t*, ptrdiff_t, ptrdiff_t, ptrdiff_t, fftw_complex*, fftw_complex*,
                                 MPI_Comm, int, unsigned) {
    fprintf(stderr, "fftw shim: the MPI transforms of the 2-D transverse build are not provided\n");
    exit(3);
}

void fftw_mpi_execute_dft(fftw_plan, fftw_complex*, fftw_complex*) {
    fprintf(stderr, "fftw shim: the MPI transforms of the 2-D transverse build are not provided\n");
    exit(3);
}

double gsl_sf_bessel_J0(double x) { return j0(x); }
double gsl_sf_bessel_J1(double x) { return j1(x); }

double gsl_sf_bessel_zero_J0(unsigned int s) {
    if (s == 0) return 0.0;
    // McMahon: j ~ b + 1/(8b) - 124/(3 (8b)^3) + 120928/(15 (8b)^5), b = (s - 1/4) pi
    const double b = ((double)s - 0.25) * M_PI;
    const double e = 8.0 * b;
    double x = b + 1.0 / e - 124.0 / (3.0 * e * e * e) + 120928.0 / (15.0 * e * e * e * e * e);
    for (int it = 0; it < 30; it++) {   // Newton on J0, J0' = -J1
        const double dx = j0(x) / j1(x);
        x += dx;
        if (std::fabs(dx) <= 1e-16 * x) break;
    }
    return x;
}

double gsl_sf_gamma(double x) { return std::tgamma(x); }

static const gsl_root_fdfsolver_type g_secant = {"secant"};
const gsl_root_fdfsolver_type* gsl_root_fdfsolver_secant = &g_secant;

gsl_root_fdfsolver* gsl_root_fdfsolver_alloc(const gsl_root_fdfsolver_type* T) {
    gsl_root_fdfsolver* s = new gsl_root_fdfsolver();
    s->type = T;
    return s;
}

int gsl_root_fdfsolver_set(gsl_root_fdfsolver* s, gsl_function_fdf* fdf, double root) {
    s->fdf = fdf;
    s->root = root;
    fdf->fdf(root, fdf->params, &s->f, &s->df);
    return GSL_SUCCESS;
}

int gsl_root_fdfsolver_iterate(gsl_root_fdfsolver* s) {
    if (s->df == 0.0) return GSL_FAILURE;
    const double x1 = s->root - s->f / s->df;
    const double f1 = s->fdf->f(x1, s->fdf->params);
    s->df = (x1 != s->root) ? (f1 - s->f) / (x1 - s->root) : s->df;
    s->root = x1;
    s->f = f1;
    return GSL_SUCCESS;
}

double gsl_root_fdfsolver_root(const gsl_root_fdfsolver* s) { return s->root; }

void gsl_root_fdfsolver_free(gsl_root_fdfsolver* s) { delete s; }

int gsl_root_test_delta(double x1, double x0, double epsabs, double epsrel) {
    const double tol = epsabs + epsrel * std::fmin(std::fabs(x1), std::fabs(x0));
    return std::fabs(x1 - x0) < tol ? GSL_SUCCESS : GSL_CONTINUE;
}

}  // extern "C"
