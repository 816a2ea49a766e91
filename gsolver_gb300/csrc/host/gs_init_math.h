// gs_init_math.h -- set-up arithmetic shared by the host set-up (gs_setup.cpp, g++) and the
// device set-up kernels (gs_init.cu, nvcc): one source for both, so the two agree to the
// last rounding of the math libraries they call.  Global-namespace math functions are used
// (libm on the host, CUDA's device math library on the GPU).
#pragma once
#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define GS_HD __host__ __device__ inline
#else
#define GS_HD inline
#endif

namespace gsm {

// SIconstants.h
constexpr double kC = 299792458.0;
constexpr double kMu0 = 1.2566370615e-6;
constexpr double kE = 1.60217733e-19;
constexpr double kMe = 9.1093897e-31;
constexpr double kHbar = 1.0545727e-34;
constexpr double kHartree = 4.359748124303985e-018;
constexpr double kPi = 3.14159265358979323846;

// complete elliptic integrals K(m), E(m) by the arithmetic-geometric mean (extmath.cpp:154-171
// computes the same integrals)
GS_HD void ellipke(double m, double* K, double* E) {
    double a = 1, b = ::sqrt(1 - m), c = ::sqrt(m), sum = 0.5 * c * c, p = 0.5;
    for (int it = 0; it < 60 && c > 1e-17; it++) {
        const double an = 0.5 * (a + b), bn = ::sqrt(a * b);
        c = 0.5 * (a - b);
        p *= 2;
        sum += p * c * c;
        a = an;
        b = bn;
    }
    *K = kPi / (2 * a);
    *E = *K * (1 - sum);
}

// Dawson's integral (extmath.cpp:174-294 computes the same function): the power series
// D(x) = exp(-x^2) sum x^(2n+1)/(n! (2n+1)) for |x| <= 7, the asymptotic series beyond
GS_HD double dawson(double x) {
    const double ax = ::fabs(x);
    double r;
    if (ax <= 7.0) {
        const double x2 = ax * ax;
        double term = ax, sum = ax;
        for (int n = 1; n < 400; n++) {
            term *= x2 / n;
            const double t = term / (2 * n + 1);
            sum += t;
            if (t < 1e-18 * sum) break;
        }
        r = ::exp(-x2) * sum;
    } else {
        const double y = 1.0 / (2 * ax * ax);
        double term = 1, sum = 1;
        for (int k = 1; k < 60; k++) {
            const double nt = term * (2 * k - 1) * y;
            if (nt > term) break;
            term = nt;
            sum += term;
            if (term < 1e-18 * sum) break;
        }
        r = sum / (2 * ax);
    }
    return x < 0 ? -r : r;
}

// keldysh_rate_ln (ionization.cpp:203-232)
GS_HD double keldysh_rate_ln(double lnI, double k0, double U, double w0, double vg, double mred) {
    const double phase_v = w0 / k0;
    const double E = ::exp(lnI / 2) * ::sqrt(2 * phase_v / vg * phase_v * kMu0);
    const double m = kMe * mred;
    const double kg = w0 * ::sqrt(m / kE / kE * U) / E;
    const double G = kg * kg / (1 + kg * kg), X = 1 / (1 + kg * kg);
    double Kg, Eg, Kx, Ex;
    ellipke(G, &Kg, &Eg);
    ellipke(X, &Kx, &Ex);
    const double alpha = kPi * (Kg - Eg) / Ex, beta = kPi * kPi / 4.0 / Kx / Ex;
    const double x = 2 / kPi * U / kHbar / w0 * Ex / ::sqrt(G);
    const double nu = ::floor(x + 1) - x;
    int sumN = (int)::ceil(10 / alpha);
    if (sumN > 1000) sumN = 1000;
    double Q = 0;
    for (int i = 0; i < sumN; i++) Q += ::exp(-i * alpha) * dawson(::sqrt(beta * (i + 2 * nu)));
    Q *= ::sqrt(kPi / 2 / Kx);
    return ::log(2 * w0 / 9 / kPi) + 1.5 * ::log(w0 * m / kHbar) - 0.75 * ::log(G) + ::log(Q) - alpha * ::floor(x + 1);
}

// PPT_rate_ln (ionization.cpp:235-294) without the Yudin-Ivanov correction; n_eff is held
// in single precision as in the reference (`float neff`)
GS_HD double ppt_rate_ln(double lnI, double Ui, double Z, int l, double k0, double w0, double vg) {
    const double phase_v = w0 / k0;
    const double E = ::exp(lnI / 2) * ::sqrt(2 * kMu0 * phase_v * phase_v / vg);
    const double m = kMe;
    const double g = w0 * ::sqrt(2 * m / kE / kE * Ui) / E;
    const double Ueff = Ui * (1 + 1.0 / 2.0 / g / g);
    const double nu = Ueff / kHbar / w0;
    const int nu0 = (int)::floor(1 + nu);
    const double alpha = 2 * (::asinh(g) - g / ::sqrt(1 + g * g));
    const double beta = 2 * g / ::sqrt(1 + g * g);
    const double E0 = ::sqrt(2 * Ui / kE * Ui / kE * Ui / kHbar * m / kHbar);
    const float neff = (float)(Z / ::sqrt(2 * Ui / kHartree));
    double Q = 0;
    if (g > 0.1) {
        const int sumN = (int)::ceil(10 / alpha);
        for (int k = 0; k < sumN; k++) {
            const double x = k + nu0 - nu;
            Q += ::exp(-alpha * x) * dawson(::sqrt(beta * x));
        }
    } else {
        Q = ::sqrt(3 * kPi) / 4 / g / g;
    }
    const double Cnl2 = ::pow(2.0, 2.0 * neff) / (neff * ::tgamma(2.0 * neff));
    double lnW = ::log(4 * ::sqrt(2.0) / kPi * Cnl2) + ::log(2 * E0 / E / ::sqrt(1 + g * g)) * (2 * neff - 1.5);
    lnW += -2 * nu * (::asinh(g) - g * ::sqrt(1 + g * g) / (1 + 2 * g * g));
    lnW += ::log((2 * l + 1) * Ui / kHbar * g * g / (1 + g * g) * Q);
    return lnW;
}

// seeded standard normals of the start-field noise: splitmix64 counter stream, Box-Muller
GS_HD uint64_t splitmix(uint64_t seed, uint64_t j) {
    uint64_t z = seed + (j + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
GS_HD double seeded_normal(uint64_t seed, uint64_t k) {
    const double u1 = ((double)(splitmix(seed, 2 * k) >> 11) + 0.5) * 0x1.0p-53;
    const double u2 = ((double)(splitmix(seed, 2 * k + 1) >> 11) + 0.5) * 0x1.0p-53;
    return ::sqrt(-2.0 * ::log(u1)) * ::cos(2.0 * kPi * u2);
}

}  // namespace gsm
