// gs_setup.cpp -- host set-up of one pulse from a reference-format config (FP64, C++).
//
// The part of the reference's start-up that feeds the hot path: the KEY value config
// lookups (process_input.cpp:297-482), the omega grid and k(omega) (569-623), RAW
// dispersion interpolation (677-721), HO dispersion with its filters (806-871), the
// nonlinear constants (211-250, solver_main.cpp:346-393), the Raman response
// (solver_main.cpp:401-413), the Keldysh rate table (ionization.cpp:203-232, 313-355),
// the QDHT matrix (fhatha.cpp:177-198), the Kerr profile (process_input.cpp:966-975),
// the Gaussian start field (pulse_gg.cpp:6-124) and the first dz (process_input.cpp:734-753).
// Special functions are computed here from their mathematics: J0/J1 from the C library,
// Bessel zeros by McMahon's expansion refined with Newton, Dawson's integral by its
// Maclaurin series (|x| <= 7) or asymptotic series, K/E by the arithmetic-geometric mean.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "gs_setup.h"
#include "gs_init.h"
#include "gs_init_math.h"

namespace {

using cd = std::complex<double>;
using gsm::dawson;
using gsm::ellipke;
using gsm::keldysh_rate_ln;
using gsm::ppt_rate_ln;
using gsm::seeded_normal;

const double kC = 299792458.0;            // SIconstants.h
const double kMu0 = 1.2566370615e-6;
const double kE = 1.60217733e-19;
const double kMe = 9.1093897e-31;
const double kHbar = 1.0545727e-34;
const double kTol = 0.003304003148325;    // solver.h:63-74
const double kMinLn = 29.933606208922594;
const double kIntDenom = 1e16, kFieldDenom = 1e8, kIonDenom = 1e20, kIonDenomLn = 46.0517018;
const double kLayerW = 0.1, kLayerB = 10.0;
const double kIonDenomGas = 1e10, kIonDenomGasLn = 23.025850929940457;   // IONIZATION_GAS (solver.h:86-92)
const double kHartree = 4.359748124303985e-018;                            // SIconstants.h:35

struct Cfg {
    std::vector<std::pair<std::string, std::string>> pairs, over;
    std::string dir;
    const std::string* raw(const char* k) const {
        for (auto& p : over) if (p.first == k) return &p.second;
        for (auto& p : pairs) if (p.first == k) return &p.second;
        return nullptr;
    }
    double f(const char* k) const {
        const std::string* v = raw(k);
        if (!v) throw std::string("load_namedparameter: parameter ") + k + " not found";
        return std::atof(v->c_str());
    }
    double f(const char* k, double d) const { const std::string* v = raw(k); return v ? std::atof(v->c_str()) : d; }
    int i(const char* k) const {
        const std::string* v = raw(k);
        if (!v) throw std::string("load_namedint: parameter ") + k + " not found";
        return std::atoi(v->c_str());
    }
    // load_namednumfloat (process_input.cpp:321-343): NAMEi, then NAME
    double num(const char* k, int i) const {
        const std::string ki = std::string(k) + std::to_string(i);
        const std::string* v = raw(ki.c_str());
        if (!v) v = raw(k);
        if (!v) throw std::string("load_namednumfloat: parameter ") + ki + " not found";
        return std::atof(v->c_str());
    }
    std::string s(const char* k, const char* d = nullptr) const {
        const std::string* v = raw(k);
        if (!v) {
            if (!d) throw std::string("parameter ") + k + " not found";
            return d;
        }
        return *v;
    }
};

// twiddles exp(sign 2 pi i k / n), k < n/2, of fft() below
std::vector<cd> fft_twiddles(size_t n, int sign) {
    std::vector<cd> tw(n / 2);
    for (size_t k = 0; k < n / 2; k++) {
        const double ang = sign * 2.0 * M_PI * (double)k / (double)n;
        tw[k] = cd(std::cos(ang), std::sin(ang));
    }
    return tw;
}

void fft(std::vector<cd>& a, const std::vector<cd>& tw) {   // unnormalised, FFTW sign convention, n = 2^m
    const size_t n = a.size();
    for (size_t i = 1, j = 0; i < n; i++) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    for (size_t len = 2; len <= n; len <<= 1) {
        const size_t step = n / len;
        for (size_t i = 0; i < n; i += len)
            for (size_t k = 0; k < len / 2; k++) {
                const cd w = tw[k * step];
                const cd u = a[i + k], v = a[i + k + len / 2] * w;
                a[i + k] = u + v;
                a[i + k + len / 2] = u - v;
            }
    }
}

void fft(std::vector<cd>& a, int sign) { fft(a, fft_twiddles(a.size(), sign)); }

// f(i, worker) for i < n spread over the host's cores; each i is computed as it would be alone
template <typename F>
void parallel_for(int n, F f, unsigned* workers = nullptr) {
    unsigned nth = std::thread::hardware_concurrency();
    if (nth < 1) nth = 1;
    if (nth > 64) nth = 64;
    if ((int)nth > n) nth = n > 0 ? (unsigned)n : 1u;
    if (workers) *workers = nth;
    if (nth == 1) {
        for (int i = 0; i < n; i++) f(i, 0u);
        return;
    }
    std::vector<std::thread> pool;
    for (unsigned w = 0; w < nth; w++)
        pool.emplace_back([&, w]() {
            for (int i = (int)w; i < n; i += (int)nth) f(i, w);
        });
    for (std::thread& t : pool) t.join();
}

unsigned worker_count(int n) {
    unsigned nth = std::thread::hardware_concurrency();
    if (nth < 1) nth = 1;
    if (nth > 64) nth = 64;
    if ((int)nth > n) nth = n > 0 ? (unsigned)n : 1u;
    return nth;
}

double bessel_j0_zero(int s) {   // s-th positive zero of J0
    const double b = (s - 0.25) * M_PI;
    double x = b + 1.0 / (8 * b) - 124.0 / (3 * std::pow(8 * b, 3)) + 120928.0 / (15 * std::pow(8 * b, 5));
    for (int it = 0; it < 8; it++) {
        const double dx = ::j0(x) / ::j1(x);
        x += dx;
        if (std::fabs(dx) < 1e-16 * x) break;
    }
    return x;
}





struct RawDisp {
    std::vector<double> w, n;   // n interleaved re, im
};

RawDisp read_rawdisp(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::string("Unable to open file with refractive index information! ") + path;
    int hdr[2];
    RawDisp d;
    bool ok = std::fread(hdr, sizeof(int), 2, f) == 2 && hdr[0] == 3 && hdr[1] > 1;
    if (ok) {
        d.w.resize(hdr[1]);
        d.n.resize(2 * (size_t)hdr[1]);
        ok = std::fread(d.w.data(), 8, hdr[1], f) == (size_t)hdr[1] &&
             std::fread(d.n.data(), 8, 2 * (size_t)hdr[1], f) == 2 * (size_t)hdr[1];
    }
    std::fclose(f);
    if (!ok) throw std::string("only RAW (type 3) dispersion files are supported");
    return d;
}

// load_refrindex_raw: first bracketing interval, linear interpolation in |omega|
cd refr_index(const RawDisp& d, double w, double P) {
    const std::vector<double>& pw = d.w;
    size_t j = std::lower_bound(pw.begin(), pw.end(), w) - pw.begin();
    if (j == 0) j = 1;
    if (j >= pw.size()) return cd(1, 0);
    if ((pw[j - 1] - w) * (pw[j] - w) > 0) return cd(1, 0);
    const double ren_ = P * (d.n[2 * j - 2] - 1) + 1, imn_ = P * d.n[2 * j - 1];
    const double ren = P * (d.n[2 * j] - 1) + 1, imn = P * d.n[2 * j + 1];
    const double renc = ren_ + (ren - ren_) * (std::fabs(w) - pw[j - 1]) / (pw[j] - pw[j - 1]);
    const double imnc = imn_ + (imn - imn_) * (std::fabs(w) - pw[j - 1]) / (pw[j] - pw[j - 1]);
    return cd(renc, imnc);
}


}  // namespace

struct gs_setup {
    int nr = 0, nt = 0;
    gs_params p{};
    std::vector<double> rate, pf, rm, kerr, omega, wavenum, ho, kt2, C, m1, x, field, znet;
    std::vector<double> ap_z, ap_r;   // apertures, the reference's array order (last applied first)
    double r_max = 0, dz0 = 0, group_velocity = 0;
    std::string err;
};

// dev < 0: everything on the host; dev >= 0: the rate table, the QDHT matrix and the start
// field are built on that GPU (gs_init.cu), the rest on the host
static void build(gs_setup* s, const Cfg& cfg, unsigned long long seed, double sigma, int dev) {
    std::string derr;
    const double lam = cfg.f("LAMBDA_V");
    const double w0 = 2 * M_PI * kC / lam;
    double tmin = cfg.f("T_MIN", NAN);
    tmin = cfg.f("T_MIN_OMEGA", tmin * w0) / w0;
    double tmax = cfg.f("T_MAX", NAN);
    tmax = cfg.f("T_MAX_OMEGA", tmax * w0) / w0;
    const int nt = cfg.i("N_T");
    if (nt < 64 || (nt & (nt - 1))) throw std::string("N_T must be a power of two >= 64");
    const double tstep = (tmax - tmin) / nt;
    // calculate_omega
    std::vector<double> om(nt);
    const double wstep = 2 * M_PI / (tmax - tmin);
    for (int i = 0; i < nt / 2; i++) om[i] = w0 + wstep * i;
    for (int i = nt / 2; i < nt; i++) om[i] = w0 - wstep * (nt - i);
    const double P = cfg.f("PRESSURE", 1);
    std::string df = cfg.s("DISPERSION_FILE", "NO");
    if (df == "NO") throw std::string("a RAW dispersion file is required");
    if (df[0] != '/') df = cfg.dir + "/" + df;
    const RawDisp rd = read_rawdisp(df);
    double omax = *std::max_element(rd.w.begin(), rd.w.end()), omin = *std::min_element(rd.w.begin(), rd.w.end());
    // calculate_wavenumber (the per-omega tables on the GPU when dev >= 0: below)
    std::vector<cd> n(nt), k(nt);
    const double wmax_grid = *std::max_element(om.begin(), om.end());
    const double omax_raw = omax, omin_raw = omin;
    if (dev < 0) {
        for (int i = 0; i < nt; i++) {
            n[i] = refr_index(rd, om[i], P);
            k[i] = std::conj(n[i]) * om[i] / kC;
            const double d = (om[i] / wmax_grid - 1 - kLayerW) / kLayerW;
            if (d > 0) k[i] = cd(k[i].real(), k[i].imag() + (-k[i].real()) * (std::exp(kLayerB) * d * d));
        }
    }
    const cd k0 = std::conj(refr_index(rd, w0, P)) * w0 / kC;
    // calculate_HOdispersion (OMEGA0 == OMEGA[0]): the group index from n at OMEGA[0], OMEGA[1]
    // and OMEGA[N_T - 1]
    const double n0 = refr_index(rd, om[0], P).real();
    const double dndw = (refr_index(rd, om[1], P) - refr_index(rd, om[nt - 1], P)).real() / (om[1] - om[nt - 1]);
    const double ngr = n0 + w0 * dndw;
    std::vector<double> ho(nt);
    if (dev < 0) {
        for (int i = 0; i < nt; i++) {
            double h = (om[i] / kC) * (n[i].real() - ngr);
            double dh = (om[i] / omax - 1) / kLayerW;
            const double hf = dh < 0 ? 1.0 : std::exp(-kLayerB * dh * dh);
            double dl = om[i] * (1 - kLayerW) / omin - 1;
            const double lf = dl > 0 ? 1.0 : std::exp(-kLayerB * dl * dl);
            ho[i] = h * (lf * hf);
        }
    }
    const double vg = kC / ngr;
    omax = std::min(omax, (1 - kLayerW) * om[nt / 2 - 1]);
    const double tol = cfg.f("MAX_TOLERANCE", 1e-4);
    const int nr = cfg.i("N_R");
    const double rmax = cfg.f("R_MAX");
    const int nz = cfg.i("N_Z");
    const double zmin = cfg.f("Z_MIN", 0), zmax = cfg.f("Z_MAX", 0);
    const std::string zt = cfg.s("ZNET_TYPE");
    if (zt.empty() || zt[0] != 'e') throw std::string("only equidistant z nets are supported");
    std::vector<double> znet(nz);
    const double zs = (zmax - zmin) / (nz - 1);
    for (int i = 0; i < nz; i++) znet[i] = zmin + i * zs;
    // apertures (process_input.cpp:176-179): entry i holds APERTURE_Z/R number N-1-i
    const int n_ap = (int)cfg.f("APERTURE_N", 0);
    for (int i = 0; i < n_ap; i++) {
        s->ap_z.push_back(cfg.num("APERTURE_Z", n_ap - i - 1));
        s->ap_r.push_back(cfg.num("APERTURE_R", n_ap - i - 1));
    }
    const double ambient = cfg.f("AMBIENT_CARRIERS", 0) * cfg.f("NEUTRAL_DENSITY", 0);
    if (ambient != 0)
        throw std::string("AMBIENT_CARRIERS != 0 draws an unseeded random start density per row; not supported");
    const double n2 = cfg.f("NONLIN_REFRINDEX", 0) * P;
    const double fR = cfg.f("RAMAN_FRACTION"), tauR = cfg.f("TAU_RAMAN"), omR = cfg.f("OMEGA_RAMAN");
    const double rho_n = cfg.f("NEUTRAL_DENSITY") * P;
    const double tau_rec = cfg.f("RECOMBINATION_TAU"), tau_c = cfg.f("COLLISION_TAU") / P;
    // the binary the reference would run: gsolver_solid_qdht (default) or gsolver_gas_qdht
    const std::string build_kind = cfg.s("GSOLVER_BUILD", "solid_qdht");
    if (build_kind != "solid_qdht" && build_kind != "gas_qdht")
        throw std::string("GSOLVER_BUILD ") + build_kind + ": solid_qdht or gas_qdht";
    const bool gas = build_kind == "gas_qdht";
    const double ion_denom = gas ? kIonDenomGas : kIonDenom;
    double th_coeff = 0;
    if (gas) {
        if (cfg.f("NONLIN_REFRINDEX4", 0) != 0) throw std::string("NONLIN_REFRINDEX4 != 0 is not supported");
        if (cfg.s("TH_PROFILE", "NO") != "NO" || cfg.s("KERR_PROFILE", "NO") != "NO")
            throw std::string("KERR_PROFILE / TH_PROFILE files are not supported");
        th_coeff = (1 - cfg.f("RAMAN_FRACTION")) / 3.0 * cfg.f("TH_FACTOR", 1);
    }
    // MULTI_LEVEL_IONIZATION (ionization.cpp:45-84): IONIZATION_LEVEL_N levels, level n's
    // potential by load_namednumfloat("IONIZATION_POTENTIAL", n + 1) (NAMEn, then NAME)
    const int levels = gas ? (int)cfg.f("IONIZATION_LEVEL_N", 1) : 1;
    if (levels < 1 || levels > GS_MAX_ION_LEVELS) throw std::string("IONIZATION_LEVEL_N out of range (1..8)");
    std::vector<double> pots(levels);
    for (int n = 0; n < levels; n++) {
        const std::string k = "IONIZATION_POTENTIAL" + std::to_string(n + 1);
        pots[n] = (cfg.raw(k.c_str()) ? cfg.f(k.c_str()) : cfg.f("IONIZATION_POTENTIAL")) * kE;
    }
    // load_namednumfloat("IONIZATION_POTENTIAL", 1) for the gas build: NAME1, then NAME
    const double Ui = (gas && cfg.raw("IONIZATION_POTENTIAL1") ? cfg.f("IONIZATION_POTENTIAL1")
                                                                : cfg.f("IONIZATION_POTENTIAL")) * kE;
    const double mred = cfg.f("REDUCED_MASS", 1);
    const double m = kMe * mred;
    // QDHT plan
    std::vector<double> zz(nr + 1);
    for (int i = 0; i <= nr; i++) zz[i] = bessel_j0_zero(i + 1);
    const double S = zz[nr], V = S / 2.0 / M_PI;
    std::vector<double> x(nr), m1(nr), Cm((size_t)nr * nr), kt2(nr);
    for (int i = 0; i < nr; i++) m1[i] = std::fabs(::j1(zz[i]));
    if (dev >= 0) {
        if (gsi_dev_qdht_matrix(dev, zz.data(), m1.data(), S, nr, Cm.data(), &derr)) throw "device set-up: " + derr;
    } else {
        parallel_for(nr, [&](int i, unsigned) {
            for (int j = 0; j < nr; j++)
                Cm[(size_t)i + (size_t)nr * j] = 2.0 / S * ::j0(zz[i] * zz[j] / S) / m1[i] / m1[j];
        });
    }
    for (int i = 0; i < nr; i++) {
        x[i] = zz[i] / S;
        const double kt = 2 * M_PI * x[i] * V / rmax;
        kt2[i] = kt * kt;
    }
    // plasma constants
    const double k0r = k0.real();
    const double IBS = kE / m * kE * kMu0 / k0r;
    const double aval = IBS * w0 * tau_c / (1 + w0 * tau_c * w0 * tau_c);
    const double pond = IBS / 2.0 / k0r / vg / (1.0 + 1.0 / (w0 * tau_c));
    std::vector<double> pf(2 * (size_t)nt), rm(2 * (size_t)nt), kerr(nt), wn(2 * (size_t)nt);
    const double n2s = n2 * kIntDenom;
    const double Mr = tstep * (1 + omR * omR * tauR * tauR) / tauR / (omR * tauR);
    if (dev >= 0) {   // k, HO dispersion, plasma function, Raman function, Kerr profile on the GPU
        OmDevArgs oa{};
        oa.nt = nt; oa.w0 = w0; oa.wstep = wstep; oa.P = P; oa.wmax_grid = wmax_grid;
        oa.omax = omax_raw; oa.omin = omin_raw; oa.ngr = ngr; oa.c = kC; oa.layer_w = kLayerW; oa.layer_b = kLayerB;
        oa.tau_c = tau_c; oa.e = kE; oa.m = m; oa.mu0 = kMu0; oa.n2s = n2s;
        oa.fR = fR; oa.M = Mr; oa.tauR = tauR; oa.omR = omR; oa.tstep = tstep;
        if (gsi_dev_omega_tables(dev, oa, rd.w.data(), rd.n.data(), (int)rd.w.size(), wn.data(), ho.data(), pf.data(),
                                 rm.data(), kerr.data(), &derr))
            throw "device set-up: " + derr;
        for (int i = 0; i < nt; i++) k[i] = cd(wn[2 * i], wn[2 * i + 1]);
    }
    for (int i = 0; i < nt && dev < 0; i++) {
        const double a = tau_c * om[i];
        const cd v = -(a / cd(1.0, a) / 2.0 / k[i].real() * kE * kE / m * kMu0);
        pf[2 * i] = v.real();
        pf[2 * i + 1] = v.imag();
        wn[2 * i] = k[i].real();
        wn[2 * i + 1] = k[i].imag();
    }
    // Keldysh table (top entry left at zero as in the reference)
    // entries are independent: spread them over the host's cores (each is computed exactly
    // as it would be alone)
    std::vector<double> rate(8192 * (size_t)levels, 0.0);
    if (levels > 1) {   // level 0 with PPT_Z, level n >= 1 with Z = n + 1 (ionization.cpp:313-331)
        const int l = (int)cfg.f("PPT_L", 0);
        for (int n = 0; n < levels; n++) {
            const double Z = n == 0 ? cfg.f("PPT_Z", 1) : (double)(n + 1);
            double* row = rate.data() + 8192 * (size_t)n;
            parallel_for(8191, [&](int i, unsigned) {
                row[i] = ppt_rate_ln(kMinLn + kTol * i, pots[n], Z, l, k0r, w0, vg) - kIonDenomGasLn;
            });
        }
    } else if (dev >= 0) {
        if (gsi_dev_rate_table(dev, gas ? 1 : 0, k0r, Ui, w0, vg, mred, cfg.f("PPT_Z", 1), (int)cfg.f("PPT_L", 0),
                               gas ? kIonDenomGasLn : kIonDenomLn, kMinLn, kTol, rate.data(), &derr))
            throw "device set-up: " + derr;
    } else if (gas) {
        const double Z = cfg.f("PPT_Z", 1);
        const int l = (int)cfg.f("PPT_L", 0);
        parallel_for(8191, [&](int i, unsigned) {
            rate[i] = ppt_rate_ln(kMinLn + kTol * i, Ui, Z, l, k0r, w0, vg) - kIonDenomGasLn;
        });
    } else {
        parallel_for(8191, [&](int i, unsigned) {
            rate[i] = keldysh_rate_ln(kMinLn + kTol * i, k0r, Ui, w0, vg, mred) - kIonDenomLn;
        });
    }
    // Raman response
    if (dev < 0) {
        const double M = Mr;
        std::vector<cd> h(nt);
        for (int t = 0; t < nt; t++) {
            const double tt = tstep * t;
            h[t] = cd(fR * M * std::exp(-tt / tauR) * std::sin(omR * tt), 0);
        }
        fft(h, -1);
        for (int i = 0; i < nt; i++) {
            rm[2 * i] = h[i].real() + (1 - fR);
            rm[2 * i + 1] = h[i].imag();
        }
    }
    for (int i = 0; i < nt && dev < 0; i++) kerr[i] = n2s * om[i] / kC / k[i].real() * om[i] / kC;

    // create_gg
    double tau_fwhm = cfg.f("DURATION_FWHM", -1);
    tau_fwhm = cfg.f("DURATION_FWHM_OMEGA", tau_fwhm * w0) / w0;
    if (tau_fwhm < 0) throw std::string("create_gg(): DURATION_FWHM or DURATION_FWHM_OMGEA should be specified!");
    const double d_fwhm = cfg.f("DIAMETER_FWHM");
    const double cep = cfg.f("CE_PHASE", 0);
    const double sgT = cfg.f("PULSE_SG_ORDER", 1), sgR = cfg.f("BEAM_SG_ORDER", 1);
    double E = cfg.f("ENERGY", -1);
    const double EP = 2 * std::pow(std::log(2.0), 1.0 / 2.0 / sgT) / std::tgamma(1.0 / 2.0 / sgT);
    const double Pcr = 2 * M_PI * kC / k0r / w0 / n2s * kIntDenom;
    double P0 = cfg.f("POWER_CR", E / tau_fwhm * EP / Pcr) * Pcr;
    P0 = cfg.f("POWER", P0);
    E = P0 * tau_fwhm / EP;
    if (E < 0) throw std::string("create_gg(): ENERGY or POWER parameter should be specified!");
    const double A0 = std::sqrt(P0 / d_fwhm / d_fwhm * 4 * std::pow(std::log(2.0), 1.0 / sgR) / M_PI / std::tgamma(1.0 / sgR));
    const double tau = tau_fwhm / 2.0 / std::pow(std::log(std::sqrt(2.0)), 1.0 / 2.0 / sgT);
    const double ro = d_fwhm / 2.0 / std::pow(std::log(std::sqrt(2.0)), 1.0 / 2.0 / sgR);
    const double zR = k0r * ro * ro / 2;
    double C = cfg.f("CHIRP_SI", 0);
    C = cfg.f("CHIRP", C * tau * tau);
    const double Cw = cfg.f("CHIRP_SPECTRAL", 0);
    double f = cfg.f("FOCUSING_DISTANCE", 0);
    f = cfg.f("FOCUSING_DISTANCE_DIFFRACTION", f / zR);
    if (zR > 2 * f) f = zR * zR / 2 / f * (1 - std::sqrt(1 - 4 * f * f / zR / zR));
    f = cfg.f("WAVEFRONT_RADIUS", f);
    f = cfg.f("WAVEFRONT_RADIUS_DIFFRACTION", f / zR) * zR;
    std::vector<double> field(2 * (size_t)nr * nt);
    double maxI = 0;
    if (dev >= 0) {
        GgDevArgs g{};
        g.nr = nr; g.nt = nt; g.tmin = tmin; g.tstep = tstep; g.tau = tau; g.sgT = sgT; g.sgR = sgR; g.cep = cep;
        g.C = C; g.A0 = A0; g.ro = ro; g.rmax = rmax; g.f = f; g.Cw = Cw; g.w0 = w0; g.field_denom = kFieldDenom;
        g.sigma = sigma; g.seed = seed;
        std::vector<double> kr(nt);
        for (int w = 0; w < nt; w++) kr[w] = k[w].real();
        if (gsi_dev_create_gg(dev, g, x.data(), kr.data(), om.data(), field.data(), &maxI, &derr))
            throw "device set-up: " + derr;
    } else {
    const unsigned nw = worker_count(nr);
    std::vector<std::vector<cd>> rows(nw, std::vector<cd>(nt));
    const std::vector<cd> tw_fw = fft_twiddles(nt, -1), tw_bw = fft_twiddles(nt, +1);
    parallel_for(nr, [&](int r, unsigned wk) {
        std::vector<cd>& row = rows[wk];
        const double R = x[r] * rmax;
        const double amax = A0 * std::exp(-std::pow(R / ro, 2.0 * sgR));
        for (int t = 0; t < nt; t++) {
            const double tt = tmin + tstep * t, T = tt / tau;
            const double cph = cep - T * T * C;
            cd car(std::cos(cph), std::sin(cph));
            if (sigma != 0) {
                const uint64_t kk = 2 * ((uint64_t)r * nt + t);
                car += sigma * cd(seeded_normal(seed, kk), seeded_normal(seed, kk + 1));
            }
            row[t] = (amax * std::exp(-std::pow(T, 2.0 * sgT))) * car;
        }
        fft(row, tw_fw);
        for (int w = 0; w < nt; w++) {
            const double ph = (R * R * k[w].real() / 2.0 / f) - Cw * (om[w] - w0) * (om[w] - w0) / 2;
            const cd v = row[w] * cd(std::cos(ph), std::sin(ph)) / kFieldDenom;
            field[2 * ((size_t)r * nt + w)] = v.real();
            field[2 * ((size_t)r * nt + w) + 1] = v.imag();
        }
    });
    // init_zstep_kerr: max |IFFT(FIELD)/N_T|^2 (per-row maxima, then their max)
    std::vector<double> rmaxI(nr, 0.0);
    parallel_for(nr, [&](int r, unsigned wk) {
        std::vector<cd>& row = rows[wk];
        for (int w = 0; w < nt; w++) row[w] = cd(field[2 * ((size_t)r * nt + w)], field[2 * ((size_t)r * nt + w) + 1]);
        fft(row, tw_bw);
        double m = 0;
        for (int t = 0; t < nt; t++) m = std::max(m, std::norm(row[t] / (double)nt));
        rmaxI[r] = m;
    });
    for (int r = 0; r < nr; r++) maxI = std::max(maxI, rmaxI[r]);
    }
    double dz = znet.size() > 1 ? znet[1] - znet[0] : 0;
    const double kNL = w0 / kC * n2s * maxI;
    if (dz * kNL > tol) dz = tol / kNL;

    s->nr = nr;
    s->nt = nt;
    gs_params& p = s->p;
    std::memset(&p, 0, sizeof(p));
    p.n_r = nr;
    p.n_t = nt;
    p.nonlinear = 1;
    p.tstep = tstep; p.tmin = tmin; p.tmax = tmax; p.omega0 = w0;
    p.ionrate_denom = ion_denom;
    p.gas = gas ? 1 : 0;
    p.th_coeff = th_coeff;
    p.ion_levels = levels;
    for (int n = 0; n < levels && levels > 1; n++) p.ion_potentials[n] = pots[n] * (ion_denom / kIntDenom);
    p.neutral_density = rho_n;
    p.rho0 = 0.0;   // AMBIENT_CARRIERS*2*frand() with AMBIENT_CARRIERS = 0
    p.ionization_potential = Ui * (ion_denom / kIntDenom);
    p.ponderomotive = pond * ion_denom;
    p.avalanche_cs = aval;
    p.recombination_tau = tau_rec * ion_denom;
    p.raman_fraction = fR;
    p.n2 = n2s;
    p.omega_min = omin;
    p.omega_max = omax;
    p.max_tolerance = tol;
    p.raman_tau = tauR;
    p.raman_omega = omR;
    s->rate = std::move(rate); s->pf = std::move(pf); s->rm = std::move(rm); s->kerr = std::move(kerr);
    s->omega = std::move(om); s->wavenum = std::move(wn); s->ho = std::move(ho); s->kt2 = std::move(kt2);
    s->C = std::move(Cm); s->m1 = std::move(m1); s->x = std::move(x); s->field = std::move(field);
    s->znet = std::move(znet);
    s->r_max = rmax;
    s->dz0 = dz;
    s->group_velocity = vg;
}

static std::string g_setup_err;

static int setup_impl(const char* path, int n_over, const char* const* keys, const char* const* vals,
                      unsigned long long noise_seed, double noise_sigma, int dev, gs_setup** out);

int gs_setup_from_config(const char* path, int n_over, const char* const* keys, const char* const* vals,
                         unsigned long long noise_seed, double noise_sigma, gs_setup** out) {
    return setup_impl(path, n_over, keys, vals, noise_seed, noise_sigma, -1, out);
}

int gs_setup_from_config_dev(const char* path, int n_over, const char* const* keys, const char* const* vals,
                             unsigned long long noise_seed, double noise_sigma, int device, gs_setup** out) {
    if (device < 0) { g_setup_err = "gs_setup_from_config_dev: device ordinal < 0"; return GS_ERR_ARG; }
    return setup_impl(path, n_over, keys, vals, noise_seed, noise_sigma, device, out);
}

static int setup_impl(const char* path, int n_over, const char* const* keys, const char* const* vals,
                      unsigned long long noise_seed, double noise_sigma, int dev, gs_setup** out) {
    if (!path || !out) return GS_ERR_ARG;
    *out = nullptr;
    FILE* f = std::fopen(path, "r");
    if (!f) { g_setup_err = "Error opening file with starting condition."; return GS_ERR_ARG; }
    Cfg cfg;
    char a[512], b[512];
    while (std::fscanf(f, "%511s %511s", a, b) == 2) cfg.pairs.emplace_back(a, b);
    std::fclose(f);
    for (int i = 0; i < n_over; i++) cfg.over.emplace_back(keys[i], vals[i]);
    std::string dir(path);
    const size_t sl = dir.find_last_of('/');
    cfg.dir = sl == std::string::npos ? "." : dir.substr(0, sl);
    gs_setup* s = new gs_setup();
    try {
        build(s, cfg, noise_seed, noise_sigma, dev);
    } catch (const std::string& e) {
        g_setup_err = e;
        delete s;
        return GS_ERR_ARG;
    }
    *out = s;
    return GS_OK;
}

const char* gs_setup_last_error(void) { return g_setup_err.c_str(); }

int gs_setup_grid(const gs_setup* s, int* n_r, int* n_t, int* n_z) {
    if (!s) return GS_ERR_ARG;
    if (n_r) *n_r = s->nr;
    if (n_t) *n_t = s->nt;
    if (n_z) *n_z = (int)s->znet.size();
    return GS_OK;
}

int gs_setup_apertures(const gs_setup* s, int* n, double* z, double* r) {
    if (!s || !n) return GS_ERR_ARG;
    *n = (int)s->ap_z.size();
    for (int i = 0; i < *n; i++) {
        if (z) z[i] = s->ap_z[i];
        if (r) r[i] = s->ap_r[i];
    }
    return GS_OK;
}

int gs_setup_params(const gs_setup* s, gs_params* out) {
    if (!s || !out) return GS_ERR_ARG;
    *out = s->p;
    return GS_OK;
}

int gs_setup_tables(const gs_setup* s, gs_tables* t) {
    if (!s || !t) return GS_ERR_ARG;
    t->rate_ln = s->rate.data(); t->plasma_func = s->pf.data(); t->raman_func = s->rm.data();
    t->kerr = s->kerr.data(); t->omega = s->omega.data(); t->wavenum = s->wavenum.data();
    t->ho_disp = s->ho.data(); t->kt2 = s->kt2.data(); t->qdht_c = s->C.data(); t->qdht_m1 = s->m1.data();
    return GS_OK;
}

int gs_setup_field(const gs_setup* s, double* field_r_omega) {
    if (!s || !field_r_omega) return GS_ERR_ARG;
    std::memcpy(field_r_omega, s->field.data(), s->field.size() * sizeof(double));
    return GS_OK;
}

int gs_setup_znet(const gs_setup* s, double* znet, double* init_zstep, double* r_max, double* qdht_x) {
    if (!s) return GS_ERR_ARG;
    if (znet) std::memcpy(znet, s->znet.data(), s->znet.size() * sizeof(double));
    if (init_zstep) *init_zstep = s->dz0;
    if (r_max) *r_max = s->r_max;
    if (qdht_x) std::memcpy(qdht_x, s->x.data(), s->x.size() * sizeof(double));
    return GS_OK;
}

int gs_setup_destroy(gs_setup* s) {
    delete s;
    return GS_OK;
}
