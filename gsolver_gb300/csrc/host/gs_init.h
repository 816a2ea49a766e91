// gs_init.h -- the device side of the set-up (gs_init.cu), called by gs_setup.cpp.
#pragma once
#include <stdint.h>

#include <string>

struct GgDevArgs {
    int nr, nt;
    double tmin, tstep, tau, sgT, sgR, cep, C, A0, ro, rmax, f, Cw, w0, field_denom, sigma;
    uint64_t seed;
};

// The per-omega tables (process_input.cpp:569-871, solver_main.cpp:385-413): calculate_omega,
// calculate_wavenumber from the RAW table (linear interpolation in |omega|, PRESSURE scaling,
// the absorbing layer above the grid's top), calculate_HOdispersion with its filters, the
// plasma function, the Kerr profile and the Raman function.  ngr: the group index at OMEGA0;
// omax / omin: the RAW table's range; m: the carriers' mass; M: the Raman normalisation.
struct OmDevArgs {
    int nt;
    double w0, wstep, P, wmax_grid, omax, omin, ngr, c, layer_w, layer_b;
    double tau_c, e, m, mu0, n2s, fR, M, tauR, omR, tstep;
};
// wn, pf, rm: [nt] complex (interleaved); ho, kerr: [nt]; raw_n interleaved (re, im)
int gsi_dev_omega_tables(int device, const OmDevArgs& a, const double* raw_w, const double* raw_n, int nraw,
                         double* wn, double* ho, double* pf, double* rm, double* kerr, std::string* err);
// rate table entries 0..8190 (8191 left 0); gas: PPT with (Z, l), else Keldysh with mred
int gsi_dev_rate_table(int device, int gas, double k0, double U, double w0, double vg, double mred, double Z, int l,
                       double denom_ln, double min_ln, double tol, double* out8192, std::string* err);
// C[i + nr j] = 2/S J0(zz_i zz_j / S) / (m1_i m1_j)
int gsi_dev_qdht_matrix(int device, const double* zz, const double* m1, double S, int nr, double* C, std::string* err);
// create_gg's FIELD [nr][nt] complex (interleaved) and max |IFFT(FIELD)/N_T|^2
int gsi_dev_create_gg(int device, const GgDevArgs& g, const double* x, const double* kr, const double* om, double* field,
                      double* maxI, std::string* err);
