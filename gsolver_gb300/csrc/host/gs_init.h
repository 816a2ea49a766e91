// gs_init.h -- the device side of the set-up (gs_init.cu), called by gs_setup.cpp.
#pragma once
#include <stdint.h>

#include <string>

struct GgDevArgs {
    int nr, nt;
    double tmin, tstep, tau, sgT, sgR, cep, C, A0, ro, rmax, f, Cw, w0, field_denom, sigma;
    uint64_t seed;
};

// rate table entries 0..8190 (8191 left 0); gas: PPT with (Z, l), else Keldysh with mred
int gsi_dev_rate_table(int device, int gas, double k0, double U, double w0, double vg, double mred, double Z, int l,
                       double denom_ln, double min_ln, double tol, double* out8192, std::string* err);
// C[i + nr j] = 2/S J0(zz_i zz_j / S) / (m1_i m1_j)
int gsi_dev_qdht_matrix(int device, const double* zz, const double* m1, double S, int nr, double* C, std::string* err);
// create_gg's FIELD [nr][nt] complex (interleaved) and max |IFFT(FIELD)/N_T|^2
int gsi_dev_create_gg(int device, const GgDevArgs& g, const double* x, const double* kr, const double* om, double* field,
                      double* maxI, std::string* err);
