// gs_init.cu -- the set-up's FP64 builds on the GPU (no counterpart in the reference, whose
// initialisation is host code): the ionization-rate table (Keldysh or PPT, 8191 entries,
// each a series of Dawson integrals), the QDHT matrix C (N_r^2 Bessel J0 values) and the
// start field of create_gg (pulse_gg.cpp:6-124: envelope, carrier, seeded noise, one FFT
// per row, wavefront and spectral chirp) with its intensity maximum for init_zstep_kerr
// (process_input.cpp:734-753).  The arithmetic is the host set-up's own (gs_init_math.h);
// results agree with the host build to the last roundings of the two math libraries and of
// fused multiply-adds.  Used by gs_setup_from_config_dev, so batched scans of many pulses
// spend their set-up time on the GPU.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gs_handle.h"
#include "gs_internal.cuh"
#include "gs_kernels.h"
#include "host/gs_init_math.h"
#include "host/gs_init.h"

namespace gs {

__global__ void rate_table_kernel(double* out, int gas, double k0, double U, double w0, double vg, double mred,
                                  double Z, int l, double denom_ln, double min_ln, double tol) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 8191) return;
    const double lnI = min_ln + tol * i;
    out[i] = (gas ? gsm::ppt_rate_ln(lnI, U, Z, l, k0, w0, vg) : gsm::keldysh_rate_ln(lnI, k0, U, w0, vg, mred)) -
             denom_ln;
}

__global__ void qdht_matrix_kernel(double* C, const double* __restrict__ zz, const double* __restrict__ m1, double S,
                                   int nr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= nr || j >= nr) return;
    C[(size_t)i + (size_t)nr * j] = 2.0 / S * j0(zz[i] * zz[j] / S) / m1[i] / m1[j];
}

__global__ void gg_time_kernel(double2* __restrict__ buf, const double* __restrict__ x, GgDevArgs g) {
    const size_t total = (size_t)g.nr * g.nt;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(idx / g.nt), t = (int)(idx % g.nt);
        const double R = x[r] * g.rmax;
        const double amax = g.A0 * ::exp(-::pow(R / g.ro, 2.0 * g.sgR));
        const double tt = g.tmin + g.tstep * t, T = tt / g.tau;
        const double cph = g.cep - T * T * g.C;
        double cr = ::cos(cph), ci = ::sin(cph);
        if (g.sigma != 0) {
            const uint64_t kk = 2 * ((uint64_t)r * g.nt + t);
            cr += g.sigma * gsm::seeded_normal(g.seed, kk);
            ci += g.sigma * gsm::seeded_normal(g.seed, kk + 1);
        }
        const double s = amax * ::exp(-::pow(T, 2.0 * g.sgT));
        buf[idx] = make_double2(s * cr, s * ci);
    }
}

// The per-omega tables, one thread per grid point i (the host build's formulas, gs_setup.cpp):
// omega_i, n(omega_i) from the RAW table (the first bracketing interval, linear in |omega|),
// k = conj(n) omega / c with the absorbing layer, HO dispersion with its two filters, the
// plasma function, the Kerr profile, and the Raman function in closed form: the DFT of
// h_m = fR M e^{-m dt / tau} sin(Omega m dt), m < N, is the geometric sum
//     fR M / (2 j) [(1 - a^N) / (1 - a w^i) - (1 - conj(a)^N) / (1 - conj(a) w^i)],
// a = e^{dt (-1 / tau + j Omega)}, w = e^{-2 pi j / N}, plus 1 - fR.
__global__ void omega_tables_kernel(OmDevArgs a, const double* __restrict__ rw, const double* __restrict__ rn, int nraw,
                                    double* __restrict__ wn, double* __restrict__ ho, double* __restrict__ pf,
                                    double* __restrict__ rm, double* __restrict__ kerr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nt) return;
    const double om = i < a.nt / 2 ? a.w0 + a.wstep * i : a.w0 - a.wstep * (a.nt - i);
    // refr_index: lower_bound of om in the sorted RAW frequencies
    double nre = 1, nim = 0;
    {
        int lo = 0, hi = nraw;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (rw[mid] < om) lo = mid + 1;
            else hi = mid;
        }
        int j = lo == 0 ? 1 : lo;
        if (j < nraw && !((rw[j - 1] - om) * (rw[j] - om) > 0)) {
            const double ren_ = a.P * (rn[2 * j - 2] - 1) + 1, imn_ = a.P * rn[2 * j - 1];
            const double ren = a.P * (rn[2 * j] - 1) + 1, imn = a.P * rn[2 * j + 1];
            nre = ren_ + (ren - ren_) * (fabs(om) - rw[j - 1]) / (rw[j] - rw[j - 1]);
            nim = imn_ + (imn - imn_) * (fabs(om) - rw[j - 1]) / (rw[j] - rw[j - 1]);
        }
    }
    double kr = nre * om / a.c, ki = -nim * om / a.c;
    const double d = (om / a.wmax_grid - 1 - a.layer_w) / a.layer_w;
    if (d > 0) ki = ki + (-kr) * (exp(a.layer_b) * d * d);
    wn[2 * i] = kr;
    wn[2 * i + 1] = ki;
    const double h = (om / a.c) * (nre - a.ngr);
    const double dh = (om / a.omax - 1) / a.layer_w;
    const double hf = dh < 0 ? 1.0 : exp(-a.layer_b * dh * dh);
    const double dl = om * (1 - a.layer_w) / a.omin - 1;
    const double lf = dl > 0 ? 1.0 : exp(-a.layer_b * dl * dl);
    ho[i] = h * (lf * hf);
    // plasma function -(a / (1 + j a)) / 2 / k_r e^2 / m mu0, a = tau_c omega
    {
        const double x = a.tau_c * om, den = 1 + x * x;
        const double s = 1.0 / 2.0 / kr * a.e * a.e / a.m * a.mu0;
        pf[2 * i] = -(x / den) * s;
        pf[2 * i + 1] = -(-x * x / den) * s;
    }
    kerr[i] = a.n2s * om / a.c / kr * om / a.c;
    {
        const double m1 = exp(-a.tstep / a.tauR), mN = exp(-(double)a.nt * a.tstep / a.tauR);
        double s1, c1, sN, cN, sw, cw;
        sincos(a.omR * a.tstep, &s1, &c1);
        sincos(a.omR * a.tstep * a.nt, &sN, &cN);
        sincospi(-2.0 * i / a.nt, &sw, &cw);
        const double2 q = make_double2(m1 * c1, m1 * s1), qN = make_double2(mN * cN, mN * sN);
        // (1 - q^N) / (1 - q w) and its conjugate-q twin
        auto term = [&](double2 p, double2 pN) {
            const double2 num = make_double2(1 - pN.x, -pN.y);
            const double2 den = make_double2(1 - (p.x * cw - p.y * sw), -(p.x * sw + p.y * cw));
            const double dd = den.x * den.x + den.y * den.y;
            return make_double2((num.x * den.x + num.y * den.y) / dd, (num.y * den.x - num.x * den.y) / dd);
        };
        const double2 t1 = term(q, qN), t2 = term(make_double2(q.x, -q.y), make_double2(qN.x, -qN.y));
        const double2 df = make_double2(t1.x - t2.x, t1.y - t2.y);
        const double g = a.fR * a.M / 2;   // (1 / (2 j)) (x + j y) = (y - j x) / 2
        rm[2 * i] = g * df.y + (1 - a.fR);
        rm[2 * i + 1] = -g * df.x;
    }
}

// FIELD = row(omega) exp(j ph) / FIELD_DENOM, ph = R^2 k_r / (2 f) - Cw (omega - omega0)^2 / 2
__global__ void gg_phase_kernel(double2* __restrict__ field, const double2* __restrict__ row, const double* __restrict__ x,
                                const double* __restrict__ kr, const double* __restrict__ om, GgDevArgs g) {
    const size_t total = (size_t)g.nr * g.nt;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(idx / g.nt), w = (int)(idx % g.nt);
        const double R = x[r] * g.rmax;
        const double ph = (R * R * kr[w] / 2.0 / g.f) - g.Cw * (om[w] - g.w0) * (om[w] - g.w0) / 2;
        const double c = ::cos(ph), s = ::sin(ph);
        const double2 v = row[idx];
        field[idx] = make_double2((v.x * c - v.y * s) / g.field_denom, (v.x * s + v.y * c) / g.field_denom);
    }
}

// max over t of |E(r,t)/N|^2 per row (E in natural time order)
__global__ void row_max_intensity_kernel(const double2* __restrict__ E, int N, double* out) {
    const size_t base = (size_t)blockIdx.x * N;
    double m = 0;
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
        const double2 v = E[base + t];
        const double a = v.x / N, b = v.y / N;
        m = fmax(m, a * a + b * b);
    }
    __shared__ double sm[32];
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double M = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) M = fmax(M, sm[w]);
        out[blockIdx.x] = M;
    }
}

}  // namespace gs

namespace {

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

int dev_fail(std::string* err, const char* where, cudaError_t e) {
    if (err) *err = std::string(where) + ": " + cudaGetErrorString(e);
    return 1;
}

#define DCK(expr)                                              \
    do {                                                       \
        cudaError_t _e = (expr);                               \
        if (_e != cudaSuccess) return dev_fail(err, #expr, _e); \
    } while (0)

}  // namespace

int gsi_dev_rate_table(int device, int gas, double k0, double U, double w0, double vg, double mred, double Z, int l,
                       double denom_ln, double min_ln, double tol, double* out8192, std::string* err) {
    DCK(cudaSetDevice(device));
    DevBuf d;
    DCK(cudaMalloc(&d.p, 8192 * sizeof(double)));
    DCK(cudaMemset(d.p, 0, 8192 * sizeof(double)));   // the top entry stays 0 (ionization.cpp:324)
    gs::rate_table_kernel<<<(8191 + 127) / 128, 128>>>((double*)d.p, gas, k0, U, w0, vg, mred, Z, l, denom_ln, min_ln, tol);
    DCK(cudaGetLastError());
    DCK(cudaMemcpy(out8192, d.p, 8192 * sizeof(double), cudaMemcpyDeviceToHost));
    return 0;
}

int gsi_dev_omega_tables(int device, const OmDevArgs& a, const double* raw_w, const double* raw_n, int nraw,
                         double* wn, double* ho, double* pf, double* rm, double* kerr, std::string* err) {
    DCK(cudaSetDevice(device));
    const size_t nt = (size_t)a.nt;
    DevBuf dout, draw;
    DCK(cudaMalloc(&dout.p, nt * 8 * 8));   // wn (2), pf (2), rm (2), ho, kerr
    DCK(cudaMalloc(&draw.p, (size_t)nraw * 3 * 8));
    double* o = (double*)dout.p;
    double* rw = (double*)draw.p;
    DCK(cudaMemcpy(rw, raw_w, (size_t)nraw * 8, cudaMemcpyHostToDevice));
    DCK(cudaMemcpy(rw + nraw, raw_n, (size_t)nraw * 16, cudaMemcpyHostToDevice));
    gs::omega_tables_kernel<<<(unsigned)((nt + 255) / 256), 256>>>(a, rw, rw + nraw, nraw, o, o + 2 * nt, o + 3 * nt,
                                                                  o + 5 * nt, o + 7 * nt);
    DCK(cudaGetLastError());
    DCK(cudaMemcpy(wn, o, nt * 16, cudaMemcpyDeviceToHost));
    DCK(cudaMemcpy(ho, o + 2 * nt, nt * 8, cudaMemcpyDeviceToHost));
    DCK(cudaMemcpy(pf, o + 3 * nt, nt * 16, cudaMemcpyDeviceToHost));
    DCK(cudaMemcpy(rm, o + 5 * nt, nt * 16, cudaMemcpyDeviceToHost));
    DCK(cudaMemcpy(kerr, o + 7 * nt, nt * 8, cudaMemcpyDeviceToHost));
    return 0;
}

int gsi_dev_qdht_matrix(int device, const double* zz, const double* m1, double S, int nr, double* C, std::string* err) {
    DCK(cudaSetDevice(device));
    DevBuf dC, dz, dm;
    DCK(cudaMalloc(&dC.p, (size_t)nr * nr * sizeof(double)));
    DCK(cudaMalloc(&dz.p, nr * sizeof(double)));
    DCK(cudaMalloc(&dm.p, nr * sizeof(double)));
    DCK(cudaMemcpy(dz.p, zz, nr * sizeof(double), cudaMemcpyHostToDevice));
    DCK(cudaMemcpy(dm.p, m1, nr * sizeof(double), cudaMemcpyHostToDevice));
    dim3 grid((nr + 127) / 128, nr);
    gs::qdht_matrix_kernel<<<grid, 128>>>((double*)dC.p, (const double*)dz.p, (const double*)dm.p, S, nr);
    DCK(cudaGetLastError());
    DCK(cudaMemcpy(C, dC.p, (size_t)nr * nr * sizeof(double), cudaMemcpyDeviceToHost));
    return 0;
}

int gsi_dev_create_gg(int device, const GgDevArgs& g, const double* x, const double* kr, const double* om, double* field,
                      double* maxI, std::string* err) {
    using namespace gs;
    DCK(cudaSetDevice(device));
    const int nt = g.nt, nr = g.nr;
    const size_t nel = (size_t)nr * nt;
    // FP64 FFT rows of N = P M, M <= 8192 (one CTA's shared memory)
    const int M = nt <= 8192 ? nt : 8192, P = nt / M;
    if (P > 8) {
        if (err) *err = "device set-up: N_T too large";
        return 1;
    }
    int logM = 0;
    while ((1 << logM) < M) logM++;
    const std::vector<int> perm = gsi::position_map(nt, P, M, logM);
    std::vector<double> tw(2 * (size_t)nt);
    for (int j = 0; j < nt; j++) {
        const double a = 2.0 * gsm::kPi * (double)j / (double)nt;
        tw[2 * j] = ::cos(a);
        tw[2 * j + 1] = -::sin(a);
    }
    DevBuf dA, dB, dx, dkr, dom, dtw, dperm, dmax;
    DCK(cudaMalloc(&dA.p, nel * 16));
    DCK(cudaMalloc(&dB.p, nel * 16));
    DCK(cudaMalloc(&dx.p, nr * 8));
    DCK(cudaMalloc(&dkr.p, nt * 8));
    DCK(cudaMalloc(&dom.p, nt * 8));
    DCK(cudaMalloc(&dtw.p, nt * 16));
    DCK(cudaMalloc(&dperm.p, nt * 4));
    DCK(cudaMalloc(&dmax.p, nr * 8));
    DCK(cudaMemcpy(dx.p, x, nr * 8, cudaMemcpyHostToDevice));
    DCK(cudaMemcpy(dkr.p, kr, nt * 8, cudaMemcpyHostToDevice));
    DCK(cudaMemcpy(dom.p, om, nt * 8, cudaMemcpyHostToDevice));
    DCK(cudaMemcpy(dtw.p, tw.data(), nt * 16, cudaMemcpyHostToDevice));
    DCK(cudaMemcpy(dperm.p, perm.data(), nt * 4, cudaMemcpyHostToDevice));
    DCK(fft_set_smem<double>(M, nt));
    long long nl = 0;
    const unsigned blocks = 152 * 8;
    gg_time_kernel<<<blocks, 256>>>((double2*)dA.p, (const double*)dx.p, g);
    DCK(cudaGetLastError());
    FftArgs<double> fa{};
    fa.N = nt; fa.M = M; fa.P = P; fa.logM = logM; fa.rows = nr;
    fa.tw = (const double2*)dtw.p;
    DCK(launch_fft<double>(-1, (const double2*)dA.p, (double2*)dB.p, fa, nullptr, &nl));       // position order
    DCK(launch_permute<double>(-1, dB.p, dA.p, (const int*)dperm.p, nt, nel, nullptr, &nl));   // natural omega
    gg_phase_kernel<<<blocks, 256>>>((double2*)dB.p, (const double2*)dA.p, (const double*)dx.p, (const double*)dkr.p,
                                     (const double*)dom.p, g);
    DCK(cudaGetLastError());
    DCK(cudaMemcpy(field, dB.p, nel * 16, cudaMemcpyDeviceToHost));
    // init_zstep_kerr: max |IFFT(FIELD)/N_T|^2
    DCK(launch_permute<double>(+1, dB.p, dA.p, (const int*)dperm.p, nt, nel, nullptr, &nl));   // position order
    DCK(launch_fft<double>(+1, (const double2*)dA.p, (double2*)dB.p, fa, nullptr, &nl));        // natural time
    row_max_intensity_kernel<<<nr, 256>>>((const double2*)dB.p, nt, (double*)dmax.p);
    DCK(cudaGetLastError());
    std::vector<double> m(nr);
    DCK(cudaMemcpy(m.data(), dmax.p, nr * 8, cudaMemcpyDeviceToHost));
    double mx = 0;
    for (int r = 0; r < nr; r++) mx = m[r] > mx ? m[r] : mx;
    *maxI = mx;
    return 0;
}
