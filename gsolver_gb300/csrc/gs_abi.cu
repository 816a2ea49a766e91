// gs_abi.cu -- the C ABI (include/gs_abi.h): device state of one pulse and the z-step
// orchestration (propagator / calculate_NLstep / calculate_Lstep / ht_run).
//
// HBM layout per handle (n_r x n_t complex, row-major, omega contiguous, spectral rows in
// FFT position order):  A = FIELD (r,omega), S = BIGBUFFER2 (k,omega),
// NB = BIGBUFFER1 (r,omega), KP = previous RK4 stage, E = time-domain field of the
// stage, U = three scratch rows per radial point (loss, rho*E, Kerr source).
// FP64 handles hold double2, mixed handles float2 (their QDHT tables stay FP64 at
// set-up and are split for the tensor cores).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/gs_abi.h"
#include "gs_handle.h"
#include "gs_internal.cuh"
#include "gs_kernels.h"
#include "gs_qdht_tc.h"

using namespace gs;

static std::string g_create_error;


using gsi::fail;
using gsi::cuda_fail;
using gsi::run_qdht;
using gsi::permute_in;
using gsi::permute_out;
using gsi::lstep;
using gsi::plasma_args;
using gsi::ion_levels;

int gsi::fail(gs_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg; else g_create_error = msg;
    return code;
}
int gsi::cuda_fail(gs_handle* h, cudaError_t e, const char* where) {
    return fail(h, GS_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

static int ilog2(int n) { int l = 0; while ((1 << l) < n) l++; return l; }

// Position -> omega index of the device FFT (gs_internal.cuh): frequency k = k2 + P*k1
// sits at position k2*M + p_local(k1), p_local the mixed-radix digit reversal of the
// radix-16 decimation-in-frequency stages.
static std::vector<int> fft_position_map(int N, int P, int M, int logM) {
    const int J = fft_num_stages(logM);
    std::vector<int> R(J), sub(J), pre(J);
    int prod = 1;
    for (int j = 0; j < J; j++) {
        R[j] = fft_stage_radix(logM, j);
        pre[j] = prod;
        prod *= R[j];
        sub[j] = M / prod;
    }
    std::vector<int> perm(N);
    for (int p = 0; p < N; p++) {
        const int k2 = p / M, pl = p % M;
        int k1 = 0;
        for (int j = 0; j < J; j++) k1 += ((pl / sub[j]) % R[j]) * pre[j];
        perm[p] = k2 + P * k1;
    }
    return perm;
}

std::vector<int> gsi::position_map(int N, int P, int M, int logM) { return fft_position_map(N, P, M, logM); }

// Exported functions take C linkage from their declarations in gs_abi.h.

const char* gs_status_string(int s) {
    switch (s) {
        case GS_OK: return "ok";
        case GS_ERR_ARG: return "bad argument";
        case GS_ERR_CUDA: return "CUDA error";
        case GS_ERR_BLAST: return "Attention!!!! Intensity is too big! Keep away, blast is possible.";
        case GS_ERR_NAN: return "float_type photoionization_function(...): Intensity is nan!";
        case GS_ERR_COLLAPSE: return "Minimum Z step size reached, collapse is possible!";
        case GS_ERR_STATE: return "call out of order";
        case GS_ERR_UNSUPPORTED: return "unsupported grid";
        case GS_ERR_NOMEM: return "device allocation failed";
        default: return "unknown status";
    }
}

const char* gs_last_error(const gs_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

long long gs_launch_count(const gs_handle* h) { return h ? h->launches : 0; }

void* gs_stream(const gs_handle* h) { return h ? (void*)h->st : nullptr; }

static void free_all(gs_handle* h) {
    void* ptrs[] = {h->A, h->S, h->NB, h->KP, h->E, h->U, h->tw, h->pf, h->rm, h->kerr, h->rate,
                    h->omega, h->ho, h->kt2, h->Cm, h->m1, h->wavenum, h->staging, h->perm_dev,
                    h->iperm_dev, h->err_dev, h->max_dev, h->dump_dev, h->m1inv, h->adj, h->adj_w, h->th, h->twb,
                    h->row_ion, h->win64, h->zpos64, h->en_dev, h->en_save};
    for (void* q : ptrs) if (q) cudaFree(q);
    if (h->tc) gs::qdht_tc_destroy(h->tc);
    if (h->tcT) gs::qdht_tc_destroy(h->tcT);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->st) cudaStreamDestroy(h->st);
    for (cudaEvent_t e : h->nl_ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : h->io_ev)
        if (e) cudaEventDestroy(e);
    if (h->io_st) cudaStreamDestroy(h->io_st);
}

int gs_create(const gs_params* prm, gs_handle** out) {
    if (!prm || !out) return fail(nullptr, GS_ERR_ARG, "null argument");
    *out = nullptr;
    const int nr = prm->n_r, nt = prm->n_t;
    if (nr < 1 || nt < 64 || (nt & (nt - 1))) return fail(nullptr, GS_ERR_UNSUPPORTED, "n_t must be a power of two >= 64, n_r >= 1");
    if (prm->precision != GS_PREC_FP64 && prm->precision != GS_PREC_MIXED) return fail(nullptr, GS_ERR_ARG, "precision");
    if (prm->gas && (prm->ion_levels < 0 || prm->ion_levels > GS_MAX_ION_LEVELS))
        return fail(nullptr, GS_ERR_ARG, "ion_levels out of range (0..8)");
    if (prm->gas && prm->th_coeff != 0 && prm->n2 != 0 && prm->raman_fraction > 0.001 &&
        !(prm->raman_tau > 0 && prm->raman_omega > 0))
        return fail(nullptr, GS_ERR_UNSUPPORTED,
                    "gas build: the third harmonic with Raman needs the Raman oscillator parameters");
    gs_handle* h = new gs_handle();
    h->p = *prm;
    {
        const char* ex = std::getenv("GS_TEST_SHOOTING_EXHAUST");
        h->shoot_exhaust = (ex && ex[0] == '1') ? 1 : 0;
    }
    h->nr = nr;
    h->nt = nt;
    h->fp64 = prm->precision == GS_PREC_FP64;
    h->esz = h->fp64 ? 16 : 8;
    const int mmax = h->fp64 ? 8192 : 16384;   // one row of M complex in <= 128 KiB shared memory
    h->M = nt <= mmax ? nt : mmax;
    h->P = nt / h->M;
    if (h->P > 8) { delete h; return fail(nullptr, GS_ERR_UNSUPPORTED, "n_t too large"); }
    h->logM = ilog2(h->M);
    cudaError_t e = cudaSetDevice(prm->device);
    if (e != cudaSuccess) { delete h; return fail(nullptr, GS_ERR_CUDA, cudaGetErrorString(e)); }
    auto al = [&](void** q, size_t n) -> bool { return cudaMalloc(q, n) == cudaSuccess; };
    const size_t nel = (size_t)nr * nt;
    bool ok = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreate(&h->ev0) == cudaSuccess && cudaEventCreate(&h->ev1) == cudaSuccess;
    ok = ok && al(&h->A, nel * h->esz) && al(&h->S, nel * h->esz) && al(&h->NB, nel * h->esz) &&
         al(&h->KP, nel * h->esz) && al(&h->E, nel * h->esz) && al(&h->U, 3 * nel * h->esz) &&
         al(&h->tw, (size_t)nt * h->esz) && al(&h->pf, (size_t)nt * h->esz) && al(&h->rm, (size_t)nt * h->esz) &&
         al(&h->kerr, (size_t)nt * h->esz / 2) && al(&h->rate, 8192 * (size_t)ion_levels(h) * h->esz / 2) &&
         al((void**)&h->omega, nt * 8) && al((void**)&h->ho, nt * 8) && al((void**)&h->kt2, nr * 8) &&
         al((void**)&h->Cm, (size_t)nr * nr * 8) && al((void**)&h->m1, nr * 8) &&
         al((void**)&h->wavenum, nt * 16) && al((void**)&h->staging, nel * 16) &&
         al((void**)&h->perm_dev, nt * 4) && al((void**)&h->iperm_dev, nt * 4) && al((void**)&h->err_dev, 4) &&
         al((void**)&h->max_dev, 16) &&
         al((void**)&h->row_ion, (size_t)nr * 4);
    if (!ok) {
        cudaGetLastError();
        free_all(h);
        delete h;
        return fail(nullptr, GS_ERR_NOMEM, "device allocation failed");
    }
    h->perm = fft_position_map(nt, h->P, h->M, h->logM);
    e = cudaMemcpy(h->perm_dev, h->perm.data(), nt * 4, cudaMemcpyHostToDevice);
    {
        std::vector<int> ip(nt);
        for (int p = 0; p < nt; p++) ip[h->perm[p]] = p;
        if (e == cudaSuccess) e = cudaMemcpy(h->iperm_dev, ip.data(), nt * 4, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->p.device);
    }
    // twiddles exp(-2 pi i j / N)
    std::vector<double> tw(2 * (size_t)nt);
    for (int j = 0; j < nt; j++) {
        const double a = 2.0 * M_PI * (double)j / (double)nt;
        tw[2 * j] = std::cos(a);
        tw[2 * j + 1] = -std::sin(a);
    }
    if (e == cudaSuccess) {
        if (h->fp64) {
            e = cudaMemcpy(h->tw, tw.data(), nt * 16, cudaMemcpyHostToDevice);
        } else {
            std::vector<float> twf(tw.begin(), tw.end());
            e = cudaMemcpy(h->tw, twf.data(), nt * 8, cudaMemcpyHostToDevice);
        }
    }
    // base twiddles of the radix-16 stages: w_N^{q m scale_j}, m = 1, 2, 3, 4, 8, 12
    if (e == cudaSuccess) {
        const int nb = tw_base_count(h->logM);
        std::vector<double> b(2 * (size_t)nb);
        const int mult[6] = {1, 2, 3, 4, 8, 12};
        for (int j = 0; j < h->logM / 4; j++) {
            const int S = h->M >> (4 * j), sub = S / 16;
            const long long scale = (long long)(h->M / S) * h->P;
            const int off = tw_base_offset(h->logM, j);
            for (int k = 0; k < 6; k++)
                for (int q = 0; q < sub; q++) {
                    const long long ex = ((long long)q * mult[k] * scale) % nt;
                    const double a = 2.0 * M_PI * (double)ex / (double)nt;
                    b[2 * ((size_t)off + (size_t)k * sub + q)] = std::cos(a);
                    b[2 * ((size_t)off + (size_t)k * sub + q) + 1] = -std::sin(a);
                }
        }
        e = cudaMalloc(&h->twb, (size_t)(nb > 0 ? nb : 1) * h->esz);
        if (e == cudaSuccess && nb > 0) {
            if (h->fp64) {
                e = cudaMemcpy(h->twb, b.data(), (size_t)nb * 16, cudaMemcpyHostToDevice);
            } else {
                std::vector<float> bf(b.begin(), b.end());
                e = cudaMemcpy(h->twb, bf.data(), (size_t)nb * 8, cudaMemcpyHostToDevice);
            }
        }
    }
    if (e == cudaSuccess) e = h->fp64 ? fft_set_smem<double>(h->M, nt) : fft_set_smem<float>(h->M, nt);
    h->fused = h->P == 1 && (h->fp64 ? nl_fused_supported<double>(nt) : nl_fused_supported<float>(nt));
    if (e == cudaSuccess && h->fused) e = h->fp64 ? nl_fused_setup<double>(nt) : nl_fused_setup<float>(nt);
    h->pair = !h->fused && h->P == 2 && (h->fp64 ? nl_pair_supported<double>(nt) : nl_pair_supported<float>(nt));
    if (e == cudaSuccess && h->pair) e = h->fp64 ? nl_pair_setup<double>(nt) : nl_pair_setup<float>(nt);
    if (e == cudaSuccess) {
        double k[20], b = 1.0;
        for (int n = 1; n <= 20; n++) { b *= (0.5 - (n - 1)) / n; k[n - 1] = b; }
        e = qdht_set_sqrt_ho(k);
    }
    if (e != cudaSuccess) {
        std::string m = cudaGetErrorString(e);
        free_all(h);
        delete h;
        return fail(nullptr, GS_ERR_CUDA, m);
    }
    if (!h->fp64) {
        std::string m;
        h->tc = gs::qdht_tc_create(nr, nt, h->st, &m);
        if (!h->tc) {
            free_all(h);
            delete h;
            return fail(nullptr, GS_ERR_UNSUPPORTED, "mixed QDHT: " + m);
        }
    }
    *out = h;
    return GS_OK;
}

int gs_destroy(gs_handle* h) {
    if (!h) return GS_OK;
    cudaSetDevice(h->p.device);
    cudaStreamSynchronize(h->st);
    free_all(h);
    delete h;
    return GS_OK;
}

template <typename T>
static std::vector<T> permuted(const double* src, const std::vector<int>& perm, int comps) {
    std::vector<T> o(perm.size() * comps);
    for (size_t p = 0; p < perm.size(); p++)
        for (int c = 0; c < comps; c++) o[p * comps + c] = (T)src[(size_t)perm[p] * comps + c];
    return o;
}

int gs_upload_tables(gs_handle* h, const gs_tables* t) {
    if (!h || !t) return fail(h, GS_ERR_ARG, "null argument");
    if (!t->rate_ln || !t->plasma_func || !t->raman_func || !t->kerr || !t->omega || !t->wavenum ||
        !t->ho_disp || !t->kt2 || !t->qdht_c || !t->qdht_m1)
        return fail(h, GS_ERR_ARG, "missing table");
    CK(h, cudaSetDevice(h->p.device));
    const int nt = h->nt, nr = h->nr;
    auto up = [&](void* dst, const void* src, size_t n) { return cudaMemcpy(dst, src, n, cudaMemcpyHostToDevice); };
    if (h->fp64) {
        auto pf = permuted<double>(t->plasma_func, h->perm, 2);
        auto rm = permuted<double>(t->raman_func, h->perm, 2);
        auto ke = permuted<double>(t->kerr, h->perm, 1);
        CK(h, up(h->pf, pf.data(), nt * 16));
        CK(h, up(h->rm, rm.data(), nt * 16));
        CK(h, up(h->kerr, ke.data(), nt * 8));
        CK(h, up(h->rate, t->rate_ln, 8192 * (size_t)ion_levels(h) * 8));
    } else {
        auto pf = permuted<float>(t->plasma_func, h->perm, 2);
        auto rm = permuted<float>(t->raman_func, h->perm, 2);
        auto ke = permuted<float>(t->kerr, h->perm, 1);
        std::vector<float> rate(t->rate_ln, t->rate_ln + 8192 * (size_t)ion_levels(h));
        CK(h, up(h->pf, pf.data(), nt * 8));
        CK(h, up(h->rm, rm.data(), nt * 8));
        CK(h, up(h->kerr, ke.data(), nt * 4));
        CK(h, up(h->rate, rate.data(), rate.size() * 4));
    }
    auto om = permuted<double>(t->omega, h->perm, 1);
    auto wn = permuted<double>(t->wavenum, h->perm, 2);
    auto ho = permuted<double>(t->ho_disp, h->perm, 1);
    CK(h, up(h->omega, om.data(), nt * 8));
    CK(h, up(h->wavenum, wn.data(), nt * 16));
    CK(h, up(h->ho, ho.data(), nt * 8));
    CK(h, up(h->kt2, t->kt2, nr * 8));
    CK(h, up(h->Cm, t->qdht_c, (size_t)nr * nr * 8));
    CK(h, up(h->m1, t->qdht_m1, nr * 8));
    {
        // the transposed QDHT of the adjoint: H^T = diag(1/m1) C diag(m1) (C symmetric)
        std::vector<double> inv(nr);
        for (int i = 0; i < nr; i++) inv[i] = 1.0 / t->qdht_m1[i];
        if (!h->m1inv) CK(h, cudaMalloc((void**)&h->m1inv, nr * 8));
        CK(h, up(h->m1inv, inv.data(), nr * 8));
        if (!h->fp64) {
            h->c_host.assign(t->qdht_c, t->qdht_c + (size_t)nr * nr);
            h->m1inv_host = inv;
            if (h->tcT) {   // tables replaced: rebuild on the next adjoint call
                gs::qdht_tc_destroy(h->tcT);
                h->tcT = nullptr;
            }
        }
    }
    if (h->fp64) {
        // calculate_Lstep's window per position (omega in [min, max], some kt^2 <= Re(k^2) / 4):
        // the FP64 linear-step and masked transforms take these columns only
        std::vector<int> cm, zp;
        double kt2min = t->kt2[0];
        for (int k = 1; k < nr; k++) kt2min = std::min(kt2min, t->kt2[k]);
        for (int p = 0; p < nt; p++) {
            const double w = om[p], kr = wn[2 * p], ki = wn[2 * p + 1];
            const bool in = !(w < h->p.omega_min || w > h->p.omega_max) && !(kt2min > 0.25 * (kr * kr - ki * ki));
            if (in) {
                cm.push_back(2 * p);
                cm.push_back(2 * p + 1);
            } else {
                zp.push_back(p);
            }
        }
        while (cm.size() % 64) cm.push_back(-1);
        if (h->win64) cudaFree(h->win64);
        if (h->zpos64) cudaFree(h->zpos64);
        h->win64 = h->zpos64 = nullptr;
        h->nwin64 = (int)cm.size();
        h->nz64 = (int)zp.size();
        if (!cm.empty()) {
            CK(h, cudaMalloc((void**)&h->win64, cm.size() * 4));
            CK(h, up(h->win64, cm.data(), cm.size() * 4));
        }
        if (!zp.empty()) {
            CK(h, cudaMalloc((void**)&h->zpos64, zp.size() * 4));
            CK(h, up(h->zpos64, zp.data(), zp.size() * 4));
        }
        if (cm.empty()) {   // no column in the window: keep one padding tile so the list is non-null
            std::vector<int> pad(64, -1);
            CK(h, cudaMalloc((void**)&h->win64, 64 * 4));
            CK(h, up(h->win64, pad.data(), 64 * 4));
            h->nwin64 = 64;
        }
    }
    if (h->tc) {
        std::string m;
        // the plan's compact copies are rebuilt: FIELD (left compact by the masked inverse) and
        // BIGBUFFER2 take their window columns back first, through the old column lists
        {
            const int rc = gsi::field_sync(h);
            if (rc) return rc;
        }
        // BIGBUFFER2's double-float window columns are kept across the rebuild in FP64 (staging,
        // natural order) and split again over the new column list
        const bool keep_spec = h->s_compact;
        if (keep_spec) {
            const int rc = gsi::spec_sync(h);
            if (rc) return rc;
            const size_t nel = (size_t)nr * nt;
            CK(h, launch_permute<float>(-1, h->S, h->staging, h->perm_dev, nt, nel, h->st, &h->launches));
            CK(h, gs::qdht_tc_spec_ff(h->tc, (double*)h->staging, h->perm_dev, 0, &h->launches));
            CK(h, cudaStreamSynchronize(h->st));
            gsi::spec_written(h);
        }
        if (gs::qdht_tc_set_matrix(h->tc, t->qdht_c, t->qdht_m1, &m)) return fail(h, GS_ERR_CUDA, "mixed QDHT matrix: " + m);
        if (gs::qdht_tc_set_lstep(h->tc, om.data(), wn.data(), ho.data(), t->kt2, h->p.omega_min, h->p.omega_max, &m))
            return fail(h, GS_ERR_CUDA, "mixed QDHT: " + m);
        if (keep_spec && gs::qdht_tc_has_compact(h->tc)) {
            CK(h, gs::qdht_tc_spec_ff(h->tc, (double*)h->staging, h->perm_dev, 1, &h->launches));
            CK(h, cudaStreamSynchronize(h->st));
            h->s_compact = true;
        }
    }
    if (h->p.gas && h->p.th_coeff != 0) {
        // third harmonic (propagator.cu:712-720): th_coeff exp(j phi_t), phi_t =
        // -2 OMEGA0 (TMIN + t (TMIN - TMAX)/N_T) (the reference's sign of the step; its
        // OMEGA0 == OMEGA[0] holds on this grid), natural time order, FP64 then stored
        std::vector<double> th(2 * (size_t)nt);
        for (int t = 0; t < nt; t++) {
            const double ph = -2.0 * h->p.omega0 * (h->p.tmin + t * (h->p.tmin - h->p.tmax) / nt);
            th[2 * t] = h->p.th_coeff * std::cos(ph);
            th[2 * t + 1] = h->p.th_coeff * std::sin(ph);
        }
        if (!h->th) CK(h, cudaMalloc(&h->th, (size_t)nt * h->esz));
        if (h->fp64) {
            CK(h, up(h->th, th.data(), nt * 16));
        } else {
            std::vector<float> thf(th.begin(), th.end());
            CK(h, up(h->th, thf.data(), nt * 8));
        }
    }
    h->tables_ok = true;
    return GS_OK;
}

static LstepArgs lstep_args(gs_handle* h, double dz) {
    LstepArgs L{};
    L.dz = dz;
    if (h->ctl) {   // gs_advance: the accepted attempt's size, and no work for a rejected one
        L.dz_dev = &h->ctl->dz_lin;
        L.run = &h->ctl->accept;
    }
    L.omega = h->omega;
    L.wavenum = h->wavenum;
    L.ho = h->ho;
    L.kt2 = h->kt2;
    L.omega_min = h->p.omega_min;
    L.omega_max = h->p.omega_max;
    return L;
}

// QDHT of device array X -> Y (mode: plain / fused linear step / masked input).
int gsi::run_qdht(gs_handle* h, int mode, const void* X, void* Y, double dz, int flags) {
    if (Y == h->S && mode == QDHT_PLAIN) spec_written(h);
    if (X == h->A) {
        const int rs = field_sync(h);
        if (rs) return rs;
    }
    if (Y == h->A) field_written(h);
    // the masked inverse leaves FIELD compact only on plans that keep a compact result
    int nyc = 0;
    const bool lazy = (flags & gs::QTC_Y_LAZY) && mode == QDHT_MASKED && Y == h->A && !h->fp64 && h->tc &&
                      gs::qdht_tc_compact_y(h->tc, &nyc) && nyc > 0;
    if (!lazy) flags &= ~gs::QTC_Y_LAZY;
    LstepArgs L = lstep_args(h, dz);
    if (h->fp64) {
        const bool win = mode != QDHT_PLAIN && h->win64;
        CK(h, launch_qdht64(mode, h->Cm, h->m1, (const double*)X, (double*)Y, h->nr, 2 * h->nt, L, h->st, &h->launches,
                            win ? h->win64 : nullptr, h->nwin64, h->zpos64, h->nz64));
    } else {
        std::string m;
        cudaError_t e = gs::qdht_tc_run(h->tc, mode, (const float*)X, (float*)Y, L, &h->launches, &m, flags);
        if (e != cudaSuccess) return fail(h, GS_ERR_CUDA, "mixed QDHT: " + m + " " + cudaGetErrorString(e));
        if (lazy) h->a_compact = true;   // A itself is not written
    }
    return GS_OK;
}

int gs_nl_timing(gs_handle* h, int enable, double* ms, int* stages, int* launches) {
    if (!h) return GS_ERR_ARG;
    if (ms) *ms = h->nl_ms;
    if (stages) *stages = h->nl_stages_timed;
    if (launches) *launches = h->nl_launches_timed;
    h->nl_launches_timed = 0;
    h->nl_ms = 0;
    h->nl_stages_timed = 0;
    h->nl_ev_pending = false;
    if (enable && !h->nl_ev[0]) {
        CK(h, cudaSetDevice(h->p.device));
        for (cudaEvent_t& e : h->nl_ev) CK(h, cudaEventCreate(&e));
    }
    h->time_nl = enable != 0;
    return GS_OK;
}

int gs_qdht_timing(gs_handle* h, int enable, double* ms_total, int* launches) {
    if (!h) return GS_ERR_ARG;
    if (ms_total) *ms_total = h->qdht_ms;
    if (launches) *launches = h->qdht_n;
    h->qdht_ms = 0;
    h->qdht_n = 0;
    h->time_qdht = enable != 0;
    h->ev_pending = false;
    return GS_OK;
}

// fold the CUDA-event time of the last fused QDHT pair into the totals (stream is idle);
// also surfaces an expired wait recorded by the tensor-core kernel
static int collect_qdht_time(gs_handle* h) {
    if (h->tc) {
        std::string m;
        if (gs::qdht_tc_check(h->tc, &m)) return fail(h, GS_ERR_CUDA, m);
    }
    if (!h->ev_pending) return GS_OK;
    float ms = 0;
    CK(h, cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    h->qdht_ms += ms;
    h->qdht_n += 2;
    h->ev_pending = false;
    return GS_OK;
}

// The device address of a pinned host buffer when all of [host, host + bytes) lies in one
// pinned allocation (the driver's record of it), 16-byte aligned; else null (the copy then
// goes through the staging buffer).
static void* pinned_device_ptr(const void* host, size_t bytes) {
    if (((uintptr_t)host & 15) != 0) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
    // the driver's cuPointerGetAttribute, looked up at run time (the library links no driver symbol)
    using GetAttr = CUresult (*)(void*, CUpointer_attribute, CUdeviceptr);
    static GetAttr get_attr = [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &fn, 4000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            fn = nullptr;
        return (GetAttr)fn;
    }();
    if (!get_attr) return nullptr;
    CUdeviceptr start = 0;
    size_t size = 0;
    const CUdeviceptr d = (CUdeviceptr)(uintptr_t)at.devicePointer;
    if (get_attr(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, d) != CUDA_SUCCESS ||
        get_attr(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, d) != CUDA_SUCCESS)
        return nullptr;
    if (d < start || d - start > size || size - (d - start) < bytes) return nullptr;
    return at.devicePointer;
}

int gsi::permute_in(gs_handle* h, const double* host, void* dst) {
    const size_t nel = (size_t)h->nr * h->nt;
    if (const int rc = spec_in_finish(h)) return rc;   // the staging buffer is free again
    if (dst == h->S) spec_written(h);
    if (dst == h->A) field_written(h);
    // mixed plans keep BIGBUFFER2's window columns as a double-float pair: an FP64 spectrum
    // given here is split into its high and low parts there, so that a state read back by
    // gs_get_field and set again continues exactly
    const bool spec_ff = dst == h->S && !h->fp64 && h->tc && gs::qdht_tc_has_compact(h->tc);
    if (void* dp = pinned_device_ptr(host, nel * 16)) {   // read over the host link, no staging copy
        // (the low parts go to the free staging buffer, in position order, on the same pass)
        cudaError_t e = h->fp64 ? launch_permute_host<double>(+1, dp, dst, h->iperm_dev, h->nt, nel, h->sms, h->st, &h->launches)
                                : launch_permute_host<float>(+1, dp, dst, h->iperm_dev, h->nt, nel, h->sms, h->st, &h->launches,
                                                             spec_ff ? h->staging : nullptr);
        CK(h, e);
        if (spec_ff) {
            CK(h, gs::qdht_tc_spec_dev(h->tc, (float*)h->S, (float*)h->staging, 1, &h->launches));
            h->s_compact = true;
        }
        return GS_OK;
    }
    CK(h, cudaMemcpyAsync(h->staging, host, nel * 16, cudaMemcpyHostToDevice, h->st));
    cudaError_t e = h->fp64 ? launch_permute<double>(+1, h->staging, dst, h->perm_dev, h->nt, nel, h->st, &h->launches)
                            : launch_permute<float>(+1, h->staging, dst, h->perm_dev, h->nt, nel, h->st, &h->launches);
    CK(h, e);
    if (spec_ff) {
        CK(h, gs::qdht_tc_spec_ff(h->tc, (double*)h->staging, h->perm_dev, 1, &h->launches));
        h->s_compact = true;
    }
    return GS_OK;
}
int gsi::permute_out(gs_handle* h, const void* src, double* host) {
    const size_t nel = (size_t)h->nr * h->nt;
    if (const int rc = spec_in_finish(h)) return rc;
    if (src == h->S) {
        const int rc = spec_sync(h);
        if (rc) return rc;
    }
    if (src == h->A) {
        const int rc = field_sync(h);
        if (rc) return rc;
    }
    // BIGBUFFER2's window columns leave as their double-float value (high + low parts)
    const bool spec_ff = src == h->S && h->s_compact && !h->fp64;
    if (void* dp = pinned_device_ptr(host, nel * 16)) {   // written over the host link
        // (the compact low parts scattered into the free staging buffer first, then added on the pass)
        if (spec_ff) CK(h, gs::qdht_tc_spec_dev(h->tc, nullptr, (float*)h->staging, 0, &h->launches));
        cudaError_t e = h->fp64 ? launch_permute_host<double>(-1, src, dp, h->iperm_dev, h->nt, nel, h->sms, h->st, &h->launches)
                                : launch_permute_host<float>(-1, src, dp, h->iperm_dev, h->nt, nel, h->sms, h->st, &h->launches,
                                                             spec_ff ? h->staging : nullptr);
        CK(h, e);
        CK(h, cudaStreamSynchronize(h->st));
        return GS_OK;
    }
    cudaError_t e = h->fp64 ? launch_permute<double>(-1, src, h->staging, h->perm_dev, h->nt, nel, h->st, &h->launches)
                            : launch_permute<float>(-1, src, h->staging, h->perm_dev, h->nt, nel, h->st, &h->launches);
    CK(h, e);
    if (spec_ff) CK(h, gs::qdht_tc_spec_ff(h->tc, (double*)h->staging, h->perm_dev, 0, &h->launches));
    CK(h, cudaMemcpyAsync(host, h->staging, nel * 16, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    return GS_OK;
}

int gs_set_field(gs_handle* h, const double* field, const double* spec) {
    if (!h || !field) return fail(h, GS_ERR_ARG, "null argument");
    if (!h->tables_ok) return fail(h, GS_ERR_STATE, "tables not uploaded");
    CK(h, cudaSetDevice(h->p.device));
    int rc = permute_in(h, field, h->A);
    if (rc) return rc;
    if (spec) {
        rc = permute_in(h, spec, h->S);
    } else {
        rc = run_qdht(h, QDHT_PLAIN, h->A, h->S, 0.0);
    }
    if (rc) return rc;
    CK(h, cudaStreamSynchronize(h->st));
    h->field_ok = true;
    h->en_prev = 0;
    return GS_OK;
}

int gs_get_field(gs_handle* h, double* field, double* spec) {
    if (!h) return GS_ERR_ARG;
    if (!h->field_ok) return fail(h, GS_ERR_STATE, "field not set");
    CK(h, cudaSetDevice(h->p.device));
    int rc = GS_OK;
    if (field) rc = permute_out(h, h->A, field);
    if (!rc && spec) rc = permute_out(h, h->S, spec);
    return rc;
}

int gs_get_nl(gs_handle* h, double* bb1) {
    if (!h || !bb1) return GS_ERR_ARG;
    if (!h->nb_full_current) return fail(h, GS_ERR_STATE, "BIGBUFFER1 is kept in full by gs_nl_step only");
    CK(h, cudaSetDevice(h->p.device));
    return permute_out(h, h->NB, bb1);
}

template <typename Rl>
PlasmaArgs<Rl> gsi::plasma_args(gs_handle* h, bool raman, bool raman_scan) {
    using T2 = typename Vec2<Rl>::T;
    const size_t nel = (size_t)h->nr * h->nt;
    T2* U1 = (T2*)h->U;
    PlasmaArgs<Rl> pa{};
    pa.N = h->nt; pa.e = (const T2*)h->E; pa.u1 = U1; pa.u2 = U1 + nel; pa.u3 = U1 + 2 * nel;
    pa.rate = (const Rl*)h->rate; pa.err = h->err_dev; pa.raman = raman;
    pa.tstep_scaled = h->p.tstep * h->p.ionrate_denom;
    pa.neutral_density = h->p.neutral_density; pa.rho0 = h->p.rho0;
    pa.ionization_potential = h->p.ionization_potential; pa.ponderomotive = h->p.ponderomotive;
    pa.avalanche_cs = h->p.avalanche_cs; pa.recombination_tau = h->p.recombination_tau;
    pa.raman_scan = raman_scan;
    pa.shoot_exhaust = h->shoot_exhaust;
    pa.gas = h->p.gas;
    pa.levels = ion_levels(h);
    for (int n = 0; n < pa.levels && pa.levels > 1; n++) pa.pot[n] = h->p.ion_potentials[n];
    pa.th = (h->p.gas && h->p.th_coeff != 0) ? (const T2*)h->th : nullptr;
    if (raman_scan) {
        const double dt = h->p.tstep, tau = h->p.raman_tau, om = h->p.raman_omega;
        const double M = dt * (1 + om * om * tau * tau) / tau / (om * tau);   // solver_main.cpp:403
        pa.fRM = h->p.raman_fraction * M;
        pa.one_minus_fR = 1 - h->p.raman_fraction;
        pa.dt_over_tau = dt / tau;
        pa.dt_omega = dt * om;
        const double m1 = std::exp(-dt / tau), mN = std::exp(-(double)h->nt * dt / tau);
        pa.a_re = m1 * std::cos(om * dt);
        pa.a_im = m1 * std::sin(om * dt);
        pa.aN_re = mN * std::cos(om * dt * h->nt);
        pa.aN_im = mN * std::sin(om * dt * h->nt);
    }
    plasma_consts<Rl>(pa);
    return pa;
}

template gs::PlasmaArgs<double> gsi::plasma_args<double>(gs_handle*, bool, bool);
template gs::PlasmaArgs<float> gsi::plasma_args<float>(gs_handle*, bool, bool);

bool gsi::nl_takes_device_dz(const gs_handle* h) {
    const bool raman = h->p.raman_fraction > 0.001, kerr_on = h->p.n2 != 0;
    const bool ok_raman = raman_scan_on(h) || !raman || !kerr_on;
    return h->p.nonlinear && !h->fp64 && ion_levels(h) == 1 && ok_raman && (h->fused || h->pair);
}

bool gsi::raman_scan_on(const gs_handle* h) {
    return h->p.raman_fraction > 0.001 && h->p.n2 != 0 && h->p.raman_tau > 0 && h->p.raman_omega > 0;
}

template <typename Rl>
static int nl_step_impl(gs_handle* h, double dz, const GsTape* tape = nullptr) {
    using T2 = typename Vec2<Rl>::T;
    const int nr = h->nr, nt = h->nt;
    const size_t nel = (size_t)nr * nt;
    T2* A = (T2*)h->A;
    T2* NB = (T2*)h->NB;
    T2* KP = (T2*)h->KP;
    T2* E = (T2*)h->E;
    T2* U1 = (T2*)h->U;
    T2* U2 = U1 + nel;
    T2* U3 = U2 + nel;
    h->nbc_valid = false;   // set again below when the fused stages also write NB's compact columns
    h->nb_full_current = true;   // cleared below where the row kernel leaves the full array out
    const bool raman = h->p.raman_fraction > 0.001;
    const bool kerr_on = h->p.n2 != 0;
    // the oscillator recurrence replaces the RAMAN_FUNCTION FFT pair when its parameters are known
    const bool raman_scan = raman && kerr_on && h->p.raman_tau > 0 && h->p.raman_omega > 0;
    // without Kerr the Raman response is never used: the fused stage applies.  Several
    // ionization levels take the staged kernels (plasma_kernel's level-by-level recurrence)
    const bool multi = ion_levels(h) > 1;
    const bool fused = h->fused && (raman_scan || !raman || !kerr_on) && !multi;
    {
        // the four-stage kernel of 16384-point FP32 rows reads FIELD compactly where the masked
        // inverse left it so; every other path reads A
        if (fused && h->all_stages_thr != h->nl_threads) {   // decided once per launch shape
            h->all_stages = nl_stage_all_preferred<Rl>(nt, h->nl_threads, nr) ? 1 : 0;
            h->all_stages_thr = h->nl_threads;
        }
        int nyc = 0;
        h->nl_compact = h->p.nonlinear && fused && !h->pair && h->all_stages == 1 && !h->fp64 && h->tc &&
                        nl_stage_reads_compact<Rl>(nt, h->nl_threads) && gs::qdht_tc_compact_y(h->tc, &nyc) &&
                        gs::qdht_tc_compact_x(h->tc, nullptr, nullptr) && nyc > 0;
        if (!h->nl_compact) {
            const int rs = gsi::field_sync(h);
            if (rs) return rs;
        }
        // the fused stage kernels and the paired ones take dz and the stop flag from the device
        const bool pair_path = h->pair && !multi && (raman_scan || !raman || !kerr_on);
        h->nl_dev_dz = h->p.nonlinear && (fused || pair_path) && !tape && !h->fp64;
    }
    if (!h->p.nonlinear) {
        CK(h, launch_zero_nl<Rl>(A, NB, nel, h->max_dev, h->st, &h->launches));
        return GS_OK;
    }
    FftArgs<Rl> fa{};
    fa.N = nt; fa.M = h->M; fa.P = h->P; fa.logM = h->logM;
    fa.tw = (const T2*)h->tw;
    fa.twb = (const T2*)h->twb;
    fa.max_out = h->max_dev;
    fa.threads = h->nl_threads;
    if (h->ctl) {   // gs_advance: the attempt's size and the stop flag from the device
        fa.dz_dev = &h->ctl->zstep;
        fa.halt = &h->ctl->stop;
        fa.ac_on = &h->ctl->field_compact;
    }
    PlasmaArgs<Rl> pa = plasma_args<Rl>(h, raman, raman_scan);
    SpecArgs<Rl> sa{};
    sa.N = nt; sa.rows = nr; sa.u1 = U1; sa.u2 = U2; sa.u3 = U3;
    sa.pf = (const T2*)h->pf; sa.rm = (const T2*)h->rm; sa.kerr = (const Rl*)h->kerr;
    sa.raman = raman && !raman_scan; sa.kerr_on = kerr_on; sa.nb = NB; sa.kp = KP; sa.max_out = h->max_dev + 1;
    if (tape && !fused) return fail(h, GS_ERR_UNSUPPORTED, "recording the RK4 stages needs rows that fit one CTA");
    if (h->pair && !tape && !multi && (raman_scan || !raman || !kerr_on)) {   // rows over two CTAs (gs_nl_pair.cu)
        pa.row_ion = h->row_ion;
        sa.row_ion = h->row_ion;
        for (int s = 0; s < 4; s++) {
            FftArgs<Rl> f1 = fa;
            f1.rows = nr; f1.kp = KP;
            f1.cdz = (Rl)((s == 0) ? 0.0 : (s < 3 ? dz * 0.5 : dz));
            f1.c_stage = (s == 0) ? 0.0 : (s < 3 ? 0.5 : 1.0);
            f1.track_max = (s == 0);
            CK(h, launch_nl_pair_front<Rl>(f1, pa, A, nr, h->st, &h->launches));
            SpecArgs<Rl> s2 = sa;
            s2.stage = s;
            CK(h, launch_nl_pair_back<Rl>(fa, s2, nr, h->st, &h->launches));
        }
        return GS_OK;
    }
    if (fused) {
        pa.row_ion = h->row_ion;   // the row flags of the last stage (the adjoint keeps its own)
        // k of stages 0, 1, 2 in KP, E (free on this path) and NB; stage 3 reads all three and
        // writes the RK4 sum over NB row by row, and (mixed) its window columns compactly for
        // the linear-step transform
        T2* kst[3] = {KP, E, NB};
        const int* cinv = nullptr;
        int ncw = 0;
        float* nbc = (!h->fp64 && h->tc) ? gs::qdht_tc_compact_x(h->tc, &cinv, &ncw) : nullptr;
        if (h->all_stages == 1) {   // the four stages of each row in one launch
            FftArgs<Rl> f1 = fa;
            f1.rows = nr; f1.kp = KP;
            f1.all_stages = 1;
            f1.dzs = dz;
            PlasmaArgs<Rl> ps = pa;
            if (tape) {   // stage s's record at a constant stride from stage 0's
                ps.tape_e = (T2*)tape->e[0];
                ps.tape_rho = (Rl*)tape->rho[0];
                ps.tape_q = (Rl*)tape->q[0];
                ps.row_ion = tape->ion[0];
                ps.tape_stride = (size_t)((char*)tape->e[1] - (char*)tape->e[0]);
            }
            SpecArgs<Rl> s2 = sa;
            s2.stage = 0;
            for (int j = 0; j < 3; j++) s2.kst[j] = kst[j];
            s2.nbc = nbc;
            s2.cinv = cinv;
            s2.ncw = ncw;
            // the row kernel leaves out the full BIGBUFFER1 where only its window columns are read
            if (nbc && !h->nb_full_wanted && !tape && nl_row16k_applies(nt, h->nl_threads)) s2.nb = nullptr;
            h->nb_full_current = s2.nb != nullptr;
            // nl_compact holds; under gs_advance the device flag ac_on tells whether it is current
            if (h->a_compact || (h->ctl && h->nl_compact)) s2.ac = gs::qdht_tc_compact_y(h->tc, nullptr, &s2.cmap);
            const bool tm = h->time_nl && !tape;
            if (tm) CK(h, cudaEventRecord(h->nl_ev[0], h->st));
            CK(h, launch_nl_stage<Rl>(f1, ps, A, s2, nr, h->st, &h->launches));
            if (tm) {
                CK(h, cudaEventRecord(h->nl_ev[1], h->st));
                h->nl_ev_pending = true;
                h->nl_ev_one = true;
            }
            h->nbc_valid = nbc != nullptr;
            return GS_OK;
        }
        for (int s = 0; s < 4; s++) {
            FftArgs<Rl> f1 = fa;
            f1.rows = nr; f1.kp = s > 0 ? kst[s - 1] : KP;
            f1.cdz = (s == 0) ? 0.0 : (s < 3 ? dz * 0.5 : dz);
            f1.track_max = (s == 0);
            PlasmaArgs<Rl> ps = pa;
            if (tape) {
                ps.tape_e = (T2*)tape->e[s];
                ps.tape_rho = (Rl*)tape->rho[s];
                ps.tape_q = (Rl*)tape->q[s];
                ps.row_ion = tape->ion[s];   // the stage's row flags are kept for the adjoint
            }
            const bool tm = h->time_nl && !tape;
            SpecArgs<Rl> s2 = sa;
            s2.stage = s;
            for (int j = 0; j < 3; j++) s2.kst[j] = kst[j];
            s2.nbc = nbc;
            s2.cinv = cinv;
            s2.ncw = ncw;
            if (tm) CK(h, cudaEventRecord(h->nl_ev[2 * s], h->st));
            CK(h, launch_nl_stage<Rl>(f1, ps, A, s2, nr, h->st, &h->launches));
            if (tm) CK(h, cudaEventRecord(h->nl_ev[2 * s + 1], h->st));
        }
        if (h->time_nl && !tape) h->nl_ev_pending = true;
        h->nbc_valid = nbc != nullptr;
        return GS_OK;
    }
    for (int s = 0; s < 4; s++) {
        // stage input A + c*dz*k_prev, E = IFFT(.)/N   (propagator.cu:386-396, 640-641)
        FftArgs<Rl> f1 = fa;
        f1.rows = nr; f1.spre = 1; f1.kp = KP;
        f1.cdz = (s == 0) ? 0.0 : (s < 3 ? dz * 0.5 : dz);
        f1.track_max = (s == 0); f1.tpost = 1;
        CK(h, launch_fft<Rl>(+1, A, E, f1, h->st, &h->launches));
        CK(h, launch_plasma<Rl>(pa, nr, h->st, &h->launches));
        FftArgs<Rl> f2 = fa;
        f2.rows = (kerr_on ? 3 : 2) * nr;
        CK(h, launch_fft<Rl>(-1, U1, U1, f2, h->st, &h->launches));
        const bool fft_raman = kerr_on && raman && !raman_scan;
        if (fft_raman) CK(h, launch_spec1<Rl>(sa, h->st, &h->launches));
        if (fft_raman) {
            FftArgs<Rl> f3 = fa;
            f3.rows = nr; f3.tpost = 2; f3.e = E;
            CK(h, launch_fft<Rl>(+1, U3, U3, f3, h->st, &h->launches));
            FftArgs<Rl> f4 = fa;
            f4.rows = nr;
            CK(h, launch_fft<Rl>(-1, U3, U3, f4, h->st, &h->launches));
        }
        SpecArgs<Rl> s2 = sa;
        s2.stage = s;
        s2.fuse_plasma = !fft_raman;
        CK(h, launch_spec2<Rl>(s2, h->st, &h->launches));
    }
    return GS_OK;
}

int gsi::nl_stages(gs_handle* h, double dz, const GsTape* tape) {
    return h->fp64 ? nl_step_impl<double>(h, dz, tape) : nl_step_impl<float>(h, dz, tape);
}

static int nl_step(gs_handle* h, double dz, double* max_a2, double* max_nl2) {
    gsi::Range r("gs nl_step");
    CK(h, cudaMemsetAsync(h->max_dev, 0, 16, h->st));
    CK(h, cudaMemsetAsync(h->err_dev, 0, 4, h->st));
    int rc = h->fp64 ? nl_step_impl<double>(h, dz) : nl_step_impl<float>(h, dz);
    if (rc) return rc;
    unsigned long long mx[2];
    unsigned err = 0;
    CK(h, cudaMemcpyAsync(mx, h->max_dev, 16, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaMemcpyAsync(&err, h->err_dev, 4, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    if (h->nl_ev_pending) {   // fold the stage kernels' event times into the gs_nl_timing totals
        for (int s = 0; s < (h->nl_ev_one ? 1 : 4); s++) {
            float f = 0;
            CK(h, cudaEventElapsedTime(&f, h->nl_ev[2 * s], h->nl_ev[2 * s + 1]));
            h->nl_ms += f;
        }
        h->nl_stages_timed += 4;
        h->nl_launches_timed += h->nl_ev_one ? 1 : 4;
        h->nl_ev_one = false;
        h->nl_ev_pending = false;
    }
    double a2, n2;
    std::memcpy(&a2, &mx[0], 8);
    std::memcpy(&n2, &mx[1], 8);
    if (max_a2) *max_a2 = a2;
    if (max_nl2) *max_nl2 = n2;
    // an overflowing stage input can turn into NaN in later RK4 stages: the blast comes first
    if (err & gs::GS_ERRBIT_BOUNDS) return fail(h, GS_ERR_CUDA, gs::GS_BOUNDS_MSG);
    if (err & 1u) return fail(h, GS_ERR_BLAST, gs_status_string(GS_ERR_BLAST));
    if (err & 2u) return fail(h, GS_ERR_NAN, gs_status_string(GS_ERR_NAN));
    return GS_OK;
}

int gs_nl_step(gs_handle* h, double zstep, double* max_a2, double* max_nl2) {
    if (!h) return GS_ERR_ARG;
    if (!h->tables_ok || !h->field_ok) return fail(h, GS_ERR_STATE, "tables / field not set");
    CK(h, cudaSetDevice(h->p.device));
    h->nb_full_wanted = true;   // calculate_NLstep's BIGBUFFER1, read back by gs_get_nl
    const int rc = nl_step(h, zstep, max_a2, max_nl2);
    h->nb_full_wanted = false;
    return rc;
}

int gsi::spec_sync(gs_handle* h) {
    if (const int rc = spec_in_finish(h)) return rc;
    if (!h->s_compact) return GS_OK;
    CK(h, gs::qdht_tc_spec_copy(h->tc, (float*)h->S, 0, &h->launches));   // S stays current, the copy too
    return GS_OK;
}

void gsi::spec_written(gs_handle* h) { h->s_compact = false; }

int gsi::field_sync(gs_handle* h) {
    if (!h->a_compact) return GS_OK;
    h->a_compact = false;
    CK(h, gs::qdht_tc_expand(h->tc, (float*)h->A, &h->launches));
    return GS_OK;
}

void gsi::field_written(gs_handle* h) { h->a_compact = false; }

// BIGBUFFER2 of gs_step_host: the handle's stream waits for its copy into the staging buffer,
// then takes it as permute_in does for a staged copy (position order, and the double-float
// window columns of a mixed plan)
int gsi::spec_in_finish(gs_handle* h) {
    if (!h->spec_in_pending) return GS_OK;
    h->spec_in_pending = false;
    const size_t nel = (size_t)h->nr * h->nt;
    CK(h, cudaStreamWaitEvent(h->st, h->io_ev[1], 0));
    cudaError_t e = h->fp64 ? launch_permute<double>(+1, h->staging, h->S, h->perm_dev, h->nt, nel, h->st, &h->launches)
                            : launch_permute<float>(+1, h->staging, h->S, h->perm_dev, h->nt, nel, h->st, &h->launches);
    CK(h, e);
    if (!h->fp64 && h->tc && gs::qdht_tc_has_compact(h->tc)) {
        CK(h, gs::qdht_tc_spec_ff(h->tc, (double*)h->staging, h->perm_dev, 1, &h->launches));
        h->s_compact = true;
    }
    return GS_OK;
}

int gsi::spec_prepare(gs_handle* h) {
    if (const int rc = spec_in_finish(h)) return rc;
    if (h->s_compact || h->fp64 || !h->tc || !gs::qdht_tc_has_compact(h->tc)) return GS_OK;
    CK(h, gs::qdht_tc_spec_copy(h->tc, (float*)h->S, 1, &h->launches));
    h->s_compact = true;
    return GS_OK;
}

int gsi::lstep(gs_handle* h, double dz) {
    gsi::Range r("gs lstep");
    // mixed wide plans keep BIGBUFFER2's window columns compact from step to step
    int rc = spec_prepare(h);
    if (rc) return rc;
    const int fs = h->s_compact ? gs::QTC_S_COMPACT : 0;
    if (h->time_qdht) CK(h, cudaEventRecord(h->ev0, h->st));
    rc = run_qdht(h, QDHT_LSTEP, h->NB, h->S, dz, fs | (h->nbc_valid ? gs::QTC_X_COMPACT : 0));
    if (rc) return rc;
    // FIELD stays compact when the next NL step reads it so
    rc = run_qdht(h, QDHT_MASKED, h->S, h->A, dz, fs | ((h->a_lazy_ok && h->nl_compact) ? gs::QTC_Y_LAZY : 0));
    if (rc) return rc;
    if (h->time_qdht) {
        CK(h, cudaEventRecord(h->ev1, h->st));
        h->ev_pending = true;
    }
    return GS_OK;
}

int gs_lstep(gs_handle* h, double zstep) {
    if (!h) return GS_ERR_ARG;
    if (!h->tables_ok || !h->field_ok) return fail(h, GS_ERR_STATE, "tables / field not set");
    CK(h, cudaSetDevice(h->p.device));
    int rc = lstep(h, zstep);
    if (rc) return rc;
    CK(h, cudaStreamSynchronize(h->st));
    return collect_qdht_time(h);
}

int gs_qdht(gs_handle* h, double* data) {
    if (!h || !data) return GS_ERR_ARG;
    if (!h->tables_ok) return fail(h, GS_ERR_STATE, "tables not uploaded");
    CK(h, cudaSetDevice(h->p.device));
    const size_t nel = (size_t)h->nr * h->nt;
    char* U1 = (char*)h->U;
    void* U2 = U1 + nel * h->esz;
    int rc = permute_in(h, data, U1);
    if (!rc) rc = run_qdht(h, QDHT_PLAIN, U1, U2, 0.0);
    if (!rc) rc = permute_out(h, U2, data);
    if (!rc) rc = collect_qdht_time(h);
    return rc;
}

int gs_step(gs_handle* h, double current_z, double znet_cur, double znet_prev, double* zstep_inout,
            unsigned* step_n_inout, double* max_a2_out, double* max_nl2_out) {
    if (!h || !zstep_inout) return GS_ERR_ARG;
    if (!h->tables_ok || !h->field_ok) return fail(h, GS_ERR_STATE, "tables / field not set");
    CK(h, cudaSetDevice(h->p.device));
    gsi::Range r("gs_step");
    const double tol = h->p.max_tolerance;
    double zstep = *zstep_inout;
    for (;;) {
        double max_a2 = 0, max_nl2 = 0;
        int rc = nl_step(h, zstep, &max_a2, &max_nl2);
        if (rc) return rc;
        // propagator.cu:147-164
        bool repeat = false;
        if (zstep * zstep * max_nl2 > tol * tol * max_a2) {
            repeat = true;
            if (step_n_inout) (*step_n_inout)++;
        }
        zstep = 0.5 * tol * std::sqrt(max_a2 / max_nl2);
        if (zstep < 1e-10 * (znet_cur - znet_prev) || !(zstep > 0)) {
            *zstep_inout = zstep;
            return fail(h, GS_ERR_COLLAPSE, gs_status_string(GS_ERR_COLLAPSE));
        }
        const double lim = znet_cur - current_z;
        if (lim < zstep) zstep = lim;
        if (max_a2_out) *max_a2_out = max_a2;
        if (max_nl2_out) *max_nl2_out = max_nl2;
        if (!repeat) {
            if (h->en_tol > 0) {   // the optional photon-number check (gs_set_energy_tolerance)
                rc = gsi::lstep_checked(h, &zstep, 1e-10 * (znet_cur - znet_prev));
                *zstep_inout = zstep;
            } else {
                *zstep_inout = zstep;
                rc = lstep(h, zstep);
            }
            if (rc) return rc;
            // apertures (propagator.cu:232-261), with CURRENT_Z the z before this step
            if (!h->ap_z.empty() && current_z >= h->ap_z.back()) {
                const int k0 = h->ap_row0.back();
                rc = gsi::field_sync(h);
                if (rc) return rc;
                if (k0 < h->nr)
                    CK(h, cudaMemsetAsync((char*)h->A + (size_t)k0 * h->nt * h->esz, 0,
                                          (size_t)(h->nr - k0) * h->nt * h->esz, h->st));
                rc = run_qdht(h, QDHT_PLAIN, h->A, h->S, 0.0);
                if (rc) return rc;
                h->en_prev = 0;   // the photon number of the field the aperture left is taken anew
                h->ap_z.pop_back();
                h->ap_row0.pop_back();
            }
            CK(h, cudaStreamSynchronize(h->st));
            return collect_qdht_time(h);
        }
    }
}

int gs_step_host(gs_handle* h, double* field, double* spec, double current_z, double znet_cur, double znet_prev,
                 double* zstep_inout, unsigned* step_n_inout, double* max_a2, double* max_nl2) {
    if (!h || !field || !spec || !zstep_inout) return fail(h, GS_ERR_ARG, "null argument");
    const size_t bytes = (size_t)h->nr * h->nt * 16;
    if ((const char*)field < (const char*)spec + bytes && (const char*)spec < (const char*)field + bytes)
        return fail(h, GS_ERR_ARG, "gs_step_host: FIELD and BIGBUFFER2 overlap");
    if (!h->tables_ok) return fail(h, GS_ERR_STATE, "tables not uploaded");
    CK(h, cudaSetDevice(h->p.device));
    gsi::Range r("gs_step_host");
    if (!h->io_st) {
        CK(h, cudaStreamCreateWithFlags(&h->io_st, cudaStreamNonBlocking));
        for (cudaEvent_t& e : h->io_ev) CK(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    // FIELD first (the NL attempt reads nothing else), then BIGBUFFER2 on the copy stream into
    // the staging buffer while the attempt runs; the linear step takes it (spec_in_finish)
    int rc = gsi::permute_in(h, field, h->A);
    if (rc) return rc;
    gsi::spec_written(h);
    CK(h, cudaEventRecord(h->io_ev[0], h->st));
    CK(h, cudaStreamWaitEvent(h->io_st, h->io_ev[0], 0));
    CK(h, cudaMemcpyAsync(h->staging, spec, (size_t)h->nr * h->nt * 16, cudaMemcpyHostToDevice, h->io_st));
    CK(h, cudaEventRecord(h->io_ev[1], h->io_st));
    h->spec_in_pending = true;
    h->field_ok = true;
    h->en_prev = 0;
    rc = gs_step(h, current_z, znet_cur, znet_prev, zstep_inout, step_n_inout, max_a2, max_nl2);
    const int rf = gsi::spec_in_finish(h);   // a failed call still leaves BIGBUFFER2 installed
    if (rc) return rc;
    if (rf) return rf;
    rc = gsi::permute_out(h, h->S, spec);
    if (!rc) rc = gsi::permute_out(h, h->A, field);
    return rc;
}

#if GS_CHECK
// buf has more than len + 1 elements: the tested index len is inside the allocation
__global__ void bounds_probe_kernel(float* buf, int len, unsigned* err) {
    const int idx = len;
    if (gs::in_bounds(idx < len, err)) buf[idx] = 1.f;
}
#endif

int gs_check_build(void) { return GS_CHECK ? 1 : 0; }

int gs_selftest_bounds(gs_handle* h) {
    if (!h) return GS_ERR_ARG;
#if GS_CHECK
    CK(h, cudaSetDevice(h->p.device));
    CK(h, cudaMemsetAsync(h->err_dev, 0, 4, h->st));
    bounds_probe_kernel<<<1, 1, 0, h->st>>>(reinterpret_cast<float*>(h->staging), 1, h->err_dev);
    h->launches++;
    CK(h, cudaGetLastError());
    unsigned err = 0;
    CK(h, cudaMemcpyAsync(&err, h->err_dev, 4, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    CK(h, cudaMemsetAsync(h->err_dev, 0, 4, h->st));
    if (err & gs::GS_ERRBIT_BOUNDS) return fail(h, GS_ERR_CUDA, gs::GS_BOUNDS_MSG);
    return fail(h, GS_ERR_STATE, "gs_selftest_bounds: the index test did not report");
#else
    return fail(h, GS_ERR_UNSUPPORTED, "gs_selftest_bounds: built without GS_CHECK");
#endif
}

int gs_selftest_bounded_wait(gs_handle* h, double limit_s) {
    if (!h || !(limit_s > 0) || limit_s > 1.0) return fail(h, GS_ERR_ARG, "gs_selftest_bounded_wait: 0 < limit <= 1 s");
    if (!h->tc) return fail(h, GS_ERR_UNSUPPORTED, "gs_selftest_bounded_wait: mixed handles only");
    CK(h, cudaSetDevice(h->p.device));
    CK(h, gs::qdht_tc_wait_probe(h->tc, limit_s, &h->launches));
    std::string m;
    if (gs::qdht_tc_check(h->tc, &m)) return fail(h, GS_ERR_CUDA, m);
    return GS_OK;
}

int gs_set_apertures(gs_handle* h, int n, const double* z, const double* r, const double* qdht_x, double r_max) {
    if (!h || n < 0 || (n > 0 && (!z || !r || !qdht_x))) return fail(h, GS_ERR_ARG, "gs_set_apertures: bad argument");
    h->ap_z.assign(z, z + n);
    h->ap_row0.assign(n, h->nr);
    for (int i = 0; i < n; i++) {
        // rows with R = x_n R_MAX > r are zeroed; x_n increases with n
        int k0 = h->nr;
        for (int k = 0; k < h->nr; k++)
            if (qdht_x[k] * r_max > r[i]) { k0 = k; break; }
        for (int k = k0; k < h->nr; k++)
            if (!(qdht_x[k] * r_max > r[i])) return fail(h, GS_ERR_ARG, "gs_set_apertures: QDHT points not increasing");
        h->ap_row0[i] = k0;
    }
    return GS_OK;
}

// ------------------------------------------------------------------ autotuning --
// Candidate launch shapes of the fused RK4-stage kernels (threads per radial row: the FFT's
// parallelism and the recurrences' chunk length L = n_t / threads) are timed on this
// handle's own rows and the fastest is kept; the choice is cached per (precision, n_r, n_t)
// for the process, so a batch of pulses on the same grid tunes once.
static std::map<std::tuple<int, int, int>, std::pair<int, double>> g_tune_cache;

int gs_autotune(gs_handle* h, int* threads_out, double* ms_per_stage_out) {
    if (!h) return GS_ERR_ARG;
    if (!h->tables_ok || !h->field_ok) return fail(h, GS_ERR_STATE, "tables / field not set");
    CK(h, cudaSetDevice(h->p.device));
    const int nt = h->nt;
    const auto key = std::make_tuple(h->fp64 ? 1 : 0, h->nr, nt);
    auto it = g_tune_cache.find(key);
    if (it == g_tune_cache.end()) {
        int best = 0;
        double best_ms = 0;
        if (h->fused && h->p.nonlinear) {
            const int cand[4] = {nt / 32, nt / 16, nt / 8, nt / 4};
            for (int c : cand) {
                const bool ok = h->fp64 ? nl_fused_threads_ok<double>(nt, c) : nl_fused_threads_ok<float>(nt, c);
                if (!ok) continue;
                h->nl_threads = c;
                // stages read FIELD and write only scratch (BIGBUFFER1, the stage buffers)
                int rc = GS_OK;
                for (int w = 0; w < 2 && !rc; w++) rc = gsi::nl_stages(h, 0.0, nullptr);
                if (rc) return rc;
                CK(h, cudaEventRecord(h->ev0, h->st));
                const int reps = 5;
                for (int r = 0; r < reps && !rc; r++) rc = gsi::nl_stages(h, 0.0, nullptr);
                if (rc) return rc;
                CK(h, cudaEventRecord(h->ev1, h->st));
                CK(h, cudaEventSynchronize(h->ev1));
                float ms = 0;
                CK(h, cudaEventElapsedTime(&ms, h->ev0, h->ev1));
                const double per = ms / (4.0 * reps);
                if (best == 0 || per < best_ms) {
                    best = c;
                    best_ms = per;
                }
            }
            CK(h, cudaMemsetAsync(h->err_dev, 0, 4, h->st));
            CK(h, cudaStreamSynchronize(h->st));
        }
        it = g_tune_cache.emplace(key, std::make_pair(best, best_ms)).first;
    }
    h->nl_threads = it->second.first;
    if (threads_out)
        *threads_out = h->nl_threads > 0 ? h->nl_threads
                                          : (h->fp64 ? nl_fused_default_threads<double>(nt) : nl_fused_default_threads<float>(nt));
    if (ms_per_stage_out) *ms_per_stage_out = it->second.second;
    return GS_OK;
}

int gs_set_nl_threads(gs_handle* h, int threads) {
    if (!h) return GS_ERR_ARG;
    if (threads != 0) {
        const bool ok = h->fp64 ? nl_fused_threads_ok<double>(h->nt, threads) : nl_fused_threads_ok<float>(h->nt, threads);
        if (!ok || !h->fused) return fail(h, GS_ERR_ARG, "threads per row not valid for this grid");
    }
    h->nl_threads = threads;
    return GS_OK;
}

int gs_get_nl_threads(const gs_handle* h) {
    if (!h) return 0;
    if (h->nl_threads > 0) return h->nl_threads;
    return h->fp64 ? nl_fused_default_threads<double>(h->nt) : nl_fused_default_threads<float>(h->nt);
}

// ------------------------------------------------------------------ dump reductions --
template <typename Rl>
static int dump_impl(gs_handle* h, const double* qdht_x, double r_max, double* max_I, double* flux,
                     double* plasma_max, double* field_axis, double* avg_spectrum) {
    using T2 = typename Vec2<Rl>::T;
    const int nr = h->nr, nt = h->nt;
    if (!h->dump_dev) CK(h, cudaMalloc((void**)&h->dump_dev, sizeof(double) * (4 * (size_t)nr + 2 * (size_t)nt)));
    double* d_maxI = h->dump_dev;
    double* d_flux = d_maxI + nr;
    double* d_pmax = d_flux + nr;
    double* d_w = d_pmax + nr;
    double* d_spec = d_w + nr;
    // E = BW-FFT(FIELD)/N_T, natural time order
    FftArgs<Rl> f{};
    f.N = nt; f.M = h->M; f.P = h->P; f.logM = h->logM; f.rows = nr;
    f.tw = (const T2*)h->tw; f.tpost = 1;
    f.twb = (const T2*)h->twb;
    {
        const int rs = gsi::field_sync(h);
        if (rs) return rs;
    }
    CK(h, launch_fft<Rl>(+1, (const T2*)h->A, (T2*)h->E, f, h->st, &h->launches));
    if (max_I || flux) CK(h, launch_row_intensity<Rl>((const T2*)h->E, nr, nt, h->p.tstep, d_maxI, d_flux, h->st, &h->launches));
    if (plasma_max) {
        CK(h, cudaMemsetAsync(h->err_dev, 0, 4, h->st));
        PlasmaArgs<Rl> pa = plasma_args<Rl>(h, true, false);
        pa.density_only = 1;
        CK(h, launch_plasma<Rl>(pa, nr, h->st, &h->launches));
        CK(h, launch_row_max_re<Rl>((const T2*)h->U + (size_t)nr * nt, nr, nt, d_pmax, h->st, &h->launches));
    }
    std::vector<double> spec_pos;
    if (avg_spectrum) {
        if (!qdht_x || nr < 2) return fail(h, GS_ERR_ARG, "average spectrum needs the QDHT points");
        // dump_type_average_spectrum_class, uniaxial branch (dump_types.cpp:441-453)
        std::vector<double> w(nr);
        w[0] = qdht_x[0] * (qdht_x[1] - qdht_x[0]);
        for (int r = 1; r < nr; r++) w[r] = qdht_x[r] * (qdht_x[r] - qdht_x[r - 1]);
        CK(h, cudaMemcpyAsync(d_w, w.data(), sizeof(double) * nr, cudaMemcpyHostToDevice, h->st));
        CK(h, launch_spectrum<Rl>((const T2*)h->A, nr, nt, d_w, r_max * r_max / 2.0, d_spec, h->st, &h->launches));
        spec_pos.resize(nt);
        CK(h, cudaMemcpyAsync(spec_pos.data(), d_spec, sizeof(double) * nt, cudaMemcpyDeviceToHost, h->st));
    }
    if (max_I) CK(h, cudaMemcpyAsync(max_I, d_maxI, sizeof(double) * nr, cudaMemcpyDeviceToHost, h->st));
    if (flux) CK(h, cudaMemcpyAsync(flux, d_flux, sizeof(double) * nr, cudaMemcpyDeviceToHost, h->st));
    if (plasma_max) CK(h, cudaMemcpyAsync(plasma_max, d_pmax, sizeof(double) * nr, cudaMemcpyDeviceToHost, h->st));
    std::vector<T2> axis;
    if (field_axis) {
        axis.resize(nt);
        CK(h, cudaMemcpyAsync(axis.data(), h->E, sizeof(T2) * nt, cudaMemcpyDeviceToHost, h->st));
    }
    unsigned err = 0;
    CK(h, cudaMemcpyAsync(&err, h->err_dev, 4, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    for (int t = 0; t < (field_axis ? nt : 0); t++) {
        field_axis[2 * t] = (double)axis[t].x;
        field_axis[2 * t + 1] = (double)axis[t].y;
    }
    if (avg_spectrum)
        for (int p = 0; p < nt; p++) avg_spectrum[h->perm[p]] = spec_pos[p];
    if (err & gs::GS_ERRBIT_BOUNDS) return fail(h, GS_ERR_CUDA, gs::GS_BOUNDS_MSG);
    if (err & 1u) return fail(h, GS_ERR_BLAST, gs_status_string(GS_ERR_BLAST));
    if (err & 2u) return fail(h, GS_ERR_NAN, gs_status_string(GS_ERR_NAN));
    return GS_OK;
}

int gs_dump_reductions(gs_handle* h, const double* qdht_x, double r_max, double* max_I, double* flux,
                       double* plasma_max, double* field_axis, double* avg_spectrum) {
    if (!h) return GS_ERR_ARG;
    if (!h->tables_ok || !h->field_ok) return fail(h, GS_ERR_STATE, "tables / field not set");
    CK(h, cudaSetDevice(h->p.device));
    return h->fp64 ? dump_impl<double>(h, qdht_x, r_max, max_I, flux, plasma_max, field_axis, avg_spectrum)
                   : dump_impl<float>(h, qdht_x, r_max, max_I, flux, plasma_max, field_axis, avg_spectrum);
}

int gs_get_time_field(gs_handle* h, double* e_r_t) {
    if (!h || !e_r_t) return GS_ERR_ARG;
    if (!h->tables_ok || !h->field_ok) return fail(h, GS_ERR_STATE, "tables / field not set");
    CK(h, cudaSetDevice(h->p.device));
    const size_t nel = (size_t)h->nr * h->nt;
    {
        const int rs = gsi::field_sync(h);
        if (rs) return rs;
    }
    cudaError_t e;
    if (h->fp64) {
        FftArgs<double> f{};
        f.N = h->nt; f.M = h->M; f.P = h->P; f.logM = h->logM; f.rows = h->nr;
        f.tw = (const double2*)h->tw; f.tpost = 1;
        f.twb = (const double2*)h->twb;
        e = launch_fft<double>(+1, (const double2*)h->A, h->staging, f, h->st, &h->launches);
    } else {
        FftArgs<float> f{};
        f.N = h->nt; f.M = h->M; f.P = h->P; f.logM = h->logM; f.rows = h->nr;
        f.tw = (const float2*)h->tw; f.tpost = 1;
        f.twb = (const float2*)h->twb;
        e = launch_fft<float>(+1, (const float2*)h->A, (float2*)h->E, f, h->st, &h->launches);
        if (e == cudaSuccess) {
            // widen to FP64 in natural order (time rows are natural): identity permutation copy
            std::vector<float2> tmp(nel);
            e = cudaMemcpyAsync(tmp.data(), h->E, nel * 8, cudaMemcpyDeviceToHost, h->st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
            for (size_t i = 0; e == cudaSuccess && i < nel; i++) {
                e_r_t[2 * i] = tmp[i].x;
                e_r_t[2 * i + 1] = tmp[i].y;
            }
            CK(h, e);
            return GS_OK;
        }
    }
    CK(h, e);
    CK(h, cudaMemcpyAsync(e_r_t, h->staging, nel * 16, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    return GS_OK;
}
