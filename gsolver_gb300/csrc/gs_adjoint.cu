// gs_adjoint.cu -- gradients of an output objective with respect to the input field, by
// the adjoint of the z-step (no counterpart in the reference, which has no adjoint).
//
// The forward is the reference's propagator() with the controller's step sizes given
// (dz_rk[n] for the RK4 stages of step n, dz_lin[n] for its linear step, as a run with
// the adaptive controller produced them), so the map FIELD_0 -> FIELD_N is smooth and its
// discrete adjoint is exact.  Objective J = sum_{r,omega} w |FIELD_N|^2 (band energy with
// the QDHT radial weights, fluence, ... by the choice of w).  Cotangents follow
// g = dJ/dRe + i dJ/dIm.
//
// Per step, backwards (cotangents A_bar of FIELD (r,omega), S_bar of BIGBUFFER2 (k,omega)):
//   F_bar = H^T A_bar;  linear-step adjoint -> S_bar, B1_bar;  R_bar = H^T B1_bar;
//   four stage VJPs (gs_nl_vjp.cu) from the recorded stages -> A_bar.
// Finally A_bar += H^T S_bar (BIGBUFFER2 starts as QDHT(FIELD)).  H^T is the QDHT with
// 1/m1 in place of m1.
//
// Memory: checkpointing.  The forward stores (FIELD, BIGBUFFER2) every K steps and records
// the four RK4 stages of every step of the last segment (E/N, rho, Q per sample); the
// backward sweep walks that segment back, then re-runs each earlier segment from its
// checkpoint, recording its stages, and walks it back.  Device memory: 7 work arrays, 2 per
// checkpoint and 4 (E, rho, Q) triples per step of a segment.  The n - K steps before the
// last segment run twice, so K is as large as memory allows: unless given, every step is
// recorded during the forward when that fits in half of the device memory that is free (the
// handle's own adjoint arrays counted as free), else the largest K that fits, and at least
// ceil(sqrt(n)) (the forward then runs about twice in all).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gs_handle.h"

using namespace gs;

namespace {

struct AdjLayout {
    size_t nel, esz, rsz;
    int K, nck;
    size_t work_bytes() const { return 7 * nel * esz; }
    // per checkpoint: FIELD, BIGBUFFER2 and (mixed) its window columns as double-float pairs
    size_t spec_bytes = 0;
    size_t ck_slot() const { return 2 * nel * esz + spec_bytes; }
    size_t ck_bytes() const { return (size_t)(nck > 1 ? nck - 1 : 0) * ck_slot(); }   // the last segment is recorded
    int nr;
    size_t ion_bytes() const { return ((size_t)nr * 4 + 255) & ~(size_t)255; }
    size_t tape_step_bytes() const { return 4 * (nel * (esz + 2 * rsz) + ion_bytes()); }
    size_t total() const { return work_bytes() + ck_bytes() + (size_t)K * tape_step_bytes(); }
};

struct AdjPtrs {
    void *Ab, *Sb, *Rb, *KB, *Eb, *Fb;
    void* Sl;   // mixed: the low parts of BIGBUFFER2's cotangent (double-float pairs Sb + Sl)
    char* ck;
    char* tape;
};

int ensure_adj(gs_handle* h, const AdjLayout& L, AdjPtrs* P) {
    const size_t need = L.total();
    if (h->adj_bytes < need) {
        if (h->adj) cudaFree(h->adj);
        h->adj = nullptr;
        h->adj_bytes = 0;
        if (cudaMalloc(&h->adj, need) != cudaSuccess) {
            cudaGetLastError();
            return gsi::fail(h, GS_ERR_NOMEM, "adjoint: cannot allocate " + std::to_string(need >> 20) +
                                                  " MiB (work arrays, checkpoints, stage records); "
                                                  "give a smaller checkpoint stride");
        }
        h->adj_bytes = need;
    }
    char* b = (char*)h->adj;
    const size_t a = L.nel * L.esz;
    P->Ab = b; P->Sb = b + a; P->Rb = b + 2 * a; P->KB = b + 3 * a; P->Eb = b + 4 * a; P->Fb = b + 5 * a;
    P->Sl = b + 6 * a;
    P->ck = b + L.work_bytes();
    P->tape = P->ck + L.ck_bytes();
    return GS_OK;
}

// the checkpoint stride for n steps when none is given (see the memory note above)
int auto_stride(gs_handle* h, AdjLayout L, int n) {
    const int ks = (int)std::ceil(std::sqrt((double)n));
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        return ks;
    }
    const size_t budget = (fr + h->adj_bytes) / 2;
    int K = n;
    for (int it = 0; it < 64 && K > ks; it++) {
        L.K = K;
        L.nck = (n + K - 1) / K;
        if (L.total() <= budget) return K;
        const size_t fixed = L.work_bytes() + L.ck_bytes();
        const long long fit = budget > fixed ? (long long)((budget - fixed) / L.tape_step_bytes()) : 0;
        K = (int)std::max<long long>(ks, std::min<long long>(K - 1, fit));
    }
    return std::max(K, ks);
}

GsTape tape_of(const AdjLayout& L, char* base, int slot) {
    GsTape t;
    char* s = base + (size_t)slot * L.tape_step_bytes();
    for (int k = 0; k < 4; k++) {
        t.e[k] = s;
        s += L.nel * L.esz;
        t.rho[k] = s;
        s += L.nel * L.rsz;
        t.q[k] = s;
        s += L.nel * L.rsz;
        t.ion[k] = (int*)s;
        s += L.ion_bytes();
    }
    return t;
}

// objective weights in position order, plus the partial sums of J
int upload_weights(gs_handle* h, const double* w, int nblocks) {
    const size_t nel = (size_t)h->nr * h->nt;
    const size_t need = (nel + nblocks + 8) * sizeof(double);
    if (h->adj_w_bytes < need) {
        if (h->adj_w) cudaFree(h->adj_w);
        h->adj_w = nullptr;
        h->adj_w_bytes = 0;
        if (cudaMalloc((void**)&h->adj_w, need) != cudaSuccess) {
            cudaGetLastError();
            return gsi::fail(h, GS_ERR_NOMEM, "adjoint: cannot allocate the objective weights");
        }
        h->adj_w_bytes = need;
    }
    std::vector<double> wp(nel);
    for (int r = 0; r < h->nr; r++)
        for (int p = 0; p < h->nt; p++) wp[(size_t)r * h->nt + p] = w[(size_t)r * h->nt + h->perm[p]];
    CK(h, cudaMemcpyAsync(h->adj_w, wp.data(), nel * sizeof(double), cudaMemcpyHostToDevice, h->st));
    CK(h, cudaStreamSynchronize(h->st));   // wp is a host temporary
    return GS_OK;
}

int run_qdht_t(gs_handle* h, const void* X, void* Y) {
    LstepArgs L{};
    if (h->fp64) {
        CK(h, launch_qdht64(QDHT_PLAIN, h->Cm, h->m1inv, (const double*)X, (double*)Y, h->nr, 2 * h->nt, L, h->st,
                            &h->launches));
        return GS_OK;
    }
    if (!h->tcT) {
        std::string m;
        h->tcT = gs::qdht_tc_create(h->nr, h->nt, h->st, &m);
        if (!h->tcT) return gsi::fail(h, GS_ERR_UNSUPPORTED, "transposed mixed QDHT: " + m);
        if (gs::qdht_tc_set_matrix(h->tcT, h->c_host.data(), h->m1inv_host.data(), &m))
            return gsi::fail(h, GS_ERR_CUDA, "transposed mixed QDHT matrix: " + m);
    }
    std::string m;
    cudaError_t e = gs::qdht_tc_run(h->tcT, QDHT_PLAIN, (const float*)X, (float*)Y, L, &h->launches, &m);
    if (e != cudaSuccess) return gsi::fail(h, GS_ERR_CUDA, "transposed mixed QDHT: " + m + " " + cudaGetErrorString(e));
    return GS_OK;
}

int check_adjoint_supported(gs_handle* h) {
    if (!h->tables_ok) return gsi::fail(h, GS_ERR_STATE, "tables not uploaded");
    if (!h->p.nonlinear) return GS_OK;
    if (h->p.gas) return gsi::fail(h, GS_ERR_UNSUPPORTED, "adjoint: the gas build is not differentiated");
    const bool raman = h->p.raman_fraction > 0.001 && h->p.n2 != 0;
    if (raman && !gsi::raman_scan_on(h))
        return gsi::fail(h, GS_ERR_UNSUPPORTED, "adjoint: the Raman response needs its oscillator parameters");
    const bool ok = h->fused && (h->fp64 ? nl_vjp_supported<double>(h->nt) : nl_vjp_supported<float>(h->nt));
    if (!ok)
        return gsi::fail(h, GS_ERR_UNSUPPORTED,
                         "adjoint: rows must fit one CTA's shared memory (n_t <= 8192 mixed, <= 4096 FP64)");
    // the shared-memory size is a per-kernel attribute: set it for this grid on every call
    const cudaError_t e = h->fp64 ? nl_vjp_setup<double>(h->nt) : nl_vjp_setup<float>(h->nt);
    if (e != cudaSuccess) return gsi::cuda_fail(h, e, "nl_vjp_setup");
    return GS_OK;
}

template <typename Rl>
int stage_vjps(gs_handle* h, const AdjPtrs& P, const GsTape& tp, double dz) {
    using T2 = typename Vec2<Rl>::T;
    const bool raman = h->p.raman_fraction > 0.001;
    const bool scan = gsi::raman_scan_on(h);
    const PlasmaArgs<Rl> pa = gsi::plasma_args<Rl>(h, raman, scan);
    VjpArgs<Rl> v{};
    v.N = h->nt;
    v.logM = h->logM;
    v.tw = (const T2*)h->tw;
    v.twb = (const T2*)h->twb;
    v.pf = (const T2*)h->pf;
    v.kerr = (const Rl*)h->kerr;
    v.rate = (const Rl*)h->rate;
    v.ebar = (T2*)P.Eb;
    v.ab = (T2*)P.Ab;
    v.rbar = (const T2*)P.Rb;
    v.kerr_on = h->p.n2 != 0;
    v.raman_scan = scan;
    v.tstep_scaled = pa.tstep_scaled;
    v.neutral_density = pa.neutral_density;
    v.ionization_potential = pa.ionization_potential;
    v.ponderomotive = pa.ponderomotive;
    v.avalanche_cs = pa.avalanche_cs;
    v.recombination_tau = pa.recombination_tau;
    v.a_re = pa.a_re; v.a_im = pa.a_im; v.aN_re = pa.aN_re; v.aN_im = pa.aN_im;
    v.fRM = pa.fRM; v.one_minus_fR = pa.one_minus_fR;
    v.threads = 0;   // N/16: measured faster for the VJP than the forward's tuned shape at 256x4096
    // R = (k1 + 2 k2 + 2 k3 + k4)/6 with stage inputs A + dz/2 k1, A + dz/2 k2, A + dz k3
    const double cR_next[4] = {0.0, 1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0};   // weight of k_{s-1} in R
    const double cdz_next[4] = {0.0, 0.5 * dz, 0.5 * dz, dz};          // stage s input coefficient
    for (int s = 3; s >= 0; s--) {
        VjpArgs<Rl> a = v;
        a.kb = (s == 3) ? (const T2*)P.Rb : (const T2*)P.KB;
        a.kb_scale = (s == 3) ? 1.0 / 6.0 : 1.0;
        a.tape_e = (const T2*)tp.e[s];
        a.tape_rho = (const Rl*)tp.rho[s];
        a.tape_q = (const Rl*)tp.q[s];
        a.tape_ion = tp.ion[s];
        a.ab_add = s != 3;
        a.kb_out = (s > 0) ? (T2*)P.KB : nullptr;
        a.cR = cR_next[s];
        a.cdz = cdz_next[s];
        CK(h, launch_nl_vjp<Rl>(a, h->nr, h->st, &h->launches));
    }
    return GS_OK;
}

// cotangents (A_bar, S_bar) after step -> before it; tp = the step's recorded stages
int adjoint_step(gs_handle* h, const AdjPtrs& P, const GsTape& tp, double dz_rk, double dz_lin) {
    gsi::Range r("gs adjoint_step");
    const size_t nel = (size_t)h->nr * h->nt;
    int rc = run_qdht_t(h, P.Ab, P.Fb);
    if (rc) return rc;
    LstepArgs L{};
    L.dz = dz_lin;
    L.omega = h->omega;
    L.wavenum = h->wavenum;
    L.ho = h->ho;
    L.kt2 = h->kt2;
    L.omega_min = h->p.omega_min;
    L.omega_max = h->p.omega_max;
    if (h->fp64)
        CK(h, launch_lstep_adj<double>((const double2*)P.Fb, (double2*)P.Sb, (double2*)P.KB, h->nr, h->nt, L, h->st,
                                       &h->launches));
    else   // the arithmetic of the mixed forward's fused epilogue (double-float where it is)
        CK(h, gs::qdht_tc_lstep_adj(h->tc, (const float*)P.Fb, (float*)P.Sb, (float*)P.Sl, (float*)P.KB, dz_lin,
                                    &h->launches));
    if (!h->p.nonlinear) {   // N = 0: FIELD enters the step only through the NL response
        CK(h, cudaMemsetAsync(P.Ab, 0, nel * h->esz, h->st));
        return GS_OK;
    }
    rc = run_qdht_t(h, P.KB, P.Rb);
    if (rc) return rc;
    return h->fp64 ? stage_vjps<double>(h, P, tp, dz_rk) : stage_vjps<float>(h, P, tp, dz_rk);
}

int read_err(gs_handle* h) {
    unsigned err = 0;
    CK(h, cudaMemcpyAsync(&err, h->err_dev, 4, cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    if (h->tc || h->tcT) {
        std::string m;
        if (h->tc && gs::qdht_tc_check(h->tc, &m)) return gsi::fail(h, GS_ERR_CUDA, m);
        if (h->tcT && gs::qdht_tc_check(h->tcT, &m)) return gsi::fail(h, GS_ERR_CUDA, m);
    }
    if (err & GS_ERRBIT_BOUNDS) return gsi::fail(h, GS_ERR_CUDA, GS_BOUNDS_MSG);
    if (err & 1u) return gsi::fail(h, GS_ERR_BLAST, gs_status_string(GS_ERR_BLAST));
    if (err & 2u) return gsi::fail(h, GS_ERR_NAN, gs_status_string(GS_ERR_NAN));
    return GS_OK;
}

int objective(gs_handle* h, const AdjPtrs* P, double* J) {
    const size_t nel = (size_t)h->nr * h->nt;
    const int nb = 4 * 152;
    double* part = h->adj_w + nel;
    double* jd = part + nb;
    void* ab = P ? P->Ab : h->KP;   // the forward alone: A_bar lands in scratch
    const int rs = gsi::field_sync(h);
    if (rs) return rs;
    if (h->fp64)
        CK(h, launch_adj_seed<double>((const double2*)h->A, h->adj_w, (double2*)ab, nel, part, nb, jd, h->st,
                                      &h->launches));
    else
        CK(h, launch_adj_seed<float>((const float2*)h->A, h->adj_w, (float2*)ab, nel, part, nb, jd, h->st,
                                     &h->launches));
    CK(h, cudaMemcpyAsync(J, jd, sizeof(double), cudaMemcpyDeviceToHost, h->st));
    return GS_OK;
}

int check_args(gs_handle* h, const double* field_in, int n_steps, const double* dz_rk, const double* dz_lin,
               const double* weights) {
    if (!field_in || !dz_rk || !dz_lin || !weights || n_steps < 1)
        return gsi::fail(h, GS_ERR_ARG, "null argument or n_steps < 1");
    for (int n = 0; n < n_steps; n++)
        if (!(dz_rk[n] > 0) || !(dz_lin[n] > 0)) return gsi::fail(h, GS_ERR_ARG, "step sizes must be > 0");
    return GS_OK;
}

}  // namespace

int gs_forward_fixed(gs_handle* h, const double* field_in, int n_steps, const double* dz_rk, const double* dz_lin,
                     const double* weights, double* objective_out, double* field_out) {
    if (!h) return GS_ERR_ARG;
    int rc = check_args(h, field_in, n_steps, dz_rk, dz_lin, weights);
    if (rc) return rc;
    if (!h->tables_ok) return gsi::fail(h, GS_ERR_STATE, "tables not uploaded");
    CK(h, cudaSetDevice(h->p.device));
    rc = upload_weights(h, weights, 4 * 152);
    if (rc) return rc;
    CK(h, cudaMemsetAsync(h->err_dev, 0, 4, h->st));
    rc = gsi::permute_in(h, field_in, h->A);
    if (!rc) rc = gsi::run_qdht(h, QDHT_PLAIN, h->A, h->S, 0.0);
    h->field_ok = rc == GS_OK;
    for (int n = 0; n < n_steps && !rc; n++) {
        rc = gsi::nl_stages(h, dz_rk[n], nullptr);
        if (!rc) rc = gsi::lstep(h, dz_lin[n]);
    }
    if (rc) return rc;
    double J = 0;
    rc = objective(h, nullptr, &J);
    if (!rc) rc = read_err(h);
    if (rc) return rc;
    if (objective_out) *objective_out = J;
    if (field_out) rc = gsi::permute_out(h, h->A, field_out);
    return rc;
}

int gs_gradient(gs_handle* h, const double* field_in, int n_steps, const double* dz_rk, const double* dz_lin,
                const double* weights, int checkpoint_stride, double* objective_out, double* grad_field) {
    if (!h) return GS_ERR_ARG;
    int rc = check_args(h, field_in, n_steps, dz_rk, dz_lin, weights);
    if (rc) return rc;
    if (!grad_field) return gsi::fail(h, GS_ERR_ARG, "null gradient output");
    rc = check_adjoint_supported(h);
    if (rc) return rc;
    CK(h, cudaSetDevice(h->p.device));
    AdjLayout L;
    L.nel = (size_t)h->nr * h->nt;
    L.nr = h->nr;
    L.esz = h->esz;
    L.rsz = h->esz / 2;
    float *spc = nullptr, *spl = nullptr;   // BIGBUFFER2's compact double-float columns (mixed)
    int spn = 0;
    if (!h->fp64 && h->tc) gs::qdht_tc_spec_pairs(h->tc, &spc, &spl, &spn);
    const size_t spb = (size_t)h->nr * spn * sizeof(float);
    L.spec_bytes = spc ? 2 * spb : 0;
    L.K = checkpoint_stride > 0 ? checkpoint_stride : auto_stride(h, L, n_steps);
    if (L.K > n_steps) L.K = n_steps;
    h->adj_stride = L.K;
    L.nck = (n_steps + L.K - 1) / L.K;
    AdjPtrs P;
    rc = ensure_adj(h, L, &P);
    if (!rc) rc = upload_weights(h, weights, 4 * 152);
    if (rc) return rc;
    CK(h, cudaMemsetAsync(h->err_dev, 0, 4, h->st));
    const size_t arr = L.nel * L.esz;

    // forward, storing a checkpoint every K steps; the last segment records its stages now,
    // so the backward sweep starts without re-running it
    const int last0 = (L.nck - 1) * L.K;
    std::vector<char> ck_pairs((size_t)L.nck, 0);   // whether checkpoint k holds the compact pairs
    rc = gsi::permute_in(h, field_in, h->A);
    if (!rc) rc = gsi::run_qdht(h, QDHT_PLAIN, h->A, h->S, 0.0);
    h->field_ok = rc == GS_OK;
    for (int n = 0; n < n_steps && !rc; n++) {
        if (n % L.K == 0 && n < last0) {
            char* ck = P.ck + (size_t)(n / L.K) * L.ck_slot();
            rc = gsi::field_sync(h);
            if (rc) return rc;
            CK(h, cudaMemcpyAsync(ck, h->A, arr, cudaMemcpyDeviceToDevice, h->st));
            rc = gsi::spec_sync(h);
            if (rc) return rc;
            CK(h, cudaMemcpyAsync(ck + arr, h->S, arr, cudaMemcpyDeviceToDevice, h->st));
            if (spc && h->s_compact) {   // the low parts too: a re-run segment repeats the forward exactly
                CK(h, cudaMemcpyAsync(ck + 2 * arr, spc, spb, cudaMemcpyDeviceToDevice, h->st));
                CK(h, cudaMemcpyAsync(ck + 2 * arr + spb, spl, spb, cudaMemcpyDeviceToDevice, h->st));
                ck_pairs[n / L.K] = 1;
            }
        }
        const bool rec = h->p.nonlinear && n >= last0;
        const GsTape tp = tape_of(L, P.tape, rec ? n - last0 : 0);
        rc = gsi::nl_stages(h, dz_rk[n], rec ? &tp : nullptr);
        if (!rc) rc = gsi::lstep(h, dz_lin[n]);
    }
    if (rc) return rc;
    double J = 0;
    rc = objective(h, &P, &J);   // A_bar = 2 w FIELD_N
    if (rc) return rc;
    CK(h, cudaMemsetAsync(P.Sb, 0, arr, h->st));
    CK(h, cudaMemsetAsync(P.Sl, 0, arr, h->st));

    // backward, one checkpoint segment at a time
    for (int seg = L.nck - 1; seg >= 0 && !rc; seg--) {
        const int n0 = seg * L.K, n1 = std::min(n_steps, n0 + L.K);
        if (seg < L.nck - 1) {   // re-run the segment from its checkpoint, recording its stages
            const char* ck = P.ck + (size_t)seg * L.ck_slot();
            gsi::spec_written(h);
            gsi::field_written(h);
            CK(h, cudaMemcpyAsync(h->A, ck, arr, cudaMemcpyDeviceToDevice, h->st));
            CK(h, cudaMemcpyAsync(h->S, ck + arr, arr, cudaMemcpyDeviceToDevice, h->st));
            if (ck_pairs[seg]) {
                CK(h, cudaMemcpyAsync(spc, ck + 2 * arr, spb, cudaMemcpyDeviceToDevice, h->st));
                CK(h, cudaMemcpyAsync(spl, ck + 2 * arr + spb, spb, cudaMemcpyDeviceToDevice, h->st));
                h->s_compact = true;
            }
            for (int m = n0; m < n1 && !rc; m++) {
                const GsTape tp = tape_of(L, P.tape, m - n0);
                rc = gsi::nl_stages(h, dz_rk[m], h->p.nonlinear ? &tp : nullptr);
                if (!rc && m + 1 < n1) rc = gsi::lstep(h, dz_lin[m]);
            }
        }
        for (int m = n1 - 1; m >= n0 && !rc; m--) rc = adjoint_step(h, P, tape_of(L, P.tape, m - n0), dz_rk[m], dz_lin[m]);
    }
    if (rc) return rc;
    // BIGBUFFER2_0 = QDHT(FIELD_0)
    rc = run_qdht_t(h, P.Sb, P.Fb);
    if (rc) return rc;
    if (h->fp64) CK(h, launch_cadd<double>((double2*)P.Ab, (const double2*)P.Fb, L.nel, h->st, &h->launches));
    else CK(h, launch_cadd<float>((float2*)P.Ab, (const float2*)P.Fb, L.nel, h->st, &h->launches));
    rc = read_err(h);
    if (rc) return rc;
    if (objective_out) *objective_out = J;
    return gsi::permute_out(h, P.Ab, grad_field);
}

int gs_adjoint_stride(gs_handle* h, int* stride) {
    if (!h || !stride) return GS_ERR_ARG;
    *stride = h->adj_stride;
    return GS_OK;
}

int gs_adjoint_step(gs_handle* h, double dz_rk, double dz_lin, double* field_bar, double* spec_bar) {
    if (!h || !field_bar || !spec_bar) return GS_ERR_ARG;
    if (!(dz_rk > 0) || !(dz_lin > 0)) return gsi::fail(h, GS_ERR_ARG, "step sizes must be > 0");
    if (!h->field_ok) return gsi::fail(h, GS_ERR_STATE, "field not set");
    int rc = check_adjoint_supported(h);
    if (rc) return rc;
    CK(h, cudaSetDevice(h->p.device));
    AdjLayout L;
    L.nel = (size_t)h->nr * h->nt;
    L.nr = h->nr;
    L.esz = h->esz;
    L.rsz = h->esz / 2;
    L.K = 1;
    L.nck = 0;
    AdjPtrs P;
    rc = ensure_adj(h, L, &P);
    if (rc) return rc;
    CK(h, cudaMemsetAsync(h->err_dev, 0, 4, h->st));
    const GsTape tp = tape_of(L, P.tape, 0);
    rc = gsi::nl_stages(h, dz_rk, h->p.nonlinear ? &tp : nullptr);
    if (!rc) rc = gsi::lstep(h, dz_lin);
    if (!rc) rc = gsi::permute_in(h, field_bar, P.Ab);
    if (!rc) rc = gsi::permute_in(h, spec_bar, P.Sb);
    if (!rc) CK(h, cudaMemsetAsync(P.Sl, 0, L.nel * L.esz, h->st));
    if (!rc) rc = adjoint_step(h, P, tp, dz_rk, dz_lin);
    if (!rc) rc = read_err(h);
    if (!rc) rc = gsi::permute_out(h, P.Ab, field_bar);
    if (!rc) rc = gsi::permute_out(h, P.Sb, spec_bar);
    return rc;
}
