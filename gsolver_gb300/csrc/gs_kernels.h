// gs_kernels.h -- argument blocks and launchers shared between the orchestration
// (gs_abi.cu) and the kernel translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace gs {

template <typename Rl> struct Vec2;
template <> struct Vec2<double> { using T = double2; };
template <> struct Vec2<float> { using T = float2; };

template <typename Rl> struct FftArgs {
    int N, M, P, logM, rows;                 // rows of length N = P*M
    const typename Vec2<Rl>::T* tw;          // exp(-2 pi i j / N), j < N
    int spre;                                // spectral-side load op (inverse)
    Rl cdz;                                  // stage coefficient c*dz (SPRE_STAGE), row precision
    const typename Vec2<Rl>::T* kp;          // previous RK4 stage (SPRE_STAGE)
    int track_max;                           // max |input|^2 -> max_out
    unsigned long long* max_out;
    int tpost;                               // time-side store op (inverse)
    const typename Vec2<Rl>::T* e;           // time-domain field (TPOST_DIVN_MULE)
    int threads;                             // fused kernels: threads per row (0: N/16, capped)
    const typename Vec2<Rl>::T* twb;         // per-stage base twiddles (tw_base_offset) or null
    int ahead;                               // fused kernels: rows resident at once; each CTA
                                             // prefetches into L2 the inputs of row + ahead
    int all_stages;                          // fused stage kernel: all four RK4 stages per launch
    double dzs;                              // ... with this step size (c dz per stage inside)
    // steps controlled on the device (gs_advance, nl_row16k_kernel): the step size is *dz_dev
    // instead of dzs, the launch does nothing while *halt != 0, and FIELD is read compactly
    // (SpecArgs::ac) only while *ac_on != 0
    const double* dz_dev;
    const int* halt;
    const int* ac_on;
    double c_stage;   // ... the stage's c (0, 1/2, 1/2, 1) where a kernel forms c dz from *dz_dev
};

template <typename Rl> struct PlasmaArgs {
    int N;
    const typename Vec2<Rl>::T* e;
    typename Vec2<Rl>::T *u1, *u2, *u3;
    const Rl* rate;
    unsigned* err;
    int raman;        // 1: U3 = |E|^2 for the FFT convolution; 0: U3 = |E|^2 E (Raman off)
    int raman_scan;   // 1: U3 = Q E with Q from the one-pole recurrence below
    int density_only; // 1: stop after the recurrence, rho left in U2.x (the plasma dumps)
    int shoot_exhaust; // test hook: the carrier-density shooting ignores its stopping test and runs
                       // its full bound of iterations (one more than the chunks), which reproduces
                       // the sequential recurrence exactly
    double tstep_scaled, neutral_density, rho0, ionization_potential, ponderomotive;
    double avalanche_cs, recombination_tau;
    // Raman oscillator h_k = fRM Im(a^k), a = exp(dt (-1/tau + i Omega)); circular wrap a^N
    double a_re, a_im, aN_re, aN_im, fRM, one_minus_fR, dt_over_tau, dt_omega;
    // optional record of the stage for the adjoint (fused kernel only): E/N, rho, Q per sample
    typename Vec2<Rl>::T* tape_e;
    Rl *tape_rho, *tape_q;
    size_t tape_stride;   // all four stages per launch: bytes from stage s's tape arrays and row
                          // flags to stage s + 1's
    // gas build: single-level PPT ionization with neutral depletion (no avalanche, no
    // recombination) and, when th is set, the third-harmonic source th[t] E_t^3 added to the
    // Kerr source (th[t] = (KERR_TH/KERR) exp(j phi_t), natural time order)
    int gas;
    const typename Vec2<Rl>::T* th;
    // several ionization levels (the gas build's MULTI_LEVEL_IONIZATION, ionization.cpp:45-84):
    // rate holds [levels][8192] rows, pot the levels' potentials (scaled as ionization_potential)
    int levels;
    double pot[8];
    // fused front kernel: per row, whether any sample ionizes (some W_t > 0) or rho starts
    // above 0; where not, the density stays exactly 0, loss and rho E are 0 and are not written
    int* row_ion;
    // the scalars above in the rows' precision, converted once on the host (plasma_args):
    // converting a double on the device runs on the FP64 pipe, which is slow on this GPU
    struct Consts {
        Rl ND, invND, tstep, U, Pc, AV, invTAU, rho0, a_re, a_im, oma_re, oma_im, fRM, omf;
        Rl pot[8];
    } k;
};

// fill PlasmaArgs::k from the double fields (host; call after setting them)
template <typename Rl> inline void plasma_consts(PlasmaArgs<Rl>& pa) {
    pa.k.ND = (Rl)pa.neutral_density;
    pa.k.invND = (Rl)1 / pa.k.ND;
    pa.k.tstep = (Rl)pa.tstep_scaled;
    pa.k.U = (Rl)pa.ionization_potential;
    pa.k.Pc = (Rl)pa.ponderomotive;
    pa.k.AV = (Rl)pa.avalanche_cs;
    pa.k.invTAU = (Rl)1 / (Rl)pa.recombination_tau;
    pa.k.rho0 = (Rl)pa.rho0;
    pa.k.a_re = (Rl)pa.a_re;
    pa.k.a_im = (Rl)pa.a_im;
    pa.k.oma_re = (Rl)(1.0 - pa.aN_re);
    pa.k.oma_im = (Rl)(-pa.aN_im);
    pa.k.fRM = (Rl)pa.fRM;
    pa.k.omf = (Rl)pa.one_minus_fR;
    for (int n = 0; n < 8; n++) pa.k.pot[n] = (Rl)pa.pot[n];
}

// ---- adjoint of one RK4 stage's NL response (gs_nl_vjp.cu), rows that fit one CTA
template <typename Rl> struct VjpArgs {
    int N, logM;
    const typename Vec2<Rl>::T* tw;
    const typename Vec2<Rl>::T* kb;       // cotangent of the stage's N (spectral), times kb_scale
    double kb_scale;
    const typename Vec2<Rl>::T* tape_e;   // the stage's E/N, rho, Q (natural time order)
    const Rl *tape_rho, *tape_q;
    const int* tape_ion;                  // per row: the stage's row ionizes (0: loss, plasma and
                                          // density terms of the adjoint are exactly 0), or null
    const typename Vec2<Rl>::T* pf;       // PLASMA_FUNC (position order)
    const Rl* kerr;                       // KERR_PROFILE (position order)
    const Rl* rate;                       // IONIZATION_RATE_LN
    typename Vec2<Rl>::T* ebar;           // scratch [rows][N]
    typename Vec2<Rl>::T* ab;             // cotangent of FIELD: = or += (dN/dY)^H kb
    int ab_add;
    const typename Vec2<Rl>::T* rbar;     // next stage's cotangent kb_out = cR rbar + cdz ybar
    typename Vec2<Rl>::T* kb_out;         // may be kb itself, or null
    double cR, cdz;
    int kerr_on, raman_scan;
    double tstep_scaled, neutral_density, ionization_potential, ponderomotive, avalanche_cs, recombination_tau;
    double a_re, a_im, aN_re, aN_im, fRM, one_minus_fR;
    int threads;                          // threads per row (0 or not valid: N/16, capped)
    const typename Vec2<Rl>::T* twb;      // per-stage base twiddles (tw_base_offset) or null
};
template <typename Rl> bool nl_vjp_supported(int N);
template <typename Rl> cudaError_t nl_vjp_setup(int N);
template <typename Rl> cudaError_t launch_nl_vjp(const VjpArgs<Rl>& v, int rows, cudaStream_t st, long long* nl);
// J partial sums of w |A|^2 per block and A_bar = 2 w A; then one block sums the partials
template <typename Rl>
cudaError_t launch_adj_seed(const typename Vec2<Rl>::T* A, const double* w, typename Vec2<Rl>::T* ab, size_t n,
                            double* partial, int nblocks, double* out, cudaStream_t st, long long* nl);
// y += x over n complex elements
template <typename Rl>
cudaError_t launch_cadd(typename Vec2<Rl>::T* y, const typename Vec2<Rl>::T* x, size_t n, cudaStream_t st,
                        long long* nl);

template <typename Rl> struct SpecArgs {
    int N, rows;
    typename Vec2<Rl>::T *u1, *u2, *u3;
    const typename Vec2<Rl>::T *pf, *rm;
    const Rl* kerr;
    int raman, kerr_on, stage;
    int fuse_plasma;   // spec2 also adds PLASMA_FUNC * FFT(rho E) (spec1 skipped)
    typename Vec2<Rl>::T *nb, *kp;
    unsigned long long* max_out;
    const int* row_ion;   // fused back kernel: rows flagged 0 have only the Kerr source (or none)
    // the fused stage kernel: k of stages 0..2, each in its own array (k of stage s is written
    // to kst[s]; stage 3 forms the RK4 sum from them and writes nb, which may be kst[2])
    typename Vec2<Rl>::T* kst[3];
    // optional (FP32): stage 3 also writes the RK4 sum of the spectral window's positions into
    // this compact [rows][ncw] array, nbc[row][cinv[p]] (cinv[p] >= 0), the linear-step input
    float* nbc;
    const int* cinv;
    int ncw;
    // != nullptr: FIELD (the stage input A) as the masked inverse's compact [rows][ncw] array
    // at the same columns, zero outside the window; read by the four-stage kernel of
    // 16384-point FP32 rows at 1024 threads (nl_stage_reads_compact) instead of A.  cmap[c]:
    // the real column of compact column c (-1 in the padding)
    const float* ac;
    const int* cmap;
};

template <typename Rl>
cudaError_t launch_fft(int sign, const typename Vec2<Rl>::T* in, typename Vec2<Rl>::T* out, FftArgs<Rl> a,
                       cudaStream_t st, long long* nlaunch);
template <typename Rl> cudaError_t fft_set_smem(int M, int N);
template <typename Rl> cudaError_t launch_plasma(PlasmaArgs<Rl> a, int rows, cudaStream_t st, long long* nlaunch);
template <typename Rl> cudaError_t launch_spec1(SpecArgs<Rl> a, cudaStream_t st, long long* nlaunch);
template <typename Rl> cudaError_t launch_spec2(SpecArgs<Rl> a, cudaStream_t st, long long* nlaunch);
template <typename Rl>
cudaError_t launch_zero_nl(const typename Vec2<Rl>::T* A, typename Vec2<Rl>::T* nb, size_t total,
                           unsigned long long* max_out, cudaStream_t st, long long* nlaunch);
template <typename Rl>
cudaError_t launch_permute(int dir, const void* src, void* dst, const int* perm, int N, size_t total,
                           cudaStream_t st, long long* nlaunch);
// the same with the FP64 side a device-mapped pinned host buffer (iperm: natural -> position);
// lo (optional, position order like the device side): dir > 0 writes the remainders of the FP64
// values after rounding (the low parts of double-float values), dir < 0 adds them to the output
template <typename Rl>
cudaError_t launch_permute_host(int dir, const void* src, void* dst, const int* iperm, int N, size_t total, int sms,
                                cudaStream_t st, long long* nlaunch, void* lo = nullptr);

// ---- fused RK4 stage (gs_nl_fused.cu), rows that fit one CTA's shared memory
template <typename Rl> bool nl_fused_supported(int N);
// a thread count the fused kernels accept for rows of N (multiple of 32, divides N, fits)
template <typename Rl> bool nl_fused_threads_ok(int N, int threads);
template <typename Rl> int nl_fused_default_threads(int N);
template <typename Rl> cudaError_t nl_fused_setup(int N);
// one RK4 stage per launch: f the stage input (cdz, kp = k of the previous stage), a the
// plasma / Raman parameters and the optional tape, s the spectral combination (kp = k of this
// stage, written over the previous one row by row; nb the RK4 sum; u1..u3 scratch rows)
template <typename Rl>
cudaError_t launch_nl_stage(FftArgs<Rl> f, PlasmaArgs<Rl> a, const typename Vec2<Rl>::T* A, SpecArgs<Rl> s,
                            int rows, cudaStream_t st, long long* nl);
// whether one launch of all four stages (f.all_stages) suits a grid of this many rows
template <typename Rl> bool nl_stage_all_preferred(int N, int threads, int rows);
// whether the four-stage launch of this shape can read FIELD compactly (SpecArgs::ac)
template <typename Rl> bool nl_stage_reads_compact(int N, int threads);
// ---- the four RK4 stages of 16384-point FP32 rows, 1024 threads each (gs_nl_row16k.cu):
// the four-stage launch of that shape without a stage record
bool nl_row16k_applies(int N, int threads);
cudaError_t nl_row16k_setup();
cudaError_t launch_nl_row16k(FftArgs<float> f, PlasmaArgs<float> a, const float2* A, SpecArgs<float> s, int rows,
                             int ahead, cudaStream_t st, long long* nl);
int nl_row16k_resident(int* ctas);   // CTAs resident on the device at once (cudaError_t)

// ---- one RK4 stage over two CTAs per row (gs_nl_pair.cu): rows of N = 2H stored in the
// P = 2 position order, FP32 N = 32768 / FP64 N = 16384
template <typename Rl> bool nl_pair_supported(int N);
template <typename Rl> cudaError_t nl_pair_setup(int N);
template <typename Rl>
cudaError_t launch_nl_pair_front(FftArgs<Rl> f, PlasmaArgs<Rl> a, const typename Vec2<Rl>::T* A, int rows,
                                 cudaStream_t st, long long* nl);
template <typename Rl>
cudaError_t launch_nl_pair_back(FftArgs<Rl> f, SpecArgs<Rl> s, int rows, cudaStream_t st, long long* nl);

// ---- dump reductions (gs_dumps.cu)
template <typename Rl>
cudaError_t launch_row_intensity(const typename Vec2<Rl>::T* E, int rows, int N, double tstep, double* maxI,
                                 double* flux, cudaStream_t st, long long* nl);
template <typename Rl>
cudaError_t launch_row_max_re(const typename Vec2<Rl>::T* U, int rows, int N, double* out, cudaStream_t st,
                              long long* nl);
template <typename Rl>
cudaError_t launch_spectrum(const typename Vec2<Rl>::T* F, int nr, int N, const double* w, double scale,
                            double* out, cudaStream_t st, long long* nl);

// ---- QDHT: Y[i][c] = m1_i * sum_j C(i,j) X[j][c] / m1_j over the 2*n_t real columns
struct LstepArgs {
    double dz;
    const double* omega;      // position order
    const double2* wavenum;   // position order
    const double* ho;         // position order
    const double* kt2;        // [n_r]
    double omega_min, omega_max;
    // steps controlled on the device (gs_advance, mixed wide plans): the linear step's size is
    // *dz_dev instead of dz, and the transform does nothing while *run == 0 (a rejected attempt)
    const double* dz_dev;
    const int* run;
};

// the error word's bit for a failed index test of a GS_CHECK build (gs_internal.cuh in_bounds)
constexpr unsigned GS_ERRBIT_BOUNDS = 1u << 16;
constexpr const char* GS_BOUNDS_MSG = "index out of bounds (GS_CHECK build)";

// The z-loop's state on the device (gs_advance): propagator()'s step-size controller
// (propagator.cu:139-164) and the z-loop's bookkeeping (solver_main.cpp:202-225) run in a
// one-thread kernel between each attempt's NL step and its linear step.
struct DevCtl {
    double z;            // CURRENT_Z
    double zstep;        // ZSTEP: the next attempt's NL step size; after it, the new proposal
    double dz_lin;       // the accepted attempt's linear-step size
    unsigned step_n;     // STEP_N
    int n_z;             // ZNET index of the next dump point
    int calls, max_calls;   // accepted propagator() calls so far / at most
    int stop;            // 0 running, 1 CURRENT_Z reached ZNET[n_z], 2 max_calls, 3 collapse, 4 NL error
    int accept;          // the attempt in flight is accepted: its linear step runs
    int field_compact;   // FIELD is the masked inverse's compact result
    unsigned err;        // the NL error bits that stopped the loop
    int iter;            // attempts of the current batch that ran
    int acc_log[64];     // per attempt of the batch: accepted (its linear step ran)
};
cudaError_t launch_step_ctl(DevCtl* c, const double* znet, unsigned long long* max_dev, unsigned* err, double tol,
                            int slot, cudaStream_t st, long long* nl);
enum { QDHT_PLAIN = 0, QDHT_LSTEP = 1, QDHT_MASKED = 2 };
// cmap[nc] / zpos[nz]: the spectral window's columns (padded to 64 with -1) and the positions
// outside it; the linear-step and masked transforms then run on the window only (null: all)
cudaError_t launch_qdht64(int mode, const double* C, const double* m1, const double* X, double* Y, int nr,
                          int ncols, const LstepArgs& L, cudaStream_t st, long long* nlaunch, const int* cmap = nullptr,
                          int nc = 0, const int* zpos = nullptr, int nz = 0);
cudaError_t qdht_set_sqrt_ho(const double* coeffs20);
// adjoint of the linear step (gs_qdht64.cu): fb = cotangent of FIELD (k,omega) after the
// step, sb of BIGBUFFER2 (in: after, out: before), b1b out: of BIGBUFFER1 (k,omega)
template <typename Rl>
cudaError_t launch_lstep_adj(const typename Vec2<Rl>::T* fb, typename Vec2<Rl>::T* sb, typename Vec2<Rl>::T* b1b,
                             int nr, int nt, const LstepArgs& L, cudaStream_t st, long long* nlaunch);

}  // namespace gs
