// gs_handle.h -- the device state behind a gs_handle and the orchestration helpers that
// gs_abi.cu (forward) and gs_adjoint.cu (adjoint) share.  Private to the library.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <string>
#include <vector>

#include "../../include/gs_abi.h"
#include "gs_kernels.h"
#include "gs_qdht_tc.h"

// Per-stage record of the four RK4 stages of one step for the adjoint: E/N (complex),
// rho and Q (real), [n_r][n_t] each, natural time order.
struct GsTape {
    void* e[4];
    void* rho[4];
    void* q[4];
    int* ion[4];   // per row: the stage's row ionizes (0: rho stays 0 and W = dW = 0 along it)
};

struct gs_handle {
    gs_params p{};
    int nr = 0, nt = 0, P = 1, M = 0, logM = 0;
    bool fp64 = true;
    bool fused = false;        // one-CTA rows: the fused front/back kernels per RK4 stage
    bool pair = false;         // rows over two CTAs (P = 2: FP32 32768, FP64 16384), gs_nl_pair.cu
    int nl_threads = 0;        // fused kernels' threads per row (0: default; gs_autotune sets it)
    int shoot_exhaust = 0;     // test hook (GS_TEST_SHOOTING_EXHAUST=1 at gs_create): no early stop
                               // of the carrier-density shooting
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    size_t esz = 16;           // bytes per complex element
    void *A = nullptr, *S = nullptr, *NB = nullptr, *KP = nullptr, *E = nullptr, *U = nullptr;
    void* tw = nullptr;        // twiddles, position-order independent
    void *pf = nullptr, *rm = nullptr, *kerr = nullptr, *rate = nullptr;
    double *omega = nullptr, *ho = nullptr, *kt2 = nullptr, *Cm = nullptr, *m1 = nullptr;
    double2* wavenum = nullptr;
    double2* staging = nullptr;
    int* perm_dev = nullptr;
    int* iperm_dev = nullptr;   // natural index -> position
    int sms = 0;
    unsigned* err_dev = nullptr;
    unsigned long long* max_dev = nullptr;
    std::vector<int> perm;
    gs::QdhtTc* tc = nullptr;  // mixed-precision QDHT (tcgen05)
    bool tables_ok = false, field_ok = false;
    long long launches = 0;
    double qdht_ms = 0;
    int qdht_n = 0;
    bool time_qdht = false, ev_pending = false;
    // gs_nl_timing: events around each fused front / back launch of one NL step (start, mid,
    // end per RK4 stage), folded into the totals after the step's own synchronisation
    bool time_nl = false, nl_ev_pending = false;
    cudaEvent_t nl_ev[8] = {};   // before / after each RK4-stage launch
    double nl_ms = 0;
    bool nl_ev_one = false;   // the pending events bracket one launch of all four stages
    int all_stages = -1;      // fused path: all four stages per launch (1) or one per stage (0)
    int all_stages_thr = -1;  // ... decided for this nl_threads value
    int adj_stride = 0;   // checkpoint stride of the last gs_gradient
    // gs_advance: the device-side z-loop state while its attempts are enqueued (null otherwise:
    // the kernels then take the host's step sizes), ZNET on the device, per-attempt timing events
    gs::DevCtl* ctl = nullptr;
    gs::DevCtl* ctl_dev = nullptr;
    double* znet_dev = nullptr;
    int znet_cap = 0;
    std::vector<cudaEvent_t> adv_ev;
    bool nbc_valid = false;   // the last NL step also wrote NB's window columns compactly (mixed)
    // BIGBUFFER1 in full: gs_nl_step asks for it (nb_full_wanted); propagator()'s paths need only
    // the window columns the linear step reads, and the row kernel then writes those alone
    bool nb_full_wanted = false;
    bool nb_full_current = true;   // NB holds the last NL increment everywhere
    bool s_compact = false;   // BIGBUFFER2's window columns are current only in the plan's compact copy
    bool a_compact = false;   // FIELD is current only as the masked inverse's compact result
    bool a_lazy_ok = true;    // the masked inverse may leave FIELD compact (not in captured graphs)
    bool nl_compact = false;  // the last NL step ran the kernel that reads a compact FIELD
    bool nl_dev_dz = false;   // ... ran fused stage kernels, which take dz / halt from the device
    // gs_step_host: BIGBUFFER2 travels host -> staging on io_st (copy engine) while the first NL
    // attempt runs; spec_in_pending until the handle's stream has waited on io_ev[1] and
    // installed it (spec_in_finish, before anything reads BIGBUFFER2 or the staging buffer)
    cudaStream_t io_st = nullptr;
    cudaEvent_t io_ev[2] = {};
    bool spec_in_pending = false;
    // FP64 QDHT: the spectral window's columns (padded to 64 with -1) and the positions outside
    int *win64 = nullptr, *zpos64 = nullptr;
    int nwin64 = 0, nz64 = 0;
    int nl_stages_timed = 0, nl_launches_timed = 0;
    double* dump_dev = nullptr;   // 3 n_r + 2 n_t doubles of reduction output, r weights
    void* twb = nullptr;          // per-stage base twiddles of the M-point row FFTs (tw_base_offset)
    int* row_ion = nullptr;       // [n_r] fused NL kernels: row ionizes in the current RK4 stage
    void* th = nullptr;           // gas build: third-harmonic factors th_coeff exp(j phi_t), [n_t]
    std::vector<double> ap_z;      // apertures not yet applied, reference order (last applied first)
    std::vector<int> ap_row0;      // first row outside each aperture's radius
    std::string err;
    // adjoint (gs_adjoint.cu)
    double* m1inv = nullptr;                   // 1/m1: the transposed QDHT (FP64 path)
    std::vector<double> c_host, m1inv_host;    // mixed: C and 1/m1, to build the transposed matrix
    gs::QdhtTc* tcT = nullptr;                 // mixed transposed QDHT (tcgen05)
    void* adj = nullptr;                       // one allocation: adjoint buffers, checkpoints, tape
    size_t adj_bytes = 0;
    double* adj_w = nullptr;                   // objective weights (position order) + partial sums
    size_t adj_w_bytes = 0;
    // energy / photon number (gs_state.cu): radial weights of the average spectrum, the reduction's
    // partial sums, the optional photon-number check of gs_step and its state
    double* en_dev = nullptr;                  // [n_r] weights, then partial sums and the two results
    double en_scale = 0;                       // R_MAX^2 / 2
    bool en_weights = false;
    double en_tol = 0;                         // 0: no check (the reference's controller alone)
    double en_prev = 0;                        // photon number of FIELD after the last accepted step (0: unknown)
    double en_last = 0;                        // |N1 / N0 - 1| of the last accepted step
    long long en_rejects = 0;
    void* en_save = nullptr;                   // BIGBUFFER2 before the linear step, for a rejected one
    size_t en_save_bytes = 0;
};

namespace gsi {
int fail(gs_handle* h, int code, const std::string& msg);
int cuda_fail(gs_handle* h, cudaError_t e, const char* where);
// QDHT of device array X -> Y (gs::QDHT_PLAIN / _LSTEP / _MASKED)
// flags: the tensor-core plan's QTC_* flags (gs_qdht_tc.h; 0 for the FP64 path)
int run_qdht(gs_handle* h, int mode, const void* X, void* Y, double dz, int flags = 0);
// BIGBUFFER2 kept compact by the mixed plan between steps (window columns): spec_sync writes
// them back into S before S is read outside the steps; spec_written marks S as rewritten
// (the copy is taken again at the next step); spec_prepare takes the copy now (before a
// CUDA-graph capture of steps, which must not contain it)
int spec_sync(gs_handle* h);
void spec_written(gs_handle* h);
int spec_prepare(gs_handle* h);
int spec_in_finish(gs_handle* h);
// gs_advance's test: the handle's attempts can run with the step controller on the device
bool advance_on_device(const gs_handle* h);
// FIELD left compact by the masked inverse (the next NL step reads it so): field_sync expands
// it into A before A is read by anything else; field_written marks A as rewritten
int field_sync(gs_handle* h);
void field_written(gs_handle* h);
// calculate_NLstep's four RK4 stages: NB = RK4 increment of A (no host sync); with a tape
// the stages are recorded (fused rows only)
int nl_stages(gs_handle* h, double dz, const GsTape* tape);
// QDHT(NB) with the linear step into S, then A = QDHT(window S) (no host sync)
int lstep(gs_handle* h, double dz);
int permute_in(gs_handle* h, const double* host, void* dst);
// an NVTX range over a scope (named phases in Nsight timelines; a no-op without a tool attached)
struct Range {
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range&) = delete;
    Range& operator=(const Range&) = delete;
};
// ionization levels of the rate table (the gas build's IONIZATION_LEVEL_N; 1 otherwise)
inline int ion_levels(const gs_handle* h) { return (h->p.gas && h->p.ion_levels > 1) ? h->p.ion_levels : 1; }
int permute_out(gs_handle* h, const void* src, double* host);
template <typename Rl> gs::PlasmaArgs<Rl> plasma_args(gs_handle* h, bool raman, bool raman_scan);
// the Raman recurrence applies (oscillator parameters known, Kerr on)
bool raman_scan_on(const gs_handle* h);
// the handle's NL step runs kernels that take dz and the stop flag from the device (the fused
// stage kernels, the row kernel of 16384 points, the paired kernels): known from its parameters
// alone, before any step (nl_step_impl sets nl_dev_dz from the same test)
bool nl_takes_device_dz(const gs_handle* h);
// position -> omega index of the device FFT of rows N = P M (M = 2^logM per CTA)
std::vector<int> position_map(int N, int P, int M, int logM);
// the linear step with the photon-number check of gs_set_energy_tolerance (gs_state.cu): repeated
// with half the step while |N1 / N0 - 1| exceeds the tolerance; dz_inout the step taken
int lstep_checked(gs_handle* h, double* dz_inout, double dz_min);
}  // namespace gsi

#define CK(h, expr)                                                    \
    do {                                                               \
        cudaError_t _e = (expr);                                       \
        if (_e != cudaSuccess) return gsi::cuda_fail((h), _e, #expr);  \
    } while (0)
