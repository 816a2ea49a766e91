// gs_batch.cu -- many independent pulses advanced together, one CUDA graph launch per z-step
// (no counterpart in the reference, which runs one pulse per MPI job).
//
// Every pulse keeps its own handle (grid, tables, state) and stream.  A z-step of the batch
// is every pulse's propagator() work -- the four RK4 stages and the QDHT pair with the
// linear step -- issued on the pulses' own streams between a fork and a join on the
// batch's stream, so pulses of different grids run concurrently and fill the GPU together.
// The whole z-step is captured once into a CUDA graph and replayed, so the host issues one
// launch per z-step instead of ~10 per pulse.  Step sizes are fixed per pulse (the graph
// holds them; a new set of sizes captures a new graph).  gs_batch_advance runs every pulse's
// adaptive controller on the device instead: one graph launch per attempt of all pulses.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "gs_handle.h"

struct gs_batch {
    std::vector<gs_handle*> h;
    int device = 0;
    cudaStream_t st = nullptr;        // fork / join stream, the graph's launch stream
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<double> graph_dz;     // the step sizes captured in `exec`
    long long launches = 0;           // kernels issued (graph replays count their kernels)
    long long kernels_per_step = 0;
    std::string err;
};

static std::string g_batch_err;

static int bfail(gs_batch* b, int code, const std::string& m) {
    if (b) b->err = m; else g_batch_err = m;
    return code;
}

#define BCK(b, expr)                                                                            \
    do {                                                                                        \
        cudaError_t _e = (expr);                                                                \
        if (_e != cudaSuccess) return bfail((b), GS_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    } while (0)

static void batch_free_graph(gs_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_dz.clear();
}

const char* gs_batch_last_error(const gs_batch* b) { return b ? b->err.c_str() : g_batch_err.c_str(); }

int gs_batch_create(int n, gs_handle* const* pulses, gs_batch** out) {
    if (!out || n < 1 || !pulses) return bfail(nullptr, GS_ERR_ARG, "gs_batch_create: null argument or n < 1");
    *out = nullptr;
    const int dev = pulses[0] ? pulses[0]->p.device : 0;
    for (int i = 0; i < n; i++) {
        if (!pulses[i]) return bfail(nullptr, GS_ERR_ARG, "gs_batch_create: null pulse handle");
        if (pulses[i]->p.device != dev) return bfail(nullptr, GS_ERR_ARG, "gs_batch_create: pulses on different devices");
        for (int j = 0; j < i; j++)
            if (pulses[j] == pulses[i]) return bfail(nullptr, GS_ERR_ARG, "gs_batch_create: a pulse appears twice");
    }
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) return bfail(nullptr, GS_ERR_CUDA, cudaGetErrorString(e));
    gs_batch* b = new gs_batch();
    b->h.assign(pulses, pulses + n);
    b->device = dev;
    b->join.assign(n, nullptr);
    bool ok = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; i < n && ok; i++) ok = cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        gs_batch_destroy(b);
        return bfail(nullptr, GS_ERR_CUDA, "gs_batch_create: stream/event creation failed");
    }
    *out = b;
    return GS_OK;
}

int gs_batch_destroy(gs_batch* b) {
    if (!b) return GS_OK;
    cudaSetDevice(b->device);
    batch_free_graph(b);
    for (cudaEvent_t e : b->join)
        if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return GS_OK;
}

void* gs_batch_stream(const gs_batch* b) { return b ? (void*)b->st : nullptr; }

long long gs_batch_launch_count(const gs_batch* b) { return b ? b->launches : 0; }

// one z-step of every pulse between a fork and a join on b->st (captured or not)
static int batch_enqueue_step(gs_batch* b, const double* dz, long long* nk) {
    BCK(b, cudaEventRecord(b->fork, b->st));
    for (size_t i = 0; i < b->h.size(); i++) {
        gs_handle* h = b->h[i];
        const long long l0 = h->launches;
        BCK(b, cudaStreamWaitEvent(h->st, b->fork, 0));
        int rc = gsi::nl_stages(h, dz[i], nullptr);
        if (!rc) rc = gsi::lstep(h, dz[i]);
        if (rc) return bfail(b, rc, "pulse " + std::to_string(i) + ": " + h->err);
        BCK(b, cudaEventRecord(b->join[i], h->st));
        BCK(b, cudaStreamWaitEvent(b->st, b->join[i], 0));
        *nk += h->launches - l0;
    }
    return GS_OK;
}

int gs_batch_step(gs_batch* b, int n_steps, const double* dz, int use_graph) {
    if (!b || !dz || n_steps < 0) return bfail(b, GS_ERR_ARG, "gs_batch_step: null argument or n_steps < 0");
    for (size_t i = 0; i < b->h.size(); i++) {
        gs_handle* h = b->h[i];
        if (!h->tables_ok || !h->field_ok) return bfail(b, GS_ERR_STATE, "pulse " + std::to_string(i) + ": tables / field not set");
        if (!(dz[i] > 0)) return bfail(b, GS_ERR_ARG, "gs_batch_step: step sizes must be > 0");
        if (h->time_qdht) return bfail(b, GS_ERR_STATE, "pulse " + std::to_string(i) + ": QDHT timing is on");
    }
    BCK(b, cudaSetDevice(b->device));
    for (gs_handle* h : b->h) BCK(b, cudaMemsetAsync(h->err_dev, 0, 4, h->st));
    // the compact copies of BIGBUFFER2 are taken now, outside any graph capture
    // and FIELD is kept expanded (a captured step must not depend on the state it starts from)
    for (size_t i = 0; i < b->h.size(); i++) {
        b->h[i]->a_lazy_ok = false;
        if (gsi::spec_prepare(b->h[i]) || gsi::field_sync(b->h[i]))
            return bfail(b, GS_ERR_CUDA, "pulse " + std::to_string(i) + ": " + b->h[i]->err);
    }
    // the pulses' streams may hold earlier work: the batch stream waits for all of it
    for (size_t i = 0; i < b->h.size(); i++) {
        BCK(b, cudaEventRecord(b->join[i], b->h[i]->st));
        BCK(b, cudaStreamWaitEvent(b->st, b->join[i], 0));
    }
    if (use_graph) {
        const bool same = b->exec && b->graph_dz.size() == b->h.size() &&
                          std::equal(b->graph_dz.begin(), b->graph_dz.end(), dz);
        if (!same) {
            batch_free_graph(b);
            long long nk = 0;
            BCK(b, cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
            const int rc = batch_enqueue_step(b, dz, &nk);
            cudaGraph_t g = nullptr;
            const cudaError_t ee = cudaStreamEndCapture(b->st, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (ee != cudaSuccess) return bfail(b, GS_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(ee));
            b->graph = g;
            BCK(b, cudaGraphInstantiate(&b->exec, b->graph, 0));
            b->graph_dz.assign(dz, dz + b->h.size());
            b->kernels_per_step = nk;   // kernel nodes of one replay
        }
        for (int s = 0; s < n_steps; s++) {
            BCK(b, cudaGraphLaunch(b->exec, b->st));
            b->launches += b->kernels_per_step;
        }
    } else {
        for (int s = 0; s < n_steps; s++) {
            long long nk = 0;
            const int rc = batch_enqueue_step(b, dz, &nk);
            if (rc) return rc;
            b->launches += nk;
        }
    }
    BCK(b, cudaStreamSynchronize(b->st));
    for (size_t i = 0; i < b->h.size(); i++) {
        gs_handle* h = b->h[i];
        unsigned err = 0;
        BCK(b, cudaMemcpy(&err, h->err_dev, 4, cudaMemcpyDeviceToHost));
        if (h->tc) {
            std::string m;
            if (gs::qdht_tc_check(h->tc, &m)) return bfail(b, GS_ERR_CUDA, "pulse " + std::to_string(i) + ": " + m);
        }
        if (err & gs::GS_ERRBIT_BOUNDS) return bfail(b, GS_ERR_CUDA, "pulse " + std::to_string(i) + ": " + gs::GS_BOUNDS_MSG);
        if (err & 1u) return bfail(b, GS_ERR_BLAST, "pulse " + std::to_string(i) + ": " + gs_status_string(GS_ERR_BLAST));
        if (err & 2u) return bfail(b, GS_ERR_NAN, "pulse " + std::to_string(i) + ": " + gs_status_string(GS_ERR_NAN));
    }
    return GS_OK;
}

// gs_advance for every pulse at once.  Each pulse gets the device z-loop state of gs_advance
// (DevCtl, its ZNET on the device); one attempt of every pulse -- NL step, controller kernel,
// linear step, each reading the attempt's step size and decision from the device -- is
// captured between a fork and a join and replayed, one graph launch per attempt; a pulse
// whose loop stopped (ZNET point, call budget, collapse, NL error) skips its kernels.  The
// host reads the pulses' states every REPLAYS launches.  FIELD is kept expanded (the masked
// inverse not lazy), so the captured attempt is the same whatever state it starts from.
int gs_batch_advance(gs_batch* b, const double* const* znet, const int* nz, const int* n_z, double* current_z,
                     double* zstep, unsigned* step_n, int max_calls, int* calls_done, int* reached) {
    if (!b || !znet || !nz || !n_z || !current_z || !zstep || !step_n || max_calls < 0)
        return bfail(b, GS_ERR_ARG, "gs_batch_advance: null argument or max_calls < 0");
    const size_t n = b->h.size();
    for (size_t i = 0; i < n; i++) {
        gs_handle* h = b->h[i];
        const std::string who = "pulse " + std::to_string(i) + ": ";
        if (!znet[i] || nz[i] < 2 || n_z[i] < 1 || n_z[i] >= nz[i])
            return bfail(b, GS_ERR_ARG, who + "bad ZNET index or size");
        if (!h->tables_ok || !h->field_ok) return bfail(b, GS_ERR_STATE, who + "tables / field not set");
        if (h->time_qdht || h->time_nl) return bfail(b, GS_ERR_STATE, who + "kernel timing is on");
        if (calls_done) calls_done[i] = 0;
        if (reached) reached[i] = 0;
    }
    for (size_t i = 0; i < n; i++) {   // every pulse can run on the device, checked before any work
        const gs_handle* h = b->h[i];
        if (h->fp64 || !h->tc || !gs::qdht_tc_has_compact(h->tc) || h->en_tol > 0 || !h->ap_z.empty() ||
            !gsi::nl_takes_device_dz(h))
            return bfail(b, GS_ERR_UNSUPPORTED, "pulse " + std::to_string(i) +
                                                    ": its attempts need the host (FP64, the staged NL kernels, a "
                                                    "photon-number check or an aperture)");
    }
    BCK(b, cudaSetDevice(b->device));
    std::vector<int> done(n, 0);
    // as gs_advance: a pulse whose NL path is not known yet takes its first call on the host
    for (size_t i = 0; i < n; i++) {
        gs_handle* h = b->h[i];
        if (gsi::advance_on_device(h) || h->nl_compact || h->nl_dev_dz || max_calls == 0 ||
            current_z[i] >= znet[i][n_z[i]])
            continue;
        double dz = zstep[i];
        unsigned sn = step_n[i];
        const int rc = gs_step(h, current_z[i], znet[i][n_z[i]], znet[i][n_z[i] - 1], &dz, &sn, nullptr, nullptr);
        if (rc) return bfail(b, rc, "pulse " + std::to_string(i) + ": " + h->err);
        step_n[i] = sn + 1;
        current_z[i] += dz;
        zstep[i] = dz;
        done[i] = 1;
    }
    for (size_t i = 0; i < n; i++)
        if (!gsi::advance_on_device(b->h[i]))
            return bfail(b, GS_ERR_UNSUPPORTED, "pulse " + std::to_string(i) +
                                                    ": its attempts need the host (FP64, the staged or paired NL "
                                                    "kernels, a photon-number check or an aperture)");
    // the device z-loops
    struct Restore {   // every pulse back in host mode on every way out
        gs_batch* b;
        ~Restore() {
            for (gs_handle* h : b->h) {
                h->ctl = nullptr;
                h->a_lazy_ok = true;
            }
        }
    } restore{b};
    std::vector<gs::DevCtl> c(n);
    for (size_t i = 0; i < n; i++) {
        gs_handle* h = b->h[i];
        const std::string who = "pulse " + std::to_string(i) + ": ";
        if (h->znet_cap < nz[i]) {
            if (h->znet_dev) cudaFree(h->znet_dev);
            h->znet_dev = nullptr;
            h->znet_cap = 0;
            BCK(b, cudaMalloc(&h->znet_dev, (size_t)nz[i] * sizeof(double)));
            h->znet_cap = nz[i];
        }
        if (!h->ctl_dev) BCK(b, cudaMalloc(&h->ctl_dev, sizeof(gs::DevCtl)));
        BCK(b, cudaMemcpyAsync(h->znet_dev, znet[i], (size_t)nz[i] * sizeof(double), cudaMemcpyHostToDevice, h->st));
        h->a_lazy_ok = false;
        if (gsi::spec_prepare(h) || gsi::field_sync(h)) return bfail(b, GS_ERR_CUDA, who + h->err);
        gs::DevCtl& ci = c[i];
        ci = gs::DevCtl{};
        ci.z = current_z[i];
        ci.zstep = zstep[i];
        ci.step_n = step_n[i];
        ci.n_z = n_z[i];
        ci.max_calls = max_calls - done[i];
        ci.field_compact = 0;
        // a pulse with nothing to do is stopped from the start: its kernels skip
        if (ci.max_calls <= 0) ci.stop = 2;
        if (current_z[i] >= znet[i][n_z[i]]) ci.stop = 1;
        BCK(b, cudaMemcpyAsync(h->ctl_dev, &ci, sizeof(gs::DevCtl), cudaMemcpyHostToDevice, h->st));
        BCK(b, cudaMemsetAsync(h->max_dev, 0, 16, h->st));
        BCK(b, cudaMemsetAsync(h->err_dev, 0, 4, h->st));
        h->ctl = h->ctl_dev;
    }
    for (size_t i = 0; i < n; i++) {   // the batch stream waits for the pulses' set-up
        BCK(b, cudaEventRecord(b->join[i], b->h[i]->st));
        BCK(b, cudaStreamWaitEvent(b->st, b->join[i], 0));
    }
    // one attempt of every pulse, captured
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ex = nullptr;
    long long nk = 0;
    BCK(b, cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    int rc = GS_OK;
    {
        cudaError_t e = cudaEventRecord(b->fork, b->st);
        for (size_t i = 0; i < n && rc == GS_OK && e == cudaSuccess; i++) {
            gs_handle* h = b->h[i];
            const long long l0 = h->launches;
            e = cudaStreamWaitEvent(h->st, b->fork, 0);
            if (e != cudaSuccess) break;
            rc = gsi::nl_stages(h, zstep[i], nullptr);   // the kernels read the device's step size
            if (rc == GS_OK) {
                e = gs::launch_step_ctl(h->ctl_dev, h->znet_dev, h->max_dev, h->err_dev, h->p.max_tolerance, 0, h->st,
                                        &h->launches);
                if (e == cudaSuccess) rc = gsi::lstep(h, zstep[i]);
            }
            if (rc == GS_OK && e == cudaSuccess) e = cudaEventRecord(b->join[i], h->st);
            if (rc == GS_OK && e == cudaSuccess) e = cudaStreamWaitEvent(b->st, b->join[i], 0);
            nk += h->launches - l0;
            if (rc) rc = bfail(b, rc, "pulse " + std::to_string(i) + ": " + h->err);
        }
        const cudaError_t ee = cudaStreamEndCapture(b->st, &g);
        if (rc == GS_OK && e != cudaSuccess) rc = bfail(b, GS_ERR_CUDA, std::string("batch attempt: ") + cudaGetErrorString(e));
        if (rc == GS_OK && ee != cudaSuccess)
            rc = bfail(b, GS_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(ee));
    }
    if (rc == GS_OK && cudaGraphInstantiate(&ex, g, 0) != cudaSuccess)
        rc = bfail(b, GS_ERR_CUDA, "gs_batch_advance: graph instantiation failed");
    constexpr int REPLAYS = 16;
    while (rc == GS_OK) {
        for (int r = 0; r < REPLAYS; r++) {
            if (cudaGraphLaunch(ex, b->st) != cudaSuccess) {
                rc = bfail(b, GS_ERR_CUDA, "gs_batch_advance: graph launch failed");
                break;
            }
            b->launches += nk;
        }
        if (rc) break;
        bool all = true;
        for (size_t i = 0; i < n && rc == GS_OK; i++) {
            if (cudaMemcpyAsync(&c[i], b->h[i]->ctl_dev, sizeof(gs::DevCtl), cudaMemcpyDeviceToHost, b->st) != cudaSuccess)
                rc = bfail(b, GS_ERR_CUDA, "gs_batch_advance: state read failed");
        }
        if (rc == GS_OK && cudaStreamSynchronize(b->st) != cudaSuccess)
            rc = bfail(b, GS_ERR_CUDA, "gs_batch_advance: synchronisation failed");
        for (size_t i = 0; i < n; i++) all = all && c[i].stop != 0;
        if (all) break;
    }
    if (ex) cudaGraphExecDestroy(ex);
    if (g) cudaGraphDestroy(g);
    if (rc) return rc;
    for (size_t i = 0; i < n; i++) {
        gs_handle* h = b->h[i];
        const std::string who = "pulse " + std::to_string(i) + ": ";
        h->a_compact = false;   // every accepted attempt's masked inverse expanded FIELD
        current_z[i] = c[i].z;
        zstep[i] = c[i].zstep;
        step_n[i] = c[i].step_n;
        if (calls_done) calls_done[i] = done[i] + c[i].calls;
        if (reached) reached[i] = c[i].z >= znet[i][n_z[i]] ? 1 : 0;
        std::string m;
        if (gs::qdht_tc_check(h->tc, &m)) return bfail(b, GS_ERR_CUDA, who + m);
        if (c[i].stop == 3) return bfail(b, GS_ERR_COLLAPSE, who + gs_status_string(GS_ERR_COLLAPSE));
        if (c[i].stop == 4) {
            if (c[i].err & gs::GS_ERRBIT_BOUNDS) return bfail(b, GS_ERR_CUDA, who + gs::GS_BOUNDS_MSG);
            if (c[i].err & 1u) return bfail(b, GS_ERR_BLAST, who + gs_status_string(GS_ERR_BLAST));
            return bfail(b, GS_ERR_NAN, who + gs_status_string(GS_ERR_NAN));
        }
    }
    return GS_OK;
}

// Batch-level choice between the default launch shapes and every pulse's own tuned shape
// (gs_autotune, timed alone): concurrent pulses compete for SMs, so a shape that wins alone
// can lose in the batch.  One graph z-step is timed each way from the same state (FIELD and
// BIGBUFFER2 of every pulse are saved in a temporary snapshot and restored), and the faster
// set of shapes is kept.
int gs_batch_autotune(gs_batch* b, const double* dz, double* ms_default, double* ms_tuned, int* chose_tuned) {
    if (!b || !dz) return bfail(b, GS_ERR_ARG, "gs_batch_autotune: null argument");
    BCK(b, cudaSetDevice(b->device));
    const size_t n = b->h.size();
    std::vector<int> tuned(n);
    for (size_t i = 0; i < n; i++) {
        int t = 0;
        const int rc = gs_autotune(b->h[i], &t, nullptr);
        if (rc) return bfail(b, rc, "pulse " + std::to_string(i) + ": " + b->h[i]->err);
        tuned[i] = b->h[i]->nl_threads;
    }
    // snapshot of every pulse's FIELD and BIGBUFFER2 (a temporary allocation: tuning only)
    std::vector<char*> snap(n, nullptr);
    for (size_t i = 0; i < n; i++) {
        gs_handle* h = b->h[i];
        if (cudaMalloc((void**)&snap[i], 2 * (size_t)h->nr * h->nt * h->esz) != cudaSuccess) {
            cudaGetLastError();
            for (char* q : snap)
                if (q) cudaFree(q);
            return bfail(b, GS_ERR_NOMEM, "gs_batch_autotune: no memory for the state snapshot");
        }
    }
    auto save = [&](bool restore) -> int {
        for (size_t i = 0; i < n; i++) {
            gs_handle* h = b->h[i];
            const size_t bytes = (size_t)h->nr * h->nt * h->esz;
            char* st = snap[i];
            if (!restore) {
                if (gsi::field_sync(h)) return bfail(b, GS_ERR_CUDA, "pulse " + std::to_string(i) + ": " + h->err);
                BCK(b, cudaMemcpyAsync(st, h->A, bytes, cudaMemcpyDeviceToDevice, h->st));
                if (gsi::spec_sync(h)) return bfail(b, GS_ERR_CUDA, "pulse " + std::to_string(i) + ": " + h->err);
                BCK(b, cudaMemcpyAsync(st + bytes, h->S, bytes, cudaMemcpyDeviceToDevice, h->st));
            } else {
                BCK(b, cudaMemcpyAsync(h->A, st, bytes, cudaMemcpyDeviceToDevice, h->st));
                BCK(b, cudaMemcpyAsync(h->S, st + bytes, bytes, cudaMemcpyDeviceToDevice, h->st));
                gsi::spec_written(h);
                gsi::field_written(h);
            }
        }
        return GS_OK;
    };
    cudaEvent_t e0, e1;
    BCK(b, cudaEventCreate(&e0));
    BCK(b, cudaEventCreate(&e1));
    double ms[2] = {0, 0};
    int rc = GS_OK;
    for (int pass = 0; pass < 2 && !rc; pass++) {
        for (size_t i = 0; i < n; i++) b->h[i]->nl_threads = pass ? tuned[i] : 0;
        batch_free_graph(b);   // shapes are baked into the graph
        if (!rc && pass == 0) rc = save(false);
        if (!rc) rc = gs_batch_step(b, 1, dz, 1);   // capture + warm-up
        if (!rc) rc = save(true);
        const int reps = 3;
        if (!rc) {
            for (gs_handle* h : b->h) cudaStreamSynchronize(h->st);
            cudaEventRecord(e0, b->st);
            rc = gs_batch_step(b, reps, dz, 1);
            cudaEventRecord(e1, b->st);
            cudaEventSynchronize(e1);
            float t = 0;
            cudaEventElapsedTime(&t, e0, e1);
            ms[pass] = t / reps;
        }
        if (!rc) rc = save(true);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (gs_handle* h : b->h) cudaStreamSynchronize(h->st);
    for (char* q : snap) cudaFree(q);
    if (rc) return rc;
    const bool use_tuned = ms[1] < ms[0];
    for (size_t i = 0; i < n; i++) b->h[i]->nl_threads = use_tuned ? tuned[i] : 0;
    batch_free_graph(b);
    for (gs_handle* h : b->h) BCK(b, cudaStreamSynchronize(h->st));
    if (ms_default) *ms_default = ms[0];
    if (ms_tuned) *ms_tuned = ms[1];
    if (chose_tuned) *chose_tuned = use_tuned ? 1 : 0;
    return GS_OK;
}
