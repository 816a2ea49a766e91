// gs_ctl.cu -- the z-loop advanced on the device (gs_advance).
//
// solver_main.cpp:202-225 calls propagator() (propagator.cu:125-266) until CURRENT_Z reaches the
// next ZNET point; each call tries NL steps until one passes the error test and then takes the
// linear step with the new step size.  Host-driven (gs_step) that is one host round trip per
// attempt.  Here each attempt is an NL launch, then step_ctl_kernel (one thread: the test, the
// new ZSTEP, the collapse and ZNET-clamp rules, the z-loop's STEP_N / CURRENT_Z update), then
// the linear step's transforms, which read the accepted size from device memory and do nothing
// for a rejected attempt; attempts are enqueued back to back and the host synchronises once
// per batch.  Kernels that see the stop flag set (a ZNET point reached, the call budget spent, a
// collapse or an NL error) return at once, so a batch may end with a few empty attempts.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "gs_handle.h"

using namespace gs;

namespace {

__global__ void step_ctl_kernel(DevCtl* c, const double* __restrict__ znet, unsigned long long* maxv,
                                unsigned* err, double tol, int slot) {
    if (c->stop) {
        c->accept = 0;
        return;
    }
    c->iter = slot + 1;
    const double a2 = __longlong_as_double((long long)maxv[0]);
    const double n2 = __longlong_as_double((long long)maxv[1]);
    maxv[0] = 0ull;   // the next attempt's NL maxima start from 0 (as gs_step's memset)
    maxv[1] = 0ull;
    c->accept = 0;
    c->acc_log[slot] = 0;
    const unsigned e = *err;
    if (e) {   // blast or NaN in the NL step: the host maps the bits to its status
        c->err = e;
        c->stop = 4;
        return;
    }
    // propagator.cu:147-164
    const double zs = c->zstep;
    const bool repeat = zs * zs * n2 > tol * tol * a2;
    if (repeat) c->step_n++;
    double znew = 0.5 * tol * sqrt(a2 / n2);
    const double zc = znet[c->n_z], zp = znet[c->n_z - 1];
    if (znew < 1e-10 * (zc - zp) || !(znew > 0)) {
        c->zstep = znew;
        c->stop = 3;
        return;
    }
    const double lim = zc - c->z;
    if (lim < znew) znew = lim;
    c->zstep = znew;
    if (repeat) return;
    c->accept = 1;
    c->acc_log[slot] = 1;
    c->dz_lin = znew;
    c->field_compact = 1;   // the masked inverse leaves FIELD compact
    // the z-loop after propagator(): STEP_N++, CURRENT_Z += ZSTEP, and the dump test at its top
    c->step_n++;
    c->z += znew;
    c->calls++;
    if (c->z >= zc) c->stop = 1;
    else if (c->calls >= c->max_calls) c->stop = 2;
}

// the handle can run its attempts on the device: the NL step is the four-stage kernel of
// 16384-point FP32 rows reading FIELD compactly and the linear step the compact tensor-core
// plan; no photon-number check and no aperture left to apply (both need the host)
bool device_ok(const gs_handle* h) {
    return !h->fp64 && h->tc && h->p.nonlinear && (h->nl_compact || h->nl_dev_dz) && gs::qdht_tc_has_compact(h->tc) &&
           h->en_tol <= 0 && h->ap_z.empty();
}

}  // namespace

bool gsi::advance_on_device(const gs_handle* h) { return device_ok(h); }

namespace gs {
cudaError_t launch_step_ctl(DevCtl* c, const double* znet, unsigned long long* max_dev, unsigned* err, double tol,
                            int slot, cudaStream_t st, long long* nl) {
    step_ctl_kernel<<<1, 1, 0, st>>>(c, znet, max_dev, err, tol, slot);
    (*nl)++;
    return cudaGetLastError();
}
}  // namespace gs

int gs_advance(gs_handle* h, const double* znet, int nz, int n_z, double* current_z, double* zstep,
               unsigned* step_n, int max_calls, int* calls_done, int* reached) {
    if (!h || !znet || !current_z || !zstep || !step_n) return GS_ERR_ARG;
    if (nz < 2 || n_z < 1 || n_z >= nz || max_calls < 0) return gsi::fail(h, GS_ERR_ARG, "gs_advance: bad ZNET index or call count");
    if (!h->tables_ok || !h->field_ok) return gsi::fail(h, GS_ERR_STATE, "tables / field not set");
    CK(h, cudaSetDevice(h->p.device));
    gsi::Range range("gs_advance");
    int done = 0;
    if (calls_done) *calls_done = 0;
    if (reached) *reached = 0;
    double cz = *current_z, dz = *zstep;
    unsigned sn = *step_n;
    auto host_call = [&]() -> int {   // one propagator() call and the z-loop's update, on the host
        int rc = gs_step(h, cz, znet[n_z], znet[n_z - 1], &dz, &sn, nullptr, nullptr);
        if (rc == GS_OK) {
            sn++;
            cz += dz;
            done++;
        }
        return rc;
    };
    int rc = GS_OK;
    // the first call on the host when the NL path is not known yet (it decides nl_compact and
    // nl_dev_dz: whether the NL kernels take their step size from the device)
    if (!device_ok(h) && !h->nl_compact && !h->nl_dev_dz && done < max_calls && cz < znet[n_z]) rc = host_call();
    if (rc == GS_OK && !device_ok(h)) {   // everything else on the host, call by call
        while (rc == GS_OK && done < max_calls && cz < znet[n_z]) rc = host_call();
    } else if (rc == GS_OK && done < max_calls && cz < znet[n_z]) {
        if (h->znet_cap < nz) {
            if (h->znet_dev) cudaFree(h->znet_dev);
            h->znet_dev = nullptr;
            h->znet_cap = 0;
            CK(h, cudaMalloc(&h->znet_dev, (size_t)nz * sizeof(double)));
            h->znet_cap = nz;
        }
        if (!h->ctl_dev) CK(h, cudaMalloc(&h->ctl_dev, sizeof(DevCtl)));
        CK(h, cudaMemcpyAsync(h->znet_dev, znet, (size_t)nz * sizeof(double), cudaMemcpyHostToDevice, h->st));
        rc = gsi::spec_prepare(h);   // BIGBUFFER2's window columns compact from the start
        if (rc) return rc;
        DevCtl c{};
        c.z = cz;
        c.zstep = dz;
        c.step_n = sn;
        c.n_z = n_z;
        c.max_calls = max_calls - done;
        c.field_compact = h->a_compact ? 1 : 0;
        CK(h, cudaMemcpyAsync(h->ctl_dev, &c, sizeof(DevCtl), cudaMemcpyHostToDevice, h->st));
        CK(h, cudaMemsetAsync(h->max_dev, 0, 16, h->st));
        CK(h, cudaMemsetAsync(h->err_dev, 0, 4, h->st));
        // timing (gs_nl_timing / gs_qdht_timing): events around each attempt's NL launch and
        // its linear step, folded in after the batch (linear steps of accepted attempts only)
        const bool tn = h->time_nl, tq = h->time_qdht;
        h->time_nl = h->time_qdht = false;
        constexpr int BATCH = 32;
        if (tn || tq) {
            while ((int)h->adv_ev.size() < 4 * BATCH) {
                cudaEvent_t e;
                if (cudaEventCreate(&e) != cudaSuccess) break;
                h->adv_ev.push_back(e);
            }
        }
        const bool have_ev = (int)h->adv_ev.size() >= 4 * BATCH;
        struct Restore {   // the handle back in host mode on every way out
            gs_handle* h;
            bool tn, tq;
            ~Restore() {
                h->ctl = nullptr;
                h->time_nl = tn;
                h->time_qdht = tq;
            }
        } restore{h, tn, tq};
        h->ctl = h->ctl_dev;
        const double tol = h->p.max_tolerance;
        for (;;) {
            const int left = c.max_calls - c.calls;
            const int nb = std::min(BATCH, std::max(1, left));
            for (int k = 0; k < nb && rc == GS_OK; k++) {
                if (tn && have_ev) cudaEventRecord(h->adv_ev[4 * k], h->st);
                rc = gsi::nl_stages(h, dz, nullptr);   // dz unused: the kernel reads the device's
                if (rc) break;
                if (tn && have_ev) cudaEventRecord(h->adv_ev[4 * k + 1], h->st);
                CK(h, launch_step_ctl(h->ctl_dev, h->znet_dev, h->max_dev, h->err_dev, tol, k, h->st, &h->launches));
                if (tq && have_ev) cudaEventRecord(h->adv_ev[4 * k + 2], h->st);
                rc = gsi::lstep(h, dz);
                if (tq && have_ev) cudaEventRecord(h->adv_ev[4 * k + 3], h->st);
            }
            if (rc) break;
            CK(h, cudaMemcpyAsync(&c, h->ctl_dev, sizeof(DevCtl), cudaMemcpyDeviceToHost, h->st));
            CK(h, cudaStreamSynchronize(h->st));
            if (have_ev) {
                for (int k = 0; k < c.iter && k < nb; k++) {
                    float f = 0;
                    if (tn && cudaEventElapsedTime(&f, h->adv_ev[4 * k], h->adv_ev[4 * k + 1]) == cudaSuccess) {
                        h->nl_ms += f;
                        h->nl_stages_timed += 4;
                        h->nl_launches_timed += 1;
                    }
                    if (tq && c.acc_log[k] &&
                        cudaEventElapsedTime(&f, h->adv_ev[4 * k + 2], h->adv_ev[4 * k + 3]) == cudaSuccess) {
                        h->qdht_ms += f;
                        h->qdht_n += 2;   // the linear-step transform and the masked inverse
                    }
                }
            }
            if (c.stop) break;
            CK(h, cudaMemsetAsync(&h->ctl_dev->iter, 0, sizeof(int), h->st));
        }
        if (rc) return rc;
        h->a_compact = h->nl_compact && c.field_compact != 0;   // only the row kernel's masked inverse is lazy
        cz = c.z;
        dz = c.zstep;
        sn = c.step_n;
        done += c.calls;
        // the state after the last accepted call (and, on a collapse, the collapsed proposal)
        *current_z = cz;
        *zstep = dz;
        *step_n = sn;
        if (calls_done) *calls_done = done;
        std::string m;
        if (gs::qdht_tc_check(h->tc, &m)) return gsi::fail(h, GS_ERR_CUDA, m);
        if (c.stop == 3) return gsi::fail(h, GS_ERR_COLLAPSE, gs_status_string(GS_ERR_COLLAPSE));
        if (c.stop == 4) {
            if (c.err & GS_ERRBIT_BOUNDS) return gsi::fail(h, GS_ERR_CUDA, GS_BOUNDS_MSG);
            if (c.err & 1u) return gsi::fail(h, GS_ERR_BLAST, gs_status_string(GS_ERR_BLAST));
            return gsi::fail(h, GS_ERR_NAN, gs_status_string(GS_ERR_NAN));
        }
    }
    *current_z = cz;
    *zstep = dz;
    *step_n = sn;
    if (calls_done) *calls_done = done;
    if (reached) *reached = cz >= znet[n_z] ? 1 : 0;
    return rc;
}
