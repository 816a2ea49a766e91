// gs_state.cu -- energy and photon number of FIELD (FP64 device reductions), the optional
// photon-number check of gs_step, and checkpoints of a handle's state (include/gs_abi.h).
//
// Energy is the sum of the reference's average spectrum (dump_type_average_spectrum_class,
// dump_types.cpp:427-457, uniaxial branch): E = R_MAX^2 / 2 sum_omega sum_r w_r |FIELD(r, omega)|^2
// with w_0 = x_0 (x_1 - x_0), w_r = x_r (x_r - x_{r-1}) (x the QDHT points); the photon number
// weights each omega > 0 by 1 / omega.  Both are summed in FP64 on the device in a fixed order
// (per column over the rows, then the columns' block sums in block order), so they repeat bit for
// bit.  FIELD is read where it is current: the masked inverse's compact window columns when the
// mixed plan left it there (zeros outside the window need no reading), else the full array.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gs_abi.h"
#include "gs_handle.h"
#include "gs_internal.cuh"
#include "gs_kernels.h"
#include "gs_qdht_tc.h"

using gsi::fail;

namespace {

constexpr int EN_THREADS = 256;
constexpr int EN_BLOCKS = 256;   // partial sums: fixed, so that the summation order is fixed

// F: [nr] rows of ncols complex columns (row stride ld complex elements); column c holds spectral
// position pos(c) = colmap ? colmap[2 c] / 2 (-1: padding) : c.  One thread per column (strided),
// rows summed in order; block sums written to partial[blockIdx] (E) and partial[gridDim + .] (N).
template <typename Rl>
__global__ void energy_cols_kernel(const typename gs::Vec2<Rl>::T* __restrict__ F, size_t ld, int ncols, int nr,
                                   const int* __restrict__ colmap, const double* __restrict__ w,
                                   const double* __restrict__ omega, double* __restrict__ partial) {
    __shared__ double se[EN_THREADS], sn[EN_THREADS];
    double e = 0.0, n = 0.0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncols; c += gridDim.x * blockDim.x) {
        const int p = colmap ? (colmap[2 * c] < 0 ? -1 : colmap[2 * c] >> 1) : c;
        if (p < 0) continue;
        double s = 0.0;
        for (int r = 0; r < nr; r++) {
            const typename gs::Vec2<Rl>::T v = F[(size_t)r * ld + c];
            s += ((double)v.x * v.x + (double)v.y * v.y) * w[r];
        }
        e += s;
        if (omega[p] > 0) n += s / omega[p];
    }
    se[threadIdx.x] = e;
    sn[threadIdx.x] = n;
    __syncthreads();
    for (int h = EN_THREADS / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            se[threadIdx.x] += se[threadIdx.x + h];
            sn[threadIdx.x] += sn[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = se[0];
        partial[gridDim.x + blockIdx.x] = sn[0];
    }
}

__global__ void energy_final_kernel(const double* __restrict__ partial, int nb, double scale, double* __restrict__ out) {
    if (threadIdx.x != 0) return;
    double e = 0.0, n = 0.0;
    for (int b = 0; b < nb; b++) {
        e += partial[b];
        n += partial[nb + b];
    }
    out[0] = e * scale;
    out[1] = n * scale;
}

int set_weights(gs_handle* h, const double* x, double r_max) {
    const int nr = h->nr;
    if (!x || nr < 2 || !(r_max > 0)) return fail(h, GS_ERR_ARG, "energy: needs the QDHT points (n_r >= 2) and R_MAX");
    if (!h->en_dev) CK(h, cudaMalloc((void**)&h->en_dev, sizeof(double) * ((size_t)nr + 2 * EN_BLOCKS + 2)));
    std::vector<double> w(nr);
    w[0] = x[0] * (x[1] - x[0]);
    for (int r = 1; r < nr; r++) w[r] = x[r] * (x[r] - x[r - 1]);
    CK(h, cudaMemcpy(h->en_dev, w.data(), sizeof(double) * nr, cudaMemcpyHostToDevice));
    h->en_scale = r_max * r_max / 2.0;
    h->en_weights = true;
    return GS_OK;
}

// E and N of the current FIELD into h->en_dev[nr + 2 EN_BLOCKS + 0/1], on the handle's stream
int launch_energy(gs_handle* h) {
    const int nr = h->nr;
    double* w = h->en_dev;
    double* partial = w + nr;
    double* out = partial + 2 * EN_BLOCKS;
    int nyc = 0;
    const int* cmap = nullptr;
    const float* yc = (h->a_compact && h->tc) ? gs::qdht_tc_compact_y(h->tc, &nyc, &cmap) : nullptr;
    cudaError_t e;
    if (yc) {
        energy_cols_kernel<float><<<EN_BLOCKS, EN_THREADS, 0, h->st>>>((const float2*)yc, (size_t)nyc / 2, nyc / 2, nr, cmap,
                                                                       w, h->omega, partial);
    } else if (h->fp64) {
        energy_cols_kernel<double><<<EN_BLOCKS, EN_THREADS, 0, h->st>>>((const double2*)h->A, (size_t)h->nt, h->nt, nr,
                                                                        nullptr, w, h->omega, partial);
    } else {
        energy_cols_kernel<float><<<EN_BLOCKS, EN_THREADS, 0, h->st>>>((const float2*)h->A, (size_t)h->nt, h->nt, nr,
                                                                       nullptr, w, h->omega, partial);
    }
    energy_final_kernel<<<1, 32, 0, h->st>>>(partial, EN_BLOCKS, h->en_scale, out);
    h->launches += 2;
    e = cudaGetLastError();
    CK(h, e);
    return GS_OK;
}

int read_energy(gs_handle* h, double* E, double* N) {
    double v[2];
    CK(h, cudaMemcpyAsync(v, h->en_dev + h->nr + 2 * EN_BLOCKS, sizeof(v), cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    if (E) *E = v[0];
    if (N) *N = v[1];
    return GS_OK;
}

int photons_now(gs_handle* h, double* N) {
    int rc = launch_energy(h);
    if (!rc) rc = read_energy(h, nullptr, N);
    return rc;
}

// BIGBUFFER2 as the linear step reads and writes it: the mixed plan's double-float compact copy,
// else the full array
int spec_state(gs_handle* h, void** p0, void** p1, size_t* bytes) {
    float *sc = nullptr, *sl = nullptr;
    int nc = 0;
    if (!h->fp64 && h->tc && h->s_compact) gs::qdht_tc_spec_pairs(h->tc, &sc, &sl, &nc);
    if (sc) {
        *p0 = sc;
        *p1 = sl;
        *bytes = (size_t)h->nr * nc * sizeof(float);
    } else {
        *p0 = h->S;
        *p1 = nullptr;
        *bytes = (size_t)h->nr * h->nt * h->esz;
    }
    return GS_OK;
}

}  // namespace

int gsi::lstep_checked(gs_handle* h, double* dz_inout, double dz_min) {
    int rc = gsi::spec_prepare(h);   // the state the linear step will update, taken now
    if (rc) return rc;
    if (!(h->en_prev > 0)) {
        rc = photons_now(h, &h->en_prev);
        if (rc) return rc;
    }
    void *p0, *p1;
    size_t bytes;
    spec_state(h, &p0, &p1, &bytes);
    const size_t need = bytes * (p1 ? 2 : 1);
    if (h->en_save_bytes < need) {
        if (h->en_save) cudaFree(h->en_save);
        h->en_save = nullptr;
        h->en_save_bytes = 0;
        CK(h, cudaMalloc(&h->en_save, need));
        h->en_save_bytes = need;
    }
    CK(h, cudaMemcpyAsync(h->en_save, p0, bytes, cudaMemcpyDeviceToDevice, h->st));
    if (p1) CK(h, cudaMemcpyAsync((char*)h->en_save + bytes, p1, bytes, cudaMemcpyDeviceToDevice, h->st));
    double dz = *dz_inout;
    for (;;) {
        rc = gsi::lstep(h, dz);
        if (rc) return rc;
        double n1 = 0;
        rc = photons_now(h, &n1);
        if (rc) return rc;
        const double rel = std::fabs(n1 / h->en_prev - 1.0);
        if (rel <= h->en_tol) {
            h->en_prev = n1;
            h->en_last = rel;
            *dz_inout = dz;
            return GS_OK;
        }
        // rejected: BIGBUFFER2 as it was, half the step; the NL increment (taken with the
        // previous step size, as propagator() does) is reused
        h->en_rejects++;
        CK(h, cudaMemcpyAsync(p0, h->en_save, bytes, cudaMemcpyDeviceToDevice, h->st));
        if (p1) CK(h, cudaMemcpyAsync(p1, (char*)h->en_save + bytes, bytes, cudaMemcpyDeviceToDevice, h->st));
        dz *= 0.5;
        if (dz < dz_min) {
            *dz_inout = dz;
            return fail(h, GS_ERR_COLLAPSE, gs_status_string(GS_ERR_COLLAPSE));
        }
    }
}

int gs_energy(gs_handle* h, const double* qdht_x, double r_max, double* energy, double* photons) {
    if (!h) return GS_ERR_ARG;
    if (!h->tables_ok || !h->field_ok) return fail(h, GS_ERR_STATE, "tables / field not set");
    CK(h, cudaSetDevice(h->p.device));
    int rc = set_weights(h, qdht_x, r_max);
    if (!rc) rc = launch_energy(h);
    if (!rc) rc = read_energy(h, energy, photons);
    return rc;
}

int gs_set_energy_tolerance(gs_handle* h, double tol, const double* qdht_x, double r_max) {
    if (!h || !(tol >= 0)) return fail(h, GS_ERR_ARG, "gs_set_energy_tolerance: tolerance >= 0");
    CK(h, cudaSetDevice(h->p.device));
    if (tol > 0) {
        const int rc = set_weights(h, qdht_x, r_max);
        if (rc) return rc;
    }
    h->en_tol = tol;
    h->en_prev = 0;
    h->en_last = 0;
    h->en_rejects = 0;
    return GS_OK;
}

int gs_energy_stats(const gs_handle* h, double* last_rel_change, long long* rejections) {
    if (!h) return GS_ERR_ARG;
    if (last_rel_change) *last_rel_change = h->en_last;
    if (rejections) *rejections = h->en_rejects;
    return GS_OK;
}

// ---------------------------------------------------------------------------- checkpoints --
namespace {

struct CkptHeader {
    char magic[8];
    int version, n_r, n_t, precision, nc, spec_pairs;
    double current_z, zstep;
    int n_z;
    unsigned step_n;
};

const char kMagic[8] = {'G', 'S', 'C', 'K', 'P', 'T', '1', 0};

int write_dev(gs_handle* h, FILE* f, const void* dev, size_t bytes) {
    std::vector<unsigned char> buf(bytes);
    CK(h, cudaMemcpy(buf.data(), dev, bytes, cudaMemcpyDeviceToHost));
    if (fwrite(buf.data(), 1, bytes, f) != bytes) return fail(h, GS_ERR_ARG, "checkpoint: write failed");
    return GS_OK;
}

int read_dev(gs_handle* h, FILE* f, void* dev, size_t bytes) {
    std::vector<unsigned char> buf(bytes);
    if (fread(buf.data(), 1, bytes, f) != bytes) return fail(h, GS_ERR_ARG, "checkpoint: file too short");
    CK(h, cudaMemcpy(dev, buf.data(), bytes, cudaMemcpyHostToDevice));
    return GS_OK;
}

}  // namespace

int gs_checkpoint_save(gs_handle* h, const char* path, double current_z, double zstep, int n_z, unsigned step_n) {
    if (!h || !path) return GS_ERR_ARG;
    if (!h->tables_ok || !h->field_ok) return fail(h, GS_ERR_STATE, "tables / field not set");
    CK(h, cudaSetDevice(h->p.device));
    int rc = gsi::field_sync(h);
    if (!rc) rc = gsi::spec_sync(h);
    if (rc) return rc;
    CK(h, cudaStreamSynchronize(h->st));
    float *sc = nullptr, *sl = nullptr;
    int nc = 0;
    if (!h->fp64 && h->tc && h->s_compact) gs::qdht_tc_spec_pairs(h->tc, &sc, &sl, &nc);
    CkptHeader hd{};
    std::memcpy(hd.magic, kMagic, 8);
    hd.version = 1;
    hd.n_r = h->nr;
    hd.n_t = h->nt;
    hd.precision = h->p.precision;
    hd.nc = nc;
    hd.spec_pairs = sc ? 1 : 0;
    hd.current_z = current_z;
    hd.zstep = zstep;
    hd.n_z = n_z;
    hd.step_n = step_n;
    FILE* f = fopen(path, "wb");
    if (!f) return fail(h, GS_ERR_ARG, std::string("checkpoint: cannot write ") + path);
    const size_t nel = (size_t)h->nr * h->nt;
    rc = fwrite(&hd, sizeof(hd), 1, f) == 1 ? GS_OK : fail(h, GS_ERR_ARG, "checkpoint: write failed");
    if (!rc) rc = write_dev(h, f, h->A, nel * h->esz);
    if (!rc) rc = write_dev(h, f, h->S, nel * h->esz);
    if (!rc && sc) rc = write_dev(h, f, sc, (size_t)h->nr * nc * sizeof(float));
    if (!rc && sc) rc = write_dev(h, f, sl, (size_t)h->nr * nc * sizeof(float));
    if (fclose(f) != 0 && !rc) rc = fail(h, GS_ERR_ARG, "checkpoint: close failed");
    return rc;
}

int gs_checkpoint_load(gs_handle* h, const char* path, double* current_z, double* zstep, int* n_z, unsigned* step_n) {
    if (!h || !path) return GS_ERR_ARG;
    if (!h->tables_ok) return fail(h, GS_ERR_STATE, "tables not uploaded");
    CK(h, cudaSetDevice(h->p.device));
    FILE* f = fopen(path, "rb");
    if (!f) return fail(h, GS_ERR_ARG, std::string("checkpoint: cannot read ") + path);
    CkptHeader hd{};
    int rc = fread(&hd, sizeof(hd), 1, f) == 1 ? GS_OK : fail(h, GS_ERR_ARG, "checkpoint: file too short");
    float *sc = nullptr, *sl = nullptr;
    int nc = 0;
    if (!h->fp64 && h->tc) gs::qdht_tc_spec_pairs(h->tc, &sc, &sl, &nc);
    if (!rc && (std::memcmp(hd.magic, kMagic, 8) != 0 || hd.version != 1))
        rc = fail(h, GS_ERR_ARG, "checkpoint: not a checkpoint of this library");
    if (!rc && (hd.n_r != h->nr || hd.n_t != h->nt || hd.precision != h->p.precision))
        rc = fail(h, GS_ERR_ARG, "checkpoint: grid or precision differs from the handle's");
    if (!rc && hd.spec_pairs && (!sc || hd.nc != nc))
        rc = fail(h, GS_ERR_ARG, "checkpoint: spectral window differs from the handle's tables");
    const size_t nel = (size_t)h->nr * h->nt;
    if (!rc) {
        gsi::field_written(h);
        gsi::spec_written(h);
        rc = read_dev(h, f, h->A, nel * h->esz);
    }
    if (!rc) rc = read_dev(h, f, h->S, nel * h->esz);
    if (!rc && hd.spec_pairs) rc = read_dev(h, f, sc, (size_t)h->nr * nc * sizeof(float));
    if (!rc && hd.spec_pairs) rc = read_dev(h, f, sl, (size_t)h->nr * nc * sizeof(float));
    fclose(f);
    if (rc) return rc;
    h->s_compact = hd.spec_pairs != 0;
    h->field_ok = true;
    h->nbc_valid = false;
    h->en_prev = 0;
    if (current_z) *current_z = hd.current_z;
    if (zstep) *zstep = hd.zstep;
    if (n_z) *n_z = hd.n_z;
    if (step_n) *step_n = hd.step_n;
    return GS_OK;
}
