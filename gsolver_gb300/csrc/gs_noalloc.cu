// gs_noalloc.cu -- an entry point that allocates no device memory.
//
// gs_plasma_max_noalloc runs the FP64 carrier-density recurrence (the plasma_max dump's
// computation) on caller-provided device buffers.  Its per-sample scratch (photoionization
// rates, avalanche prefactors and the density itself) lives in one file-scope device array of
// fixed size instead of coming from cudaMalloc.  It is for host code that cannot allocate
// device memory at the point where it needs this result: for example an application whose
// device memory is handed out by its own allocator, which has reserved the GPU up front and
// forbids further cudaMalloc calls from libraries it links.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "../../include/gs_abi.h"
#include "gs_internal.cuh"
#include "gs_kernels.h"

namespace {

// 16 MiB: a 256-byte error word, then 2 x rows x n_t x 16 bytes of recurrence scratch
constexpr size_t kScratchBytes = 16u << 20;
constexpr size_t kErrBytes = 256;

// Every GPU that loads this library holds this array until the process exits.  In host code
// its name is only a host-side stand-in for the symbol, not a device address: kernels get the
// address that cudaGetSymbolAddress returns for the current device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::string g_noalloc_err;

int fail(int code, const std::string& m) {
    g_noalloc_err = m;
    return code;
}

}  // namespace

extern "C" const char* gs_noalloc_last_error(void) { return g_noalloc_err.c_str(); }

extern "C" size_t gs_noalloc_max_samples(void) { return (kScratchBytes - kErrBytes) / (2 * sizeof(double2)); }

extern "C" int gs_plasma_max_noalloc(const gs_params* p, const double* rate_ln_dev, const double* e_r_t_dev, int rows,
                                     double* plasma_max_dev, void* stream) {
    if (!p || !rate_ln_dev || !e_r_t_dev || !plasma_max_dev || rows < 1)
        return fail(GS_ERR_ARG, "gs_plasma_max_noalloc: null pointer or rows < 1");
    const int nt = p->n_t;
    if (nt < 64 || (nt & (nt - 1))) return fail(GS_ERR_ARG, "gs_plasma_max_noalloc: n_t must be a power of two >= 64");
    const size_t samples = (size_t)rows * (size_t)nt;
    if (samples > gs_noalloc_max_samples())
        return fail(GS_ERR_ARG, "gs_plasma_max_noalloc: rows * n_t = " + std::to_string(samples) +
                                    " exceeds the fixed scratch of " + std::to_string(gs_noalloc_max_samples()) +
                                    " samples (16 MiB); split the rows into several calls");
    // The array's device address on the current device, looked up on every call: the lookup
    // allocates nothing, and a cached address would go stale after cudaDeviceReset or a new
    // primary context.  The first call on a device also loads this library's device code
    // there, so make that first call before any stream capture begins on the device.
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) return fail(GS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    unsigned char* base = (unsigned char*)ptr;
    unsigned* err_dev = (unsigned*)base;
    double2* u1 = (double2*)(base + kErrBytes);
    double2* u2 = u1 + samples;
    cudaStream_t st = (cudaStream_t)stream;
    long long nl = 0;
    // the array keeps the previous call's contents: the error word must start at zero
    e = cudaMemsetAsync(err_dev, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return fail(GS_ERR_CUDA, cudaGetErrorString(e));
    gs::PlasmaArgs<double> a{};
    a.N = nt;
    a.e = (const double2*)e_r_t_dev;
    a.u1 = u1;
    a.u2 = u2;
    a.u3 = nullptr;
    a.rate = rate_ln_dev;
    a.err = err_dev;
    a.raman = 1;
    a.raman_scan = 0;
    a.density_only = 1;
    a.gas = p->gas;
    a.tstep_scaled = p->tstep * p->ionrate_denom;
    a.neutral_density = p->neutral_density;
    a.rho0 = p->rho0;
    a.ionization_potential = p->ionization_potential;
    a.ponderomotive = p->ponderomotive;
    a.avalanche_cs = p->avalanche_cs;
    a.recombination_tau = p->recombination_tau;
    gs::plasma_consts<double>(a);
    e = gs::launch_plasma<double>(a, rows, st, &nl);
    if (e == cudaSuccess) e = gs::launch_row_max_re<double>(u2, rows, nt, plasma_max_dev, st, &nl);
    if (e != cudaSuccess) return fail(GS_ERR_CUDA, cudaGetErrorString(e));
    unsigned err = 0;
    e = cudaMemcpyAsync(&err, err_dev, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(GS_ERR_CUDA, cudaGetErrorString(e));
    if (err & 1u) return fail(GS_ERR_BLAST, gs_status_string(GS_ERR_BLAST));
    if (err & 2u) return fail(GS_ERR_NAN, gs_status_string(GS_ERR_NAN));
    return GS_OK;
}
