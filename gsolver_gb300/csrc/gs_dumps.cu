// gs_dumps.cu -- device reductions behind the reference's .udf dumps (dump_types.cpp).
//
// All of them start from FIELD (r, omega) resident in HBM, so the field never travels to
// the host at a ZNET point; only the reduced slabs do:
//   maxI / flux (dump_types.cpp:104-165)   E = BW-FFT(FIELD)/N_T per row, max |E|^2 and
//                                           sum |E|^2 * TSTEP (FILTER_TYPE NO)
//   plasma_max (535-555)                    the plasma recurrence of E per row, max rho
//   field_axis (404-417)                    E of row 0
//   average_spectrum (427-457)              sum_r |FIELD(r, omega)|^2 w_r, w the reference's
//                                           trapezoid-like weights on the QDHT points
#include "gs_internal.cuh"
#include "gs_kernels.h"

namespace gs {

template <typename Rl>
__global__ void row_intensity_kernel(const C2<Rl>* __restrict__ E, int N, double tstep, double* maxI,
                                     double* flux) {
    const size_t base = (size_t)blockIdx.x * N;
    double m = 0.0, s = 0.0;
    for (int t = threadIdx.x; t < N; t += blockDim.x) {
        const C2<Rl> e = E[base + t];
        const double I = (double)e.x * e.x + (double)e.y * e.y;
        m = fmax(m, I);
        s += I;
    }
    __shared__ double sm[32], ss[32];
    for (int o = 16; o > 0; o >>= 1) {
        m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    if ((threadIdx.x & 31) == 0) { sm[threadIdx.x >> 5] = m; ss[threadIdx.x >> 5] = s; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double M = 0, S = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) { M = fmax(M, sm[w]); S += ss[w]; }
        if (maxI) maxI[blockIdx.x] = M;
        if (flux) flux[blockIdx.x] = S * tstep;
    }
}

template <typename Rl>
__global__ void row_max_re_kernel(const C2<Rl>* __restrict__ U, int N, double* out) {
    const size_t base = (size_t)blockIdx.x * N;
    double m = 0.0;
    for (int t = threadIdx.x; t < N; t += blockDim.x) m = fmax(m, (double)U[base + t].x);
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

template <typename Rl>
__global__ void spectrum_kernel(const C2<Rl>* __restrict__ F, int nr, int N, const double* __restrict__ w,
                                double scale, double* out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N) return;
    double s = 0.0;
    for (int r = 0; r < nr; r++) {
        const C2<Rl> v = F[(size_t)r * N + p];
        s += ((double)v.x * v.x + (double)v.y * v.y) * w[r];
    }
    out[p] = s * scale;
}

template <typename Rl>
cudaError_t launch_row_intensity(const C2<Rl>* E, int rows, int N, double tstep, double* maxI, double* flux,
                                 cudaStream_t st, long long* nl) {
    row_intensity_kernel<Rl><<<rows, 256, 0, st>>>(E, N, tstep, maxI, flux);
    (*nl)++;
    return cudaGetLastError();
}
template <typename Rl>
cudaError_t launch_row_max_re(const C2<Rl>* U, int rows, int N, double* out, cudaStream_t st, long long* nl) {
    row_max_re_kernel<Rl><<<rows, 256, 0, st>>>(U, N, out);
    (*nl)++;
    return cudaGetLastError();
}
template <typename Rl>
cudaError_t launch_spectrum(const C2<Rl>* F, int nr, int N, const double* w, double scale, double* out,
                            cudaStream_t st, long long* nl) {
    spectrum_kernel<Rl><<<(N + 255) / 256, 256, 0, st>>>(F, nr, N, w, scale, out);
    (*nl)++;
    return cudaGetLastError();
}

#define GS_DUMP_INST(Rl)                                                                                    \
    template cudaError_t launch_row_intensity<Rl>(const C2<Rl>*, int, int, double, double*, double*,       \
                                                  cudaStream_t, long long*);                               \
    template cudaError_t launch_row_max_re<Rl>(const C2<Rl>*, int, int, double*, cudaStream_t, long long*); \
    template cudaError_t launch_spectrum<Rl>(const C2<Rl>*, int, int, const double*, double, double*,      \
                                             cudaStream_t, long long*);
GS_DUMP_INST(double)
GS_DUMP_INST(float)

}  // namespace gs
