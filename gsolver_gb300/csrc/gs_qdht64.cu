// gs_qdht64.cu -- FP64 quasi-discrete Hankel transform (QDHT) with the fused linear step.
//
// ht_run -> qdht_plan::run_many (fhatha.cpp:218-230) applies, per omega column,
//   x /= m1;  y_i = sum_j C[i + N*j] x_j;  x = y * m1,
// i.e. one real N_r x N_r by N_r x (2 N_t) GEMM over the interleaved (re, im) columns of
// a [n_r][n_t] complex array.  This is the FP64 parity path (CUDA-core DFMA; GB300's
// FP64 rate bounds it): 64 x 64 output tiles, K-tiles of 16, one sequential FMA chain
// per output in ascending j as the reference sums.
//   QDHT_PLAIN   Y = QDHT(X)
//   QDHT_LSTEP   X = BIGBUFFER1 (r,omega); the epilogue applies calculate_Lstep
//                (propagator.cu:570-625) to BIGBUFFER2 in place: inside the spectral
//                window  B2 += dz*N/(1+s);  B2 *= exp(dz*(-j(D + k_r s) + k_i)).
//   QDHT_MASKED  X = BIGBUFFER2 read as FIELD: zero outside the window (what
//                calculate_Lstep writes into FIELD there), Y = FIELD (r,omega).
#include <algorithm>

#include "gs_kernels.h"
#include "gs_internal.cuh"

namespace gs {

__constant__ double c_sqrt_ho[20];   // binom(1/2, n), n = 1..20 (extmath.h:234-256)

__device__ __forceinline__ double sqrt_ho(double x) {
    double r = 0, xn = x;
#pragma unroll
    for (int j = 0; j < 20; j++) { r += c_sqrt_ho[j] * xn; xn *= x; }
    return r;
}

__device__ __forceinline__ bool in_window(const LstepArgs& L, int k, int p) {
    const double w = L.omega[p];
    if (w < L.omega_min || w > L.omega_max) return false;
    const double2 kk = L.wavenum[p];
    if (L.kt2[k] > 0.25 * (kk.x * kk.x - kk.y * kk.y)) return false;
    return true;
}

constexpr int BM = 64, BN = 64, BK = 16;

// cmap (or null: column c itself): the real column of X / Y that operand column c stands for
// (-1: padding).  The linear-step and masked transforms take the spectral window's columns
// only: outside it the linear step leaves BIGBUFFER2 untouched and the masked inverse's
// columns are zero (written by qdht64_zero_kernel).
template <int MODE>
__global__ void __launch_bounds__(256) qdht64_kernel(const double* __restrict__ C, const double* __restrict__ m1,
                                                     const double* __restrict__ X, double* __restrict__ Y, int nr,
                                                     int ncols, LstepArgs L, const int* __restrict__ cmap) {
    __shared__ double As[2][BK][BM];
    __shared__ __align__(16) double Bs[2][BK][BN];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int i0 = blockIdx.y * BM, c0 = blockIdx.x * BN;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = 0.0;

    const int lm = tid & 63, lk = tid >> 6;   // loader: 64 wide, 4 k-rows per pass
    double ra[4], rb[4];
    auto load = [&](int k0) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int k = lk + 4 * u, j = k0 + k, i = i0 + lm, c = cmap ? cmap[c0 + lm] : c0 + lm;
            ra[u] = (i < nr && j < nr) ? C[(size_t)i + (size_t)nr * j] : 0.0;
            double v = 0.0;
            if (j < nr && c >= 0) {
                v = X[(size_t)j * ncols + c];
                if (MODE == QDHT_MASKED && !in_window(L, j, c >> 1)) v = 0.0;
                v = v / m1[j];
            }
            rb[u] = v;
        }
    };
    auto store = [&](int buf) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
            As[buf][lk + 4 * u][lm] = ra[u];
            Bs[buf][lk + 4 * u][lm] = rb[u];
        }
    };
    const int nk = (nr + BK - 1) / BK;
    load(0);
    store(0);
    __syncthreads();
    for (int kt = 0; kt < nk; kt++) {
        const int cur = kt & 1;
        if (kt + 1 < nk) load((kt + 1) * BK);
#pragma unroll
        for (int k = 0; k < BK; k++) {
            double a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; u++) a[u] = As[cur][k][ty * 4 + u];
            const double2 b01 = *reinterpret_cast<const double2*>(&Bs[cur][k][tx * 4]);
            const double2 b23 = *reinterpret_cast<const double2*>(&Bs[cur][k][tx * 4 + 2]);
            b[0] = b01.x; b[1] = b01.y; b[2] = b23.x; b[3] = b23.y;
#pragma unroll
            for (int u = 0; u < 4; u++)
#pragma unroll
                for (int v = 0; v < 4; v++) acc[u][v] = fma(a[u], b[v], acc[u][v]);
        }
        if (kt + 1 < nk) store(cur ^ 1);
        __syncthreads();
    }

#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int i = i0 + ty * 4 + u;
        if (i >= nr) continue;
        const double mi = m1[i];
        // the two (re, im) pairs of this thread's four operand columns
        const int rc0 = cmap ? cmap[c0 + tx * 4] : c0 + tx * 4, rc1 = cmap ? cmap[c0 + tx * 4 + 2] : c0 + tx * 4 + 2;
        if (MODE != QDHT_LSTEP) {
            if (rc0 >= 0) *reinterpret_cast<double2*>(&Y[(size_t)i * ncols + rc0]) = make_double2(acc[u][0] * mi, acc[u][1] * mi);
            if (rc1 >= 0) *reinterpret_cast<double2*>(&Y[(size_t)i * ncols + rc1]) = make_double2(acc[u][2] * mi, acc[u][3] * mi);
        } else {
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int rc = e ? rc1 : rc0;
                if (rc < 0) continue;
                const int p = rc >> 1;
                double* y2 = &Y[(size_t)i * ncols + rc];
                if (!in_window(L, i, p)) continue;   // FIELD = 0 there; BIGBUFFER2 untouched
                const double vr = acc[u][2 * e] * mi, vi = acc[u][2 * e + 1] * mi;
                const double2 kk = L.wavenum[p];
                const double k1 = kk.x, k2 = kk.y;
                const double sq = sqrt_ho(-L.kt2[i] / k1 / k1);
                double2 b2 = *reinterpret_cast<const double2*>(y2);
                b2.x += L.dz * vr / (1 + sq);
                b2.y += L.dz * vi / (1 + sq);
                const double er = L.dz * k2, ei = L.dz * (-L.ho[p] - sq * k1);
                double s, c;
                sincos(ei, &s, &c);
                const double m = exp(er);
                const double pr = m * c, pi = m * s;
                double2 f;
                f.x = b2.x * pr - b2.y * pi;
                f.y = b2.x * pi + b2.y * pr;
                *reinterpret_cast<double2*>(y2) = f;
            }
        }
    }
}

__global__ void qdht64_zero_kernel(double* __restrict__ Y, int ncols, int nr, const int* __restrict__ zpos, int nz) {
    const size_t total = (size_t)nr * nz;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        const size_t i = idx / nz;
        const int z = (int)(idx - i * nz);
        *reinterpret_cast<double2*>(Y + i * ncols + 2 * zpos[z]) = make_double2(0.0, 0.0);
    }
}

cudaError_t launch_qdht64(int mode, const double* C, const double* m1, const double* X, double* Y, int nr,
                          int ncols, const LstepArgs& L, cudaStream_t st, long long* nlaunch, const int* cmap, int nc,
                          const int* zpos, int nz) {
    if (!cmap) nc = ncols;
    if (mode == QDHT_MASKED && cmap && nz > 0) {
        const size_t tot = (size_t)nr * nz;
        qdht64_zero_kernel<<<(unsigned)std::min<size_t>((tot + 255) / 256, 4096), 256, 0, st>>>(Y, ncols, nr, zpos, nz);
        (*nlaunch)++;
    }
    if (nc == 0) return cudaGetLastError();
    dim3 grid(nc / BN, (nr + BM - 1) / BM);
    switch (mode) {
        case QDHT_PLAIN: qdht64_kernel<QDHT_PLAIN><<<grid, 256, 0, st>>>(C, m1, X, Y, nr, ncols, L, nullptr); break;
        case QDHT_LSTEP: qdht64_kernel<QDHT_LSTEP><<<grid, 256, 0, st>>>(C, m1, X, Y, nr, ncols, L, cmap); break;
        case QDHT_MASKED: qdht64_kernel<QDHT_MASKED><<<grid, 256, 0, st>>>(C, m1, X, Y, nr, ncols, L, cmap); break;
        default: return cudaErrorInvalidValue;
    }
    (*nlaunch)++;
    return cudaGetLastError();
}

cudaError_t qdht_set_sqrt_ho(const double* coeffs20) {
    return cudaMemcpyToSymbol(c_sqrt_ho, coeffs20, sizeof(double) * 20);
}

// Adjoint of calculate_Lstep per (k, omega): inside the window T = B2 + dz N/(1+s),
// FIELD = B2' = T P, so T_bar = conj(P) (FIELD_bar + B2'_bar), B2_bar = T_bar and
// N_bar = dz T_bar / (1+s); outside it FIELD = 0 and B2 is untouched (B2_bar passes, N_bar = 0).
// P is evaluated in FP64 as the forward epilogue does.
template <typename Rl>
__global__ void lstep_adj_kernel(const C2<Rl>* __restrict__ fb, C2<Rl>* __restrict__ sb, C2<Rl>* __restrict__ b1b,
                                 int nt, size_t total, LstepArgs L) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int k = (int)(idx / nt), p = (int)(idx % nt);
    if (!in_window(L, k, p)) {
        b1b[idx] = C2<Rl>{0, 0};
        return;
    }
    const double2 kk = L.wavenum[p];
    const double sq = sqrt_ho(-L.kt2[k] / kk.x / kk.x);
    const double er = L.dz * kk.y, ei = L.dz * (-L.ho[p] - sq * kk.x);
    double sn, cs;
    sincos(ei, &sn, &cs);
    const double m = exp(er);
    const double pr = m * cs, pi = m * sn;
    const C2<Rl> f = fb[idx], s = sb[idx];
    const double gr = (double)f.x + (double)s.x, gi = (double)f.y + (double)s.y;
    const double tr = pr * gr + pi * gi, ti = pr * gi - pi * gr;
    sb[idx] = C2<Rl>{(Rl)tr, (Rl)ti};
    b1b[idx] = C2<Rl>{(Rl)(L.dz * tr / (1 + sq)), (Rl)(L.dz * ti / (1 + sq))};
}

template <typename Rl>
cudaError_t launch_lstep_adj(const typename Vec2<Rl>::T* fb, typename Vec2<Rl>::T* sb, typename Vec2<Rl>::T* b1b,
                             int nr, int nt, const LstepArgs& L, cudaStream_t st, long long* nlaunch) {
    const size_t total = (size_t)nr * nt;
    lstep_adj_kernel<Rl><<<(unsigned)((total + 255) / 256), 256, 0, st>>>(fb, sb, b1b, nt, total, L);
    (*nlaunch)++;
    return cudaGetLastError();
}
template cudaError_t launch_lstep_adj<double>(const double2*, double2*, double2*, int, int, const LstepArgs&,
                                              cudaStream_t, long long*);
template cudaError_t launch_lstep_adj<float>(const float2*, float2*, float2*, int, int, const LstepArgs&,
                                             cudaStream_t, long long*);

}  // namespace gs
