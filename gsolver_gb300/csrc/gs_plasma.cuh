// gs_plasma.cuh -- device pieces of the plasma response shared by the NL kernels.
#pragma once
#include "gs_internal.cuh"

namespace gs {

// solver.h:55-107 constants of the ionization table
#define GS_ION_TOL 0.003304003148325
#define GS_ION_MIN_LN 29.933606208922594
#define GS_INT_DENOM_LN 36.841361487904734

// photoionization_function without the rho > rho_n test (ionization.cpp:98-147,
// KELDYSH solid branch): 0 below 1e13 W/m^2, log-interpolated table above.
template <typename Rl>
__device__ __forceinline__ Rl photo_rate(Rl I, const Rl* __restrict__ tab, unsigned* err) {
    if (I < (Rl)(1e13 / 1e16)) return (Rl)0;
    Rl lnI = log(I) + (Rl)GS_INT_DENOM_LN;
    if (isnan(lnI)) { atomicOr(err, ERRBIT_NAN); return (Rl)0; }
    int n = (int)floor((lnI - (Rl)GS_ION_MIN_LN) / (Rl)GS_ION_TOL);
    if (n > 8192 - 2) { atomicOr(err, ERRBIT_BLAST); return (Rl)0; }
    if (n < 0) return (Rl)0;
    Rl lnIn = (Rl)GS_ION_MIN_LN + n * (Rl)GS_ION_TOL;
    Rl w0 = __ldg(&tab[n]), w1 = __ldg(&tab[n + 1]);
    Rl lnW = w0 + (lnI - lnIn) * (w1 - w0) / (Rl)GS_ION_TOL;
    return exp(lnW);
}

// photo_rate split in two so that a batch of table reads can be issued together: returns the
// table index n (-1 where the rate is 0) and dl = lnI - lnI_n; the rate is then
// photo_rate_from(tab[n], tab[n + 1], dl), bit-identical to photo_rate.
template <typename Rl>
__device__ __forceinline__ int photo_index(Rl I, Rl* dl, unsigned* err) {
    if (I < (Rl)(1e13 / 1e16)) return -1;
    Rl lnI = log(I) + (Rl)GS_INT_DENOM_LN;
    if (isnan(lnI)) { atomicOr(err, ERRBIT_NAN); return -1; }
    int n = (int)floor((lnI - (Rl)GS_ION_MIN_LN) / (Rl)GS_ION_TOL);
    if (n > 8192 - 2) { atomicOr(err, ERRBIT_BLAST); return -1; }
    if (n < 0) return -1;
    *dl = lnI - ((Rl)GS_ION_MIN_LN + n * (Rl)GS_ION_TOL);
    return n;
}
template <typename Rl>
__device__ __forceinline__ Rl photo_rate_from(Rl w0, Rl w1, Rl dl) {
    return exp(w0 + dl * (w1 - w0) / (Rl)GS_ION_TOL);
}

// One Heun step of the carrier density (ionization.cpp:29-40) from rho with rates (W0, g0)
// at the previous sample and (W1, g1) at this one (g = AV I / (U + P I)); returns the new
// density and multiplies *d by d(new)/d(rho).
template <typename Rl>
__device__ __forceinline__ Rl heun_step(Rl ro, Rl W0, Rl g0, Rl W1, Rl g1, Rl tstep, Rl ND, Rl invND, Rl invTAU,
                                        Rl* d) {
    const bool in1 = !(ro < 0 || ro > ND);
    const Rl W01 = (ro > ND) ? (Rl)0 : W0;
    Rl av = in1 ? g0 * ro * (1 - ro * invND) : (Rl)0;
    Rl rc = (ro > 0) ? ro * invTAU : (Rl)0;
    const Rl k1 = tstep * (W01 + av - rc);
    // derivatives for Newton's method only: at rho = 0 exactly the recombination term's
    // one-sided slope from above (rho >= 0 on every trajectory; the values are continuous
    // there, so nothing computed changes)
    const Rl dk1 = tstep * ((in1 ? g0 * (1 - 2 * ro * invND) : (Rl)0) - ((ro >= 0) ? invTAU : (Rl)0));
    const Rl r2 = ro + k1;
    const bool in2 = !(r2 < 0 || r2 > ND);
    const Rl W11 = (r2 > ND) ? (Rl)0 : W1;
    av = in2 ? g1 * r2 * (1 - r2 * invND) : (Rl)0;
    rc = (r2 > 0) ? r2 * invTAU : (Rl)0;
    const Rl k2 = tstep * (W11 + av - rc);
    const Rl dk2 = tstep * ((in2 ? g1 * (1 - 2 * r2 * invND) : (Rl)0) - ((r2 >= 0) ? invTAU : (Rl)0)) * (1 + dk1);
    Rl rn = ro + (Rl)0.5 * (k1 + k2);
    Rl dn = 1 + (Rl)0.5 * (dk1 + dk2);
    if (rn > ND) { rn = ND; dn = 0; }
    *d *= dn;
    return rn;
}

// One step of the gas build's ionization with one level (ionization.cpp:45-60): taken only
// where the previous sample is above IONIZATION_MIN_I (W0 >= 0; below it W0 carries -1);
// k1 = dt W0 (rho_n - rho), k2 = dt W1 (rho_n - rho - k1), each clamped at 0;
// rho' = min(rho + (k1 + k2)/2, rho_n).  Multiplies *d by d rho'/d rho.
template <typename Rl>
__device__ __forceinline__ Rl gas_step(Rl ro, Rl W0, Rl W1, Rl tstep, Rl ND, Rl* d) {
    if (W0 < 0) return ro;
    W1 = W1 < 0 ? (Rl)0 : W1;
    Rl k1 = tstep * W0 * (ND - ro);
    Rl dk1 = -tstep * W0;
    if (k1 < 0) { k1 = 0; dk1 = 0; }
    Rl k2 = tstep * W1 * (ND - ro - k1);
    Rl dk2 = -tstep * W1 * (1 + dk1);
    if (k2 < 0) { k2 = 0; dk2 = 0; }
    Rl rn = ro + (Rl)0.5 * (k1 + k2);
    Rl dn = 1 + (Rl)0.5 * (dk1 + dk2);
    if (rn > ND) { rn = ND; dn = 0; }
    *d *= dn;
    return rn;
}

// Gas-build rate slot of a sample: W(I) where the sample is above IONIZATION_MIN_I (and not
// the first one, which the recurrence takes as E_0 = 0), -1 otherwise.
template <typename Rl>
__device__ __forceinline__ Rl gas_rate_slot(int t, Rl I, Rl W) {
    return (t > 0 && I > (Rl)(1e13 / 1e16)) ? W : (Rl)-1;
}

// loss factor of the gas build at a sample above the threshold (ionization.cpp:60):
// -(k1/dt)/2 (U + P I)/I, k1 = dt W (rho_n - rho) clamped at 0
template <typename Rl>
__device__ __forceinline__ Rl gas_loss_factor(Rl W, Rl ro, Rl I, Rl tstep, Rl ND, Rl U, Rl Pc) {
    Rl k1 = tstep * W * (ND - ro);
    if (k1 < 0) k1 = 0;
    return -(Rl)0.5 * k1 / tstep * (U + Pc * I) / I;
}

// ---- derivatives for the adjoint -------------------------------------------------------
// Per-sample rates of one Heun step and their intensity derivatives: the photoionization
// rate W (log-linear table: dW/dI = W slope / I) and the avalanche prefactor
// g = AV I / (U + P I) (dg/dI = AV U / (U + P I)^2).  Invalid intensities give 0 (the
// forward reports them).
template <typename Rl> struct RateD { Rl W, dW, g, dg; };

template <typename Rl>
__device__ __forceinline__ RateD<Rl> rate_with_derivs(Rl I, const Rl* __restrict__ tab, Rl U, Rl Pc, Rl AV) {
    RateD<Rl> r{0, 0, 0, 0};
    const Rl den = U + Pc * I;
    r.g = AV / den * I;
    r.dg = AV * U / (den * den);
    if (!(I >= (Rl)(1e13 / 1e16))) return r;
    const Rl lnI = log(I) + (Rl)GS_INT_DENOM_LN;
    const int n = (int)floor((lnI - (Rl)GS_ION_MIN_LN) / (Rl)GS_ION_TOL);
    if (n < 0 || n > 8192 - 2) return r;
    const Rl w0 = __ldg(&tab[n]), w1 = __ldg(&tab[n + 1]);
    r.W = photo_rate_from<Rl>(w0, w1, lnI - ((Rl)GS_ION_MIN_LN + n * (Rl)GS_ION_TOL));
    r.dW = r.W * ((w1 - w0) / (Rl)GS_ION_TOL) / I;
    return r;
}

// Partial derivatives of heun_step (same branches): d = d rho_t / d rho_{t-1},
// a = d rho_t / d I_{t-1}, b = d rho_t / d I_t; all 0 where the density is clamped at rho_n.
template <typename Rl>
__device__ __forceinline__ void heun_partials(Rl ro, const RateD<Rl>& r0, const RateD<Rl>& r1, Rl tstep, Rl ND,
                                              Rl invND, Rl invTAU, Rl* d, Rl* a, Rl* b) {
    const bool in1 = !(ro < 0 || ro > ND);
    const Rl W01 = (ro > ND) ? (Rl)0 : r0.W, dW01 = (ro > ND) ? (Rl)0 : r0.dW;
    Rl av = in1 ? r0.g * ro * (1 - ro * invND) : (Rl)0;
    Rl rc = (ro > 0) ? ro * invTAU : (Rl)0;
    const Rl k1 = tstep * (W01 + av - rc);
    const Rl k1r = tstep * ((in1 ? r0.g * (1 - 2 * ro * invND) : (Rl)0) - ((ro > 0) ? invTAU : (Rl)0));
    const Rl k1I = tstep * (dW01 + (in1 ? r0.dg * ro * (1 - ro * invND) : (Rl)0));
    const Rl r2 = ro + k1;
    const bool in2 = !(r2 < 0 || r2 > ND);
    const Rl W11 = (r2 > ND) ? (Rl)0 : r1.W, dW11 = (r2 > ND) ? (Rl)0 : r1.dW;
    av = in2 ? r1.g * r2 * (1 - r2 * invND) : (Rl)0;
    rc = (r2 > 0) ? r2 * invTAU : (Rl)0;
    const Rl k2 = tstep * (W11 + av - rc);
    const Rl k2r = tstep * ((in2 ? r1.g * (1 - 2 * r2 * invND) : (Rl)0) - ((r2 > 0) ? invTAU : (Rl)0));
    const Rl k2I = tstep * (dW11 + (in2 ? r1.dg * r2 * (1 - r2 * invND) : (Rl)0));
    if (ro + (Rl)0.5 * (k1 + k2) > ND) {
        *d = 0; *a = 0; *b = 0;
        return;
    }
    *d = 1 + (Rl)0.5 * (k1r + k2r * (1 + k1r));
    *a = (Rl)0.5 * k1I * (1 + k2r);
    *b = (Rl)0.5 * k2I;
}

// Block-wide inclusive scan of affine maps x -> A x + B (composition left to right, i.e.
// thread c ends with map_c o ... o map_0).  T is the real type or a complex struct with
// the mul/add helpers below; sA/sB hold 32 entries.  All threads must call it.
template <typename T> __device__ __forceinline__ T amul(T a, T b);
template <> __device__ __forceinline__ float amul<float>(float a, float b) { return a * b; }
template <> __device__ __forceinline__ double amul<double>(double a, double b) { return a * b; }
template <> __device__ __forceinline__ float2 amul<float2>(float2 a, float2 b) { return cmul(a, b); }
template <> __device__ __forceinline__ double2 amul<double2>(double2 a, double2 b) { return cmul(a, b); }
template <typename T> __device__ __forceinline__ T aadd(T a, T b);
template <> __device__ __forceinline__ float aadd<float>(float a, float b) { return a + b; }
template <> __device__ __forceinline__ double aadd<double>(double a, double b) { return a + b; }
template <> __device__ __forceinline__ float2 aadd<float2>(float2 a, float2 b) { return cadd(a, b); }
template <> __device__ __forceinline__ double2 aadd<double2>(double2 a, double2 b) { return cadd(a, b); }
template <typename T> __device__ __forceinline__ T shfl_up(T v, int o);
template <> __device__ __forceinline__ float shfl_up<float>(float v, int o) { return __shfl_up_sync(0xffffffffu, v, o); }
template <> __device__ __forceinline__ double shfl_up<double>(double v, int o) { return __shfl_up_sync(0xffffffffu, v, o); }
template <> __device__ __forceinline__ float2 shfl_up<float2>(float2 v, int o) {
    return make_float2(__shfl_up_sync(0xffffffffu, v.x, o), __shfl_up_sync(0xffffffffu, v.y, o));
}
template <> __device__ __forceinline__ double2 shfl_up<double2>(double2 v, int o) {
    return make_double2(__shfl_up_sync(0xffffffffu, v.x, o), __shfl_up_sync(0xffffffffu, v.y, o));
}

template <typename T>
__device__ __forceinline__ void block_affine_scan(T& A, T& B, T one, T zero, T* sA, T* sB) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T pa = shfl_up(A, o), pb = shfl_up(B, o);
        if (lane >= o) { B = aadd(amul(A, pb), B); A = amul(A, pa); }
    }
    if (lane == 31) { sA[wid] = A; sB[wid] = B; }
    __syncthreads();
    if (wid == 0) {
        T xa = lane < nw ? sA[lane] : one, xb = lane < nw ? sB[lane] : zero;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T pa = shfl_up(xa, o), pb = shfl_up(xb, o);
            if (lane >= o) { xb = aadd(amul(xa, pb), xb); xa = amul(xa, pa); }
        }
        sA[lane] = xa;
        sB[lane] = xb;
    }
    __syncthreads();
    if (wid > 0) {
        const T pa = sA[wid - 1], pb = sB[wid - 1];
        B = aadd(amul(A, pb), B);
        A = amul(A, pa);
    }
    __syncthreads();
}

}  // namespace gs
