// gs_nl.cu -- kernels of the nonlinear RK4 increment (calculate_NLstep, propagator.cu:268-426).
//
// One RK4 stage of one radial row is the reference's calculate_NLresponse
// (propagator.cu:629-783): six length-N_T FFTs, the causal plasma recurrence
// (ionization.cpp:9-95) and pointwise spectral products.  Here every piece runs batched
// over all N_r rows:
//   fft_sub_kernel    one CTA per (sub-)row, the row resident in shared memory,
//                     radix-16 register butterflies; fused stage input A + c*dz*k_prev,
//                     max|A|^2, 1/N scaling and the time-domain products.
//   fft_cross_kernel  the radix-P first/last pass when N_T exceeds one CTA's shared
//                     memory (N_T = P * M): coalesced, one thread per (row, n1).
//   plasma_kernel     intensities and rates in parallel, the carrier-density recurrence
//                     sequentially per row (it is not linear: clamps and the quadratic
//                     avalanche term), then loss and rho*E in parallel.
//   spec1/spec2       spectral combination and the RK4 accumulation with max|N|^2.
// Templates instantiate the FP64 parity path (double) and the mixed path (float).
#include "gs_internal.cuh"
#include "gs_kernels.h"
#include "gs_plasma.cuh"

namespace gs {

// ------------------------------------------------------------------ FFT kernels --
// Spectral-side load ops (inverse transforms) and time-side ops.
enum { SPRE_NONE = 0, SPRE_STAGE = 1 };
enum { TPOST_STORE = 0, TPOST_DIVN = 1, TPOST_DIVN_MULE = 2 };

// shared memory of fft_sub_kernel: the padded row, then the two twiddle tables
template <typename Rl> __host__ __device__ inline size_t fft_smem_bytes(int M, int N) {
    return ((size_t)padded_len(M) + N / 64 + 64) * sizeof(typename Vec2<Rl>::T);
}

template <typename Rl, int SIGN>
__global__ void __launch_bounds__(sizeof(Rl) == 8 ? 512 : 1024) fft_sub_kernel(const C2<Rl>* __restrict__ in,
                                                                              C2<Rl>* __restrict__ out, FftArgs<Rl> a) {
    using T2 = C2<Rl>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* buf = reinterpret_cast<T2*>(smem_raw);
    const int M = a.M;
    T2* twh = buf + padded_len(M);
    T2* twl = twh + a.N / 64;
    const size_t base = (size_t)blockIdx.x * M;   // sub-rows are contiguous blocks of M
    const int tid = threadIdx.x, nthr = blockDim.x;
    load_twiddles<Rl>(twh, twl, a.tw, a.N, tid, nthr);

    // ---- load (with the spectral-side op for inverse transforms)
    Rl lmax = 0;
    for (int i = tid; i < M; i += nthr) {
        T2 v = in[base + i];
        if (SIGN > 0 && a.spre == SPRE_STAGE) {
            if (a.track_max) lmax = fmax(lmax, v.x * v.x + v.y * v.y);
            if (a.cdz != 0) {
                T2 k = a.kp[base + i];
                v.x = v.x + (Rl)a.cdz * k.x;
                v.y = v.y + (Rl)a.cdz * k.y;
            }
        }
        buf[pad16(i)] = v;
    }
    if (SIGN > 0 && a.track_max) {
        for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
        if ((tid & 31) == 0) atomic_max_nonneg(a.max_out, (double)lmax);
    }
    __syncthreads();
    const TwTab<Rl> tw{twh, twl, a.twb};
    smem_fft<SIGN, Rl>(buf, M, a.logM, tw, a.P, tid, nthr);

    // ---- store (time-side op only when this kernel finishes an inverse transform)
    const Rl rn = (Rl)a.N;
    for (int i = tid; i < M; i += nthr) {
        T2 v = buf[pad16(i)];
        if (SIGN > 0 && a.P == 1 && a.tpost != TPOST_STORE) {
            v.x = v.x / rn;
            v.y = v.y / rn;
            if (a.tpost == TPOST_DIVN_MULE) v = cmul(v, a.e[base + i]);
        }
        out[base + i] = v;
    }
}

template <typename Rl, int SIGN, int P>
__global__ void __launch_bounds__(256) fft_cross_kernel(const C2<Rl>* __restrict__ in, C2<Rl>* __restrict__ out,
                                                        FftArgs<Rl> a) {
    using T2 = C2<Rl>;
    const int M = a.M;
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = (size_t)a.rows * M;
    if (idx >= total) return;
    const size_t row = idx / M;
    const int n1 = (int)(idx - row * M);
    const size_t base = row * (size_t)a.N;
    T2 x[P];
    if (SIGN < 0) {
        // forward: y_k2[n1] = w_N^{n1 k2} sum_n2 x[n1 + M n2] w_P^{n2 k2}, stored at k2*M + n1
#pragma unroll
        for (int n2 = 0; n2 < P; n2++) x[n2] = in[base + n1 + (size_t)M * n2];
        RegDFT<P, -1, Rl, T2>::run(x);
#pragma unroll
        for (int k2 = 1; k2 < P; k2++) x[k2] = cmul(x[k2], __ldg(&a.tw[n1 * k2]));
#pragma unroll
        for (int k2 = 0; k2 < P; k2++) out[base + (size_t)k2 * M + n1] = x[k2];
    } else {
        // inverse: x[n1 + M n2] = sum_k2 w_P^{-n2 k2} (w_N^{-n1 k2} z_k2[n1])
#pragma unroll
        for (int k2 = 0; k2 < P; k2++) x[k2] = in[base + (size_t)k2 * M + n1];
#pragma unroll
        for (int k2 = 1; k2 < P; k2++) x[k2] = cmul(x[k2], cconj(__ldg(&a.tw[n1 * k2])));
        RegDFT<P, +1, Rl, T2>::run(x);
        const Rl rn = (Rl)a.N;
#pragma unroll
        for (int n2 = 0; n2 < P; n2++) {
            T2 v = x[n2];
            const size_t o = base + n1 + (size_t)M * n2;
            if (a.tpost != TPOST_STORE) {
                v.x = v.x / rn;
                v.y = v.y / rn;
                if (a.tpost == TPOST_DIVN_MULE) v = cmul(v, a.e[o]);
            }
            out[o] = v;
        }
    }
}

// ------------------------------------------------------------------- plasma ----
// The gas build's MULTI_LEVEL_IONIZATION branch of calculate_plasmadensity_losses_small
// (ionization.cpp:19-24, 45-84) for one row per CTA: per sample nt >= 1 whose predecessor is
// above IONIZATION_MIN_I, level 0 takes a Heun step towards the neutral density and level n >= 1
// one towards level n - 1 (already stepped), each clamped by what it moves towards; the density
// is the levels' sum, the loss factor at sample nt - 1 sums -k1_n / 2 / dt (U_n + P I) / I over
// the levels.  Level n's recurrence is scalar once level n - 1 is known along the row, so the
// levels are solved in turn, each by the multiple shooting of the single-level recurrence
// (Newton on the chunk starts, exact after chunks + 1 iterations).  Scratch per sample: U1 =
// (table index or -1, ln-intensity offset), U3 = (level n's rate or -1, level n - 1's density);
// U2 accumulates (loss factor, density).  Leaves U1 = loss E, U2 = density E (density in U2.x
// when a.density_only).
template <typename Rl>
__device__ void plasma_levels(const PlasmaArgs<Rl>& a) {
    using T2 = C2<Rl>;
    __shared__ Rl s_start[256], sA[256], sB[256], red[64];
    __shared__ int s_done;
    const int N = a.N;
    const size_t base = (size_t)blockIdx.x * N;
    const T2* E = a.e + base;
    T2* U1 = a.u1 + base;
    T2* U2 = a.u2 + base;
    T2* U3 = a.u3 + base;
    Rl* u1 = reinterpret_cast<Rl*>(U1);   // scalar views: the x / y halves written apart
    Rl* u2 = reinterpret_cast<Rl*>(U2);
    Rl* u3 = reinterpret_cast<Rl*>(U3);
    const int tid = threadIdx.x, nthr = blockDim.x;
    const Rl ND = a.k.ND, tstep = a.k.tstep, Pc = a.k.Pc;
    const Rl thr = (Rl)(1e13 / 1e16);
    bool any = false;
    for (int t = tid; t < N; t += nthr) {
        Rl nn = -1, dl = 0;
        if (t > 0) {
            const T2 e = E[t];
            const Rl I = e.x * e.x + e.y * e.y;
            Rl d = 0;
            const int n = photo_index<Rl>(I, &d, a.err);
            if (n >= 0 && I > thr) {   // as the single-level slot: a step is taken from this sample
                nn = (Rl)n;
                dl = d;
                any = true;
            }
        }
        U1[t] = T2{nn, dl};
        U2[t] = T2{(Rl)0, (Rl)0};
        u3[2 * t + 1] = ND;   // level 0 moves towards the neutral density
    }
    const bool ion = __syncthreads_or(any ? 1 : 0) != 0;
    const int P = min(nthr, N);
    const int L = N / P;
    const int c = tid;
    const int lane = tid & 31, wid = tid >> 5;
    const Rl tol = sizeof(Rl) == 8 ? (Rl)1e-13 : (Rl)1e-5;
    for (int lv = 0; lv < (ion ? a.levels : 0); lv++) {
        const Rl* tab = a.rate + (size_t)lv * 8192;
        const Rl pot = a.k.pot[lv];
        for (int t = tid; t < N; t += nthr) {   // level lv's rate per sample (-1: no step from it)
            const Rl nn = u1[2 * t];
            Rl W = -1;
            if (nn >= 0) {
                const int n = (int)nn;
                W = photo_rate_from<Rl>(__ldg(&tab[n]), __ldg(&tab[n + 1]), u1[2 * t + 1]);
            }
            u3[2 * t] = W;
        }
        __syncthreads();
        // the chunk of steps [c L, c L + L) from start s; write: the final pass (density,
        // loss factor, this level's density as the next level's target)
        auto run_chunk = [&](Rl s, bool write, Rl* dout) -> Rl {
            Rl ro = s, d = 1;
            const int nt0 = c * L;
            Rl W0 = nt0 > 0 ? u3[2 * (nt0 - 1)] : (Rl)-1;
            for (int i = 0; i < L; i++) {
                const int nt = nt0 + i;
                const Rl W1 = u3[2 * nt];
                if (nt > 0) {
                    const Rl src = u3[2 * nt + 1];
                    const Rl r0 = ro;
                    ro = gas_step<Rl>(ro, W0, W1, tstep, src, &d);
                    if (write) {
                        if (W0 >= 0) {   // k1 of this level's step: the loss at sample nt - 1
                            Rl k1 = tstep * W0 * (src - r0);
                            if (k1 < 0) k1 = 0;
                            const T2 e = E[nt - 1];
                            const Rl I0 = e.x * e.x + e.y * e.y;
                            u2[2 * (nt - 1)] -= (Rl)0.5 * k1 / tstep * (pot + Pc * I0) / I0;
                        }
                        u2[2 * nt + 1] += ro;
                        u3[2 * nt + 1] = ro;
                    }
                }
                W0 = W1;
            }
            if (dout) *dout = d;
            return ro;
        };
        if (c < P) s_start[c] = 0;
        if (tid == 0) s_done = 0;
        __syncthreads();
        for (int it = 0; it < P + 1; it++) {
            Rl A = 1, B = 0;
            if (c < P) {
                const Rl sc = s_start[c];
                Rl D;
                const Rl e = run_chunk(sc, false, &D);
                A = D;
                B = e - D * sc;
            }
            for (int o = 1; o < 32; o <<= 1) {
                const Rl pa = __shfl_up_sync(0xffffffffu, A, o), pb = __shfl_up_sync(0xffffffffu, B, o);
                if (lane >= o) { B = A * pb + B; A = A * pa; }
            }
            if (lane == 31) { sA[wid] = A; sB[wid] = B; }
            __syncthreads();
            if (wid == 0) {
                const int nw = nthr >> 5;
                Rl wa = lane < nw ? sA[lane] : (Rl)1, wb = lane < nw ? sB[lane] : (Rl)0;
                for (int o = 1; o < 32; o <<= 1) {
                    const Rl pa = __shfl_up_sync(0xffffffffu, wa, o), pb = __shfl_up_sync(0xffffffffu, wb, o);
                    if (lane >= o) { wb = wa * pb + wb; wa = wa * pa; }
                }
                if (lane < nw) { sA[lane] = wa; sB[lane] = wb; }
            }
            __syncthreads();
            if (wid > 0) {
                const Rl pa = sA[wid - 1], pb = sB[wid - 1];
                B = A * pb + B;
                A = A * pa;
            }
            const Rl next = A * s_start[0] + B;   // the start of chunk c + 1
            __syncthreads();
            Rl change = 0, mag = 0;
            if (c + 1 < P) {
                change = fabs(next - s_start[c + 1]);
                mag = fabs(next);
                s_start[c + 1] = next;
            }
            for (int o = 16; o > 0; o >>= 1) {
                change = fmax(change, __shfl_xor_sync(0xffffffffu, change, o));
                mag = fmax(mag, __shfl_xor_sync(0xffffffffu, mag, o));
            }
            if (lane == 0) { red[wid] = change; red[32 + wid] = mag; }
            __syncthreads();
            if (tid == 0) {
                Rl cm = 0, mm = 0;
                for (int w = 0; w < (nthr >> 5); w++) { cm = fmax(cm, red[w]); mm = fmax(mm, red[32 + w]); }
                s_done = (cm <= tol * mm && !a.shoot_exhaust) ? 1 : 0;
            }
            __syncthreads();
            if (s_done) break;
        }
        if (c < P) run_chunk(s_start[c], true, nullptr);
        __syncthreads();
    }
    for (int t = tid; t < N; t += nthr) {
        const T2 e = E[t];
        const Rl tl = ion ? u2[2 * t] : (Rl)0, rho = ion ? u2[2 * t + 1] : (Rl)0;
        U1[t] = t < N - 1 ? T2{tl * e.x, tl * e.y} : T2{0, 0};
        U2[t] = a.density_only ? T2{rho, (Rl)0} : T2{rho * e.x, rho * e.y};
    }
    __syncthreads();
}

// calculate_plasmadensity_losses_small (ionization.cpp:9-95), single-level branch, for
// one row per CTA.  Inputs: E (time row).  Outputs: U1 = loss, U2 = rho*E,
// U3 = |E|^2 (Raman on) or |E|^2 * E (Raman off).  The first recurrence step sees
// E_0 = 0 as the reference does (ionization.cpp:25).
template <typename Rl>
__global__ void __launch_bounds__(256) plasma_kernel(PlasmaArgs<Rl> a) {
    using T2 = C2<Rl>;
    __shared__ Rl sW[256], sG[256], sR[256];
    const int N = a.N;
    const size_t base = (size_t)blockIdx.x * N;
    const T2* E = a.e + base;
    T2* U1 = a.u1 + base;
    T2* U2 = a.u2 + base;
    T2* U3 = a.u3 + base;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const Rl ND = a.k.ND, tstep = a.k.tstep, U = a.k.U, Pc = a.k.Pc, AV = a.k.AV;
    // several ionization levels: density and loss by plasma_levels (U1 = loss E, U2 = rho E);
    // the Kerr / Raman source below is common
    const bool ml = a.levels > 1;
    if (ml) {
        plasma_levels<Rl>(a);
        if (a.density_only) return;
    }

    // phase A: W_t and the avalanche prefactor g_t = AV/(U + P I_t) * I_t (t >= 1)
    const bool gas = a.gas != 0;
    bool anyw = false;
    for (int t = tid; t < N && !ml; t += nthr) {
        Rl W = 0, g = 0;
        if (t > 0) {
            T2 e = E[t];
            Rl I = e.x * e.x + e.y * e.y;
            W = photo_rate<Rl>(I, a.rate, a.err);
            anyw = anyw || W > (Rl)0;
            g = AV / (U + Pc * I) * I;
            if (gas) W = gas_rate_slot<Rl>(t, I, W);
        } else if (gas) {
            W = (Rl)-1;   // the recurrence starts from E_0 = 0
        }
        U1[t] = T2{W, g};
    }
    // no sample with W > 0 and rho starting at 0: every step adds exactly 0, the density
    // stays 0 along the row and the recurrence below is skipped
    const bool ion = (__syncthreads_or(anyw ? 1 : 0) != 0 || a.k.rho0 != (Rl)0) && !ml;

    // phase B: the Heun recurrence by multiple shooting.  Thread c owns the L consecutive
    // steps nt in [c L, c L + L); its start value s_c = rho_{cL-1} is refined by Newton
    // iterations: every thread runs its chunk exactly from s_c (end e_c, derivative D_c),
    // then s_{c+1} <- e_c + D_c (s_c' - s_c) is an affine recurrence over the chunks,
    // solved by a block scan.  Quadratic convergence (the map is affine up to the small
    // avalanche rho^2 term and the clamps); the last pass writes rho with the converged
    // starts, i.e. the sequential recurrence up to rounding.
    const int P = min(nthr, N);
    const int L = N / P;
    const Rl invND = a.k.invND, invTAU = a.k.invTAU;
    Rl* s_start = sW;            // [P] chunk start values
    Rl* s_scanA = sG;            // [P] scan scratch
    Rl* s_scanB = sR;            // [P]
    __shared__ Rl red[32];
    __shared__ int s_done;
    const int c = tid;
    auto run_chunk = [&](Rl s0, bool write, Rl* dout) -> Rl {
        Rl ro = s0, d = (Rl)1;
        const int nt0 = c * L;
        T2 w0 = U1[nt0 > 0 ? nt0 - 1 : 0];
#pragma unroll 8
        for (int i = 0; i < L; i++) {
            const int nt = nt0 + i;
            const T2 w1 = U1[nt];
            if (nt > 0 && gas) {
                ro = gas_step<Rl>(ro, w0.x, w1.x, tstep, ND, &d);
                if (write) { T2 v = U2[nt]; v.x = ro; U2[nt] = v; }
            } else if (nt > 0) {
                const Rl W0 = w0.x, g0 = w0.y, W1 = w1.x, g1 = w1.y;
                const bool in1 = !(ro < 0 || ro > ND);
                Rl W01 = (ro > ND) ? (Rl)0 : W0;
                Rl av = in1 ? g0 * ro * (1 - ro * invND) : (Rl)0;
                Rl rc = (ro > 0) ? ro * invTAU : (Rl)0;
                Rl k1 = tstep * (W01 + av - rc);
                // Newton derivative: one-sided slope from above at rho = 0 (values unchanged)
                Rl dk1 = tstep * ((in1 ? g0 * (1 - 2 * ro * invND) : (Rl)0) - ((ro >= 0) ? invTAU : (Rl)0));
                Rl r2 = ro + k1;
                const bool in2 = !(r2 < 0 || r2 > ND);
                Rl W11 = (r2 > ND) ? (Rl)0 : W1;
                av = in2 ? g1 * r2 * (1 - r2 * invND) : (Rl)0;
                rc = (r2 > 0) ? r2 * invTAU : (Rl)0;
                Rl k2 = tstep * (W11 + av - rc);
                Rl dk2 = tstep * ((in2 ? g1 * (1 - 2 * r2 * invND) : (Rl)0) - ((r2 >= 0) ? invTAU : (Rl)0)) * (1 + dk1);
                ro += (Rl)0.5 * (k1 + k2);
                d *= 1 + (Rl)0.5 * (dk1 + dk2);
                if (ro > ND) { ro = ND; d = 0; }
                if (write) { T2 v = U2[nt]; v.x = ro; U2[nt] = v; }
            } else if (write) {
                T2 v = U2[0]; v.x = ro; U2[0] = v;
            }
            w0 = w1;
        }
        if (dout) *dout = d;
        return ro;
    };
    if (c < P) s_start[c] = (c == 0) ? a.k.rho0 : (Rl)0;
    if (tid == 0) s_done = 0;
    __syncthreads();
    // stop when the starts move less than tol (relative): Newton converges quadratically, so
    // the starts then carry ~tol^2 + rounding; far below the parity bars (1e-10 / 1e-5).  After
    // k iterations the starts of chunks 0..k equal the sequential recurrence's (each computed
    // from an exact predecessor), so P + 1 iterations bound the loop with an exact result
    const Rl tol = sizeof(Rl) == 8 ? (Rl)1e-13 : (Rl)1e-5;
    for (int it = 0; it < (ion ? P + 1 : 0); it++) {
        Rl A = 1, B = 0, sc = 0;
        if (c < P) {
            sc = s_start[c];
            Rl D;
            const Rl e = run_chunk(sc, false, &D);
            A = D;
            B = e - D * sc;             // s_{c+1}' = A s_c' + B
        }
        // inclusive scan of the maps x -> A x + B, composed left to right over the chunks
        const int lane = tid & 31, wid = tid >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            const Rl pa = __shfl_up_sync(0xffffffffu, A, o), pb = __shfl_up_sync(0xffffffffu, B, o);
            if (lane >= o) { B = A * pb + B; A = A * pa; }
        }
        if (lane == 31) { s_scanA[wid] = A; s_scanB[wid] = B; }
        __syncthreads();
        if (wid == 0) {
            const int nw = nthr >> 5;
            Rl wa = lane < nw ? s_scanA[lane] : (Rl)1, wb = lane < nw ? s_scanB[lane] : (Rl)0;
            for (int o = 1; o < 32; o <<= 1) {
                const Rl pa = __shfl_up_sync(0xffffffffu, wa, o), pb = __shfl_up_sync(0xffffffffu, wb, o);
                if (lane >= o) { wb = wa * pb + wb; wa = wa * pa; }
            }
            if (lane < nw) { s_scanA[lane] = wa; s_scanB[lane] = wb; }
        }
        __syncthreads();
        if (wid > 0) {   // prepend the prefix of the previous warps
            const Rl pa = s_scanA[wid - 1], pb = s_scanB[wid - 1];
            B = A * pb + B;
            A = A * pa;
        }
        const Rl s0 = s_start[0];
        const Rl next = A * s0 + B;     // new start of chunk c + 1
        __syncthreads();
        Rl change = 0, mag = 0;
        if (c + 1 < P) {
            const Rl old = s_start[c + 1];
            change = fabs(next - old);
            mag = fabs(next);
            s_start[c + 1] = next;
        }
        // block max of change and magnitude
        for (int o = 16; o > 0; o >>= 1) {
            change = fmax(change, __shfl_xor_sync(0xffffffffu, change, o));
            mag = fmax(mag, __shfl_xor_sync(0xffffffffu, mag, o));
        }
        if (lane == 0) { red[wid] = change; red[16 + wid] = mag; }
        __syncthreads();
        if (tid == 0) {
            Rl cm = 0, mm = 0;
            for (int w = 0; w < (nthr >> 5); w++) { cm = fmax(cm, red[w]); mm = fmax(mm, red[16 + w]); }
            s_done = (cm <= tol * mm && !a.shoot_exhaust) ? 1 : 0;
        }
        __syncthreads();
        if (s_done) break;
    }
    if (ion && c < P) run_chunk(s_start[c], true, nullptr);
    __syncthreads();

    // phase C: loss[t] (uses W_t, I_t, rho_t at step t+1), rho*E, intensity terms
    if (a.density_only && !ion)
        for (int t = tid; t < N; t += nthr) U2[t] = T2{0, 0};
    if (a.density_only) return;
    for (int t = tid; t < N; t += nthr) {
        T2 e = E[t];
        const Rl rho = ion ? U2[t].x : (Rl)0;
        T2 w = ml ? T2{0, 0} : U1[t];
        T2 loss = T2{0, 0};
        if (ml) {
            // U1, U2 written by plasma_levels
        } else if (gas) {
            // loss[t] = tl E_t (ionization.cpp:60-81), where sample t is above the threshold
            if (t < N - 1 && w.x >= 0) {
                const Rl I0 = e.x * e.x + e.y * e.y;
                const Rl s = gas_loss_factor<Rl>(w.x, rho, I0, tstep, ND, U, Pc);
                loss = T2{s * e.x, s * e.y};
            }
        } else if (t < N - 1 && t > 0) {
            Rl I0 = e.x * e.x + e.y * e.y;
            Rl W01 = (rho > ND) ? (Rl)0 : w.x;
            // the reference compares the intensity with the log threshold (ionization.cpp:43)
            if (I0 > (Rl)GS_ION_MIN_LN) {
                Rl s = -(Rl)0.5 * W01 * (U + Pc * I0) / I0;
                loss = T2{s * e.x, s * e.y};
            }
        }
        if (!ml) {
            U1[t] = loss;
            U2[t] = T2{rho * e.x, rho * e.y};
        }
        Rl I = e.x * e.x + e.y * e.y;
        if (!a.raman_scan) {
            T2 src = a.raman ? T2{I, (Rl)0} : T2{I * e.x - (Rl)0 * e.y, I * e.y + (Rl)0 * e.x};
            if (a.th && !a.raman) {   // third harmonic: + th_t E^3 (the Kerr profile, scaled)
                const T2 h = cmul(a.th[t], cmul(cmul(e, e), e));
                src.x += h.x;
                src.y += h.y;
            }
            U3[t] = src;
        }
    }
    if (!a.raman_scan) return;

    // phase D: the delayed Kerr source Q = (1 - f_R) I + h (*) I without FFTs.  The
    // reference forms IFFT(FFT(I) R)/N with R = FFT(h) + 1 - f_R (solver_main.cpp:401-413,
    // propagator.cu:697-705): a circular convolution with h_k = fRM Im(a^k).  With the
    // causal one-pole sum z_t = a z_{t-1} + I_t it is exactly
    //     (h (*) I)_t = fRM Im((1 - a^N) z_t + a^{t+1} z_{N-1}),
    // and z is a linear recurrence: chunk-local sums, an exclusive scan of chunk starts
    // (complex affine maps with the common multiplier a^L), then a second chunk pass.
    __syncthreads();
    const T2 ra = T2{a.k.a_re, a.k.a_im};
    T2 zl = T2{0, 0};
    T2 aL = T2{1, 0};
    if (c < P) {
        for (int i = 0; i < L; i++) {
            const T2 e = E[c * L + i];
            zl = cmul(ra, zl);
            zl.x += e.x * e.x + e.y * e.y;
            aL = cmul(aL, ra);
        }
    }
    // exclusive scan over chunks: start_{c+1} = aL * start_c + zl_c
    {
        T2 A = aL, B = zl;
        const int lane = tid & 31, wid = tid >> 5;
        if (c >= P) { A = T2{1, 0}; B = T2{0, 0}; }
        for (int o = 1; o < 32; o <<= 1) {
            T2 pa, pb;
            pa.x = __shfl_up_sync(0xffffffffu, A.x, o); pa.y = __shfl_up_sync(0xffffffffu, A.y, o);
            pb.x = __shfl_up_sync(0xffffffffu, B.x, o); pb.y = __shfl_up_sync(0xffffffffu, B.y, o);
            if (lane >= o) { B = cadd(cmul(A, pb), B); A = cmul(A, pa); }
        }
        __shared__ T2 wA[8], wB[8];
        __shared__ T2 zend;
        if (lane == 31) { wA[wid] = A; wB[wid] = B; }
        __syncthreads();
        if (wid == 0) {
            const int nw = nthr >> 5;
            T2 xa = lane < nw ? wA[lane] : T2{1, 0}, xb = lane < nw ? wB[lane] : T2{0, 0};
            for (int o = 1; o < 32; o <<= 1) {
                T2 pa, pb;
                pa.x = __shfl_up_sync(0xffffffffu, xa.x, o); pa.y = __shfl_up_sync(0xffffffffu, xa.y, o);
                pb.x = __shfl_up_sync(0xffffffffu, xb.x, o); pb.y = __shfl_up_sync(0xffffffffu, xb.y, o);
                if (lane >= o) { xb = cadd(cmul(xa, pb), xb); xa = cmul(xa, pa); }
            }
            if (lane < nw) { wA[lane] = xa; wB[lane] = xb; }
            if (lane == nw - 1) zend = xb;   // z_{N-1}: all chunks composed from start 0
        }
        __syncthreads();
        if (wid > 0) { B = cadd(cmul(A, wB[wid - 1]), B); }
        // inclusive prefix B = z at the end of chunk c; the start of chunk c is the end of c-1
        __shared__ T2 cend[256];
        cend[tid] = B;
        __syncthreads();
        const T2 zs = (c == 0) ? T2{0, 0} : cend[c - 1];
        const T2 zN = zend;
        if (c < P) {
            const T2 oma = T2{a.k.oma_re, a.k.oma_im};
            // a^{t+1} at the first sample of the chunk, a (a^L)^c by binary powering (the
            // chunks share a^L), then advanced by a
            T2 pw = T2{1, 0};
            {
                T2 b = aL;
                for (int e = c; e > 0; e >>= 1) {
                    if (e & 1) pw = cmul(pw, b);
                    b = cmul(b, b);
                }
                pw = cmul(pw, ra);
            }
            T2 z = zs;
            const Rl fRM = a.k.fRM, omf = a.k.omf;
            for (int i = 0; i < L; i++) {
                const int t = c * L + i;
                const T2 e = E[t];
                const Rl I = e.x * e.x + e.y * e.y;
                z = cmul(ra, z);
                z.x += I;
                const T2 v = cadd(cmul(oma, z), cmul(pw, zN));
                const Rl Q = omf * I + fRM * v.y;
                T2 src = T2{Q * e.x, Q * e.y};
                if (a.th) {
                    const T2 h = cmul(a.th[t], cmul(cmul(e, e), e));
                    src.x += h.x;
                    src.y += h.y;
                }
                U3[t] = src;
                pw = cmul(pw, ra);
            }
        }
    }
}

// ------------------------------------------------------------- spectral ops ----
template <typename Rl>
__global__ void spec1_kernel(SpecArgs<Rl> a) {
    using T2 = C2<Rl>;
    const size_t total = (size_t)a.rows * a.N;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int p = (int)(i % a.N);
        // N = FFT(loss) + FFT(rho E) * PLASMA_FUNC (propagator.cu:679-686)
        a.u1[i] = cadd(a.u1[i], cmul(a.u2[i], a.pf[p]));
        if (a.raman) a.u3[i] = cmul(a.u3[i], a.rm[p]);   // FFT(I) * RAMAN_FUNCTION
    }
}

template <typename Rl>
__global__ void spec2_kernel(SpecArgs<Rl> a) {
    using T2 = C2<Rl>;
    const size_t total = (size_t)a.rows * a.N;
    Rl lmax = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int p = (int)(i % a.N);
        T2 k = a.u1[i];
        // fused spec1 (no FFT Raman pair pending): FFT(loss) + FFT(rho E) * PLASMA_FUNC
        if (a.fuse_plasma) k = cadd(k, cmul(a.u2[i], a.pf[p]));
        if (a.kerr_on) {   // += -j * KERR_PROFILE * FFT(Q E)
            const Rl K = a.kerr[p];
            T2 q = a.u3[i];
            k.x += K * q.y;
            k.y += -K * q.x;
        }
        T2 nb;
        if (a.stage == 0) {
            nb = k;
        } else if (a.stage < 3) {
            T2 o = a.nb[i];
            nb = T2{o.x + (Rl)2 * k.x, o.y + (Rl)2 * k.y};
        } else {
            T2 o = a.nb[i];
            nb = T2{(o.x + k.x) / (Rl)6, (o.y + k.y) / (Rl)6};
            lmax = fmax(lmax, nb.x * nb.x + nb.y * nb.y);
        }
        a.nb[i] = nb;
        if (a.stage < 3) a.kp[i] = k;
    }
    if (a.stage == 3) {
        for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
        if ((threadIdx.x & 31) == 0) atomic_max_nonneg(a.max_out, (double)lmax);
    }
}

// zero NL response (NONLINEARITY_ON undefined): BIGBUFFER1 = 0 and max|A|^2
template <typename Rl>
__global__ void zero_nl_kernel(const C2<Rl>* __restrict__ A, C2<Rl>* __restrict__ nb, size_t total,
                               unsigned long long* max_out) {
    Rl lmax = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        C2<Rl> v = A[i];
        lmax = fmax(lmax, v.x * v.x + v.y * v.y);
        nb[i] = C2<Rl>{0, 0};
    }
    for (int o = 16; o > 0; o >>= 1) lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(max_out, (double)lmax);
}

// natural <-> position order, with precision conversion from / to FP64 staging
template <typename Rl>
__global__ void permute_in_kernel(const double2* __restrict__ src, C2<Rl>* __restrict__ dst,
                                  const int* __restrict__ perm, int N, size_t total) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t row = i / N;
        const int p = (int)(i - row * N);
        double2 v = src[row * N + perm[p]];
        dst[i] = C2<Rl>{(Rl)v.x, (Rl)v.y};
    }
}
template <typename Rl>
__global__ void permute_out_kernel(const C2<Rl>* __restrict__ src, double2* __restrict__ dst,
                                   const int* __restrict__ perm, int N, size_t total) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t row = i / N;
        const int p = (int)(i - row * N);
        C2<Rl> v = src[i];
        dst[row * N + perm[p]] = make_double2((double)v.x, (double)v.y);
    }
}

// The same maps with the FP64 side in pinned host memory, read or written by the kernel over
// the host link: that side goes in natural order (consecutive threads, consecutive 16-byte
// elements), iperm[q] the position of natural index q; four elements in flight per thread.
template <typename Rl>
__global__ void permute_in_host_kernel(const double2* __restrict__ src, C2<Rl>* __restrict__ dst,
                                       C2<Rl>* __restrict__ lo, const int* __restrict__ iperm, int N, size_t total) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < total; i0 += 4 * stride) {
        double2 v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const size_t i = i0 + u * stride;
            v[u] = i < total ? src[i] : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const size_t i = i0 + u * stride;
            if (i >= total) break;
            const size_t row = i / N;
            const int q = (int)(i - row * N);
            const C2<Rl> h{(Rl)v[u].x, (Rl)v[u].y};
            dst[row * N + iperm[q]] = h;
            // the remainder v - h (zero in FP64): the low parts of a double-float value
            if (lo) lo[row * N + iperm[q]] = C2<Rl>{(Rl)(v[u].x - (double)h.x), (Rl)(v[u].y - (double)h.y)};
        }
    }
}
template <typename Rl>
__global__ void permute_out_host_kernel(const C2<Rl>* __restrict__ src, const C2<Rl>* __restrict__ lo,
                                        double2* __restrict__ dst, const int* __restrict__ iperm, int N,
                                        size_t total) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < total; i0 += 4 * stride) {
        double2 v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const size_t i = i0 + u * stride;
            if (i < total) {
                const size_t row = i / N;
                const size_t pos = row * N + iperm[(int)(i - row * N)];
                const C2<Rl> h = src[pos];
                v[u] = make_double2((double)h.x, (double)h.y);
                if (lo) {   // high + low parts, exact in FP64
                    const C2<Rl> l = lo[pos];
                    v[u].x += (double)l.x;
                    v[u].y += (double)l.y;
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const size_t i = i0 + u * stride;
            if (i < total) dst[i] = v[u];
        }
    }
}

// ------------------------------------------------------------------ launchers --
template <typename Rl>
static int fft_threads(int M) {
    const int maxt = sizeof(Rl) == 8 ? 512 : 1024;
    int t = M / 16;
    if (t < 32) t = 32;
    if (t > maxt) t = maxt;
    return t;
}

template <typename Rl>
cudaError_t launch_fft(int sign, const C2<Rl>* in, C2<Rl>* out, FftArgs<Rl> a, cudaStream_t st, long long* nlaunch) {
    // a.rows full rows of length a.N = a.P * a.M
    const size_t smem = fft_smem_bytes<Rl>(a.M, a.N);
    const int nsub = a.rows * a.P;
    const int thr = fft_threads<Rl>(a.M);
    const int cross_thr = 256;
    const unsigned cross_blocks = (unsigned)(((size_t)a.rows * a.M + cross_thr - 1) / cross_thr);
    if (sign < 0) {
        const C2<Rl>* src = in;
        if (a.P > 1) {
            switch (a.P) {
                case 2: fft_cross_kernel<Rl, -1, 2><<<cross_blocks, cross_thr, 0, st>>>(in, out, a); break;
                case 4: fft_cross_kernel<Rl, -1, 4><<<cross_blocks, cross_thr, 0, st>>>(in, out, a); break;
                case 8: fft_cross_kernel<Rl, -1, 8><<<cross_blocks, cross_thr, 0, st>>>(in, out, a); break;
                default: return cudaErrorInvalidValue;
            }
            (*nlaunch)++;
            src = out;
        }
        fft_sub_kernel<Rl, -1><<<nsub, thr, smem, st>>>(src, out, a);
        (*nlaunch)++;
    } else {
        C2<Rl>* mid = out;
        fft_sub_kernel<Rl, +1><<<nsub, thr, smem, st>>>(in, mid, a);
        (*nlaunch)++;
        if (a.P > 1) {
            switch (a.P) {
                case 2: fft_cross_kernel<Rl, +1, 2><<<cross_blocks, cross_thr, 0, st>>>(mid, out, a); break;
                case 4: fft_cross_kernel<Rl, +1, 4><<<cross_blocks, cross_thr, 0, st>>>(mid, out, a); break;
                case 8: fft_cross_kernel<Rl, +1, 8><<<cross_blocks, cross_thr, 0, st>>>(mid, out, a); break;
                default: return cudaErrorInvalidValue;
            }
            (*nlaunch)++;
        }
    }
    return cudaGetLastError();
}

template <typename Rl>
cudaError_t fft_set_smem(int M, int N) {
    // a per-kernel ceiling shared by every handle of the process: the device maximum, so
    // that a handle on a smaller grid never lowers it for a larger one
    (void)M;
    (void)N;
    const int smem = 227 * 1024;
    cudaError_t e = cudaFuncSetAttribute(fft_sub_kernel<Rl, -1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(fft_sub_kernel<Rl, +1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

static unsigned grid_for(size_t total, int thr) {
    size_t b = (total + thr - 1) / thr;
    if (b > 152 * 32) b = 152 * 32;
    if (b < 1) b = 1;
    return (unsigned)b;
}

template <typename Rl>
cudaError_t launch_plasma(PlasmaArgs<Rl> a, int rows, cudaStream_t st, long long* nlaunch) {
    plasma_kernel<Rl><<<rows, 256, 0, st>>>(a);
    (*nlaunch)++;
    return cudaGetLastError();
}

template <typename Rl>
cudaError_t launch_spec1(SpecArgs<Rl> a, cudaStream_t st, long long* nlaunch) {
    spec1_kernel<Rl><<<grid_for((size_t)a.rows * a.N, 256), 256, 0, st>>>(a);
    (*nlaunch)++;
    return cudaGetLastError();
}

template <typename Rl>
cudaError_t launch_spec2(SpecArgs<Rl> a, cudaStream_t st, long long* nlaunch) {
    spec2_kernel<Rl><<<grid_for((size_t)a.rows * a.N, 256), 256, 0, st>>>(a);
    (*nlaunch)++;
    return cudaGetLastError();
}

template <typename Rl>
cudaError_t launch_zero_nl(const C2<Rl>* A, C2<Rl>* nb, size_t total, unsigned long long* max_out,
                           cudaStream_t st, long long* nlaunch) {
    zero_nl_kernel<Rl><<<grid_for(total, 256), 256, 0, st>>>(A, nb, total, max_out);
    (*nlaunch)++;
    return cudaGetLastError();
}

template <typename Rl>
cudaError_t launch_permute(int dir, const void* src, void* dst, const int* perm, int N, size_t total,
                           cudaStream_t st, long long* nlaunch) {
    if (dir > 0)
        permute_in_kernel<Rl><<<grid_for(total, 256), 256, 0, st>>>((const double2*)src, (C2<Rl>*)dst, perm, N, total);
    else
        permute_out_kernel<Rl><<<grid_for(total, 256), 256, 0, st>>>((const C2<Rl>*)src, (double2*)dst, perm, N, total);
    (*nlaunch)++;
    return cudaGetLastError();
}

template <typename Rl>
cudaError_t launch_permute_host(int dir, const void* src, void* dst, const int* iperm, int N, size_t total, int sms,
                                cudaStream_t st, long long* nlaunch, void* lo) {
    const unsigned g = (unsigned)(sms > 0 ? 8 * sms : 1024);
    if (dir > 0)
        permute_in_host_kernel<Rl><<<g, 256, 0, st>>>((const double2*)src, (C2<Rl>*)dst, (C2<Rl>*)lo, iperm, N, total);
    else
        permute_out_host_kernel<Rl><<<g, 256, 0, st>>>((const C2<Rl>*)src, (const C2<Rl>*)lo, (double2*)dst, iperm, N,
                                                       total);
    (*nlaunch)++;
    return cudaGetLastError();
}

#define GS_INST(Rl)                                                                                          \
    template cudaError_t launch_fft<Rl>(int, const C2<Rl>*, C2<Rl>*, FftArgs<Rl>, cudaStream_t, long long*); \
    template cudaError_t fft_set_smem<Rl>(int, int);                                                              \
    template cudaError_t launch_plasma<Rl>(PlasmaArgs<Rl>, int, cudaStream_t, long long*);                   \
    template cudaError_t launch_spec1<Rl>(SpecArgs<Rl>, cudaStream_t, long long*);                           \
    template cudaError_t launch_spec2<Rl>(SpecArgs<Rl>, cudaStream_t, long long*);                           \
    template cudaError_t launch_zero_nl<Rl>(const C2<Rl>*, C2<Rl>*, size_t, unsigned long long*,             \
                                            cudaStream_t, long long*);                                       \
    template cudaError_t launch_permute<Rl>(int, const void*, void*, const int*, int, size_t, cudaStream_t,  \
                                            long long*);                                                     \
    template cudaError_t launch_permute_host<Rl>(int, const void*, void*, const int*, int, size_t, int,      \
                                                 cudaStream_t, long long*, void*);
GS_INST(double)
GS_INST(float)

}  // namespace gs
