// gs_nl_vjp.cu -- adjoint of one RK4 stage of calculate_NLresponse (propagator.cu:629-783),
// one CTA per radial row, the row resident in shared memory.
//
// With the stage's recorded E (= IFFT(Y)/N), rho and Q, and the cotangent kb of its
// spectral output N = FFT(loss) + PF FFT(rho E) - j K FFT(Q E), the kernel computes
// ybar = (dN/dY)^H kb (cotangents g = dJ/dRe + i dJ/dIm):
//   q = IFFT(j K kb)       E_bar  = Q q,        Q_bar = Re(conj(E) q)
//   Raman transpose        I_bar  = (1-fR) Q_bar + fR M Im(sum_t a^((t-s) mod N) Q_bar_t)
//   l = IFFT(kb)           E_bar += s l,        I_bar += s'(I) Re(conj(E) l)   (loss = s E)
//   p = IFFT(conj(PF) kb)  E_bar += rho p,      rho_bar = Re(conj(E) p)
//   density, backwards     lam_{t-1} = rho_bar_{t-1} + d_t lam_t;  I_{t-1}, I_t += lam_t x partials
//   ybar = FFT(E_bar + 2 I_bar E) / N
// The two reverse recurrences are linear, so each runs exactly as chunked affine maps
// composed by one block scan (chunks taken in reverse order).  The same kernel folds in
// the RK4 bookkeeping: A_bar (+)= ybar and the next stage's kb = cR rbar + cdz ybar.
#include "gs_internal.cuh"
#include "gs_kernels.h"
#include "gs_plasma.cuh"

namespace gs {

template <typename Rl> static int vjp_threads(int N) {
    const int maxt = 512;
    int t = N / 16;
    if (t < 32) t = 32;
    if (t > maxt) t = maxt;
    return t;
}

template <typename Rl> static size_t vjp_smem(int N, int nthr) {
    using T2 = C2<Rl>;
    return (size_t)padded_len(N) * sizeof(T2)      // the row being transformed
           + (size_t)(N / 64 + 64) * sizeof(T2)    // twiddles
           + 2 * (size_t)wb_count(N) * sizeof(Rl)  // I_bar; Q_bar then rho_bar
           + (size_t)nthr * sizeof(T2)              // chunk results of the scans
           + (size_t)nthr * sizeof(Rl)              // density-adjoint terms across chunk edges
           + 64 * sizeof(T2) + 64 * sizeof(Rl);     // scan scratch
}

template <typename Rl>
__global__ void __launch_bounds__(512) nl_vjp_kernel(VjpArgs<Rl> v) {
    using T2 = C2<Rl>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = v.N;
    const int tid = threadIdx.x, nthr = blockDim.x;
    T2* buf = reinterpret_cast<T2*>(smem_raw);
    T2* twh = buf + padded_len(N);
    T2* twl = twh + N / 64;
    Rl* Ib = reinterpret_cast<Rl*>(twl + 64);
    Rl* Xr = Ib + wb_count(N);
    T2* cend = reinterpret_cast<T2*>(Xr + wb_count(N));
    Rl* bnd = reinterpret_cast<Rl*>(cend + nthr);
    T2* scA = reinterpret_cast<T2*>(bnd + nthr);
    T2* scB = scA + 32;
    Rl* rA = reinterpret_cast<Rl*>(scB + 32);
    Rl* rB = rA + 32;
    Rl* cendr = reinterpret_cast<Rl*>(cend);

    const size_t base = (size_t)blockIdx.x * N;
    const T2* kb = v.kb + base;
    const T2* te = v.tape_e + base;
    const Rl* trho = v.tape_rho + base;
    const Rl* tq = v.tape_q + base;
    T2* Eb = v.ebar + base;
    const Rl ks = (Rl)v.kb_scale;
    load_twiddles<Rl>(twh, twl, v.tw, N, tid, nthr);
    const TwTab<Rl> tw{twh, twl, v.twb};
    const int L = N / nthr;

    // A row that did not ionize in this stage (no sample above the rate table: W = dW = 0,
    // rho = 0) has s = ds = 0 in the loss term, rho E = 0 and d rho / d I = 0: the loss, plasma
    // and density-adjoint passes below add exact zeros there and are skipped, and its E_bar
    // (= Q q) is formed again from q, still in the row buffer, instead of kept in EBAR.
    const bool ion = v.tape_ion ? v.tape_ion[blockIdx.x] != 0 : true;
    // the loops over the row take SB points per thread, every global read of a batch issued
    // before its use
    constexpr int SB = 4;

    // ---- Kerr: q = IFFT(j K kb)
    if (v.kerr_on) {
        for (int pb = tid; pb < N; pb += SB * nthr) {
            T2 k[SB];
            Rl K[SB];
#pragma unroll
            for (int u = 0; u < SB; u++) {
                const int p = pb + u * nthr;
                k[u] = p < N ? kb[p] : T2{0, 0};
                K[u] = p < N ? v.kerr[p] : (Rl)0;
            }
#pragma unroll
            for (int u = 0; u < SB; u++) {
                const int p = pb + u * nthr;
                const Rl Kp = K[u] * ks;
                if (p < N) buf[pad16(p)] = T2{-Kp * k[u].y, Kp * k[u].x};
            }
        }
        __syncthreads();
        smem_fft<+1, Rl>(buf, N, v.logM, tw, 1, tid, nthr);
        for (int tb = tid; tb < N; tb += SB * nthr) {
            T2 q[SB], e[SB];
            Rl Q[SB];
#pragma unroll
            for (int u = 0; u < SB; u++) {
                const int t = tb + u * nthr;
                const bool in = t < N;
                q[u] = in ? buf[pad16(t)] : T2{0, 0};
                e[u] = in ? te[t] : T2{0, 0};
                Q[u] = (in && ion) ? tq[t] : (Rl)0;
            }
#pragma unroll
            for (int u = 0; u < SB; u++) {
                const int t = tb + u * nthr;
                if (t >= N) continue;
                if (ion) Eb[t] = T2{Q[u] * q[u].x, Q[u] * q[u].y};
                Xr[pad32(t)] = e[u].x * q[u].x + e[u].y * q[u].y;
            }
        }
    } else {
        for (int t = tid; t < N; t += nthr) {
            if (ion) Eb[t] = T2{0, 0};
            Xr[pad32(t)] = 0;
        }
    }
    __syncthreads();

    // ---- Raman transpose: w_s = a w_{s+1} + Q_bar_s (from the right), y_s = (1-a^N) w_s + a^(N-s) w_0
    {
        const int c = nthr - 1 - tid;   // chunk of this thread: chunks in reverse order for the scan
        const int t0 = c * L;
        if (v.kerr_on && v.raman_scan) {
            const T2 ra = T2{(Rl)v.a_re, (Rl)v.a_im};
            T2 wl = T2{0, 0}, aL = T2{1, 0};
            for (int i = L - 1; i >= 0; i--) {
                wl = cmul(ra, wl);
                wl.x += Xr[pad32(t0 + i)];
                aL = cmul(aL, ra);
            }
            T2 Am = aL, Bm = wl;
            block_affine_scan<T2>(Am, Bm, T2{1, 0}, T2{0, 0}, scA, scB);
            cend[tid] = Bm;   // w at the start of chunk c
            __syncthreads();
            T2 w = (tid == 0) ? T2{0, 0} : cend[tid - 1];
            const T2 w0 = cend[nthr - 1];
            // a^(N - t) at t = t0 + L - 1 is a^(tid L + 1) = a (a^L)^tid
            T2 b = aL, pr = T2{1, 0};
            for (int e = tid; e > 0; e >>= 1) {
                if (e & 1) pr = cmul(pr, b);
                b = cmul(b, b);
            }
            T2 pw = cmul(pr, ra);
            const T2 oma = T2{(Rl)(1.0 - v.aN_re), (Rl)(-v.aN_im)};
            const Rl fRM = (Rl)v.fRM, omf = (Rl)v.one_minus_fR;
            for (int i = L - 1; i >= 0; i--) {
                const int t = t0 + i;
                const Rl qb = Xr[pad32(t)];
                w = cmul(ra, w);
                w.x += qb;
                const T2 y = cadd(cmul(oma, w), cmul(pw, w0));
                Ib[pad32(t)] = omf * qb + fRM * y.y;
                pw = cmul(pw, ra);
            }
        } else {
            for (int i = 0; i < L; i++) Ib[pad32(t0 + i)] = Xr[pad32(t0 + i)];
        }
    }
    __syncthreads();

    const Rl ND = (Rl)v.neutral_density, tstep = (Rl)v.tstep_scaled;
    const Rl U = (Rl)v.ionization_potential, Pc = (Rl)v.ponderomotive, AV = (Rl)v.avalanche_cs;
    const Rl invND = (Rl)1 / ND, invTAU = (Rl)1 / (Rl)v.recombination_tau;

    if (ion) {
    // ---- loss: l = IFFT(kb); loss_t = s(I_t) E_t for 0 < t < N-1 above the (log) threshold
    for (int p = tid; p < N; p += nthr) {
        const T2 k = kb[p];
        buf[pad16(p)] = T2{k.x * ks, k.y * ks};
    }
    __syncthreads();
    smem_fft<+1, Rl>(buf, N, v.logM, tw, 1, tid, nthr);
    for (int t = tid; t < N; t += nthr) {
        const T2 e = te[t];
        const Rl I = e.x * e.x + e.y * e.y;
        if (t > 0 && t < N - 1 && I > (Rl)GS_ION_MIN_LN) {
            const T2 l = buf[pad16(t)];
            RateD<Rl> r = rate_with_derivs<Rl>(I, v.rate, U, Pc, AV);
            if (trho[t] > ND) { r.W = 0; r.dW = 0; }
            const Rl s = -(Rl)0.5 * r.W * (U + Pc * I) / I;
            const Rl ds = -(Rl)0.5 * (r.dW * (U + Pc * I) / I - r.W * U / (I * I));
            T2 eb = Eb[t];
            eb.x += s * l.x;
            eb.y += s * l.y;
            Eb[t] = eb;
            Ib[pad32(t)] += ds * (e.x * l.x + e.y * l.y);
        }
    }
    __syncthreads();

    // ---- plasma: p = IFFT(conj(PF) kb)
    for (int p = tid; p < N; p += nthr) {
        const T2 k = kb[p], f = v.pf[p];
        buf[pad16(p)] = T2{ks * (k.x * f.x + k.y * f.y), ks * (k.y * f.x - k.x * f.y)};
    }
    __syncthreads();
    smem_fft<+1, Rl>(buf, N, v.logM, tw, 1, tid, nthr);
    for (int t = tid; t < N; t += nthr) {
        const T2 pv = buf[pad16(t)], e = te[t];
        const Rl r = trho[t];
        T2 eb = Eb[t];
        eb.x += r * pv.x;
        eb.y += r * pv.y;
        Eb[t] = eb;
        Xr[pad32(t)] = e.x * pv.x + e.y * pv.y;
    }
    __syncthreads();

    // ---- density recurrence backwards: lam_{t-1} = rho_bar_{t-1} + d_t lam_t (lam_{N-1} = rho_bar_{N-1})
    {
        const int c = nthr - 1 - tid;
        const int t0 = c * L;
        auto rate_at = [&](int t) -> RateD<Rl> {
            if (t == 0) return RateD<Rl>{0, 0, 0, 0};   // the recurrence starts from E_0 = 0
            const T2 e = te[t];
            return rate_with_derivs<Rl>(e.x * e.x + e.y * e.y, v.rate, U, Pc, AV);
        };
        Rl dd, aa, bb;
        // chunk map lam_{t0} = Am lam_{t0+L} + Bm
        Rl Am = 1, Bm = 0;
        {
            RateD<Rl> rt = rate_at(t0 + L - 1);
            Rl dn = 0;
            if (t0 + L <= N - 1) {
                heun_partials<Rl>(trho[t0 + L - 1], rt, rate_at(t0 + L), tstep, ND, invND, invTAU, &dd, &aa, &bb);
                dn = dd;
            }
            for (int i = L - 1; i >= 0; i--) {
                const int t = t0 + i;
                Am = dn * Am;
                Bm = Xr[pad32(t)] + dn * Bm;
                if (t >= 1) {
                    const RateD<Rl> rp = rate_at(t - 1);
                    heun_partials<Rl>(trho[t - 1], rp, rt, tstep, ND, invND, invTAU, &dd, &aa, &bb);
                    dn = dd;
                    rt = rp;
                }
            }
        }
        block_affine_scan<Rl>(Am, Bm, (Rl)1, (Rl)0, rA, rB);
        cendr[tid] = Bm;   // lam at the start of chunk c
        bnd[c] = 0;
        __syncthreads();
        Rl lam = (tid == 0) ? (Rl)0 : cendr[tid - 1];   // lam_{t0+L}
        RateD<Rl> rt = rate_at(t0 + L - 1);
        Rl dn = 0;
        if (t0 + L <= N - 1) {
            heun_partials<Rl>(trho[t0 + L - 1], rt, rate_at(t0 + L), tstep, ND, invND, invTAU, &dd, &aa, &bb);
            dn = dd;
        }
        for (int i = L - 1; i >= 0; i--) {
            const int t = t0 + i;
            const Rl lt = Xr[pad32(t)] + dn * lam;
            if (t >= 1) {
                const RateD<Rl> rp = rate_at(t - 1);
                heun_partials<Rl>(trho[t - 1], rp, rt, tstep, ND, invND, invTAU, &dd, &aa, &bb);
                Ib[pad32(t)] += lt * bb;
                if (t - 1 >= 1) {
                    if (i >= 1) Ib[pad32(t - 1)] += lt * aa;
                    else bnd[c] = lt * aa;   // I_{t0-1} belongs to chunk c-1
                }
                dn = dd;
                rt = rp;
            }
            lam = lt;
        }
        __syncthreads();
        if (c + 1 < nthr) Ib[pad32(t0 + L - 1)] += bnd[c + 1];
    }
    __syncthreads();
    }   // ion

    // ---- ybar = FFT(E_bar + 2 I_bar E) / N, then the RK4 bookkeeping
    for (int tb = tid; tb < N; tb += SB * nthr) {
        T2 e[SB], eb[SB];
        Rl Q[SB];
#pragma unroll
        for (int u = 0; u < SB; u++) {
            const int t = tb + u * nthr;
            const bool in = t < N;
            e[u] = in ? te[t] : T2{0, 0};
            eb[u] = (in && ion) ? Eb[t] : T2{0, 0};
            Q[u] = (in && !ion && v.kerr_on) ? tq[t] : (Rl)0;
        }
#pragma unroll
        for (int u = 0; u < SB; u++) {
            const int t = tb + u * nthr;
            if (t >= N) continue;
            if (!ion && v.kerr_on) {   // E_bar = Q q, q still in the row buffer
                const T2 q = buf[pad16(t)];
                eb[u] = T2{Q[u] * q.x, Q[u] * q.y};
            }
            const Rl i2 = 2 * Ib[pad32(t)];
            buf[pad16(t)] = T2{eb[u].x + i2 * e[u].x, eb[u].y + i2 * e[u].y};
        }
    }
    __syncthreads();
    smem_fft<-1, Rl>(buf, N, v.logM, tw, 1, tid, nthr);
    const Rl rn = (Rl)N, cR = (Rl)v.cR, cdz = (Rl)v.cdz;
    for (int pb = tid; pb < N; pb += SB * nthr) {
        T2 o[SB], r[SB];
#pragma unroll
        for (int u = 0; u < SB; u++) {
            const int p = pb + u * nthr;
            const bool in = p < N;
            o[u] = (in && v.ab_add) ? v.ab[base + p] : T2{0, 0};
            r[u] = (in && v.kb_out) ? v.rbar[base + p] : T2{0, 0};
        }
#pragma unroll
        for (int u = 0; u < SB; u++) {
            const int p = pb + u * nthr;
            if (p >= N) continue;
            const T2 y = buf[pad16(p)];
            const T2 yb = T2{y.x / rn, y.y / rn};
            T2 a = yb;
            if (v.ab_add) {
                a.x += o[u].x;
                a.y += o[u].y;
            }
            v.ab[base + p] = a;
            if (v.kb_out) v.kb_out[base + p] = T2{cR * r[u].x + cdz * yb.x, cR * r[u].y + cdz * yb.y};
        }
    }
}

template <typename Rl> bool nl_vjp_supported(int N) {
    const int nthr = vjp_threads<Rl>(N);
    return N >= 64 && N % nthr == 0 && vjp_smem<Rl>(N, nthr) <= 227 * 1024;
}

template <typename Rl> cudaError_t nl_vjp_setup(int N) {
    (void)N;   // a per-kernel ceiling shared by all handles: the device maximum
    return cudaFuncSetAttribute(nl_vjp_kernel<Rl>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

template <typename Rl> cudaError_t launch_nl_vjp(const VjpArgs<Rl>& v, int rows, cudaStream_t st, long long* nl) {
    int nthr = vjp_threads<Rl>(v.N);
    const int t = v.threads;
    if (t >= 32 && t <= 512 && t % 32 == 0 && v.N % t == 0 && vjp_smem<Rl>(v.N, t) <= 227 * 1024) nthr = t;
    nl_vjp_kernel<Rl><<<rows, nthr, vjp_smem<Rl>(v.N, nthr), st>>>(v);
    (*nl)++;
    return cudaGetLastError();
}

// ---- objective and small vector kernels ------------------------------------------------
template <typename Rl>
__global__ void adj_seed_kernel(const C2<Rl>* __restrict__ A, const double* __restrict__ w, C2<Rl>* __restrict__ ab,
                                size_t n, double* partial) {
    __shared__ double sm[32];
    double s = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const C2<Rl> a = A[i];
        const double wi = w[i];
        s += wi * ((double)a.x * a.x + (double)a.y * a.y);
        ab[i] = C2<Rl>{(Rl)(2 * wi * a.x), (Rl)(2 * wi * a.y)};
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += sm[k];
        partial[blockIdx.x] = t;
    }
}

__global__ void sum_partials_kernel(const double* __restrict__ partial, int n, double* out) {
    __shared__ double sm[32];
    double s = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += sm[k];
        *out = t;
    }
}

template <typename Rl>
cudaError_t launch_adj_seed(const typename Vec2<Rl>::T* A, const double* w, typename Vec2<Rl>::T* ab, size_t n,
                            double* partial, int nblocks, double* out, cudaStream_t st, long long* nl) {
    adj_seed_kernel<Rl><<<nblocks, 256, 0, st>>>(A, w, ab, n, partial);
    sum_partials_kernel<<<1, 256, 0, st>>>(partial, nblocks, out);
    (*nl) += 2;
    return cudaGetLastError();
}

template <typename Rl>
__global__ void cadd_kernel(C2<Rl>* __restrict__ y, const C2<Rl>* __restrict__ x, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    C2<Rl> a = y[i];
    const C2<Rl> b = x[i];
    a.x += b.x;
    a.y += b.y;
    y[i] = a;
}

template <typename Rl>
cudaError_t launch_cadd(typename Vec2<Rl>::T* y, const typename Vec2<Rl>::T* x, size_t n, cudaStream_t st,
                        long long* nl) {
    cadd_kernel<Rl><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(y, x, n);
    (*nl)++;
    return cudaGetLastError();
}

#define GS_VJP_INST(Rl)                                                                                      \
    template bool nl_vjp_supported<Rl>(int);                                                                 \
    template cudaError_t nl_vjp_setup<Rl>(int);                                                              \
    template cudaError_t launch_nl_vjp<Rl>(const VjpArgs<Rl>&, int, cudaStream_t, long long*);              \
    template cudaError_t launch_adj_seed<Rl>(const Vec2<Rl>::T*, const double*, Vec2<Rl>::T*, size_t, double*, \
                                             int, double*, cudaStream_t, long long*);                        \
    template cudaError_t launch_cadd<Rl>(Vec2<Rl>::T*, const Vec2<Rl>::T*, size_t, cudaStream_t, long long*);
GS_VJP_INST(double)
GS_VJP_INST(float)

}  // namespace gs
