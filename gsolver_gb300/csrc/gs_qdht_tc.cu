// gs_qdht_tc.cu -- mixed-precision QDHT on the 5th-generation tensor cores (sm_103a).
//
// ht_run (qdht_plan::run_many, fhatha.cpp:218-230) is the real GEMM
//   Y[i][c] = sum_j H(i,j) X[j][c],  H(i,j) = m1_i C(i,j) / m1_j   (folded in FP64 at set-up)
// over the 2*n_t interleaved (re, im) float columns of a [n_r][n_t] complex array.
// It runs with split operands and FP32 accumulation, D = Hh Xh + Hh Xl + Hl Xh: on grids with
// 2 n_t a multiple of 256 as FP16 pairs with power-of-two row / column scales (the wide-tile
// path below), otherwise as 3xTF32 (round-to-nearest TF32 parts, relative error ~2^-21) in
// the kernel described here.
//
// Persistent: one CTA per SM walks 128 (i) x 128 (c) output tiles (tile T = row tile T % MT
// of column tile T / MT, so the row tiles of a column block run side by side and share X in
// L2), K looped in blocks of 32 (one 128-byte swizzle row of FP32); the 3-stage operand ring
// (64 KiB stages) and the 2-deep raw X ring run on across tiles:
//   warp 0      TMA producer: cp.async.bulk.tensor loads of the Hh/Hl tiles (SWIZZLE_128B)
//               onto an mbarrier with expect-tx; owns the TMEM allocation.
//   warp 1      MMA issuer: one thread issues tcgen05.mma.kind::tf32 (M=128, N=128, K=8)
//               x 4 K-steps x 3 terms per stage, accumulator in TMEM (128 columns), and
//               tcgen05.commit releases the stage.
//               It also streams the raw FP32 X tile (32 rows x 128 columns) by TMA into a
//               2-deep ring.
//   warps 2-9   B producers: read the X tile from that ring, apply the
//               spectral-window mask of the inverse transform, split into TF32 hi/lo and
//               write them K-major in the 128B-swizzled layout the MMA descriptor reads.
//   warps 10-17 epilogue: tcgen05.ld of the accumulator (handed back to the MMA issuer
//               right after), then either a plain store or the fused calculate_Lstep
//               update of BIGBUFFER2 (propagator.cu:570-625), overlapping the next tile.
// Every mbarrier wait is bounded; on expiry the kernel records an error, drains what it
// issued, frees TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gs_internal.cuh"
#include "gs_qdht_tc.h"

namespace gs {

namespace tc {

constexpr int BM = 128, BN = 128, BK = 32, STAGES = 3, RAW_STAGES = 2;
constexpr int TILE_BYTES = BM * BK * 4;                 // 16 KiB: one 128 x 32 FP32 tile
constexpr int STAGE_BYTES = 4 * TILE_BYTES;             // Ah, Al, Bh, Bl
constexpr int RAW_BYTES = BK * BN * 4;                  // 16 KiB: 32 rows x 128 columns of X
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + RAW_STAGES * RAW_BYTES + 1024 + 256;   // + barriers, TMEM slot
constexpr int NCONV = 256;                              // warps 2..9: B producers
constexpr int NEPI = 8;                                 // warps 10..17: epilogue
constexpr int THREADS = 64 + NCONV + 32 * NEPI;
constexpr unsigned long long WAIT_NS = 200ull * 1000 * 1000;   // 200 ms; legitimate waits are < 1 ms

__constant__ float c_sqrt_ho_f[20];

struct TcArgs {
    const float* X;
    float* Y;
    int nr, ncols, mode;
    float dz;
    const float* kr;
    const float* ki;
    const float* ho;
    const float* kt2;
    const int* kmax;
    unsigned* err;
    // FP16 operands: Y[i][c] = hscale[i] xscale[c] (H' X')[i][c] (powers of two)
    const float* hscale;
    const float* xscale;
    // wide path: nc operand columns, compact column c' holding column cmap[c'] of X and Y
    // (-1: padding), or cmap null and nc = ncols
    int nc;
    const int* cmap;
    float* yc;   // non-null: the output goes to this [nr][nc] compact array instead of Y
    int ycompact;   // linear step: Y is the compact [nr][nc] copy of BIGBUFFER2's window columns
    // linear step on BIGBUFFER2's double-float compact copy (Y = its high parts, ylo its low
    // parts): theta per [pair][row] and k_i per pair as double-float pairs, 1 / (1 + s) per
    // [pair][row] (0 outside the window and in the padding), dz as a double-float pair
    const float2* theta;
    const float2* kiff;
    const float* inv1ps;
    float* ylo;
    float dz_lo;
    // gs_advance: the step size *dz_dev (instead of dz, dz_lo) and no work while *run == 0
    const double* dz_dev;
    const int* run;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

// non-blocking probe of the phase with the given parity
__device__ __forceinline__ bool mbar_try(uint64_t* bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// wall-clock bounded wait: false when limit_ns expired.  try_wait suspends the thread until the
// phase completes or a short hardware time window passes, so a completed phase wakes the waiter
// at once (a test_wait poll with a sleep between tries woke it up to a sleep later)
__device__ __forceinline__ bool mbar_wait_ns(uint64_t* bar, unsigned parity, unsigned long long limit_ns) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = globaltimer_ns();
    for (;;) {
        if (mbar_try(bar, parity)) return true;
        if (globaltimer_ns() - t0 > limit_ns) return false;
    }
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) { return mbar_wait_ns(bar, parity, WAIT_NS); }

// first expired wait of a launch: code | k-block << 8 | warp << 20, kept for the host
__device__ __forceinline__ void record_stall(unsigned* err, unsigned code, int kb, int warp) {
    atomicOr(err, code);
    atomicCAS(err + 1, 0u, code | ((unsigned)(kb & 0xfff) << 8) | ((unsigned)warp << 20));
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// tcgen05 shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                 // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;       // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;                 // descriptor version (sm_100 family)
    d |= (uint64_t)2 << 61;                 // SWIZZLE_128B
    return d;
}

// instruction descriptor: kind::tf32, D = F32, A = B = TF32, both K-major, M = 128, N = 128
__host__ __device__ constexpr uint32_t make_idesc() {
    return (1u << 4)                     // D format F32
           | (2u << 7)                   // A format TF32
           | (2u << 10)                  // B format TF32
           | ((uint32_t)(BN >> 3) << 17)  // N / 8
           | ((uint32_t)(BM >> 4) << 24); // M / 16
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, float a, float b, float c, float d) {
    asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}

// The load and its tcgen05.wait::ld are one asm statement: tcgen05.ld is asynchronous, so
// its destination registers may be read only after the wait.  (As two statements the
// compiler may schedule reads of the registers before the wait, which returns stale values
// when the load is slow, e.g. while MMAs into another accumulator buffer are running.)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int k = 0; k < 32; k++) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ float sqrt_ho_f(float x) {
    float r = 0.f, xn = x;
#pragma unroll
    for (int j = 0; j < 20; j++) { r = fmaf(c_sqrt_ho_f[j], xn, r); xn *= x; }
    return r;
}

__global__ void __launch_bounds__(THREADS, 1) qdht_tc_kernel(const __grid_constant__ CUtensorMap map_hi,
                                                             const __grid_constant__ CUtensorMap map_lo,
                                                             const __grid_constant__ CUtensorMap map_x, TcArgs a) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* raw = smem + STAGES * STAGE_BYTES;   // [RAW_STAGES] raw X tiles (TMA, unswizzled)
    uint64_t* bars = (uint64_t*)(raw + RAW_STAGES * RAW_BYTES);
    uint64_t* full_a = bars;                  // [STAGES]  TMA tx
    uint64_t* full_b = bars + STAGES;         // [STAGES]  256 converter arrivals
    uint64_t* empty = bars + 2 * STAGES;      // [STAGES]  MMA commit
    uint64_t* done = bars + 3 * STAGES;       // every MMA of this CTA complete
    uint64_t* raw_full = bars + 3 * STAGES + 1;                 // [RAW_STAGES] TMA tx
    uint64_t* raw_empty = raw_full + RAW_STAGES;                // [RAW_STAGES] 256 converter arrivals
    uint64_t* acc_full = raw_empty + RAW_STAGES;                // MMA commit: accumulator ready
    uint64_t* acc_empty = acc_full + 1;                         // NEPI epilogue warps: read out
    uint32_t* tmem_slot = (uint32_t*)(acc_empty + 1);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int MT = a.nr / BM;
    const int ntiles = MT * (a.ncols / BN);
    const int nk = a.nr / BK;
    // this CTA's tiles: blockIdx.x + k gridDim.x; tile T is row tile T % MT of column tile
    // T / MT, so the row tiles of one column block run side by side (X shared in L2)
    const int my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full_a[s], 1);
            mbar_init(&full_b[s], NCONV);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        for (int r = 0; r < RAW_STAGES; r++) {
            mbar_init(&raw_full[r], 1);
            mbar_init(&raw_empty[r], NCONV);
        }
        mbar_init(acc_full, 1);
        mbar_init(acc_empty, NEPI);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        // ------------------------------------------------ TMA producer (A = Hh, Hl; raw X)
        if (lane == 0) {
            int issued = 0, issued_raw = 0;   // global K-block counters
            for (int it = 0; it < my_tiles && !*abort_flag; it++) {
                const int T = blockIdx.x + it * gridDim.x;
                const int m0 = (T % MT) * BM, c0 = (T / MT) * BN;
                for (int kb = 0; kb < nk; kb++) {
                    const int g = it * nk + kb;
                    const int s = g % STAGES;
                    if (g >= STAGES && !mbar_wait(&empty[s], ((g / STAGES) + 1) & 1)) {
                        record_stall(a.err, 4u, kb, warp);
                        *abort_flag = 1;
                        break;
                    }
                    if (*abort_flag) break;
                    unsigned char* st = smem + s * STAGE_BYTES;
                    mbar_expect_tx(&full_a[s], 2 * TILE_BYTES);
                    tma_load_2d(st, &map_hi, kb * BK, m0, &full_a[s]);
                    tma_load_2d(st + TILE_BYTES, &map_lo, kb * BK, m0, &full_a[s]);
                    issued = g + 1;
                    const int r = g % RAW_STAGES;
                    if (g >= RAW_STAGES && !mbar_wait(&raw_empty[r], ((g / RAW_STAGES) + 1) & 1)) {
                        record_stall(a.err, 512u, kb, warp);
                        *abort_flag = 1;
                        break;
                    }
                    mbar_expect_tx(&raw_full[r], RAW_BYTES);
                    tma_load_2d(raw + r * RAW_BYTES, &map_x, c0, kb * BK, &raw_full[r]);
                    issued_raw = g + 1;
                }
            }
            // drain: every issued TMA load has landed before the CTA may exit
            for (int g = (issued > STAGES ? issued - STAGES : 0); g < issued; g++)
                if (!mbar_wait(&full_a[g % STAGES], (g / STAGES) & 1)) record_stall(a.err, 128u, g % nk, warp);
            for (int g = (issued_raw > RAW_STAGES ? issued_raw - RAW_STAGES : 0); g < issued_raw; g++)
                if (!mbar_wait(&raw_full[g % RAW_STAGES], (g / RAW_STAGES) & 1)) record_stall(a.err, 1024u, g % nk, warp);
        }
        __syncwarp();   // the warp reconverges before any block-wide barrier
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            const uint32_t idesc = make_idesc();
            for (int it = 0; it < my_tiles && !*abort_flag; it++) {
                // the epilogue has read the previous tile's accumulator out of tensor memory
                if (it >= 1 && !mbar_wait(acc_empty, (it - 1) & 1)) {
                    record_stall(a.err, 4096u, 0, warp);
                    *abort_flag = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t dt = tmem;
                uint32_t acc = 0;
                bool ok = true;
                for (int kb = 0; kb < nk; kb++) {
                    const int g = it * nk + kb;
                    const int s = g % STAGES;
                    const unsigned ph = (g / STAGES) & 1;
                    if (!mbar_wait(&full_a[s], ph)) {
                        record_stall(a.err, 8u, kb, warp);
                        ok = false;
                        break;
                    }
                    if (!mbar_wait(&full_b[s], ph)) {
                        record_stall(a.err, 256u, kb, warp);
                        ok = false;
                        break;
                    }
                    if (*abort_flag) { ok = false; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    unsigned char* st = smem + s * STAGE_BYTES;
                    const uint32_t ah = smem_u32(st), al = ah + TILE_BYTES;
                    const uint32_t bh = ah + 2 * TILE_BYTES, bl = ah + 3 * TILE_BYTES;
#pragma unroll
                    for (int kk = 0; kk < BK / 8; kk++) {
                        const uint32_t off = kk * 32;   // 8 TF32 = 32 bytes along K inside the swizzle row
                        mma_tf32(dt, make_desc(al + off), make_desc(bh + off), idesc, acc);
                        acc = 1;
                        mma_tf32(dt, make_desc(ah + off), make_desc(bl + off), idesc, 1);
                        mma_tf32(dt, make_desc(ah + off), make_desc(bh + off), idesc, 1);
                    }
                    mma_commit(&empty[s]);
                }
                if (!ok) {
                    *abort_flag = 1;
                    break;
                }
                mma_commit(acc_full);
            }
            mma_commit(done);
        }
        __syncwarp();
    } else if (warp < 2 + NCONV / 32) {
        // ------------------------------------------------ B producers (X -> TF32 hi/lo, K-major)
        const int t = threadIdx.x - 64;        // 0..255
        const int n = t & (BN - 1), kh = t >> 7;
        const uint32_t rowoff = (uint32_t)((n >> 3) * 1024 + (n & 7) * 128);
        for (int it = 0; it < my_tiles && !*abort_flag; it++) {
            const int T = blockIdx.x + it * gridDim.x;
            const int c = (T / MT) * BN + n;
            const int kmx = (a.mode == QDHT_MASKED) ? a.kmax[c >> 1] : 0x7fffffff;
            bool ok = true;
            for (int kb = 0; kb < nk; kb++) {
                const int g = it * nk + kb;
                const int s = g % STAGES;
                const int r = g % RAW_STAGES;
                // the raw X tile (32 rows j x 128 columns) from the TMA ring: column n, rows 16 kh ..
                if (!mbar_wait(&raw_full[r], (g / RAW_STAGES) & 1)) {
                    record_stall(a.err, 2048u, kb, warp);
                    ok = false;
                    break;
                }
                float xv[16];
                const float* rt = reinterpret_cast<const float*>(raw + r * RAW_BYTES) + (16 * kh) * BN + n;
#pragma unroll
                for (int u = 0; u < 16; u++) {
                    const int j = kb * BK + 16 * kh + u;
                    const float v = rt[u * BN];
                    xv[u] = (j > kmx) ? 0.f : v;
                }
                mbar_arrive(&raw_empty[r]);
                if (g >= STAGES && !mbar_wait(&empty[s], ((g / STAGES) + 1) & 1)) {
                    record_stall(a.err, 16u, kb, warp);
                    ok = false;
                    break;
                }
                if (*abort_flag) { ok = false; break; }
                float hi[16], lo[16];
#pragma unroll
                for (int u = 0; u < 16; u++) {
                    hi[u] = tf32_rna(xv[u]);
                    lo[u] = tf32_rna(xv[u] - hi[u]);
                }
                const uint32_t bh = smem_u32(smem + s * STAGE_BYTES + 2 * TILE_BYTES) + rowoff;
                const uint32_t bl = bh + TILE_BYTES;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const uint32_t ch = (uint32_t)((((4 * kh + q) ^ (n & 7))) << 4);
                    st_shared_v4(bh + ch, hi[4 * q], hi[4 * q + 1], hi[4 * q + 2], hi[4 * q + 3]);
                    st_shared_v4(bl + ch, lo[4 * q], lo[4 * q + 1], lo[4 * q + 2], lo[4 * q + 3]);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(&full_b[s]);
            }
            if (!ok) {
                *abort_flag = 1;
                break;
            }
        }
    } else {
        // ------------------------------------------------ epilogue (NEPI warps: two per TMEM
        // lane quarter, 64 columns each).  Each warp copies its accumulator columns into
        // registers and hands tensor memory back at once: the MMA issuer then starts the next
        // tile, and this tile's arithmetic and stores overlap the next tile's main loop.
        const int ew = warp - 2 - NCONV / 32;   // 0..7
        const int q = warp & 3;                 // TMEM lane quarter this warp may read
        const int half = ew >> 2;               // which 64 columns
        for (int it = 0; it < my_tiles; it++) {
            const bool ok = __all_sync(0xffffffffu, mbar_wait(acc_full, it & 1) ? 1 : 0) != 0;
            if (!ok) {
                if (lane == 0) record_stall(a.err, 32u, it, warp);
                *abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (__any_sync(0xffffffffu, *abort_flag)) break;   // warp-uniform: tcgen05.ld is .sync.aligned
            const int T = blockIdx.x + it * gridDim.x;
            const int m0 = (T % MT) * BM, c0 = (T / MT) * BN;
            const int i = m0 + 32 * q + lane;
            const float kt2i = a.kt2 ? a.kt2[i] : 0.f;
            float acc[64];
            tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(64 * half), acc);
            tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(64 * half + 32), acc + 32);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(acc_empty);
#pragma unroll
            for (int cc = 0; cc < 2; cc++) {
                const int col0 = 64 * half + 32 * cc;
                const float* v = acc + 32 * cc;
                float* yrow = a.Y + (size_t)i * a.ncols + c0 + col0;
                if (a.mode != QDHT_LSTEP) {
#pragma unroll
                    for (int k = 0; k < 32; k += 4)
                        *reinterpret_cast<float4*>(yrow + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
                } else {
                    const int p0 = (c0 + col0) >> 1;
#pragma unroll
                    for (int e = 0; e < 16; e++) {
                        const int p = p0 + e;
                        if (i > a.kmax[p]) continue;        // outside the window: BIGBUFFER2 untouched
                        const float k1 = a.kr[p], k2 = a.ki[p];
                        const float sq = sqrt_ho_f(-kt2i / k1 / k1);
                        float2 b2 = *reinterpret_cast<float2*>(yrow + 2 * e);
                        const float inv = 1.f / (1.f + sq);
                        b2.x += a.dz * v[2 * e] * inv;
                        b2.y += a.dz * v[2 * e + 1] * inv;
                        float sn, cs;
                        sincosf(a.dz * (-a.ho[p] - sq * k1), &sn, &cs);
                        const float m = expf(a.dz * k2);
                        const float pr = m * cs, pi = m * sn;
                        float2 f;
                        f.x = b2.x * pr - b2.y * pi;
                        f.y = b2.x * pi + b2.y * pr;
                        *reinterpret_cast<float2*>(yrow + 2 * e) = f;
                    }
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }

    __syncthreads();
    if (warp == 1) {
        // the accumulator is released only after every issued MMA has completed
        if (lane == 0 && !mbar_wait(done, 0)) record_stall(a.err, 64u, nk, warp);
        __syncwarp();
    }
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN));
    }
}

// Adjoint of the fused linear step above, elementwise with the same FP32 tables and
// window: T_bar = conj(P) (FIELD_bar + B2'_bar), B2_bar = T_bar, N_bar = dz T_bar/(1+s);
// outside the window B2_bar passes unchanged and N_bar = 0.
__global__ void lstep_adj_kernel(const float2* __restrict__ fb, float2* __restrict__ sb, float2* __restrict__ b1b,
                                 int nt, size_t total, float dz, const float* __restrict__ kr,
                                 const float* __restrict__ ki, const float* __restrict__ ho,
                                 const float* __restrict__ kt2, const int* __restrict__ kmax) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int i = (int)(idx / nt), p = (int)(idx % nt);
    if (i > kmax[p]) {
        b1b[idx] = make_float2(0.f, 0.f);
        return;
    }
    const float k1 = kr[p], k2 = ki[p];
    const float sq = sqrt_ho_f(-kt2[i] / k1 / k1);
    const float inv = 1.f / (1.f + sq);
    float sn, cs;
    sincosf(dz * (-ho[p] - sq * k1), &sn, &cs);
    const float m = expf(dz * k2);
    const float pr = m * cs, pi = m * sn;
    const float2 f = fb[idx], b = sb[idx];
    const float gr = f.x + b.x, gi = f.y + b.y;
    const float tr = pr * gr + pi * gi, ti = pr * gi - pi * gr;
    sb[idx] = make_float2(tr, ti);
    b1b[idx] = make_float2(dz * tr * inv, dz * ti * inv);
}


// ======================================================================= wide-tile path --
// For grids with 2 n_t a multiple of 256 the operands are FP16 pairs with power-of-two scales:
// H[i][j] = hscale[i] (Hh + Hl) (split once at set-up) and X[j][c] = xscale[c] (Xh + Xl), so
//   Y[i][c] = hscale[i] xscale[c] (Hh Xh + Hh Xl + Hl Xh)   (FP32 accumulation)
// with ~22 significant bits per operand, three products at the FP16 tensor rate (twice the
// TF32 rate) and half the operand bytes of TF32 parts.
//   qdht_split16_kernel  X [n_r][2 n_t] -> xscale and XhT, XlT [2 n_t][n_r] (K-major: the row
//                        index j contiguous), the inverse transform's window mask applied.
//   qdht_tc2_kernel      the GEMM on 128 (i) x 128 (c) tiles with every operand streamed by
//                        TMA in the K-major layout with the 64-byte swizzle (no conversion in
//                        shared memory): K-blocks of 32 (one 64-byte row), 32 KiB stages, six
//                        in flight; tcgen05.mma.kind::f16 M = 128, N = 128, K = 16, summed in
//                        chunks of 64 of K into three rotating TMEM accumulators.  Warp 0
//                        TMA, warp 1 MMA issuer, warps 2-17 epilogue (four per TMEM lane
//                        quarter, 32 columns each): each chunk is added into FP32 registers,
//                        then the scales are undone and the tile stored / updated.
constexpr int WIDE_COLS = 256;                         // the path takes grids with 2 n_t a multiple of this
constexpr int BN2 = 128, BK2 = 32, STAGES2 = 6;        // K-blocks of 32 FP16 (one 64-byte swizzle row)
constexpr int KCHUNK2 = 2;                              // K-blocks per accumulation chunk (64 of K)
constexpr int NACC2 = 3;                                // TMEM accumulators: the MMA runs NACC2 - 1 chunks ahead
constexpr int TMEM_COLS2 = NACC2 * BN2 <= 256 ? 256 : 512;   // the allocation (a power of two)
static_assert(NACC2 * BN2 <= 512, "accumulators fit tensor memory");
constexpr int A2_BYTES = BM * BK2 * 2;                  // 8 KiB
constexpr int B2_BYTES = BN2 * BK2 * 2;                 // 8 KiB
constexpr int STAGE2_BYTES = 2 * A2_BYTES + 2 * B2_BYTES;
constexpr int NEPI2 = 16;
constexpr int THREADS2 = 64 + 32 * NEPI2;
constexpr int SMEM2_BYTES = STAGES2 * STAGE2_BYTES + 1024 + 256;
// Operand parts are scaled so that the row / column maximum lies in [2^13, 2^14): the low
// parts then stay in FP16's normal range down to 2^-17 of the maximum (scaled to at most 1
// they would fall below it at 2^-3).  Products stay below 2^28 and K-sums below 2^38.
constexpr int OPERAND_EXP = 14;

// Per column c a power of two xscale[c] > 2^-14 max_j |X[j][c]|, then X / xscale[c] = Xh + Xl
// in round-to-nearest FP16 parts, written K-major.  One CTA owns a
// strip of 16 columns: it reads the strip once into shared memory, finds the column maxima
// there and writes the parts as pairs of halves along j.  In shared memory rows j and j + 1
// (j even) share a line of 33 floats (element (j, c) at (j / 2) 33 + (j % 2) 16 + c), so the
// row-wise stores, the column scans and the pair-wise reads are all free of bank conflicts.
// Relative error of the parts ~2^-22 of each value, or 2^-39 of its column's maximum where Xl
// falls below the FP16 normal range.  Dynamic shared memory: (nr / 2) * 33 floats.
constexpr int SPLIT_COLS = 16, SPLIT_THREADS = 512;
__global__ void __launch_bounds__(SPLIT_THREADS) qdht_split16_kernel(const float* __restrict__ X,
                                                                     __half* __restrict__ XhT,
                                                                     __half* __restrict__ XlT,
                                                                     float* __restrict__ xscale, int nr, int ncols,
                                                                     const int* __restrict__ kmax,
                                                                     const int* __restrict__ cmap, int xcompact,
                                                                     const int* __restrict__ run) {
    if (run && *run == 0) return;   // gs_advance: a rejected attempt
    extern __shared__ float strip[];   // [nr / 2][33]
    auto at = [](int j, int c) { return (j >> 1) * 33 + (j & 1) * 16 + c; };
    __shared__ float part[SPLIT_THREADS / SPLIT_COLS][SPLIT_COLS];
    __shared__ float inv[SPLIT_COLS];
    const int tid = threadIdx.x;
    const int c0 = blockIdx.x * SPLIT_COLS;
    // load: a thread takes one (re, im) column pair (a float2) of a row, 32 rows per pass;
    // compact column pairs map to pairs of X's columns (cmap[2q] even, -1: padding, zeros)
    {
        const int q = tid & 7, r0 = tid >> 3;
        const int cm = cmap ? cmap[c0 + 2 * q] : c0 + 2 * q;   // the column (position pair) it stands for
        const int k0 = cm < 0 ? -1 : (kmax ? kmax[cm >> 1] : nr);
        const int ca = xcompact ? c0 + 2 * q : cm;               // where it is read: X is [nr][ncols]
        constexpr int RS = SPLIT_THREADS / 8, LB = 8;   // rows per pass; loads in flight per thread
        for (int jb = r0; jb < nr; jb += LB * RS) {
            float2 v[LB];
#pragma unroll
            for (int u = 0; u < LB; u++) {
                const int j = jb + u * RS;
                // rows past the window (and padding) are zero and not read
                v[u] = (j < nr && j <= k0) ? *reinterpret_cast<const float2*>(X + (size_t)j * ncols + ca)
                                           : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < LB; u++) {
                const int j = jb + u * RS;
                if (j >= nr) break;
                float* d = strip + at(j, 2 * q);
                d[0] = v[u].x;
                d[1] = v[u].y;
            }
        }
    }
    __syncthreads();
    {
        const int c = tid & (SPLIT_COLS - 1), p = tid / SPLIT_COLS;
        float m = 0.f;
        for (int j = p; j < nr; j += SPLIT_THREADS / SPLIT_COLS) m = fmaxf(m, fabsf(strip[at(j, c)]));
        part[p][c] = m;
    }
    __syncthreads();
    if (tid < SPLIT_COLS) {
        float m = 0.f;
        for (int p = 0; p < SPLIT_THREADS / SPLIT_COLS; p++) m = fmaxf(m, part[p][tid]);
        int e = 0;
        if (m > 0.f) frexpf(m, &e);   // m = f 2^e, f in [0.5, 1): |X 2^(14 - e)| < 2^14
        e = max(e, -108);             // keeps both powers of two below inside FP32's normal range
        xscale[c0 + tid] = ldexpf(1.f, e - OPERAND_EXP);
        inv[tid] = ldexpf(1.f, OPERAND_EXP - e);   // exact
    }
    __syncthreads();
    // write: pairs (j, j + 1) of column c as half2, consecutive threads along j
    const int half_rows = nr >> 1;
    for (int idx = tid; idx < SPLIT_COLS * half_rows; idx += SPLIT_THREADS) {
        const int c = idx / half_rows, jp = idx - c * half_rows;
        const float s = inv[c];
        const float v0 = strip[jp * 33 + c] * s, v1 = strip[jp * 33 + 16 + c] * s;
        const __half h0 = __float2half_rn(v0), h1 = __float2half_rn(v1);
        const size_t o = (size_t)(c0 + c) * nr + 2 * jp;
        *reinterpret_cast<__half2*>(XhT + o) = __halves2half2(h0, h1);
        *reinterpret_cast<__half2*>(XlT + o) =
            __halves2half2(__float2half_rn(v0 - __half2float(h0)), __float2half_rn(v1 - __half2float(h1)));
    }
}

__device__ __forceinline__ void mma_f16(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

// shared-memory matrix descriptor for K-major tiles in the 64-byte swizzle: rows of 32 FP16,
// 8-row groups 512 B apart
__device__ __forceinline__ uint64_t make_desc64(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                 // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(512 >> 4) << 32;        // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;                 // descriptor version (sm_100 family)
    d |= (uint64_t)4 << 61;                 // SWIZZLE_64B
    return d;
}

// instruction descriptor: kind::f16, D = F32, A = B = F16 (format code 0), both K-major, M = 128
__host__ __device__ constexpr uint32_t make_idesc_f16(int n) {
    return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

// ---- double-float arithmetic (Dekker's pairs: a value hi + lo, |lo| <= ulp(hi) / 2, built on
// Knuth's TwoSum and the FMA product error), ~48 significant bits on the FP32 pipe ----
struct ff2 {
    float h, l;
};
__device__ __forceinline__ ff2 ff_fast_sum(float a, float b) {   // |a| >= |b|
    const float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ ff2 ff_two_sum(float a, float b) {   // any magnitudes
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
// the sum renormalised by a full TwoSum: under cancellation the error term can exceed the high
// sum, and every stored pair stays canonical (hi = RN(hi + lo)), so a state written out as
// hi + lo in FP64 and split again continues bit for bit
__device__ __forceinline__ ff2 ff_add(ff2 a, ff2 b) {
    const float s = a.h + b.h;
    const float bb = s - a.h;
    const float e = (a.h - (s - bb)) + (b.h - bb) + a.l + b.l;
    return ff_two_sum(s, e);
}
__device__ __forceinline__ ff2 ff_mul(ff2 a, ff2 b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, fmaf(a.l, b.h, e));
    return ff_fast_sum(p, e);
}
__device__ __forceinline__ ff2 ff_mul_f(ff2 a, float b) {
    const float p = a.h * b;
    const float e = fmaf(a.h, b, -p) + a.l * b;
    return ff_fast_sum(p, e);
}
__device__ __forceinline__ ff2 ff_neg(ff2 a) { return {-a.h, -a.l}; }
__host__ __device__ constexpr float ff_hi(double d) { return (float)d; }
__host__ __device__ constexpr float ff_lo(double d) { return (float)(d - (double)(float)d); }

// exp(z) of a complex double-float z = x + i y: the linear step's propagator factor
// exp(dz (k_i + i theta)).  Phase: y reduced by the nearest multiple of pi/2 (Cody and Waite's
// additive reduction with a double-float pi/2), then sin and cos of |r| <= pi/4 from their
// Taylor series (the two leading terms of each in double-float, the rest in FP32: below 2^-46
// absolute); amplitude: exp(x) from its Taylor series for |x| < 2^-6, else the FP32 exponential
// (x is dz times the absorbing layer's k_i, zero inside the medium's window).
__device__ __forceinline__ void ff_cexp(ff2 x, ff2 y, ff2* re, ff2* im) {
    constexpr double PIO2 = 1.57079632679489661923132169163975144;
    const float k = rintf(y.h * (float)(1.0 / PIO2));
    const ff2 r = k == 0.f ? y : ff_add(y, ff_neg(ff_mul_f(ff2{ff_hi(PIO2), ff_lo(PIO2)}, k)));
    const ff2 r2 = ff_mul(r, r);
    const float u = r2.h;
    // sin r = r + r^3 (-1/6 + u/120 + u^2 Ts(u)),  cos r = 1 - u/2 + u^2 (1/24 - u/720 + u^2 Tc(u))
    const float ts = u * (u * (u * (u * (u * (-1.0f / 1307674368000.0f) + 1.0f / 6227020800.0f) - 1.0f / 39916800.0f) +
                               1.0f / 362880.0f) -
                          1.0f / 5040.0f);
    const float tc = u * (u * (u * (u * (u * (1.0f / 20922789888000.0f) - 1.0f / 87178291200.0f) + 1.0f / 479001600.0f) -
                               1.0f / 3628800.0f) +
                          1.0f / 40320.0f);
    const ff2 s_poly = ff_add(ff2{ff_hi(-1.0 / 6), ff_lo(-1.0 / 6)},
                              ff_mul(r2, ff_add(ff2{ff_hi(1.0 / 120), ff_lo(1.0 / 120)}, ff2{ts, 0.f})));
    const ff2 sn = ff_add(r, ff_mul(ff_mul(r, r2), s_poly));
    const ff2 c_poly = ff_add(ff2{ff_hi(1.0 / 24), ff_lo(1.0 / 24)},
                              ff_mul(r2, ff_add(ff2{ff_hi(-1.0 / 720), ff_lo(-1.0 / 720)}, ff2{tc, 0.f})));
    const ff2 cs = ff_add(ff2{1.f, 0.f}, ff_add(ff_mul_f(r2, -0.5f), ff_mul(ff_mul(r2, r2), c_poly)));
    const int q = ((int)k) & 3;
    ff2 c = cs, sv = sn;
    if (q == 1) { c = ff_neg(sn); sv = cs; }
    else if (q == 2) { c = ff_neg(cs); sv = ff_neg(sn); }
    else if (q == 3) { c = sn; sv = ff_neg(cs); }
    if (x.h == 0.f && x.l == 0.f) {   // no absorption (k_i = 0 inside the medium's window)
        *re = c;
        *im = sv;
        return;
    }
    ff2 a;
    if (fabsf(x.h) < 0.015625f) {   // 1 + x + x^2/2 + x^3 (1/6 + x/24 + ...)
        const float t3 = x.h * x.h * x.h * (1.0f / 6 + x.h * (1.0f / 24 + x.h * (1.0f / 120 + x.h * (1.0f / 720))));
        a = ff_add(ff2{1.f, 0.f}, ff_add(x, ff_add(ff_mul_f(ff_mul(x, x), 0.5f), ff2{t3, 0.f})));
    } else {
        a = ff2{expf(x.h), 0.f};
    }
    *re = ff_mul(a, c);
    *im = ff_mul(a, sv);
}

// 32 accumulator columns of row i starting at output column cg: a plain store or the fused
// calculate_Lstep update of BIGBUFFER2 (propagator.cu:570-625)
__device__ __forceinline__ void epilogue_cols(const TcArgs& a, float* v, int i, int cg, float kt2i, float dzh,
                                              float dzl) {
    float* yrow = a.Y + (size_t)i * a.ncols + cg;
    if (a.xscale) {   // FP16 operands: undo the row and column scales (exact: powers of two,
                      // applied one at a time so that their product cannot underflow)
        const float si = a.hscale[i];
#pragma unroll
        for (int k = 0; k < 32; k += 4) {
            const float4 xs = *reinterpret_cast<const float4*>(a.xscale + cg + k);
            v[k] = (v[k] * si) * xs.x;
            v[k + 1] = (v[k + 1] * si) * xs.y;
            v[k + 2] = (v[k + 2] * si) * xs.z;
            v[k + 3] = (v[k + 3] * si) * xs.w;
        }
    }
    if (a.mode != QDHT_LSTEP) {
        if (a.yc) {   // the compact output array, expanded by qdht_expand_kernel
            float* y = a.yc + (size_t)i * a.nc + cg;
#pragma unroll
            for (int k = 0; k < 32; k += 4)
                *reinterpret_cast<float4*>(y + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
            return;
        }
        if (a.cmap) {   // compact columns: pairs scattered back to their columns
            float* y = a.Y + (size_t)i * a.ncols;
#pragma unroll
            for (int k = 0; k < 32; k += 2) {
                const int rc = a.cmap[cg + k];
                if (rc >= 0 && in_bounds(rc + 2 <= a.ncols, a.err))
                    *reinterpret_cast<float2*>(y + rc) = make_float2(v[k], v[k + 1]);
            }
            return;
        }
#pragma unroll
        for (int k = 0; k < 32; k += 4)
            *reinterpret_cast<float4*>(yrow + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
        return;
    }
    if (a.ylo) {
        // BIGBUFFER2's compact copy as double-float pairs, (B2 + dz N / (1 + s)) P with ~48
        // significant bits, so that factors within 2^-24 of 1 (small k_t near omega0, where the
        // step's phase is tiny) still turn the state instead of being lost to FP32 rounding.
        // P = exp(dz (k_i + i theta)) is formed here in double-float arithmetic from the FP64
        // theta table (ff_cexp); outside the window and in the padding (1 / (1 + s) = 0) P = 1, so
        // every element is handled alike and those stay unchanged.  The tables are [pair][row] (a
        // warp's lanes are consecutive rows: coalesced); the loads of four positions are issued
        // before their arithmetic.
        const size_t nr = (size_t)a.nr;
        const size_t t0 = (size_t)(cg >> 1) * nr + i;
        const ff2 dz{dzh, dzl};
        float* yh = a.Y + (size_t)i * a.nc + cg;
        float* yl = a.ylo + (size_t)i * a.nc + cg;
#pragma unroll
        for (int e0 = 0; e0 < 16; e0 += 4) {
            float2 th[4], kk[4];
            float inv[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                th[u] = a.theta[t0 + (size_t)(e0 + u) * nr];
                inv[u] = a.inv1ps[t0 + (size_t)(e0 + u) * nr];
                kk[u] = a.kiff[(cg >> 1) + e0 + u];
            }
            const float4 h0 = *reinterpret_cast<const float4*>(yh + 2 * e0);
            const float4 h1 = *reinterpret_cast<const float4*>(yh + 2 * e0 + 4);
            const float4 l0 = *reinterpret_cast<const float4*>(yl + 2 * e0);
            const float4 l1 = *reinterpret_cast<const float4*>(yl + 2 * e0 + 4);
            const float bh[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
            const float bl[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
            float oh[8], ol[8];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int e = e0 + u;
                if (inv[u] == 0.f) {   // P = 1, nothing added: the pair stays as it is
                    oh[2 * u] = bh[2 * u];
                    oh[2 * u + 1] = bh[2 * u + 1];
                    ol[2 * u] = bl[2 * u];
                    ol[2 * u + 1] = bl[2 * u + 1];
                    continue;
                }
                ff2 pr, pi;
                ff_cexp(ff_mul(dz, ff2{kk[u].x, kk[u].y}), ff_mul(dz, ff2{th[u].x, th[u].y}), &pr, &pi);
                const ff2 br = ff_add(ff2{bh[2 * u], bl[2 * u]}, ff2{dzh * v[2 * e] * inv[u], 0.f});
                const ff2 bi = ff_add(ff2{bh[2 * u + 1], bl[2 * u + 1]}, ff2{dzh * v[2 * e + 1] * inv[u], 0.f});
                const ff2 fr = ff_add(ff_mul(br, pr), ff_neg(ff_mul(bi, pi)));
                const ff2 fi = ff_add(ff_mul(br, pi), ff_mul(bi, pr));
                oh[2 * u] = fr.h;
                oh[2 * u + 1] = fi.h;
                ol[2 * u] = fr.l;
                ol[2 * u + 1] = fi.l;
            }
            *reinterpret_cast<float4*>(yh + 2 * e0) = make_float4(oh[0], oh[1], oh[2], oh[3]);
            *reinterpret_cast<float4*>(yh + 2 * e0 + 4) = make_float4(oh[4], oh[5], oh[6], oh[7]);
            *reinterpret_cast<float4*>(yl + 2 * e0) = make_float4(ol[0], ol[1], ol[2], ol[3]);
            *reinterpret_cast<float4*>(yl + 2 * e0 + 4) = make_float4(ol[4], ol[5], ol[6], ol[7]);
        }
        return;
    }
#pragma unroll
    for (int e = 0; e < 16; e++) {
        const int rc = a.cmap ? a.cmap[cg + 2 * e] : cg + 2 * e;
        if (rc < 0) continue;               // padding
        const int p = rc >> 1;
        if (i > a.kmax[p]) continue;        // outside the window: BIGBUFFER2 untouched
        float2* y2 = reinterpret_cast<float2*>(a.ycompact ? a.Y + (size_t)i * a.nc + cg + 2 * e
                                                          : a.Y + (size_t)i * a.ncols + rc);
        const float k1 = a.kr[p], k2 = a.ki[p];
        const float sq = sqrt_ho_f(-kt2i / k1 / k1);
        float2 b2 = *y2;
        const float inv = 1.f / (1.f + sq);
        b2.x += dzh * v[2 * e] * inv;
        b2.y += dzh * v[2 * e + 1] * inv;
        float sn, cs;
        sincosf(dzh * (-a.ho[p] - sq * k1), &sn, &cs);
        const float m = expf(dzh * k2);
        const float pr = m * cs, pi = m * sn;
        float2 f;
        f.x = b2.x * pr - b2.y * pi;
        f.y = b2.x * pi + b2.y * pr;
        *y2 = f;
    }
}

// Adjoint of the double-float linear step (epilogue_cols with a.ylo) on [n_r][n_t] cotangents:
// T_bar = FIELD_bar + B2_bar, B2_bar = conj(P) T_bar, N_bar = dz T_bar conj(P) / (1 + s), where
// P = exp(dz (k_i + i theta)) comes from the same [pair][row] tables (position p's pair
// cinv[p] / 2) and ff_cexp as the forward's, and B2_bar is carried as double-float pairs
// (sb + sbl) across steps, as the forward carries BIGBUFFER2: factors within 2^-24 of 1 and
// their rounding repeated over many steps would otherwise build up in an FP32 cotangent.
// Outside the window (cinv[p] < 0, or 1 / (1 + s) = 0) B2_bar passes unchanged and N_bar = 0.
__global__ void lstep_adj_ff_kernel(const float2* __restrict__ fb, float2* __restrict__ sb, float2* __restrict__ sbl,
                                    float2* __restrict__ b1b, int nr, int nt, float dzh, float dzl,
                                    const int* __restrict__ cinv, const float2* __restrict__ theta,
                                    const float2* __restrict__ kiff, const float* __restrict__ inv1ps) {
    const size_t total = (size_t)nr * nt;
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int i = (int)(idx / nt), p = (int)(idx % nt);
    const int c = cinv[p];
    const size_t tq = c >= 0 ? (size_t)(c >> 1) * nr + i : 0;
    const float inv = c >= 0 ? inv1ps[tq] : 0.f;
    if (inv == 0.f) {
        b1b[idx] = make_float2(0.f, 0.f);
        return;
    }
    const ff2 dz{dzh, dzl};
    const float2 th = theta[tq], kk = kiff[c >> 1];
    ff2 cr, ci;   // conj(P)
    ff_cexp(ff_mul(dz, ff2{kk.x, kk.y}), ff_neg(ff_mul(dz, ff2{th.x, th.y})), &cr, &ci);
    const float2 f = fb[idx], bh = sb[idx], bl = sbl[idx];
    const ff2 tr = ff_add(ff2{bh.x, bl.x}, ff2{f.x, 0.f});
    const ff2 ti = ff_add(ff2{bh.y, bl.y}, ff2{f.y, 0.f});
    const ff2 rr = ff_add(ff_mul(cr, tr), ff_neg(ff_mul(ci, ti)));
    const ff2 ri = ff_add(ff_mul(cr, ti), ff_mul(ci, tr));
    sb[idx] = make_float2(rr.h, ri.h);
    sbl[idx] = make_float2(rr.l, ri.l);
    b1b[idx] = make_float2(dzh * rr.h * inv, dzh * ri.h * inv);
}

// The masked inverse's result from its compact array: row i of Y (all n_t positions, coalesced)
// takes the pair cinv[p] of yc where p is inside the spectral window and zeros elsewhere.
// Two positions per thread (one 16-byte store), four stores in flight per thread.
__global__ void qdht_expand_kernel(const float* __restrict__ yc, float* __restrict__ Y, int nr, int nt, int nc,
                                   const int* __restrict__ cinv, const int* __restrict__ run) {
    if (run && *run == 0) return;   // gs_advance: a rejected attempt (the masked inverse did not run)
    const size_t total = (size_t)nr * nt / 2;   // position pairs (n_t even)
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t q0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q0 < total; q0 += 4 * stride) {
        float4 v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const size_t q = q0 + u * stride;
            v[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (q < total) {
                const size_t idx = 2 * q, i = idx / nt;
                const int p = (int)(idx - i * nt);
                const int2 c = *reinterpret_cast<const int2*>(cinv + p);
                const float* row = yc + i * nc;
                if (c.x >= 0) { const float2 a = *reinterpret_cast<const float2*>(row + c.x); v[u].x = a.x; v[u].y = a.y; }
                if (c.y >= 0) { const float2 b = *reinterpret_cast<const float2*>(row + c.y); v[u].z = b.x; v[u].w = b.y; }
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const size_t q = q0 + u * stride;
            if (q < total) *reinterpret_cast<float4*>(Y + 4 * q) = v[u];
        }
    }
}

// BIGBUFFER2's window columns to / from their compact double-float copy sc + sl: dir > 0
// S -> sc, sl = 0 (padding columns zero), dir < 0 sc -> S.  One (re, im) pair per thread.
__global__ void qdht_spec_copy_kernel(float* __restrict__ S, float* __restrict__ sc, float* __restrict__ sl, int nr,
                                      int ncols, int nc, const int* __restrict__ cmap, int dir) {
    const size_t total = (size_t)nr * (nc / 2);
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        const size_t i = idx / (nc / 2);
        const int c = 2 * (int)(idx - i * (nc / 2));
        const int rc = cmap[c];
        float2* cpt = reinterpret_cast<float2*>(sc + i * nc + c);
        if (dir > 0) {   // a fresh copy: its low parts are zero
            *cpt = rc >= 0 ? *reinterpret_cast<const float2*>(S + i * ncols + rc) : make_float2(0.f, 0.f);
            *reinterpret_cast<float2*>(sl + i * nc + c) = make_float2(0.f, 0.f);
        } else if (rc >= 0) {   // S takes the high parts (the double-float value rounded to FP32)
            *reinterpret_cast<float2*>(S + i * ncols + rc) = *cpt;
        }
    }
}

// BIGBUFFER2's compact double-float copy from / into an FP64 array X [nr][nt] complex whose
// column q holds position p with q = perm[p] (perm null: q = p): take (dir > 0) sets
// sc = fl32(X), sl = fl32(X - sc) at the window's pairs (zeros in the padding); add (dir < 0)
// adds sl into X at the window's pairs, so that X = sc + sl exactly where X already holds sc.
// X may be pinned host memory reached over the host link.  One pair per thread.
__global__ void qdht_spec_ff_kernel(double2* __restrict__ X, float* __restrict__ sc, float* __restrict__ sl, int nr,
                                    int nt, int nc, const int* __restrict__ cmap, const int* __restrict__ perm,
                                    int dir) {
    const size_t total = (size_t)nr * (nc / 2);
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        const size_t i = idx / (nc / 2);
        const int c = 2 * (int)(idx - i * (nc / 2));
        const int rc = cmap[c];
        float2* hp = reinterpret_cast<float2*>(sc + i * nc + c);
        float2* lp = reinterpret_cast<float2*>(sl + i * nc + c);
        if (rc < 0) {
            if (dir > 0) {
                *hp = make_float2(0.f, 0.f);
                *lp = make_float2(0.f, 0.f);
            }
            continue;
        }
        const int pp = rc >> 1;
        double2* x = X + i * (size_t)nt + (perm ? perm[pp] : pp);
        if (dir > 0) {
            const double2 v = *x;
            const float hx = (float)v.x, hy = (float)v.y;
            *hp = make_float2(hx, hy);
            *lp = make_float2((float)(v.x - (double)hx), (float)(v.y - (double)hy));
        } else {
            const float2 l = *lp;
            double2 v = *x;
            v.x += (double)l.x;
            v.y += (double)l.y;
            *x = v;
        }
    }
}

// The compact double-float copy from device arrays in position order, S (high parts) and lo
// (low parts), both [nr][ncols] floats: take (dir > 0) sets sc, sl at the window's pairs (zeros
// in the padding); scatter (dir < 0) writes lo over all of [nr][ncols]: sl at the window's pairs,
// zeros elsewhere (cinv[p]: the compact column of position p, or -1).
__global__ void qdht_spec_dev_kernel(const float* __restrict__ S, float* __restrict__ lo, float* __restrict__ sc,
                                     float* __restrict__ sl, int nr, int ncols, int nc, const int* __restrict__ cmap,
                                     const int* __restrict__ cinv, int dir) {
    if (dir > 0) {
        const size_t total = (size_t)nr * (nc / 2);
        for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
            const size_t i = idx / (nc / 2);
            const int c = 2 * (int)(idx - i * (nc / 2));
            const int rc = cmap[c];
            float2 h = make_float2(0.f, 0.f), l = make_float2(0.f, 0.f);
            if (rc >= 0) {
                h = *reinterpret_cast<const float2*>(S + i * ncols + rc);
                l = *reinterpret_cast<const float2*>(lo + i * ncols + rc);
            }
            *reinterpret_cast<float2*>(sc + i * nc + c) = h;
            *reinterpret_cast<float2*>(sl + i * nc + c) = l;
        }
        return;
    }
    const size_t total = (size_t)nr * (ncols / 2);
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        const size_t i = idx / (ncols / 2);
        const int p = (int)(idx - i * (ncols / 2));
        const int c = cinv[p];
        *reinterpret_cast<float2*>(lo + i * ncols + 2 * p) =
            c >= 0 ? *reinterpret_cast<const float2*>(sl + i * nc + c) : make_float2(0.f, 0.f);
    }
}

// Self-test of the bounded waits: one thread waits on a shared-memory mbarrier that nothing
// arrives at, with the same helper as the GEMM's waits (limit_ns instead of WAIT_NS), records the
// expiry in the plan's error words as they do and returns.  No copy is in flight, so returning is
// safe; the host reads the record through qdht_tc_check, as after a GEMM.
__global__ void wait_probe_kernel(unsigned* err, unsigned long long limit_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (!mbar_wait_ns(&bar, 0, limit_ns)) record_stall(err, 256u, 0, 0);
    }
}

// Zeros of the masked inverse outside the spectral window: Y[i][2 p], Y[i][2 p + 1] = 0 for
// the positions p in zpos[nz] (their whole column of the operand is masked)
__global__ void qdht_zero_cols_kernel(float* __restrict__ Y, int ncols, int nr, const int* __restrict__ zpos, int nz,
                                      const int* __restrict__ run) {
    if (run && *run == 0) return;   // gs_advance: a rejected attempt
    const size_t total = (size_t)nr * nz;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        const size_t i = idx / nz;
        const int z = (int)(idx - i * nz);
        *reinterpret_cast<float2*>(Y + i * ncols + 2 * zpos[z]) = make_float2(0.f, 0.f);
    }
}

__global__ void __launch_bounds__(THREADS2, 1) qdht_tc2_kernel(const __grid_constant__ CUtensorMap map_hi,
                                                               const __grid_constant__ CUtensorMap map_lo,
                                                               const __grid_constant__ CUtensorMap map_bh,
                                                               const __grid_constant__ CUtensorMap map_bl, TcArgs a) {
    if (a.run && *a.run == 0) return;   // gs_advance: a rejected attempt (before any set-up)
    float dzh = a.dz, dzl = a.dz_lo;
    if (a.dz_dev) {
        const double d = *a.dz_dev;
        dzh = (float)d;
        dzl = (float)(d - (double)dzh);
    }
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = (uint64_t*)(smem + STAGES2 * STAGE2_BYTES);
    uint64_t* full = bars;                    // [STAGES2] TMA tx
    uint64_t* empty = bars + STAGES2;         // [STAGES2] MMA commit
    uint64_t* acc_full = bars + 2 * STAGES2;  // [NACC2] MMA commit: a chunk's accumulator ready
    uint64_t* acc_empty = acc_full + NACC2;   // [NACC2] NEPI2 epilogue warps: read out
    uint64_t* done = acc_empty + NACC2;       // every MMA of this CTA complete
    uint32_t* tmem_slot = (uint32_t*)(done + 1);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int MT = a.nr / BM;
    const int ntiles = MT * (a.nc / BN2);
    const int nk = a.nr / BK2;
    const int nch = nk / KCHUNK2;             // accumulation chunks per tile
    const int my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES2; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < NACC2; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], NEPI2);
        }
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS2));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        // ------------------------------------------------ TMA producer (Hh, Hl, XhT, XlT)
        if (lane == 0) {
            int issued = 0;
            for (int it = 0; it < my_tiles && !*abort_flag; it++) {
                const int T = blockIdx.x + it * gridDim.x;
                const int m0 = (T % MT) * BM, c0 = (T / MT) * BN2;
                for (int kb = 0; kb < nk; kb++) {
                    const int g = it * nk + kb;
                    const int s = g % STAGES2;
                    if (g >= STAGES2 && !mbar_wait(&empty[s], ((g / STAGES2) + 1) & 1)) {
                        record_stall(a.err, 4u, kb, warp);
                        *abort_flag = 1;
                        break;
                    }
                    if (*abort_flag) break;
                    unsigned char* st = smem + s * STAGE2_BYTES;
                    mbar_expect_tx(&full[s], STAGE2_BYTES);
                    tma_load_2d(st, &map_hi, kb * BK2, m0, &full[s]);
                    tma_load_2d(st + A2_BYTES, &map_lo, kb * BK2, m0, &full[s]);
                    tma_load_2d(st + 2 * A2_BYTES, &map_bh, kb * BK2, c0, &full[s]);
                    tma_load_2d(st + 2 * A2_BYTES + B2_BYTES, &map_bl, kb * BK2, c0, &full[s]);
                    issued = g + 1;
                }
            }
            for (int g = (issued > STAGES2 ? issued - STAGES2 : 0); g < issued; g++)
                if (!mbar_wait(&full[g % STAGES2], (g / STAGES2) & 1)) record_stall(a.err, 128u, g % nk, warp);
        }
        __syncwarp();
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        // Each chunk of KCHUNK2 K-blocks is summed afresh into accumulator buffer u % NACC2 (u the
        // CTA's running chunk count), the correction products Hh Xl + Hl Xh of the chunk first
        // and its main products Hh Xh last; the epilogue adds the chunks in FP32 registers.
        // The tensor core's accumulation truncates: with a fresh, small accumulator per chunk
        // and the small terms summed first, its error stays ~2^-22 of the result instead of
        // growing with the whole K = n_r sum.
        if (lane == 0) {
            constexpr uint32_t idesc = make_idesc_f16(BN2);
            bool ok = true;
            for (int it = 0; it < my_tiles && ok && !*abort_flag; it++) {
                for (int c = 0; c < nch; c++) {
                    const int u = it * nch + c, b = u % NACC2;
                    if (u >= NACC2 && !mbar_wait(&acc_empty[b], ((u / NACC2) - 1) & 1)) {
                        record_stall(a.err, 4096u, c, warp);
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    uint32_t st_addr[KCHUNK2];
                    int st_idx[KCHUNK2];
                    for (int j = 0; j < KCHUNK2 && ok; j++) {
                        const int g = it * nk + c * KCHUNK2 + j;
                        const int s = g % STAGES2;
                        if (!mbar_wait(&full[s], (g / STAGES2) & 1)) {
                            record_stall(a.err, 8u, c * KCHUNK2 + j, warp);
                            ok = false;
                        }
                        st_idx[j] = s;
                        st_addr[j] = smem_u32(smem + s * STAGE2_BYTES);
                    }
                    if (!ok || *abort_flag) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t d = tmem + (uint32_t)(b * BN2);
                    uint32_t acc = 0;
#pragma unroll
                    for (int j = 0; j < KCHUNK2; j++) {
                        const uint32_t ah = st_addr[j], al = ah + A2_BYTES;
                        const uint32_t bh = ah + 2 * A2_BYTES, bl = bh + B2_BYTES;
#pragma unroll
                        for (int kk = 0; kk < BK2 / 16; kk++) {
                            const uint32_t off = kk * 32;   // 16 FP16 = 32 bytes along K inside the swizzle row
                            mma_f16(d, make_desc64(al + off), make_desc64(bh + off), idesc, acc);
                            acc = 1;
                            mma_f16(d, make_desc64(ah + off), make_desc64(bl + off), idesc, 1);
                        }
                    }
#pragma unroll
                    for (int j = 0; j < KCHUNK2; j++) {
                        const uint32_t ah = st_addr[j], bh = ah + 2 * A2_BYTES;
#pragma unroll
                        for (int kk = 0; kk < BK2 / 16; kk++) {
                            const uint32_t off = kk * 32;
                            mma_f16(d, make_desc64(ah + off), make_desc64(bh + off), idesc, 1);
                        }
                    }
                    for (int j = 0; j < KCHUNK2; j++) mma_commit(&empty[st_idx[j]]);
                    mma_commit(&acc_full[b]);
                }
            }
            if (!ok) *abort_flag = 1;
            mma_commit(done);
        }
        __syncwarp();
    } else {
        // ------------------------------------------------ epilogue: each warp reads its 32
        // accumulator columns of every chunk, hands the buffer back, adds the chunk to its
        // running sums (round-to-nearest FP32), and after the last chunk stores / updates
        const int q = warp & 3;                 // TMEM lane quarter this warp may read
        const int part = (warp - 2) >> 2;       // which 32 columns (0..3)
        bool ok = true;
        for (int it = 0; it < my_tiles && ok; it++) {
            const int T = blockIdx.x + it * gridDim.x;
            const int m0 = (T % MT) * BM, c0 = (T / MT) * BN2;
            const int i = m0 + 32 * q + lane;
            float sum[32];
            for (int c = 0; c < nch; c++) {
                const int u = it * nch + c, b = u % NACC2;
                ok = __all_sync(0xffffffffu, mbar_wait(&acc_full[b], (u / NACC2) & 1) ? 1 : 0) != 0;
                if (!ok) {
                    if (lane == 0) record_stall(a.err, 32u, c, warp);
                    *abort_flag = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                if (__any_sync(0xffffffffu, *abort_flag)) {   // warp-uniform: tcgen05.ld is .sync.aligned
                    ok = false;
                    break;
                }
                float v[32];
                tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * BN2 + 32 * part), v);
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&acc_empty[b]);
                if (c == 0) {
#pragma unroll
                    for (int k = 0; k < 32; k++) sum[k] = v[k];
                } else {
#pragma unroll
                    for (int k = 0; k < 32; k++) sum[k] = __fadd_rn(sum[k], v[k]);
                }
            }
            if (!ok) break;
            const float kt2i = a.kt2 ? a.kt2[i] : 0.f;
            epilogue_cols(a, sum, i, c0 + 32 * part, kt2i, dzh, dzl);
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }

    __syncthreads();
    if (warp == 1) {
        if (lane == 0 && !mbar_wait(done, 0)) record_stall(a.err, 64u, nk, warp);
        __syncwarp();
    }
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS2));
    }
}

}  // namespace tc

struct QdhtTc {
    int nr = 0, nt = 0;
    int sms = 0;   // persistent grid: one CTA per SM
    cudaStream_t st = nullptr;
    float *hh = nullptr, *hl = nullptr;
    float *kr = nullptr, *ki = nullptr, *ho = nullptr, *kt2 = nullptr;
    int* kmax = nullptr;
    unsigned* err = nullptr;
    CUtensorMap map_hi, map_lo;
    bool have_lstep = false;
    // wide-tile path (2 n_t a multiple of 256): X split once into K-major FP16 hi / lo parts
    // of X / xscale[c], H held as FP16 hi / lo parts of H[i][j] / hscale[i]
    bool wide = false;
    float *xhT = nullptr, *xlT = nullptr;   // [2 n_t][n_r] halves
    __half *hh16 = nullptr, *hl16 = nullptr;
    float *hs = nullptr, *xs = nullptr;     // hscale[n_r], xscale[2 n_t]
    // the spectral window's columns (kmax >= 0) for the linear-step and masked transforms:
    // cmap[nc_act] (padded with -1 to a multiple of 256) and the positions outside, zpos[nz]
    int *cmap = nullptr, *zpos = nullptr;
    int nc_act = 0, nz = 0;
    int* cinv = nullptr;      // [n_t]: compact column of position p's pair (even), or -1
    float* yc = nullptr;      // [n_r][nc_act]: the masked inverse's compact result
    float* xc = nullptr;      // [n_r][nc_act]: a compact linear-step input written by its producer
    float* sc = nullptr;      // [n_r][nc_act]: BIGBUFFER2's window columns kept compact between steps
    float* sl = nullptr;      // [n_r][nc_act]: their low parts (the compact copy is the double-float sc + sl)
    // the linear step's factors on the compact columns, per pair c / 2 and row i ([nc_act / 2][n_r]):
    // theta = -HO - sqrtHO(-kt2 / k_r^2) k_r and k_i (per pair) as double-float pairs, 1 / (1 + s)
    float2* theta = nullptr;
    float2* kiff = nullptr;
    float* inv1ps = nullptr;
    CUtensorMap map_bh, map_bl, map_hi64, map_lo64;   // 32-half boxes in the 64-byte swizzle
    // tensor maps of the X operands seen so far (the handle's few state arrays)
    std::vector<std::pair<const float*, CUtensorMap>> xmaps;
};

static PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

static cudaError_t split_smem_ceiling() {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, tc::qdht_split16_kernel);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(tc::qdht_split16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(227 * 1024 - fa.sharedSizeBytes));
}

QdhtTc* qdht_tc_create(int nr, int nt, cudaStream_t st, std::string* msg) {
    if (nr % tc::BM != 0) {
        if (msg) *msg = "the tensor-core QDHT needs N_R to be a multiple of 128";
        return nullptr;
    }
    if ((2 * nt) % tc::BN != 0) {
        if (msg) *msg = "N_T must be a multiple of 64";
        return nullptr;
    }
    if (!get_encode()) {
        if (msg) *msg = "cuTensorMapEncodeTiled unavailable";
        return nullptr;
    }
    QdhtTc* q = new QdhtTc();
    q->nr = nr;
    q->nt = nt;
    q->st = st;
    bool ok = cudaMalloc(&q->hh, (size_t)nr * nr * 4) == cudaSuccess && cudaMalloc(&q->hl, (size_t)nr * nr * 4) == cudaSuccess &&
              cudaMalloc(&q->kr, nt * 4) == cudaSuccess && cudaMalloc(&q->ki, nt * 4) == cudaSuccess &&
              cudaMalloc(&q->ho, nt * 4) == cudaSuccess && cudaMalloc(&q->kt2, nr * 4) == cudaSuccess &&
              cudaMalloc(&q->kmax, nt * 4) == cudaSuccess && cudaMalloc(&q->err, 8) == cudaSuccess;
    if (ok) ok = cudaMemset(q->err, 0, 8) == cudaSuccess;
    int dev = 0;
    if (ok) ok = cudaGetDevice(&dev) == cudaSuccess &&
                 cudaDeviceGetAttribute(&q->sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && q->sms > 0;
    if (ok) ok = cudaFuncSetAttribute(tc::qdht_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES) ==
                 cudaSuccess;
    if (!ok) {
        if (msg) *msg = "allocation / attribute failed";
        qdht_tc_destroy(q);
        return nullptr;
    }
    auto enc = get_encode();
    for (int w = 0; w < 2; w++) {
        CUtensorMap* m = w ? &q->map_lo : &q->map_hi;
        cuuint64_t gdim[2] = {(cuuint64_t)nr, (cuuint64_t)nr};           // {K (j), M (i)}
        cuuint64_t gstride[1] = {(cuuint64_t)nr * 4};
        cuuint32_t box[2] = {(cuuint32_t)tc::BK, (cuuint32_t)tc::BM};   // 32 floats = 128 B inner
        cuuint32_t estr[2] = {1, 1};
        CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, w ? (void*)q->hl : (void*)q->hh, gdim, gstride, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) {
            if (msg) *msg = "cuTensorMapEncodeTiled failed";
            qdht_tc_destroy(q);
            return nullptr;
        }
    }
    q->wide = (2 * nt) % tc::WIDE_COLS == 0;
    if (q->wide) {
        const size_t ncols = 2 * (size_t)nt;
        bool okw = cudaMalloc(&q->xhT, ncols * nr * 2) == cudaSuccess && cudaMalloc(&q->xlT, ncols * nr * 2) == cudaSuccess &&
                   cudaMalloc(&q->hh16, (size_t)nr * nr * 2) == cudaSuccess &&
                   cudaMalloc(&q->hl16, (size_t)nr * nr * 2) == cudaSuccess && cudaMalloc(&q->hs, nr * 4) == cudaSuccess &&
                   cudaMalloc(&q->xs, ncols * 4) == cudaSuccess &&
                   cudaFuncSetAttribute(tc::qdht_tc2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        tc::SMEM2_BYTES) == cudaSuccess &&
                   (size_t)(nr / 2) * 33 * 4 <= 227 * 1024 &&
                   // a per-kernel ceiling shared by every plan of the process: the device maximum
                   // less the kernel's static shared memory, so that a plan for fewer rows never
                   // lowers it below a larger plan's need
                   split_smem_ceiling() == cudaSuccess;
        for (int w = 0; okw && w < 2; w++) {
            // [2 n_t rows c][n_r halves j]: boxes of 32 j (64 B, swizzled) x 256 c
            cuuint64_t gdim[2] = {(cuuint64_t)nr, (cuuint64_t)ncols};
            cuuint64_t gstride[1] = {(cuuint64_t)nr * 2};
            cuuint32_t box[2] = {(cuuint32_t)tc::BK2, (cuuint32_t)tc::BN2};
            cuuint32_t estr[2] = {1, 1};
            okw = enc(w ? &q->map_bl : &q->map_bh, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, w ? (void*)q->xlT : (void*)q->xhT,
                      gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
        }
        for (int w = 0; okw && w < 2; w++) {   // H hi / lo in 32-half boxes of 128 rows
            cuuint64_t gdim[2] = {(cuuint64_t)nr, (cuuint64_t)nr};
            cuuint64_t gstride[1] = {(cuuint64_t)nr * 2};
            cuuint32_t box[2] = {(cuuint32_t)tc::BK2, (cuuint32_t)tc::BM};
            cuuint32_t estr[2] = {1, 1};
            okw = enc(w ? &q->map_lo64 : &q->map_hi64, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2,
                      w ? (void*)q->hl16 : (void*)q->hh16, gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                      CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                      CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
        }
        if (!okw) {
            if (msg) *msg = "wide-tile QDHT set-up failed";
            qdht_tc_destroy(q);
            return nullptr;
        }
    }
    float k[20];
    double b = 1.0;
    for (int n = 1; n <= 20; n++) { b *= (0.5 - (n - 1)) / n; k[n - 1] = (float)b; }
    if (cudaMemcpyToSymbol(tc::c_sqrt_ho_f, k, sizeof(k)) != cudaSuccess) {
        if (msg) *msg = "constant upload failed";
        qdht_tc_destroy(q);
        return nullptr;
    }
    return q;
}

int qdht_tc_set_matrix(QdhtTc* q, const double* C, const double* m1, std::string* msg) {
    const int nr = q->nr;
    std::vector<float> hh((size_t)nr * nr), hl((size_t)nr * nr);
    for (int i = 0; i < nr; i++)
        for (int j = 0; j < nr; j++) {
            const double h = m1[i] * C[(size_t)i + (size_t)nr * j] / m1[j];
            // round-to-nearest TF32 (10 explicit mantissa bits) high part, FP32 remainder
            float f = (float)h;
            uint32_t u;
            std::memcpy(&u, &f, 4);
            u = (u + 0x1000u) & 0xFFFFE000u;
            float hi;
            std::memcpy(&hi, &u, 4);
            hh[(size_t)i * nr + j] = hi;
            hl[(size_t)i * nr + j] = (float)(h - (double)hi);
        }
    if (cudaMemcpy(q->hh, hh.data(), hh.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(q->hl, hl.data(), hl.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
        if (msg) *msg = "matrix upload failed";
        return 1;
    }
    if (q->wide) {
        // FP16 parts of H[i][j] / hscale[i], hscale[i] the power of two above 2^-14 of the row's
        // largest |H|: Hh round-to-nearest, Hl the rounded remainder (computed in FP64)
        std::vector<__half> h16((size_t)nr * nr), l16((size_t)nr * nr);
        std::vector<float> hs(nr);
        for (int i = 0; i < nr; i++) {
            double m = 0;
            for (int j = 0; j < nr; j++) m = std::max(m, std::fabs(m1[i] * C[(size_t)i + (size_t)nr * j] / m1[j]));
            int e = 0;
            if (m > 0) std::frexp(m, &e);
            e = std::max(e, -108);
            const double sc = std::ldexp(1.0, e - tc::OPERAND_EXP);   // |H / sc| < 2^14
            hs[i] = (float)sc;
            for (int j = 0; j < nr; j++) {
                const double h = m1[i] * C[(size_t)i + (size_t)nr * j] / m1[j] / sc;
                const __half hi = __float2half_rn((float)h);
                h16[(size_t)i * nr + j] = hi;
                l16[(size_t)i * nr + j] = __float2half_rn((float)(h - (double)__half2float(hi)));
            }
        }
        if (cudaMemcpy(q->hh16, h16.data(), h16.size() * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(q->hl16, l16.data(), l16.size() * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(q->hs, hs.data(), nr * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
            if (msg) *msg = "matrix upload failed";
            return 1;
        }
    }
    return 0;
}

int qdht_tc_set_lstep(QdhtTc* q, const double* omega, const double* wavenum, const double* ho, const double* kt2,
                      double omega_min, double omega_max, std::string* msg) {
    const int nt = q->nt, nr = q->nr;
    std::vector<float> kr(nt), ki(nt), hf(nt), k2(nr);
    std::vector<int> kmax(nt);
    for (int p = 0; p < nt; p++) {
        kr[p] = (float)wavenum[2 * p];
        ki[p] = (float)wavenum[2 * p + 1];
        hf[p] = (float)ho[p];
        // calculate_Lstep's window, decided in FP64: omega in [min, max] and kt2 <= 0.25 Re(k^2)
        int km = -1;
        if (!(omega[p] < omega_min || omega[p] > omega_max)) {
            const double lim = 0.25 * (wavenum[2 * p] * wavenum[2 * p] - wavenum[2 * p + 1] * wavenum[2 * p + 1]);
            for (int k = 0; k < nr; k++)
                if (!(kt2[k] > lim)) km = k;
        }
        kmax[p] = km;
    }
    for (int k = 0; k < nr; k++) k2[k] = (float)kt2[k];
    bool ok = cudaMemcpy(q->kr, kr.data(), nt * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(q->ki, ki.data(), nt * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(q->ho, hf.data(), nt * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(q->kt2, k2.data(), nr * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(q->kmax, kmax.data(), nt * 4, cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) {
        if (msg) *msg = "linear-step table upload failed";
        return 1;
    }
    if (q->wide) {
        // compact column list of the window (pairs of real columns), padded to whole tiles
        std::vector<int> cm, zp;
        for (int p = 0; p < nt; p++) {
            if (kmax[p] >= 0) {
                cm.push_back(2 * p);
                cm.push_back(2 * p + 1);
            } else {
                zp.push_back(p);
            }
        }
        while (cm.size() % tc::BN2) cm.push_back(-1);
        std::vector<int> ci(nt, -1);
        for (size_t c = 0; c < cm.size(); c += 2)
            if (cm[c] >= 0) ci[cm[c] >> 1] = (int)c;
        if (q->cmap) cudaFree(q->cmap);
        if (q->zpos) cudaFree(q->zpos);
        if (q->cinv) cudaFree(q->cinv);
        if (q->yc) cudaFree(q->yc);
        if (q->xc) cudaFree(q->xc);
        if (q->sc) cudaFree(q->sc);
        if (q->sl) cudaFree(q->sl);
        q->sl = nullptr;
        q->cmap = q->zpos = q->cinv = nullptr;
        q->yc = q->xc = q->sc = nullptr;
        q->nc_act = (int)cm.size();
        q->nz = (int)zp.size();
        bool okc = (cm.empty() || (cudaMalloc(&q->cmap, cm.size() * 4) == cudaSuccess &&
                                   cudaMemcpy(q->cmap, cm.data(), cm.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess)) &&
                   (zp.empty() || (cudaMalloc(&q->zpos, zp.size() * 4) == cudaSuccess &&
                                   cudaMemcpy(q->zpos, zp.data(), zp.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess)) &&
                   cudaMalloc(&q->cinv, (size_t)nt * 4) == cudaSuccess &&
                   cudaMemcpy(q->cinv, ci.data(), (size_t)nt * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
                   (cm.empty() || (cudaMalloc(&q->yc, (size_t)nr * cm.size() * 4) == cudaSuccess &&
                                   cudaMalloc(&q->xc, (size_t)nr * cm.size() * 4) == cudaSuccess &&
                                   cudaMalloc(&q->sc, (size_t)nr * cm.size() * 4) == cudaSuccess &&
                                   cudaMalloc(&q->sl, (size_t)nr * cm.size() * 4) == cudaSuccess &&
                                   cudaMemset(q->sl, 0, (size_t)nr * cm.size() * 4) == cudaSuccess &&
                                   cudaMemset(q->xc, 0, (size_t)nr * cm.size() * 4) == cudaSuccess));
        if (!okc) {
            if (msg) *msg = "window column list upload failed";
            return 1;
        }
        // theta and 1 / (1 + s) per compact pair and row ([pair][row]: the epilogue's lanes are rows)
        // in FP64 (calculate_Lstep, propagator.cu:614-616, with the reference's 20-term sqrtHO,
        // extmath.h:245-256); 1 / (1 + s) = 0 marks elements outside the window and padding, whose
        // factor is exactly 1 so that the linear step leaves them unchanged
        double hk[20], bc = 1.0;
        for (int n = 1; n <= 20; n++) { bc *= (0.5 - (n - 1)) / n; hk[n - 1] = bc; }
        const size_t npair = cm.size() / 2;
        std::vector<float2> th((size_t)nr * npair, make_float2(0.f, 0.f)), kf(npair, make_float2(0.f, 0.f));
        std::vector<float> iv((size_t)nr * npair, 0.f);
        for (size_t c2 = 0; c2 < npair; c2++) {
            const int rc = cm[2 * c2];
            if (rc < 0) continue;
            const int pp = rc >> 1;
            const double k1 = wavenum[2 * pp], k2 = wavenum[2 * pp + 1];
            kf[c2] = make_float2((float)k2, (float)(k2 - (double)(float)k2));
            for (int i = 0; i <= kmax[pp]; i++) {
                const double x = -kt2[i] / k1 / k1;
                double sq = 0, xn = x;
                for (int j = 0; j < 20; j++) { sq += hk[j] * xn; xn *= x; }
                const double t = -ho[pp] - sq * k1;
                th[c2 * (size_t)nr + i] = make_float2((float)t, (float)(t - (double)(float)t));
                iv[c2 * (size_t)nr + i] = (float)(1.0 / (1.0 + sq));
            }
        }
        if (q->theta) cudaFree(q->theta);
        if (q->kiff) cudaFree(q->kiff);
        if (q->inv1ps) cudaFree(q->inv1ps);
        q->theta = nullptr;
        q->kiff = nullptr;
        q->inv1ps = nullptr;
        if (npair > 0) {
            const size_t ne = (size_t)nr * npair;
            const bool okf = cudaMalloc(&q->theta, ne * sizeof(float2)) == cudaSuccess &&
                             cudaMalloc(&q->kiff, npair * sizeof(float2)) == cudaSuccess &&
                             cudaMalloc(&q->inv1ps, ne * sizeof(float)) == cudaSuccess &&
                             cudaMemcpy(q->theta, th.data(), ne * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess &&
                             cudaMemcpy(q->kiff, kf.data(), npair * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess &&
                             cudaMemcpy(q->inv1ps, iv.data(), ne * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
            if (!okf) {
                if (msg) *msg = "linear-step factor tables: allocation or upload failed";
                return 1;
            }
        }
    }
    q->have_lstep = true;
    return 0;
}

cudaError_t qdht_tc_run(QdhtTc* q, int mode, const float* X, float* Y, const LstepArgs& L, long long* nlaunch,
                        std::string* msg, int flags) {
    if (mode != QDHT_PLAIN && !q->have_lstep) {
        if (msg) *msg = "linear-step tables not set";
        return cudaErrorInvalidValue;
    }
    tc::TcArgs a;
    a.X = X;
    a.Y = Y;
    a.nr = q->nr;
    a.ncols = 2 * q->nt;
    a.mode = mode;
    a.dz = (float)L.dz;
    a.kr = q->kr;
    a.ki = q->ki;
    a.ho = q->ho;
    a.kt2 = q->kt2;
    a.kmax = q->kmax;
    a.err = q->err;
    a.hscale = nullptr;
    a.xscale = nullptr;
    a.nc = a.ncols;
    a.cmap = nullptr;
    a.yc = nullptr;
    a.ycompact = 0;
    a.theta = nullptr;
    a.kiff = nullptr;
    a.inv1ps = nullptr;
    a.ylo = nullptr;
    a.dz_lo = (float)(L.dz - (double)(float)L.dz);
    a.dz_dev = L.dz_dev;
    a.run = L.run;
    if (q->wide) {
        // The linear step leaves BIGBUFFER2 untouched outside the spectral window and the masked
        // inverse transforms a zero column there: both run on the window's columns only (the
        // compact list), the masked one writing the zeros of the other columns directly.
        const bool compact = mode != QDHT_PLAIN;
        if (compact) {
            a.nc = q->nc_act;
            a.cmap = q->cmap;
            if (mode == QDHT_MASKED && a.nc > 0) a.yc = q->yc;   // expanded into Y below
            if (mode == QDHT_MASKED && a.nc == 0 && q->nz > 0) {
                const size_t tot = (size_t)q->nr * q->nz;
                const unsigned gz = (unsigned)std::min<size_t>((tot + 255) / 256, (size_t)q->sms * 16);
                tc::qdht_zero_cols_kernel<<<gz, 256, 0, q->st>>>(Y, a.ncols, q->nr, q->zpos, q->nz, L.run);
                (*nlaunch)++;
            }
        }
        if (a.nc == 0) return cudaGetLastError();
        const bool s_comp = compact && (flags & QTC_S_COMPACT) && q->sc;
        // where the split reads a compact X: BIGBUFFER1's window columns (linear step) or
        // BIGBUFFER2's compact copy (masked inverse)
        const float* xsrc = nullptr;
        if (mode == QDHT_LSTEP && (flags & QTC_X_COMPACT)) xsrc = q->xc;
        if (mode == QDHT_MASKED && s_comp) xsrc = q->sc;
        const bool xc = xsrc != nullptr;
        if (mode == QDHT_LSTEP && s_comp) {   // the epilogue updates the compact double-float copy
            Y = q->sc;
            a.Y = q->sc;
            a.ycompact = 1;
            if (q->theta) {
                a.ylo = q->sl;
                a.theta = q->theta;
                a.kiff = q->kiff;
                a.inv1ps = q->inv1ps;
            }
        }

        // split X into the K-major FP16 hi / lo operands and the column scales (the window mask
        // of the inverse applied), then the GEMM on 128 x 128 tiles
        tc::qdht_split16_kernel<<<(unsigned)(a.nc / tc::SPLIT_COLS), tc::SPLIT_THREADS, (size_t)(q->nr / 2) * 33 * 4,
                                  q->st>>>(xc ? xsrc : X, (__half*)q->xhT, (__half*)q->xlT, q->xs, q->nr,
                                           xc ? a.nc : a.ncols, mode == QDHT_MASKED ? q->kmax : nullptr, a.cmap, xc,
                                           L.run);
        (*nlaunch)++;
        a.hscale = q->hs;
        a.xscale = q->xs;
        const int nt2 = (q->nr / tc::BM) * (a.nc / tc::BN2);
        const unsigned g2 = (unsigned)(nt2 < q->sms ? nt2 : q->sms);
        tc::qdht_tc2_kernel<<<g2, tc::THREADS2, tc::SMEM2_BYTES, q->st>>>(q->map_hi64, q->map_lo64, q->map_bh, q->map_bl, a);
        (*nlaunch)++;
        if (a.yc && !(flags & QTC_Y_LAZY)) return qdht_tc_expand(q, Y, nlaunch, L.run);
        return cudaGetLastError();
    }
    const int ntiles = (q->nr / tc::BM) * (a.ncols / tc::BN);
    const unsigned grid = (unsigned)(ntiles < q->sms ? ntiles : q->sms);
    const CUtensorMap* mx = nullptr;
    for (auto& e : q->xmaps)
        if (e.first == X) mx = &e.second;
    if (!mx) {
        // X as [n_r rows][2 n_t floats]; boxes of 32 rows x 128 columns, unswizzled (the
        // column coordinate c0 is a multiple of 128 floats: 16-byte aligned)
        CUtensorMap m;
        cuuint64_t gdim[2] = {(cuuint64_t)(2 * q->nt), (cuuint64_t)q->nr};
        cuuint64_t gstride[1] = {(cuuint64_t)(2 * q->nt) * 4};
        cuuint32_t box[2] = {(cuuint32_t)tc::BN, (cuuint32_t)tc::BK};
        cuuint32_t estr[2] = {1, 1};
        CUresult r = get_encode()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)X, gdim, gstride, box, estr,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) {
            if (msg) *msg = "cuTensorMapEncodeTiled (X) failed";
            return cudaErrorInvalidValue;
        }
        q->xmaps.emplace_back(X, m);
        mx = &q->xmaps.back().second;
    }
    tc::qdht_tc_kernel<<<grid, tc::THREADS, tc::SMEM_BYTES, q->st>>>(q->map_hi, q->map_lo, *mx, a);
    (*nlaunch)++;
    return cudaGetLastError();
}

cudaError_t qdht_tc_lstep_adj(QdhtTc* q, const float* fb, float* sb, float* sbl, float* b1b, double dz,
                              long long* nlaunch) {
    if (!q->have_lstep) return cudaErrorInvalidValue;
    const size_t total = (size_t)q->nr * q->nt;
    if (sbl && qdht_tc_lstep_adj_ff(q)) {   // the double-float forward's adjoint
        const float dzh = (float)dz, dzl = (float)(dz - (double)dzh);
        tc::lstep_adj_ff_kernel<<<(unsigned)((total + 255) / 256), 256, 0, q->st>>>(
            (const float2*)fb, (float2*)sb, (float2*)sbl, (float2*)b1b, q->nr, q->nt, dzh, dzl, q->cinv, q->theta,
            q->kiff, q->inv1ps);
    } else {
        tc::lstep_adj_kernel<<<(unsigned)((total + 255) / 256), 256, 0, q->st>>>(
            (const float2*)fb, (float2*)sb, (float2*)b1b, q->nt, total, (float)dz, q->kr, q->ki, q->ho, q->kt2, q->kmax);
    }
    (*nlaunch)++;
    return cudaGetLastError();
}

bool qdht_tc_lstep_adj_ff(const QdhtTc* q) {
    return q && q->wide && q->cinv && q->theta && q->kiff && q->inv1ps;
}

bool qdht_tc_has_compact(const QdhtTc* q) { return q && q->wide && q->sc != nullptr; }

cudaError_t qdht_tc_spec_copy(QdhtTc* q, float* S, int to_compact, long long* nlaunch) {
    if (!qdht_tc_has_compact(q)) return cudaErrorInvalidValue;
    const size_t tot = (size_t)q->nr * (q->nc_act / 2);
    tc::qdht_spec_copy_kernel<<<(unsigned)std::min<size_t>((tot + 255) / 256, (size_t)q->sms * 16), 256, 0, q->st>>>(
        S, q->sc, q->sl, q->nr, 2 * q->nt, q->nc_act, q->cmap, to_compact ? 1 : -1);
    (*nlaunch)++;
    return cudaGetLastError();
}

cudaError_t qdht_tc_spec_ff(QdhtTc* q, double* X, const int* perm, int take, long long* nlaunch) {
    if (!qdht_tc_has_compact(q)) return cudaErrorInvalidValue;
    const size_t tot = (size_t)q->nr * (q->nc_act / 2);
    tc::qdht_spec_ff_kernel<<<(unsigned)std::min<size_t>((tot + 255) / 256, (size_t)q->sms * 16), 256, 0, q->st>>>(
        reinterpret_cast<double2*>(X), q->sc, q->sl, q->nr, q->nt, q->nc_act, q->cmap, perm, take ? 1 : -1);
    (*nlaunch)++;
    return cudaGetLastError();
}

cudaError_t qdht_tc_spec_dev(QdhtTc* q, float* S, float* lo, int take, long long* nlaunch) {
    if (!qdht_tc_has_compact(q)) return cudaErrorInvalidValue;
    const size_t tot = take ? (size_t)q->nr * (q->nc_act / 2) : (size_t)q->nr * q->nt;
    tc::qdht_spec_dev_kernel<<<(unsigned)std::min<size_t>((tot + 255) / 256, (size_t)q->sms * 16), 256, 0, q->st>>>(
        S, lo, q->sc, q->sl, q->nr, 2 * q->nt, q->nc_act, q->cmap, q->cinv, take ? 1 : -1);
    (*nlaunch)++;
    return cudaGetLastError();
}

void qdht_tc_spec_pairs(QdhtTc* q, float** sc, float** sl, int* nc) {
    const bool has = qdht_tc_has_compact(q);
    if (sc) *sc = has ? q->sc : nullptr;
    if (sl) *sl = has ? q->sl : nullptr;
    if (nc) *nc = has ? q->nc_act : 0;
}

const float* qdht_tc_compact_y(QdhtTc* q, int* nc, const int** cmap) {
    if (!q || !q->wide || !q->yc) return nullptr;
    if (nc) *nc = q->nc_act;
    if (cmap) *cmap = q->cmap;
    return q->yc;
}

cudaError_t qdht_tc_expand(QdhtTc* q, float* Y, long long* nlaunch, const int* run) {
    if (!q || !q->yc || q->nc_act == 0) return cudaErrorInvalidValue;
    const size_t tot = (size_t)q->nr * q->nt / 2;
    tc::qdht_expand_kernel<<<(unsigned)std::min<size_t>((tot + 1023) / 1024, (size_t)q->sms * 8), 256, 0, q->st>>>(
        q->yc, Y, q->nr, q->nt, q->nc_act, q->cinv, run);
    (*nlaunch)++;
    return cudaGetLastError();
}

float* qdht_tc_compact_x(QdhtTc* q, const int** cinv, int* nc) {
    if (!q || !q->wide || !q->xc) return nullptr;
    if (cinv) *cinv = q->cinv;
    if (nc) *nc = q->nc_act;
    return q->xc;
}

cudaError_t qdht_tc_wait_probe(QdhtTc* q, double limit_s, long long* nlaunch) {
    tc::wait_probe_kernel<<<1, 32, 0, q->st>>>(q->err, (unsigned long long)(limit_s * 1e9));
    (*nlaunch)++;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(q->st);
    return e;
}

int qdht_tc_check(QdhtTc* q, std::string* msg) {
    unsigned e[2] = {0, 0};
    if (cudaMemcpy(e, q->err, 8, cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
    if (e[0] & GS_ERRBIT_BOUNDS) {
        if (msg) *msg = GS_BOUNDS_MSG;
        cudaMemset(q->err, 0, 8);
        return 1;
    }
    if (e[0]) {
        if (msg)
            *msg = "tensor-core QDHT wait expired (codes " + std::to_string(e[0]) + ", first: code " +
                   std::to_string(e[1] & 0xff) + " k-block " + std::to_string((e[1] >> 8) & 0xfff) + " warp " +
                   std::to_string(e[1] >> 20) + ")";
        cudaMemset(q->err, 0, 8);
        return 1;
    }
    return 0;
}

void qdht_tc_destroy(QdhtTc* q) {
    if (!q) return;
    void* ptrs[] = {q->hh, q->hl, q->kr, q->ki, q->ho, q->kt2, q->kmax, q->err, q->xhT, q->xlT, q->hh16, q->hl16, q->hs, q->xs,
                    q->cmap, q->zpos, q->cinv, q->yc, q->xc, q->sc, q->sl, q->theta, q->kiff, q->inv1ps};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete q;
}

}  // namespace gs
