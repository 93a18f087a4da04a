// Taylor propagation of the three-section mixed form (AFQ_PREC_MIXED_FAST)
// on the tensor cores (prop/chol_afqmc_ops.py:173-183, prop/utils.py:20-31):
//   W1 = W + (E - I) W;   out = W1 + sum_{k=1..K} (i sqrt_dt V)^k / k! W1;
//   W' = out + (E - I) out
// with E = exp(-dt h1 / 2) and V = sum_g x_g L_g of the walker.
//
// Each complex product is one real GEMM per 128-row tile of the walker:
//   [Yr | Yi] = [Vr | Vi] . B,   B = [[Tr, Ti], [-Ti, Tr]]   (K = 2n)
// on tcgen05.mma kind::f16 (M = 128, K = 16).  Operands are two-piece bf16
// splits, x = hi + mid, and each K step issues A_hi . [B_hi; B_mid] (N = 128,
// the hi.hi and hi.mid products land in separate accumulator columns and A is
// read once) and A_mid . B_hi (N = 64, into the hi.mid columns): hi.hi +
// hi.mid + mid.hi, ~2^-17 relative, the precision of the three-section
// GEMMs.  Keeping hi.hi in an accumulator of its own bounds the tensor
// cores' truncating fp32 accumulation to one add per K step of the dominant
// sum.  The E - I products
// use A = [(E - I) | 0], i.e. only the top half of B's K range.
//
// A (V of the walker, or E - I: hi and mid tiles of 128 rows x 64 K) streams
// by TMA through a three-stage ring.  B, the current Taylor term, lives in
// shared memory in the 128-byte-swizzled K-major layout the MMA reads, and is
// rewritten by the epilogue warps after each product: rows c < o hold
// [Tr; -Ti] of column c, rows 32 + c hold [Ti; Tr] (so output column c is Yr
// and 32 + c is Yi), rows 64.. the same for the mid piece.  The top half of
// B's K range holds rows 0..n-1 at K = i, the bottom half at K = 16 S + i
// (S = ceil(n / 16) K steps per half), so no K step straddles the two halves.
// Tensor memory (512 columns): per 128-row tile 128 accumulator columns
// (hi.hi | hi.mid + mid.hi, summed by the epilogue with a round-to-nearest
// add), then per tile 64 columns of the running walker update and 64 of the
// fp32 copy of the walker's rows.
//
// The walker update W' - W = (E - I) W + sum_k T_k + (E - I) out is summed in
// fp32 by the epilogue thread that owns the row (in tensor memory, next to
// an fp32 copy of the row for the operand sums), and added to the binary64
// walker once: per entry the binary64 pipe converts W once and the update
// once and adds once.
//
// Warps: 0 TMA producer, 1 MMA issuer and tensor-memory owner, 2-9 epilogue
// (warp w reads lanes 32 (w % 4).. of the accumulator of tile (w - 2) / 4,
// as tcgen05.ld allows).  Persistent over the chunk's walkers, one walker at
// a time per CTA.  Every mbarrier wait is bounded; on a timeout the CTA
// raises *err and unwinds (the producer waits for its copies in flight, the
// MMA thread for its MMAs, and the tensor memory is freed).
#include "afq_internal.cuh"
#include "tc_common.cuh"

namespace afq {
namespace tc {

constexpr int TT_THREADS = 320;
constexpr int TT_N = 64;                 // output columns: 32 Yr, 32 Yi (nocc <= 32)
constexpr int TT_STG = 3;                // A stages
constexpr int TT_TILE = 128 * 64 * 2;    // one 128 x 64 bf16 tile, 16 KB
constexpr int TT_STAGE = 2 * TT_TILE;    // hi + mid
constexpr int TT_BBLK = 2 * TT_N * 128;  // one 64-wide K block of B (hi rows 0-63, mid rows 64-127), 16 KB
constexpr int TT_MAXKBB = 8;             // B K blocks for norb <= 256
constexpr int TT_TCOLS = 2 * TT_N;       // accumulator columns per tile: hi.hi | hi.mid + mid.hi
constexpr int TT_SCOL = 2 * TT_TCOLS;    // running update: tile t at TT_SCOL + t TT_N (Re 32, Im 32)
constexpr int TT_FCOL = TT_SCOL + 2 * TT_N;  // fp32 copy of the rows, same layout
constexpr int TT_SMEM = TT_MAXKBB * TT_BBLK + TT_STG * TT_STAGE + 1024 + 256;
constexpr uint32_t TT_IDESC128 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(128 >> 3) << 17) |
                                 ((uint32_t)(128 >> 4) << 24);
constexpr uint32_t TT_IDESC64 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(64 >> 3) << 17) |
                                ((uint32_t)(128 >> 4) << 24);
static_assert(TT_SMEM <= 227 * 1024, "tensor-core Trotter shared memory");

// B is K-major with the 128-byte swizzle (16-byte chunk index XOR row % 8
// within each 8-row, 1024-byte atom): element (row r, K index k) sits at byte
//   (k >> 6) TT_BBLK + (r >> 3) 1024 + (r & 7) 128 + ((((k & 63) >> 3) ^ (r & 7)) << 4) + 2 (k & 7)
// = kb(k) + rb(r) + (kx(k) ^ ((r & 7) << 4)) with the K parts
// kb(k) = (k >> 6) TT_BBLK + 2 (k & 7), kx(k) = ((k & 63) >> 3) << 4 fixed
// per thread (its rows k = i and k = kb0 + i) and rb(r) = (r >> 3) 1024 +
// (r & 7) 128 a constant once the column loops are unrolled.
struct TTRow {
    uint32_t kb0, kx0;  // k = i: the top half of B's K range
    uint32_t kb1, kx1;  // k = kb0 + i: the bottom half
};
__device__ __forceinline__ TTRow tt_row(int i, int kbot) {
    const int k1 = kbot + i;
    return TTRow{(uint32_t)((i >> 6) * TT_BBLK + ((i & 7) << 1)), (uint32_t)(((i & 63) >> 3) << 4),
                 (uint32_t)((k1 >> 6) * TT_BBLK + ((k1 & 7) << 1)), (uint32_t)(((k1 & 63) >> 3) << 4)};
}
__device__ __forceinline__ void tt_st16(uint8_t* p, uint32_t v) { *(uint16_t*)p = (uint16_t)v; }

// B <- the embedding of T(i, c) = t, c < o, for this thread's row: rows c
// and 32 + c of the hi piece (64 + ... of the mid piece) get [Tr; -Ti] and
// [Ti; Tr] over the two K halves.  Re and Im are rounded together; -Ti's
// pieces are Ti's with the sign bit flipped (round-to-nearest is odd).
__device__ __forceinline__ void tt_write_b(uint8_t* b, const TTRow& q, int c, float2 t) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(t.x, t.y);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 m = __floats2bfloat162_rn(t.x - hf.x, t.y - hf.y);
    const uint32_t hv = *(const uint32_t*)&h, mv = *(const uint32_t*)&m;
    const uint32_t sw = (uint32_t)((c & 7) << 4);
    uint8_t* p0 = b + q.kb0 + (q.kx0 ^ sw);
    uint8_t* p1 = b + q.kb1 + (q.kx1 ^ sw);
    const int rc = (c >> 3) * 1024 + (c & 7) * 128;  // rb(c); rb(32 + c) = rc + 4096, +8192 for the mid piece
    tt_st16(p0 + rc, hv);                            // (c, i) = Tr
    tt_st16(p0 + rc + 8192, mv);
    tt_st16(p1 + rc, (hv >> 16) ^ 0x8000u);          // (c, kb0 + i) = -Ti
    tt_st16(p1 + rc + 8192, (mv >> 16) ^ 0x8000u);
    tt_st16(p0 + rc + 4096, hv >> 16);               // (32 + c, i) = Ti
    tt_st16(p0 + rc + 4096 + 8192, mv >> 16);
    tt_st16(p1 + rc + 4096, hv);                     // (32 + c, kb0 + i) = Tr
    tt_st16(p1 + rc + 4096 + 8192, mv);
}
static_assert(TT_N == 64, "tt_write_b: row offsets of 32 + c (4096) and of the mid piece (8192)");

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

#define TT_R8(i)                                                                                               \
    "=r"(r[i]), "=r"(r[i + 1]), "=r"(r[i + 2]), "=r"(r[i + 3]), "=r"(r[i + 4]), "=r"(r[i + 5]), "=r"(r[i + 6]), \
        "=r"(r[i + 7])
// Two 8-column loads (one wait) and stores (then wait for the stores).
__device__ __forceinline__ void tmem_ld8x2(uint32_t a0, uint32_t a1, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%16];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8, %9, %10, %11, %12, %13, %14, %15}, [%17];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : TT_R8(0), TT_R8(8)
        : "r"(a0), "r"(a1)
        : "memory");
}
#undef TT_R8
// Four 8-column loads, one wait.
#define TT_R8(i)                                                                                               \
    "=r"(r[i]), "=r"(r[i + 1]), "=r"(r[i + 2]), "=r"(r[i + 3]), "=r"(r[i + 4]), "=r"(r[i + 5]), "=r"(r[i + 6]), \
        "=r"(r[i + 7])
__device__ __forceinline__ void tmem_ld8x4(uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%32];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8, %9, %10, %11, %12, %13, %14, %15}, [%33];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16, %17, %18, %19, %20, %21, %22, %23}, [%34];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%24, %25, %26, %27, %28, %29, %30, %31}, [%35];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : TT_R8(0), TT_R8(8), TT_R8(16), TT_R8(24)
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3)
        : "memory");
}
#undef TT_R8
__device__ __forceinline__ void tmem_st8x2(uint32_t a0, uint32_t a1, const uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%2, %3, %4, %5, %6, %7, %8, %9};\n\t"
        "tcgen05.st.sync.aligned.32x32b.x8.b32 [%1], {%10, %11, %12, %13, %14, %15, %16, %17};\n\t"
        "tcgen05.wait::st.sync.aligned;" ::"r"(a0),
        "r"(a1), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),
        "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
        : "memory");
}

__global__ void __launch_bounds__(TT_THREADS, 1)
    k_trotter_tc(const __grid_constant__ CUtensorMap mVh, const __grid_constant__ CUtensorMap mVm,
                 const __grid_constant__ CUtensorMap mEh, const __grid_constant__ CUtensorMap mEm, int wc, int n,
                 int o, int n_terms, float sqrt_dt, const double2* win, double2* wout, int* __restrict__ err) {
    extern __shared__ uint8_t tt_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)tt_raw + 1023) & ~(uintptr_t)1023);
    const int S = (n + 15) >> 4;             // K steps per half
    const int KBB = (2 * S + 3) >> 2;        // B K blocks
    const int kbh = (n + 63) >> 6;           // A K blocks per half
    const int MT = (n + 127) >> 7;           // 128-row tiles
    const int R = n_terms + 2;               // products per walker
    uint8_t* sB = smem;
    uint8_t* sA = smem + TT_MAXKBB * TT_BBLK;
    uint64_t* bars = (uint64_t*)(sA + TT_STG * TT_STAGE);
    uint32_t* tmem_slot = (uint32_t*)(bars + 2 * TT_STG + 3);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + TT_STG);
    const uint32_t dfull = smem_u32(bars + 2 * TT_STG), bready = smem_u32(bars + 2 * TT_STG + 1);
    const uint32_t drain = smem_u32(bars + 2 * TT_STG + 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TT_STG; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        mbar_init(dfull, 1);
        mbar_init(bready, TT_THREADS - 64);
        mbar_init(drain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&mVh) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&mVm) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&mEh) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&mEm) : "memory");
            int stage = 0;
            uint32_t phase = 0;
            int issued[TT_STG];
            uint32_t issued_par[TT_STG];
            for (int s = 0; s < TT_STG; ++s) issued[s] = 0;
            bool ok = true;
            for (int w = blockIdx.x; ok && w < wc; w += gridDim.x) {
                for (int r = 0; ok && r < R; ++r) {
                    const bool e = (r == 0 || r == R - 1);
                    for (int mt = 0; ok && mt < MT; ++mt)
                        for (int hf = 0; ok && hf < (e ? 1 : 2); ++hf)
                            for (int kb = 0; kb < kbh; ++kb) {
                                if (!mbar_wait(empty0 + 8 * stage, phase ^ 1, abort_flag)) { ok = false; break; }
                                issued[stage] = 0;
                                const uint32_t full = full0 + 8 * stage;
                                const uint32_t dh = smem_u32(sA + stage * TT_STAGE), dm = dh + TT_TILE;
                                mbar_expect_tx(full, TT_STAGE);
                                if (e) {
                                    tma_load_2d(dh, &mEh, kb * 64, mt * 128, full);
                                    tma_load_2d(dm, &mEm, kb * 64, mt * 128, full);
                                } else {  // rows past n of the last tile read as zero
                                    tma_load_3d(dh, &mVh, kb * 64, mt * 128, hf * wc + w, full);
                                    tma_load_3d(dm, &mVm, kb * 64, mt * 128, hf * wc + w, full);
                                }
                                issued[stage] = 1;
                                issued_par[stage] = phase;
                                if (++stage == TT_STG) { stage = 0; phase ^= 1; }
                            }
                }
            }
            if (!ok) {
                atomicExch(err, 1);
                *abort_flag = 1;
            }
            // every copy this thread issued lands before the CTA exits (after an
            // abort elsewhere in the CTA nobody else waits for them)
            for (int s = 0; s < TT_STG; ++s)
                if (issued[s]) mbar_wait(full0 + 8 * s, issued_par[s], nullptr);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0, rr = 0;
            bool ok = true;
            const uint32_t b0 = smem_u32(sB);
            for (int w = blockIdx.x; ok && w < wc; w += gridDim.x) {
                for (int r = 0; ok && r < R; ++r, ++rr) {
                    const bool e = (r == 0 || r == R - 1);
                    if (!mbar_wait(bready, rr & 1, abort_flag)) { ok = false; break; }
                    tc_fence_after();
                    for (int mt = 0; ok && mt < MT; ++mt) {
                        uint32_t acc = 0;
                        const uint32_t d = tmem + mt * TT_TCOLS;
                        for (int hf = 0; ok && hf < (e ? 1 : 2); ++hf)
                            for (int kb = 0; kb < kbh; ++kb) {
                                if (!mbar_wait(full0 + 8 * stage, phase, abort_flag)) { ok = false; break; }
                                tc_fence_after();
                                const uint32_t ah = smem_u32(sA + stage * TT_STAGE), am = ah + TT_TILE;
                                for (int s = 0; s < 4; ++s) {
                                    const int t = kb * 4 + s;
                                    if (t >= S) break;
                                    const int g = hf * S + t;  // K step within B
                                    const uint64_t db = desc_k128(b0 + (uint32_t)((g >> 2) * TT_BBLK + (g & 3) * 32));
                                    // hi . [hi; mid] -> columns 0-127, mid . hi added to columns 64-127
                                    umma_bf16_i(d, desc_k128(ah + 32 * s), db, TT_IDESC128, acc);
                                    umma_bf16_i(d + TT_N, desc_k128(am + 32 * s), db, TT_IDESC64, 1);
                                    acc = 1;
                                }
                                umma_commit(empty0 + 8 * stage);
                                if (++stage == TT_STG) { stage = 0; phase ^= 1; }
                            }
                    }
                    if (ok) umma_commit(dfull);
                }
            }
            if (!ok) {
                atomicExch(err, 1);
                *abort_flag = 1;
            }
            // every MMA issued finishes before the tensor memory is freed, also
            // when the epilogue gave up waiting for it
            umma_commit(drain);
            mbar_wait(drain, 0, nullptr);
        }
    } else {
        const int q = warp & 3, mt = (warp - 2) >> 2;
        const int i = mt * 128 + q * 32 + lane;
        const bool row = i < n;
        const int kb0 = 16 * S;  // K index of the bottom half
        const TTRow trow = tt_row(i, kb0);
        // B starts (and its padding stays) zero
        for (int e = threadIdx.x - 64; e < KBB * TT_BBLK / 16; e += TT_THREADS - 64)
            ((uint4*)sB)[e] = make_uint4(0, 0, 0, 0);
        asm volatile("bar.sync 1, %0;" ::"r"(TT_THREADS - 64) : "memory");
        uint32_t rr = 0;
        bool ok = true;
        for (int w = blockIdx.x; ok && w < wc; w += gridDim.x) {
            double2* Wr = wout + ((size_t)w * n + i) * o;  // this thread's row
            const double2* Wi = win + ((size_t)w * n + i) * o;
            const uint32_t lq = (uint32_t)(q * 32) << 16;
            const uint32_t ta = tmem + mt * TT_TCOLS + lq;            // accumulator
            const uint32_t ts = tmem + TT_SCOL + mt * TT_N + lq;      // running update
            const uint32_t tf = tmem + TT_FCOL + mt * TT_N + lq;      // fp32 copy of the row
            // the row's loads go out 16 at a time ahead of the shared-memory
            // writes (which the compiler may not move loads across)
#pragma unroll
            for (int hb = 0; hb < 32; hb += 16) {
                float2 f[16];
#pragma unroll
                for (int u = 0; u < 16; ++u) {
                    const int c = hb + u;
                    const double2 v = (row && c < o) ? Wi[c] : make_double2(0.0, 0.0);
                    f[u] = make_float2((float)v.x, (float)v.y);
                }
#pragma unroll
                for (int cb = 0; cb < 16; cb += 8) {
                    uint32_t fv[16];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int c = hb + cb + u;
                        if (row && c < o) tt_write_b(sB, trow, c, f[cb + u]);
                        fv[u] = __float_as_uint(f[cb + u].x);
                        fv[8 + u] = __float_as_uint(f[cb + u].y);
                    }
                    tmem_st8x2(tf + hb + cb, tf + 32 + hb + cb, fv);
                }
            }
            tc_fence_before();
            fence_proxy_async();
            mbar_arrive(bready);
            for (int r = 0; r < R; ++r, ++rr) {
                if (row && r == R - 1) {  // rows read after the last product: this walker's, the next one's
                    for (int b = 0; b < o * 16; b += 128) prefetch_l2((const char*)Wi + b);
                    if (w + (int)gridDim.x < wc)
                        for (int b = 0; b < o * 16; b += 128)
                            prefetch_l2((const char*)(Wi + (size_t)gridDim.x * n * o) + b);
                }
                if (!mbar_wait_inl(dfull, rr & 1, abort_flag)) {
                    atomicExch(err, 1);
                    *abort_flag = 1;
                    ok = false;
                    break;
                }
                tc_fence_after();
                const float sk = sqrt_dt / (float)(r > 0 ? r : 1);
                if (r == R - 1) {  // W' = W + (S + (E - I) out): the one binary64 update
#pragma unroll
                    for (int cb = 0; cb < 32; cb += 8) {
                        double2 wv[8];  // loaded ahead of the stores (Wi and Wr alias)
#pragma unroll
                        for (int u = 0; u < 8; ++u)
                            wv[u] = (row && cb + u < o) ? Wi[cb + u] : make_double2(0.0, 0.0);
                        uint32_t y[32], sv[16];
                        tmem_ld8x4(ta + cb, ta + TT_N + cb, ta + 32 + cb, ta + TT_N + 32 + cb, y);
                        tmem_ld8x2(ts + cb, ts + 32 + cb, sv);
                        if (row) {
#pragma unroll
                            for (int u = 0; u < 8; ++u) {
                                const int c = cb + u;
                                const float yr = __uint_as_float(y[u]) + __uint_as_float(y[8 + u]);
                                const float yi = __uint_as_float(y[16 + u]) + __uint_as_float(y[24 + u]);
                                const float sr = __uint_as_float(sv[u]), si = __uint_as_float(sv[8 + u]);
                                if (c < o) Wr[c] = make_double2(wv[u].x + (double)(sr + yr), wv[u].y + (double)(si + yi));
                            }
                        }
                    }
                    tc_fence_before();
                    continue;
                }
#pragma unroll
                for (int cb = 0; cb < 32; cb += 8) {
                    // Y columns cb..cb+7 of Yr and Yi (hi.hi + corrections); S and the row copy
                    uint32_t y[32], sf[32];
                    tmem_ld8x4(ta + cb, ta + TT_N + cb, ta + 32 + cb, ta + TT_N + 32 + cb, y);
                    tmem_ld8x4(ts + cb, ts + 32 + cb, tf + cb, tf + 32 + cb, sf);
                    uint32_t sv[16];
                    if (row) {
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            const int c = cb + u;
                            const float yr = __uint_as_float(y[u]) + __uint_as_float(y[8 + u]);
                            const float yi = __uint_as_float(y[16 + u]) + __uint_as_float(y[24 + u]);
                            float sr = __uint_as_float(sf[u]), si = __uint_as_float(sf[8 + u]);
                            const float fr = __uint_as_float(sf[16 + u]), fi = __uint_as_float(sf[24 + u]);
                            if (c < o) {
                                if (r == 0) {  // W1 = W + (E - I) W
                                    sr = yr;
                                    si = yi;
                                    tt_write_b(sB, trow, c, make_float2(fr + yr, fi + yi));
                                } else {  // T_r = (i sqrt_dt / r) Y
                                    const float2 t = make_float2(-sk * yi, sk * yr);
                                    sr += t.x;
                                    si += t.y;
                                    if (r < n_terms) tt_write_b(sB, trow, c, t);
                                    else tt_write_b(sB, trow, c, make_float2(fr + sr, fi + si));  // out = W1 + sum T_k
                                }
                            }
                            sv[u] = __float_as_uint(sr);
                            sv[8 + u] = __float_as_uint(si);
                        }
                    }
                    tmem_st8x2(ts + cb, ts + 32 + cb, sv);
                }
                tc_fence_before();
                fence_proxy_async();
                mbar_arrive(bready);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
    }
}

}  // namespace tc

bool trotter_tc_supported(int n, int o) { return n % 8 == 0 && n <= 256 && o <= 32; }

int launch_trotter_tc(int wc, int n, int o, int n_terms, double sqrt_dt, const __nv_bfloat16* eh,
                      const __nv_bfloat16* em, const __nv_bfloat16* vh, const __nv_bfloat16* vm, const double2* win,
                      double2* wout, int* err, cudaStream_t s) {
    using namespace tc;
    if (wc <= 0) return AFQ_OK;
    if (!trotter_tc_supported(n, o))
        return fail(AFQ_E_UNSUPPORTED, "tensor-core Trotter: norb=%d nocc=%d (needs norb %% 8 == 0, <= 256, nocc <= 32)",
                    n, o);
    static DeviceOnce smem_once;
    AFQ_TRY(get_encode());
    int nsm = 0;
    AFQ_TRY(device_sms(&nsm));
    AFQ_TRY(raise_smem_once(smem_once, k_trotter_tc, TT_SMEM));
    CUtensorMap mvh, mvm, meh, mem;
    AFQ_TRY(make_map3(&mvh, vh, 2LL * wc, n, n, n, 128));
    AFQ_TRY(make_map3(&mvm, vm, 2LL * wc, n, n, n, 128));
    AFQ_TRY(make_map(&meh, eh, n, n, n, 128));
    AFQ_TRY(make_map(&mem, em, n, n, n, 128));
    const int grid = wc < nsm ? wc : nsm;
    k_trotter_tc<<<grid, TT_THREADS, TT_SMEM, s>>>(mvh, mvm, meh, mem, wc, n, o, n_terms, (float)sqrt_dt, win, wout,
                                                 err);
    AFQ_LAUNCHED("k_trotter_tc");
    return AFQ_OK;
}

// (E - I) as bf16 hi and mid pieces (n x n), the A operand of the E products.
__global__ void k_e_minus_i_split(int n, const double* __restrict__ E, __nv_bfloat16* __restrict__ eh,
                                  __nv_bfloat16* __restrict__ em) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * n; e += gridDim.x * blockDim.x) {
        const float v = (float)(E[e] - ((e / n) == (e % n) ? 1.0 : 0.0));
        const __nv_bfloat16 h = __float2bfloat16(v);
        eh[e] = h;
        em[e] = __float2bfloat16(v - __bfloat162float(h));
    }
}

int launch_e_minus_i_split(int n, const double* E, __nv_bfloat16* eh, __nv_bfloat16* em, cudaStream_t s) {
    k_e_minus_i_split<<<(n * n + 255) / 256, 256, 0, s>>>(n, E, eh, em);
    AFQ_LAUNCHED("k_e_minus_i_split");
    return AFQ_OK;
}

}  // namespace afq
