// Taylor propagation of the three-section mixed form (AFQ_PREC_MIXED_FAST)
// on the tensor cores (prop/chol_afqmc_ops.py:173-183, prop/utils.py:20-31):
//   W1 = W + (E - I) W;   out = W1 + sum_{k=1..K} (i sqrt_dt V)^k / k! W1;
//   W' = out + (E - I) out
// with E = exp(-dt h1 / 2) and V = sum_g x_g L_g of the walker.
//
// Each complex product Y = V T (T the current n x o term) is one real GEMM
// in transposed form, D = A B^T on tcgen05.mma kind::f16 (M = 128, K = 16):
//   B = V itself, row j over K = [Vr[j, :] | Vi[j, :]] (two K halves of
//       N = n rounded up to 16 each), streamed by TMA from the V-build's
//       output; N = the orbital rows j (one MMA covers all of them, N <= 256);
//   A = the term's embedding, one row per (orbital c, piece p, part q), held
//       in tensor memory: row (c, p, Re) = piece p of [Tr[:, c] | -Ti[:, c]],
//       row (c, p, Im) = piece p of [Ti[:, c] | Tr[:, c]], so that
//       D[(c, p, Re), j] = (V T_p)r[j, c] and D[(c, p, Im), j] = (V T_p)i[j, c].
// Pieces are two-piece bf16 splits x = hi + mid of both operands; each K step
// issues A.B_hi and A.B_mid into the same accumulator, so the sum over the
// two A rows of a (c, q) pair is (T_hi + T_mid)(V_hi + V_mid), ~2^-17
// relative, the precision of the three-section GEMMs.  The E - I products use
// B = (E - I) and the top K half only.  Tensor memory (512 columns): the
// accumulator in columns [0, N), the A operand in [256, 256 + N) (two bf16 a
// column, K index k in column k / 2, even k in the low half).
//
// With the term as the tensor-memory operand the MMA reads only B from
// shared memory, and N = n per instruction instead of the 2 o columns of a
// term-as-B layout: a 128 x 208 x 16 MMA issues in the time of a 128 x 64 x 16
// one from shared memory.
//
// The running sum U = W + (E - I) W + sum_k T_k (= out after the last V
// product) is kept in fp32 registers; W' = W + ((U - W32) + (E - I) out) is
// formed with one binary64 add per entry, W32 being W cut to fp32 by integer
// operations (d2f_trunc: the same bits in the first and the last use).  Lane (c, p, q)
// of the accumulator belongs to the epilogue thread that holds TMEM lane
// 4c + 2p + q; the four lanes of an orbital c are in one warp and exchange
// the piece sums and the Re/Im parts by shuffles.  U(j, c, q) is held by
// lane (c, j & 1, q).  The walker is read and written by the epilogue lanes
// themselves: lane (c, p, q) loads part q of W[j][c] (a warp reads 128
// contiguous bytes of a row j), takes the other part by the xor-1 shuffle,
// and at the end stores its own entries.
//
// Warps: 0 TMA producer, 1 MMA issuer and tensor-memory owner, 2-17 epilogue
// (warp w reads lanes 32 (w % 4).. of tensor memory, as tcgen05.ld allows;
// the four warps of a lane quarter take a quarter of the columns each).
// Persistent over the chunk's walkers, one walker at a time per CTA.  Every
// mbarrier wait is bounded; on a timeout the CTA raises *err and unwinds (the
// producer waits for its copies in flight, the MMA thread for its MMAs, and
// the tensor memory is freed).
#include "afq_internal.cuh"
#include "tc_common.cuh"

namespace afq {
namespace tc {

constexpr int TT_THREADS = 576;          // 18 warps
constexpr int TT_EPI = TT_THREADS - 64;  // epilogue threads
constexpr uint32_t TT_ACOL = 256;        // tensor-memory column of the A operand
constexpr int TT_SMEM_MAX = 227 * 1024;

__host__ __device__ constexpr uint32_t tt_idesc(int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

struct TTGeo {
    int N;     // n rounded up to 16: the MMA's N, the B tiles' rows, the K extent of each half
    int S;     // K steps of 16 per half
    int kbh;   // 64-wide K blocks per half (the last may hold fewer than four steps)
    int stg;   // B ring stages (hi + mid tiles of N rows x 64 K each)
    int smem;  // dynamic shared memory
};

static TTGeo tt_geo(int n, int o) {
    TTGeo g;
    g.N = (n + 15) / 16 * 16;
    g.S = g.N / 16;
    g.kbh = (g.N + 63) / 64;
    const int stage = 2 * g.N * 128;
    g.stg = (TT_SMEM_MAX - 1024 - 256) / stage;
    if (g.stg > 4) g.stg = 4;
    g.smem = 1024 + g.stg * stage + 256;
    return g;
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

__device__ __forceinline__ void umma_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void tmem_ld4(uint32_t a, uint32_t (&r)[4]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
        : "r"(a)
        : "memory");
}
__device__ __forceinline__ void tmem_st2(uint32_t a, uint32_t v0, uint32_t v1) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1, %2};" ::"r"(a), "r"(v0), "r"(v1) : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Piece p of (a, b) as a bf16 pair (a in the low half): p = 0 the
// round-to-nearest bf16 of each, p = 1 the bf16 of the remainder, as the
// bf16 of fma(npf, h, (a, b)) with npf = -p (the remainder is exact; for p =
// 0 the fma returns a and b themselves).
__device__ __forceinline__ uint32_t tt_piece2(float a, float b, float2 npf) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    const float2 r = __ffma2_rn(npf, __bfloat1622float2(h), make_float2(a, b));
    const __nv_bfloat162 x = __floats2bfloat162_rn(r.x, r.y);
    return *(const uint32_t*)&x;
}

// 16 and 8 consecutive fp32 columns of this warp's lanes; the wait is part
// of the same statement, so no use of the registers can move above it.
#define TT_O8(i)                                                                                               \
    "=r"(v[i]), "=r"(v[i + 1]), "=r"(v[i + 2]), "=r"(v[i + 3]), "=r"(v[i + 4]), "=r"(v[i + 5]), "=r"(v[i + 6]), \
        "=r"(v[i + 7])
__device__ __forceinline__ void tmem_ld16_wait(uint32_t a, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : TT_O8(0), TT_O8(8)
        : "r"(a)
        : "memory");
}
__device__ __forceinline__ void tmem_ld8_wait(uint32_t a, uint32_t (&v)[8]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : TT_O8(0)
        : "r"(a)
        : "memory");
}
#undef TT_O8

// MAXCH: the largest count of 4-column chunks an epilogue thread takes
// (N / 16; the instantiations cover N <= 64, 128, 208 and 256).
template <int MAXCH>
__global__ void __launch_bounds__(TT_THREADS, 1)
    k_trotter_tc(const __grid_constant__ CUtensorMap mVh, const __grid_constant__ CUtensorMap mVm,
                 const __grid_constant__ CUtensorMap mEh, const __grid_constant__ CUtensorMap mEm, int wc, int n,
                 int o, int n_terms, float sqrt_dt, TTGeo g, const double2* win, double2* wout,
                 int* __restrict__ err) {
    extern __shared__ uint8_t tt_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)tt_raw + 1023) & ~(uintptr_t)1023);
    const int N = g.N, S = g.S, kbh = g.kbh, STG = g.stg;
    const uint32_t TILE = (uint32_t)N * 128u, STAGE = 2u * TILE;
    const int R = n_terms + 2;  // products per walker: E, n_terms V, E
    uint8_t* ring = smem;
    uint64_t* bars = (uint64_t*)(smem + (size_t)STG * STAGE);
    uint32_t* tmem_slot = (uint32_t*)(bars + 2 * STG + 3);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STG);
    const uint32_t dfull = smem_u32(bars + 2 * STG), bready = smem_u32(bars + 2 * STG + 1);
    const uint32_t drain = smem_u32(bars + 2 * STG + 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STG; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        mbar_init(dfull, 1);
        mbar_init(bready, TT_EPI);
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
            int issued[4] = {0, 0, 0, 0};
            uint32_t issued_par[4] = {0, 0, 0, 0};
            bool ok = true;
            for (int w = blockIdx.x; ok && w < wc; w += gridDim.x) {
                for (int r = 0; ok && r < R; ++r) {
                    const bool e = (r == 0 || r == R - 1);
                    for (int hf = 0; ok && hf < (e ? 1 : 2); ++hf)
                        for (int kb = 0; kb < kbh; ++kb) {
                            if (!mbar_wait(empty0 + 8 * stage, phase ^ 1, abort_flag)) { ok = false; break; }
                            issued[stage] = 0;
                            const uint32_t full = full0 + 8 * stage;
                            const uint32_t dh = smem_u32(ring + stage * STAGE), dm = dh + TILE;
                            mbar_expect_tx(full, STAGE);
                            if (e) {  // rows and columns past n read as zero
                                tma_load_2d(dh, &mEh, kb * 64, 0, full);
                                tma_load_2d(dm, &mEm, kb * 64, 0, full);
                            } else {
                                tma_load_3d(dh, &mVh, kb * 64, 0, hf * wc + w, full);
                                tma_load_3d(dm, &mVm, kb * 64, 0, hf * wc + w, full);
                            }
                            issued[stage] = 1;
                            issued_par[stage] = phase;
                            if (++stage == STG) { stage = 0; phase ^= 1; }
                        }
                }
            }
            if (!ok) {
                atomicExch(err, 1);
                *abort_flag = 1;
            }
            // every copy this thread issued lands before the CTA exits (after an
            // abort elsewhere in the CTA nobody else waits for them)
            for (int s = 0; s < STG; ++s)
                if (issued[s]) mbar_wait(full0 + 8 * s, issued_par[s], nullptr);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0, rr = 0;
            bool ok = true;
            const uint32_t idesc = tt_idesc(N);
            const uint32_t rb = smem_u32(ring);
            for (int w = blockIdx.x; ok && w < wc; w += gridDim.x) {
                for (int r = 0; ok && r < R; ++r, ++rr) {
                    const bool e = (r == 0 || r == R - 1);
                    if (!mbar_wait(bready, rr & 1, abort_flag)) { ok = false; break; }
                    tc_fence_after();
                    uint32_t acc = 0;
                    for (int hf = 0; ok && hf < (e ? 1 : 2); ++hf)
                        for (int kb = 0; kb < kbh; ++kb) {
                            if (!mbar_wait(full0 + 8 * stage, phase, abort_flag)) { ok = false; break; }
                            tc_fence_after();
                            const uint32_t bh = rb + stage * STAGE, bm = bh + TILE;
                            const int t0 = kb * 4, nt = S - t0 < 4 ? S - t0 : 4;
                            uint32_t a = tmem + TT_ACOL + 8u * (uint32_t)(hf * S + t0);
                            for (int s = 0; s < nt; ++s, a += 8) {
                                umma_ts(tmem, a, desc_k128(bh + 32 * s), idesc, acc);
                                umma_ts(tmem, a, desc_k128(bm + 32 * s), idesc, 1);
                                acc = 1;
                            }
                            umma_commit(empty0 + 8 * stage);
                            if (++stage == STG) { stage = 0; phase ^= 1; }
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
        const int ew = warp - 2, q4 = warp & 3, et = threadIdx.x - 64;
        const int L = 32 * q4 + lane, c = L >> 2, p = (L >> 1) & 1, q = L & 1;
        const bool valid = c < o;
        const float sg = q ? 1.f : -1.f;  // an A row's bottom half is sg times the other part
        // the bottom half's pieces are the partner lane's (L ^ 1) pieces of its own half, times sg: a shuffle
        // of the packed pair and a flip of both sign bits where sg < 0 (bf16 rounding is sign-symmetric)
        const uint32_t sflip = q ? 0u : 0x80008000u;
        const float2 npf = p ? make_float2(-1.f, -1.f) : make_float2(0.f, 0.f);
        const int NC = N >> 2, nch = NC >> 2, j0 = (ew >> 2) * NC;  // columns j0 .. j0 + NC - 1, nch chunks of 4
        const uint32_t lf = (uint32_t)(32 * q4) << 16;
        const uint32_t tD = tmem + lf + (uint32_t)j0;
        const uint32_t tA = tmem + lf + TT_ACOL + (uint32_t)(j0 >> 1), tAb = tA + (uint32_t)(N >> 1);
        uint32_t rr = 0;
        bool ok = true;
        // U in registers: U[2 k + i] = own part q of column j0 + 4 k + 2 i + p
        float U[2 * MAXCH];
#pragma unroll
        for (int m = 0; m < 2 * MAXCH; ++m) U[m] = 0.f;
        for (int w = blockIdx.x; ok && w < wc; w += gridDim.x) {
            // part q of W[j][c] at Wq[2 j o]: a warp reads 128 contiguous bytes a row
            const double* Wq = (const double*)(win + (size_t)w * n * o + c) + q;
            // A <- the split of W32 (own part loaded, the other by the xor-1 shuffle); U <- its own entries
#pragma unroll
            for (int kb = 0; kb < (MAXCH + 1) / 2; ++kb) {  // 8 columns, their loads in flight together
                if (2 * kb >= nch) break;
                double wv[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int j = j0 + 8 * kb + u;
                    wv[u] = (valid && 2 * kb + (u >> 2) < nch && j < n) ? Wq[(size_t)2 * j * o] : 0.0;
                }
#pragma unroll
                for (int cc = 0; cc < 2; ++cc) {
                    const int k = 2 * kb + cc;
                    if (k >= nch) break;
                    float t[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) t[u] = d2f_trunc(wv[4 * cc + u]);
                    U[2 * k] = p ? t[1] : t[0];
                    U[2 * k + 1] = p ? t[3] : t[2];
                    const uint32_t t0 = tt_piece2(t[0], t[1], npf), t1 = tt_piece2(t[2], t[3], npf);
                    tmem_st2(tA + 2 * k, t0, t1);
                    tmem_st2(tAb + 2 * k, __shfl_xor_sync(0xffffffffu, t0, 1) ^ sflip,
                             __shfl_xor_sync(0xffffffffu, t1, 1) ^ sflip);
                }
            }
            tmem_wait_st();
            tc_fence_before();
            mbar_arrive(bready);
            for (int r = 0; r < R; ++r, ++rr) {
                if (!mbar_wait_inl(dfull, rr & 1, abort_flag)) { ok = false; break; }
                tc_fence_after();
                if (r == R - 2) {  // this walker's rows (read again at the end) and the next walker's
                    const char* me = (const char*)(win + (size_t)w * n * o);
                    for (int b = et * 128; b < n * o * 16; b += TT_EPI * 128) prefetch_l2(me + b);
                    if (w + (int)gridDim.x < wc)
                        for (int b = et * 128; b < n * o * 16; b += TT_EPI * 128)
                            prefetch_l2(me + (size_t)gridDim.x * n * o * 16 + b);
                }
                const float sk = sqrt_dt / (float)(r > 0 ? r : 1), sgsk = sg * sk;
                const bool last = r == R - 1;
                const bool x_is_u = !last && (r == 0 || r == R - 2);  // the next operand is U (W1, or out)
                const bool term_is_y = r == 0 || last;                // the term added to U: Y, else T_r
                // the middle products (T_r, r = 1 .. R - 3): each lane keeps its partner's (L ^ 1) share of
                // U and forms the partner's part of T_r from its own Y, which needs no exchange of Y; U
                // is swapped into that arrangement before them and back before product R - 2
                const bool mid = !term_is_y && !x_is_u;
                if (R >= 4 && (r == 1 || r == R - 2)) {
#pragma unroll
                    for (int m = 0; m < 2 * MAXCH; ++m) U[m] = __shfl_xor_sync(0xffffffffu, U[m], 1);
                }
                const float nsgsk = -sgsk;  // the partner's sg sk
#pragma unroll
                for (int kb = 0; kb < (MAXCH + 3) / 4; ++kb) {  // 16-column batches of the accumulator
                    if (4 * kb >= nch) break;
                    uint32_t v[16];
                    if (4 * kb + 4 <= nch) {
                        tmem_ld16_wait(tD + 16 * kb, v);
                    } else {
#pragma unroll
                        for (int cc = 0; cc < 3; ++cc) {
                            if (4 * kb + cc >= nch) break;
                            uint32_t v4[4];
                            tmem_ld4(tD + 16 * kb + 4 * cc, v4);
#pragma unroll
                            for (int u = 0; u < 4; ++u) v[4 * cc + u] = v4[u];
                        }
                    }
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc) {
                        const int k = 4 * kb + cc;
                        if (k >= nch) break;
                        if (mid) {
                            float tp[4];  // the partner's own part of T_r
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                const float y = __uint_as_float(v[4 * cc + u]);
                                tp[u] = nsgsk * (y + __shfl_xor_sync(0xffffffffu, y, 2));
                            }
                            U[2 * k] += p ? tp[1] : tp[0];
                            U[2 * k + 1] += p ? tp[3] : tp[2];
                            // the top half is the partner's pieces of its tp (this lane's part of T_r),
                            // the bottom half sg times this lane's tp
                            const uint32_t x0 = tt_piece2(tp[0], tp[1], npf), x1 = tt_piece2(tp[2], tp[3], npf);
                            tmem_st2(tA + 2 * k, __shfl_xor_sync(0xffffffffu, x0, 1),
                                     __shfl_xor_sync(0xffffffffu, x1, 1));
                            tmem_st2(tAb + 2 * k, x0 ^ sflip, x1 ^ sflip);
                            continue;
                        }
                        float yp[4], tq[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const float y = __uint_as_float(v[4 * cc + u]);
                            yp[u] = y + __shfl_xor_sync(0xffffffffu, y, 2);           // own part of Y
                            const float yo = __shfl_xor_sync(0xffffffffu, yp[u], 1);  // the other part
                            tq[u] = term_is_y ? yp[u] : sgsk * yo;  // own part of T_r = (i sqrt_dt / r) Y
                        }
                        U[2 * k] += p ? tq[1] : tq[0];
                        U[2 * k + 1] += p ? tq[3] : tq[2];
                        if (last) continue;
                        float xq[4];
                        if (x_is_u) {
#pragma unroll
                            for (int i = 0; i < 2; ++i) {
                                const float mine = U[2 * k + i];
                                const float other = __shfl_xor_sync(0xffffffffu, mine, 2);
                                xq[2 * i] = p ? other : mine;
                                xq[2 * i + 1] = p ? mine : other;
                            }
                        } else {
#pragma unroll
                            for (int u = 0; u < 4; ++u) xq[u] = tq[u];
                        }
                        // the bottom half: sg times the other part (the partner's xq), as its pieces.  The
                        // rows of columns c >= nocc stay zero (zero walker entries, zero products).
                        const uint32_t x0 = tt_piece2(xq[0], xq[1], npf), x1 = tt_piece2(xq[2], xq[3], npf);
                        tmem_st2(tA + 2 * k, x0, x1);
                        tmem_st2(tAb + 2 * k, __shfl_xor_sync(0xffffffffu, x0, 1) ^ sflip,
                                 __shfl_xor_sync(0xffffffffu, x1, 1) ^ sflip);
                    }
                }
                tc_fence_before();
                if (!last) {
                    tmem_wait_st();
                    tc_fence_before();
                    mbar_arrive(bready);
                }
            }
            if (!ok) break;
            // W' = W + ((U - W32) + (E - I) out), the own entries of this lane
            double* Wo = (double*)(wout + (size_t)w * n * o + c) + q;
#pragma unroll
            for (int kb = 0; kb < (MAXCH + 3) / 4; ++kb) {
                if (4 * kb >= nch) break;
                double wv[8];
#pragma unroll
                for (int m = 0; m < 8; ++m) {  // own columns j0 + 16 kb + 2 m + p
                    const int j = j0 + 16 * kb + 2 * m + p;
                    wv[m] = (valid && 4 * kb + (m >> 1) < nch && j < n) ? Wq[(size_t)2 * j * o] : 0.0;
                }
#pragma unroll
                for (int m = 0; m < 8; ++m) {
                    const int j = j0 + 16 * kb + 2 * m + p;
                    if (valid && 4 * kb + (m >> 1) < nch && j < n)
                        Wo[(size_t)2 * j * o] = wv[m] + f2d_exact(U[8 * kb + m] - d2f_trunc(wv[m]));
                }
            }
        }
        if (!ok) {
            atomicExch(err, 1);
            *abort_flag = 1;
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

bool trotter_tc_supported(int n, int o) {
    if (!(n % 8 == 0 && n > 0 && n <= 256 && o > 0 && o <= 32)) return false;
    return tc::tt_geo(n, o).stg >= 2;
}

int launch_trotter_tc(int wc, int n, int o, int n_terms, double sqrt_dt, const __nv_bfloat16* eh,
                      const __nv_bfloat16* em, const __nv_bfloat16* vh, const __nv_bfloat16* vm, const double2* win,
                      double2* wout, int* err, cudaStream_t s) {
    using namespace tc;
    if (wc <= 0) return AFQ_OK;
    if (!trotter_tc_supported(n, o))
        return fail(AFQ_E_UNSUPPORTED, "tensor-core Trotter: norb=%d nocc=%d (needs norb %% 8 == 0, <= 256, nocc <= 32)",
                    n, o);
    if (n_terms < 0) return fail(AFQ_E_INVALID_ARGUMENT, "n_exp_terms=%d must be >= 0", n_terms);
    const TTGeo g = tt_geo(n, o);
    static DeviceOnce smem_once[4];
    AFQ_TRY(get_encode());
    int nsm = 0;
    AFQ_TRY(device_sms(&nsm));
    const int nch = g.N / 16;
    const int inst = nch <= 4 ? 0 : nch <= 8 ? 1 : nch <= 13 ? 2 : 3;
    switch (inst) {
        case 0: AFQ_TRY(raise_smem_once(smem_once[0], k_trotter_tc<4>, TT_SMEM_MAX)); break;
        case 1: AFQ_TRY(raise_smem_once(smem_once[1], k_trotter_tc<8>, TT_SMEM_MAX)); break;
        case 2: AFQ_TRY(raise_smem_once(smem_once[2], k_trotter_tc<13>, TT_SMEM_MAX)); break;
        default: AFQ_TRY(raise_smem_once(smem_once[3], k_trotter_tc<16>, TT_SMEM_MAX)); break;
    }
    CUtensorMap mvh, mvm, meh, mem;
    AFQ_TRY(make_map3(&mvh, vh, 2LL * wc, n, n, n, g.N));
    AFQ_TRY(make_map3(&mvm, vm, 2LL * wc, n, n, n, g.N));
    AFQ_TRY(make_map(&meh, eh, n, n, n, g.N));
    AFQ_TRY(make_map(&mem, em, n, n, n, g.N));
    const int grid = wc < nsm ? wc : nsm;
#define AFQ_TT(MC)                                                                                         \
    k_trotter_tc<MC><<<grid, TT_THREADS, g.smem, s>>>(mvh, mvm, meh, mem, wc, n, o, n_terms, (float)sqrt_dt, g, win, \
                                                    wout, err)
    switch (inst) {
        case 0: AFQ_TT(4); break;
        case 1: AFQ_TT(8); break;
        case 2: AFQ_TT(13); break;
        default: AFQ_TT(16); break;
    }
#undef AFQ_TT
    AFQ_LAUNCHED("k_trotter_tc");
    return AFQ_OK;
}

// (E - I) as bf16 hi and mid pieces (n x n), the B operand of the E products
// (row j over K = k: (E - I)[j, k]).
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
