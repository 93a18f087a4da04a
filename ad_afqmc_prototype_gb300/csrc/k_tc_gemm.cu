// Tensor-core GEMM for sm_103a: C[M x N] (fp32) = A[M x K] . B[N x K]^T with
// bf16 operands, both K-major (row-major with K contiguous).
//
// Blackwell path: TMA (cp.async.bulk.tensor, 128-byte swizzle) stages
// 128x64 A and 256x64 B tiles through a 4-deep shared-memory ring guarded by
// mbarriers; one thread issues tcgen05.mma (kind::f16, M=128, N=256, K=16)
// into a double-buffered fp32 accumulator in tensor memory; four epilogue
// warps read the accumulator back with tcgen05.ld and store it.  The kernel
// is persistent (one CTA per SM, static round-robin over tiles, M-tiles
// fastest so CTAs working at the same time share B tiles in L2).
//
// Mixed-precision products use the operand layout, not the kernel: a split
// x = hi + lo (both bf16) is written along K in sections, A = [a_hi a_hi a_lo]
// and B = [b_hi b_lo b_hi], so one GEMM returns a_hi b_hi + a_hi b_lo +
// a_lo b_hi (relative error ~2^-17 instead of 2^-9).
//
// Every mbarrier wait is bounded (1 s of %globaltimer); on a timeout the CTA
// raises *err, every role leaves its loop, the producer waits (bounded) for
// the copies it issued, and the tensor memory is freed before returning.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "afq_internal.cuh"
#include "tc_common.cuh"

namespace afq {
namespace tc {

constexpr int BM = 128, BN = 256, BK = 64, STAGES = 4;
constexpr int A_BYTES = BM * BK * 2;
constexpr int B_BYTES = BN * BK * 2;
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int ACC_COLS = BN;
constexpr int TMEM_COLS = 2 * ACC_COLS;
constexpr int THREADS = 192;  // warp 0: TMA, warp 1: MMA + TMEM owner, warps 2-5: epilogue
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;

// instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A bf16 (7-9 = 1),
// B bf16 (10-12 = 1), both K-major (bits 15, 16 = 0), N>>3 at 17, M>>4 at 24
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    umma_bf16_i(d_tmem, adesc, bdesc, IDESC, accumulate);
}
__global__ void __launch_bounds__(THREADS, 1)
    k_gemm_tn(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, float* __restrict__ C,
              int M, int N, int K, long long ldc, int* __restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = smem;
    uint8_t* sB = smem + STAGES * A_BYTES;
    uint64_t* bars = (uint64_t*)(smem + STAGES * STAGE_BYTES);
    uint32_t* tmem_slot = (uint32_t*)(bars + 2 * STAGES + 5);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES);
    const uint32_t tfull0 = smem_u32(bars + 2 * STAGES), tempty0 = smem_u32(bars + 2 * STAGES + 2);
    const uint32_t drain = smem_u32(bars + 2 * STAGES + 4);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mt = (M + BM - 1) / BM, nt = (N + BN - 1) / BN, kt = K / BK;
    const int ntiles = mt * nt;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(tfull0 + 8 * a, 1);
            mbar_init(tempty0 + 8 * a, 128);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&tmA) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&tmB) : "memory");
            int stage = 0;
            uint32_t phase = 0;
            int issued[STAGES];
            uint32_t issued_par[STAGES];
            for (int s = 0; s < STAGES; ++s) issued[s] = 0;
            bool ok = true;
            for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
                const int mb = t % mt, nb = t / mt;
                for (int kb = 0; kb < kt; ++kb) {
                    if (!mbar_wait(empty0 + 8 * stage, phase ^ 1, abort_flag)) { ok = false; break; }
                    issued[stage] = 0;  // the consumer released it: its copy had landed
                    mbar_expect_tx(full0 + 8 * stage, STAGE_BYTES);
                    tma_load_2d(smem_u32(sA + stage * A_BYTES), &tmA, kb * BK, mb * BM, full0 + 8 * stage);
                    tma_load_2d(smem_u32(sB + stage * B_BYTES), &tmB, kb * BK, nb * BN, full0 + 8 * stage);
                    issued[stage] = 1;
                    issued_par[stage] = phase;
                    if (++stage == STAGES) { stage = 0; phase ^= 1; }
                }
            }
            if (!ok) {
                atomicExch(err, 1);
                *abort_flag = 1;
            }
            // every copy this thread issued lands before the CTA exits (after an
            // abort elsewhere in the CTA nobody else waits for them)
            for (int s = 0; s < STAGES; ++s)
                if (issued[s]) mbar_wait(full0 + 8 * s, issued_par[s], nullptr);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int stage = 0, acc = 0;
            uint32_t phase = 0, acc_phase = 0;
            bool ok = true;
            for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
                if (!mbar_wait(tempty0 + 8 * acc, acc_phase ^ 1, abort_flag)) { ok = false; break; }
                tc_fence_after();
                const uint32_t d = tmem + acc * ACC_COLS;
                for (int kb = 0; kb < kt; ++kb) {
                    if (!mbar_wait(full0 + 8 * stage, phase, abort_flag)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t a0 = smem_u32(sA + stage * A_BYTES), b0 = smem_u32(sB + stage * B_BYTES);
#pragma unroll
                    for (int k = 0; k < BK / 16; ++k)
                        umma_bf16(d, desc_k128(a0 + 32 * k), desc_k128(b0 + 32 * k), (kb | k) != 0);
                    umma_commit(empty0 + 8 * stage);
                    if (++stage == STAGES) { stage = 0; phase ^= 1; }
                }
                if (!ok) break;
                umma_commit(tfull0 + 8 * acc);
                if (++acc == 2) { acc = 0; acc_phase ^= 1; }
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
        const int q = warp & 3;  // TMEM lane quarter this warp may access
        int acc = 0;
        uint32_t acc_phase = 0;
        const bool vec = (ldc % 4) == 0 && (((uintptr_t)C) & 15) == 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
            const int mb = t % mt, nb = t / mt;
            if (!mbar_wait(tfull0 + 8 * acc, acc_phase, abort_flag)) {
                atomicExch(err, 1);
                *abort_flag = 1;
                break;
            }
            tc_fence_after();
            const int row = mb * BM + q * 32 + lane;
            float* dst_row = C + (long long)row * ldc;
#pragma unroll 1
            for (int c = 0; c < BN; c += 32) {
                uint32_t r[32];
                tmem_ld32(tmem + acc * ACC_COLS + c + ((uint32_t)(q * 32) << 16), r);
                const int col0 = nb * BN + c;
                if (row < M && col0 < N) {
                    float* dst = dst_row + col0;
                    if (vec && col0 + 32 <= N) {
#pragma unroll
                        for (int j = 0; j < 32; j += 4)
                            *(float4*)(dst + j) = make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]),
                                                              __uint_as_float(r[j + 2]), __uint_as_float(r[j + 3]));
                    } else {
#pragma unroll
                        for (int j = 0; j < 32; ++j)
                            if (col0 + j < N) dst[j] = __uint_as_float(r[j]);
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(tempty0 + 8 * acc);
            if (++acc == 2) { acc = 0; acc_phase ^= 1; }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// ----------------------------------------------------------------- drained --
// Same pipeline, but the fp32 sum over K is formed outside the tensor cores.
// The tensor cores' fp32 accumulation truncates: summing K positive terms
// drifts low by ~K/16 * 2^-25 relative (about -3e-5 at K = 16384, measured),
// and that drift is coherent across a whole contraction.  Here every 64-wide
// K block starts a fresh partial in tensor memory (4 MMAs, bias < 2^-23), and
// eight epilogue warps add the partials into fp32 registers with
// round-to-nearest adds (two lanes per instruction) while the MMA thread
// fills the next slot.  Warp w may only read TMEM lanes 32*(w%4)..+31, so
// warps 2-5 and 6-9 each cover all 128 rows, one column half each.
constexpr int DTMEM_COLS = 512;

// 64 + 32 EWN threads (warp 0 TMA, warp 1 MMA + TMEM owner, EWN epilogue
// warps, EWN / 4 of them on each 32-lane quarter of the accumulator); each
// epilogue thread sums CW = 4 BNT / EWN columns of one row.  Sixteen
// epilogue warps drain a 128 x 256 partial in about half the time of eight
// (the drain has to keep up with the MMAs of the next partial).
template <int BNT, int EWN = 8>
struct Drain {
    static_assert(EWN == 8 || EWN == 16, "eight or sixteen epilogue warps");
    static constexpr int THREADS = 64 + 32 * EWN;
    static constexpr int EW0 = 2;  // first epilogue warp
    static constexpr int SLOTS = DTMEM_COLS / BNT;
    static constexpr int STG = BNT == 128 ? 6 : 4;
    static constexpr int B_BYTES = BNT * BK * 2;
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static constexpr int SMEM = STG * STAGE + 1024 + 256;
    static constexpr int CW = 4 * BNT / EWN;  // columns per epilogue warp
    static constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BNT >> 3) << 17) |
                                      ((uint32_t)(BM >> 4) << 24);
};
static_assert(Drain<128>::SMEM <= 227 * 1024, "drained GEMM shared memory");
static_assert(Drain<256>::SMEM <= 227 * 1024, "drained GEMM shared memory (256-wide tiles)");

// Epilogue of the exchange-fused energy GEMM (MODE 2): a 32 x 33 fp32
// transpose buffer per epilogue warp after the barriers.
constexpr int XT_BYTES = 8 * 32 * 33 * 4;
constexpr int EXCH_BNT = 256;  // tile width of the exchange-fused GEMM
static_assert(Drain<EXCH_BNT>::SMEM + XT_BYTES <= 227 * 1024, "exchange-fused GEMM shared memory");

// Outputs of MODE 2 (the local energy's exchange, meas/rhf.py:36-50).  Rows
// of the product are (walker, part, k) with 32 rows per part (k >= nocc zero)
// and columns (g, i) with 32 per Cholesky vector, so a 128 x 256 tile holds
// the Re and Im planes of f_g[i, k] for two walkers and eight vectors.
//   x[(w nhalf + h) 2 + part] = sum over the 128-column half h of
//                               sum_{i,k} F_part[k, i] F_part[i, k]
//   c[(w G + g) 2 + part]     = sum_k F_part[k, k]   (the trace of f_g)
struct ExchOut {
    float* x = nullptr;
    float* c = nullptr;
    int G = 0;       // Cholesky vectors
    int nw = 0;      // walkers in this product
    int nhalf = 0;   // column halves per row = 2 x column tiles
};

// Transpose, in each half-warp, of a 16 x 16 block of 32-bit words held one
// row a lane (v[j] = word j of row `lane`) into one column a lane (v[r] =
// word lane & 15 of row 16 (lane >> 4) + r): four butterfly stages, each
// lane trading half of its words with lane ^ d.
__device__ __forceinline__ void halfwarp_transpose16(uint32_t (&v)[16], int lane) {
#pragma unroll
    for (int d = 8; d >= 1; d >>= 1) {
        const bool upper = (lane & d) != 0;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            if (j & d) continue;
            const uint32_t send = upper ? v[j] : v[j | d];
            const uint32_t recv = __shfl_xor_sync(0xffffffffu, send, d);
            if (upper) v[j] = recv;
            else v[j | d] = recv;
        }
    }
}

// MODE 0: fp32 C.  MODE 1 (split): the two-piece bf16 split of each sum to
// Ch (hi) and Cm (mid = bf16(c - hi)), same row stride ldc.  MODE 2: the
// exchange contraction of each 32 x 32 block (ExchOut) instead of C.
//
// Tile order of the persistent schedule: order < 0, N tiles fastest; order =
// gm > 0, M tiles fastest within groups of gm M tiles (all N tiles of a group
// before the next group).
__device__ __forceinline__ void drain_tile(int t, int mt, int nt, int order, int& mb, int& nb) {
    if (order < 0) {
        mb = t / nt;
        nb = t % nt;
        return;
    }
    const int g = t / (order * nt), r = t - g * order * nt, m0 = g * order, gsz = min(order, mt - m0);
    mb = m0 + r % gsz;
    nb = r / gsz;
}

// Each CTA loads its own A and B tiles with plain TMA copies.  Tile order:
// with M tiles fastest the CTAs resident at one time work on one or two N
// tiles, so a B tile is read from DRAM about once and served from L2 to the
// CTAs that share it, while the group's A tiles are re-read from L2 once per
// N tile; the launcher picks N tiles fastest when A is the large operand and
// B fits in L2, and groups the M tiles when neither fits (each group's A then
// stays in L2 beside the output stream, B is read once per group).
template <int BNT, int MODE, int EWN>
__global__ void __launch_bounds__(Drain<BNT, EWN>::THREADS, 1)
    k_gemm_tn_drain(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    float* __restrict__ C, __nv_bfloat16* __restrict__ Ch, __nv_bfloat16* __restrict__ Cm, int M,
                    int N, int K, long long ldc, int kd, int* __restrict__ err, ExchOut xo, int order) {
    using D = Drain<BNT, EWN>;
    static_assert(MODE != 2 || EWN == 8, "the exchange epilogue's transpose buffers are sized for eight warps");
    constexpr bool SPLIT = MODE == 1;
    static_assert(MODE != 2 || BNT % 64 == 0, "the exchange epilogue takes whole 32 x 32 blocks per warp");
    constexpr int STG = D::STG, SLOTS = D::SLOTS, CW = D::CW;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sA = smem;
    uint8_t* sB = smem + STG * A_BYTES;
    uint64_t* bars = (uint64_t*)(smem + STG * D::STAGE);
    uint32_t* tmem_slot = (uint32_t*)(bars + 2 * STG + 2 * SLOTS + 1);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STG);
    const uint32_t tfull0 = smem_u32(bars + 2 * STG), tempty0 = smem_u32(bars + 2 * STG + SLOTS);
    const uint32_t drain = smem_u32(bars + 2 * STG + 2 * SLOTS);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mt = (M + BM - 1) / BM, nt = (N + BNT - 1) / BNT, kt = K / BK;
    const int ntiles = mt * nt, np = (kt + kd - 1) / kd;  // np: partials per tile

    if (threadIdx.x == 0) {
        for (int s = 0; s < STG; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        for (int a = 0; a < SLOTS; ++a) {
            mbar_init(tfull0 + 8 * a, 1);
            mbar_init(tempty0 + 8 * a, 32 * EWN);  // every epilogue thread
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(DTMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&tmA) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&tmB) : "memory");
            int stage = 0;
            uint32_t phase = 0;
            int issued[STG];
            uint32_t issued_par[STG];
            for (int s = 0; s < STG; ++s) issued[s] = 0;
            bool ok = true;
            for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
                int mb, nb;
                drain_tile(t, mt, nt, order, mb, nb);
                for (int kb = 0; kb < kt; ++kb) {
                    if (!mbar_wait(empty0 + 8 * stage, phase ^ 1, abort_flag)) { ok = false; break; }
                    issued[stage] = 0;
                    mbar_expect_tx(full0 + 8 * stage, D::STAGE);
                    const uint32_t fb = full0 + 8 * stage;
                    tma_load_2d(smem_u32(sA + stage * A_BYTES), &tmA, kb * BK, mb * BM, fb);
                    tma_load_2d(smem_u32(sB + stage * D::B_BYTES), &tmB, kb * BK, nb * BNT, fb);
                    issued[stage] = 1;
                    issued_par[stage] = phase;
                    if (++stage == STG) { stage = 0; phase ^= 1; }
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
            int stage = 0, slot = 0;
            uint32_t phase = 0, slot_phase = 0;
            bool ok = true;
            for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
                for (int kb = 0; kb < kt; ++kb) {
                    const int g = kb % kd;  // position inside the current partial
                    if (!mbar_wait(full0 + 8 * stage, phase, abort_flag)) { ok = false; break; }
                    if (g == 0 && !mbar_wait(tempty0 + 8 * slot, slot_phase ^ 1, abort_flag)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t a0 = smem_u32(sA + stage * A_BYTES), b0 = smem_u32(sB + stage * D::B_BYTES);
#pragma unroll
                    for (int k = 0; k < BK / 16; ++k)
                        umma_bf16_i(tmem + slot * BNT, desc_k128(a0 + 32 * k), desc_k128(b0 + 32 * k), D::IDESC,
                                    (k != 0) || (g != 0));
                    umma_commit(empty0 + 8 * stage);
                    if (g == kd - 1 || kb == kt - 1) {
                        umma_commit(tfull0 + 8 * slot);
                        if (++slot == SLOTS) { slot = 0; slot_phase ^= 1; }
                    }
                    if (++stage == STG) { stage = 0; phase ^= 1; }
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
    } else if (warp >= D::EW0) {
        const int q = warp & 3, cb = ((warp - D::EW0) >> 2) * CW;
        int slot = 0;
        uint32_t slot_phase = 0;
        const bool vec = SPLIT ? (ldc % 8) == 0 && ((((uintptr_t)Ch) | ((uintptr_t)Cm)) & 15) == 0
                               : (ldc % 4) == 0 && (((uintptr_t)C) & 15) == 0;
        bool ok = true;
        for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
            int mb, nb;
            drain_tile(t, mt, nt, order, mb, nb);
            float2 acc[CW / 2];
#pragma unroll
            for (int j = 0; j < CW / 2; ++j) acc[j] = make_float2(0.f, 0.f);
            for (int p = 0; p < np; ++p) {
                if (!mbar_wait_inl(tfull0 + 8 * slot, slot_phase, abort_flag)) {
                    atomicExch(err, 1);
                    *abort_flag = 1;
                    ok = false;
                    break;
                }
                tc_fence_after();
                // chunks of LC columns; the sums of a chunk are complete before the
                // next load, so at most LC staged values are live
                constexpr int LC = EWN == 16 ? 16 : BNT == 128 ? 64 : 32;
#pragma unroll
                for (int c = 0; c < CW; c += LC) {
                    uint32_t r[LC];
                    const uint32_t ta = tmem + slot * BNT + cb + c + ((uint32_t)(q * 32) << 16);
                    if constexpr (LC == 64) tmem_ld64(ta, r);
                    else if constexpr (LC == 32) tmem_ld32(ta, r);
                    else tmem_ld16(ta, r);
#pragma unroll
                    for (int j = 0; j < LC / 2; ++j) {
                        if constexpr (BNT == 128) {
                            acc[c / 2 + j] = __fadd2_rn(acc[c / 2 + j], make_float2(__uint_as_float(r[2 * j]),
                                                                                    __uint_as_float(r[2 * j + 1])));
                        } else {  // scalar adds: fewer registers than paired ones at 128 sums a thread
                            acc[c / 2 + j].x += __uint_as_float(r[2 * j]);
                            acc[c / 2 + j].y += __uint_as_float(r[2 * j + 1]);
                        }
                    }
                    if constexpr (BNT == 128) {
#pragma unroll
                        for (int j = 0; j < LC / 2; ++j)
                            asm volatile("" : "+f"(acc[c / 2 + j].x), "+f"(acc[c / 2 + j].y));
                    }
                }
                tc_fence_before();
                mbar_arrive(tempty0 + 8 * slot);
                if (++slot == SLOTS) { slot = 0; slot_phase ^= 1; }
            }
            if (!ok) break;
            if constexpr (MODE == 2) {
                // this warp's 32 rows are (walker wl, part) rows k = lane of 32 x 32 blocks;
                // the thread's CW columns are the blocks of CW / 32 Cholesky vectors
                float* tr = (float*)(smem + STG * D::STAGE + 256) + (warp - D::EW0) * 32 * 33;
                const int wl = mb * 2 + (q >> 1), part = q & 1;
                float ex = 0.f;
#pragma unroll
                for (int jj = 0; jj < CW / 32; ++jj) {
                    const int g = (nb * BNT + cb) / 32 + jj;
#pragma unroll
                    for (int i = 0; i < 32; i += 2) {
                        tr[lane * 33 + i] = acc[jj * 16 + i / 2].x;
                        tr[lane * 33 + i + 1] = acc[jj * 16 + i / 2].y;
                    }
                    __syncwarp();
                    float e2 = 0.f;
#pragma unroll
                    for (int i = 0; i < 32; i += 2) {
                        e2 = fmaf(acc[jj * 16 + i / 2].x, tr[i * 33 + lane], e2);
                        e2 = fmaf(acc[jj * 16 + i / 2].y, tr[(i + 1) * 33 + lane], e2);
                    }
                    ex += e2;
                    float d = tr[lane * 33 + lane];
#pragma unroll
                    for (int off = 16; off > 0; off >>= 1) d += __shfl_xor_sync(0xffffffffu, d, off);
                    if (lane == 0 && wl < xo.nw && g < xo.G) xo.c[((size_t)wl * xo.G + g) * 2 + part] = d;
                    __syncwarp();
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) ex += __shfl_xor_sync(0xffffffffu, ex, off);
                if (lane == 0 && wl < xo.nw)
                    xo.x[((size_t)wl * xo.nhalf + nb * (BNT / CW) + cb / CW) * 2 + part] = ex;
                continue;
            }
            const int row = mb * BM + q * 32 + lane;
            const int col0 = nb * BNT + cb;
            if constexpr (SPLIT && CW == 64) {
                // the warp's 32 rows x 64 columns of bf16 pairs (hi, mid) in 16-word halves, each
                // transposed within the half-warps so that one store writes 64 contiguous bytes
                // (two whole sectors) of each of two rows
                if (vec && col0 + CW <= N && __activemask() == 0xffffffffu) {
                    const int rw = mb * BM + q * 32 + 16 * (lane >> 4), wc = lane & 15;
#pragma unroll
                    for (int half = 0; half < 2; ++half) {
                        uint32_t hv[16], mv[16];
#pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            const float2 a = acc[16 * half + j];
                            const __nv_bfloat162 h = __floats2bfloat162_rn(a.x, a.y);
                            const float2 hf = __bfloat1622float2(h);
                            const __nv_bfloat162 m = __floats2bfloat162_rn(a.x - hf.x, a.y - hf.y);
                            hv[j] = *(const uint32_t*)&h;
                            mv[j] = *(const uint32_t*)&m;
                        }
                        halfwarp_transpose16(hv, lane);
                        halfwarp_transpose16(mv, lane);
                        const long long c = col0 + 32 * half + 2 * wc;
#pragma unroll
                        for (int r = 0; r < 16; ++r) {
                            if (rw + r < M) {
                                __stcs((uint32_t*)(Ch + (long long)(rw + r) * ldc + c), hv[r]);
                                __stcs((uint32_t*)(Cm + (long long)(rw + r) * ldc + c), mv[r]);
                            }
                        }
                    }
                    continue;
                }
            }
            if (row < M && SPLIT) {
                __nv_bfloat16* dh = Ch + (long long)row * ldc + col0;
                __nv_bfloat16* dm = Cm + (long long)row * ldc + col0;
                if (vec && col0 + CW <= N) {
#pragma unroll
                    for (int j = 0; j < CW / 2; j += 4) {
                        uint32_t ph[4], pm[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const __nv_bfloat162 h = __floats2bfloat162_rn(acc[j + u].x, acc[j + u].y);
                            const float2 hf = __bfloat1622float2(h);
                            const __nv_bfloat162 m = __floats2bfloat162_rn(acc[j + u].x - hf.x, acc[j + u].y - hf.y);
                            ph[u] = *(const uint32_t*)&h;
                            pm[u] = *(const uint32_t*)&m;
                        }
                        // streaming stores: the output is read once, by another kernel
                        __stcs((uint4*)(dh + 2 * j), make_uint4(ph[0], ph[1], ph[2], ph[3]));
                        __stcs((uint4*)(dm + 2 * j), make_uint4(pm[0], pm[1], pm[2], pm[3]));
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < CW; ++j) {
                        if (col0 + j < N) {
                            const float v = (j & 1) ? acc[j / 2].y : acc[j / 2].x;
                            const __nv_bfloat16 h = __float2bfloat16(v);
                            dh[j] = h;
                            dm[j] = __float2bfloat16(v - __bfloat162float(h));
                        }
                    }
                }
            } else if (row < M) {
                float* dst = C + (long long)row * ldc + col0;
                if (vec && col0 + CW <= N) {
#pragma unroll
                    for (int j = 0; j < CW / 2; j += 2)
                        __stcs((float4*)(dst + 2 * j), make_float4(acc[j].x, acc[j].y, acc[j + 1].x, acc[j + 1].y));
                } else {
#pragma unroll
                    for (int j = 0; j < CW / 2; ++j) {
                        if (col0 + 2 * j < N) dst[2 * j] = acc[j].x;
                        if (col0 + 2 * j + 1 < N) dst[2 * j + 1] = acc[j].y;
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(DTMEM_COLS) : "memory");
    }
}

}  // namespace tc

static DeviceOnce g_tn_smem;

int launch_tc_gemm_tn(int M, int N, int K, const void* A, long long lda, const void* B, long long ldb, float* C,
                      long long ldc, int* err, cudaStream_t s) {
    using namespace tc;
    if (M <= 0 || N <= 0) return AFQ_OK;
    if (K <= 0 || K % BK) return fail(AFQ_E_INVALID_ARGUMENT, "tc gemm: K=%d must be a positive multiple of %d", K, BK);
    AFQ_TRY(get_encode());
    CUtensorMap ma, mb;
    AFQ_TRY(make_map(&ma, A, M, K, lda, BM));
    AFQ_TRY(make_map(&mb, B, N, K, ldb, BN));
    int sms = 0;
    AFQ_TRY(device_sms(&sms));
    AFQ_TRY(raise_smem_once(g_tn_smem, k_gemm_tn, SMEM_BYTES));
    const long long tiles = (long long)((M + BM - 1) / BM) * ((N + BN - 1) / BN);
    const int grid = (int)(tiles < sms ? tiles : sms);
    k_gemm_tn<<<grid, THREADS, SMEM_BYTES, s>>>(ma, mb, C, M, N, K, ldc, err);
    AFQ_LAUNCHED("k_gemm_tn");
    return AFQ_OK;
}

// Persistent launch: one CTA per SM (the shared-memory ring admits one), or
// one per tile when there are fewer tiles.
template <int BNT, int MODE, int EWN>
static int launch_drain(int M, int N, int K, const void* A, long long lda, const void* B, long long ldb, float* C,
                        __nv_bfloat16* Ch, __nv_bfloat16* Cm, long long ldc, int kd, int* err, cudaStream_t s,
                        tc::ExchOut xo = tc::ExchOut{}, int mgroup = 0) {
    using namespace tc;
    static DeviceOnce smem_once;
    constexpr int SMEM = Drain<BNT, EWN>::SMEM + (MODE == 2 ? XT_BYTES : 0);
    auto kern = k_gemm_tn_drain<BNT, MODE, EWN>;
    CUtensorMap ma, mb;
    AFQ_TRY(make_map(&ma, A, M, K, lda, BM));
    AFQ_TRY(make_map(&mb, B, N, K, ldb, BNT));
    int sms = 0;
    AFQ_TRY(device_sms(&sms));
    AFQ_TRY(raise_smem_once(smem_once, kern, SMEM));
    const long long tiles = (long long)((M + BM - 1) / BM) * ((N + BNT - 1) / BNT);
    const int grid = (int)(tiles < sms ? tiles : sms);
    // tile order: the operand re-read once per tile of the other should fit in
    // L2 beside the streams; if A does not and B does, N tiles run fastest (the
    // force-bias and energy GEMMs: full-size DRAM reads within 1.1x of the
    // operands' bytes); if neither does, M tiles run fastest in groups whose A
    // tiles take at most kAGroup bytes (the V-build)
    constexpr long long kL2Keep = 48LL << 20, kAGroup = 32LL << 20;
    const int mt = (M + BM - 1) / BM;
    const long long a_bytes = (long long)M * K * 2, b_bytes = (long long)N * K * 2;
    int order;
    if (a_bytes > kL2Keep && b_bytes <= kL2Keep) {
        order = -1;
    } else {
        const long long tile_a = (long long)BM * K * 2;
        const int ng = (int)(((long long)mt * tile_a + kAGroup - 1) / kAGroup);
        order = mgroup > 0 ? mgroup : (mt + ng - 1) / ng;
    }
    kern<<<grid, Drain<BNT, EWN>::THREADS, SMEM, s>>>(ma, mb, C, Ch, Cm, M, N, K, ldc, kd, err, xo, order);
    AFQ_LAUNCHED(MODE == 2 ? "k_gemm_tn_drain(exchange)" : "k_gemm_tn_drain");
    return AFQ_OK;
}

static int drain_prologue(int K, int kd) {
    using namespace tc;
    if (K <= 0 || K % BK) return fail(AFQ_E_INVALID_ARGUMENT, "tc gemm: K=%d must be a positive multiple of %d", K, BK);
    if (kd < 1) return fail(AFQ_E_INVALID_ARGUMENT, "tc gemm: k blocks per partial %d < 1", kd);
    AFQ_TRY(get_encode());
    return AFQ_OK;
}
int launch_tc_gemm_tn_drain(int M, int N, int K, const void* A, long long lda, const void* B, long long ldb, float* C,
                            long long ldc, int* err, cudaStream_t s, int kd) {
    if (M <= 0 || N <= 0) return AFQ_OK;
    AFQ_TRY(drain_prologue(K, kd));
    return launch_drain<256, 0, 16>(M, N, K, A, lda, B, ldb, C, nullptr, nullptr, ldc, kd, err, s);
}

int launch_tc_gemm_tn_drain_split(int M, int N, int K, const void* A, long long lda, const void* B, long long ldb,
                                  __nv_bfloat16* Ch, __nv_bfloat16* Cm, long long ldc, int* err, cudaStream_t s,
                                  int kd) {
    if (M <= 0 || N <= 0) return AFQ_OK;
    AFQ_TRY(drain_prologue(K, kd));
    return launch_drain<256, 1, 16>(M, N, K, A, lda, B, ldb, nullptr, Ch, Cm, ldc, kd, err, s);
}

int launch_tc_gemm_exchange(int nw, int G, int K, const void* A, long long lda, const void* B, long long ldb,
                            float* x, float* c, int* err, cudaStream_t s, int kd) {
    if (nw <= 0 || G <= 0) return AFQ_OK;
    AFQ_TRY(drain_prologue(K, kd));
    const int M = 64 * nw, N = 32 * G;
    tc::ExchOut xo;
    xo.x = x;
    xo.c = c;
    xo.G = G;
    xo.nw = nw;
    xo.nhalf = exchange_halves(G);
    return launch_drain<tc::EXCH_BNT, 2, 8>(M, N, K, A, lda, B, ldb, nullptr, nullptr, nullptr, 0, kd, err, s, xo);
}

int exchange_halves(int G) { return 2 * ((32 * G + tc::EXCH_BNT - 1) / tc::EXCH_BNT); }

}  // namespace afq
