// m = C^T W for every walker of the mixed forms as one tensor-core
// contraction with binary64-level accuracy (meas/rhf.py:22-24: the overlap
// matrix of the RHF trial C, real, with each walker W).
//
// Both operands are cut into 7 signed base-128 digits on a power-of-two
// grid (the integer-slicing idea of Ozaki, Ogita, Oishi and Rump, 2012):
//   W[i][b].part = 2^E_r  sum_{s=1..7} w_s[i] 2^(-7 s),  |w_s| <= 64,
//   C[i][a]      = 2^F_a  sum_{t=1..7} c_t[i] 2^(-7 t),  |c_t| <= 64,
// with E_r two above the exponent of the largest entry of the row r =
// (walker, b, part), F_a the same for column a of C (so the scaled entries
// are below 1/4 and the top digit stays in range), each digit an integer
// bf16 holds exactly.  The product D = A B^T takes A row r with orbital i's
// digits in the eight K slots 8 i .. 8 i + 7 (w_1 .. w_7, then a zero), and B
// row (a, d), d = 2..9, with c_{d-s} in the slot of w_s (zero where d - s is
// not a digit index):
//   D[r][(a, d)] = sum_{s + t = d} sum_i w_s[i] c_t[i],
// an integer of magnitude <= 7 x norb x 2^12 < 2^24 for norb <= 584, so the
// tensor cores' fp32 sums are exact.  Then
//   m = 2^(E_r + F_a) sum_{d=2..9} D_d 2^(-7 d)
// with the terms s + t > 9 left out (each below 2^-51 of 2^(E_r + F_a) an
// orbital) and the digits cut toward zero at 2^-49: m to ~2^-43 of the
// product of the row's and the column's largest entries (sums over the
// orbitals of errors ~2^-49 each), the accuracy class of the double-float m
// it replaces, given as a double-float pair.
//
// k_oz_m builds A itself: the walkers' rows are bulk-copied into shared
// memory beside each B tile, sixteen producer warps cut them into digits and
// write the 128-byte-swizzled A tile, one thread issues the MMAs, four
// epilogue warps recombine the digit sums from tensor memory, and four more
// warps find the next tile's row scales E_r.  A never goes through HBM.
#include "afq_internal.cuh"
#include "tc_common.cuh"

namespace afq {

OzDims oz_dims(int n, int o) {
    OzDims z;
    z.nks = (n + 7) / 8;
    z.K = 64 * z.nks;
    z.NB = 8 * (o + (o & 1));
    return z;
}

namespace {

// Balanced base-128 digits d_t in [-64, 64) of X (|X| < 2^47), X = sum d_t
// 128^t, are the plain base-128 digits of X + OZ_OFF minus 64.
constexpr long long OZ_OFF = 64LL * ((1LL << 49) - 1) / 127;

// The 7 signed base-128 digits of x 2^-E (|x| 2^-E < 1/4) cut toward zero at
// 2^-49, most significant first, by integer operations: x = +-mant 2^(eb -
// 1075), so the 49-bit fixed-point value (|X| < 2^47) is mant shifted right by
// E + 1026 - eb (>= 6).  Zero for zero, subnormal and non-finite x.
__device__ __forceinline__ unsigned long long oz_fixed(double x, int E) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const int eb = (int)((u >> 52) & 0x7ffu), rs = E + 1026 - eb;
    long long X = 0;
    if (eb != 0 && eb != 0x7ff && rs < 64) {
        X = (long long)(((u & 0xfffffffffffffull) | (1ull << 52)) >> rs);
        if ((long long)u < 0) X = -X;
    }
    return (unsigned long long)(X + OZ_OFF);
}
__device__ __forceinline__ uint32_t oz_bf2(float lo, float hi) {  // two small integers as a bf16 pair (exact)
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *(const uint32_t*)&v;
}
// Orbital i's eight K slots of an A row (w_1 .. w_7 and a zero) from the two
// words of x, with Ep = E + 1026, in 32-bit operations: the digits of |x| (of
// |X| + OZ_OFF's base-128 fields f, each f - 64) times the sign of x, which
// is again a balanced expansion (of X) with |digits| <= 64.  A digit is
// fma(sign, 2^23 + f, -sign (2^23 + 64)), exact.
__device__ __forceinline__ uint4 oz_chunk(uint32_t ulo, uint32_t uhi, int Ep) {
    const int eb = (int)((uhi >> 20) & 0x7ffu), rs = Ep - eb;
    uint32_t xl = 0, xh = 0;
    if (eb != 0 && eb != 0x7ff && rs < 64) {
        const uint32_t mh = (uhi & 0xfffffu) | 0x100000u;
        if (rs < 32) {
            xl = __funnelshift_r(ulo, mh, rs);
            xh = mh >> rs;
        } else {
            xl = mh >> (rs - 32);
        }
    }
    const unsigned long long Y = (((unsigned long long)xh << 32) | xl) + (unsigned long long)OZ_OFF;
    const uint32_t lo = (uint32_t)Y, hi = (uint32_t)(Y >> 28);
    const float sg = __int_as_float(0x3f800000u | (uhi & 0x80000000u)), c = -8388672.f * sg;
#define OZ_F(v, sh) fmaf(sg, __int_as_float(0x4B000000u | (((v) >> (sh)) & 127u)), c)
    return make_uint4(oz_bf2(OZ_F(hi, 14), OZ_F(hi, 7)), oz_bf2(OZ_F(hi, 0), OZ_F(lo, 21)),
                      oz_bf2(OZ_F(lo, 14), OZ_F(lo, 7)), oz_bf2(OZ_F(lo, 0), 0.f));
#undef OZ_F
}
__device__ __forceinline__ int oz_digit(double x, int E, int s) {  // w_s, s = 1..7
    const unsigned long long Y = oz_fixed(x, E);
    return (int)((Y >> (7 * (7 - s))) & 127u) - 64;
}
__device__ __forceinline__ int oz_ebits(double x) {  // biased binary64 exponent (2047 for inf / nan)
    return (int)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ffu);
}

// B (NB x K, K-major) and F_a from the trial C (n x o, real part used): one
// CTA per B row (a, d), each finding its column's scale.
__global__ void __launch_bounds__(256) k_oz_split_c(int n, int o, const double2* __restrict__ mo,
                                                    __nv_bfloat16* __restrict__ B, int* __restrict__ fa, int K) {
    __shared__ int s_e;
    const int row = blockIdx.x, a = row >> 3, d = (row & 7) + 2;
    if (threadIdx.x == 0) s_e = 0;
    __syncthreads();
    if (a < o)
        for (int i = threadIdx.x; i < n; i += blockDim.x) atomicMax(&s_e, oz_ebits(mo[(size_t)i * o + a].x));
    __syncthreads();
    const int F = s_e - 1020;
    if (threadIdx.x == 0 && (row & 7) == 0 && a < o) fa[a] = F;
    // B[(a, d)][8 i + s - 1] = c_{d - s}[i][a] for 1 <= d - s <= 7
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const int i = k >> 3, s = (k & 7) + 1, t = d - s;
        int v = 0;
        if (a < o && i < n && s <= 7 && t >= 1 && t <= 7) v = oz_digit(mo[(size_t)i * o + a].x, F, t);
        B[(size_t)row * K + k] = __float2bfloat16((float)v);
    }
}

constexpr int OZ_BM = 128;               // A rows a tile: two walkers of 64 rows (2 b + part, b < 32)
constexpr int OZ_THREADS = 26 * 32;      // warp 0: copies, 1: MMA, 2-17: digits, 18-21: epilogue, 22-25: E_r
constexpr int OZ_PW0 = 2, OZ_EW0 = 18, OZ_XW0 = 22;  // first producer / epilogue / exponent warp
constexpr int OZ_PWARPS = OZ_EW0 - OZ_PW0;
constexpr int OZ_STG = 4;
constexpr int OZ_A_BYTES = OZ_BM * 64 * 2;
constexpr int OZ_SLOT_COLS = 256;        // tensor-memory columns between the two accumulators
// dynamic shared memory of the largest layout (nocc 32: B 32 KB, walker rows 8 KB a stage), beside ~1 KB static
constexpr int OZ_SMEM_MAX = OZ_STG * (OZ_A_BYTES + 32 * 1024 + 8 * 1024) + 1024 + 256;

struct OzGeo {
    int b_bytes, w_bytes, stage, smem;
};
__host__ __device__ inline OzGeo oz_geo(int o) {
    OzGeo g;
    g.b_bytes = 8 * (o + (o & 1)) * 128;             // NB rows of 64 bf16
    g.w_bytes = (2 * 8 * o * 16 + 1023) / 1024 * 1024;  // two walkers' eight orbital rows
    g.stage = OZ_A_BYTES + g.b_bytes + g.w_bytes;
    g.smem = OZ_STG * g.stage + 1024 + 256;
    return g;
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"((unsigned long long)src), "r"(bytes), "r"(bar)
                 : "memory");
}
// L2 prefetch of bytes at src (16-byte aligned, a multiple of 16 bytes), 32 KB a request
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
    for (uint32_t off = 0; off < bytes; off += 32768u) {
        const uint32_t len = min(32768u, bytes - off);
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"((unsigned long long)src + off), "r"(len)
                     : "memory");
    }
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "r"(taddr)
        : "memory");
}

// m of walkers 2 t, 2 t + 1 for the tiles t of this CTA (persistent).
// Barriers a stage: ld_full (B tile and the walkers' rows landed), a_full
// (the producer warps wrote the A tile), empty (the MMAs that read
// the stage finished).  The row scales E_r of a tile (two above the largest
// binary64 exponent of the row, OZ_NONFINITE for a row holding inf or nan)
// are found by four warps a tile ahead, into one of two shared slots: e_full
// (written), e_empty (the producers and the epilogue have read them).
// Every wait is bounded; on a timeout the CTA raises *err and every role
// unwinds (the copy thread waits, bounded, for its copies, the MMA thread
// for its MMAs before the tensor memory is freed).
__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_oz_m(const __grid_constant__ CUtensorMap tmB, int W, int n, int o, const double2* __restrict__ walkers,
           const int* __restrict__ fa, float2* __restrict__ mout, int* __restrict__ err) {
    using namespace tc;
    const OzGeo geo = oz_geo(o);
    const int NB = 8 * (o + (o & 1)), nks = (n + 7) / 8, ntiles = (W + 1) / 2;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = (uint64_t*)(smem + OZ_STG * geo.stage);
    uint32_t* tmem_slot = (uint32_t*)(bars + 3 * OZ_STG + 4 + 1 + 4);
    volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
    __shared__ int s_fa[32];
    __shared__ int s_er[2][OZ_BM];
    const uint32_t ldf0 = smem_u32(bars), af0 = smem_u32(bars + OZ_STG), emp0 = smem_u32(bars + 2 * OZ_STG);
    const uint32_t tfull0 = smem_u32(bars + 3 * OZ_STG), tempty0 = smem_u32(bars + 3 * OZ_STG + 2);
    const uint32_t drain = smem_u32(bars + 3 * OZ_STG + 4);
    const uint32_t exf0 = smem_u32(bars + 3 * OZ_STG + 5), exe0 = smem_u32(bars + 3 * OZ_STG + 7);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < OZ_STG; ++s) {
            mbar_init(ldf0 + 8 * s, 1);
            mbar_init(af0 + 8 * s, OZ_PWARPS);  // one arrival per producer warp
            mbar_init(emp0 + 8 * s, 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(tfull0 + 8 * a, 1);
            mbar_init(tempty0 + 8 * a, 128);  // every epilogue thread
        }
        mbar_init(drain, 1);
        for (int a = 0; a < 2; ++a) {
            mbar_init(exf0 + 8 * a, OZ_THREADS / 32 - OZ_XW0);        // one arrival per exponent warp
            mbar_init(exe0 + 8 * a, OZ_PWARPS + (OZ_XW0 - OZ_EW0));  // producer and epilogue warps
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x < o) s_fa[threadIdx.x] = fa[threadIdx.x];
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(2 * OZ_SLOT_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            asm volatile("prefetch.tensormap [%0];" ::"l"((unsigned long long)&tmB) : "memory");
            int stage = 0;
            uint32_t phase = 0;
            int issued[OZ_STG];
            uint32_t issued_par[OZ_STG];
            for (int s = 0; s < OZ_STG; ++s) issued[s] = 0;
            bool ok = true;
            // the walkers' rows reach shared memory from L2: this tile's and, a tile ahead, the next one's
            if (blockIdx.x < ntiles)
                bulk_prefetch_l2(walkers + (size_t)2 * blockIdx.x * n * o,
                                 (uint32_t)(min(2, W - 2 * (int)blockIdx.x) * n * o * 16));
            for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
                const int nw = min(2, W - 2 * t);
                if (t + (int)gridDim.x < ntiles) {
                    const int tn = t + gridDim.x;
                    bulk_prefetch_l2(walkers + (size_t)2 * tn * n * o, (uint32_t)(min(2, W - 2 * tn) * n * o * 16));
                }
                for (int kk = 0; kk < nks; ++kk) {
                    if (!mbar_wait(emp0 + 8 * stage, phase ^ 1, abort_flag)) { ok = false; break; }
                    issued[stage] = 0;
                    uint8_t* st = smem + stage * geo.stage;
                    const uint32_t fb = ldf0 + 8 * stage;
                    const uint32_t rb = (uint32_t)(min(8, n - 8 * kk) * o * 16);  // one walker's rows
                    mbar_expect_tx(fb, (uint32_t)geo.b_bytes + nw * rb);
                    tma_load_2d(smem_u32(st + OZ_A_BYTES), &tmB, 64 * kk, 0, fb);
                    for (int wl = 0; wl < nw; ++wl)
                        bulk_load(smem_u32(st + OZ_A_BYTES + geo.b_bytes + wl * 8 * o * 16),
                                  walkers + ((size_t)(2 * t + wl) * n + 8 * kk) * o, rb, fb);
                    issued[stage] = 1;
                    issued_par[stage] = phase;
                    if (++stage == OZ_STG) { stage = 0; phase ^= 1; }
                }
            }
            if (!ok) {
                atomicExch(err, 1);
                *abort_flag = 1;
            }
            // every copy this thread issued lands before the CTA exits
            for (int s = 0; s < OZ_STG; ++s)
                if (issued[s]) mbar_wait(ldf0 + 8 * s, issued_par[s], nullptr);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NB >> 3) << 17) |
                                   ((uint32_t)(OZ_BM >> 4) << 24);
            int stage = 0, slot = 0;
            uint32_t phase = 0, slot_phase = 0;
            bool ok = true;
            for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
                for (int kk = 0; kk < nks; ++kk) {
                    // the producers waited for the copies of this stage before writing A
                    if (!mbar_wait_inl(af0 + 8 * stage, phase, abort_flag)) { ok = false; break; }
                    if (!mbar_wait_inl(ldf0 + 8 * stage, phase, abort_flag)) { ok = false; break; }
                    if (kk == 0 && !mbar_wait(tempty0 + 8 * slot, slot_phase ^ 1, abort_flag)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t a0 = smem_u32(smem + stage * geo.stage), b0 = a0 + OZ_A_BYTES;
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        umma_bf16_i(tmem + slot * OZ_SLOT_COLS, desc_k128(a0 + 32 * k), desc_k128(b0 + 32 * k), idesc,
                                    (kk | k) != 0);
                    umma_commit(emp0 + 8 * stage);
                    if (kk == nks - 1) {
                        umma_commit(tfull0 + 8 * slot);
                        if (++slot == 2) { slot = 0; slot_phase ^= 1; }
                    }
                    if (++stage == OZ_STG) { stage = 0; phase ^= 1; }
                }
            }
            if (!ok) {
                atomicExch(err, 1);
                *abort_flag = 1;
            }
            umma_commit(drain);
            mbar_wait(drain, 0, nullptr);
        }
    } else if (warp < OZ_EW0) {
        // producers: row r of the tile, orbitals 2 h, 2 h + 1 of each K step
        const int p = threadIdx.x - 32 * OZ_PW0, r = p & (OZ_BM - 1), h = p >> 7;
        const int wl = r >> 6, b = (r & 63) >> 1, part = r & 1;
        int stage = 0;
        uint32_t phase = 0;
        bool ok = true;
        for (int t = blockIdx.x, it = 0; ok && t < ntiles; t += gridDim.x, ++it) {
            const int w = 2 * t + wl;
            const bool valid = w < W && b < o;
            if (!mbar_wait(exf0 + 8 * (it & 1), (it >> 1) & 1, abort_flag)) {
                atomicExch(err, 1);
                *abort_flag = 1;
                break;
            }
            int E = s_er[it & 1][r];
            __syncwarp();
            if (lane == 0) mbar_arrive(exe0 + 8 * (it & 1));
            if (!valid || E == OZ_NONFINITE) E = 0;  // digits of no use: the epilogue writes nan for the row
            const int Ep = E + 1026;
            for (int kk = 0; kk < nks; ++kk) {
                if (!mbar_wait(ldf0 + 8 * stage, phase, abort_flag)) {
                    atomicExch(err, 1);
                    *abort_flag = 1;
                    ok = false;
                    break;
                }
                uint8_t* st = smem + stage * geo.stage;
                const uint2* wrow = (const uint2*)(st + OZ_A_BYTES + geo.b_bytes + wl * 8 * o * 16) + part;
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int ii = 2 * h + u;
                    const uint2 x = (valid && 8 * kk + ii < n) ? wrow[2 * (ii * o + b)] : make_uint2(0u, 0u);
                    *(uint4*)(st + r * 128 + ((ii ^ (r & 7)) << 4)) = oz_chunk(x.x, x.y, Ep);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(af0 + 8 * stage);
                if (++stage == OZ_STG) { stage = 0; phase ^= 1; }
            }
        }
    } else if (warp >= OZ_XW0) {
        // E_r of each row of the CTA's tiles, a tile ahead of the producers: row x of a tile by thread x,
        // the largest biased exponent over the walker's orbitals (8-byte loads, a warp's lanes contiguous)
        const int x = threadIdx.x - 32 * OZ_XW0, wl = x >> 6, b = (x & 63) >> 1, part = x & 1;
        for (int t = blockIdx.x, it = 0; t < ntiles; t += gridDim.x, ++it) {
            if (!mbar_wait(exe0 + 8 * (it & 1), ((it >> 1) & 1) ^ 1, abort_flag)) {
                atomicExch(err, 1);
                *abort_flag = 1;
                break;
            }
            const int w = 2 * t + wl;
            int e = 0;
            if (w < W && b < o) {
                const unsigned long long* Wq =
                    (const unsigned long long*)(walkers + (size_t)w * n * o + b) + part;
                int e1 = 0, e2 = 0, e3 = 0;
                int i = 0;
                for (; i + 4 <= n; i += 4) {
                    e = max(e, (int)((Wq[2 * (size_t)i * o] >> 52) & 0x7ffu));
                    e1 = max(e1, (int)((Wq[2 * (size_t)(i + 1) * o] >> 52) & 0x7ffu));
                    e2 = max(e2, (int)((Wq[2 * (size_t)(i + 2) * o] >> 52) & 0x7ffu));
                    e3 = max(e3, (int)((Wq[2 * (size_t)(i + 3) * o] >> 52) & 0x7ffu));
                }
                for (; i < n; ++i) e = max(e, (int)((Wq[2 * (size_t)i * o] >> 52) & 0x7ffu));
                e = max(max(e, e1), max(e2, e3));
                e = e == 0x7ff ? OZ_NONFINITE : e - 1020;
            }
            s_er[it & 1][x] = e;
            __syncwarp();
            if (lane == 0) mbar_arrive(exf0 + 8 * (it & 1));
        }
    } else {
        // epilogue: this warp's 32 rows (lane quadrant q), every trial orbital
        const int q = warp & 3;
        const int r = 32 * q + lane, wl = r >> 6, b = (r & 63) >> 1, part = r & 1;
        int slot = 0;
        uint32_t slot_phase = 0;
        for (int t = blockIdx.x, it = 0; t < ntiles; t += gridDim.x, ++it) {
            if (!mbar_wait_inl(tfull0 + 8 * slot, slot_phase, abort_flag) ||
                !mbar_wait_inl(exf0 + 8 * (it & 1), (it >> 1) & 1, abort_flag)) {
                atomicExch(err, 1);
                *abort_flag = 1;
                break;
            }
            tc_fence_after();
            const int w = 2 * t + wl;
            const bool valid = w < W && b < o;
            const int E = s_er[it & 1][r];
            __syncwarp();
            if (lane == 0) mbar_arrive(exe0 + 8 * (it & 1));
            for (int a = 0; a < o; ++a) {
                uint32_t v[8];
                __syncwarp();
                tmem_ld8(tmem + slot * OZ_SLOT_COLS + 8 * a + ((uint32_t)(32 * q) << 16), v);
                if (valid) {
                    // the terms D_d 2^(-7 d) are exact in fp32 (|D_d| < 2^24); their sum as a
                    // double-float pair by two-sums from the smallest, then scaled by 2^(E + F)
                    float sm = __uint_as_float(v[7]) * 0x1p-63f, er2 = 0.f;
#pragma unroll
                    for (int d = 8; d >= 2; --d) {
                        const float tt = __uint_as_float(v[d - 2]) * __int_as_float((127 - 7 * d) << 23);
                        const float s2 = sm + tt, bb = s2 - sm;
                        er2 += (sm - (s2 - bb)) + (tt - bb);
                        sm = s2;
                    }
                    const float hi = sm + er2, lo = er2 - (hi - sm);
                    float2 out;
                    if (E == OZ_NONFINITE) {
                        out = make_float2(__int_as_float(0x7fc00000), 0.f);
                    } else {
                        const int sc = E + s_fa[a];
                        const float p2 = (unsigned)(sc + 126) < 253u ? __int_as_float((sc + 127) << 23) : ldexpf(1.f, sc);
                        out = make_float2(hi * p2, lo * p2);
                    }
                    mout[(((size_t)w * o + a) * o + b) * 2 + part] = out;
                }
            }
            tc_fence_before();
            mbar_arrive(tempty0 + 8 * slot);
            if (++slot == 2) { slot = 0; slot_phase ^= 1; }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * OZ_SLOT_COLS)
                     : "memory");
    }
}

DeviceOnce g_oz_smem;

}  // namespace

int launch_oz_split_c(int n, int o, const double2* mo, __nv_bfloat16* B, int* fa, cudaStream_t s) {
    if (o > 32) return fail(AFQ_E_UNSUPPORTED, "ozaki m: nocc=%d > 32", o);
    const OzDims z = oz_dims(n, o);
    k_oz_split_c<<<z.NB, 256, 0, s>>>(n, o, mo, B, fa, z.K);
    AFQ_LAUNCHED("k_oz_split_c");
    return AFQ_OK;
}

int launch_oz_m(int W, int n, int o, const double2* walkers, const __nv_bfloat16* B, const int* fa, float2* m,
                int* err, cudaStream_t s) {
    using namespace tc;
    if (W <= 0) return AFQ_OK;
    if (o > 32) return fail(AFQ_E_UNSUPPORTED, "ozaki m: nocc=%d > 32", o);
    if (n > 584) return fail(AFQ_E_UNSUPPORTED, "ozaki m: norb=%d > 584 (digit sums past 2^24)", n);
    if (((uintptr_t)walkers) & 15) return fail(AFQ_E_INVALID_ARGUMENT, "ozaki m: walkers not 16-byte aligned");
    const OzDims z = oz_dims(n, o);
    const OzGeo g = oz_geo(o);
    if (g.smem > OZ_SMEM_MAX) return fail(AFQ_E_UNSUPPORTED, "ozaki m: %d bytes of shared memory", g.smem);
    AFQ_TRY(get_encode());
    CUtensorMap mb;
    AFQ_TRY(make_map(&mb, B, z.NB, z.K, z.K, z.NB));
    int sms = 0;
    AFQ_TRY(device_sms(&sms));
    AFQ_TRY(raise_smem_once(g_oz_smem, k_oz_m, OZ_SMEM_MAX));
    const int tiles = (W + 1) / 2, grid = tiles < sms ? tiles : sms;
    k_oz_m<<<grid, OZ_THREADS, g.smem, s>>>(mb, W, n, o, walkers, fa, m, err);
    AFQ_LAUNCHED("k_oz_m");
    return AFQ_OK;
}

}  // namespace afq
