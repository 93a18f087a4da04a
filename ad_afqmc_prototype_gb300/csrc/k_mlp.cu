// The exchange-energy network of the control-variate measurement: a
// multilayer perceptron F -> H -> H -> 1 with GELU activations, bf16
// weights, trained on the GPU by these kernels.
//
//   z1 = W1 x + b1,  h1 = gelu(z1),  z2 = W2 h1 + b2,  h2 = gelu(z2),
//   y  = w3 . h2 + b3,   x = (features - mean) / std (applied by the caller)
//
// Parameters live twice: an fp32 master copy (the Adam update's target) and
// the bf16 copy every forward and backward product reads.  Layout of both
// (element offsets): W1 (H x F), b1 (H), W2 (H x H), b2 (H), w3 (H), b3 (1).
// gelu(z) = z Phi(z) with the standard normal CDF Phi (erf form).
//
// Tensor cores: every product is mma.sync m16n8k16 (bf16 operands, fp32
// accumulation).  The weights are bf16 by definition; the fp32 operands
// (features, activations, their gradients) enter as two bf16 pieces, x = hi +
// lo (16 significant bits), so a weight product is two MMAs (hi, lo) and an
// activation-activation product (the weight gradients) three (hh, hl, lh):
// fp32-level sums.  One CTA takes MLP_TR = 32 rows of the batch; the forward
// keeps its activations in shared memory, the backward forms the CTA's share
// of every gradient, written to its own slot of a partial-gradient buffer;
// k_mlp_reduce_adam then adds the slots in a fixed order (a deterministic
// gradient) and applies Adam.
#include "afq_internal.cuh"

namespace afq {

constexpr int MLP_TR = 32;       // batch rows per CTA
constexpr int MLP_THREADS = 256;
constexpr int MLP_HMAX = 256;    // hidden width handled (one thread a hidden unit in the column passes)

struct MlpOff {
    size_t w1, b1, w2, b2, w3, b3, total;
};
__host__ __device__ inline MlpOff mlp_offsets(int F, int H) {
    MlpOff o;
    o.w1 = 0;
    o.b1 = o.w1 + (size_t)H * F;
    o.w2 = o.b1 + H;
    o.b2 = o.w2 + (size_t)H * H;
    o.w3 = o.b2 + H;
    o.b3 = o.w3 + H;
    o.total = o.b3 + 1;
    return o;
}

__device__ __forceinline__ float gelu_f(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// ------------------------------------------------------ mma.sync helpers --
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}
__device__ __forceinline__ uint32_t ld2(const __nv_bfloat16* p) { return *(const uint32_t*)p; }
// Fragments of m16n8k16 (g = lane / 4, t = lane % 4): A element pairs (g, 2t..),
// (g + 8, 2t..), (g, 2t + 8..), (g + 8, 2t + 8..); B pairs (k 2t.., n g), (k 2t + 8.., n g).
// A[m][k] = p[m ld + k] (row-major)
__device__ __forceinline__ void frag_a(uint32_t (&a)[4], const __nv_bfloat16* p, int ld, int m0, int k0, int lane) {
    const int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* q = p + (size_t)(m0 + g) * ld + k0 + 2 * t;
    a[0] = ld2(q);
    a[1] = ld2(q + 8 * ld);
    a[2] = ld2(q + 8);
    a[3] = ld2(q + 8 * ld + 8);
}
// A[m][k] = p[k ld + m] (stored transposed)
__device__ __forceinline__ void frag_at(uint32_t (&a)[4], const __nv_bfloat16* p, int ld, int m0, int k0, int lane) {
    const int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* q = p + (size_t)(k0 + 2 * t) * ld + m0 + g;
    a[0] = pack2(q[0], q[ld]);
    a[1] = pack2(q[8], q[ld + 8]);
    a[2] = pack2(q[8 * ld], q[9 * ld]);
    a[3] = pack2(q[8 * ld + 8], q[9 * ld + 8]);
}
// B[k][n] = p[n ld + k] (stored N x K, row-major)
__device__ __forceinline__ void frag_b(uint32_t (&b)[2], const __nv_bfloat16* p, int ld, int k0, int n0, int lane) {
    const int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* q = p + (size_t)(n0 + g) * ld + k0 + 2 * t;
    b[0] = ld2(q);
    b[1] = ld2(q + 8);
}
// B[k][n] = p[k ld + n] (stored K x N, row-major)
__device__ __forceinline__ void frag_bt(uint32_t (&b)[2], const __nv_bfloat16* p, int ld, int k0, int n0, int lane) {
    const int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* q = p + (size_t)(k0 + 2 * t) * ld + n0 + g;
    b[0] = pack2(q[0], q[ld]);
    b[1] = pack2(q[8 * ld], q[9 * ld]);
}
// x = hi + lo as two bf16 pieces
__device__ __forceinline__ void split_bf(float x, __nv_bfloat16& h, __nv_bfloat16& l) {
    h = __float2bfloat16(x);
    l = __float2bfloat16(x - __bfloat162float(h));
}

// Shared memory of one CTA (TR rows): features (hi, lo), z1 (fp32; dz1 in
// place), h1 (hi, lo; dz1's pieces after the W2 gradient), z2 (fp32; dz2 in
// place), dz2 (hi, lo), per-row outputs.
struct MlpSmem {
    __nv_bfloat16 *xh, *xl, *h1h, *h1l, *d2h, *d2l;
    float *z1, *z2, *y, *d;
    int ldx, ldh;
};
__host__ __device__ inline size_t mlp_smem_bytes(int F, int H) {
    return (size_t)MLP_TR * (2 * F + 4 * H) * sizeof(__nv_bfloat16) + (size_t)MLP_TR * (2 * H + 2) * sizeof(float);
}
__device__ inline MlpSmem mlp_smem(uint8_t* base, int F, int H) {
    MlpSmem m;
    float* fp = (float*)base;
    m.z1 = fp;
    m.z2 = fp + MLP_TR * H;
    m.y = fp + 2 * MLP_TR * H;
    m.d = m.y + MLP_TR;
    __nv_bfloat16* bp = (__nv_bfloat16*)(m.d + MLP_TR);
    m.xh = bp;
    m.xl = bp + MLP_TR * F;
    m.h1h = bp + 2 * MLP_TR * F;
    m.h1l = m.h1h + MLP_TR * H;
    m.d2h = m.h1l + MLP_TR * H;
    m.d2l = m.d2h + MLP_TR * H;
    m.ldx = F;
    m.ldh = H;
    return m;
}

// Forward of the CTA's rows: z1, h1 (pieces), z2 into shared memory, y into
// sm.y.  Output tiles (16 rows x 8 units): warp w takes row block w % 2 and
// unit blocks w / 2, w / 2 + 4, ...
__device__ void mlp_forward_tile(const MlpSmem& sm, int F, int H, const __nv_bfloat16* __restrict__ p, const MlpOff& off,
                                 int rows) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int m0 = (warp & 1) * 16;
    // z1 = x W1^T + b1 (B[k][j] = W1[j][k], stored H x F)
    for (int nb = warp >> 1; nb < H / 8; nb += 4) {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int k0 = 0; k0 < F; k0 += 16) {
            uint32_t ah[4], al[4], b[2];
            frag_a(ah, sm.xh, sm.ldx, m0, k0, lane);
            frag_a(al, sm.xl, sm.ldx, m0, k0, lane);
            frag_b(b, p + off.w1, F, k0, nb * 8, lane);
            mma_bf16(acc, ah, b);
            mma_bf16(acc, al, b);
        }
        const int j = nb * 8 + 2 * t;
        const float b0 = __bfloat162float(p[off.b1 + j]), b1 = __bfloat162float(p[off.b1 + j + 1]);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r = m0 + g + 8 * h;
            const float za = acc[2 * h] + b0, zb = acc[2 * h + 1] + b1;
            sm.z1[r * H + j] = za;
            sm.z1[r * H + j + 1] = zb;
            __nv_bfloat16 hh, hl;
            split_bf(gelu_f(za), hh, hl);
            sm.h1h[r * H + j] = hh;
            sm.h1l[r * H + j] = hl;
            split_bf(gelu_f(zb), hh, hl);
            sm.h1h[r * H + j + 1] = hh;
            sm.h1l[r * H + j + 1] = hl;
        }
    }
    __syncthreads();
    // z2 = h1 W2^T + b2 (B[j][k] = W2[k][j], stored H x H)
    for (int nb = warp >> 1; nb < H / 8; nb += 4) {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int k0 = 0; k0 < H; k0 += 16) {
            uint32_t ah[4], al[4], b[2];
            frag_a(ah, sm.h1h, sm.ldh, m0, k0, lane);
            frag_a(al, sm.h1l, sm.ldh, m0, k0, lane);
            frag_b(b, p + off.w2, H, k0, nb * 8, lane);
            mma_bf16(acc, ah, b);
            mma_bf16(acc, al, b);
        }
        const int j = nb * 8 + 2 * t;
        const float b0 = __bfloat162float(p[off.b2 + j]), b1 = __bfloat162float(p[off.b2 + j + 1]);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r = m0 + g + 8 * h;
            sm.z2[r * H + j] = acc[2 * h] + b0;
            sm.z2[r * H + j + 1] = acc[2 * h + 1] + b1;
        }
    }
    __syncthreads();
    // y = w3 . gelu(z2) + b3: eight threads a row, H / 8 units each, then a
    // fixed-order shuffle sum
    {
        const int r = threadIdx.x >> 3, q = threadIdx.x & 7, per = H / 8;
        float v = 0.f;
        for (int j = q * per; j < (q + 1) * per; ++j) v = fmaf(__bfloat162float(p[off.w3 + j]), gelu_f(sm.z2[r * H + j]), v);
        v += __shfl_xor_sync(0xffffffffu, v, 1);
        v += __shfl_xor_sync(0xffffffffu, v, 2);
        v += __shfl_xor_sync(0xffffffffu, v, 4);
        if (q == 0) sm.y[r] = r < rows ? v + __bfloat162float(p[off.b3]) : 0.f;
    }
    __syncthreads();
}

// Rows [r0, r0 + rows) of x into the pieces; rows past the batch are zero.
__device__ __forceinline__ void mlp_load_x(const MlpSmem& sm, int F, const float* __restrict__ x, int r0, int rows) {
    for (int e = threadIdx.x; e < MLP_TR * F; e += blockDim.x) {
        const int r = e / F;
        const float v = r < rows ? x[(size_t)(r0 + r) * F + e % F] : 0.f;
        __nv_bfloat16 h, l;
        split_bf(v, h, l);
        sm.xh[e] = h;
        sm.xl[e] = l;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(MLP_THREADS) k_mlp_forward(int B, int F, int H, const __nv_bfloat16* __restrict__ p,
                                                             const float* __restrict__ x, float* __restrict__ y) {
    extern __shared__ __align__(16) uint8_t mlp_raw[];
    const MlpSmem sm = mlp_smem(mlp_raw, F, H);
    const MlpOff off = mlp_offsets(F, H);
    const int r0 = blockIdx.x * MLP_TR, rows = min(MLP_TR, B - r0);
    mlp_load_x(sm, F, x, r0, rows);
    mlp_forward_tile(sm, F, H, p, off, rows);
    if (threadIdx.x < rows) y[r0 + threadIdx.x] = sm.y[threadIdx.x];
}

// Forward and backward of the CTA's rows for the loss mean (y - t)^2 / 2 over
// the batch of B rows: the CTA's share of the gradient (every parameter) to
// part[blockIdx.x P ...], of the loss to lpart[blockIdx.x].
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_grad_tile(int B, int F, int H, const __nv_bfloat16* __restrict__ p,
                                                               const float* __restrict__ x, const float* __restrict__ tgt,
                                                               float* __restrict__ part, float* __restrict__ lpart) {
    extern __shared__ __align__(16) uint8_t mlp_raw[];
    const MlpSmem sm = mlp_smem(mlp_raw, F, H);
    const MlpOff off = mlp_offsets(F, H);
    const int r0 = blockIdx.x * MLP_TR, rows = min(MLP_TR, B - r0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float* gp = part + (size_t)blockIdx.x * off.total;
    mlp_load_x(sm, F, x, r0, rows);
    mlp_forward_tile(sm, F, H, p, off, rows);
    // d_r = (y_r - t_r) / B; the CTA's loss share and db3
    if (threadIdx.x < MLP_TR) {
        const int r = threadIdx.x;
        const float e = r < rows ? sm.y[r] - tgt[r0 + r] : 0.f;
        sm.d[r] = e / (float)B;
        sm.y[r] = 0.5f * e * e / (float)B;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float l = 0.f, db = 0.f;
        for (int r = 0; r < MLP_TR; ++r) {
            l += sm.y[r];
            db += sm.d[r];
        }
        lpart[blockIdx.x] = l;
        gp[off.b3] = db;
    }
    // unit j: dw3_j = sum_r d_r h2[r, j]; dz2[r, j] = d_r w3_j gelu'(z2[r, j]) (fp32 in place of
    // z2, and as pieces); db2_j = sum_r dz2[r, j]
    for (int j = threadIdx.x; j < H; j += blockDim.x) {
        const float w3 = __bfloat162float(p[off.w3 + j]);
        float gw3 = 0.f, gb2 = 0.f;
        for (int r = 0; r < MLP_TR; ++r) {
            const float z = sm.z2[r * H + j], dr = sm.d[r];
            gw3 = fmaf(dr, gelu_f(z), gw3);
            const float dz = dr * w3 * gelu_d(z);
            sm.z2[r * H + j] = dz;
            __nv_bfloat16 h, l;
            split_bf(dz, h, l);
            sm.d2h[r * H + j] = h;
            sm.d2l[r * H + j] = l;
            gb2 += dz;
        }
        gp[off.w3 + j] = gw3;
        gp[off.b2 + j] = gb2;
    }
    __syncthreads();
    // dW2[j][k] = sum_r dz2[r][j] h1[r][k]: A[j][r] = dz2 (stored [r][j]), B[r][k] = h1 (stored [r][k])
    for (int tile = warp; tile < (H / 16) * (H / 8); tile += MLP_THREADS / 32) {
        const int jb = tile / (H / 8), kb = tile % (H / 8);
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int k0 = 0; k0 < MLP_TR; k0 += 16) {
            uint32_t ah[4], al[4], bh[2], bl[2];
            frag_at(ah, sm.d2h, H, jb * 16, k0, lane);
            frag_at(al, sm.d2l, H, jb * 16, k0, lane);
            frag_bt(bh, sm.h1h, H, k0, kb * 8, lane);
            frag_bt(bl, sm.h1l, H, k0, kb * 8, lane);
            mma_bf16(acc, ah, bh);
            mma_bf16(acc, ah, bl);
            mma_bf16(acc, al, bh);
        }
        float* dst = gp + off.w2 + (size_t)(jb * 16 + g) * H + kb * 8 + 2 * t;
        dst[0] = acc[0];
        dst[1] = acc[1];
        dst[8 * H] = acc[2];
        dst[8 * H + 1] = acc[3];
    }
    // dh1[r][k] = sum_j dz2[r][j] W2[j][k] (B stored [j][k]); dz1 = dh1 gelu'(z1), fp32 in place of z1
    {
        const int m0 = (warp & 1) * 16;
        for (int nb = warp >> 1; nb < H / 8; nb += 4) {
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            for (int k0 = 0; k0 < H; k0 += 16) {
                uint32_t ah[4], al[4], b[2];
                frag_a(ah, sm.d2h, H, m0, k0, lane);
                frag_a(al, sm.d2l, H, m0, k0, lane);
                frag_bt(b, p + off.w2, H, k0, nb * 8, lane);
                mma_bf16(acc, ah, b);
                mma_bf16(acc, al, b);
            }
            const int k = nb * 8 + 2 * t;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = m0 + g + 8 * h;
                sm.z1[r * H + k] = acc[2 * h] * gelu_d(sm.z1[r * H + k]);
                sm.z1[r * H + k + 1] = acc[2 * h + 1] * gelu_d(sm.z1[r * H + k + 1]);
            }
        }
    }
    __syncthreads();  // dW2 has read h1's pieces; dz1 is complete
    // unit k: db1_k = sum_r dz1[r][k]; dz1's pieces over h1's
    for (int k = threadIdx.x; k < H; k += blockDim.x) {
        float gb1 = 0.f;
        for (int r = 0; r < MLP_TR; ++r) {
            const float dz = sm.z1[r * H + k];
            gb1 += dz;
            __nv_bfloat16 h, l;
            split_bf(dz, h, l);
            sm.h1h[r * H + k] = h;
            sm.h1l[r * H + k] = l;
        }
        gp[off.b1 + k] = gb1;
    }
    __syncthreads();
    // dW1[j][k] = sum_r dz1[r][j] x[r][k]
    for (int tile = warp; tile < (H / 16) * (F / 8); tile += MLP_THREADS / 32) {
        const int jb = tile / (F / 8), kb = tile % (F / 8);
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int k0 = 0; k0 < MLP_TR; k0 += 16) {
            uint32_t ah[4], al[4], bh[2], bl[2];
            frag_at(ah, sm.h1h, H, jb * 16, k0, lane);
            frag_at(al, sm.h1l, H, jb * 16, k0, lane);
            frag_bt(bh, sm.xh, F, k0, kb * 8, lane);
            frag_bt(bl, sm.xl, F, k0, kb * 8, lane);
            mma_bf16(acc, ah, bh);
            mma_bf16(acc, ah, bl);
            mma_bf16(acc, al, bh);
        }
        float* dst = gp + off.w1 + (size_t)(jb * 16 + g) * F + kb * 8 + 2 * t;
        dst[0] = acc[0];
        dst[1] = acc[1];
        dst[8 * F] = acc[2];
        dst[8 * F + 1] = acc[3];
    }
}

// Gradient = the tiles' partial gradients added in tile order (one thread a
// parameter: deterministic), loss likewise; then, if w is given, Adam
// (bias-corrected) on the fp32 master copy and its bf16 copy.
__global__ void k_mlp_reduce_adam(size_t n, int ntile, const float* __restrict__ part, const float* __restrict__ lpart,
                                  float* __restrict__ g_out, float* __restrict__ loss_out, float* __restrict__ w,
                                  __nv_bfloat16* __restrict__ wb, float* __restrict__ m, float* __restrict__ v, float lr,
                                  float b1, float b2, float eps, float c1, float c2) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && loss_out) {
        float l = 0.f;
        for (int k = 0; k < ntile; ++k) l += lpart[k];
        *loss_out = l;
    }
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        float gg = 0.f;
        for (int k = 0; k < ntile; ++k) gg += part[(size_t)k * n + e];
        if (g_out) g_out[e] = gg;
        if (!w) continue;
        const float mm = b1 * m[e] + (1.f - b1) * gg;
        const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
        m[e] = mm;
        v[e] = vv;
        const float upd = lr * (mm / c1) / (sqrtf(vv / c2) + eps);
        const float nw = w[e] - upd;
        w[e] = nw;
        wb[e] = __float2bfloat16(nw);
    }
}

__global__ void k_f32_to_bf16(size_t n, const float* __restrict__ w, __nv_bfloat16* __restrict__ wb) {
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
        wb[e] = __float2bfloat16(w[e]);
}

size_t mlp_param_count(int F, int H) { return mlp_offsets(F, H).total; }

bool mlp_shape_supported(int F, int H) {
    return F >= 16 && F % 16 == 0 && H >= 32 && H % 32 == 0 && H <= MLP_HMAX &&
           mlp_smem_bytes(F, H) <= 200 * 1024;
}

int launch_mlp_forward(int B, int F, int H, const __nv_bfloat16* p, const float* x, float* y, cudaStream_t s) {
    if (B <= 0) return AFQ_OK;
    if (!mlp_shape_supported(F, H)) return fail(AFQ_E_UNSUPPORTED, "mlp: F=%d H=%d", F, H);
    const size_t smem = mlp_smem_bytes(F, H);
    if (smem > 32 * 1024)  // with the kernel's static shared memory the default limit is below 48 KB
        AFQ_CUDA(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_mlp_forward<<<(B + MLP_TR - 1) / MLP_TR, MLP_THREADS, smem, s>>>(B, F, H, p, x, y);
    AFQ_LAUNCHED("k_mlp_forward");
    return AFQ_OK;
}

size_t mlp_train_ws_floats(int B, int F, int H) {
    const size_t nt = (size_t)(B + MLP_TR - 1) / MLP_TR;
    return nt * mlp_param_count(F, H) + nt;
}

// Gradient (and loss) of a batch; with w given, the Adam step as well.
// ws: tiles x P partial gradients, then tiles partial losses (floats).
int launch_mlp_grad_adam(int B, int F, int H, const __nv_bfloat16* wb_in, const float* x, const float* t, float* ws,
                         float* g_out, float* loss_out, float* w, __nv_bfloat16* wb, float* m, float* v, float lr,
                         int step, cudaStream_t s) {
    if (B <= 0) return AFQ_OK;
    if (!mlp_shape_supported(F, H)) return fail(AFQ_E_UNSUPPORTED, "mlp: F=%d H=%d", F, H);
    const MlpOff off = mlp_offsets(F, H);
    const int nt = (B + MLP_TR - 1) / MLP_TR;
    float* part = ws;
    float* lpart = ws + (size_t)nt * off.total;
    const size_t smem = mlp_smem_bytes(F, H);
    if (smem > 32 * 1024)  // with the kernel's static shared memory the default limit is below 48 KB
        AFQ_CUDA(cudaFuncSetAttribute(k_mlp_grad_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_mlp_grad_tile<<<nt, MLP_THREADS, smem, s>>>(B, F, H, wb_in, x, t, part, lpart);
    AFQ_LAUNCHED("k_mlp_grad_tile");
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)(step > 0 ? step : 1)), c2 = 1.f - powf(b2, (float)(step > 0 ? step : 1));
    k_mlp_reduce_adam<<<(unsigned)((off.total + 255) / 256), 256, 0, s>>>(off.total, nt, part, lpart, g_out, loss_out, w,
                                                                           wb, m, v, lr, b1, b2, 1e-8f, c1, c2);
    AFQ_LAUNCHED("k_mlp_reduce_adam");
    return AFQ_OK;
}

int launch_mlp_sync_bf16(size_t n, const float* w, __nv_bfloat16* wb, cudaStream_t s) {
    k_f32_to_bf16<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, w, wb);
    AFQ_LAUNCHED("k_f32_to_bf16");
    return AFQ_OK;
}

}  // namespace afq
