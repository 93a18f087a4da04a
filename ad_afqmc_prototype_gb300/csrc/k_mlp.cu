// The exchange-energy network of the control-variate measurement: a
// multilayer perceptron F -> H -> H -> 1 with GELU activations, bf16
// weights and fp32 arithmetic, trained on the GPU by these kernels.
//
//   z1 = W1 x + b1,  h1 = gelu(z1),  z2 = W2 h1 + b2,  h2 = gelu(z2),
//   y  = w3 . h2 + b3,   x = (features - mean) / std (applied by the caller)
//
// Parameters live twice: an fp32 master copy (the Adam update's target) and
// the bf16 copy every forward and backward product reads.  Layout of both
// (element offsets): W1 (H x F), b1 (H), W2 (H x H), b2 (H), w3 (H), b3 (1).
// gelu(z) = z Phi(z) with the standard normal CDF Phi (erf form).
#include "afq_internal.cuh"

namespace afq {

constexpr int MLP_ROWS = 32;  // batch rows per CTA of the forward kernel

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

// Forward pass of MLP_ROWS rows per CTA, H threads (thread j = hidden unit j).
// act (optional, training): z1, z2, h1, h2 per row (4 H floats each).
__global__ void k_mlp_forward(int B, int F, int H, const __nv_bfloat16* __restrict__ p, const float* __restrict__ x,
                              float* __restrict__ y, float* __restrict__ act) {
    extern __shared__ float ms[];
    float* xs = ms;                        // MLP_ROWS x F
    float* hs = xs + MLP_ROWS * F;         // MLP_ROWS x H (h1, then h2)
    __shared__ float red[MLP_ROWS][33];
    const MlpOff off = mlp_offsets(F, H);
    const int r0 = blockIdx.x * MLP_ROWS, j = threadIdx.x;
    const int rows = min(MLP_ROWS, B - r0);
    for (int e = threadIdx.x; e < MLP_ROWS * F; e += blockDim.x) {
        const int r = e / F;
        xs[e] = r < rows ? x[(size_t)(r0 + r) * F + e % F] : 0.f;
    }
    __syncthreads();
    float acc[MLP_ROWS];
    // layer 1
    {
        const float b = __bfloat162float(p[off.b1 + j]);
#pragma unroll
        for (int r = 0; r < MLP_ROWS; ++r) acc[r] = b;
        for (int k = 0; k < F; ++k) {
            const float wv = __bfloat162float(p[off.w1 + (size_t)j * F + k]);
#pragma unroll
            for (int r = 0; r < MLP_ROWS; ++r) acc[r] = fmaf(wv, xs[r * F + k], acc[r]);
        }
#pragma unroll
        for (int r = 0; r < MLP_ROWS; ++r) {
            const float h = gelu_f(acc[r]);
            hs[r * H + j] = h;
            if (act && r < rows) {
                act[(size_t)(r0 + r) * 4 * H + j] = acc[r];
                act[(size_t)(r0 + r) * 4 * H + 2 * H + j] = h;
            }
        }
    }
    __syncthreads();
    // layer 2
    {
        const float b = __bfloat162float(p[off.b2 + j]);
#pragma unroll
        for (int r = 0; r < MLP_ROWS; ++r) acc[r] = b;
        for (int k = 0; k < H; ++k) {
            const float wv = __bfloat162float(p[off.w2 + (size_t)j * H + k]);
#pragma unroll
            for (int r = 0; r < MLP_ROWS; ++r) acc[r] = fmaf(wv, hs[r * H + k], acc[r]);
        }
    }
    __syncthreads();  // every thread is done reading h1
    const float w3 = __bfloat162float(p[off.w3 + j]);
#pragma unroll
    for (int r = 0; r < MLP_ROWS; ++r) {
        const float h = gelu_f(acc[r]);
        if (act && r < rows) {
            act[(size_t)(r0 + r) * 4 * H + H + j] = acc[r];
            act[(size_t)(r0 + r) * 4 * H + 3 * H + j] = h;
        }
        acc[r] = w3 * h;  // this unit's share of y
    }
    // y = sum_j w3_j h2_j + b3: warp sums, then across warps
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int r = 0; r < MLP_ROWS; ++r) {
        float v = acc[r];
#pragma unroll
        for (int o2 = 16; o2 > 0; o2 >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o2);
        if (lane == 0) red[r][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < rows) {
        float v = __bfloat162float(p[off.b3]);
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) v += red[threadIdx.x][q];
        y[r0 + threadIdx.x] = v;
    }
}

// Loss L = mean (y - t)^2 / 2.  dz2[r, j] = (y_r - t_r) / B * w3_j * gelu'(z2),
// gradients of w3 and b3 accumulated (the caller zeroes g first).
__global__ void k_mlp_out_grad(int B, int F, int H, const __nv_bfloat16* __restrict__ p, const float* __restrict__ y,
                               const float* __restrict__ t, const float* __restrict__ act, float* __restrict__ dz2,
                               float* __restrict__ g, float* __restrict__ loss) {
    const MlpOff off = mlp_offsets(F, H);
    const int j = threadIdx.x;
    float gw3 = 0.f, gb3 = 0.f, l = 0.f;
    for (int r = blockIdx.x; r < B; r += gridDim.x) {
        const float d = (y[r] - t[r]) / (float)B;
        const float* a = act + (size_t)r * 4 * H;
        gw3 = fmaf(d, a[3 * H + j], gw3);
        dz2[(size_t)r * H + j] = d * __bfloat162float(p[off.w3 + j]) * gelu_d(a[H + j]);
        if (j == 0) {
            gb3 += d;
            l += 0.5f * (y[r] - t[r]) * (y[r] - t[r]) / (float)B;
        }
    }
    atomicAdd(g + off.w3 + j, gw3);
    if (j == 0) {
        atomicAdd(g + off.b3, gb3);
        atomicAdd(loss, l);
    }
}

// dz1[r, k] = (sum_j dz2[r, j] W2[j, k]) gelu'(z1[r, k]): one CTA per row,
// thread k.
__global__ void k_mlp_hidden_grad(int B, int F, int H, const __nv_bfloat16* __restrict__ p,
                                  const float* __restrict__ dz2, const float* __restrict__ act,
                                  float* __restrict__ dz1) {
    extern __shared__ float d2[];
    const MlpOff off = mlp_offsets(F, H);
    const int r = blockIdx.x, k = threadIdx.x;
    d2[k] = dz2[(size_t)r * H + k];
    __syncthreads();
    float s = 0.f;
    for (int j = 0; j < H; ++j) s = fmaf(d2[j], __bfloat162float(p[off.w2 + (size_t)j * H + k]), s);
    dz1[(size_t)r * H + k] = s * gelu_d(act[(size_t)r * 4 * H + k]);
}

// Weight and bias gradients of a layer: gW[j, k] += sum_r dz[r, j] in[r, k],
// gb[j] += sum_r dz[r, j].  in[r, k] = src[r * ld + off + k].  One CTA per
// 16 x 16 tile of gW (and, in the first column of tiles, the bias).
__global__ void k_mlp_weight_grad(int B, int J, int K, const float* __restrict__ dz, const float* __restrict__ src,
                                  long long ld, long long soff, float* __restrict__ gW, float* __restrict__ gb) {
    __shared__ float a[16][17], b[16][17];
    const int j0 = blockIdx.y * 16, k0 = blockIdx.x * 16, tj = threadIdx.y, tk = threadIdx.x;
    float s = 0.f, sb = 0.f;
    for (int r0 = 0; r0 < B; r0 += 16) {
        const int ra = r0 + tk, rb = r0 + tj;
        a[tj][tk] = (ra < B && j0 + tj < J) ? dz[(size_t)ra * J + j0 + tj] : 0.f;    // a[j][r]
        b[tj][tk] = (rb < B && k0 + tk < K) ? src[(size_t)rb * ld + soff + k0 + tk] : 0.f;  // b[r][k]
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            s = fmaf(a[tj][q], b[q][tk], s);
            sb += a[tj][q];
        }
        __syncthreads();
    }
    if (j0 + tj < J && k0 + tk < K) gW[(size_t)(j0 + tj) * K + k0 + tk] += s;
    if (blockIdx.x == 0 && tk == 0 && j0 + tj < J) gb[j0 + tj] += sb;
}

// Adam (bias-corrected) on the fp32 master copy, then the bf16 copy.
__global__ void k_mlp_adam(size_t n, float* __restrict__ w, __nv_bfloat16* __restrict__ wb, const float* __restrict__ g,
                           float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2, float eps,
                           float c1, float c2) {
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const float gg = g[e];
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

int launch_mlp_forward(int B, int F, int H, const __nv_bfloat16* p, const float* x, float* y, float* act,
                       cudaStream_t s) {
    if (B <= 0) return AFQ_OK;
    const size_t smem = (size_t)MLP_ROWS * (F + H) * sizeof(float);
    if (smem > 48 * 1024) AFQ_CUDA(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        (int)smem));
    k_mlp_forward<<<(B + MLP_ROWS - 1) / MLP_ROWS, H, smem, s>>>(B, F, H, p, x, y, act);
    AFQ_LAUNCHED("k_mlp_forward");
    return AFQ_OK;
}

// One training step on a batch: forward (activations kept), backward, Adam.
// ws: 4 B H (activations) + 2 B H (dz2, dz1) + B (y) + P (gradients) + 1 (loss) floats.
int launch_mlp_train_step(int B, int F, int H, float* w, __nv_bfloat16* wb, float* m, float* v, const float* x,
                          const float* t, float lr, int step, float* ws, float* loss_out, cudaStream_t s) {
    const MlpOff off = mlp_offsets(F, H);
    float* act = ws;
    float* dz2 = act + (size_t)4 * B * H;
    float* dz1 = dz2 + (size_t)B * H;
    float* y = dz1 + (size_t)B * H;
    float* g = y + B;
    float* loss = g + off.total;
    AFQ_CUDA(cudaMemsetAsync(g, 0, (off.total + 1) * sizeof(float), s));
    AFQ_TRY(launch_mlp_forward(B, F, H, wb, x, y, act, s));
    k_mlp_out_grad<<<B < 1024 ? B : 1024, H, 0, s>>>(B, F, H, wb, y, t, act, dz2, g, loss);
    AFQ_LAUNCHED("k_mlp_out_grad");
    // layer 2: gW2 = dz2^T h1, gb2; then dz1
    k_mlp_weight_grad<<<dim3((H + 15) / 16, (H + 15) / 16), dim3(16, 16), 0, s>>>(B, H, H, dz2, act, 4LL * H, 2LL * H,
                                                                                 g + off.w2, g + off.b2);
    AFQ_LAUNCHED("k_mlp_weight_grad");
    k_mlp_hidden_grad<<<B, H, H * sizeof(float), s>>>(B, F, H, wb, dz2, act, dz1);
    AFQ_LAUNCHED("k_mlp_hidden_grad");
    // layer 1: gW1 = dz1^T x, gb1
    k_mlp_weight_grad<<<dim3((F + 15) / 16, (H + 15) / 16), dim3(16, 16), 0, s>>>(B, H, F, dz1, x, F, 0, g + off.w1,
                                                                                 g + off.b1);
    AFQ_LAUNCHED("k_mlp_weight_grad");
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_mlp_adam<<<(unsigned)((off.total + 255) / 256), 256, 0, s>>>(off.total, w, wb, g, m, v, lr, b1, b2, 1e-8f, c1,
                                                                    c2);
    AFQ_LAUNCHED("k_mlp_adam");
    if (loss_out) AFQ_CUDA(cudaMemcpyAsync(loss_out, loss, sizeof(float), cudaMemcpyDeviceToDevice, s));
    return AFQ_OK;
}

int launch_mlp_sync_bf16(size_t n, const float* w, __nv_bfloat16* wb, cudaStream_t s) {
    k_f32_to_bf16<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, w, wb);
    AFQ_LAUNCHED("k_f32_to_bf16");
    return AFQ_OK;
}

}  // namespace afq
