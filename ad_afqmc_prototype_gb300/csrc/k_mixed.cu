// Kernels of the mixed-precision step (AFQ_PREC_MIXED).
//
// Precision plan: the V-build, force-bias and energy contractions run on
// tensor cores (k_tc_gemm.cu) with bf16 hi/lo split operands and fp32
// accumulation (~2^-17 relative); the Taylor series multiplies in fp32 but
// adds every term into binary64 walkers, and applies E_half as
// W + (E_half - I) W with the small correction in fp32, so the walkers carry
// binary64 and do not drift; overlaps (det), QR, weights, the phaseless
// cut and every energy accumulator stay binary64.
#include "afq_internal.cuh"

namespace afq {

// ------------------------------------------------------ operand preparation
// dst row r (Kt entries): sections at 0, S, 2S of split(src(r, k)), k < K;
// entries [3S, Kt) and [K, S) of each section are zero.
// src(r, k) = src[r * rs + k * ks].
__global__ void k_split_rows(long long rows, int K, int S, int Kt, const double* __restrict__ src, long long rs,
                             long long ks, __nv_bfloat16* __restrict__ dst, int left) {
    const long long total = rows * (long long)Kt;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long r = e % rows;  // rows fastest: coalesced reads of column-major sources
        const int kk = (int)(e / rows);
        __nv_bfloat16* row = dst + r * Kt;
        if (kk < S) {
            const double x = kk < K ? src[r * rs + (long long)kk * ks] : 0.0;
            split_store3(row, S, kk, x, left != 0);
        } else if (kk >= 3 * S) {
            row[kk] = __double2bfloat16(0.0);
        }
    }
}

int launch_split_rows(long long rows, int K, int S, int Kt, const double* src, long long rs, long long ks,
                      __nv_bfloat16* dst, int left, cudaStream_t s) {
    const long long total = rows * (long long)Kt;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    k_split_rows<<<(unsigned)blocks, 256, 0, s>>>(rows, K, S, Kt, src, rs, ks, dst, left);
    AFQ_LAUNCHED("k_split_rows");
    return AFQ_OK;
}

// E_half - I in fp32 (the one-body correction applied in the mixed Taylor kernel)
__global__ void k_e_minus_i(int n, const double* __restrict__ E, float* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n * n) out[e] = (float)(E[e] - ((e / n == e % n) ? 1.0 : 0.0));
}

int launch_e_minus_i(int n, const double* E, float* out, cudaStream_t s) {
    k_e_minus_i<<<(n * n + 255) / 256, 256, 0, s>>>(n, E, out);
    AFQ_LAUNCHED("k_e_minus_i");
    return AFQ_OK;
}

// ------------------------------------------------------------ field shift
// As k_field_shift (prop/afqmc.py:97-101) with the force bias read from the
// tensor-core output fbm (rows w: Re, rows W + w: Im, fb = 2 fbm) and the
// shifted fields written as the split left operand of the V-build GEMM:
// per walker chunk [w0, w0 + wc) the Re rows come first, then the Im rows.
__global__ void k_field_shift_mixed(int W, int G, int Wc, double sqrt_dt, const double* __restrict__ x,
                                    const float* __restrict__ fbm, long long ldf, const double2* __restrict__ mf,
                                    __nv_bfloat16* __restrict__ av, int S, int Kt, double2* __restrict__ shift_term,
                                    double2* __restrict__ fb_term) {
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= W) return;
    const int w0 = (w / Wc) * Wc;
    const int wc = min(Wc, W - w0);
    __nv_bfloat16* re_row = av + (long long)(2 * w0 + (w - w0)) * Kt;
    __nv_bfloat16* im_row = av + (long long)(2 * w0 + wc + (w - w0)) * Kt;
    double sr = 0.0, si = 0.0, br = 0.0, bi = 0.0;
    for (int g = lane; g < S; g += 32) {
        if (g < G) {
            const double2 f = make_double2(2.0 * (double)fbm[(long long)w * ldf + g],
                                           2.0 * (double)fbm[(long long)(W + w) * ldf + g]);
            const double2 m = mf[g];
            const double xv = x[(size_t)w * G + g];
            const double2 fs = make_double2(-sqrt_dt * (-f.y - m.x), -sqrt_dt * (f.x - m.y));
            const double2 xt = make_double2(xv - fs.x, -fs.y);
            split_store3(re_row, S, g, xt.x, true);
            split_store3(im_row, S, g, xt.y, true);
            sr += xt.x * m.x - xt.y * m.y;
            si += xt.x * m.y + xt.y * m.x;
            br += xv * fs.x - 0.5 * (fs.x * fs.x - fs.y * fs.y);
            bi += xv * fs.y - 0.5 * (2.0 * fs.x * fs.y);
        } else {
            split_store3(re_row, S, g, 0.0, true);
            split_store3(im_row, S, g, 0.0, true);
        }
    }
    for (int k = 3 * S + lane; k < Kt; k += 32) {
        re_row[k] = __double2bfloat16(0.0);
        im_row[k] = __double2bfloat16(0.0);
    }
    sr = warp_sum(sr); si = warp_sum(si); br = warp_sum(br); bi = warp_sum(bi);
    if (lane == 0) {
        shift_term[w] = make_double2(sr, si);
        fb_term[w] = make_double2(br, bi);
    }
}

int launch_field_shift_mixed(int W, int G, int Wc, double sqrt_dt, const double* x, const float* fbm, long long ldf,
                             const double2* mf, __nv_bfloat16* av, int S, int Kt, double2* shift_term,
                             double2* fb_term, cudaStream_t s) {
    k_field_shift_mixed<<<(W + 7) / 8, 256, 0, s>>>(W, G, Wc, sqrt_dt, x, fbm, ldf, mf, av, S, Kt, shift_term,
                                                    fb_term);
    AFQ_LAUNCHED("k_field_shift_mixed");
    return AFQ_OK;
}

// ------------------------------------------------------- Taylor propagation
// Per CTA: one walker, OC columns.  Thread tile NR rows x CC columns; the
// current Taylor term T is fp32 in shared memory, the operator (V or
// E_half - I) is streamed through shared memory BJ columns at a time, and the
// running sum lives in the binary64 output walker, which each thread updates
// only at its own entries (so walkers_out may alias walkers_in):
//   W1 = W + (E-I) W;  out = W1 + sum_k (i sqrt_dt V)^k / k! W1;
//   W' = out + (E-I) out.
constexpr int TM_THREADS = 256, TM_CC = 4, TM_BJ = 16;

template <int OC, int NR, bool REAL_M>
__device__ __forceinline__ void tm_matmul(int n, const float* __restrict__ Mr, const float* __restrict__ Mi,
                                          const float2* __restrict__ T, float2* __restrict__ Ms,
                                          float2 (&acc)[NR][TM_CC], int cg, int rg) {
    constexpr int CG = OC / TM_CC, RG = TM_THREADS / CG;
#pragma unroll
    for (int q = 0; q < NR; ++q)
#pragma unroll
        for (int j = 0; j < TM_CC; ++j) acc[q][j] = make_float2(0.f, 0.f);
    float* Msr = (float*)Ms;
    for (int j0 = 0; j0 < n; j0 += TM_BJ) {
        const int jn = min(TM_BJ, n - j0);
        for (int e = threadIdx.x; e < n * TM_BJ; e += TM_THREADS) {
            const int i = e / TM_BJ, jj = e % TM_BJ;
            const size_t src = (size_t)i * n + j0 + jj;
            if (REAL_M) Msr[e] = jj < jn ? Mr[src] : 0.f;
            else Ms[e] = jj < jn ? make_float2(Mr[src], Mi[src]) : make_float2(0.f, 0.f);
        }
        __syncthreads();
        for (int jj = 0; jj < jn; ++jj) {
            const float4* tp = (const float4*)(T + (j0 + jj) * OC + cg * TM_CC);
            const float4 t01 = tp[0], t23 = tp[1];
            const float2 t[TM_CC] = {make_float2(t01.x, t01.y), make_float2(t01.z, t01.w), make_float2(t23.x, t23.y),
                                     make_float2(t23.z, t23.w)};
#pragma unroll
            for (int q = 0; q < NR; ++q) {
                const int i = rg + RG * q;
                if (i < n) {
                    if (REAL_M) {
                        const float m = Msr[i * TM_BJ + jj];
#pragma unroll
                        for (int j = 0; j < TM_CC; ++j) {
                            acc[q][j].x = fmaf(m, t[j].x, acc[q][j].x);
                            acc[q][j].y = fmaf(m, t[j].y, acc[q][j].y);
                        }
                    } else {
                        const float2 m = Ms[i * TM_BJ + jj];
#pragma unroll
                        for (int j = 0; j < TM_CC; ++j) {
                            acc[q][j].x = fmaf(m.x, t[j].x, acc[q][j].x);
                            acc[q][j].x = fmaf(-m.y, t[j].y, acc[q][j].x);
                            acc[q][j].y = fmaf(m.x, t[j].y, acc[q][j].y);
                            acc[q][j].y = fmaf(m.y, t[j].x, acc[q][j].y);
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
}

template <int OC, int NR>
__global__ void __launch_bounds__(TM_THREADS) k_trotter_mixed(int n, int o, int n_terms, float sqrt_dt,
                                                              const float* __restrict__ emi, const float* __restrict__ vm,
                                                              long long ldv, int wc, const double2* win, double2* wout) {
    constexpr int CG = OC / TM_CC, RG = TM_THREADS / CG;
    extern __shared__ float2 smf2[];
    float2* T = smf2;                     // n x OC
    float2* Ms = smf2 + (size_t)n * OC;   // n x BJ
    const int w = blockIdx.y, c0 = blockIdx.x * OC;
    const int cg = threadIdx.x % CG, rg = threadIdx.x / CG;
    const double2* Wp = win + (size_t)w * n * o;
    double2* Wo = wout + (size_t)w * n * o;
    const float* Vr = vm + (long long)w * ldv;
    const float* Vi = vm + (long long)(wc + w) * ldv;

    for (int e = threadIdx.x; e < n * OC; e += TM_THREADS) {
        const int i = e / OC, cc = e % OC;
        if (c0 + cc < o) {
            const double2 v = Wp[(size_t)i * o + c0 + cc];
            T[e] = make_float2((float)v.x, (float)v.y);
        } else {
            T[e] = make_float2(0.f, 0.f);
        }
    }
    __syncthreads();
    float2 acc[NR][TM_CC];
    // W1 = W + (E - I) W
    tm_matmul<OC, NR, true>(n, emi, nullptr, T, Ms, acc, cg, rg);
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        const int i = rg + RG * q;
#pragma unroll
        for (int j = 0; j < TM_CC; ++j) {
            const int cl = cg * TM_CC + j, c = c0 + cl;
            if (i < n && c < o) {
                const double2 v = Wp[(size_t)i * o + c];
                const double2 w1 = make_double2(v.x + (double)acc[q][j].x, v.y + (double)acc[q][j].y);
                Wo[(size_t)i * o + c] = w1;
                T[i * OC + cl] = make_float2((float)w1.x, (float)w1.y);
            }
        }
    }
    __syncthreads();
    for (int k = 1; k <= n_terms; ++k) {
        tm_matmul<OC, NR, false>(n, Vr, Vi, T, Ms, acc, cg, rg);
        const float sk = sqrt_dt / (float)k;  // (i sqrt_dt / k) z = sk (-z.y, z.x)
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            const int i = rg + RG * q;
#pragma unroll
            for (int j = 0; j < TM_CC; ++j) {
                const int cl = cg * TM_CC + j, c = c0 + cl;
                const float2 t = make_float2(-sk * acc[q][j].y, sk * acc[q][j].x);
                if (i < n) T[i * OC + cl] = (c < o) ? t : make_float2(0.f, 0.f);
                if (i < n && c < o) {
                    double2 v = Wo[(size_t)i * o + c];
                    v.x += (double)t.x;
                    v.y += (double)t.y;
                    Wo[(size_t)i * o + c] = v;
                }
            }
        }
        __syncthreads();
    }
    // W' = out + (E - I) out
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        const int i = rg + RG * q;
#pragma unroll
        for (int j = 0; j < TM_CC; ++j) {
            const int cl = cg * TM_CC + j, c = c0 + cl;
            if (i < n && c < o) {
                const double2 v = Wo[(size_t)i * o + c];
                T[i * OC + cl] = make_float2((float)v.x, (float)v.y);
            }
        }
    }
    __syncthreads();
    tm_matmul<OC, NR, true>(n, emi, nullptr, T, Ms, acc, cg, rg);
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        const int i = rg + RG * q;
#pragma unroll
        for (int j = 0; j < TM_CC; ++j) {
            const int c = c0 + cg * TM_CC + j;
            if (i < n && c < o) {
                double2 v = Wo[(size_t)i * o + c];
                v.x += (double)acc[q][j].x;
                v.y += (double)acc[q][j].y;
                Wo[(size_t)i * o + c] = v;
            }
        }
    }
}

template <class K>
static int smem_attr(K kernel, size_t bytes) {
    if (bytes > 227 * 1024) return fail(AFQ_E_UNSUPPORTED, "mixed kernel needs %zu bytes of shared memory", bytes);
    if (bytes > 48 * 1024)
        AFQ_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return AFQ_OK;
}

template <int OC>
static int trotter_mixed_oc(int wc, int n, int o, int n_terms, double sqrt_dt, const float* emi, const float* vm,
                            long long ldv, const double2* win, double2* wout, cudaStream_t s) {
    constexpr int RG = TM_THREADS / (OC / TM_CC);
    const int nr = (n + RG - 1) / RG;
    const size_t smem = (size_t)n * (OC + TM_BJ) * sizeof(float2);
    dim3 grid((o + OC - 1) / OC, wc);
#define AFQ_TM(NRV)                                                                                    \
    do {                                                                                               \
        AFQ_TRY(smem_attr(k_trotter_mixed<OC, NRV>, smem));                                             \
        k_trotter_mixed<OC, NRV><<<grid, TM_THREADS, smem, s>>>(n, o, n_terms, (float)sqrt_dt, emi, vm, ldv, wc, \
                                                              win, wout);                             \
    } while (0)
    if (nr <= 1) AFQ_TM(1);
    else if (nr <= 2) AFQ_TM(2);
    else if (nr <= 4) AFQ_TM(4);
    else if (nr <= 8) AFQ_TM(8);
    else if (nr <= 16) AFQ_TM(16);
    else return fail(AFQ_E_UNSUPPORTED, "mixed trotter: norb=%d too large", n);
#undef AFQ_TM
    AFQ_LAUNCHED("k_trotter_mixed");
    return AFQ_OK;
}

int launch_trotter_mixed(int wc, int n, int o, int n_terms, double sqrt_dt, const float* emi, const float* vm,
                         long long ldv, const double2* win, double2* wout, cudaStream_t s) {
    if (wc <= 0) return AFQ_OK;
    if (wc > 65535) return fail(AFQ_E_UNSUPPORTED, "mixed trotter: chunk of %d walkers > 65535", wc);
    if (o <= 16) return trotter_mixed_oc<16>(wc, n, o, n_terms, sqrt_dt, emi, vm, ldv, win, wout, s);
    return trotter_mixed_oc<32>(wc, n, o, n_terms, sqrt_dt, emi, vm, ldv, win, wout, s);
}

// ------------------------------------------------------------------ energy
// Mixed energy (meas/rhf.py:36-50) for a chunk of walkers: the tensor-core
// GEMM produced F[(g, i), (w, part, k)] = sum_j L~[g, i, j] G_part[w, k, j]
// (part 0 = Re, 1 = Im of G_half); this kernel forms, per walker and chunk of
// Cholesky vectors, sum_g c_g^2 and sum_g sum_ik f_g[i,k] f_g[k,i] in fp64.
constexpr int EX_G = 8;  // Cholesky vectors per CTA
__global__ void __launch_bounds__(256) k_exchange_reduce(int G, int o, const float* __restrict__ F, long long ldf,
                                                         double2* __restrict__ partial, int nchunk) {
    extern __shared__ float2 fs[];  // EX_G x o x o complex
    const int w = blockIdx.y, g0 = blockIdx.x * EX_G;
    const int ng = min(EX_G, G - g0);
    const int oo = o * o;
    for (int e = threadIdx.x; e < ng * oo; e += blockDim.x) {
        const int g = e / oo, r = e % oo, i = r / o, k = r % o;
        const float* row = F + (long long)((g0 + g) * o + i) * ldf + (long long)(2 * w) * o;
        fs[e] = make_float2(row[k], row[o + k]);
    }
    __syncthreads();
    double xr = 0.0, xi = 0.0, cr = 0.0, ci = 0.0;
    for (int e = threadIdx.x; e < ng * oo; e += blockDim.x) {
        const int g = e / oo, r = e % oo, i = r / o, k = r % o;
        const float2 a = fs[e], b = fs[g * oo + k * o + i];
        xr += (double)a.x * b.x - (double)a.y * b.y;
        xi += (double)a.x * b.y + (double)a.y * b.x;
    }
    for (int g = threadIdx.x; g < ng; g += blockDim.x) {
        double tr = 0.0, ti = 0.0;
        for (int i = 0; i < o; ++i) {
            tr += fs[g * oo + i * o + i].x;
            ti += fs[g * oo + i * o + i].y;
        }
        cr += tr * tr - ti * ti;
        ci += 2.0 * tr * ti;
    }
    __shared__ double red[4][8];
    cr = warp_sum(cr); ci = warp_sum(ci); xr = warp_sum(xr); xi = warp_sum(xi);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { red[0][wid] = cr; red[1][wid] = ci; red[2][wid] = xr; red[3][wid] = xi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s4[4] = {0, 0, 0, 0};
        for (int q = 0; q < 4; ++q)
            for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s4[q] += red[q][k];
        partial[((size_t)w * nchunk + blockIdx.x) * 2 + 0] = make_double2(s4[0], s4[1]);
        partial[((size_t)w * nchunk + blockIdx.x) * 2 + 1] = make_double2(s4[2], s4[3]);
    }
}

int exchange_chunks(int G) { return (G + EX_G - 1) / EX_G; }

int launch_exchange_reduce(int wc, int G, int o, const float* F, long long ldf, double2* partial, cudaStream_t s) {
    if (wc <= 0) return AFQ_OK;
    const size_t smem = (size_t)EX_G * o * o * sizeof(float2);
    AFQ_TRY(smem_attr(k_exchange_reduce, smem));
    dim3 grid(exchange_chunks(G), wc);
    k_exchange_reduce<<<grid, 256, smem, s>>>(G, o, F, ldf, partial, exchange_chunks(G));
    AFQ_LAUNCHED("k_exchange_reduce");
    return AFQ_OK;
}

// Green's function rows for the energy GEMM: row (w*2 + part)*o + k holds
// split(G_part[w, k, :]) with K = n in sections of S.
__global__ void k_green_rows(int wc, int n, int o, const double2* __restrict__ green, __nv_bfloat16* __restrict__ dst,
                             int S, int Kt) {
    const long long rows = (long long)wc * o * 2;
    const long long total = rows * (long long)Kt;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / Kt;
        const int kk = (int)(e % Kt);
        __nv_bfloat16* row = dst + r * Kt;
        const int k = (int)(r % o), part = (int)((r / o) % 2), w = (int)(r / (2 * o));
        if (kk < S) {
            double x = 0.0;
            if (kk < n) {
                const double2 v = green[((size_t)w * o + k) * n + kk];
                x = part ? v.y : v.x;
            }
            split_store3(row, S, kk, x, false);
        } else if (kk >= 3 * S) {
            row[kk] = __double2bfloat16(0.0);
        }
    }
}

int launch_green_rows(int wc, int n, int o, const double2* green, __nv_bfloat16* dst, int S, int Kt, cudaStream_t s) {
    const long long total = (long long)wc * o * 2 * Kt;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    k_green_rows<<<(unsigned)blocks, 256, 0, s>>>(wc, n, o, green, dst, S, Kt);
    AFQ_LAUNCHED("k_green_rows");
    return AFQ_OK;
}

}  // namespace afq
