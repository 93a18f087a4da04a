// Kernels of the mixed-precision steps (AFQ_PREC_MIXED, AFQ_PREC_MIXED_FAST).
//
// Precision plan: the V-build, force-bias and energy contractions run on
// tensor cores (k_tc_gemm.cu) with bf16 split operands (six sections, every
// product above 2^-24, or three sections, ~2^-17) and drained fp32
// accumulation; the Taylor series multiplies in fp32 (here, or on the tensor
// cores in k_trotter_tc.cu) and updates binary64 walkers, applying E_half as
// W + (E_half - I) W with the small correction in fp32, so the walkers carry
// binary64 and do not drift.  The overlap matrix and the QR run in
// double-float (fp32 pairs) on the fp32 pipe; the determinant's LU, the
// phaseless cut, the weights and every energy accumulator stay binary64.
#include "afq_internal.cuh"

namespace afq {

// ------------------------------------------------------ operand preparation
// dst row r (Kt entries): sections at 0, S, 2S of split(src(r, k)), k < K;
// entries [3S, Kt) and [K, S) of each section are zero.
// src(r, k) = src[r * rs + k * ks].  With grp > 0 source row r goes to dst
// row (r / grp) grp_pad + r % grp (groups padded to grp_pad rows; the pad
// rows are not written).
__global__ void k_split_rows(long long rows, int K, int S, int Kt, const double* __restrict__ src, long long rs,
                             long long ks, __nv_bfloat16* __restrict__ dst, int left, int sec, int grp, int grp_pad) {
    const long long total = rows * (long long)Kt;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long r = e % rows;  // rows fastest: coalesced reads of column-major sources
        const int kk = (int)(e / rows);
        const long long dr = grp > 0 ? (r / grp) * grp_pad + r % grp : r;
        __nv_bfloat16* row = dst + dr * Kt;
        if (kk < S) {
            const double x = kk < K ? src[r * rs + (long long)kk * ks] : 0.0;
            split_store(row, S, kk, x, left != 0, sec);
        } else if (kk >= sec * S) {
            row[kk] = __double2bfloat16(0.0);
        }
    }
}

int launch_split_rows(long long rows, int K, int S, int Kt, const double* src, long long rs, long long ks,
                      __nv_bfloat16* dst, int left, int sec, cudaStream_t s, int grp, int grp_pad) {
    const long long total = rows * (long long)Kt;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    k_split_rows<<<(unsigned)blocks, 256, 0, s>>>(rows, K, S, Kt, src, rs, ks, dst, left, sec, grp, grp_pad);
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
// The six-section form: all of it in binary64 (k_field_shift_f32 below is the
// three-section form's).
__global__ void k_field_shift_mixed(int W, int G, int Wc, double sqrt_dt, const double* __restrict__ x,
                                    const float* __restrict__ fbm, long long ldf, const double2* __restrict__ mf,
                                    __nv_bfloat16* __restrict__ av, int S, int Kt, int sec,
                                    double2* __restrict__ shift_term, double2* __restrict__ fb_term) {
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
            split_store(re_row, S, g, xt.x, true, sec);
            split_store(im_row, S, g, xt.y, true, sec);
            sr += xt.x * m.x - xt.y * m.y;
            si += xt.x * m.y + xt.y * m.x;
            br += xv * fs.x - 0.5 * (fs.x * fs.x - fs.y * fs.y);
            bi += xv * fs.y - 0.5 * (2.0 * fs.x * fs.y);
        } else {
            split_store(re_row, S, g, 0.0, true, sec);
            split_store(im_row, S, g, 0.0, true, sec);
        }
    }
    for (int k = sec * S + lane; k < Kt; k += 32) {
        re_row[k] = __double2bfloat16(0.0);
        im_row[k] = __double2bfloat16(0.0);
    }
    sr = warp_sum(sr); si = warp_sum(si); br = warp_sum(br); bi = warp_sum(bi);
    if (lane == 0) {
        shift_term[w] = make_double2(sr, si);
        fb_term[w] = make_double2(br, bi);
    }
}

// The three-section form (operands of bf16 x 3 = 24 bits): the shifted field
// is formed and split in fp32 (the force bias is fp32 already).  The CTA's
// eight walkers share the mean-field shifts, staged once a CTA as fp32 in
// chunks of FS_CH; each lane sums its ~G/32 terms of the four weight sums in
// fp32 and the warp adds the lanes' sums in binary64.
constexpr int FS_CH = 1024;
__global__ void __launch_bounds__(256) k_field_shift_f32(int W, int G, int Wc, float sdt, const double* __restrict__ x,
                                                         const float* __restrict__ fbm, long long ldf,
                                                         const double2* __restrict__ mf,
                                                         __nv_bfloat16* __restrict__ av, int S, int Kt, int sec,
                                                         double2* __restrict__ shift_term,
                                                         double2* __restrict__ fb_term) {
    __shared__ float2 s_mf[FS_CH];
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    const bool active = w < W;  // every thread takes part in the staging barriers
    const int w0 = (w / Wc) * Wc;
    const int wc = min(Wc, W - w0);
    __nv_bfloat16* re_row = av + (long long)(2 * w0 + (w - w0)) * Kt;
    __nv_bfloat16* im_row = av + (long long)(2 * w0 + wc + (w - w0)) * Kt;
    float sr = 0.f, si = 0.f, br = 0.f, bi = 0.f;
    for (int g0 = 0; g0 < S; g0 += FS_CH) {
        __syncthreads();
        for (int e = threadIdx.x; e < FS_CH; e += blockDim.x) {
            const int g = g0 + e;
            const double2 m = g < G ? mf[g] : make_double2(0.0, 0.0);
            s_mf[e] = make_float2((float)m.x, (float)m.y);
        }
        __syncthreads();
        if (!active) continue;
        const int g1 = min(S, g0 + FS_CH);
        for (int g = g0 + lane; g < g1; g += 32) {
            if (g < G) {
                const float fr = 2.f * fbm[(long long)w * ldf + g], fi = 2.f * fbm[(long long)(W + w) * ldf + g];
                const float2 m = s_mf[g - g0];
                const float xv = (float)x[(size_t)w * G + g];
                const float fsx = -sdt * (-fi - m.x), fsy = -sdt * (fr - m.y);
                const float xr = xv - fsx, xi = -fsy;
                split_storef(re_row, S, g, xr, true, sec);
                split_storef(im_row, S, g, xi, true, sec);
                sr += xr * m.x - xi * m.y;
                si += xr * m.y + xi * m.x;
                br += xv * fsx - 0.5f * (fsx * fsx - fsy * fsy);
                bi += xv * fsy - fsx * fsy;
            } else {
                split_storef(re_row, S, g, 0.f, true, sec);
                split_storef(im_row, S, g, 0.f, true, sec);
            }
        }
    }
    if (!active) return;
    for (int k = sec * S + lane; k < Kt; k += 32) {
        re_row[k] = __float2bfloat16(0.f);
        im_row[k] = __float2bfloat16(0.f);
    }
    const double tr = warp_sum((double)sr), ti = warp_sum((double)si);
    const double ur = warp_sum((double)br), ui = warp_sum((double)bi);
    if (lane == 0) {
        shift_term[w] = make_double2(tr, ti);
        fb_term[w] = make_double2(ur, ui);
    }
}

int launch_field_shift_mixed(int W, int G, int Wc, double sqrt_dt, const double* x, const float* fbm, long long ldf,
                             const double2* mf, __nv_bfloat16* av, int S, int Kt, int sec, double2* shift_term,
                             double2* fb_term, cudaStream_t s) {
    if (sec == 3)
        k_field_shift_f32<<<(W + 7) / 8, 256, 0, s>>>(W, G, Wc, (float)sqrt_dt, x, fbm, ldf, mf, av, S, Kt, sec,
                                                      shift_term, fb_term);
    else
        k_field_shift_mixed<<<(W + 7) / 8, 256, 0, s>>>(W, G, Wc, sqrt_dt, x, fbm, ldf, mf, av, S, Kt, sec,
                                                        shift_term, fb_term);
    AFQ_LAUNCHED("k_field_shift_mixed");
    return AFQ_OK;
}

// ------------------------------------------------------- Taylor propagation
// One CTA per (walker, 32 columns).  The current Taylor term T (fp32, all n
// rows x 32 columns) stays in shared memory; the operand (V of this walker,
// or E_half - I) streams through a two-stage cp.async ring, TR_BJ columns per
// stage, so the next columns are in flight while the current ones are
// multiplied.  Thread (rg, cg) owns rows rg + RG q (q < NR) and the complex
// columns 2cg, 2cg+1, 16+2cg, 16+2cg+1 (so a warp's T reads are contiguous
// 128-byte rows).  Each thread touches only its own entries of the output
// walker (walkers_out may alias walkers_in) and of the fp32 scratch Ts that
// sums the series terms, so the binary64 pipe sees three additions per
// entry, not one per term:
//   W1 = W + (E-I) W;  Ts = sum_k (i sqrt_dt V)^k / k! W1 (fp32);
//   out = W1 + Ts;  W' = out + (E-I) out.
constexpr int TR_CG = 8, TR_OC = 32, TR_BJ = 8;
// Row stride (floats) of a staged operand plane: 16-byte rows for cp.async,
// and rows 0..3 of a warp start in different banks.
constexpr int TR_VS = TR_BJ + 4;

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Columns [j0, j0 + TR_BJ) of rows 0..n-1 of the operand planes (row stride
// n floats) into a stage; columns past n are zero.
__device__ __forceinline__ void tr_stage(int n, int j0, const float* __restrict__ re, const float* __restrict__ im,
                                         float* sr, float* si, bool v16) {
    const int jn = min(TR_BJ, n - j0);
    const int planes = im ? 2 : 1;
    if (v16) {  // n % 4 == 0 and 16-byte aligned planes: jn is a multiple of 4
        constexpr int CH = TR_BJ / 4;
        for (int e = threadIdx.x; e < n * CH * planes; e += blockDim.x) {
            const int i = e / (CH * planes), r = e % (CH * planes), pl = r / CH, h = r % CH;
            float* dst = (pl ? si : sr) + i * TR_VS + 4 * h;
            if (4 * h < jn) cp_async16(dst, (pl ? im : re) + (size_t)i * n + j0 + 4 * h);
            else *(float4*)dst = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    } else {
        for (int e = threadIdx.x; e < n * TR_BJ * planes; e += blockDim.x) {
            const int i = e / (TR_BJ * planes), r = e % (TR_BJ * planes), pl = r / TR_BJ, jj = r % TR_BJ;
            float* dst = (pl ? si : sr) + i * TR_VS + jj;
            if (jj < jn) cp_async4(dst, (pl ? im : re) + (size_t)i * n + j0 + jj);
            else *dst = 0.f;
        }
    }
    cp_async_commit();
}

// acc = M T for the n x n operand M (real when im == nullptr).  stg holds two
// stages of two planes, rows padded to RG*NR and zero beyond n.  Ends with a
// barrier, so the caller may overwrite T and the stages.
template <int NR, bool CPLX>
__device__ __forceinline__ void tr_matmul(int n, const float* __restrict__ re, const float* __restrict__ im,
                                          const float4* __restrict__ T4, float* stg, int rows, float2 (&acc)[NR][4],
                                          int cg, int rg, int RG, bool v16) {
#pragma unroll
    for (int q = 0; q < NR; ++q)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[q][j] = make_float2(0.f, 0.f);
    const int plane = rows * TR_VS;
    const int nb = (n + TR_BJ - 1) / TR_BJ;
    tr_stage(n, 0, re, im, stg, stg + plane, v16);
    for (int b = 0; b < nb; ++b) {
        cp_async_wait_all();
        __syncthreads();
        const float* sr = stg + (b & 1) * 2 * plane;
        const float* si = sr + plane;
        if (b + 1 < nb) {
            float* nr_ = stg + ((b + 1) & 1) * 2 * plane;
            tr_stage(n, (b + 1) * TR_BJ, re, im, nr_, nr_ + plane, v16);
        }
        const float4* tb = T4 + (size_t)b * TR_BJ * (TR_OC / 2);
#pragma unroll 1
        for (int jj = 0; jj < TR_BJ; jj += 2) {
            float2 mr[NR], mi[NR];
#pragma unroll
            for (int q = 0; q < NR; ++q) {
                const int i = rg + RG * q;
                mr[q] = *(const float2*)(sr + i * TR_VS + jj);
                if (CPLX) mi[q] = *(const float2*)(si + i * TR_VS + jj);
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const float4 ta = tb[(jj + h) * (TR_OC / 2) + cg], tc = tb[(jj + h) * (TR_OC / 2) + TR_CG + cg];
                const float2 t[4] = {make_float2(ta.x, ta.y), make_float2(ta.z, ta.w), make_float2(tc.x, tc.y),
                                     make_float2(tc.z, tc.w)};
                float2 tn[4];  // i t
#pragma unroll
                for (int j = 0; j < 4; ++j) tn[j] = make_float2(-t[j].y, t[j].x);
#pragma unroll
                for (int q = 0; q < NR; ++q) {  // acc += a t + b (i t), two lanes per instruction
                    const float a = h ? mr[q].y : mr[q].x;
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[q][j] = __ffma2_rn(make_float2(a, a), t[j], acc[q][j]);
                    if (CPLX) {
                        const float bq = h ? mi[q].y : mi[q].x;
#pragma unroll
                        for (int j = 0; j < 4; ++j) acc[q][j] = __ffma2_rn(make_float2(bq, bq), tn[j], acc[q][j]);
                    }
                }
            }
        }
    }
    __syncthreads();
}

__device__ __forceinline__ int tr_col(int cg, int j) { return j < 2 ? 2 * cg + j : TR_OC / 2 + 2 * cg + (j - 2); }

template <int NR>
__global__ void __launch_bounds__(512) k_trotter_mixed(int n, int o, int n_terms, float sqrt_dt,
                                                          const float* __restrict__ emi, const float* __restrict__ vm,
                                                          long long ldv, int wc, const double2* win, double2* wout,
                                                          float2* __restrict__ tsum, int v16) {
    extern __shared__ float4 smf4[];
    const int RG = blockDim.x / TR_CG, rows = RG * NR;
    const int nT = (n + TR_BJ - 1) / TR_BJ * TR_BJ;
    float4* T4 = smf4;                              // nT x 32 complex, as float4 pairs
    float2* T = (float2*)smf4;
    float* stg = (float*)(smf4 + (size_t)nT * (TR_OC / 2));  // 2 stages x 2 planes x rows x TR_VS
    const int w = blockIdx.y, c0 = blockIdx.x * TR_OC;
    const int cg = threadIdx.x % TR_CG, rg = threadIdx.x / TR_CG;
    const double2* Wp = win + (size_t)w * n * o;
    double2* Wo = wout + (size_t)w * n * o;
    const float* Vr = vm + (long long)w * ldv;
    const float* Vi = vm + (long long)(wc + w) * ldv;
    float2* Ts = tsum + (size_t)w * n * o;

    for (int e = threadIdx.x; e < 4 * rows * TR_VS; e += blockDim.x) stg[e] = 0.f;
    for (int e = threadIdx.x; e < nT * TR_OC; e += blockDim.x) {
        const int i = e / TR_OC, cc = e % TR_OC;
        float2 t = make_float2(0.f, 0.f);
        if (i < n && c0 + cc < o) {
            const double2 v = Wp[(size_t)i * o + c0 + cc];
            t = make_float2((float)v.x, (float)v.y);
        }
        T[e] = t;
    }
    __syncthreads();
    float2 acc[NR][4];
    int rgl;  // rg, opaque to the compiler: entry addresses are recomputed per epilogue, not held in registers
    // W1 = W + (E - I) W
    tr_matmul<NR, false>(n, emi, nullptr, T4, stg, rows, acc, cg, rg, RG, v16);
    rgl = rg;
    asm volatile("" : "+r"(rgl));
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        const int i = rgl + RG * q;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int cl = tr_col(cg, j), c = c0 + cl;
            if (i < n && c < o) {
                const double2 v = Wp[(size_t)i * o + c];
                const double2 w1 = make_double2(v.x + (double)acc[q][j].x, v.y + (double)acc[q][j].y);
                Wo[(size_t)i * o + c] = w1;
                T[i * TR_OC + cl] = make_float2((float)w1.x, (float)w1.y);
            }
        }
    }
    __syncthreads();
    for (int k = 1; k <= n_terms; ++k) {
        tr_matmul<NR, true>(n, Vr, Vi, T4, stg, rows, acc, cg, rg, RG, v16);
        const float sk = sqrt_dt / (float)k;  // (i sqrt_dt / k) z = sk (-z.y, z.x)
        rgl = rg;
        asm volatile("" : "+r"(rgl));
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            const int i = rgl + RG * q;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int cl = tr_col(cg, j), c = c0 + cl;
                const float2 t = make_float2(-sk * acc[q][j].y, sk * acc[q][j].x);
                if (i < n) T[i * TR_OC + cl] = (c < o) ? t : make_float2(0.f, 0.f);
                if (i < n && c < o) {
                    float2* ts = Ts + (size_t)i * o + c;
                    if (k == 1) {
                        *ts = t;
                    } else {
                        const float2 u = *ts;
                        *ts = make_float2(u.x + t.x, u.y + t.y);
                    }
                }
            }
        }
        __syncthreads();
    }
    // out = W1 + Ts;  W' = out + (E - I) out
    rgl = rg;
    asm volatile("" : "+r"(rgl));
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        const int i = rgl + RG * q;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int cl = tr_col(cg, j), c = c0 + cl;
            if (i < n && c < o) {
                double2 v = Wo[(size_t)i * o + c];
                if (n_terms > 0) {
                    const float2 u = Ts[(size_t)i * o + c];
                    v.x += (double)u.x;
                    v.y += (double)u.y;
                    Wo[(size_t)i * o + c] = v;
                }
                T[i * TR_OC + cl] = make_float2((float)v.x, (float)v.y);
            }
        }
    }
    __syncthreads();
    tr_matmul<NR, false>(n, emi, nullptr, T4, stg, rows, acc, cg, rg, RG, v16);
    rgl = rg;
    asm volatile("" : "+r"(rgl));
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        const int i = rgl + RG * q;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = c0 + tr_col(cg, j);
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
    if (bytes > 32 * 1024)  // with the kernel's static shared memory the default limit is below 48 KB
        AFQ_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return AFQ_OK;
}

int launch_trotter_mixed(int wc, int n, int o, int n_terms, double sqrt_dt, const float* emi, const float* vm,
                         long long ldv, const double2* win, double2* wout, float2* tsum, cudaStream_t s) {
    if (wc <= 0) return AFQ_OK;
    if (wc > 65535) return fail(AFQ_E_UNSUPPORTED, "mixed trotter: chunk of %d walkers > 65535", wc);
    // 256 threads (32 row groups) up to 7 rows each, else 512 threads
    const int threads = n <= 32 * 7 ? 256 : 512, RG = threads / TR_CG;
    const int nr = (n + RG - 1) / RG;
    if (nr > 8) return fail(AFQ_E_UNSUPPORTED, "mixed trotter: norb=%d too large", n);
    const int nT = (n + TR_BJ - 1) / TR_BJ * TR_BJ;
    const size_t smem = (size_t)nT * TR_OC * sizeof(float2) + (size_t)4 * RG * nr * TR_VS * sizeof(float);
    const int v16 = (n % 4 == 0) && (ldv % 4 == 0) && ((((uintptr_t)vm) | ((uintptr_t)emi)) & 15) == 0;
    dim3 grid((o + TR_OC - 1) / TR_OC, wc);
#define AFQ_TM(NRV)                                                                                      \
    case NRV:                                                                                            \
        AFQ_TRY(smem_attr(k_trotter_mixed<NRV>, smem));                                                  \
        k_trotter_mixed<NRV><<<grid, threads, smem, s>>>(n, o, n_terms, (float)sqrt_dt, emi, vm, ldv, wc, win, \
                                                         wout, tsum, v16);                               \
        break;
    switch (nr) {
        AFQ_TM(1) AFQ_TM(2) AFQ_TM(3) AFQ_TM(4) AFQ_TM(5) AFQ_TM(6) AFQ_TM(7) AFQ_TM(8)
    }
#undef AFQ_TM
    AFQ_LAUNCHED("k_trotter_mixed");
    return AFQ_OK;
}

// ------------------------------------------- overlap + force-bias operand
// Mixed-form replacement of k_green for the overlap (meas/rhf.py:22-24) and
// the next step's force-bias operand (meas/rhf.py:15-19, 27-33):
//   m = C^H W; LU with partial pivoting gives det(m) and the overlap
//   det(m)^2 (binary64, or with DF in double-float with the determinant's
//   product of pivots in binary64);
//   m^-1 by fp32 Gauss-Jordan on a float copy of m, and
//   G_half^T = W m^-1 in fp32, written as the bf16 split operand (which
//   resolves at most ~2^-24, so fp32 here costs no accuracy downstream)
//   and/or, widened, as the Green's function G_half (o x n) the mixed
//   energy reads (its bf16 split resolves less than fp32 as well).
// Pivot reciprocals are computed once per pivot and shared through shared
// memory.  Real trial orbitals (the mixed form requires them).
//
// DF: m by double-float arithmetic on the fp32 pipe instead of binary64
// FMAs (the binary64 pipe runs ~1/64 of the fp32 rate on this GPU).  C and W
// are split as x = x_hi + x_lo (fp32 pair, 48 significant bits); each term's
// c_hi w_hi is formed exactly (TwoProd: product and fma residual) and summed
// by TwoSum into (s, e), while the residual, c_hi w_lo and c_lo w_hi go to
// the fp32 error sum e: m = s + e to ~2^-44 relative, binary64 for the
// determinant's purposes, from fp32 instructions only.
constexpr int OS_CH = 32;  // rows of W per staging chunk (double-float m, then G_half)

// (s, e) += c (wr, wi) on two lanes at once with the paired fp32
// instructions (f32x2), for one double-float c = (ch, cl) and a pair
// w = (wr, wi) with hi and lo parts in wh and wl: per lane p = ch wh and
// pe = fma(ch, wh, -p) (TwoProd, exact), t + r = s + p (Knuth's TwoSum,
// exact), s <- t and e <- e + ((r + pe) + fma(ch, wl, cl wh)).  A
// subtraction y - x is fma(x, -1, y) (one rounding, as fsub), and -p comes
// from (-c) w exactly.
__device__ __forceinline__ void df_acc2(float2& s, float2& e, float ch, float cl, float2 wh, float2 wl) {
    const float2 m1 = make_float2(-1.f, -1.f);
    const float2 c2 = make_float2(ch, ch);
    const float2 np = __fmul2_rn(make_float2(-ch, -ch), wh);  // -p
    const float2 pe = __ffma2_rn(c2, wh, np);                 // exact: c wh = p + pe
    const float2 t = __ffma2_rn(np, m1, s);                   // s + p
    const float2 v = __ffma2_rn(s, m1, t);                    // t - s
    const float2 a2 = __ffma2_rn(__ffma2_rn(v, m1, t), m1, s);  // s - (t - v)
    const float2 r = __ffma2_rn(__fadd2_rn(np, v), m1, a2);   // exact: s + p = t + r
    s = t;
    e = __fadd2_rn(e, __fadd2_rn(__fadd2_rn(r, pe), __ffma2_rn(c2, wl, __fmul2_rn(make_float2(cl, cl), wh))));
}

// (s, e) += (sb, eb) for two double-float pairs on two lanes (Knuth's two-sum
// of the heads, the tails and the rounding error added to the tail).
__device__ __forceinline__ void df_add2(float2& s, float2& e, float2 sb, float2 eb) {
    const float2 m1 = make_float2(-1.f, -1.f);
    const float2 t = __fadd2_rn(s, sb);
    const float2 v = __ffma2_rn(s, m1, t);                                        // t - s
    const float2 r = __fadd2_rn(__ffma2_rn(__ffma2_rn(v, m1, t), m1, s), __ffma2_rn(v, m1, sb));
    s = t;
    e = __fadd2_rn(__fadd2_rn(e, eb), r);
}

// Double-float (fp32 pair, ~2^-44) complex arithmetic for the overlap's LU,
// after the QD library's algorithms (Hida, Li and Bailey): Knuth's two-sum,
// the fma two-product, the "sloppy" pair addition, and the reciprocal by one
// Newton-Raphson step from the fp32 reciprocal.  A complex value is a float4
// (re hi, re lo, im hi, im lo).
__device__ __forceinline__ float2 df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ float2 df_quick(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float2 s = df_two_sum(a.x, b.x);
    return df_quick(s.x, __fadd_rn(s.y, __fadd_rn(a.y, b.y)));
}
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, e));
    return df_quick(p, e);
}
__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float4 zdf_mul(float4 a, float4 b) {
    const float2 ar = make_float2(a.x, a.y), ai = make_float2(a.z, a.w);
    const float2 br = make_float2(b.x, b.y), bi = make_float2(b.z, b.w);
    const float2 re = df_add(df_mul(ar, br), df_neg(df_mul(ai, bi)));
    const float2 im = df_add(df_mul(ar, bi), df_mul(ai, br));
    return make_float4(re.x, re.y, im.x, im.y);
}
__device__ __forceinline__ float4 zdf_sub(float4 a, float4 b) {
    const float2 re = df_add(make_float2(a.x, a.y), make_float2(-b.x, -b.y));
    const float2 im = df_add(make_float2(a.z, a.w), make_float2(-b.z, -b.w));
    return make_float4(re.x, re.y, im.x, im.y);
}
__device__ __forceinline__ float2 df_rcp(float2 d) {
    const float2 r0 = make_float2(1.0f / d.x, 0.f);
    const float2 e = df_add(make_float2(1.f, 0.f), df_neg(df_mul(d, r0)));  // 1 - d r0
    return df_add(r0, df_mul(r0, e));
}
__device__ __forceinline__ float4 zdf_rcp(float4 p) {  // 1 / (a + i b) = (a - i b) / (a^2 + b^2)
    const float2 a = make_float2(p.x, p.y), b = make_float2(p.z, p.w);
    const float2 inv = df_rcp(df_add(df_mul(a, a), df_mul(b, b)));
    const float2 re = df_mul(a, inv), im = df_neg(df_mul(b, inv));
    return make_float4(re.x, re.y, im.x, im.y);
}

// The same double-float operations on the (Re, Im) lanes of a complex value
// at once with the paired fp32 instructions (f32x2): a value is a float4
// (re hi, im hi, re lo, im lo) = heads h and tails l; results are bitwise
// those of the scalar forms above (the same roundings in the same order).
struct dfc {
    float2 h, l;
};
__device__ __forceinline__ dfc dfc_of(float4 v) { return {make_float2(v.x, v.y), make_float2(v.z, v.w)}; }
__device__ __forceinline__ float4 dfc_f4(dfc v) { return make_float4(v.h.x, v.h.y, v.l.x, v.l.y); }
__device__ __forceinline__ dfc dfc_add(dfc a, dfc b) {  // df_add on both lanes
    const float2 m1 = make_float2(-1.f, -1.f);
    const float2 s = __fadd2_rn(a.h, b.h);
    const float2 bb = __ffma2_rn(a.h, m1, s);                                       // s - a
    const float2 e1 = __ffma2_rn(__ffma2_rn(bb, m1, s), m1, a.h);                  // a - (s - bb)
    const float2 e = __fadd2_rn(__fadd2_rn(e1, __ffma2_rn(bb, m1, b.h)), __fadd2_rn(a.l, b.l));
    const float2 hs = __fadd2_rn(s, e);                                             // df_quick(s, e)
    return {hs, __ffma2_rn(__ffma2_rn(s, m1, hs), m1, e)};
}
// (x.re x u.re, x.re x u.im) with the broadcast head x.re in (xh, xh), its
// negation in nxh and its tail in xl: df_mul on both lanes.
__device__ __forceinline__ dfc dfc_mul_b(float2 xh, float2 nxh, float2 xl, float2 uh, float2 ul) {
    const float2 m1 = make_float2(-1.f, -1.f);
    const float2 np = __fmul2_rn(nxh, uh);                                          // -p
    const float2 e = __ffma2_rn(xh, ul, __ffma2_rn(xl, uh, __ffma2_rn(xh, uh, np)));
    const float2 hs = __ffma2_rn(np, m1, e);                                        // p + e
    return {hs, __ffma2_rn(__fadd2_rn(hs, np), m1, e)};                             // e - (hs - p)
}

template <int MA, bool STAGE_W, bool DF>
__global__ void __launch_bounds__(256, MA <= 4 ? 5 : 1) k_overlap_split(int n, int o, const double2* __restrict__ mo,
                                                       const double2* __restrict__ walkers,
                                                       double2* __restrict__ ovlp_out, SplitOut split,
                                                       double2* __restrict__ green_out,
                                                       const float2* __restrict__ cs) {
    extern __shared__ double2 smd[];
    double2* m = smd;                              // o x o binary64 (LU in place)
    float4* md = (float4*)smd;                     // DF: the same storage as double-float pairs
    float2* mf = (float2*)(m + o * o);             // o x o fp32 copy -> Gauss-Jordan
    float2* invf = mf + o * o;                     // o x o fp32 inverse
    float2* wf = invf + o * o;                     // n x o fp32 copy of W (its hi part)
    float2* wl = wf + (size_t)OS_CH * o;           // DF: lo part of a chunk of OS_CH rows
    const int w = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const double2* Wp = walkers + (size_t)w * n * o;

    if (DF) {  // m in double-float from the split of W, staged OS_CH rows at a time
        const int AG = blockDim.x / o;
        const int b = tid % o, ag = tid / o;
        float2 s2[MA], e2[MA];  // (Re, Im) sums and their error terms
#pragma unroll
        for (int k = 0; k < MA; ++k) s2[k] = e2[k] = make_float2(0.f, 0.f);
        for (int i0 = 0; i0 < n; i0 += OS_CH) {
            const int rows = min(OS_CH, n - i0);
            __syncthreads();
            for (int e = tid; e < rows * o; e += blockDim.x) {
                const double2 x = Wp[(size_t)i0 * o + e];
                const float2 re = split_d2f(x.x), im = split_d2f(x.y);
                wf[e] = make_float2(re.x, im.x);
                wl[e] = make_float2(re.y, im.y);
            }
            __syncthreads();
            if (ag < AG) {
                for (int i = 0; i < rows; ++i) {
                    const float2 xh = wf[i * o + b], xl = wl[i * o + b];
#pragma unroll
                    for (int k = 0; k < MA; ++k) {
                        const int a = ag + AG * k;
                        if (a < o) {
                            const float2 c = cs[(i0 + i) * o + a];  // (hi, lo) of C[i, a]
                            df_acc2(s2[k], e2[k], c.x, c.y, xh, xl);
                        }
                    }
                }
            }
        }
        if (ag < AG) {
#pragma unroll
            for (int k = 0; k < MA; ++k) {
                const int a = ag + AG * k;
                if (a < o) {
                    const float2 re = df_quick(s2[k].x, e2[k].x), im = df_quick(s2[k].y, e2[k].y);
                    md[a * o + b] = make_float4(re.x, re.y, im.x, im.y);
                    mf[a * o + b] = make_float2(re.x, im.x);
                }
            }
        }
        for (int e = tid; e < o * o; e += blockDim.x)
            invf[e] = make_float2((e / o) == (e % o) ? 1.f : 0.f, 0.f);
    } else {  // m (binary64) and the fp32 copy of W
        const int AG = blockDim.x / o;
        const int b = tid % o, ag = tid / o;
        double2 acc[MA];
#pragma unroll
        for (int k = 0; k < MA; ++k) acc[k] = make_double2(0.0, 0.0);
        if (ag < AG) {
            for (int i = 0; i < n; ++i) {
                const double2 x = Wp[(size_t)i * o + b];
                if (STAGE_W && ag == 0) wf[i * o + b] = make_float2((float)x.x, (float)x.y);
#pragma unroll
                for (int k = 0; k < MA; ++k) {
                    const int a = ag + AG * k;
                    if (a < o) rfma(acc[k], mo[i * o + a].x, x);
                }
            }
#pragma unroll
            for (int k = 0; k < MA; ++k) {
                const int a = ag + AG * k;
                if (a < o) {
                    m[a * o + b] = acc[k];
                    mf[a * o + b] = make_float2((float)acc[k].x, (float)acc[k].y);
                }
            }
        }
        for (int e = tid; e < o * o; e += blockDim.x)
            invf[e] = make_float2((e / o) == (e % o) ? 1.f : 0.f, 0.f);
    }
    __syncthreads();

    // The two factorisations of m, each by one warp with no block barrier
    // inside (the other warps go on to the barrier below):
    //   warp 0: LU with partial pivoting for det(m) only (double-float with
    //     DF, else binary64): rows are swapped and eliminated from column k
    //     on, the multipliers of step k are formed by their rows' lanes;
    //   warp 1: fp32 Gauss-Jordan with partial pivoting on [mf | I], giving
    //     invf = m^-1 for G_half.
    // Pivots: the largest |Re| + |Im| of the column (ties to the lower row).
    constexpr int OMAX = MA <= 4 ? 32 : 64;   // nocc bound of this instantiation (AG = 256 / o >= o / MA)
    __shared__ float4 s_lmul[OMAX];           // LU multipliers (double-float, or binary64 as double2)
    __shared__ float2 s_fmul[OMAX];           // Gauss-Jordan multipliers
    if (wid == 0) {
        double2 det = make_double2(1.0, 0.0);
        bool zero = false;
        for (int k = 0; k < o && !zero; ++k) {
            float best = -1.f;
            int bi = k;
            for (int r = k + lane; r < o; r += 32) {
                float v;
                if (DF) {
                    const float4 x = md[r * o + k];
                    v = fabsf(x.x) + fabsf(x.z);
                } else {
                    const double2 x = m[r * o + k];
                    v = (float)(fabs(x.x) + fabs(x.y));
                }
                if (v > best) { best = v; bi = r; }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const float ob = __shfl_xor_sync(0xffffffffu, best, off);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (bi != k)  // 16-byte entries: binary64 complex, or double-float
                for (int j = k + lane; j < o; j += 32) {
                    const double2 t = m[k * o + j];
                    m[k * o + j] = m[bi * o + j];
                    m[bi * o + j] = t;
                }
            __syncwarp();
            double2 piv;
            float4 rpd = make_float4(0.f, 0.f, 0.f, 0.f);
            double2 rp = make_double2(0.0, 0.0);
            if (DF) {
                const float4 pk = md[k * o + k];
                piv = make_double2((double)pk.x + (double)pk.y, (double)pk.z + (double)pk.w);
                if (pk.x == 0.f && pk.y == 0.f && pk.z == 0.f && pk.w == 0.f) zero = true;
                else rpd = zdf_rcp(pk);
            } else {
                piv = m[k * o + k];
                if (piv.x == 0.0 && piv.y == 0.0) zero = true;
                else rp = cdiv(make_double2(1.0, 0.0), piv);
            }
            if (lane == 0) {
                const double2 d = cmul(det, piv);
                det = (bi != k) ? make_double2(-d.x, -d.y) : d;
            }
            if (zero) break;
            for (int r = k + 1 + lane; r < o; r += 32) {  // multipliers, by their rows' lanes
                if (DF) s_lmul[r] = zdf_mul(md[r * o + k], rpd);
                else ((double2*)s_lmul)[r] = cmul(m[r * o + k], rp);
            }
            __syncwarp();
            for (int j = k + 1 + lane; j < o; j += 32) {  // columns by lanes, rows in turn
                if (DF) {
                    const float4 ukj = md[k * o + j];
                    for (int r = k + 1; r < o; ++r) md[r * o + j] = zdf_sub(md[r * o + j], zdf_mul(s_lmul[r], ukj));
                } else {
                    const double2 ukj = m[k * o + j];
                    for (int r = k + 1; r < o; ++r)
                        m[r * o + j] = csub(m[r * o + j], cmul(((const double2*)s_lmul)[r], ukj));
                }
            }
            __syncwarp();
        }
        // an exactly zero pivot: m is singular and det(m) is exactly 0 (as LAPACK's LU gives it)
        if (lane == 0 && ovlp_out) ovlp_out[w] = zero ? make_double2(0.0, 0.0) : cmul(det, det);
    } else if (wid == 1) {
        for (int k = 0; k < o; ++k) {
            float best = -1.f;
            int bi = k;
            for (int r = k + lane; r < o; r += 32) {
                const float2 v = mf[r * o + k];
                const float a = fabsf(v.x) + fabsf(v.y);
                if (a > best) { best = a; bi = r; }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const float ob = __shfl_xor_sync(0xffffffffu, best, off);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            // swap rows k and bi (columns k.. of the copy, all of the inverse), then scale row k by 1 / pivot
            const float2 pv = mf[bi * o + k];
            const float den = pv.x * pv.x + pv.y * pv.y;
            const float2 rp = make_float2(pv.x / den, -pv.y / den);
            __syncwarp();  // every lane has read the pivot before row k is rewritten
            for (int j = lane; j < 2 * o; j += 32) {
                float2* X = j < o ? mf : invf;
                const int jj = j < o ? j : j - o;
                if (j < o && jj < k) continue;
                const float2 a = X[k * o + jj], b = X[bi * o + jj];
                if (bi != k) X[bi * o + jj] = a;
                X[k * o + jj] = make_float2(b.x * rp.x - b.y * rp.y, b.x * rp.y + b.y * rp.x);
            }
            __syncwarp();
            for (int r = lane; r < o; r += 32) s_fmul[r] = mf[r * o + k];  // multipliers (row k's is 1)
            __syncwarp();
            for (int j = lane; j < 2 * o; j += 32) {  // eliminate column k from every other row
                float2* X = j < o ? mf : invf;
                const int jj = j < o ? j : j - o;
                if (j < o && jj <= k) continue;
                const float2 v = X[k * o + jj];
                for (int r = 0; r < o; ++r) {
                    if (r == k) continue;
                    const float2 f = s_fmul[r], x = X[r * o + jj];
                    X[r * o + jj] = make_float2(x.x - (f.x * v.x - f.y * v.y), x.y - (f.x * v.y + f.y * v.x));
                }
            }
            __syncwarp();
        }
    }
    __syncthreads();

    // G_half[b, i] = sum_a W[i, a] inv[a, b] in fp32 -> split operand / green_out
    __nv_bfloat16* re_row = split.ptr ? split.ptr + (size_t)w * split.ld : nullptr;
    __nv_bfloat16* im_row = split.ptr ? split.ptr + (size_t)(split.W + w) * split.ld : nullptr;
    double2* Gp = green_out ? green_out + (size_t)w * o * n : nullptr;
    constexpr int BG = 4;  // columns a task: a 32-row chunk at nocc 30 is 256 tasks, one per thread
    const int nbg = (o + BG - 1) / BG;
    // DF: W's fp32 copy is staged again OS_CH rows at a time (fewer bytes of shared memory, more CTAs)
    for (int i0 = 0; i0 < n; i0 += DF ? OS_CH : n) {
    const int rows = DF ? min(OS_CH, n - i0) : n;
    if (DF) {
        __syncthreads();
        for (int e = tid; e < rows * o; e += blockDim.x) {
            const double2 x = Wp[(size_t)i0 * o + e];
            wf[e] = make_float2(d2f_trunc(x.x), d2f_trunc(x.y));
        }
        __syncthreads();
    }
    for (int t = tid; t < rows * nbg; t += blockDim.x) {
        const int il = t % rows, bg = t / rows, i = i0 + il;
        float2 acc[BG];
#pragma unroll
        for (int j = 0; j < BG; ++j) acc[j] = make_float2(0.f, 0.f);
        for (int a = 0; a < o; ++a) {
            float2 x;
            if (STAGE_W) {
                x = wf[il * o + a];
            } else {
                const double2 v = Wp[(size_t)i * o + a];
                x = make_float2((float)v.x, (float)v.y);
            }
#pragma unroll
            for (int j = 0; j < BG; ++j) {
                const int b = bg * BG + j;
                if (b < o) {
                    const float2 v = invf[a * o + b];
                    acc[j].x = fmaf(x.x, v.x, acc[j].x); acc[j].x = fmaf(-x.y, v.y, acc[j].x);
                    acc[j].y = fmaf(x.x, v.y, acc[j].y); acc[j].y = fmaf(x.y, v.x, acc[j].y);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < BG; ++j) {
            const int b = bg * BG + j;
            if (b < o) {
                if (re_row) {
                    split_storef(re_row, split.S, b * n + i, acc[j].x, true, split.sec);
                    split_storef(im_row, split.S, b * n + i, acc[j].y, true, split.sec);
                }
                if (Gp) Gp[(size_t)b * n + i] = make_double2(acc[j].x, acc[j].y);
            }
        }
    }
    }
    if (!re_row) return;
    for (int e = n * o + tid; e < split.S; e += blockDim.x) {
        split_storef(re_row, split.S, e, 0.f, true, split.sec);
        split_storef(im_row, split.S, e, 0.f, true, split.sec);
    }
    for (long long e = (long long)split.sec * split.S + tid; e < split.ld; e += blockDim.x) {
        re_row[e] = __float2bfloat16(0.f);
        im_row[e] = __float2bfloat16(0.f);
    }
}

// The overlap, its Green's function and the force-bias operand of the mixed
// forms from a given double-float m = C^T W (k_ozaki.cu; meas/rhf.py:15-33),
// one CTA of 256 threads per walker:
//   warps 0-3: LU of m with partial pivoting in double-float, for det(m)
//     (overlap = det(m)^2 for the restricted walker);
//   warps 4-7: fp32 Gauss-Jordan on [m | I], for m^-1 (G_half's factor).
// Each step of both runs four threads a row with one barrier of the group:
// rows are addressed through a permutation (no row swaps), the pivot of step
// k + 1 (the largest |Re| + |Im| of the column, ties to the lower row) is
// found while step k updates column k + 1 (a shared-memory atomicMax over
// (value, -row) keys, three in rotation), and Gauss-Jordan leaves each pivot
// row unscaled (row k of the inverse is scaled by 1 / pivot_k at the end,
// the multipliers carry the factor meanwhile).  Then G_half = W m^-1 in fp32
// by all warps, W staged OG_CH rows a time, one row by four columns a thread.
constexpr int OG_CH = 32;  // rows of W per G_half staging chunk

__device__ __forceinline__ unsigned long long piv_key(float v, int r) {  // v >= 0: its bits order as values
    return ((unsigned long long)__float_as_uint(v) << 32) | (unsigned)(0xffff - r);
}
__device__ __forceinline__ int piv_row(unsigned long long key) { return 0xffff - (int)(key & 0xffffu); }
__host__ __device__ constexpr int og_xs(int o) {  // float2 entries of [m | I], and of the packed inverse
    return 2 * o * o > o * ((o + 3) & ~3) ? 2 * o * o : o * ((o + 3) & ~3);
}
__host__ __device__ constexpr int og_a16(int o) {  // 16-byte units of the region of m, later of staged W
    return o * o > OG_CH * (o | 1) ? o * o : OG_CH * (o | 1);
}
__device__ __forceinline__ void group_bar(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }

__global__ void __launch_bounds__(256, 5) k_overlap_oz(int n, int o, const float4* __restrict__ m_in,
                                                       const double2* __restrict__ walkers,
                                                       double2* __restrict__ ovlp_out, SplitOut split,
                                                       double2* __restrict__ green_out) {
    extern __shared__ float4 smf[];
    const int o2 = 2 * o, ws = o | 1, IS = (o + 3) & ~3;
    float4* md = smf;                       // o x o double-float m (re hi, im hi, re lo, im lo), LU in place
    float4* wf = smf;                       // then OG_CH x ws staged fp32 rows of W as (re, re, im, im)
    float2* X = (float2*)(smf + og_a16(o)); // o x 2o fp32 [m | I], Gauss-Jordan in place
    float2* inv = X;                        // then o x IS: row a of m^-1
    __shared__ unsigned long long s_key[2][3];
    __shared__ int s_perm[2][2][32];        // [LU, GJ][ping-pong][logical row] -> physical row
    __shared__ int s_pf[32];                // GJ: physical row of logical row k from step k on
    __shared__ float2 s_rp[32];             // GJ: 1 / pivot_k
    const int w = blockIdx.x, tid = threadIdx.x;

    const float4* mw = m_in + (size_t)w * o * o;
    for (int e = tid; e < o * o; e += blockDim.x) {
        const float4 x = mw[e];  // (re hi, re lo, im hi, im lo)
        const int r = e / o, c = e - r * o;
        md[e] = make_float4(x.x, x.z, x.y, x.w);
        X[r * o2 + c] = make_float2(x.x, x.z);
        X[r * o2 + o + c] = make_float2(r == c ? 1.f : 0.f, 0.f);
    }
    if (tid < 32) s_perm[0][0][tid] = s_perm[1][0][tid] = tid;
    if (tid < 6) (&s_key[0][0])[tid] = 0ull;
    __syncthreads();
    if (tid < o) {  // the pivot keys of step 0 (column 0; the same fp32 heads for both)
        const float4 x = md[tid * o];
        const unsigned long long key = piv_key(fabsf(x.x) + fabsf(x.y), tid);
        atomicMax(&s_key[0][0], key);
        atomicMax(&s_key[1][0], key);
    }
    __syncthreads();

    if (tid < 128) {  // LU (double-float)
        const int rr = tid >> 2, q = tid & 3;
        double2 det = make_double2(1.0, 0.0);
        bool zero = false;
        for (int k = 0; k < o; ++k) {
            const int* pc = s_perm[0][k & 1];
            int* pn = s_perm[0][(k + 1) & 1];
            const int bi = piv_row(s_key[0][k % 3]);
            const int pr = pc[bi];
            const float4 pq = md[pr * o + k];
            const float4 pk = make_float4(pq.x, pq.z, pq.y, pq.w);  // (re hi, re lo, im hi, im lo)
            // an exactly zero pivot: m is singular and det(m) is exactly 0 (as LAPACK's LU gives it)
            if (pk.x == 0.f && pk.y == 0.f && pk.z == 0.f && pk.w == 0.f) { zero = true; break; }
            if (tid == 0) {
                const double2 d = cmul(det, make_double2((double)pk.x + (double)pk.y, (double)pk.z + (double)pk.w));
                det = bi != k ? make_double2(-d.x, -d.y) : d;
                s_key[0][(k + 2) % 3] = 0ull;
            }
            const float4 rpd = zdf_rcp(pk);
            const int r = k + 1 + rr;
            if (r < o) {
                const int p = r == bi ? pc[k] : pc[r];
                if (q == 0) pn[r] = p;
                const float4 lq = md[p * o + k];
                const float4 l = zdf_mul(make_float4(lq.x, lq.z, lq.y, lq.w), rpd);
                // -l broadcast: (-l.re, -l.re) and (l.im, -l.im), so that the two products sum to -l u
                const float2 ah = make_float2(-l.x, -l.x), nah = make_float2(l.x, l.x), al = make_float2(-l.y, -l.y);
                const float2 bh = make_float2(l.z, -l.z), nbh = make_float2(-l.z, l.z), bl = make_float2(l.w, -l.w);
                for (int j = k + 1 + q; j < o; j += 4) {
                    const float4 u = md[pr * o + j];
                    const dfc t = dfc_add(dfc_mul_b(ah, nah, al, make_float2(u.x, u.y), make_float2(u.z, u.w)),
                                          dfc_mul_b(bh, nbh, bl, make_float2(u.y, u.x), make_float2(u.w, u.z)));
                    const dfc v = dfc_add(dfc_of(md[p * o + j]), t);
                    md[p * o + j] = dfc_f4(v);
                    if (j == k + 1) atomicMax(&s_key[0][(k + 1) % 3], piv_key(fabsf(v.h.x) + fabsf(v.h.y), r));
                }
            }
            group_bar(1);
        }
        if (tid == 0 && ovlp_out) ovlp_out[w] = zero ? make_double2(0.0, 0.0) : cmul(det, det);
    } else {  // Gauss-Jordan (fp32)
        const int t = tid - 128, rr = t >> 2, q = t & 3;
        for (int k = 0; k < o; ++k) {
            const int* pc = s_perm[1][k & 1];
            int* pn = s_perm[1][(k + 1) & 1];
            const int bi = piv_row(s_key[1][k % 3]);
            const int pr = pc[bi];
            const float2 pv = X[pr * o2 + k];
            const float den = pv.x * pv.x + pv.y * pv.y;
            const float2 rp = make_float2(pv.x / den, -pv.y / den);
            if (t == 0) {
                s_key[1][(k + 2) % 3] = 0ull;
                s_pf[k] = pr;
                s_rp[k] = rp;
            }
            if (rr < o - 1) {
                const int r = rr < k ? rr : rr + 1;  // every logical row but k
                const int p = r < k ? s_pf[r] : (r == bi ? pc[k] : pc[r]);
                if (q == 0 && r > k) pn[r] = p;
                const float2 x = X[p * o2 + k];
                const float2 f = make_float2(x.x * rp.x - x.y * rp.y, x.x * rp.y + x.y * rp.x);
                for (int c = k + 1 + q; c < o2; c += 4) {
                    const float2 u = X[pr * o2 + c], y = X[p * o2 + c];
                    const float2 v = make_float2(y.x - (f.x * u.x - f.y * u.y), y.y - (f.x * u.y + f.y * u.x));
                    X[p * o2 + c] = v;
                    if (c == k + 1 && r > k && c < o)
                        atomicMax(&s_key[1][(k + 1) % 3], piv_key(fabsf(v.x) + fabsf(v.y), r));
                }
            }
            group_bar(2);
        }
    }
    __syncthreads();
    {  // row a of m^-1 = (physical row pf[a] of the right half) / pivot_a, packed at stride IS
        float2 t4[4];  // o * o <= 4 x 256
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int e = tid + 256 * u;
            if (e < o * o) {
                const int a = e / o, b = e - a * o;
                const float2 x = X[s_pf[a] * o2 + o + b], rp = s_rp[a];
                t4[u] = make_float2(x.x * rp.x - x.y * rp.y, x.x * rp.y + x.y * rp.x);
            }
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int e = tid + 256 * u;
            if (e < o * o) inv[(e / o) * IS + e % o] = t4[u];
        }
        for (int e = tid; e < o * (IS - o); e += blockDim.x) inv[(e / (IS - o)) * IS + o + e % (IS - o)] = make_float2(0.f, 0.f);
    }

    // G_half[b, i] = sum_a W[i, a] inv[a, b] in fp32 -> split operand / green_out: a thread takes row il of
    // a chunk and columns b0..b0+3; with W staged as (re, re, im, im) the products accumulate as pairs
    //   A[b] += re W[i, a] inv[a, b],  B[b] += im W[i, a] inv[a, b]   (f32x2 fma, broadcast factors)
    // and G_half[b, i] = (A.re - B.im, A.im + B.re).
    const double2* Wp = walkers + (size_t)w * n * o;
    __nv_bfloat16* re_row = split.ptr ? split.ptr + (size_t)w * split.ld : nullptr;
    __nv_bfloat16* im_row = split.ptr ? split.ptr + (size_t)(split.W + w) * split.ld : nullptr;
    double2* Gp = green_out ? green_out + (size_t)w * o * n : nullptr;
    const int il = tid & 31, b0 = 4 * (tid >> 5);
    for (int i0 = 0; i0 < n; i0 += OG_CH) {
        const int rows = min(OG_CH, n - i0);
        __syncthreads();
        for (int e = tid; e < rows * o; e += blockDim.x) {
            const double2 x = Wp[(size_t)i0 * o + e];
            const float xr = d2f_trunc(x.x), xi = d2f_trunc(x.y);
            wf[(e / o) * ws + e % o] = make_float4(xr, xr, xi, xi);
        }
        __syncthreads();
        if (b0 >= o || il >= rows) continue;
        float2 A[4], B[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) A[j] = B[j] = make_float2(0.f, 0.f);
        const float4* xp = wf + il * ws;
#pragma unroll 2
        for (int a = 0; a < o; ++a) {
            const float4 x = xp[a];
            const float4 va = *(const float4*)(inv + a * IS + b0), vb = *(const float4*)(inv + a * IS + b0 + 2);
            const float2 xr = make_float2(x.x, x.y), xi = make_float2(x.z, x.w);
            const float2 v[4] = {make_float2(va.x, va.y), make_float2(va.z, va.w), make_float2(vb.x, vb.y),
                                 make_float2(vb.z, vb.w)};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                A[j] = __ffma2_rn(xr, v[j], A[j]);
                B[j] = __ffma2_rn(xi, v[j], B[j]);
            }
        }
        const int i = i0 + il;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int b = b0 + j;
            if (b < o) {
                const float gr = A[j].x - B[j].y, gi = A[j].y + B[j].x;
                if (re_row) {
                    split_storef(re_row, split.S, b * n + i, gr, true, split.sec);
                    split_storef(im_row, split.S, b * n + i, gi, true, split.sec);
                }
                if (Gp) Gp[(size_t)b * n + i] = make_double2(gr, gi);
            }
        }
    }
    if (!re_row) return;
    for (int e = n * o + tid; e < split.S; e += blockDim.x) {
        split_storef(re_row, split.S, e, 0.f, true, split.sec);
        split_storef(im_row, split.S, e, 0.f, true, split.sec);
    }
    for (long long e = (long long)split.sec * split.S + tid; e < split.ld; e += blockDim.x) {
        re_row[e] = __float2bfloat16(0.f);
        im_row[e] = __float2bfloat16(0.f);
    }
}

int launch_overlap_split(int W, int n, int o, const double2* mo, const double2* walkers, double2* ovlp_out,
                         SplitOut split, cudaStream_t s, double2* green_out, const float2* cs, const float4* m_in) {
    if (W <= 0) return AFQ_OK;
    const size_t base = (size_t)o * o * sizeof(double2) + 2 * (size_t)o * o * sizeof(float2);
    const size_t wbytes = (size_t)n * o * sizeof(float2);
    const size_t dfbytes = 2 * (size_t)OS_CH * o * sizeof(float2);
    if (m_in) {  // m given (double-float)
        if (o > 32) return fail(AFQ_E_UNSUPPORTED, "overlap from a given m: nocc=%d > 32", o);
        const size_t sm = (size_t)og_a16(o) * sizeof(float4) + (size_t)og_xs(o) * sizeof(float2);
        AFQ_TRY(smem_attr(k_overlap_oz, sm));
        k_overlap_oz<<<W, 256, sm, s>>>(n, o, m_in, walkers, ovlp_out, split, green_out);
        AFQ_LAUNCHED("k_overlap_oz");
        return AFQ_OK;
    }
    const bool df = cs != nullptr;        // double-float m, W staged in chunks
    const bool stage = df || base + wbytes <= 160 * 1024;  // else read W from global in the last loop
    const size_t smem = base + (df ? dfbytes : stage ? wbytes : 0);
    const int ag = 256 / o, ma = (o + ag - 1) / ag;
#define AFQ_OS(MAV)                                                                                              \
    do {                                                                                                         \
        if (df) {                                                                                                \
            AFQ_TRY(smem_attr(k_overlap_split<MAV, true, true>, smem));                                          \
            k_overlap_split<MAV, true, true><<<W, 256, smem, s>>>(n, o, mo, walkers, ovlp_out, split, green_out,   \
                                                                 cs);                                            \
        } else if (stage) {                                                                                      \
            AFQ_TRY(smem_attr(k_overlap_split<MAV, true, false>, smem));                                         \
            k_overlap_split<MAV, true, false><<<W, 256, smem, s>>>(n, o, mo, walkers, ovlp_out, split, green_out,  \
                                                                  nullptr);                                      \
        } else {                                                                                                 \
            AFQ_TRY(smem_attr(k_overlap_split<MAV, false, false>, smem));                                        \
            k_overlap_split<MAV, false, false><<<W, 256, smem, s>>>(n, o, mo, walkers, ovlp_out, split, green_out, \
                                                                   nullptr);                                     \
        }                                                                                                        \
    } while (0)
    if (ma <= 1) AFQ_OS(1);
    else if (ma <= 2) AFQ_OS(2);
    else if (ma <= 4) AFQ_OS(4);
    else if (ma <= 8) AFQ_OS(8);
    else AFQ_OS(16);
#undef AFQ_OS
    AFQ_LAUNCHED("k_overlap_split");
    return AFQ_OK;
}

// ---------------------------------------------------- orthonormalisation --
// Mixed-form QR with the reference's output (walkers.py:169-211: the unique
// Q with diag(R) real and > 0), by CholeskyQR2 in shared memory, one CTA per
// walker, with the walker held as fp32 pairs x = x_hi + x_lo (48 significant
// bits) and its products formed in double-float arithmetic on the fp32 pipe
// (df_acc2: TwoProd + TwoSum), which runs ~64x the binary64 rate here:
//   pass 1: G1 = W_hi^H W_hi in fp32, R1 = chol(G1) in binary64,
//           X = W R1^-1 by double-float forward substitution;
//   pass 2: G2 = X^H X in double-float, R2 = chol(G2) in binary64,
//           Q = X R2^-1 in double-float, widened to binary64.
// X spans W's columns to ~2^-44 whatever the error of R1 (R1 only
// preconditions), and pass 2 restores orthonormality; Q = W (R2 R1)^-1 with
// R2 R1 upper triangular with a positive real diagonal, the Householder
// form's Q.  If a pivot of the fp32 Gram matrix falls below 1e-5 of its
// column's squared norm (cond(W) beyond ~300, where fp32 rounding would
// leave X far from orthonormal), G1 is recomputed in double-float.  A
// numerically rank-deficient W (a non-positive pivot) gets the pivot 1 and a
// zero row of R there, so the output stays finite; such a walker has a
// vanishing overlap and no weight.

// Upper-triangle entry e (row-major) -> (j, k), j <= k.
__device__ __forceinline__ void cq_entry(int o, int e, int& j, int& k) {
    j = 0;
    while (e >= o - j) { e -= o - j; ++j; }
    k = j + e;
}

// Gram matrix of the columns of A = Ah + Al (column-major, leading dim ld)
// into Gm (upper triangle, binary64): from Ah alone in fp32 (DF false) or in
// double-float (DF true).
template <bool DF>
__device__ __forceinline__ void cq_gram(int n, int o, int ld, const float2* Ah, const float2* Al, double2* Gm) {
    const int P = o * (o + 1) / 2;
    for (int e = threadIdx.x; e < P; e += blockDim.x) {
        int j, k;
        cq_entry(o, e, j, k);
        const float2* ah = Ah + (size_t)j * ld;
        const float2* bh = Ah + (size_t)k * ld;
        float sr = 0.f, si = 0.f;
        if (DF) {
            const float2* al = Al + (size_t)j * ld;
            const float2* bl = Al + (size_t)k * ld;
            // conj(a) b: (Re, Im) += a_r (b_r, b_i) + a_i (b_i, -b_r), in two chains (even / odd i)
            float2 s2 = make_float2(0.f, 0.f), e2 = s2, s3 = s2, e3 = s2;
            int i = 0;
            for (; i + 1 < n; i += 2) {
                const float2 xh = ah[i], xl = al[i], yh = bh[i], yl = bl[i];
                const float2 xh1 = ah[i + 1], xl1 = al[i + 1], yh1 = bh[i + 1], yl1 = bl[i + 1];
                df_acc2(s2, e2, xh.x, xl.x, yh, yl);
                df_acc2(s3, e3, xh1.x, xl1.x, yh1, yl1);
                df_acc2(s2, e2, xh.y, xl.y, make_float2(yh.y, -yh.x), make_float2(yl.y, -yl.x));
                df_acc2(s3, e3, xh1.y, xl1.y, make_float2(yh1.y, -yh1.x), make_float2(yl1.y, -yl1.x));
            }
            if (i < n) {
                const float2 xh = ah[i], xl = al[i], yh = bh[i], yl = bl[i];
                df_acc2(s2, e2, xh.x, xl.x, yh, yl);
                df_acc2(s2, e2, xh.y, xl.y, make_float2(yh.y, -yh.x), make_float2(yl.y, -yl.x));
            }
            df_add2(s2, e2, s3, e3);
            Gm[j * o + k] = make_double2((double)s2.x + (double)e2.x, (double)s2.y + (double)e2.y);
        } else {
            for (int i = 0; i < n; ++i) {
                const float2 x = ah[i], y = bh[i];
                sr = fmaf(x.x, y.x, fmaf(x.y, y.y, sr));
                si = fmaf(x.x, y.y, fmaf(-x.y, y.x, si));
            }
            Gm[j * o + k] = make_double2(sr, si);
        }
    }
}

// In-place upper Cholesky G = R^H R of the upper triangle of Gm (row-major,
// R[k][j] at Gm[k o + j]); thread 0 multiplies the pivots into *det.
// Returns (uniformly) whether a pivot was not above rel_tol times the
// column's diagonal entry before elimination (d0, o entries of scratch); such
// a pivot becomes 1 with a zero row.  Thread 0 takes each pivot's square
// root and reciprocal and hands them to the block through piv[2] (a
// negative reciprocal marks a rejected pivot).
__device__ __forceinline__ bool cq_chol(int o, double2* Gm, double* det, double rel_tol, double* d0,
                                        double* piv) {
    for (int k = threadIdx.x; k < o; k += blockDim.x) d0[k] = Gm[k * o + k].x;
    __syncthreads();
    bool bad = false;
    for (int k = 0; k < o; ++k) {
        if (threadIdx.x == 0) {
            const double gkk = Gm[k * o + k].x;
            const bool b = !(gkk > rel_tol * d0[k]) || !(gkk > 0.0);
            const double r = b ? 1.0 : sqrt(gkk);
            *det *= r;
            piv[0] = r;
            piv[1] = b ? -1.0 : 1.0 / r;
        }
        __syncthreads();
        const double rkk = piv[0], ir = piv[1];
        const bool b = ir < 0.0;
        bad |= b;
        for (int j = k + threadIdx.x; j < o; j += blockDim.x) {
            const double2 g = Gm[k * o + j];
            Gm[k * o + j] = j == k ? make_double2(rkk, 0.0) : (b ? make_double2(0.0, 0.0) : cscale(g, ir));
        }
        __syncthreads();
        const int m = o - k - 1;
        for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
            const int i = k + 1 + e / m, j = k + 1 + e % m;
            if (i <= j) Gm[i * o + j] = csub(Gm[i * o + j], cmulc(Gm[k * o + i], Gm[k * o + j]));
        }
        __syncthreads();
    }
    return bad;
}

// R (upper triangle of Gm, binary64) as double-float pairs for the solve, in
// place (Rd aliases Gm; each entry is read and rewritten by one thread):
// Rd[j o + k] = (re hi, re lo, im hi, im lo); rinv[k] = (hi, lo) of 1 / R_kk.
__device__ __forceinline__ void cq_rsplit(int o, double2* Gm, float4* Rd, float2* rinv) {
    for (int e = threadIdx.x; e < o * o; e += blockDim.x) {
        const double2 r = Gm[e];
        if (e % (o + 1) == 0) {
            const double v = 1.0 / r.x;
            const float h = (float)v;
            rinv[e / (o + 1)] = make_float2(h, (float)(v - (double)h));
        }
        const float rh = (float)r.x, ih = (float)r.y;
        Rd[e] = make_float4(rh, (float)(r.x - (double)rh), ih, (float)(r.y - (double)ih));
    }
    __syncthreads();
}

// A <- A R^-1 in place in double-float, one thread per row of A.
__device__ __forceinline__ void cq_solve(int n, int o, int ld, float2* Ah, float2* Al, const float4* Rd,
                                         const float2* rinv) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        for (int k = 0; k < o; ++k) {
            const float2 ah = Ah[(size_t)k * ld + i], al = Al[(size_t)k * ld + i];
            float2 s2 = ah, e2 = al;  // (Re, Im) and their error terms: even j here, odd j in (s3, e3)
            float2 s3 = make_float2(0.f, 0.f), e3 = s3;
            // a -= x r: (Re, Im) += -x_r (r_r, r_i) + x_i (r_i, -r_r)
            int j = 0;
            for (; j + 1 < k; j += 2) {
                const float2 xh = Ah[(size_t)j * ld + i], xl = Al[(size_t)j * ld + i];
                const float2 xh1 = Ah[(size_t)(j + 1) * ld + i], xl1 = Al[(size_t)(j + 1) * ld + i];
                const float4 r = Rd[j * o + k], r1 = Rd[(j + 1) * o + k];
                df_acc2(s2, e2, -xh.x, -xl.x, make_float2(r.x, r.z), make_float2(r.y, r.w));
                df_acc2(s3, e3, -xh1.x, -xl1.x, make_float2(r1.x, r1.z), make_float2(r1.y, r1.w));
                df_acc2(s2, e2, xh.y, xl.y, make_float2(r.z, -r.x), make_float2(r.w, -r.y));
                df_acc2(s3, e3, xh1.y, xl1.y, make_float2(r1.z, -r1.x), make_float2(r1.w, -r1.y));
            }
            if (j < k) {
                const float2 xh = Ah[(size_t)j * ld + i], xl = Al[(size_t)j * ld + i];
                const float4 r = Rd[j * o + k];
                df_acc2(s2, e2, -xh.x, -xl.x, make_float2(r.x, r.z), make_float2(r.y, r.w));
                df_acc2(s2, e2, xh.y, xl.y, make_float2(r.z, -r.x), make_float2(r.w, -r.y));
            }
            df_add2(s2, e2, s3, e3);
            const float sr = s2.x, er = e2.x, si = s2.y, ei = e2.y;
            const float2 q = rinv[k];  // x = (s + e) q, renormalised to a pair
            float2 h, l;
            {
                const float p = __fmul_rn(sr, q.x);
                const float t = __fadd_rn(__fmaf_rn(sr, q.x, -p), __fmaf_rn(sr, q.y, __fmul_rn(er, q.x)));
                h.x = __fadd_rn(p, t);
                l.x = __fsub_rn(t, __fsub_rn(h.x, p));
            }
            {
                const float p = __fmul_rn(si, q.x);
                const float t = __fadd_rn(__fmaf_rn(si, q.x, -p), __fmaf_rn(si, q.y, __fmul_rn(ei, q.x)));
                h.y = __fadd_rn(p, t);
                l.y = __fsub_rn(t, __fsub_rn(h.y, p));
            }
            Ah[(size_t)k * ld + i] = h;
            Al[(size_t)k * ld + i] = l;
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(256, 2) k_cholqr2(int n, int o, const double2* __restrict__ win,
                                                    double2* __restrict__ wout, double2* __restrict__ det_out) {
    extern __shared__ double2 csm[];
    __shared__ double s_det;  // prod diag(R1) prod diag(R2) = prod diag(R)
    __shared__ double s_d0[64];
    __shared__ double s_piv[2];
    const int ld = n | 1;
    double2* Gm = csm;                                // o x o binary64 Gram matrix, then R
    float4* Rd = (float4*)Gm;                         // o x o double-float R, in place of Gm
    float2* rinv = (float2*)(Gm + o * o);             // o
    float2* Ah = rinv + ((o + 1) & ~1);               // ld x o: A[j ld + i] = W[i, j], hi
    float2* Al = Ah + (size_t)ld * o;                 // lo
    const int w = blockIdx.x;
    const double2* Wp = win + (size_t)w * n * o;
    constexpr int LU = 8;  // loads in flight per thread
    for (int e0 = 0; e0 < n * o; e0 += LU * blockDim.x) {
        double2 x[LU];
#pragma unroll
        for (int u = 0; u < LU; ++u) {
            const int e = e0 + u * blockDim.x + threadIdx.x;
            if (e < n * o) x[u] = Wp[e];
        }
#pragma unroll
        for (int u = 0; u < LU; ++u) {
            const int e = e0 + u * blockDim.x + threadIdx.x;
            if (e < n * o) {
                const float2 re = split_d2f(x[u].x), im = split_d2f(x[u].y);
                const size_t d = (size_t)(e % o) * ld + e / o;
                Ah[d] = make_float2(re.x, im.x);
                Al[d] = make_float2(re.y, im.y);
            }
        }
    }
    if (threadIdx.x == 0) s_det = 1.0;
    __syncthreads();
    cq_gram<false>(n, o, ld, Ah, Al, Gm);
    __syncthreads();
    if (cq_chol(o, Gm, &s_det, 1e-5, s_d0, s_piv)) {  // fp32 cannot resolve W's conditioning: double-float G1
        if (threadIdx.x == 0) s_det = 1.0;
        cq_gram<true>(n, o, ld, Ah, Al, Gm);
        __syncthreads();
        cq_chol(o, Gm, &s_det, 0.0, s_d0, s_piv);
    }
    cq_rsplit(o, Gm, Rd, rinv);
    cq_solve(n, o, ld, Ah, Al, Rd, rinv);
    cq_gram<true>(n, o, ld, Ah, Al, Gm);
    __syncthreads();
    cq_chol(o, Gm, &s_det, 0.0, s_d0, s_piv);
    cq_rsplit(o, Gm, Rd, rinv);
    cq_solve(n, o, ld, Ah, Al, Rd, rinv);
    double2* Wo = wout + (size_t)w * n * o;
    for (int e = threadIdx.x; e < n * o; e += blockDim.x) {
        const size_t d = (size_t)(e % o) * ld + e / o;
        const float2 h = Ah[d], l = Al[d];
        Wo[e] = make_double2(f2d_exact(h.x) + f2d_exact(l.x), f2d_exact(h.y) + f2d_exact(l.y));
    }
    if (det_out && threadIdx.x == 0) det_out[w] = make_double2(s_det, 0.0);
}

int launch_cholqr2(int W, int n, int o, const double2* win, double2* wout, double2* det_r, cudaStream_t s) {
    if (W <= 0) return AFQ_OK;
    if (o > 64) return fail(AFQ_E_UNSUPPORTED, "qr: nocc=%d > 64", o);
    const size_t smem = (size_t)o * o * sizeof(double2) + (size_t)((o + 1) & ~1) * sizeof(float2) +
                        2 * (size_t)(n | 1) * o * sizeof(float2);
    // walkers whose double-float copy does not fit in shared memory: the binary64 Householder QR
    if (smem > 220 * 1024) return launch_qr(W, n, o, win, wout, det_r, s);
    AFQ_TRY(smem_attr(k_cholqr2, smem));
    k_cholqr2<<<W, 256, smem, s>>>(n, o, win, wout, det_r);
    AFQ_LAUNCHED("k_cholqr2");
    return AFQ_OK;
}

// ------------------------------------------------------------------ energy
// Mixed energy (meas/rhf.py:36-50) for a chunk of walkers: the tensor-core
// GEMM produced F[(w, part, k), (g, i)] = sum_j G_part[w, k, j] L~[g, i, j]
// (part 0 = Re, 1 = Im of G_half), so each walker's f_g blocks lie along
// contiguous runs of a row; this kernel forms, per walker and chunk of
// Cholesky vectors, sum_g c_g^2 and sum_g sum_ik f_g[i,k] f_g[k,i].
// The chunk's rows are copied into shared memory as they lie in F (plane
// part, row k, column g o + i = f_g[i,k]) by cp.async, all copies in flight
// at once.  The fp32 products are summed in fp32 per thread (EX_G o^2 / 256
// terms, ~28) and per warp; the warp sums accumulate in fp64.
constexpr int EX_G = 8;  // Cholesky vectors per CTA
__global__ void __launch_bounds__(256) k_exchange_reduce(int G, int o, const float* __restrict__ F, long long ldf,
                                                         double2* __restrict__ partial, int nchunk, int v16) {
    extern __shared__ float fsm[];  // [part][k][RS]: RS = EX_G o + 4 (16-byte rows, shifted banks)
    const int w = blockIdx.y, g0 = blockIdx.x * EX_G;
    const int ng = min(EX_G, G - g0);
    const int oo = o * o, nc = ng * o, RS = EX_G * o + 4;
    float* Pr = fsm;
    float* Pi = fsm + o * RS;
    const float* Fr = F + (long long)(2 * w) * o * ldf + (long long)g0 * o;
    const float* Fi = F + (long long)(2 * w + 1) * o * ldf + (long long)g0 * o;
    if (v16 && (nc & 3) == 0) {
        const int q = nc / 4;  // 16-byte chunks per row
        for (int e = threadIdx.x; e < 2 * o * q; e += blockDim.x) {
            const int c = e % q, r = e / q, part = r / o, k = r % o;
            cp_async16((part ? Pi : Pr) + k * RS + 4 * c, (part ? Fi : Fr) + (long long)k * ldf + 4 * c);
        }
    } else {
        for (int e = threadIdx.x; e < 2 * o * nc; e += blockDim.x) {
            const int c = e % nc, r = e / nc, part = r / o, k = r % o;
            cp_async4((part ? Pi : Pr) + k * RS + c, (part ? Fi : Fr) + (long long)k * ldf + c);
        }
    }
    cp_async_commit();
    // this thread's (i, k) entries, the same for every g: offsets of f[i,k] and f[k,i]
    constexpr int EX_R = 64 * 64 / 256;  // nocc <= 64
    int oa[EX_R], ob[EX_R];
#pragma unroll
    for (int j = 0; j < EX_R; ++j) {
        const int r = threadIdx.x + 256 * j, i = r / o, k = r % o;
        oa[j] = r < oo ? k * RS + i : -1;  // f[i,k] at row k, column i
        ob[j] = i * RS + k;                // f[k,i] at row i, column k
    }
    cp_async_wait_all();
    __syncthreads();
    double cr = 0.0, ci = 0.0;
    float sr = 0.f, si = 0.f;
    for (int g = 0; g < ng; ++g) {
        const float* fr = Pr + g * o;
        const float* fi = Pi + g * o;
#pragma unroll
        for (int j = 0; j < EX_R; ++j) {
            if (oa[j] >= 0) {
                const float ar = fr[oa[j]], ai = fi[oa[j]], br = fr[ob[j]], bi = fi[ob[j]];
                sr = fmaf(ar, br, fmaf(-ai, bi, sr));
                si = fmaf(ar, bi, fmaf(ai, br, si));
            }
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, off);
        si += __shfl_xor_sync(0xffffffffu, si, off);
    }
    const double xr = (double)sr, xi = (double)si;
    for (int g = threadIdx.x; g < ng; g += blockDim.x) {
        double tr = 0.0, ti = 0.0;
        for (int i = 0; i < o; ++i) {
            tr += Pr[i * RS + g * o + i];
            ti += Pi[i * RS + g * o + i];
        }
        cr += tr * tr - ti * ti;
        ci += 2.0 * tr * ti;
    }
    __shared__ double red[4][8];
    if (threadIdx.x < 32) { cr = warp_sum(cr); ci = warp_sum(ci); }  // the c_g sums live in warp 0 (ng <= 32)
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

// The exchange-fused energy GEMM's outputs (launch_tc_gemm_exchange) to the
// partials of k_exchange_reduce with one chunk: partial[w 2] = sum_g c_g^2,
// partial[w 2 + 1] = (sum_g Re sum_ik f_g[i,k] f_g[k,i], 0); one warp per
// walker, fixed summation order.  Only the real part of the exchange is
// formed: the block measurement reads Re E_loc (prop/blocks.py:63).
__global__ void k_exchange_finish(int nw, int G, int nhalf, const float* __restrict__ x, const float* __restrict__ c,
                                  double2* __restrict__ partial) {
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (w >= nw) return;
    double cr = 0.0, ci = 0.0, xr = 0.0;
    for (int g = lane; g < G; g += 32) {
        const double tr = c[((size_t)w * G + g) * 2], ti = c[((size_t)w * G + g) * 2 + 1];
        cr += tr * tr - ti * ti;
        ci += 2.0 * tr * ti;
    }
    for (int h = lane; h < nhalf; h += 32)
        xr += (double)x[((size_t)w * nhalf + h) * 2] - (double)x[((size_t)w * nhalf + h) * 2 + 1];
    cr = warp_sum(cr);
    ci = warp_sum(ci);
    xr = warp_sum(xr);
    if (lane == 0) {
        partial[(size_t)w * 2] = make_double2(cr, ci);
        partial[(size_t)w * 2 + 1] = make_double2(xr, 0.0);
    }
}

int launch_exchange_finish(int nw, int G, const float* x, const float* c, double2* partial, cudaStream_t s) {
    if (nw <= 0) return AFQ_OK;
    k_exchange_finish<<<(nw + 7) / 8, 256, 0, s>>>(nw, G, exchange_halves(G), x, c, partial);
    AFQ_LAUNCHED("k_exchange_finish");
    return AFQ_OK;
}

int launch_exchange_reduce(int wc, int G, int o, const float* F, long long ldf, double2* partial, cudaStream_t s) {
    if (wc <= 0) return AFQ_OK;
    const size_t smem = (size_t)2 * o * (EX_G * o + 4) * sizeof(float);
    AFQ_TRY(smem_attr(k_exchange_reduce, smem));
    const int v16 = (ldf % 4) == 0 && (((uintptr_t)F) & 15) == 0;
    dim3 grid(exchange_chunks(G), wc);
    k_exchange_reduce<<<grid, 256, smem, s>>>(G, o, F, ldf, partial, exchange_chunks(G), v16);
    AFQ_LAUNCHED("k_exchange_reduce");
    return AFQ_OK;
}

// (hi, lo) fp32 pair of each real trial orbital coefficient, for the
// double-float overlap.
__global__ void k_split_c(int count, const double2* __restrict__ mo, float2* __restrict__ cs) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
        const double c = mo[e].x;
        const float h = (float)c;
        cs[e] = make_float2(h, (float)(c - (double)h));
    }
}

int launch_split_c(int count, const double2* mo, float2* cs, cudaStream_t s) {
    k_split_c<<<(count + 255) / 256, 256, 0, s>>>(count, mo, cs);
    AFQ_LAUNCHED("k_split_c");
    return AFQ_OK;
}

// Green's function rows for the energy GEMM: row (w*2 + part)*P + k holds
// split(G_part[w, k, :]) with K = n in sections of S; rows k >= o (P > o,
// the exchange-fused layout) are zero.
__global__ void k_green_rows(int wc, int n, int o, int P, const double2* __restrict__ green,
                             __nv_bfloat16* __restrict__ dst, int S, int Kt, int sec) {
    const long long rows = (long long)wc * P * 2;
    const long long total = rows * (long long)Kt;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / Kt;
        const int kk = (int)(e % Kt);
        __nv_bfloat16* row = dst + r * Kt;
        const int k = (int)(r % P), part = (int)((r / P) % 2), w = (int)(r / (2 * P));
        if (kk < S) {
            double x = 0.0;
            if (kk < n && k < o) {
                const double2 v = green[((size_t)w * o + k) * n + kk];
                x = part ? v.y : v.x;
            }
            split_store(row, S, kk, x, false, sec);
        } else if (kk >= sec * S) {
            row[kk] = __double2bfloat16(0.0);
        }
    }
}

int launch_green_rows(int wc, int n, int o, int P, const double2* green, __nv_bfloat16* dst, int S, int Kt, int sec,
                      cudaStream_t s) {
    const long long total = (long long)wc * P * 2 * Kt;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    k_green_rows<<<(unsigned)blocks, 256, 0, s>>>(wc, n, o, P, green, dst, S, Kt, sec);
    AFQ_LAUNCHED("k_green_rows");
    return AFQ_OK;
}

}  // namespace afq
