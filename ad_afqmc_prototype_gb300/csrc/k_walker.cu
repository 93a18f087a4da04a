// Per-walker binary64 kernels of the AFQMC step and block.
//
// Layouts: walkers (W, n, o) complex, row-major; G_half (W, o, n) complex;
// fields / shifted fields (W, G); chol (G, n, n) real; rot_chol (G, o, n)
// real (real trial) or complex.
#include "afq_internal.cuh"

namespace afq {

template <class K>
static int set_smem(K kernel, size_t bytes) {
    if (bytes > 227 * 1024) return fail(AFQ_E_UNSUPPORTED, "kernel needs %zu bytes of shared memory", bytes);
    if (bytes > 32 * 1024)  // with the kernel's static shared memory the default limit is below 48 KB
        AFQ_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return AFQ_OK;
}

// =====================================================================
// Overlap matrix, determinant and half-rotated Green's function.
//   m = C^H W (o x o); Gauss-Jordan with partial pivoting gives det(m) and
//   m^-1; overlap = det(m)^2 (meas/rhf.py:22-24); G_half^T = W m^-1, i.e.
//   G_half = solve(m^T, W^T) (meas/rhf.py:15-19).  One CTA per walker.
// =====================================================================
template <bool CR, int MA>
__global__ void __launch_bounds__(256) k_green(int n, int o, const double2* __restrict__ mo,
                                               const double2* __restrict__ walkers,
                                               double2* __restrict__ ovlp_out,
                                               double2* __restrict__ green_out, SplitOut split, int ov_square) {
    extern __shared__ double2 sm[];
    double2* m = sm;          // o x o
    double2* inv = sm + o * o;  // o x o
    __shared__ int s_piv, s_zero;
    __shared__ double2 s_det;
    const int w = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const double2* Wp = walkers + (size_t)w * n * o;

    // m[a, b] = sum_i conj(C[i, a]) W[i, b]: thread <-> column b and rows
    // a = ag + AG k, so each thread streams its column of W once (coalesced
    // across b) and takes C from L1.
    {
        // MA >= ceil(o / AG) rows per thread, a template argument so that the
        // accumulators stay in registers without inflating smaller cases
        const int AG = blockDim.x / o;
        const int b = tid % o, ag = tid / o;
        double2 acc[MA];
#pragma unroll
        for (int k = 0; k < MA; ++k) acc[k] = make_double2(0.0, 0.0);
        if (ag < AG) {
            for (int i = 0; i < n; ++i) {
                const double2 x = Wp[(size_t)i * o + b];
#pragma unroll
                for (int k = 0; k < MA; ++k) {
                    const int a = ag + AG * k;
                    if (a < o) {
                        const double2 c = mo[i * o + a];
                        if (CR) {
                            rfma(acc[k], c.x, x);
                        } else {
                            acc[k].x = fma(c.x, x.x, acc[k].x); acc[k].x = fma(c.y, x.y, acc[k].x);
                            acc[k].y = fma(c.x, x.y, acc[k].y); acc[k].y = fma(-c.y, x.x, acc[k].y);
                        }
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < MA; ++k) {
                const int a = ag + AG * k;
                if (a < o) m[a * o + b] = acc[k];
            }
        }
        for (int e = tid; e < o * o; e += blockDim.x)
            inv[e] = make_double2((e / o) == (e % o) ? 1.0 : 0.0, 0.0);
    }
    if (tid == 0) {
        s_det = make_double2(1.0, 0.0);
        s_zero = 0;
    }
    __syncthreads();

    for (int k = 0; k < o; ++k) {
        if (wid == 0) {
            double best = -1.0;
            int bi = k;
            for (int r = k + lane; r < o; r += 32) {
                double v = cabs2(m[r * o + k]);
                if (v > best) { best = v; bi = r; }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                double ob = __shfl_xor_sync(0xffffffffu, best, off);
                int oi = __shfl_xor_sync(0xffffffffu, bi, off);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (lane == 0) s_piv = bi;
        }
        __syncthreads();
        const int p = s_piv;
        if (p != k) {
            for (int j = tid; j < 2 * o; j += blockDim.x) {
                double2* X = j < o ? m : inv;
                int jj = j < o ? j : j - o;
                double2 t = X[k * o + jj];
                X[k * o + jj] = X[p * o + jj];
                X[p * o + jj] = t;
            }
        }
        __syncthreads();
        const double2 piv = m[k * o + k];
        if (tid == 0) {
            double2 d = cmul(s_det, piv);
            s_det = (p != k) ? make_double2(-d.x, -d.y) : d;
            if (piv.x == 0.0 && piv.y == 0.0) s_zero = 1;
        }
        const double2 rp = cdiv(make_double2(1.0, 0.0), piv);
        __syncthreads();
        // scale pivot row (columns > k of m, all of inv)
        for (int j = tid; j < 2 * o; j += blockDim.x) {
            if (j < o) { if (j > k) m[k * o + j] = cmul(m[k * o + j], rp); }
            else inv[k * o + (j - o)] = cmul(inv[k * o + (j - o)], rp);
        }
        __syncthreads();
        // eliminate column k from every other row (column k of m is left as is)
        for (int e = tid; e < o * 2 * o; e += blockDim.x) {
            int r = e / (2 * o), j = e % (2 * o);
            if (r == k) continue;
            double2 f = m[r * o + k];
            if (j < o) {
                if (j > k) m[r * o + j] = csub(m[r * o + j], cmul(f, m[k * o + j]));
            } else {
                inv[r * o + (j - o)] = csub(inv[r * o + (j - o)], cmul(f, inv[k * o + (j - o)]));
            }
        }
        __syncthreads();
    }
    // An exactly zero pivot (the rest of its column is zero too: m is singular)
    // makes det(m) exactly 0, as LAPACK's LU gives it (getrf leaves the zero
    // on U's diagonal); the division by it has made the inverse, and so the
    // Green's function, non-finite, as the reference's solve does.
    if (ovlp_out && tid == 0)
        ovlp_out[w] = s_zero ? make_double2(0.0, 0.0) : ov_square ? cmul(s_det, s_det) : s_det;
    if (!green_out && !split.ptr) return;
    // G_half[b, i] = sum_a W[i, a] inv[a, b]
    if (green_out) {
        double2* Gp = green_out + (size_t)w * o * n;
        for (int e = tid; e < n * o; e += blockDim.x) {
            int b = e / n, i = e % n;
            double2 acc = make_double2(0.0, 0.0);
            for (int a = 0; a < o; ++a) cfma(acc, Wp[i * o + a], inv[a * o + b]);
            Gp[e] = acc;
        }
    }
    if (!split.ptr) return;
    // Force-bias operand: the same product in fp32 (the bf16 hi/lo split that
    // consumes it resolves ~2^-17), written as the split left operand.
    __nv_bfloat16* re_row = split.ptr + (size_t)w * split.ld;
    __nv_bfloat16* im_row = split.ptr + (size_t)(split.W + w) * split.ld;
    float2* invf = (float2*)(inv + o * o);
    for (int e = tid; e < o * o; e += blockDim.x) invf[e] = make_float2((float)inv[e].x, (float)inv[e].y);
    __syncthreads();
    {
        constexpr int BG = 8;
        const int nbg = (o + BG - 1) / BG;
        for (int t = tid; t < n * nbg; t += blockDim.x) {
            const int i = t % n, bg = t / n;
            float2 acc[BG];
#pragma unroll
            for (int j = 0; j < BG; ++j) acc[j] = make_float2(0.f, 0.f);
            for (int a = 0; a < o; ++a) {
                const double2 wv = Wp[(size_t)i * o + a];
                const float2 x = make_float2((float)wv.x, (float)wv.y);
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
                    split_store(re_row, split.S, b * n + i, (double)acc[j].x, true, split.sec);
                    split_store(im_row, split.S, b * n + i, (double)acc[j].y, true, split.sec);
                }
            }
        }
    }
    {  // zero the section gaps and the tail of the row
        for (int e = n * o + tid; e < split.S; e += blockDim.x) {
            split_store(re_row, split.S, e, 0.0, true, split.sec);
            split_store(im_row, split.S, e, 0.0, true, split.sec);
        }
        for (long long e = (long long)split.sec * split.S + tid; e < split.ld; e += blockDim.x) {
            re_row[e] = __double2bfloat16(0.0);
            im_row[e] = __double2bfloat16(0.0);
        }
    }
}

int launch_green_split(int W, int n, int o, const double2* mo, int trial_real, const double2* walkers,
                       double2* ovlp_out, double2* green_out, SplitOut split, cudaStream_t s, int ov_square) {
    if (W <= 0) return AFQ_OK;
    size_t smem = 2 * (size_t)o * o * sizeof(double2) + (split.ptr ? (size_t)o * o * sizeof(float2) : 0);
    const int ag = 256 / o, ma = (o + ag - 1) / ag;  // rows of m per thread
#define AFQ_GREEN(CRV, MAV)                                                                  \
    do {                                                                                     \
        AFQ_TRY(set_smem(k_green<CRV, MAV>, smem));                                          \
        k_green<CRV, MAV><<<W, 256, smem, s>>>(n, o, mo, walkers, ovlp_out, green_out, split, ov_square); \
    } while (0)
#define AFQ_GREEN_MA(CRV)                \
    do {                                 \
        if (ma <= 1) AFQ_GREEN(CRV, 1);  \
        else if (ma <= 2) AFQ_GREEN(CRV, 2); \
        else if (ma <= 4) AFQ_GREEN(CRV, 4); \
        else if (ma <= 8) AFQ_GREEN(CRV, 8); \
        else AFQ_GREEN(CRV, 16);         \
    } while (0)
    if (trial_real) AFQ_GREEN_MA(true);
    else AFQ_GREEN_MA(false);
#undef AFQ_GREEN_MA
#undef AFQ_GREEN
    AFQ_LAUNCHED("k_green");
    return AFQ_OK;
}

int launch_green(int W, int n, int o, const double2* mo, int trial_real, const double2* walkers,
                 double2* ovlp_out, double2* green_out, cudaStream_t s) {
    return launch_green_split(W, n, o, mo, trial_real, walkers, ovlp_out, green_out, SplitOut{}, s, 1);
}

int launch_green_det(int W, int n, int o, const double2* mo, int trial_real, const double2* walkers,
                     double2* det_out, double2* green_out, cudaStream_t s) {
    return launch_green_split(W, n, o, mo, trial_real, walkers, det_out, green_out, SplitOut{}, s, 0);
}

// =====================================================================
// Trotter propagation  E_half . sum_{k<=K} (i sqrt_dt V)^k / k! . E_half . W
// (prop/chol_afqmc_ops.py:173-183, prop/utils.py:20-31).  Walker columns are
// independent, so a CTA owns (walker, OC columns): the current Taylor term
// lives in shared memory, the running sum in registers, and V / E_half are
// streamed through shared memory BJ columns at a time.
// =====================================================================
constexpr int TR_OC = 8, TR_BJ = 16, TR_THREADS = 256, TR_NRG = TR_THREADS / TR_OC;

template <int NR, bool REAL_M>
__device__ __forceinline__ void tr_matmul(int n, const void* __restrict__ Mg, const double2* __restrict__ T,
                                          double2* __restrict__ Ms, double2 (&acc)[NR], int c, int rg) {
#pragma unroll
    for (int q = 0; q < NR; ++q) acc[q] = make_double2(0.0, 0.0);
    double* Msr = (double*)Ms;
    for (int j0 = 0; j0 < n; j0 += TR_BJ) {
        const int jn = min(TR_BJ, n - j0);
        for (int e = threadIdx.x; e < n * TR_BJ; e += TR_THREADS) {
            int i = e / TR_BJ, jj = e % TR_BJ;
            if (REAL_M) Msr[e] = (jj < jn) ? ((const double*)Mg)[(size_t)i * n + j0 + jj] : 0.0;
            else Ms[e] = (jj < jn) ? ((const double2*)Mg)[(size_t)i * n + j0 + jj] : make_double2(0.0, 0.0);
        }
        __syncthreads();
        for (int jj = 0; jj < jn; ++jj) {
            const double2 t = T[(j0 + jj) * TR_OC + c];
#pragma unroll
            for (int q = 0; q < NR; ++q) {
                const int i = rg + TR_NRG * q;
                if (i < n) {
                    if (REAL_M) rfma(acc[q], Msr[i * TR_BJ + jj], t);
                    else cfma(acc[q], Ms[i * TR_BJ + jj], t);
                }
            }
        }
        __syncthreads();
    }
}

template <int NR>
__global__ void __launch_bounds__(TR_THREADS) k_trotter(int n, int o, int n_terms, double sqrt_dt,
                                                        const double* __restrict__ E,
                                                        const double2* __restrict__ V,
                                                        const double2* win, double2* wout, int vdiv) {
    extern __shared__ double2 sm[];
    double2* T = sm;                    // n x OC
    double2* Ms = sm + (size_t)n * TR_OC;  // n x BJ
    const int w = blockIdx.y, c0 = blockIdx.x * TR_OC;
    const int tid = threadIdx.x, c = tid % TR_OC, rg = tid / TR_OC;
    const double2* Wp = win + (size_t)w * n * o;
    const double2* Vw = V + (size_t)(w / vdiv) * n * n;

    for (int e = tid; e < n * TR_OC; e += TR_THREADS) {
        int i = e / TR_OC, cc = e % TR_OC;
        T[e] = (c0 + cc < o) ? Wp[(size_t)i * o + c0 + cc] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    double2 acc[NR], out[NR];
    tr_matmul<NR, true>(n, E, T, Ms, acc, c, rg);
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        const int i = rg + TR_NRG * q;
        out[q] = acc[q];
        if (i < n) T[i * TR_OC + c] = acc[q];
    }
    __syncthreads();
    for (int k = 1; k <= n_terms; ++k) {
        tr_matmul<NR, false>(n, Vw, T, Ms, acc, c, rg);
        const double s = sqrt_dt / k;  // (i sqrt_dt / k) * z = s * (-z.y, z.x)
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            const int i = rg + TR_NRG * q;
            double2 t = make_double2(-s * acc[q].y, s * acc[q].x);
            out[q] = cadd(out[q], t);
            if (i < n) T[i * TR_OC + c] = t;
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        const int i = rg + TR_NRG * q;
        if (i < n) T[i * TR_OC + c] = out[q];
    }
    __syncthreads();
    tr_matmul<NR, true>(n, E, T, Ms, acc, c, rg);
    double2* Wo = wout + (size_t)w * n * o;
#pragma unroll
    for (int q = 0; q < NR; ++q) {
        const int i = rg + TR_NRG * q;
        if (i < n && c0 + c < o) Wo[(size_t)i * o + c0 + c] = acc[q];
    }
}

int launch_trotter(int W, int n, int o, int n_terms, double sqrt_dt, const double* E, const double2* V,
                   const double2* win, double2* wout, cudaStream_t s, int vdiv) {
    if (W <= 0) return AFQ_OK;
    const int nr = (n + TR_NRG - 1) / TR_NRG;
    size_t smem = (size_t)n * (TR_OC + TR_BJ) * sizeof(double2);
    dim3 grid((o + TR_OC - 1) / TR_OC, W);
    if (W > 65535) return fail(AFQ_E_UNSUPPORTED, "trotter: chunk of %d walkers > 65535", W);
#define AFQ_TR(NRV)                                                                   \
    do {                                                                              \
        AFQ_TRY(set_smem(k_trotter<NRV>, smem));                                      \
        k_trotter<NRV><<<grid, TR_THREADS, smem, s>>>(n, o, n_terms, sqrt_dt, E, V, win, wout, vdiv); \
    } while (0)
    if (nr <= 1) AFQ_TR(1);
    else if (nr <= 2) AFQ_TR(2);
    else if (nr <= 4) AFQ_TR(4);
    else if (nr <= 8) AFQ_TR(8);
    else if (nr <= 16) AFQ_TR(16);
    else return fail(AFQ_E_UNSUPPORTED, "trotter: norb=%d > %d", n, 16 * TR_NRG);
#undef AFQ_TR
    AFQ_LAUNCHED("k_trotter");
    return AFQ_OK;
}

// =====================================================================
// Field shifts (prop/afqmc.py:97-101), one warp per walker:
//   fs = -sqrt_dt (i fb - mf);  x~ = x - fs;
//   shift_term = sum_g x~ mf;   fb_term = sum_g (x fs - fs^2 / 2)
// =====================================================================
__global__ void k_field_shift(int W, int G, double sqrt_dt, const double* __restrict__ x,
                              const double2* __restrict__ fb, const double2* __restrict__ mf,
                              double2* __restrict__ xs, double2* __restrict__ shift_term,
                              double2* __restrict__ fb_term) {
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= W) return;
    double sr = 0.0, si = 0.0, br = 0.0, bi = 0.0;
    for (int g = lane; g < G; g += 32) {
        const size_t e = (size_t)w * G + g;
        const double2 f = fb[e], m = mf[g];
        const double xv = x[e];
        // i fb - mf = (-f.y - m.x, f.x - m.y)
        const double2 fs = make_double2(-sqrt_dt * (-f.y - m.x), -sqrt_dt * (f.x - m.y));
        const double2 xt = make_double2(xv - fs.x, -fs.y);
        xs[e] = xt;
        sr += xt.x * m.x - xt.y * m.y;
        si += xt.x * m.y + xt.y * m.x;
        br += xv * fs.x - 0.5 * (fs.x * fs.x - fs.y * fs.y);
        bi += xv * fs.y - 0.5 * (2.0 * fs.x * fs.y);
    }
    sr = warp_sum(sr); si = warp_sum(si); br = warp_sum(br); bi = warp_sum(bi);
    if (lane == 0) {
        shift_term[w] = make_double2(sr, si);
        fb_term[w] = make_double2(br, bi);
    }
}

int launch_field_shift(int W, int G, double sqrt_dt, const double* x, const double2* fb, const double2* mf,
                       double2* xs, double2* shift_term, double2* fb_term, cudaStream_t s) {
    if (W <= 0) return AFQ_OK;
    k_field_shift<<<(W + 7) / 8, 256, 0, s>>>(W, G, sqrt_dt, x, fb, mf, xs, shift_term, fb_term);
    AFQ_LAUNCHED("k_field_shift");
    return AFQ_OK;
}

// =====================================================================
// Importance weights with the phaseless cut (prop/afqmc.py:116-138): one
// thread a walker over W / 256 CTAs (the binary64 exp / sincos / atan2 of a
// walker are a few hundred binary64 operations), then one CTA reduces the
// mean weight feeding the population-control shift in a fixed order
// (thread t sums walkers t, t + 1024, ...; then the warps and the CTA).
//
// Non-finite walkers: a NaN or infinite new overlap or weight propagates as
// in the reference (its floor and cap comparisons are false for NaN, so the
// weight stays NaN and the mean weight, hence the population shift, turns
// NaN).  With a status word (status != nullptr) every such walker is counted
// into status[1] and status[0] is set to AFQ_STATUS_NONFINITE if it was 0.
// =====================================================================
__global__ void __launch_bounds__(256) k_weight_update(
    int W, double dt, double sqrt_dt, double w_floor, double w_cap, double2 h0_prop,
    const double2* __restrict__ shift_term, const double2* __restrict__ fb_term,
    const double2* __restrict__ ovlp_new, double* __restrict__ weights, double2* __restrict__ overlaps,
    const double* __restrict__ pop_shift, int* __restrict__ status) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    const double ps = pop_shift[0];
    const double2 on = ovlp_new[w];
    double imp_ph = weight_factor(dt, sqrt_dt, ps, h0_prop, shift_term[w], fb_term[w], on, overlaps[w]).imp_ph;
    if (imp_ph < w_floor) imp_ph = 0.0;
    if (imp_ph > w_cap) imp_ph = 0.0;
    double wn = weights[w] * imp_ph;
    if (wn > w_cap) wn = 0.0;
    weights[w] = wn;
    overlaps[w] = on;
    if (status && !(isfinite(wn) && isfinite(on.x) && isfinite(on.y))) {
        atomicAdd(status + 1, 1);
        atomicCAS(status, 0, AFQ_STATUS_NONFINITE);
    }
}

__global__ void __launch_bounds__(1024) k_weight_mean(int W, double dt, double damping,
                                                      const double* __restrict__ weights,
                                                      double* __restrict__ pop_shift,
                                                      const double* __restrict__ e_est) {
    double local = 0.0;
    for (int w = threadIdx.x; w < W; w += blockDim.x) local += weights[w];
    __shared__ double red[32];
    local = warp_sum(local);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) {
            double avg = v / W;
            avg = (avg < 1.0e-300) ? 1.0e-300 : avg;  // NaN passes through, as with clip
            pop_shift[0] = e_est[0] - damping * (log(avg) / dt);
        }
    }
}

// Overlaps after a QR from those before it: det(C^H Q)^2 = det(C^H W)^2 /
// det(R)^2 for Q = W R^-1 (walkers.py:183-203's restricted normalisation).
__global__ void k_overlap_div_det2(int W, const double2* __restrict__ det_r, double2* __restrict__ overlaps) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    const double2 r = det_r[w];
    overlaps[w] = cdiv(overlaps[w], cmul(r, r));
}

int launch_overlap_div_det2(int W, const double2* det_r, double2* overlaps, cudaStream_t s) {
    if (W <= 0) return AFQ_OK;
    k_overlap_div_det2<<<(W + 255) / 256, 256, 0, s>>>(W, det_r, overlaps);
    AFQ_LAUNCHED("k_overlap_div_det2");
    return AFQ_OK;
}

int launch_weight_update(int W, const afq_params* p, double sqrt_dt, double dt, double2 h0_prop,
                         const double2* shift_term, const double2* fb_term, const double2* ovlp_new,
                         double* weights, double2* overlaps, double* pop_shift, const double* e_est,
                         cudaStream_t s, int* status) {
    if (W <= 0) return AFQ_OK;
    k_weight_update<<<(W + 255) / 256, 256, 0, s>>>(W, dt, sqrt_dt, p->weight_floor, p->weight_cap, h0_prop,
                                                    shift_term, fb_term, ovlp_new, weights, overlaps, pop_shift,
                                                    status);
    AFQ_LAUNCHED("k_weight_update");
    k_weight_mean<<<1, 1024, 0, s>>>(W, dt, p->pop_control_damping, weights, pop_shift, e_est);
    AFQ_LAUNCHED("k_weight_mean");
    return AFQ_OK;
}

// =====================================================================
// Local energy (meas/rhf.py:36-50).  f_g = L~_g G_half^T (o x o) for a chunk
// of NG Cholesky vectors per CTA; the tile keeps whole o x o blocks so that
// c_g = tr f_g and exc_g = sum_ij f_g[i,j] f_g[j,i] are reduced in the CTA
// and f never reaches global memory.  partial[w, chunk] = (sum c^2, sum exc).
// =====================================================================
constexpr int EN_BJ = 32, EN_R = 16, EN_THREADS = 256;

template <bool CR>
__global__ void __launch_bounds__(EN_THREADS) k_energy_partial(int n, int o, int G, int NG,
                                                               const double2* __restrict__ green,
                                                               const void* __restrict__ rotv,
                                                               double2* __restrict__ partial) {
    extern __shared__ double2 sm[];
    const int nchunk = gridDim.x;
    const int w = blockIdx.y, g0 = blockIdx.x * NG;
    const int ng = min(NG, G - g0);
    const int tid = threadIdx.x;
    const int nout = ng * o * o;
    double2* Gs = sm;                          // o x BJ
    double2* Ls = sm + o * EN_BJ;              // ng*o x BJ (complex or real)
    double* Lsr = (double*)Ls;
    double2* F = sm + o * EN_BJ + (CR ? (NG * o * EN_BJ + 1) / 2 : NG * o * EN_BJ);  // ng x o x o
    const double2* Gw = green + (size_t)w * o * n;

    double2 acc[EN_R];
    int offL[EN_R], offG[EN_R];
#pragma unroll
    for (int r = 0; r < EN_R; ++r) {
        acc[r] = make_double2(0.0, 0.0);
        int e = tid + EN_THREADS * r;
        int g = e / (o * o), rem = e % (o * o), i = rem / o, k = rem % o;
        offL[r] = (g * o + i) * EN_BJ;
        offG[r] = k * EN_BJ;
    }
    for (int j0 = 0; j0 < n; j0 += EN_BJ) {
        const int jn = min(EN_BJ, n - j0);
        for (int e = tid; e < o * EN_BJ; e += EN_THREADS) {
            int k = e / EN_BJ, jj = e % EN_BJ;
            Gs[e] = jj < jn ? Gw[(size_t)k * n + j0 + jj] : make_double2(0.0, 0.0);
        }
        for (int e = tid; e < ng * o * EN_BJ; e += EN_THREADS) {
            int gi = e / EN_BJ, jj = e % EN_BJ;  // gi = g*o + i
            size_t src = ((size_t)g0 * o + gi) * n + j0 + jj;
            if (CR) Lsr[e] = jj < jn ? ((const double*)rotv)[src] : 0.0;
            else Ls[e] = jj < jn ? ((const double2*)rotv)[src] : make_double2(0.0, 0.0);
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < EN_R; ++r) {
            if (tid + EN_THREADS * r < nout) {
                for (int jj = 0; jj < jn; ++jj) {
                    if (CR) rfma(acc[r], Lsr[offL[r] + jj], Gs[offG[r] + jj]);
                    else cfma(acc[r], Ls[offL[r] + jj], Gs[offG[r] + jj]);
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < EN_R; ++r) {
        int e = tid + EN_THREADS * r;
        if (e < nout) F[e] = acc[r];
    }
    __syncthreads();
    // per g: c = tr f, exc = sum_ik f[i,k] f[k,i]; thread-strided over (g, i, k)
    double cr = 0.0, ci = 0.0, xr = 0.0, xi = 0.0;
    for (int e = tid; e < nout; e += EN_THREADS) {
        int g = e / (o * o), rem = e % (o * o), i = rem / o, k = rem % o;
        double2 a = F[e], b = F[g * o * o + k * o + i];
        double2 p = cmul(a, b);
        xr += p.x; xi += p.y;
    }
    // sum_g c_g^2 : one thread per g
    for (int g = tid; g < ng; g += EN_THREADS) {
        double2 c = make_double2(0.0, 0.0);
        for (int i = 0; i < o; ++i) c = cadd(c, F[g * o * o + i * o + i]);
        double2 c2 = cmul(c, c);
        cr += c2.x; ci += c2.y;
    }
    __shared__ double red[4][EN_THREADS / 32];
    cr = warp_sum(cr); ci = warp_sum(ci); xr = warp_sum(xr); xi = warp_sum(xi);
    if ((tid & 31) == 0) {
        red[0][tid >> 5] = cr; red[1][tid >> 5] = ci; red[2][tid >> 5] = xr; red[3][tid >> 5] = xi;
    }
    __syncthreads();
    if (tid == 0) {
        double s[4] = {0, 0, 0, 0};
        for (int q = 0; q < 4; ++q)
            for (int k = 0; k < EN_THREADS / 32; ++k) s[q] += red[q][k];
        partial[((size_t)w * nchunk + blockIdx.x) * 2 + 0] = make_double2(s[0], s[1]);
        partial[((size_t)w * nchunk + blockIdx.x) * 2 + 1] = make_double2(s[2], s[3]);
    }
}

// energy = h0 + 2 sum G_half * rot_h1 + 2 sum c^2 - exc, one warp per walker
__global__ void k_energy_finish(int W, int n, int o, int nchunk, double h0, const double2* __restrict__ green,
                                const double2* __restrict__ rot_h1, const double2* __restrict__ partial,
                                double2* __restrict__ energy) {
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= W) return;
    const double2* Gw = green + (size_t)w * o * n;
    double er = 0.0, ei = 0.0;
    for (int e = lane; e < o * n; e += 32) {
        double2 p = cmul(Gw[e], rot_h1[e]);
        er += p.x; ei += p.y;
    }
    er = warp_sum(er); ei = warp_sum(ei);
    double cr = 0.0, ci = 0.0, xr = 0.0, xi = 0.0;
    for (int c = lane; c < nchunk; c += 32) {
        double2 a = partial[((size_t)w * nchunk + c) * 2 + 0], b = partial[((size_t)w * nchunk + c) * 2 + 1];
        cr += a.x; ci += a.y; xr += b.x; xi += b.y;
    }
    cr = warp_sum(cr); ci = warp_sum(ci); xr = warp_sum(xr); xi = warp_sum(xi);
    if (lane == 0) energy[w] = make_double2(h0 + 2.0 * er + 2.0 * cr - xr, 2.0 * ei + 2.0 * ci - xi);
}

static int energy_ng(int o, int G) {
    int ng = (EN_R * EN_THREADS) / (o * o);
    if (ng < 1) ng = 1;
    if (ng > G) ng = G;
    return ng;
}

size_t energy_partial_count(int W, int o, int G) {  // number of double2
    int ng = energy_ng(o, G);
    return (size_t)W * ((G + ng - 1) / ng) * 2;
}

int energy_partial_chunks(int o, int G) {
    const int ng = energy_ng(o, G);
    return (G + ng - 1) / ng;
}

int launch_energy(int W, int n, int o, int G, double h0, const double2* green, const void* rot_chol,
                  int trial_real, const double2* rot_h1, double* partial_d, double2* energy, cudaStream_t s) {
    if (W <= 0) return AFQ_OK;
    AFQ_TRY(launch_energy_partial(W, n, o, G, green, rot_chol, trial_real, partial_d, s));
    return launch_energy_finish(W, n, o, energy_partial_chunks(o, G), h0, green, rot_h1, (const double2*)partial_d,
                                energy, s);
}

int launch_energy_partial(int W, int n, int o, int G, const double2* green, const void* rot_chol, int trial_real,
                          double* partial_d, cudaStream_t s) {
    if (W <= 0) return AFQ_OK;
    if (o * o > EN_R * EN_THREADS) return fail(AFQ_E_UNSUPPORTED, "energy: nocc=%d > 64", o);
    const int ng = energy_ng(o, G);
    const int nchunk = (G + ng - 1) / ng;
    double2* partial = (double2*)partial_d;
    size_t lsz = trial_real ? (size_t)(ng * o * EN_BJ + 1) / 2 : (size_t)ng * o * EN_BJ;
    size_t smem = ((size_t)o * EN_BJ + lsz + (size_t)ng * o * o) * sizeof(double2);
    dim3 grid(nchunk, W);
    if (W > 65535) return fail(AFQ_E_UNSUPPORTED, "energy: %d walkers > 65535 per call", W);
    if (trial_real) {
        AFQ_TRY(set_smem(k_energy_partial<true>, smem));
        k_energy_partial<true><<<grid, EN_THREADS, smem, s>>>(n, o, G, ng, green, rot_chol, partial);
    } else {
        AFQ_TRY(set_smem(k_energy_partial<false>, smem));
        k_energy_partial<false><<<grid, EN_THREADS, smem, s>>>(n, o, G, ng, green, rot_chol, partial);
    }
    AFQ_LAUNCHED("k_energy_partial");
    return AFQ_OK;
}

int launch_energy_finish(int W, int n, int o, int nchunk, double h0, const double2* green, const double2* rot_h1,
                         const double2* partial, double2* energy, cudaStream_t s) {
    k_energy_finish<<<(W + 7) / 8, 256, 0, s>>>(W, n, o, nchunk, h0, green, rot_h1, partial, energy);
    AFQ_LAUNCHED("k_energy_finish");
    return AFQ_OK;
}

// =====================================================================
// Householder QR with diag(R) real >= 0 (walkers.py:169-180), in place in
// shared memory, column-major with odd leading dimension.  Q is formed in
// place by backward accumulation of the reflectors H_k = I - 2 u u^H.
// =====================================================================
// GLOBAL: the walker is factorised in place in wout (element (i, j) at
// A[i o + j], wout already holding the input), for walkers too large for
// shared memory; otherwise A[j ld + i] in shared memory.
template <bool GLOBAL>
__global__ void __launch_bounds__(256) k_qr(int n, int o, const double2* __restrict__ win,
                                            double2* __restrict__ wout, double2* __restrict__ det_out) {
    extern __shared__ double2 Asm[];
    __shared__ double2 s_alpha[64];
    __shared__ double s_red[8];
    __shared__ double s_sigma;
    const int ld = GLOBAL ? 1 : (n | 1);  // column stride
    const int rs = GLOBAL ? o : 1;        // row stride
    const int w = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int nw = blockDim.x >> 5;
    double2* A = GLOBAL ? wout + (size_t)w * n * o : Asm;
    if (!GLOBAL) {
        const double2* Wp = win + (size_t)w * n * o;
        for (int e = tid; e < n * o; e += blockDim.x) {
            int i = e / o, j = e % o;
            A[j * ld + i] = Wp[e];
        }
    }
    __syncthreads();
    for (int k = 0; k < o; ++k) {
        double2* x = A + k * ld;
        double sg = 0.0;
        for (int i = k + 1 + tid; i < n; i += blockDim.x) sg += cabs2(x[i * rs]);
        sg = warp_sum(sg);
        if (lane == 0) s_red[wid] = sg;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int q = 0; q < nw; ++q) t += s_red[q];
            s_sigma = t;
        }
        __syncthreads();
        const double sigma = s_sigma;
        const double2 x0 = x[k * rs];
        const double ax0 = sqrt(cabs2(x0));
        const double nx = sqrt(ax0 * ax0 + sigma);
        const double2 ph = ax0 == 0.0 ? make_double2(1.0, 0.0) : make_double2(x0.x / ax0, x0.y / ax0);
        const double2 alpha = make_double2(-ph.x * nx, -ph.y * nx);
        const double2 v0 = csub(x0, alpha);
        const double vn2 = cabs2(v0) + sigma;
        const double sc = vn2 > 0.0 ? 1.0 / sqrt(vn2) : 0.0;
        __syncthreads();
        for (int i = k + tid; i < n; i += blockDim.x) x[i * rs] = (i == k) ? cscale(v0, sc) : cscale(x[i * rs], sc);
        if (tid == 0) s_alpha[k] = alpha;
        __syncthreads();
        // columns j > k: A[k:, j] -= 2 u (u^H A[k:, j]); one warp per column
        for (int j = k + 1 + wid; j < o; j += nw) {
            double2* y = A + j * ld;
            double dr = 0.0, di = 0.0;
            for (int i = k + lane; i < n; i += 32) {
                double2 p = cmulc(x[i * rs], y[i * rs]);
                dr += p.x; di += p.y;
            }
            dr = warp_sum(dr); di = warp_sum(di);
            const double2 d2 = make_double2(2.0 * dr, 2.0 * di);
            for (int i = k + lane; i < n; i += 32) y[i * rs] = csub(y[i * rs], cmul(x[i * rs], d2));
        }
        __syncthreads();
    }
    // backward accumulation of Q
    for (int k = o - 1; k >= 0; --k) {
        double2* u = A + k * ld;
        for (int j = k + 1 + wid; j < o; j += nw) {
            double2* y = A + j * ld;
            double dr = 0.0, di = 0.0;
            for (int i = k + lane; i < n; i += 32) {
                double2 p = cmulc(u[i * rs], y[i * rs]);
                dr += p.x; di += p.y;
            }
            dr = warp_sum(dr); di = warp_sum(di);
            const double2 d2 = make_double2(2.0 * dr, 2.0 * di);
            for (int i = k + lane; i < n; i += 32) y[i * rs] = csub(y[i * rs], cmul(u[i * rs], d2));
        }
        __syncthreads();
        const double2 uk = u[k * rs];
        __syncthreads();
        for (int i = tid; i < n; i += blockDim.x) {
            if (i < k) u[i * rs] = make_double2(0.0, 0.0);
            else if (i == k) u[i * rs] = make_double2(1.0 - 2.0 * cabs2(uk), 0.0);
            else {
                double2 t = cmulc(uk, u[i * rs]);  // u_i conj(u_k)
                u[i * rs] = make_double2(-2.0 * t.x, -2.0 * t.y);
            }
        }
        __syncthreads();
    }
    // R~_kk = alpha_k is complex here (the reference's LAPACK R has a real
    // diagonal, hence its conj(phase) fix); Q[:, k] *= alpha_k / |alpha_k|
    // gives the same unique Q with diag(R) real and >= 0.
    double2* Wo = wout + (size_t)w * n * o;
    for (int e = tid; e < n * o; e += blockDim.x) {
        int i = e / o, j = e % o;
        double2 a = s_alpha[j];
        double aa = sqrt(cabs2(a));
        double2 cph = aa == 0.0 ? make_double2(1.0, 0.0) : make_double2(a.x / aa, a.y / aa);
        Wo[e] = cmul(A[j * ld + i * rs], cph);
    }
    if (det_out && tid == 0) {
        double d = 1.0;
        for (int k = 0; k < o; ++k) d *= sqrt(cabs2(s_alpha[k]));
        det_out[w] = make_double2(d, 0.0);
    }
}

int launch_qr(int W, int n, int o, const double2* win, double2* wout, double2* det_r, cudaStream_t s) {
    if (W <= 0) return AFQ_OK;
    if (o > 64) return fail(AFQ_E_UNSUPPORTED, "qr: nocc=%d > 64", o);
    size_t smem = (size_t)(n | 1) * o * sizeof(double2);
    if (smem <= 200 * 1024) {
        AFQ_TRY(set_smem(k_qr<false>, smem));
        k_qr<false><<<W, 256, smem, s>>>(n, o, win, wout, det_r);
        AFQ_LAUNCHED("k_qr");
        return AFQ_OK;
    }
    // too large for shared memory: in place in wout
    if (wout != win)
        AFQ_CUDA(cudaMemcpyAsync(wout, win, sizeof(double2) * (size_t)W * n * o, cudaMemcpyDeviceToDevice, s));
    k_qr<true><<<W, 256, 0, s>>>(n, o, wout, wout, det_r);
    AFQ_LAUNCHED("k_qr(global)");
    return AFQ_OK;
}

// =====================================================================
// Stochastic comb (walkers.py:233-265).  The prefix sum of |w| follows the
// association order of jax.lax.associative_scan, which is what the
// reference's jnp.cumsum lowers to on CPU and GPU: an up-sweep of pairwise
// sums e_{L+1}[k] = e_L[2k] + e_L[2k+1], then a down-sweep
// s_L[2k+1] = s_{L+1}[k], s_L[0] = e_L[0], s_L[2k] = s_{L+1}[k-1] + e_L[2k].
// Each add is one IEEE binary64 add (__dadd_rn: never contracted), so the
// bits are reproducible.  The search repeats jnp.searchsorted's default
// probe sequence (ceil(log2(W+1)) rounds of mid = (lo+hi)/2,
// z <= cw[mid] ? hi = mid : lo = mid; result hi), so even an ulp-level
// inversion of cw is searched identically.  One CTA; levels in `lv`.
// =====================================================================
size_t sr_levels_size(int W) {  // doubles over all levels (<= 2W)
    size_t t = 0;
    for (size_t n = (size_t)(W > 0 ? W : 1);; n >>= 1) {
        t += n;
        if (n < 2) break;
    }
    return t;
}

__global__ void __launch_bounds__(1024) k_sr_scan(int W, const double* __restrict__ weights, double zeta,
                                                  const double* __restrict__ zeta_dev,
                                                  double* __restrict__ lv, int32_t* __restrict__ idx,
                                                  double* __restrict__ cumsum_out, double* __restrict__ avg_out) {
    __shared__ int s_off[40], s_cnt[40], s_top;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (tid == 0) {
        int off = 0, n = W, L = 0;
        for (;;) {
            s_off[L] = off;
            s_cnt[L] = n;
            off += n;
            if (n < 2) break;
            n >>= 1;
            ++L;
        }
        s_top = L;
    }
    for (int i = tid; i < W; i += nt) lv[i] = fabs(weights[i]);
    __syncthreads();
    const int top = s_top;
    for (int L = 0; L < top; ++L) {  // up-sweep
        const double* e = lv + s_off[L];
        double* r = lv + s_off[L + 1];
        for (int k = tid; k < s_cnt[L + 1]; k += nt) r[k] = __dadd_rn(e[2 * k], e[2 * k + 1]);
        __syncthreads();
    }
    for (int L = top - 1; L >= 0; --L) {  // down-sweep, in place
        double* e = lv + s_off[L];
        const double* su = lv + s_off[L + 1];
        const int nL = s_cnt[L];
        for (int k = tid; 2 * k < nL; k += nt) {
            const double ev = (k == 0) ? e[0] : __dadd_rn(su[k - 1], e[2 * k]);
            if (2 * k + 1 < nL) e[2 * k + 1] = su[k];
            e[2 * k] = ev;
        }
        __syncthreads();
    }
    if (cumsum_out)
        for (int i = tid; i < W; i += nt) cumsum_out[i] = lv[i];
    const double tot = lv[W - 1];
    const double zt = zeta_dev ? zeta_dev[0] : zeta;
    if (tid == 0 && avg_out) avg_out[0] = __ddiv_rn(tot, (double)W);
    int rounds = 0;
    while ((1ll << rounds) < (long long)W + 1) ++rounds;
    for (int k = tid; k < W; k += nt) {
        const double z = __ddiv_rn(__dmul_rn(tot, __dadd_rn((double)k, zt)), (double)W);
        int lo = 0, hi = W;
        for (int r = 0; r < rounds; ++r) {
            const int mid = (int)(((unsigned)lo + (unsigned)hi) >> 1);
            const bool left = z <= lv[mid < W ? mid : W - 1];
            lo = left ? lo : mid;
            hi = left ? mid : hi;
        }
        idx[k] = hi < W ? hi : W - 1;
    }
}

int launch_sr_scan(int W, const double* weights, double zeta, double* levels, int32_t* idx, double* cumsum_out,
                   double* avg_out, cudaStream_t s) {
    if (W <= 0) return AFQ_OK;
    k_sr_scan<<<1, 1024, 0, s>>>(W, weights, zeta, nullptr, levels, idx, cumsum_out, avg_out);
    AFQ_LAUNCHED("k_sr_scan");
    return AFQ_OK;
}

int launch_sr_scan_dev(int W, const double* weights, const double* zeta_dev, double* levels, int32_t* idx,
                       double* avg_out, cudaStream_t s) {
    if (W <= 0) return AFQ_OK;
    k_sr_scan<<<1, 1024, 0, s>>>(W, weights, 0.0, zeta_dev, levels, idx, nullptr, avg_out);
    AFQ_LAUNCHED("k_sr_scan");
    return AFQ_OK;
}

// dst[k] = src[idx[k]] for rows of `row` complex; weights_out[k] = avg
__global__ void k_gather(int W, int64_t row, const int32_t* __restrict__ idx, const double2* __restrict__ src,
                         double2* __restrict__ dst, const double* __restrict__ avg, double* __restrict__ weights_out) {
    const int k = blockIdx.y;
    const int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int j = idx[k];
    for (int64_t e = base; e < row; e += (int64_t)gridDim.x * blockDim.x)
        dst[(size_t)k * row + e] = src[(size_t)j * row + e];
    if (weights_out && blockIdx.x == 0 && threadIdx.x == 0) weights_out[k] = avg[0];
}

int launch_gather(int W, int64_t row, const int32_t* idx, const double2* src, double2* dst, const double* avg,
                  double* weights_out, cudaStream_t s) {
    if (W <= 0) return AFQ_OK;
    if (W > 65535) return fail(AFQ_E_UNSUPPORTED, "gather: %d walkers > 65535", W);
    int bx = (int)((row + 255) / 256);
    if (bx > 64) bx = 64;
    if (bx < 1) bx = 1;
    k_gather<<<dim3(bx, W), 256, 0, s>>>(W, row, idx, src, dst, avg, weights_out);
    AFQ_LAUNCHED("k_gather");
    return AFQ_OK;
}

// =====================================================================
// Block measurement (prop/blocks.py:59-79): clip |E - e_est| > sqrt(2/dt),
// weighted mean (w_sum == 0 -> e_est), EMA of the population shift.
// =====================================================================
__global__ void __launch_bounds__(1024) k_block_measure(int W, double dt, double alpha,
                                                        const double* __restrict__ weights,
                                                        const double2* __restrict__ energy,
                                                        const double* __restrict__ e_est, double* pop_shift,
                                                        double* block_energy, double* block_weight) {
    const double eref = e_est[0];
    const double thresh = sqrt(2.0 / dt);
    double sw = 0.0, swe = 0.0;
    for (int w = threadIdx.x; w < W; w += blockDim.x) {
        double e = energy[w].x;
        if (fabs(e - eref) > thresh) e = eref;
        const double wt = weights[w];
        sw += wt;
        swe += wt * e;
    }
    __shared__ double r0[32], r1[32];
    sw = warp_sum(sw); swe = warp_sum(swe);
    if ((threadIdx.x & 31) == 0) { r0[threadIdx.x >> 5] = sw; r1[threadIdx.x >> 5] = swe; }
    __syncthreads();
    if (threadIdx.x < 32) {
        const bool ok = threadIdx.x < (blockDim.x >> 5);
        double a = ok ? r0[threadIdx.x] : 0.0, b = ok ? r1[threadIdx.x] : 0.0;
        a = warp_sum(a); b = warp_sum(b);
        if (threadIdx.x == 0) {
            const double safe = (a == 0.0) ? 1.0 : a;
            double eb = b / safe;
            if (a == 0.0) eb = eref;
            block_energy[0] = eb;
            block_weight[0] = a;
            pop_shift[0] = (1.0 - alpha) * pop_shift[0] + alpha * eb;
        }
    }
}

// Files one block's energy and weight at the run's next index and advances
// the run's Philox counter (the tail of a captured block).
__global__ void k_run_record(const double* __restrict__ e, const double* __restrict__ w, double* __restrict__ es,
                             double* __restrict__ ws, int* __restrict__ idx, uint64_t* __restrict__ counter,
                             uint64_t inc) {
    const int b = idx[0];
    es[b] = e[0];
    ws[b] = w[0];
    idx[0] = b + 1;
    counter[0] += inc;
}

int launch_run_record(const double* e, const double* w, double* es, double* ws, int* idx, uint64_t* counter,
                      uint64_t inc, cudaStream_t s) {
    k_run_record<<<1, 1, 0, s>>>(e, w, es, ws, idx, counter, inc);
    AFQ_LAUNCHED("k_run_record");
    return AFQ_OK;
}

int launch_block_measure(int W, double dt, double shift_ema, const double* weights, const double2* energy,
                         const double* e_est, double* pop_shift, double* block_energy, double* block_weight,
                         cudaStream_t s) {
    k_block_measure<<<1, 1024, 0, s>>>(W, dt, shift_ema, weights, energy, e_est, pop_shift, block_energy,
                                       block_weight);
    AFQ_LAUNCHED("k_block_measure");
    return AFQ_OK;
}

// =====================================================================
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) counter-based RNG.
// Call e uses counter (lo(e), hi(e), lo(counter), hi(counter)) and key
// (lo(seed), hi(seed)); its four words give two 53-bit uniforms u, v.
// Normals: Box-Muller, r = sqrt(-2 log(1-u)), (r cos 2 pi v, r sin 2 pi v),
// evaluated in fp32 from x = fp32(1 - u) and fp32(v) (the binary64
// transcendentals cost ~80 binary64 operations a pair at 1/64 of the fp32
// rate); each normal carries fp32 rounding, ~1e-7 relative.
// =====================================================================
__device__ __forceinline__ uint4 philox10(uint4 c, uint2 k) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k.x += W0; k.y += W1; }
        const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}

__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

__global__ void k_philox(int64_t count, uint64_t seed, uint64_t counter0, int normal, double* __restrict__ out,
                         const uint64_t* __restrict__ cbase) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (2 * e >= count) return;
    const uint64_t counter = counter0 + (cbase ? cbase[0] : 0ull);
    const uint4 r = philox10(make_uint4((uint32_t)e, (uint32_t)((uint64_t)e >> 32), (uint32_t)counter,
                                        (uint32_t)(counter >> 32)),
                             make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
    const double u = u53(r.x, r.y), v = u53(r.z, r.w);
    double a = u, b = v;
    if (normal) {
        const float rad = sqrtf(-2.0f * logf((float)(1.0 - u)));
        float sn, cs;
        sincospif(2.0f * (float)v, &sn, &cs);
        a = (double)(rad * cs);
        b = (double)(rad * sn);
    }
    out[2 * e] = a;
    if (2 * e + 1 < count) out[2 * e + 1] = b;
}

// Counter base read on the device, set for the duration of a captured block
// loop (afq_run_blocks) on the calling thread; null otherwise.
thread_local const uint64_t* t_counter_base = nullptr;

int launch_philox(int64_t count, uint64_t seed, uint64_t counter, int normal, double* out, cudaStream_t s) {
    if (count <= 0) return AFQ_OK;
    int64_t pairs = (count + 1) / 2;
    k_philox<<<(unsigned)((pairs + 255) / 256), 256, 0, s>>>(count, seed, counter, normal, out, t_counter_base);
    AFQ_LAUNCHED("k_philox");
    return AFQ_OK;
}

}  // namespace afq
