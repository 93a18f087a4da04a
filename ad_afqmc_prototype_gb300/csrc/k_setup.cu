// Set-up kernels: the propagator context (prop/chol_afqmc_ops.py:53-103) and
// the half-rotated measurement context (meas/rhf.py:141-150), in binary64.
// They run once per Hamiltonian; none of them is on the step's hot path.
#include "afq_internal.cuh"

namespace afq {

// dm = rdm1[0] + rdm1[1]   (prop/chol_afqmc_ops.py:53-56)
__global__ void k_sum_spin_blocks(int nn, const double2* __restrict__ rdm1, double2* __restrict__ dm) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nn) dm[e] = cadd(rdm1[e], rdm1[nn + e]);
}

int launch_sum_spin_blocks(int n, const double2* rdm1, double2* dm, cudaStream_t s) {
    int nn = n * n;
    k_sum_spin_blocks<<<(nn + 255) / 256, 256, 0, s>>>(nn, rdm1, dm);
    AFQ_LAUNCHED("k_sum_spin_blocks");
    return AFQ_OK;
}

// get_rdm1 (trial/rhf.py:29-32): dm = C C^H (n x n), written twice, as the
// (2, n, n) spin-block stack [dm, dm].  One thread an entry.
__global__ void k_trial_rdm1(int n, int o, const double2* __restrict__ mo, double2* __restrict__ rdm1) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * n) return;
    const int i = e / n, j = e % n;
    double2 acc = make_double2(0.0, 0.0);
    for (int a = 0; a < o; ++a) {
        const double2 x = mo[i * o + a], y = mo[j * o + a];  // x conj(y)
        acc.x = fma(x.x, y.x, acc.x);
        acc.x = fma(x.y, y.y, acc.x);
        acc.y = fma(x.y, y.x, acc.y);
        acc.y = fma(-x.x, y.y, acc.y);
    }
    rdm1[e] = acc;
    rdm1[n * n + e] = acc;
}

int launch_trial_rdm1(int n, int o, const double2* mo, double2* rdm1, cudaStream_t s) {
    const int nn = n * n;
    k_trial_rdm1<<<(nn + 255) / 256, 256, 0, s>>>(n, o, mo, rdm1);
    AFQ_LAUNCHED("k_trial_rdm1");
    return AFQ_OK;
}

// mf_g = i * sum_ij L_g[i,j] dm[j,i]   (prop/chol_afqmc_ops.py:59-63)
__global__ void __launch_bounds__(256) k_mf_shifts(int n, const double* __restrict__ chol,
                                                   const double2* __restrict__ dm,
                                                   double2* __restrict__ mf) {
    const int g = blockIdx.x;
    const double* L = chol + (size_t)g * n * n;
    double re = 0.0, im = 0.0;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        int i = e / n, j = e % n;
        double2 d = dm[j * n + i];
        re = fma(L[e], d.x, re);
        im = fma(L[e], d.y, im);
    }
    __shared__ double sr[8], si[8];
    re = warp_sum(re);
    im = warp_sum(im);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sr[wid] = re; si[wid] = im; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tr = 0.0, ti = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { tr += sr[k]; ti += si[k]; }
        mf[g] = make_double2(-ti, tr);  // i * (tr + i ti)
    }
}

int launch_mf_shifts(int n, int G, const double* chol, const double2* dm, double2* mf, cudaStream_t s) {
    k_mf_shifts<<<G, 256, 0, s>>>(n, chol, dm, mf);
    AFQ_LAUNCHED("k_mf_shifts");
    return AFQ_OK;
}

// h1_eff = h1 - 0.5 sum_g L_g L_g - sum_g Re(i mf_g) L_g
// (prop/chol_afqmc_ops.py:86-94)
__global__ void __launch_bounds__(256) k_h1_eff(int n, int G, const double* __restrict__ h1,
                                                const double* __restrict__ chol,
                                                const double2* __restrict__ mf,
                                                double* __restrict__ h1_eff) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * n) return;
    int i = e / n, j = e % n;
    double v0 = 0.0, v1 = 0.0;
    for (int g = 0; g < G; ++g) {
        const double* L = chol + (size_t)g * n * n;
        double acc = 0.0;
        for (int k = 0; k < n; ++k) acc = fma(L[i * n + k], L[k * n + j], acc);
        v0 += acc;
        double mf_r = -mf[g].y;  // Re(i * mf_g)
        v1 = fma(mf_r, L[e], v1);
    }
    h1_eff[e] = h1[e] - 0.5 * v0 - v1;
}

int launch_h1_eff(int n, int G, const double* h1, const double* chol, const double2* mf,
                  double* h1_eff, cudaStream_t s) {
    int nn = n * n;
    k_h1_eff<<<(nn + 255) / 256, 256, 0, s>>>(n, G, h1, chol, mf, h1_eff);
    AFQ_LAUNCHED("k_h1_eff");
    return AFQ_OK;
}

// h0_prop = -h0 - 0.5 sum_g mf_g^2   (prop/chol_afqmc_ops.py:84)
__global__ void k_h0_prop(int G, double h0, const double2* __restrict__ mf, double2* out) {
    double re = 0.0, im = 0.0;
    for (int g = threadIdx.x; g < G; g += blockDim.x) {
        double2 m = mf[g];
        re += m.x * m.x - m.y * m.y;
        im += 2.0 * m.x * m.y;
    }
    __shared__ double sr[32], si[32];
    re = warp_sum(re);
    im = warp_sum(im);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sr[wid] = re; si[wid] = im; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tr = 0.0, ti = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { tr += sr[k]; ti += si[k]; }
        out[0] = make_double2(-h0 - 0.5 * tr, -0.5 * ti);
    }
}

int launch_h0_prop(int G, double h0, const double2* mf, double2* h0_prop, cudaStream_t s) {
    k_h0_prop<<<1, 256, 0, s>>>(G, h0, mf, h0_prop);
    AFQ_LAUNCHED("k_h0_prop");
    return AFQ_OK;
}

// ---------------------------------------------------------------- expm ----
// exp(scale * A) by scaling and squaring with a degree-18 Taylor polynomial
// evaluated in Horner form (Moler & Van Loan, "Nineteen dubious ways",
// method 3).  After scaling, ||B||_1 <= 1/2, so the truncation error
// ||B||^19/19! is below 1e-22 and the result agrees with a Pade-13
// implementation to rounding.

__global__ void k_norm1(int n, double scale, const double* __restrict__ a, double* out) {
    double best = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < n; ++i) s += fabs(scale * a[i * n + j]);
        best = fmax(best, s);
    }
    __shared__ double sm[256];
    sm[threadIdx.x] = best;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = sm[0];
}

// C = alpha * A B (+ I if add_identity), n x n real, 16x16 tiles.
__global__ void k_dgemm_sq(int n, double alpha, const double* __restrict__ A,
                           const double* __restrict__ B, double* __restrict__ C, int add_identity) {
    __shared__ double As[16][17], Bs[16][17];
    int tx = threadIdx.x, ty = threadIdx.y;
    int row = blockIdx.y * 16 + ty, col = blockIdx.x * 16 + tx;
    double acc = 0.0;
    for (int k0 = 0; k0 < n; k0 += 16) {
        As[ty][tx] = (row < n && k0 + tx < n) ? A[row * n + k0 + tx] : 0.0;
        Bs[ty][tx] = (k0 + ty < n && col < n) ? B[(k0 + ty) * n + col] : 0.0;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 16; ++k) acc = fma(As[ty][k], Bs[k][tx], acc);
        __syncthreads();
    }
    if (row < n && col < n) C[row * n + col] = alpha * acc + ((add_identity && row == col) ? 1.0 : 0.0);
}

__global__ void k_scaled_copy(int nn, double s, const double* __restrict__ a, double* __restrict__ b, int identity_n) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nn) return;
    if (identity_n > 0) b[e] = (e / identity_n == e % identity_n) ? 1.0 : 0.0;
    else b[e] = s * a[e];
}

int launch_expm(int n, double scale, const double* a, double* out, double* tmp0, double* tmp1,
                double* tmp2, double* norm_dev, cudaStream_t s) {
    const int nn = n * n;
    k_norm1<<<1, 256, 0, s>>>(n, scale, a, norm_dev);
    AFQ_LAUNCHED("k_norm1");
    double norm = 0.0;
    AFQ_CUDA(cudaMemcpyAsync(&norm, norm_dev, sizeof(double), cudaMemcpyDeviceToHost, s));
    AFQ_CUDA(cudaStreamSynchronize(s));
    int sq = 0;
    if (norm > 0.5) sq = (int)ceil(log2(norm / 0.5));
    if (sq > 60) return fail(AFQ_E_INVALID_ARGUMENT, "expm: norm %g too large", norm);
    const double bscale = scale * ldexp(1.0, -sq);
    dim3 blk(16, 16), grd((n + 15) / 16, (n + 15) / 16);
    // tmp0 = B, P (tmp1) = I
    k_scaled_copy<<<(nn + 255) / 256, 256, 0, s>>>(nn, bscale, a, tmp0, 0);
    k_scaled_copy<<<(nn + 255) / 256, 256, 0, s>>>(nn, 0.0, a, tmp1, n);
    AFQ_LAUNCHED("k_scaled_copy");
    // Horner: P <- I + (B P) / k for k = 18 .. 1
    double* P = tmp1;
    double* Q = tmp2;
    for (int k = 18; k >= 1; --k) {
        k_dgemm_sq<<<grd, blk, 0, s>>>(n, 1.0 / k, tmp0, P, Q, 1);
        double* t = P; P = Q; Q = t;
    }
    AFQ_LAUNCHED("k_dgemm_sq");
    for (int r = 0; r < sq; ++r) {
        k_dgemm_sq<<<grd, blk, 0, s>>>(n, 1.0, P, P, Q, 0);
        double* t = P; P = Q; Q = t;
    }
    AFQ_LAUNCHED("k_dgemm_sq(square)");
    AFQ_CUDA(cudaMemcpyAsync(out, P, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s));
    return AFQ_OK;
}

// ----------------------------------------------------- half rotation -----
// rot_h1[p, j] = sum_i conj(C[i, p]) h1[i, j];
// rot_chol[g, p, j] = sum_i conj(C[i, p]) L_g[i, j]   (meas/rhf.py:141-150)
template <bool REAL>
__global__ void __launch_bounds__(256) k_rot(int n, int o, int nmat, const double* __restrict__ mats,
                                             const double2* __restrict__ mo, void* __restrict__ out) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t total = (int64_t)nmat * o * n;
    if (e >= total) return;
    int j = (int)(e % n);
    int p = (int)((e / n) % o);
    int g = (int)(e / ((int64_t)n * o));
    const double* L = mats + (size_t)g * n * n;
    double re = 0.0, im = 0.0;
    for (int i = 0; i < n; ++i) {
        double l = L[i * n + j];
        double2 c = mo[i * o + p];
        re = fma(c.x, l, re);
        im = fma(-c.y, l, im);
    }
    if (REAL) ((double*)out)[e] = re;
    else ((double2*)out)[e] = make_double2(re, im);
}

int launch_rot(int n, int o, int G, const double* h1, const double* chol, const double2* mo,
               int trial_real, double2* rot_h1, void* rot_chol, cudaStream_t s) {
    int64_t t1 = (int64_t)o * n;
    k_rot<false><<<(unsigned)((t1 + 255) / 256), 256, 0, s>>>(n, o, 1, h1, mo, rot_h1);
    AFQ_LAUNCHED("k_rot(h1)");
    int64_t t2 = (int64_t)G * o * n;
    if (trial_real)
        k_rot<true><<<(unsigned)((t2 + 255) / 256), 256, 0, s>>>(n, o, G, chol, mo, rot_chol);
    else
        k_rot<false><<<(unsigned)((t2 + 255) / 256), 256, 0, s>>>(n, o, G, chol, mo, rot_chol);
    AFQ_LAUNCHED("k_rot(chol)");
    return AFQ_OK;
}

}  // namespace afq
