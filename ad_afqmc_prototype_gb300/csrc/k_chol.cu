// Modified (pivoted) Cholesky decomposition of a two-electron integral
// matrix into Cholesky vectors (integrals.py:3-46 of the reference), on the
// GPU in binary64.
//
// The matrix is the 4-fold symmetric ERI matrix M[(ij), (kl)] over pairs
// i >= j (size s = n (n + 1) / 2).  With d = diag(M), the reference runs
//   nu = argmax d,  delta_max = d[nu],  v_0 = M[nu] / sqrt(delta_max)
//   while |delta_max| > max_error and nchol + 1 < nchol_max:
//       Mapprox += v_nchol^2;  delta = d - Mapprox
//       nu = argmax |delta|;   delta_max = |delta[nu]|
//       v_{nchol+1} = (M[nu] - sum_{i <= nchol} v_i[nu] v_i) / sqrt(delta_max + 1e-10)
//       nchol += 1
// and returns v_0 .. v_{nchol-1} unpacked to symmetric n x n matrices.
// argmax takes the first index of the maximum, as numpy's does; the
// Mapprox / delta updates are the same binary64 operations; the dot
// products sum over i in ascending order.
//
// Device state (int[4] + double[2]): nu, nchol, done, pad; delta_max, pad.
// Each iteration is three launches (pivot, vector, counter) that do
// nothing once `done` is set, so the host runs them in batches and reads
// `done` between batches.
#include "afq_internal.cuh"

namespace afq {

struct CholState {
    int nu;
    int nchol;
    int done;
    int pad;
    double delta_max;
    double pad2;
};

// first-index argmax of |x| (abs_) or x over [0, s) in one CTA of 1024 threads
__device__ void block_argmax(int s, const double* __restrict__ x, bool abs_, int* out_idx, double* out_val) {
    __shared__ double sv[32];
    __shared__ int si[32];
    double best = -1.0;
    int bi = 0x7fffffff;
    for (int j = threadIdx.x; j < s; j += blockDim.x) {
        const double v = abs_ ? fabs(x[j]) : x[j];
        if (bi == 0x7fffffff || v > best) { best = v; bi = j; }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        if (oi != 0x7fffffff && (bi == 0x7fffffff || ov > best || (ov == best && oi < bi))) { best = ov; bi = oi; }
    }
    if (lane == 0) { sv[wid] = best; si[wid] = bi; }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        best = lane < nw ? sv[lane] : -1.0;
        bi = lane < nw ? si[lane] : 0x7fffffff;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, best, off);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (oi != 0x7fffffff && (bi == 0x7fffffff || ov > best || (ov == best && oi < bi))) {
                best = ov;
                bi = oi;
            }
        }
        if (lane == 0) { *out_idx = bi; *out_val = best; }
    }
}

// Diagonal of M into d, its first pivot, Mapprox = 0.
__global__ void __launch_bounds__(1024) k_mchol_init(int s, const double* __restrict__ M, double* __restrict__ d,
                                                     double* __restrict__ mapprox, CholState* st) {
    for (int j = threadIdx.x; j < s; j += blockDim.x) {
        d[j] = M[(size_t)j * s + j];
        mapprox[j] = 0.0;
    }
    __syncthreads();
    __shared__ int nu;
    __shared__ double v;
    block_argmax(s, d, false, &nu, &v);
    __syncthreads();
    if (threadIdx.x == 0) {
        st->nu = nu;
        st->nchol = 0;
        st->done = 0;
        st->delta_max = d[nu];  // v_0 uses d[nu] itself (not |d[nu]|, no 1e-10)
    }
}

// v_0 = M[nu] / sqrt(delta_max)
__global__ void k_mchol_first(int s, const double* __restrict__ M, double* __restrict__ V,
                              const CholState* __restrict__ st) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= s) return;
    V[j] = M[(size_t)st->nu * s + j] / sqrt(st->delta_max);
}

// The loop test, Mapprox += v_nchol^2, delta, and the next pivot.
__global__ void __launch_bounds__(1024) k_mchol_pivot(int s, int nchol_max, double max_error,
                                                      const double* __restrict__ d, double* __restrict__ mapprox,
                                                      double* __restrict__ delta, const double* __restrict__ V,
                                                      CholState* st) {
    __shared__ int go;
    if (threadIdx.x == 0) go = !st->done && fabs(st->delta_max) > max_error && st->nchol + 1 < nchol_max;
    __syncthreads();
    if (!go) {
        if (threadIdx.x == 0) st->done = 1;
        return;
    }
    const double* v = V + (size_t)st->nchol * s;
    for (int j = threadIdx.x; j < s; j += blockDim.x) {
        const double a = mapprox[j] + v[j] * v[j];
        mapprox[j] = a;
        delta[j] = d[j] - a;
    }
    __syncthreads();
    __shared__ int nu;
    __shared__ double dm;
    block_argmax(s, delta, true, &nu, &dm);
    __syncthreads();
    if (threadIdx.x == 0) {
        st->nu = nu;
        st->delta_max = dm;
    }
}

// v_{nchol+1}[j] = (M[nu, j] - sum_{i <= nchol} V[i, nu] V[i, j]) / sqrt(delta_max + 1e-10)
__global__ void __launch_bounds__(256) k_mchol_vec(int s, const double* __restrict__ M, double* __restrict__ V,
                                                   const CholState* __restrict__ st) {
    if (st->done) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = st->nchol, nu = st->nu;
    __shared__ double col[256];
    double r = 0.0;
    for (int i0 = 0; i0 <= k; i0 += 256) {
        const int cnt = min(256, k + 1 - i0);
        __syncthreads();
        if ((int)threadIdx.x < cnt) col[threadIdx.x] = V[(size_t)(i0 + threadIdx.x) * s + nu];
        __syncthreads();
        if (j < s)
            for (int i = 0; i < cnt; ++i) r = fma(col[i], V[(size_t)(i0 + i) * s + j], r);
    }
    if (j < s) V[(size_t)(k + 1) * s + j] = (M[(size_t)nu * s + j] - r) / sqrt(st->delta_max + 1e-10);
}

__global__ void k_mchol_count(CholState* st) {
    if (!st->done) st->nchol += 1;
}

// chol[c, m, n] = chol[c, n, m] = V[c, m (m + 1) / 2 + n] for n <= m
__global__ void k_mchol_unpack(int nvec, int n, int s, const double* __restrict__ V, double* __restrict__ out) {
    const long long total = (long long)nvec * n * n;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(e / ((long long)n * n));
        const int r = (int)(e % ((long long)n * n));
        const int m = r / n, q = r % n;
        const int hi = m > q ? m : q, lo = m > q ? q : m;
        out[e] = V[(size_t)c * s + (size_t)hi * (hi + 1) / 2 + lo];
    }
}

}  // namespace afq

using namespace afq;

static int mchol_norb(int s) {
    int n = (int)((-1.0 + sqrt(1.0 + 8.0 * s)) / 2.0 + 0.5);
    return n * (n + 1) / 2 == s ? n : -1;
}

size_t afq_modified_cholesky_workspace(int32_t size, int32_t max_vectors) {
    if (size < 1 || max_vectors < 1) return 0;
    Arena a;
    a.take<int>(64);
    a.take<CholState>(1);
    for (int k = 0; k < 3; ++k) a.take<double>(size);  // diagonal, Mapprox, residual
    a.take<double>((size_t)max_vectors * size);
    return a.used;
}

int afq_modified_cholesky(int32_t size, const double* mat, double max_error, int32_t max_vectors,
                          double* chol_out, int32_t* nchol_out, void* workspace, size_t workspace_bytes,
                          void* stream) {
    if (size < 1) return fail(AFQ_E_INVALID_ARGUMENT, "size=%d < 1", size);
    const int n = mchol_norb(size);
    if (n < 1) return fail(AFQ_E_INVALID_ARGUMENT, "size=%d is not n (n + 1) / 2", size);
    if (max_vectors < 1) return fail(AFQ_E_INVALID_ARGUMENT, "max_vectors=%d < 1", max_vectors);
    if (!mat || !chol_out || !nchol_out || !workspace) return fail(AFQ_E_INVALID_ARGUMENT, "NULL argument");
    Arena a(workspace, workspace_bytes);
    a.take<int>(64);
    CholState* st = a.take<CholState>(1);
    double* d = a.take<double>(size);
    double* mapprox = a.take<double>(size);
    double* delta = a.take<double>(size);
    double* V = a.take<double>((size_t)max_vectors * size);
    if (!a.ok()) return fail(AFQ_E_WORKSPACE, "workspace: %zu bytes < %zu", workspace_bytes, a.used);
    cudaStream_t s = as_stream(stream);
    const int nchol_max = size < max_vectors ? size : max_vectors;
    const int vb = (size + 255) / 256;
    k_mchol_init<<<1, 1024, 0, s>>>(size, mat, d, mapprox, st);
    AFQ_LAUNCHED("k_mchol_init");
    k_mchol_first<<<vb, 256, 0, s>>>(size, mat, V, st);
    AFQ_LAUNCHED("k_mchol_first");
    CholState h = {};
    for (int it = 0; it < nchol_max; it += 32) {
        for (int b = 0; b < 32; ++b) {
            k_mchol_pivot<<<1, 1024, 0, s>>>(size, nchol_max, max_error, d, mapprox, delta, V, st);
            k_mchol_vec<<<vb, 256, 0, s>>>(size, mat, V, st);
            k_mchol_count<<<1, 1, 0, s>>>(st);
        }
        AFQ_LAUNCHED("k_mchol_iteration");
        AFQ_CUDA(cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, s));
        AFQ_CUDA(cudaStreamSynchronize(s));
        if (h.done) break;
    }
    if (!h.done) return fail(AFQ_E_INVALID_ARGUMENT, "modified cholesky: no convergence in %d vectors", nchol_max);
    *nchol_out = h.nchol;
    if (h.nchol > 0) {
        const long long total = (long long)h.nchol * n * n;
        long long blocks = (total + 255) / 256;
        if (blocks > 152 * 64) blocks = 152 * 64;
        k_mchol_unpack<<<(unsigned)blocks, 256, 0, s>>>(h.nchol, n, size, V, chol_out);
        AFQ_LAUNCHED("k_mchol_unpack");
    }
    return AFQ_OK;
}
