// Binary64 GEMM with a complex left operand and a real or complex right
// operand.  Used by the FP64 step for
//   V-build     V (W x n^2) = x~ (W x G) . L (G x n^2)     (prop/chol_afqmc_ops.py:70-74)
//   force bias  fb (W x G)  = 2 G_half (W x o n) . L~^T    (meas/rhf.py:27-33)
// On GB300 binary64 runs on the SM's scalar FP64 pipe (no FP64 tensor path),
// so the kernel is a register-blocked SIMT GEMM: 64x64 tile, 4x4 complex
// outputs per thread, K staged through shared memory 16 at a time.
#include "afq_internal.cuh"

namespace afq {

namespace {
constexpr int BM = 64, BN = 64, BK = 16;

template <bool BC>
struct BElem;
template <>
struct BElem<false> { using T = double; };
template <>
struct BElem<true> { using T = double2; };

__device__ __forceinline__ double2 zero2() { return make_double2(0.0, 0.0); }
__device__ __forceinline__ void load_b(double& dst, const double* p, bool ok) { dst = ok ? *p : 0.0; }
__device__ __forceinline__ void load_b(double2& dst, const double2* p, bool ok) { dst = ok ? *p : zero2(); }
__device__ __forceinline__ void mac(double2& acc, double2 a, double b) { rfma(acc, b, a); }
__device__ __forceinline__ void mac(double2& acc, double2 a, double2 b) { cfma(acc, a, b); }
}  // namespace

// grid.z > 1 (split K): CTA layer z sums k in [z kc, min(K, (z + 1) kc)) into
// C + z cs (the caller adds the layers in a fixed order).
template <bool BC, bool BT>
__global__ void __launch_bounds__(256) k_zgemm(int M, int N, int K, double alpha,
                                               const double2* __restrict__ A, int64_t lda,
                                               const void* __restrict__ Bv, int64_t ldb,
                                               double2* __restrict__ C, int64_t ldc, int kc, int64_t cs) {
    using TB = typename BElem<BC>::T;
    const TB* B = (const TB*)Bv;
    const int kbeg = blockIdx.z * kc;
    const int kend = min(K, kbeg + kc);
    C += (int64_t)blockIdx.z * cs;
    __shared__ double2 As[BK][BM + 1];
    __shared__ TB Bs[BK][BN + 1];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;

    double2 acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = zero2();

    for (int k0 = kbeg; k0 < kend; k0 += BK) {
        // A tile: 64 rows x 16 k, k fastest for coalescing
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            int mm = (tid >> 4) + 16 * r, kk = tid & 15;
            int gm = m0 + mm, gk = k0 + kk;
            As[kk][mm] = (gm < M && gk < kend) ? A[(int64_t)gm * lda + gk] : zero2();
        }
        if (!BT) {
            // B(k, n) = B[k*ldb + n], n fastest
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                int kk = (tid >> 6) + 4 * r, nn = tid & 63;
                int gk = k0 + kk, gn = n0 + nn;
                bool ok = gk < kend && gn < N;
                load_b(Bs[kk][nn], B + (ok ? (int64_t)gk * ldb + gn : 0), ok);
            }
        } else {
            // B(k, n) = B[n*ldb + k], k fastest
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                int nn = (tid >> 4) + 16 * r, kk = tid & 15;
                int gk = k0 + kk, gn = n0 + nn;
                bool ok = gk < kend && gn < N;
                load_b(Bs[kk][nn], B + (ok ? (int64_t)gn * ldb + gk : 0), ok);
            }
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double2 a[4];
            TB b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mac(acc[i][j], a[i], b[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int gm = m0 + ty + 16 * i;
        if (gm >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int gn = n0 + tx + 16 * j;
            if (gn < N) C[(int64_t)gm * ldc + gn] = cscale(acc[i][j], alpha);
        }
    }
}

int launch_zgemm(int M, int N, int K, double alpha, const double2* A, int64_t lda, const void* B,
                 int64_t ldb, bool b_complex, bool b_trans, double2* C, int64_t ldc,
                 cudaStream_t s) {
    if (M <= 0 || N <= 0) return AFQ_OK;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
    if (grid.y > 65535u) return fail(AFQ_E_UNSUPPORTED, "zgemm: M=%d too large", M);
    if (b_complex) {
        if (b_trans) k_zgemm<true, true><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, C, ldc, K, 0);
        else k_zgemm<true, false><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, C, ldc, K, 0);
    } else {
        if (b_trans) k_zgemm<false, true><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, C, ldc, K, 0);
        else k_zgemm<false, false><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, C, ldc, K, 0);
    }
    AFQ_LAUNCHED("k_zgemm");
    return AFQ_OK;
}

// C (M x N, ldc = N) = sum_z part[z] in order z = 0 .. splits-1
__global__ void k_zsum_layers(long long count, int splits, const double2* __restrict__ part,
                              double2* __restrict__ C) {
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < count;
         e += (long long)gridDim.x * blockDim.x) {
        double2 a = part[e];
        for (int z = 1; z < splits; ++z) a = cadd(a, part[(long long)z * count + e]);
        C[e] = a;
    }
}

int zgemm_splits(int M, int N, int K) {
    const long long ctas = (long long)((N + BN - 1) / BN) * ((M + BM - 1) / BM);
    int z = 1;
    while (ctas * z < 2 * 152 && K / (z * 2) >= 4 * BK && z < 8) z *= 2;
    return z;
}

int launch_zgemm_splitk(int M, int N, int K, double alpha, const double2* A, int64_t lda, const void* B,
                        int64_t ldb, bool b_complex, bool b_trans, double2* C, double2* part, cudaStream_t s) {
    if (M <= 0 || N <= 0) return AFQ_OK;
    const int z = zgemm_splits(M, N, K);
    if (z == 1) return launch_zgemm(M, N, K, alpha, A, lda, B, ldb, b_complex, b_trans, C, N, s);
    const int kc = (K / z + BK - 1) / BK * BK;
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, z);
    if (grid.y > 65535u) return fail(AFQ_E_UNSUPPORTED, "zgemm: M=%d too large", M);
    const int64_t cs = (int64_t)M * N;
    if (b_complex) {
        if (b_trans) k_zgemm<true, true><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, part, N, kc, cs);
        else k_zgemm<true, false><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, part, N, kc, cs);
    } else {
        if (b_trans) k_zgemm<false, true><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, part, N, kc, cs);
        else k_zgemm<false, false><<<grid, 256, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, part, N, kc, cs);
    }
    AFQ_LAUNCHED("k_zgemm(split k)");
    long long blocks = (cs + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    k_zsum_layers<<<(unsigned)blocks, 256, 0, s>>>(cs, z, part, C);
    AFQ_LAUNCHED("k_zsum_layers");
    return AFQ_OK;
}

}  // namespace afq
