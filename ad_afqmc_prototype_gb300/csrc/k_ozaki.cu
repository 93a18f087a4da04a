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
// bf16 holds exactly.  The GEMM D = A B^T takes A row r = [w_1 | ... | w_7]
// (K = 7 nK, nK = norb rounded up to 8) and B row (a, d) = [c_{d-1} | c_{d-2}
// | ... ] (the digits of C whose index pairs with the slice to d = s + t,
// zero elsewhere), d = 2..9:
//   D[r][(a, d)] = sum_{s + t = d} sum_i w_s[i] c_t[i],
// an integer of magnitude <= 7 x norb x 2^12 < 2^24 for norb <= 585, so the
// tensor cores' fp32 sums are exact.  Then
//   m = 2^(E_r + F_a) sum_{d=2..9} D_d 2^(-7 d)
// with the terms s + t > 9 left out (each below 2^-51 of 2^(E_r + F_a) an
// orbital) and the digits cut toward zero at 2^-49: m to ~2^-45 of the
// product of the row's and the column's largest entries, the accuracy of the
// double-float m it replaces.  The recombination runs in the GEMM's epilogue
// (k_tc_gemm.cu, MODE 3) with integer and fp32 operations, and gives m as a
// double-float pair.
#include "afq_internal.cuh"

namespace afq {

OzDims oz_dims(int n, int o) {
    OzDims z;
    z.rows = 2 * o;
    z.nK = (n + 7) / 8 * 8;
    z.Kt = (7 * z.nK + 63) / 64 * 64;
    z.Nb = 8 * o;
    return z;
}

// The 7 signed base-128 digits of x 2^-E (|x| 2^-E < 1/4) cut toward zero at
// 2^-49, by integer operations: x = +-mant 2^(eb - 1075), so the 49-bit
// fixed-point value (|X| < 2^47) is mant shifted by eb - 1026 - E (<= -6).
__device__ __forceinline__ void oz_digits(double x, int E, int (&d)[7]) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const int eb = (int)((u >> 52) & 0x7ffu);
    long long X = 0;
    if (eb != 0 && eb != 0x7ff) {
        const unsigned long long mant = (u & 0xfffffffffffffull) | (1ull << 52);
        const int sh = eb - 1026 - E;
        if (sh > -64) X = (long long)(sh >= 0 ? mant << sh : mant >> (-sh));
        if (u >> 63) X = -X;
    }
#pragma unroll
    for (int t = 6; t >= 0; --t) {  // balanced digits in [-64, 64), least significant first
        const long long dt = ((X + 64) & 127) - 64;
        d[t] = (int)dt;
        X = (X - dt) >> 7;
    }
}

// Largest biased binary64 exponent of |x| (2047 for inf / nan).
__device__ __forceinline__ int oz_ebits(double x) {
    return (int)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ffu);
}

__device__ __forceinline__ uint32_t oz_bf2(int lo, int hi) {  // two small integers as a bf16 pair (exact)
    const __nv_bfloat162 v = __floats2bfloat162_rn((float)lo, (float)hi);
    return *(const uint32_t*)&v;
}

// B (Nb x Kt, K-major) and F_a from the trial C (n x o, real part used): one
// CTA per B row (a, d), each finding its column's scale.
__global__ void __launch_bounds__(256) k_oz_split_c(int n, int o, const double2* __restrict__ mo,
                                                    __nv_bfloat16* __restrict__ B, int* __restrict__ fa, int nK,
                                                    int Kt) {
    __shared__ int s_e;
    const int row = blockIdx.x, a = row >> 3, dd = (row & 7) + 2;
    if (threadIdx.x == 0) s_e = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) atomicMax(&s_e, oz_ebits(mo[(size_t)i * o + a].x));
    __syncthreads();
    const int F = s_e - 1020;
    if (threadIdx.x == 0 && (row & 7) == 0) fa[a] = F;
    // B[(a, d)][(s - 1) nK + i] = c_{d - s}[i][a] where 1 <= d - s <= 7
    for (int k = threadIdx.x; k < Kt; k += blockDim.x) {
        const int s = k / nK + 1, i = k % nK, t = dd - s;
        int v = 0;
        if (s <= 7 && i < n && t >= 1 && t <= 7) {
            int dg[7];
            oz_digits(mo[(size_t)i * o + a].x, F, dg);
            v = dg[t - 1];
        }
        B[(size_t)row * Kt + k] = __float2bfloat16((float)v);
    }
}

// A rows (walker, b, part) over K = (s - 1) nK + i, and E_r; one CTA per walker.
constexpr int OZ_CH = 32;  // orbital rows staged a chunk
__global__ void __launch_bounds__(256) k_oz_split_w(int n, int o, const double2* __restrict__ walkers,
                                                    __nv_bfloat16* __restrict__ A, int* __restrict__ er, int nK,
                                                    int Kt) {
    extern __shared__ double2 s_w[];  // OZ_CH x o staged rows
    __shared__ int s_e[64];
    const int w = blockIdx.x, R = 2 * o;
    const double2* Wp = walkers + (size_t)w * n * o;
    for (int r = threadIdx.x; r < R; r += blockDim.x) s_e[r] = 0;
    __syncthreads();
    for (int e = threadIdx.x; e < n * o; e += blockDim.x) {
        const double2 x = Wp[e];
        const int b = e % o;
        atomicMax(&s_e[2 * b], oz_ebits(x.x));
        atomicMax(&s_e[2 * b + 1], oz_ebits(x.y));
    }
    __syncthreads();
    for (int r = threadIdx.x; r < R; r += blockDim.x)
        er[(size_t)w * R + r] = s_e[r] == 0x7ff ? OZ_NONFINITE : s_e[r] - 1020;
    __nv_bfloat16* Aw = A + (size_t)w * R * Kt;
    // digits, two orbital rows a thread: 4-byte stores along K, a warp's 32 lanes on consecutive pairs
    for (int i0 = 0; i0 < nK; i0 += OZ_CH) {
        const int rows = min(OZ_CH, nK - i0);
        __syncthreads();
        for (int e = threadIdx.x; e < rows * o; e += blockDim.x) {
            const int i = i0 + e / o;
            s_w[e] = i < n ? Wp[(size_t)i * o + e % o] : make_double2(0.0, 0.0);
        }
        __syncthreads();
        const int pairs = rows >> 1;
        for (int t = threadIdx.x; t < R * pairs; t += blockDim.x) {
            const int r = t / pairs, ip = t % pairs, b = r >> 1, part = r & 1;
            const int il = 2 * ip;
            const double2 x0 = s_w[il * o + b], x1 = s_w[(il + 1) * o + b];
            const int E = s_e[r] == 0x7ff ? 0 : s_e[r] - 1020;
            int d0[7], d1[7];
            oz_digits(part ? x0.y : x0.x, E, d0);
            oz_digits(part ? x1.y : x1.x, E, d1);
            uint32_t* row = (uint32_t*)(Aw + (size_t)r * Kt);
#pragma unroll
            for (int s = 0; s < 7; ++s) row[(s * nK + i0 + il) >> 1] = oz_bf2(d0[s], d1[s]);
        }
    }
    // the K padding past 7 nK
    for (int t = threadIdx.x; t < R * ((Kt - 7 * nK) >> 1); t += blockDim.x) {
        const int pk = (Kt - 7 * nK) >> 1, r = t / pk, k = 7 * nK + 2 * (t % pk);
        *(uint32_t*)(Aw + (size_t)r * Kt + k) = 0u;
    }
}

int launch_oz_split_c(int n, int o, const double2* mo, __nv_bfloat16* B, int* fa, cudaStream_t s) {
    if (o > 64) return fail(AFQ_E_UNSUPPORTED, "ozaki m: nocc=%d > 64", o);
    const OzDims z = oz_dims(n, o);
    k_oz_split_c<<<z.Nb, 256, 0, s>>>(n, o, mo, B, fa, z.nK, z.Kt);
    AFQ_LAUNCHED("k_oz_split_c");
    return AFQ_OK;
}

int launch_oz_split_w(int W, int n, int o, const double2* walkers, __nv_bfloat16* A, int* er, cudaStream_t s) {
    if (W <= 0) return AFQ_OK;
    if (o > 32) return fail(AFQ_E_UNSUPPORTED, "ozaki m: nocc=%d > 32", o);
    const OzDims z = oz_dims(n, o);
    const size_t smem = (size_t)OZ_CH * o * sizeof(double2);
    k_oz_split_w<<<W, 256, smem, s>>>(n, o, walkers, A, er, z.nK, z.Kt);
    AFQ_LAUNCHED("k_oz_split_w");
    return AFQ_OK;
}

}  // namespace afq
