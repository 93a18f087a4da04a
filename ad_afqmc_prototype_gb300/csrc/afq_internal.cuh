// Internal declarations shared by the engine's translation units.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "afqmc_gb300.h"

namespace afq {

// ---------------------------------------------------------------- errors --
// Records a thread-local message and returns `code`.
int fail(int code, const char* fmt, ...);
// Checks the last launch / a runtime call.
int check_cuda(cudaError_t e, const char* what);
#define AFQ_TRY(expr)            \
    do {                         \
        int _rc = (expr);        \
        if (_rc != AFQ_OK) return _rc; \
    } while (0)
#define AFQ_CUDA(expr) AFQ_TRY(::afq::check_cuda((expr), #expr))
#define AFQ_LAUNCHED(name)                                        \
    do {                                                          \
        ::afq::count_launch();                                    \
        AFQ_TRY(::afq::check_cuda(cudaGetLastError(), name));     \
    } while (0)

// ------------------------------------------------ per-device launch facts --
// One process may drive several GPUs.  What a launcher learns on its first
// launch on a device (the SM count, a raised dynamic shared-memory limit) is
// kept per device ordinal behind a lock, never once per process.
constexpr int kMaxDevices = 64;
// Ordinal of the current device; AFQ_E_UNSUPPORTED beyond kMaxDevices.
int current_device(int* dev);
// SM count of the current device (looked up once per device).
int device_sms(int* sms);
// Per-device "done" flags of one launcher's one-time set-up (zero-initialised
// as a static object).
struct DeviceOnce {
    bool done[kMaxDevices];
};
// Runs fn(arg) once per current device for `once`, under a library-wide
// recursive lock; a failing fn leaves the flag clear.  fn returns AFQ_*.
int device_once_run(DeviceOnce& once, int (*fn)(void*), void* arg);
// Raises kernel's dynamic shared-memory limit to `bytes`, once per device.
template <class K>
int raise_smem_once(DeviceOnce& once, K kernel, int bytes) {
    struct A {
        K k;
        int b;
    } a{kernel, bytes};
    return device_once_run(
        once,
        [](void* p) -> int {
            A* x = (A*)p;
            AFQ_CUDA(cudaFuncSetAttribute(x->k, cudaFuncAttributeMaxDynamicSharedMemorySize, x->b));
            return AFQ_OK;
        },
        &a);
}

// ---------------------------------------------------------------- tracing --
// afq_trace.cu: a process-wide count of kernel launches, and (when enabled
// with afq_timing_enable) CUDA events recorded on the launching stream around
// each named phase of the step and block.
void count_launch();
struct Phase {
    const char* name;
    cudaStream_t stream;
    cudaEvent_t start;
    Phase(const char* n, cudaStream_t s);
    ~Phase();
};
#define AFQ_PHASE_CAT2(a, b) a##b
#define AFQ_PHASE_CAT(a, b) AFQ_PHASE_CAT2(a, b)
#define AFQ_PHASE(name, s) ::afq::Phase AFQ_PHASE_CAT(afq_phase_, __LINE__)(name, s)

// --------------------------------------------------------- complex maths --
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {  // conj(a) * b
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// acc += a * b
__device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
// acc += r * b  (r real)
__device__ __forceinline__ void rfma(double2& acc, double r, double2 b) {
    acc.x = fma(r, b.x, acc.x);
    acc.y = fma(r, b.y, acc.y);
}
__device__ __forceinline__ double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }

// x = hi + lo as an fp32 pair from the binary64 fields with integer
// operations only, on every path (the binary64 pipe runs at 1/64 of the fp32
// rate here, and a branch to binary64 conversions would be if-converted and
// paid for every element): hi is x cut to 24 significant bits, lo the
// remaining 29 bits rounded to 24, so |x - hi - lo| <= 2^-48 |x| for
// 2^-74 <= |x| < 2^128.  Below 2^-74 lo is a signed zero, below the fp32
// normal range hi too; beyond it hi is infinity (nan for a nan).
__device__ __forceinline__ float2 split_d2f(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned h = (unsigned)(u >> 32), l = (unsigned)u;
    const unsigned e = (h >> 20) & 0x7ffu, sign = h & 0x80000000u;
    const unsigned nrm = sign | ((((h & 0x7fffffffu) - (896u << 20)) << 3) | (l >> 29));
    const unsigned big = ((e == 0x7ffu) && ((h & 0xfffffu) | l)) ? 0x7fc00000u : (sign | 0x7f800000u);
    const float hi = __uint_as_float(e < 897u ? sign : (e > 1150u ? big : nrm));
    const float scale = __uint_as_float(((e - 948u) & 0xffu) << 23);  // 2^(e - 1075), the weight of bit 0 of l
    const float lo_n = __uint_as_float(sign | __float_as_uint(__uint2float_rn(l & 0x1fffffffu) * scale));
    const float lo = (e >= 949u && e <= 1150u) ? lo_n : __uint_as_float(sign);
    return make_float2(hi, lo);
}
// x cut to fp32 (the hi part of split_d2f).
__device__ __forceinline__ float d2f_trunc(double x) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x);
    const unsigned h = (unsigned)(u >> 32), l = (unsigned)u;
    const unsigned e = (h >> 20) & 0x7ffu, sign = h & 0x80000000u;
    const unsigned nrm = sign | ((((h & 0x7fffffffu) - (896u << 20)) << 3) | (l >> 29));
    const unsigned big = ((e == 0x7ffu) && ((h & 0xfffffu) | l)) ? 0x7fc00000u : (sign | 0x7f800000u);
    return __uint_as_float(e < 897u ? sign : (e > 1150u ? big : nrm));
}
// Exact fp32 -> binary64 by integer operations only (fp32 subnormals give a
// signed zero; inf and nan keep their class).
__device__ __forceinline__ double f2d_exact(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t e = (u >> 23) & 0xffu;
    const unsigned long long ex = e == 0u ? 0ull : (e == 0xffu ? 2047ull : (unsigned long long)(e + 896u));
    const unsigned long long m = e == 0u ? 0ull : (unsigned long long)(u & 0x7fffffu) << 29;
    return __longlong_as_double((long long)(((unsigned long long)(u >> 31) << 63) | (ex << 52) | m));
}
// complex division a / b (Smith's method)
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    if (fabs(b.x) >= fabs(b.y)) {
        double r = b.y / b.x, den = b.x + b.y * r;
        return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
    } else {
        double r = b.x / b.y, den = b.x * r + b.y;
        return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
    }
}

// Importance factor of one walker (prop/afqmc.py:116-125): imp_ph =
// |exp(exponent) ratio| cos(theta) before the floor and cap, and
// phi = exp(-sqrt_dt shift_term) ratio whose angle is theta.  Shared by the
// weight update and its adjoint so that both see the same floor/cap masks.
struct WeightFactor {
    double imp_ph;
    double2 phi;
};
__device__ __forceinline__ WeightFactor weight_factor(double dt, double sqrt_dt, double ps, double2 h0_prop,
                                                      double2 st, double2 ft, double2 on, double2 op) {
    const double2 ratio = cdiv(on, op);
    const double2 ex = make_double2(-sqrt_dt * st.x + ft.x + dt * (ps + h0_prop.x),
                                    -sqrt_dt * st.y + ft.y + dt * h0_prop.y);
    double sn, cs;
    sincos(ex.y, &sn, &cs);
    const double er = exp(ex.x);
    const double2 imp = cmul(make_double2(er * cs, er * sn), ratio);
    // theta = angle(exp(-sqrt_dt shift_term) * ratio)
    sincos(-sqrt_dt * st.y, &sn, &cs);
    const double er2 = exp(-sqrt_dt * st.x);
    const double2 ph = cmul(make_double2(er2 * cs, er2 * sn), ratio);
    const double theta = atan2(ph.y, ph.x);
    WeightFactor f;
    f.imp_ph = hypot(imp.x, imp.y) * cos(theta);
    f.phi = ph;
    return f;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// -------------------------------------------- bf16 hi/lo split operands --
// x = h + m + l with h = bf16(x), m = bf16(x - h), l = bf16(x - h - m):
// three bf16 pieces carry 24 significant bits (an fp32 value exactly).  A row
// of a split operand holds `sec` K sections starting at 0, S, 2S, ... (S >= K)
// and is zero from sec*S up to its length Kt (a multiple of 64).  Six
// sections (AFQ_PREC_MIXED): a left (A) operand stores [h h m h l m], a
// right (B) operand [h m h l h m], so that A . B^T sums hh + hm + mh + hl +
// lh + mm -- every product above 2^-24 relative.  Three sections
// (AFQ_PREC_MIXED_FAST): [h h m] and [h m h], hh + hm + mh, ~2^-17 relative
// (bf16 has 8 significant bits).
inline int split_sections(int precision) { return precision == AFQ_PREC_MIXED_FAST ? 3 : 6; }
inline bool is_mixed(int precision) { return precision == AFQ_PREC_MIXED || precision == AFQ_PREC_MIXED_FAST; }

template <class T>
__device__ __forceinline__ void split_pieces(T x, __nv_bfloat16& h, __nv_bfloat16& m, __nv_bfloat16& l);
template <>
__device__ __forceinline__ void split_pieces<double>(double x, __nv_bfloat16& h, __nv_bfloat16& m,
                                                     __nv_bfloat16& l) {
    h = __double2bfloat16(x);
    const double r1 = x - (double)__bfloat162float(h);
    m = __double2bfloat16(r1);
    l = __double2bfloat16(r1 - (double)__bfloat162float(m));
}
template <>
__device__ __forceinline__ void split_pieces<float>(float x, __nv_bfloat16& h, __nv_bfloat16& m, __nv_bfloat16& l) {
    h = __float2bfloat16(x);
    const float r1 = x - __bfloat162float(h);  // exact
    m = __float2bfloat16(r1);
    l = __float2bfloat16(r1 - __bfloat162float(m));  // exact
}

template <class T>
__device__ __forceinline__ void split_store_t(__nv_bfloat16* row, int S, int k, T x, bool left, int sec) {
    __nv_bfloat16 h, m, l;
    split_pieces<T>(x, h, m, l);
    row[k] = h;
    row[S + k] = left ? h : m;
    row[2 * S + k] = left ? m : h;
    if (sec > 3) {
        row[3 * S + k] = left ? h : l;
        row[4 * S + k] = left ? l : h;
        row[5 * S + k] = m;
    }
}
__device__ __forceinline__ void split_store(__nv_bfloat16* row, int S, int k, double x, bool left, int sec) {
    split_store_t<double>(row, S, k, x, left, sec);
}
// Same split of an fp32 value, on the fp32 pipe.
__device__ __forceinline__ void split_storef(__nv_bfloat16* row, int S, int k, float x, bool left, int sec) {
    split_store_t<float>(row, S, k, x, left, sec);
}

// Destination of a split left operand written by a per-walker kernel: walker
// w's real parts go to row w, its imaginary parts to row W + w.
struct SplitOut {
    __nv_bfloat16* ptr = nullptr;
    int W = 0;
    long long ld = 0;  // row length Kt
    int S = 0;         // section stride
    int sec = 6;       // sections per row
};

// ------------------------------------------------------------- workspace --
// Bump allocator over a caller-provided workspace; every region is aligned
// to 256 bytes.  With base == nullptr it only measures.
struct Arena {
    char* base;
    size_t cap;
    size_t used;
    explicit Arena(void* b = nullptr, size_t c = 0) : base((char*)b), cap(c), used(0) {}
    template <class T>
    T* take(size_t count) {
        size_t off = (used + 255) & ~(size_t)255;
        used = off + count * sizeof(T);
        return base ? (T*)(base + off) : nullptr;
    }
    bool ok() const { return base == nullptr || used <= cap; }
};

inline cudaStream_t as_stream(void* s) { return (cudaStream_t)s; }

// --------------------------------------------------- launch entry points --
// k_setup.cu
int launch_mf_shifts(int n, int G, const double* chol, const double2* dm, double2* mf,
                     cudaStream_t s);
int launch_h1_eff(int n, int G, const double* h1, const double* chol, const double2* mf,
                  double* h1_eff, cudaStream_t s);
int launch_expm(int n, double scale, const double* a, double* out, double* tmp0, double* tmp1,
                double* tmp2, double* norm_dev, cudaStream_t s);
int launch_trial_rdm1(int n, int o, const double2* mo, double2* rdm1, cudaStream_t s);
int launch_rot(int n, int o, int G, const double* h1, const double* chol, const double2* mo,
               int trial_real, double2* rot_h1, void* rot_chol, cudaStream_t s);
int launch_h0_prop(int G, double h0, const double2* mf, double2* h0_prop, cudaStream_t s);
int launch_sum_spin_blocks(int n, const double2* rdm1, double2* dm, cudaStream_t s);

// k_gemm.cu : C (M x N complex) = alpha * A (M x K complex, lda) * B
//   B real or complex; B_TRANS: B(k, n) at B[n*ldb + k] else B[k*ldb + n]
int launch_zgemm(int M, int N, int K, double alpha, const double2* A, int64_t lda,
                 const void* B, int64_t ldb, bool b_complex, bool b_trans, double2* C,
                 int64_t ldc, cudaStream_t s);
// Same product with K split over CTA layers when the M x N tiles alone would
// not fill the GPU; C dense (ldc = N); part: zgemm_splits(M, N, K) x M x N
// scratch; the layers are added in a fixed order (deterministic).
int zgemm_splits(int M, int N, int K);
int launch_zgemm_splitk(int M, int N, int K, double alpha, const double2* A, int64_t lda, const void* B,
                        int64_t ldb, bool b_complex, bool b_trans, double2* C, double2* part, cudaStream_t s);

// k_walker.cu
int launch_green(int W, int n, int o, const double2* mo, int trial_real, const double2* walkers,
                 double2* ovlp_out, double2* green_out, cudaStream_t s);
// vdiv walkers share each V (2: the top and bottom halves of generalized walkers)
int launch_trotter(int W, int n, int o, int n_terms, double sqrt_dt, const double* E,
                   const double2* V, const double2* win, double2* wout, cudaStream_t s, int vdiv = 1);
int launch_field_shift(int W, int G, double sqrt_dt, const double* x, const double2* fb,
                       const double2* mf, double2* xs, double2* shift_term, double2* fb_term,
                       cudaStream_t s);
// overlaps[w] /= det_r[w]^2 (the overlaps of QR'd walkers from their QR's det(R))
int launch_overlap_div_det2(int W, const double2* det_r, double2* overlaps, cudaStream_t s);
int launch_weight_update(int W, const afq_params* p, double sqrt_dt, double dt,
                         double2 h0_prop, const double2* shift_term, const double2* fb_term,
                         const double2* ovlp_new, double* weights, double2* overlaps,
                         double* pop_shift, const double* e_est, cudaStream_t s,
                         int* status = nullptr);  // status: a workspace's status word, counts non-finite walkers
int launch_energy(int W, int n, int o, int G, double h0, const double2* green,
                  const void* rot_chol, int trial_real, const double2* rot_h1,
                  double* partial, double2* energy, cudaStream_t s);
int launch_qr(int W, int n, int o, const double2* win, double2* wout, double2* det_r,
              cudaStream_t s);
int launch_sr_scan(int W, const double* weights, double zeta, double* levels, int32_t* idx,
                   double* cumsum_out, double* avg_out, cudaStream_t s);
int launch_gather(int W, int64_t row, const int32_t* idx, const double2* src, double2* dst,
                  const double* avg, double* weights_out, cudaStream_t s);
int launch_block_measure(int W, double dt, double shift_ema, const double* weights,
                         const double2* energy, const double* e_est, double* pop_shift,
                         double* block_energy, double* block_weight, cudaStream_t s);
// While non-null (one thread's captured block loop), Philox counters are
// offsets from *t_counter_base on the device.
extern thread_local const uint64_t* t_counter_base;
bool timing_enabled();
int launch_run_record(const double* e, const double* w, double* es, double* ws, int* idx, uint64_t* counter,
                      uint64_t inc, cudaStream_t s);
int launch_philox(int64_t count, uint64_t seed, uint64_t counter, int normal, double* out,
                  cudaStream_t s);
size_t sr_levels_size(int W);
int launch_sr_scan_dev(int W, const double* weights, const double* zeta_dev, double* levels, int32_t* idx,
                       double* avg_out, cudaStream_t s);

// k_tc_gemm.cu : C (M x N fp32) = A (M x K bf16) . B (N x K bf16)^T on tcgen05
int launch_tc_gemm_tn(int M, int N, int K, const void* A, long long lda, const void* B, long long ldb, float* C,
                      long long ldc, int* err, cudaStream_t s);
// Same product with the K sum formed in fp32 registers per 64-wide K block
// (round-to-nearest) instead of in the tensor cores' truncating accumulator.
int launch_tc_gemm_tn_drain(int M, int N, int K, const void* A, long long lda, const void* B, long long ldb, float* C,
                            long long ldc, int* err, cudaStream_t s, int kd = 1);
// Same product, written as the two-piece bf16 split (hi, mid) of each sum.
int launch_tc_gemm_tn_drain_split(int M, int N, int K, const void* A, long long lda, const void* B, long long ldb,
                                  __nv_bfloat16* Ch, __nv_bfloat16* Cm, long long ldc, int* err, cudaStream_t s,
                                  int kd = 1);

// k_walker.cu : Green's function with an optional split (bf16) output
int launch_green_split(int W, int n, int o, const double2* mo, int trial_real, const double2* walkers,
                       double2* ovlp_out, double2* green_out, SplitOut split, cudaStream_t s, int ov_square = 1);
// det(C^H W) per walker (not squared: the unrestricted overlap's per-spin factor)
int launch_green_det(int W, int n, int o, const double2* mo, int trial_real, const double2* walkers,
                     double2* det_out, double2* green_out, cudaStream_t s);
// the energy's per-chunk partials (sum c^2, sum exchange) without the finish
int energy_partial_chunks(int o, int G);
int launch_energy_partial(int W, int n, int o, int G, const double2* green, const void* rot_chol, int trial_real,
                          double* partial, cudaStream_t s);
size_t energy_partial_count(int W, int o, int G);
int launch_energy_finish(int W, int n, int o, int nchunk, double h0, const double2* green, const double2* rot_h1,
                         const double2* partial, double2* energy, cudaStream_t s);

// k_mixed.cu
int launch_split_rows(long long rows, int K, int S, int Kt, const double* src, long long rs, long long ks,
                      __nv_bfloat16* dst, int left, int sec, cudaStream_t s, int grp = 0, int grp_pad = 0);
int launch_e_minus_i(int n, const double* E, float* out, cudaStream_t s);
int launch_field_shift_mixed(int W, int G, int Wc, double sqrt_dt, const double* x, const float* fbm, long long ldf,
                             const double2* mf, __nv_bfloat16* av, int S, int Kt, int sec, double2* shift_term,
                             double2* fb_term, cudaStream_t s);
int launch_trotter_mixed(int wc, int n, int o, int n_terms, double sqrt_dt, const float* emi, const float* vm,
                         long long ldv, const double2* win, double2* wout, float2* tsum, cudaStream_t s);
// cs (optional): (hi, lo) fp32 pairs of the trial orbitals -> double-float m
int launch_overlap_split(int W, int n, int o, const double2* mo, const double2* walkers, double2* ovlp_out,
                         SplitOut split, cudaStream_t s, double2* green_out = nullptr, const float2* cs = nullptr,
                         const float4* m_in = nullptr);

// k_ozaki.cu: m = C^T W of every walker from integer digit slices on the
// tensor cores, nocc <= 32, norb <= 584.
struct OzDims {
    int nks;  // K steps: eight orbitals each
    int K;    // 64 nks: eight K slots per orbital
    int NB;   // B rows: 8 per trial orbital, nocc rounded up to even
};
constexpr int OZ_NONFINITE = 0x7fffffff;  // E_r of a row holding inf or nan
OzDims oz_dims(int n, int o);
// B (NB x K) and F_a (o) from the trial orbitals
int launch_oz_split_c(int n, int o, const double2* mo, __nv_bfloat16* B, int* fa, cudaStream_t s);
// m[((w o + a) o + b) 2 + part] (double-float pairs) from the walkers
int launch_oz_m(int W, int n, int o, const double2* walkers, const __nv_bfloat16* B, const int* fa, float2* m,
                int* err, cudaStream_t s);
int launch_split_c(int count, const double2* mo, float2* cs, cudaStream_t s);
int launch_cholqr2(int W, int n, int o, const double2* win, double2* wout, double2* det_r, cudaStream_t s);
// k_cv.cu, k_mlp.cu
int launch_cv_features(int W, int n, int o, int G, double h0, const double2* green, const double2* rot_h1,
                       const float* fbm, long long ldf, const double2* ovlp, const float* shift, const float* scale,
                       float* feat, double* ebase, cudaStream_t s);
int launch_cv_pick(const double* u, int stride, int* off, cudaStream_t s);
int launch_cv_green_rows(int sc, int s0, const int* off, int stride, int W, int n, int o, int P, const double2* green,
                         __nv_bfloat16* dst, int S, int Kt, int sec, cudaStream_t s);
int launch_cv_record(int W, int nchunk, const double2* partial, double* xout, cudaStream_t s);
int launch_cv_measure(int W, double dt, double alpha, const double* weights, const double* ebase, const float* ynn,
                      double y_shift, double y_scale, int m_max, int stride, const int* off, int nchunk,
                      const double2* partial, const double* e_est, double* pop_shift, double* block_energy,
                      double* block_weight, double2* energy, double* stats, cudaStream_t s);
size_t mlp_param_count(int F, int H);
bool mlp_shape_supported(int F, int H);  // F a multiple of 16, H a multiple of 32 in [32, 256]
int launch_mlp_forward(int B, int F, int H, const __nv_bfloat16* p, const float* x, float* y, cudaStream_t s);
size_t mlp_train_ws_floats(int B, int F, int H);
int launch_mlp_grad_adam(int B, int F, int H, const __nv_bfloat16* wb_in, const float* x, const float* t, float* ws,
                         float* g_out, float* loss_out, float* w, __nv_bfloat16* wb, float* m, float* v, float lr,
                         int step, cudaStream_t s);
int launch_mlp_sync_bf16(size_t n, const float* w, __nv_bfloat16* wb, cudaStream_t s);
// k_trotter_tc.cu
bool trotter_tc_supported(int n, int o);
int launch_trotter_tc(int wc, int n, int o, int n_terms, double sqrt_dt, const __nv_bfloat16* eh,
                      const __nv_bfloat16* em, const __nv_bfloat16* vh, const __nv_bfloat16* vm, const double2* win,
                      double2* wout, int* err, cudaStream_t s);
int launch_e_minus_i_split(int n, const double* E, __nv_bfloat16* eh, __nv_bfloat16* em, cudaStream_t s);
int exchange_chunks(int G);
int launch_exchange_reduce(int wc, int G, int o, const float* F, long long ldf, double2* partial, cudaStream_t s);
int launch_green_rows(int wc, int n, int o, int P, const double2* green, __nv_bfloat16* dst, int S, int Kt, int sec,
                      cudaStream_t s);
// k_tc_gemm.cu : the energy GEMM with the exchange contraction in its epilogue
// (nocc <= 32 padded to 32-row blocks): A = the Green's-function rows of nw
// walkers (2 x 32 rows each), B = L~ rows (32 per Cholesky vector); writes
// x (nw x exchange_halves(G) x 2) and c (nw x G x 2) fp32 instead of F.
int launch_tc_gemm_exchange(int nw, int G, int K, const void* A, long long lda, const void* B, long long ldb,
                            float* x, float* c, int* err, cudaStream_t s, int kd = 1);
int exchange_halves(int G);
int launch_exchange_finish(int nw, int G, const float* x, const float* c, double2* partial, cudaStream_t s);

// k_adjoint.cu : reverse-mode kernels of the binary64 step and block
int launch_taylor_tape(int W, int n, int o, int K, double sqrt_dt, const double* E, const double2* V,
                       const double2* win, double2* terms, double2* w2, cudaStream_t s);
int launch_taylor_adj(int W, int n, int o, int K, double sqrt_dt, const double* E, const double2* V,
                      const double2* wbar_post, double2* tbar, double2* wbar_pre, cudaStream_t s);
int launch_vbar(int W, int n, int o, int K, double sqrt_dt, const double2* tbar, const double2* terms, double2* vbar,
                cudaStream_t s);
int ebar_splits(int W);
int launch_ebar(int W, int n, int o, const double2* X, long long xs, const double2* Y, long long ys, double* partial,
                cudaStream_t s);
int launch_sum_partials(int count, int ns, const double* partial, double* out, cudaStream_t s);
int launch_green_adj(int W, int n, int o, const double2* mo, const double2* walkers, const double2* gbar,
                     const double2* ov, const double2* ovbar, double2* wbar, int* err, cudaStream_t s);
int launch_qr_adj(int W, int n, int o, const double2* A, const double2* Q, const double2* qbar, double2* abar,
                  int* err, cudaStream_t s);
int launch_weight_adj(int W, const afq_params* p, double sqrt_dt, double dt, double2 h0_prop,
                      const double2* shift_term, const double2* fb_term, const double* w_pre, const double2* ov_pre,
                      const double* p_pre, const double* w_post, const double2* ov_post, double* wbar,
                      double2* ovbar, double* pbar, double2* ovn_tot, double* fbt_bar, double2* shift_bar,
                      cudaStream_t s);
int launch_fs_adj(int W, int G, double sqrt_dt, const double* x, const double2* fb, const double2* mf,
                  const double* fbt_bar, const double2* shift_bar, double2* xtb, cudaStream_t s);
int launch_measure_adj(int W, double dt, double alpha, const double* weights, const double2* energy,
                       const double* e_est, const double* e_block, const double* eb_bar, const double* wb_bar,
                       double* pbar, double* wbar, double* ebar_w, cudaStream_t s);
int launch_energy_gbar(int W, int on, const double* ebar_w, const double2* rot_h1, const double2* cl,
                       const double2* y, double2* gbar, cudaStream_t s);
int launch_sg_accum(int W, int on, const double* ebar_w, const double2* g, double2* sg, cudaStream_t s);
int launch_block_transpose(int wc, int o, int G, const double2* F, double2* Ft, cudaStream_t s);
int launch_sr_adj(int W, int no, const int32_t* idx, const double2* wk_in, const double2* ob_in, const double* wb_in,
                  const double* weights, double* wsum, double2* wk_out, double2* ob_out, double* wb_out, int* err,
                  cudaStream_t s);
int launch_h1bar(int n, int o, double dt, const double* h1_eff, const double* ebar, const double2* mo,
                 const double2* sg, double* h1bar, double* tmp, cudaStream_t s);

// afq_capi.cu : one binary64 block with the inputs of each operation saved.
// Operations of a block, in order: n_prop_steps steps with a QR after every
// qr_every-th one that is not the last, the block-end QR and overlap
// refresh, the measurement.  Snapshot slot k holds the input state of
// operation k; slot n_ops - 1 (the measurement) is the state after the QR.
struct BlockSnap {
    double2* walkers = nullptr;   // n_ops x W n o
    double* weights = nullptr;    // n_ops x W
    double2* overlaps = nullptr;  // n_ops x W
    double* pop = nullptr;        // n_ops
    double2* energy = nullptr;    // W local energies of the measurement
    double2* V = nullptr;         // optional, n_prop_steps x W n n: each step's V (one walker chunk only)
};
int block_op_count(const afq_params* p);
size_t block_ws_bytes(const afq_dims* d, int n_chunks);
// forced_idx (optional): comb indices used instead of the comb's own.
int run_block_taped(const afq_problem* pb, const afq_params* p, const afq_state* st, uint64_t seed,
                    uint64_t counter, const int32_t* forced_idx, int32_t* idx_out, double* block_energy,
                    double* block_weight, const BlockSnap* snap, void* workspace, size_t workspace_bytes,
                    cudaStream_t s);

inline long long round_up(long long x, long long m) { return (x + m - 1) / m * m; }

}  // namespace afq
