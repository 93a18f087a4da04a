// extern "C" entry points of libafqmc_gb300.so (declared in afqmc_gb300.h):
// argument checks, workspace layout, and the host-side orchestration of the
// step and block.  Nothing here allocates device memory or synchronises,
// except the set-up call afq_build_prop_ctx (one norm read-back for expm).
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "afq_internal.cuh"

namespace afq {

static thread_local char g_err[512] = "";

int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int check_cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return AFQ_OK;
    return fail(AFQ_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

size_t energy_partial_count(int W, int o, int G);

static int check_dims(const afq_dims* d, bool need_chol = true) {
    if (!d) return fail(AFQ_E_INVALID_ARGUMENT, "dims is NULL");
    if (d->n_walkers < 1) return fail(AFQ_E_INVALID_ARGUMENT, "n_walkers=%d < 1", d->n_walkers);
    if (d->norb < 1) return fail(AFQ_E_INVALID_ARGUMENT, "norb=%d < 1", d->norb);
    if (d->nocc < 1 || d->nocc > d->norb)
        return fail(AFQ_E_INVALID_ARGUMENT, "nocc=%d outside [1, norb=%d]", d->nocc, d->norb);
    if (d->nocc > 64) return fail(AFQ_E_UNSUPPORTED, "nocc=%d > 64", d->nocc);
    if (d->norb > 512) return fail(AFQ_E_UNSUPPORTED, "norb=%d > 512", d->norb);
    if (need_chol && d->nchol < 1) return fail(AFQ_E_INVALID_ARGUMENT, "nchol=%d < 1", d->nchol);
    if (d->precision != AFQ_PREC_FP64 && !is_mixed(d->precision))
        return fail(AFQ_E_INVALID_ARGUMENT, "unknown precision %d", d->precision);
    return AFQ_OK;
}

#define AFQ_NOTNULL(p)                                                      \
    do {                                                                    \
        if (!(p)) return fail(AFQ_E_INVALID_ARGUMENT, "%s is NULL", #p);    \
    } while (0)

static int check_ws(const Arena& a, size_t have) {
    if (a.used > have) return fail(AFQ_E_WORKSPACE, "workspace of %zu bytes < %zu needed", have, a.used);
    return AFQ_OK;
}

// ------------------------------------------------------- workspace layouts
static int chunk_size(int W, int n_chunks) { return n_chunks <= 1 ? W : (W + n_chunks - 1) / n_chunks; }

// Split-operand geometry of the mixed-precision GEMMs: section stride S and
// row length Kt (a multiple of the GEMM's K tile).
struct LowpDims {
    int S_V, Kt_V;   // V-build:    x~ (2W x G)       . L   (n^2 x G)
    int S_F, Kt_F;   // force bias: G_half (2W x o n) . L~  (G x o n)
    int S_E, Kt_E;   // energy:     L~ (G o x n)      . G_half rows (2 o W x n)
    int sec;         // sections per split row (6 or 3)
    long long ldv;   // row stride of V (fp32)
    bool xf;         // exchange contracted in the energy GEMM's epilogue (24 < nocc <= 32)
    int Pe;          // rows per (walker, part) block and per Cholesky vector in the energy GEMM
    int kd;          // 64-wide K blocks per tensor-core partial of the drained GEMMs
};

static LowpDims lowp_dims(const afq_dims* d) {
    LowpDims L;
    const int n = d->norb, o = d->nocc, G = d->nchol;
    L.sec = split_sections(d->precision);
    L.S_V = G;
    L.Kt_V = (int)round_up((long long)L.sec * G, 64);
    L.S_F = o * n;
    L.Kt_F = (int)round_up((long long)L.sec * o * n, 64);
    L.S_E = n;
    L.Kt_E = (int)round_up((long long)L.sec * n, 64);
    L.ldv = round_up((long long)n * n, 4);
    // blocks padded to 32 rows cost (32/o)^2 more GEMM work, and save writing and
    // reading F (G o x 2 o fp32 per walker): worth it for o close to 32
    L.xf = o > 24 && o <= 32;
    L.Pe = L.xf ? 32 : o;
    // the tensor cores' truncating fp32 sum over 256 products (bias ~2^-21 relative) stays below the
    // three-section split's 2^-17; the six-section form drains every 64 (bias < 2^-23)
    L.kd = d->precision == AFQ_PREC_MIXED_FAST ? 4 : 1;
    return L;
}

// Exchange partials per walker of the mixed energy (one with the fused GEMM).
static int exch_chunks(const afq_dims* d) { return lowp_dims(d).xf ? 1 : exchange_chunks(d->nchol); }

struct LowpBufs {
    __nv_bfloat16* Bv;  // n^2 x Kt_V   right operand [hi lo hi] of chol^T
    __nv_bfloat16* Bf;  // G x Kt_F     right operand of rot_chol_flat
    __nv_bfloat16* Le;  // G o x Kt_E   left operand [hi hi lo] of rot_chol
};

static LowpBufs layout_lowp(Arena& a, const afq_dims* d) {
    const LowpDims L = lowp_dims(d);
    const size_t n = d->norb, o = d->nocc, G = d->nchol;
    LowpBufs b;
    b.Bv = a.take<__nv_bfloat16>(n * n * L.Kt_V);
    b.Bf = a.take<__nv_bfloat16>(G * L.Kt_F);
    b.Le = a.take<__nv_bfloat16>(G * L.Pe * L.Kt_E);
    (void)o;
    return b;
}

struct StepWS {
    int* status;        // device status word (offset 0 of every step / block workspace)
    double* fields;     // W*G (drawn fields)
    double2 *shift_term, *fb_term, *ovl_new;  // W
    // binary64 form
    double2* green;     // W*o*n
    double2* fb;        // W*G
    double2* xs;        // W*G
    double2* V;         // Wc*n*n
    // mixed form
    __nv_bfloat16* Ag;  // 2W x Kt_F
    float* fbm;         // 2W x G
    __nv_bfloat16* Av;  // 2W x Kt_V
    float* Vm;          // 2Wc x ldv
    float* emi;         // n*n
    float2* tsum;       // Wc*n*o: fp32 sum of the Taylor terms of a chunk
    __nv_bfloat16* esplit;  // 2 n*n: E - I as bf16 hi, mid (tensor-core Taylor products)
    float2* csplit;     // n*o: trial orbitals as (hi, lo) fp32 pairs (double-float overlap)
    // m = C^T W on the tensor cores from integer digit slices (k_ozaki.cu), nocc <= 32
    __nv_bfloat16* ozB;  // NB x K: the trial's digit rows
    int* ozF;            // o: column exponents
    float2* ozM;         // W o o x 2: m as double-float pairs
};

// The tensor-core m of the mixed forms: nocc <= 32 and the digit sums exact
// (7 norb 2^12 < 2^24).
static bool oz_supported(const afq_dims* d) { return d->nocc <= 32 && d->norb <= 584; }

static StepWS layout_step(Arena& a, const afq_dims* d, int n_chunks) {
    const size_t W = d->n_walkers, n = d->norb, o = d->nocc, G = d->nchol;
    const size_t Wc = chunk_size(d->n_walkers, n_chunks);
    StepWS s = {};
    s.status = a.take<int>(64);
    s.fields = a.take<double>(W * G);
    s.shift_term = a.take<double2>(W);
    s.fb_term = a.take<double2>(W);
    s.ovl_new = a.take<double2>(W);
    if (is_mixed(d->precision)) {
        const LowpDims L = lowp_dims(d);
        s.Ag = a.take<__nv_bfloat16>(2 * W * L.Kt_F);
        s.fbm = a.take<float>(2 * W * G);
        s.Av = a.take<__nv_bfloat16>(2 * W * L.Kt_V);
        s.Vm = a.take<float>(2 * Wc * L.ldv);
        s.emi = a.take<float>(n * n);
        s.tsum = a.take<float2>(Wc * n * o);
        s.esplit = a.take<__nv_bfloat16>(2 * n * n);
        s.csplit = a.take<float2>(n * o);
        if (oz_supported(d)) {
            const OzDims z = oz_dims((int)n, (int)o);
            s.ozB = a.take<__nv_bfloat16>((size_t)z.NB * z.K);
            s.ozF = a.take<int>(64);
            s.ozM = a.take<float2>(W * o * o * 2);
        }
    } else {
        s.green = a.take<double2>(W * o * n);
        s.fb = a.take<double2>(W * G);
        s.xs = a.take<double2>(W * G);
        s.V = a.take<double2>(Wc * n * n);
    }
    return s;
}

// walkers per energy GEMM in the mixed form: F (G o x 2 o We fp32) <= 2 GiB,
// or with the fused exchange the Green's-function rows (2 x 32 x Kt_E bf16)
static int energy_chunk(const afq_dims* d) {
    const LowpDims L = lowp_dims(d);
    const long long per = L.xf ? 2LL * 32 * L.Kt_E * 2 : (long long)d->nchol * d->nocc * 2 * d->nocc * 4;
    long long we = (2LL << 30) / (per > 0 ? per : 1);
    if (we < 1) we = 1;
    if (we > d->n_walkers) we = d->n_walkers;
    return (int)we;
}

struct BlockWS {
    StepWS step;
    double2* green;      // W*o*n (energy)
    double2* energy;     // W
    double* partial;     // energy partials
    double* levels;      // comb scan
    int32_t* idx;        // W
    double* avg;         // 1
    double* zeta;        // 1
    double2* wcopy;      // W*n*o
    double2* ocopy;      // W
    __nv_bfloat16* Bg;   // mixed energy: 2 o We x Kt_E
    float* F;            // mixed energy: G o x 2 o We (not with the fused exchange)
    float* xsum;         // fused exchange: We x exchange_halves(G) x 2
    float* ctr;          // fused exchange: We x G x 2 traces of f_g
    float* cv_feat;      // mixed: W x AFQ_CV_FEATURES
    float* cv_y;         // mixed: W network outputs
    double* cv_ebase;    // mixed: W energies without exchange
    double* cv_u;        // mixed: 1 uniform
    int* cv_off;         // mixed: sample offset
};

static BlockWS layout_block(Arena& a, const afq_dims* d, int n_chunks) {
    BlockWS b = {};
    b.step = layout_step(a, d, n_chunks);
    const size_t W = d->n_walkers;
    b.green = is_mixed(d->precision) ? a.take<double2>(W * d->nocc * d->norb) : b.step.green;
    b.energy = a.take<double2>(W);
    if (is_mixed(d->precision)) {
        const LowpDims L = lowp_dims(d);
        const size_t we = energy_chunk(d);
        b.partial = (double*)a.take<double2>(W * exch_chunks(d) * 2);
        b.Bg = a.take<__nv_bfloat16>(2 * L.Pe * we * L.Kt_E);
        if (L.xf) {
            b.xsum = a.take<float>(we * exchange_halves(d->nchol) * 2);
            b.ctr = a.take<float>(we * d->nchol * 2);
        } else {
            b.F = a.take<float>((size_t)d->nchol * d->nocc * 2 * d->nocc * we);
        }
        b.cv_feat = a.take<float>(W * AFQ_CV_FEATURES);
        b.cv_y = a.take<float>(W);
        b.cv_ebase = a.take<double>(W);
        b.cv_u = a.take<double>(1);
        b.cv_off = a.take<int>(1);
    } else {
        b.partial = (double*)a.take<double2>(energy_partial_count(d->n_walkers, d->nocc, d->nchol));
    }
    b.levels = a.take<double>(sr_levels_size(d->n_walkers));
    b.idx = a.take<int32_t>(W);
    b.avg = a.take<double>(1);
    b.zeta = a.take<double>(1);
    b.wcopy = a.take<double2>(W * d->norb * d->nocc);
    b.ocopy = a.take<double2>(W);
    return b;
}

// ------------------------------------------------------------ step pieces
static int force_bias_from_green(const afq_dims* d, const double2* green, const double* rot_chol,
                                 double2* fb, cudaStream_t s) {
    const int on = d->nocc * d->norb;
    return launch_zgemm(d->n_walkers, d->nchol, on, 2.0, green, on, rot_chol, on, !d->trial_is_real, true, fb,
                        d->nchol, s);
}

static int trotter_chunked(const afq_dims* d, int n_terms, double sqrt_dt, int n_chunks, const double* chol,
                           const double* E, const double2* win, const double2* xs, double2* wout, double2* V,
                           cudaStream_t s) {
    const int W = d->n_walkers, n = d->norb, o = d->nocc, G = d->nchol;
    const int Wc = chunk_size(W, n_chunks);
    for (int w0 = 0; w0 < W; w0 += Wc) {
        const int wc = W - w0 < Wc ? W - w0 : Wc;
        // V (wc x n^2) = x~ (wc x G) . chol (G x n^2)   (prop/chol_afqmc_ops.py:70-74)
        { AFQ_PHASE("vbuild_gemm", s);
        AFQ_TRY(launch_zgemm(wc, n * n, G, 1.0, xs + (size_t)w0 * G, G, chol, (int64_t)n * n, false, false, V,
                             (int64_t)n * n, s)); }
        { AFQ_PHASE("trotter", s);
        AFQ_TRY(launch_trotter(wc, n, o, n_terms, sqrt_dt, E, V, win + (size_t)w0 * n * o,
                               wout + (size_t)w0 * n * o, s)); }
    }
    return AFQ_OK;
}

static int check_problem(const afq_problem* pb) {
    if (!pb) return fail(AFQ_E_INVALID_ARGUMENT, "problem is NULL");
    AFQ_TRY(check_dims(&pb->dims));
    AFQ_NOTNULL(pb->chol);
    AFQ_NOTNULL(pb->mo_coeff);
    AFQ_NOTNULL(pb->exp_h1_half);
    AFQ_NOTNULL(pb->mf_shifts);
    AFQ_NOTNULL(pb->rot_h1);
    AFQ_NOTNULL(pb->rot_chol);
    if (!(pb->dt > 0.0)) return fail(AFQ_E_INVALID_ARGUMENT, "dt=%g must be > 0", pb->dt);
    if (is_mixed(pb->dims.precision)) {
        if (!pb->lowp) return fail(AFQ_E_INVALID_ARGUMENT, "precision MIXED needs afq_prepare_lowp() output in lowp");
        if (!pb->dims.trial_is_real)
            return fail(AFQ_E_UNSUPPORTED, "precision MIXED supports real trial orbitals only");
    }
    return AFQ_OK;
}

// The mixed-precision step (AFQ_PREC_MIXED): same sequence as step_impl,
// with the force bias and V-build on tensor cores and the Taylor series in
// fp32 products accumulated into the binary64 walkers.
// Destination of the force-bias operand (split G_half) in a mixed workspace.
static SplitOut fb_split(const afq_dims* d, const StepWS& ws) {
    const LowpDims L = lowp_dims(d);
    SplitOut so;
    so.ptr = ws.Ag;
    so.W = d->n_walkers;
    so.ld = L.Kt_F;
    so.S = L.S_F;
    so.sec = L.sec;
    return so;
}

// The mixed forms' overlap pass: m = C^T W on the tensor cores when the
// workspace holds the digit buffers (else in double-float inside the
// overlap kernel), then the LU, the inverse and G_half per walker.
static int overlap_mixed(const afq_problem* pb, double2* walk, double2* ovl, SplitOut split, double2* green_out,
                         const StepWS& ws, cudaStream_t s) {
    const afq_dims* d = &pb->dims;
    const int W = d->n_walkers, n = d->norb, o = d->nocc;
    const double2* mo = (const double2*)pb->mo_coeff;
    if (ws.ozB) {
        AFQ_TRY(launch_oz_split_c(n, o, mo, ws.ozB, ws.ozF, s));
        AFQ_TRY(launch_oz_m(W, n, o, walk, ws.ozB, ws.ozF, ws.ozM, ws.status, s));
        return launch_overlap_split(W, n, o, mo, walk, ovl, split, s, green_out, ws.csplit, (const float4*)ws.ozM);
    }
    return launch_overlap_split(W, n, o, mo, walk, ovl, split, s, green_out, ws.csplit);
}

// green_ready: ws.Ag already holds the split G_half of the current walkers
// (written by the previous step's overlap kernel or by the overlap refresh
// after a QR inside the same block).
// green_out (optional): the overlap pass after the propagation also writes
// the new walkers' Green's function (fp32 values in binary64 storage) there.
static int step_mixed(const afq_problem* pb, const afq_params* p, const afq_state* st, const double* fields,
                      const StepWS& ws, bool green_ready, cudaStream_t s, double2* green_out = nullptr) {
    const afq_dims* d = &pb->dims;
    const int W = d->n_walkers, n = d->norb, o = d->nocc, G = d->nchol;
    const LowpDims L = lowp_dims(d);
    Arena la((void*)pb->lowp, (size_t)-1);
    const LowpBufs lb = layout_lowp(la, d);
    const double2* mo = (const double2*)pb->mo_coeff;
    double2* walk = (double2*)st->walkers;
    if (!ws.ozB) AFQ_TRY(launch_split_c(n * o, mo, ws.csplit, s));  // the double-float m (nocc > 32)
    // force bias: G_half split straight from the Green's function kernel
    if (!green_ready) {
        AFQ_PHASE("green", s);
        AFQ_TRY(overlap_mixed(pb, walk, nullptr, fb_split(d, ws), nullptr, ws, s));
    }
    { AFQ_PHASE("fb_gemm", s);
      AFQ_TRY(launch_tc_gemm_tn_drain(2 * W, G, L.Kt_F, ws.Ag, L.Kt_F, lb.Bf, L.Kt_F, ws.fbm, G, ws.status, s,
                                      L.kd)); }
    const int Wc = chunk_size(W, p->n_chunks);
    { AFQ_PHASE("field_shift", s);
      AFQ_TRY(launch_field_shift_mixed(W, G, Wc, pb->sqrt_dt, fields, ws.fbm, G, (const double2*)pb->mf_shifts, ws.Av,
                                       L.S_V, L.Kt_V, L.sec, ws.shift_term, ws.fb_term, s)); }
    // three-section form: V-build writes V as bf16 hi/mid pieces and the
    // Taylor products run on the tensor cores
    const bool tc_taylor = d->precision == AFQ_PREC_MIXED_FAST && trotter_tc_supported(n, o) && L.ldv == (long long)n * n;
    if (tc_taylor) {
        AFQ_TRY(launch_e_minus_i_split(n, pb->exp_h1_half, ws.esplit, ws.esplit + (size_t)n * n, s));
        for (int w0 = 0; w0 < W; w0 += Wc) {
            const int wc = W - w0 < Wc ? W - w0 : Wc;
            __nv_bfloat16* vh = (__nv_bfloat16*)ws.Vm;
            __nv_bfloat16* vmid = vh + (size_t)2 * wc * L.ldv;
            { AFQ_PHASE("vbuild_gemm", s);
              AFQ_TRY(launch_tc_gemm_tn_drain_split(2 * wc, n * n, L.Kt_V, ws.Av + (size_t)2 * w0 * L.Kt_V, L.Kt_V,
                                                    lb.Bv, L.Kt_V, vh, vmid, L.ldv, ws.status, s, L.kd)); }
            { AFQ_PHASE("trotter", s);
              AFQ_TRY(launch_trotter_tc(wc, n, o, p->n_exp_terms, pb->sqrt_dt, ws.esplit, ws.esplit + (size_t)n * n, vh,
                                        vmid, walk + (size_t)w0 * n * o, walk + (size_t)w0 * n * o, ws.status, s)); }
        }
    } else {
    AFQ_TRY(launch_e_minus_i(n, pb->exp_h1_half, ws.emi, s));
    for (int w0 = 0; w0 < W; w0 += Wc) {
        const int wc = W - w0 < Wc ? W - w0 : Wc;
        { AFQ_PHASE("vbuild_gemm", s);
          AFQ_TRY(launch_tc_gemm_tn_drain(2 * wc, n * n, L.Kt_V, ws.Av + (size_t)2 * w0 * L.Kt_V, L.Kt_V, lb.Bv, L.Kt_V,
                                    ws.Vm, L.ldv, ws.status, s)); }
        { AFQ_PHASE("trotter", s);
          AFQ_TRY(launch_trotter_mixed(wc, n, o, p->n_exp_terms, pb->sqrt_dt, ws.emi, ws.Vm, L.ldv,
                                       walk + (size_t)w0 * n * o, walk + (size_t)w0 * n * o, ws.tsum, s)); }
    }
    }
    // overlaps, and the next step's force-bias operand from the same factorisation
    { AFQ_PHASE("overlap", s);
      AFQ_TRY(overlap_mixed(pb, walk, ws.ovl_new, fb_split(d, ws), green_out, ws, s)); }
    AFQ_PHASE("weight_update", s);
    return launch_weight_update(W, p, pb->sqrt_dt, pb->dt, make_double2(pb->h0_prop_re, pb->h0_prop_im),
                                ws.shift_term, ws.fb_term, ws.ovl_new, st->weights, (double2*)st->overlaps,
                                st->pop_control_ene_shift, st->e_estimate, s, ws.status);
}

// Local energies of all walkers into ws.energy (meas/rhf.py:36-50).
// green_ready: ws.green already holds the Green's function of the walkers.
static int energy_impl(const afq_problem* pb, const afq_state* st, const BlockWS& ws, cudaStream_t s,
                       bool green_ready = false) {
    const afq_dims* d = &pb->dims;
    const int W = d->n_walkers, n = d->norb, o = d->nocc, G = d->nchol;
    if (!green_ready) {
        AFQ_PHASE("green", s);
        AFQ_TRY(launch_green(W, n, o, (const double2*)pb->mo_coeff, d->trial_is_real, (const double2*)st->walkers,
                             nullptr, ws.green, s));
    }
    AFQ_PHASE("energy", s);
    if (!is_mixed(d->precision))
        return launch_energy(W, n, o, G, pb->h0, ws.green, pb->rot_chol, d->trial_is_real,
                             (const double2*)pb->rot_h1, ws.partial, ws.energy, s);
    const LowpDims L = lowp_dims(d);
    Arena la((void*)pb->lowp, (size_t)-1);
    const LowpBufs lb = layout_lowp(la, d);
    const int We = energy_chunk(d), nch = exch_chunks(d);
    double2* partial = (double2*)ws.partial;
    for (int w0 = 0; w0 < W; w0 += We) {
        const int wc = W - w0 < We ? W - w0 : We;
        { AFQ_PHASE("e_green_rows", s);
          AFQ_TRY(launch_green_rows(wc, n, o, L.Pe, ws.green + (size_t)w0 * o * n, ws.Bg, L.S_E, L.Kt_E, L.sec,
                                    s)); }
        if (L.xf) {
            { AFQ_PHASE("e_gemm", s);
              AFQ_TRY(launch_tc_gemm_exchange(wc, G, L.Kt_E, ws.Bg, L.Kt_E, lb.Le, L.Kt_E, ws.xsum, ws.ctr,
                                              ws.step.status, s, L.kd)); }
            { AFQ_PHASE("e_exchange", s);
              AFQ_TRY(launch_exchange_finish(wc, G, ws.xsum, ws.ctr, partial + (size_t)w0 * nch * 2, s)); }
            continue;
        }
        // F[(w, part, k), (g, i)]: the six sections of Bg (left) and Le
        // (right) pair up as hh + hm + mh + hl + lh + mm
        { AFQ_PHASE("e_gemm", s);
          AFQ_TRY(launch_tc_gemm_tn_drain(2 * o * wc, G * o, L.Kt_E, ws.Bg, L.Kt_E, lb.Le, L.Kt_E, ws.F,
                                          (long long)G * o, ws.step.status, s)); }
        { AFQ_PHASE("e_exchange", s);
          AFQ_TRY(launch_exchange_reduce(wc, G, o, ws.F, (long long)G * o, partial + (size_t)w0 * nch * 2, s)); }
    }
    return launch_energy_finish(W, n, o, nch, pb->h0, ws.green, (const double2*)pb->rot_h1, partial, ws.energy, s);
}

static int check_state(const afq_state* st) {
    if (!st) return fail(AFQ_E_INVALID_ARGUMENT, "state is NULL");
    AFQ_NOTNULL(st->walkers);
    AFQ_NOTNULL(st->weights);
    AFQ_NOTNULL(st->overlaps);
    AFQ_NOTNULL(st->pop_control_ene_shift);
    AFQ_NOTNULL(st->e_estimate);
    return AFQ_OK;
}

static int check_params(const afq_params* p) {
    if (!p) return fail(AFQ_E_INVALID_ARGUMENT, "params is NULL");
    if (p->n_exp_terms < 0) return fail(AFQ_E_INVALID_ARGUMENT, "n_exp_terms=%d < 0", p->n_exp_terms);
    if (p->n_prop_steps < 0) return fail(AFQ_E_INVALID_ARGUMENT, "n_prop_steps=%d < 0", p->n_prop_steps);
    if (!(p->dt > 0.0)) return fail(AFQ_E_INVALID_ARGUMENT, "dt=%g must be > 0", p->dt);
    return AFQ_OK;
}

static int step_impl(const afq_problem* pb, const afq_params* p, const afq_state* st, const double* fields,
                     uint64_t seed, uint64_t counter, const StepWS& ws, cudaStream_t s, bool green_ready = false,
                     double2* green_out = nullptr) {
    const afq_dims* d = &pb->dims;
    const int W = d->n_walkers, n = d->norb, o = d->nocc, G = d->nchol;
    const double2* mo = (const double2*)pb->mo_coeff;
    double2* walk = (double2*)st->walkers;
    if (!fields) {
        AFQ_PHASE("philox", s);
        AFQ_TRY(launch_philox((int64_t)W * G, seed, counter, 1, ws.fields, s));
        fields = ws.fields;
    }
    if (is_mixed(d->precision)) return step_mixed(pb, p, st, fields, ws, green_ready, s, green_out);
    // force bias (prop/afqmc.py:90-95)
    { AFQ_PHASE("green", s); AFQ_TRY(launch_green(W, n, o, mo, d->trial_is_real, walk, nullptr, ws.green, s)); }
    { AFQ_PHASE("fb_gemm", s); AFQ_TRY(force_bias_from_green(d, ws.green, pb->rot_chol, ws.fb, s)); }
    // shifts (prop/afqmc.py:97-101)
    { AFQ_PHASE("field_shift", s);
    AFQ_TRY(launch_field_shift(W, G, pb->sqrt_dt, fields, ws.fb, (const double2*)pb->mf_shifts, ws.xs,
                               ws.shift_term, ws.fb_term, s)); }
    // propagation (prop/afqmc.py:103-110)
    AFQ_TRY(trotter_chunked(d, p->n_exp_terms, pb->sqrt_dt, p->n_chunks, pb->chol, pb->exp_h1_half, walk, ws.xs,
                            walk, ws.V, s));
    // overlaps (prop/afqmc.py:112-114)
    { AFQ_PHASE("overlap", s); AFQ_TRY(launch_green(W, n, o, mo, d->trial_is_real, walk, ws.ovl_new, nullptr, s)); }
    AFQ_PHASE("weight_update", s);
    // weights (prop/afqmc.py:116-138)
    return launch_weight_update(W, p, pb->sqrt_dt, pb->dt, make_double2(pb->h0_prop_re, pb->h0_prop_im),
                                ws.shift_term, ws.fb_term, ws.ovl_new, st->weights, (double2*)st->overlaps,
                                st->pop_control_ene_shift, st->e_estimate, s, ws.status);
}

// QR and overlap refresh (prop/blocks.py:53-57); in the mixed form the same
// kernel also writes the next step's force-bias operand into ws->Ag.
// QR of the walkers, then their overlaps from the same pass that writes
// either the next step's force-bias operand (mixed, ws given) or, with
// green_out, the Green's function the block's energy needs.
//
// Mixed forms, when the Green's function of the walkers before the QR is
// already in place (ws given: the force-bias operand the last overlap pass
// wrote; green_kept: green_out written by the last step): Q = W R^-1 leaves
// G_half = (W m^-1)^T unchanged (m_Q = m R^-1), and det(C^H Q)^2 =
// det(C^H W)^2 / det(R)^2, so the QR's det(R) updates the overlaps and no
// overlap pass runs.  The binary64 form recomputes them, as the reference
// does (prop/blocks.py:53-57).
static int orthonormalize_refresh(const afq_problem* pb, const afq_state* st, cudaStream_t s,
                                  const StepWS* ws = nullptr, double2* green_out = nullptr,
                                  const float2* cs = nullptr, double2* det_buf = nullptr, bool green_kept = false,
                                  const StepWS* green_ws = nullptr) {
    const afq_dims* d = &pb->dims;
    double2* walk = (double2*)st->walkers;
    const bool keep = is_mixed(d->precision) && det_buf && (ws || green_kept);
    {
        AFQ_PHASE("qr", s);
        if (is_mixed(d->precision))
            AFQ_TRY(launch_cholqr2(d->n_walkers, d->norb, d->nocc, walk, walk, keep ? det_buf : nullptr, s));
        else AFQ_TRY(launch_qr(d->n_walkers, d->norb, d->nocc, walk, walk, nullptr, s));
    }
    if (keep) {
        AFQ_PHASE("overlap_rescale", s);
        return launch_overlap_div_det2(d->n_walkers, det_buf, (double2*)st->overlaps, s);
    }
    AFQ_PHASE(green_out ? "green" : "overlap", s);
    if (ws && is_mixed(d->precision))
        return overlap_mixed(pb, walk, (double2*)st->overlaps, fb_split(d, *ws), nullptr, *ws, s);
    // the three-section energy resolves less than fp32: its Green's function in fp32
    // (with m from the same tensor-core pass as every other overlap of the block)
    if (green_out && d->precision == AFQ_PREC_MIXED_FAST && green_ws)
        return overlap_mixed(pb, walk, (double2*)st->overlaps, SplitOut{}, green_out, *green_ws, s);
    if (green_out && d->precision == AFQ_PREC_MIXED_FAST)
        return launch_overlap_split(d->n_walkers, d->norb, d->nocc, (const double2*)pb->mo_coeff, walk,
                                    (double2*)st->overlaps, SplitOut{}, s, green_out, cs);
    return launch_green(d->n_walkers, d->norb, d->nocc, (const double2*)pb->mo_coeff, d->trial_is_real, walk,
                        (double2*)st->overlaps, green_out, s);
}

}  // namespace afq

using namespace afq;

extern "C" {

int afq_abi_version(void) { return AFQ_ABI_VERSION; }

const char* afq_status_string(int status) {
    switch (status) {
        case AFQ_OK: return "ok";
        case AFQ_E_INVALID_ARGUMENT: return "invalid argument";
        case AFQ_E_UNSUPPORTED: return "unsupported size or mode";
        case AFQ_E_CUDA: return "CUDA error";
        case AFQ_E_WORKSPACE: return "workspace too small";
        case AFQ_E_DEVICE_CHECK: return "device-side check failed";
        default: return "unknown status";
    }
}

const char* afq_last_error(void) { return g_err; }

// ------------------------------------------------------------------ set-up
size_t afq_build_prop_ctx_workspace(int32_t norb, int32_t nchol) {
    (void)nchol;
    Arena a;
    a.take<int>(64);  // status word: offset 0 of every workspace
    a.take<double2>((size_t)norb * norb);  // dm
    a.take<double>((size_t)norb * norb);   // h1_eff
    for (int k = 0; k < 3; ++k) a.take<double>((size_t)norb * norb);
    a.take<double>(1);
    return a.used;
}

int afq_build_prop_ctx(int32_t norb, int32_t nchol, double h0, double dt, const double* h1, const double* chol,
                       const double* rdm1, int32_t rdm1_spin_blocks, double* exp_h1_half, double* mf_shifts,
                       double* h0_prop, void* workspace, size_t workspace_bytes, void* stream) {
    if (norb < 1 || nchol < 1) return fail(AFQ_E_INVALID_ARGUMENT, "norb=%d nchol=%d", norb, nchol);
    AFQ_NOTNULL(h1); AFQ_NOTNULL(chol); AFQ_NOTNULL(rdm1);
    AFQ_NOTNULL(exp_h1_half); AFQ_NOTNULL(mf_shifts); AFQ_NOTNULL(h0_prop); AFQ_NOTNULL(workspace);
    if (!(dt > 0.0)) return fail(AFQ_E_INVALID_ARGUMENT, "dt=%g must be > 0", dt);
    cudaStream_t s = as_stream(stream);
    const int n = norb;
    Arena a(workspace, workspace_bytes);
    a.take<int>(64);  // status word: offset 0 of every workspace
    double2* dm = a.take<double2>((size_t)n * n);
    double* h1e = a.take<double>((size_t)n * n);
    double* t0 = a.take<double>((size_t)n * n);
    double* t1 = a.take<double>((size_t)n * n);
    double* t2 = a.take<double>((size_t)n * n);
    double* nrm = a.take<double>(1);
    AFQ_TRY(check_ws(a, workspace_bytes));
    const double2* dmp = (const double2*)rdm1;
    if (rdm1_spin_blocks) {
        AFQ_TRY(launch_sum_spin_blocks(n, (const double2*)rdm1, dm, s));
        dmp = dm;
    }
    AFQ_TRY(launch_mf_shifts(n, nchol, chol, dmp, (double2*)mf_shifts, s));
    AFQ_TRY(launch_h0_prop(nchol, h0, (const double2*)mf_shifts, (double2*)h0_prop, s));
    AFQ_TRY(launch_h1_eff(n, nchol, h1, chol, (const double2*)mf_shifts, h1e, s));
    AFQ_TRY(launch_expm(n, -0.5 * dt, h1e, exp_h1_half, t0, t1, t2, nrm, s));
    return AFQ_OK;
}

int afq_trial_rdm1(int32_t norb, int32_t nocc, const double* mo_coeff, double* rdm1, void* stream) {
    if (norb < 1 || nocc < 1 || nocc > norb) return fail(AFQ_E_INVALID_ARGUMENT, "norb=%d nocc=%d", norb, nocc);
    AFQ_NOTNULL(mo_coeff); AFQ_NOTNULL(rdm1);
    return launch_trial_rdm1(norb, nocc, (const double2*)mo_coeff, (double2*)rdm1, as_stream(stream));
}

int afq_build_meas_ctx(int32_t norb, int32_t nocc, int32_t nchol, const double* h1, const double* chol,
                       const double* mo_coeff, int32_t trial_is_real, double* rot_h1, double* rot_chol,
                       void* stream) {
    if (norb < 1 || nocc < 1 || nocc > norb || nchol < 1)
        return fail(AFQ_E_INVALID_ARGUMENT, "norb=%d nocc=%d nchol=%d", norb, nocc, nchol);
    AFQ_NOTNULL(h1); AFQ_NOTNULL(chol); AFQ_NOTNULL(mo_coeff); AFQ_NOTNULL(rot_h1); AFQ_NOTNULL(rot_chol);
    return launch_rot(norb, nocc, nchol, h1, chol, (const double2*)mo_coeff, trial_is_real, (double2*)rot_h1,
                      rot_chol, as_stream(stream));
}

int afq_lowp_gemm_tn(int32_t M, int32_t N, int32_t K, const void* A, int64_t lda, const void* B, int64_t ldb,
                     float* C, int64_t ldc, int32_t* err, int32_t accumulate, void* stream) {
    AFQ_NOTNULL(A); AFQ_NOTNULL(B); AFQ_NOTNULL(C); AFQ_NOTNULL(err);
    if (M < 0 || N < 0 || lda < K || ldb < K || ldc < N)
        return fail(AFQ_E_INVALID_ARGUMENT, "lowp gemm: bad sizes M=%d N=%d K=%d", M, N, K);
    if (accumulate >= 1)
        return launch_tc_gemm_tn_drain(M, N, K, A, lda, B, ldb, C, ldc, err, as_stream(stream), accumulate);
    if (accumulate != 0) return fail(AFQ_E_INVALID_ARGUMENT, "accumulate=%d must be >= 0", accumulate);
    return launch_tc_gemm_tn(M, N, K, A, lda, B, ldb, C, ldc, err, as_stream(stream));
}

int afq_workspace_counters(void* workspace, int32_t* status, int32_t* nonfinite, void* stream) {
    AFQ_NOTNULL(workspace); AFQ_NOTNULL(status);
    cudaStream_t s = as_stream(stream);
    int32_t v[2] = {0, 0};
    AFQ_CUDA(cudaMemcpyAsync(v, workspace, sizeof(v), cudaMemcpyDeviceToHost, s));
    AFQ_CUDA(cudaStreamSynchronize(s));
    *status = v[0];
    if (nonfinite) *nonfinite = v[1];
    if (v[0] != 0 || v[1] != 0) AFQ_CUDA(cudaMemsetAsync(workspace, 0, sizeof(v), s));
    if (v[0] != 0)
        return fail(AFQ_E_DEVICE_CHECK, "device-side check failed (status %d: %s)", v[0],
                    v[0] == AFQ_STATUS_WAIT_EXPIRED ? "a bounded wait expired"
                    : v[0] == AFQ_STATUS_SINGULAR   ? "singular matrix in an adjoint kernel"
                    : v[0] == AFQ_STATUS_NONFINITE  ? "non-finite walker overlaps or weights"
                                                    : "comb indices out of order or range");
    return AFQ_OK;
}

int afq_workspace_status(void* workspace, int32_t* status, void* stream) {
    return afq_workspace_counters(workspace, status, nullptr, stream);
}

size_t afq_lowp_bytes(const afq_dims* d) {
    if (check_dims(d) != AFQ_OK) return 0;
    Arena a;
    layout_lowp(a, d);
    return a.used + 256;
}

int afq_prepare_lowp(const afq_dims* d, const double* chol, const double* rot_chol, void* out, size_t out_bytes,
                     void* stream) {
    AFQ_TRY(check_dims(d));
    AFQ_NOTNULL(chol); AFQ_NOTNULL(rot_chol); AFQ_NOTNULL(out);
    if (!d->trial_is_real) return fail(AFQ_E_UNSUPPORTED, "precision MIXED supports real trial orbitals only");
    if (((uintptr_t)out) & 255) return fail(AFQ_E_INVALID_ARGUMENT, "lowp buffer must be 256-byte aligned");
    Arena a(out, out_bytes);
    const LowpBufs b = layout_lowp(a, d);
    AFQ_TRY(check_ws(a, out_bytes));
    const LowpDims L = lowp_dims(d);
    const long long n = d->norb, o = d->nocc, G = d->nchol;
    cudaStream_t s = as_stream(stream);
    // chol^T: row j = (i, k) of L_g[i, k] over g   (right operand of the V-build)
    AFQ_TRY(launch_split_rows(n * n, (int)G, L.S_V, L.Kt_V, chol, 1, n * n, b.Bv, 0, L.sec, s));
    // rot_chol_flat: row g over (p, j)              (right operand of the force bias)
    AFQ_TRY(launch_split_rows(G, (int)(o * n), L.S_F, L.Kt_F, rot_chol, o * n, 1, b.Bf, 0, L.sec, s));
    // rot_chol rows (g, p) over j                   (left operand of the energy);
    // with the fused exchange, blocks of 32 rows per g (rows p >= o zero)
    if (L.xf) {
        AFQ_CUDA(cudaMemsetAsync(b.Le, 0, sizeof(__nv_bfloat16) * (size_t)G * L.Pe * L.Kt_E, s));
        AFQ_TRY(launch_split_rows(G * o, (int)n, L.S_E, L.Kt_E, rot_chol, n, 1, b.Le, 1, L.sec, s, (int)o, L.Pe));
    } else {
        AFQ_TRY(launch_split_rows(G * o, (int)n, L.S_E, L.Kt_E, rot_chol, n, 1, b.Le, 1, L.sec, s));
    }
    return AFQ_OK;
}

// ----------------------------------------------------------- walker kernels
int afq_overlap(const afq_dims* d, const double* mo_coeff, const double* walkers, double* overlaps, void* stream) {
    AFQ_TRY(check_dims(d, false));
    AFQ_NOTNULL(mo_coeff); AFQ_NOTNULL(walkers); AFQ_NOTNULL(overlaps);
    return launch_green(d->n_walkers, d->norb, d->nocc, (const double2*)mo_coeff, d->trial_is_real,
                        (const double2*)walkers, (double2*)overlaps, nullptr, as_stream(stream));
}

int afq_half_green(const afq_dims* d, const double* mo_coeff, const double* walkers, double* green,
                   double* overlaps, void* stream) {
    AFQ_TRY(check_dims(d, false));
    AFQ_NOTNULL(mo_coeff); AFQ_NOTNULL(walkers); AFQ_NOTNULL(green);
    return launch_green(d->n_walkers, d->norb, d->nocc, (const double2*)mo_coeff, d->trial_is_real,
                        (const double2*)walkers, (double2*)overlaps, (double2*)green, as_stream(stream));
}

size_t afq_force_bias_workspace(const afq_dims* d) {
    if (check_dims(d) != AFQ_OK) return 0;
    Arena a;
    a.take<int>(64);  // status word: offset 0 of every workspace
    a.take<double2>((size_t)d->n_walkers * d->nocc * d->norb);
    return a.used;
}

int afq_force_bias(const afq_dims* d, const double* mo_coeff, const double* rot_chol, const double* walkers,
                   double* force_bias, void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_dims(d));
    AFQ_NOTNULL(mo_coeff); AFQ_NOTNULL(rot_chol); AFQ_NOTNULL(walkers); AFQ_NOTNULL(force_bias);
    AFQ_NOTNULL(workspace);
    Arena a(workspace, workspace_bytes);
    a.take<int>(64);  // status word: offset 0 of every workspace
    double2* green = a.take<double2>((size_t)d->n_walkers * d->nocc * d->norb);
    AFQ_TRY(check_ws(a, workspace_bytes));
    cudaStream_t s = as_stream(stream);
    AFQ_TRY(launch_green(d->n_walkers, d->norb, d->nocc, (const double2*)mo_coeff, d->trial_is_real,
                         (const double2*)walkers, nullptr, green, s));
    return force_bias_from_green(d, green, rot_chol, (double2*)force_bias, s);
}

size_t afq_energy_workspace(const afq_dims* d) {
    if (check_dims(d) != AFQ_OK) return 0;
    Arena a;
    a.take<int>(64);  // status word: offset 0 of every workspace
    a.take<double2>((size_t)d->n_walkers * d->nocc * d->norb);
    a.take<double2>(energy_partial_count(d->n_walkers, d->nocc, d->nchol));
    return a.used;
}

int afq_energy(const afq_dims* d, double h0, const double* mo_coeff, const double* rot_h1, const double* rot_chol,
               const double* walkers, double* energy, void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_dims(d));
    AFQ_NOTNULL(mo_coeff); AFQ_NOTNULL(rot_h1); AFQ_NOTNULL(rot_chol); AFQ_NOTNULL(walkers); AFQ_NOTNULL(energy);
    AFQ_NOTNULL(workspace);
    Arena a(workspace, workspace_bytes);
    a.take<int>(64);  // status word: offset 0 of every workspace
    double2* green = a.take<double2>((size_t)d->n_walkers * d->nocc * d->norb);
    double* partial = (double*)a.take<double2>(energy_partial_count(d->n_walkers, d->nocc, d->nchol));
    AFQ_TRY(check_ws(a, workspace_bytes));
    cudaStream_t s = as_stream(stream);
    AFQ_TRY(launch_green(d->n_walkers, d->norb, d->nocc, (const double2*)mo_coeff, d->trial_is_real,
                         (const double2*)walkers, nullptr, green, s));
    return launch_energy(d->n_walkers, d->norb, d->nocc, d->nchol, h0, green, rot_chol, d->trial_is_real,
                         (const double2*)rot_h1, partial, (double2*)energy, s);
}

size_t afq_apply_trotter_workspace(const afq_dims* d, int32_t n_chunks) {
    if (check_dims(d) != AFQ_OK) return 0;
    Arena a;
    a.take<int>(64);  // status word: offset 0 of every workspace
    a.take<double2>((size_t)chunk_size(d->n_walkers, n_chunks) * d->norb * d->norb);
    return a.used;
}

int afq_apply_trotter(const afq_dims* d, int32_t n_terms, double sqrt_dt, int32_t n_chunks, const double* chol,
                      const double* exp_h1_half, const double* walkers, const double* shifted_fields,
                      double* walkers_out, void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_dims(d));
    AFQ_NOTNULL(chol); AFQ_NOTNULL(exp_h1_half); AFQ_NOTNULL(walkers); AFQ_NOTNULL(shifted_fields);
    AFQ_NOTNULL(walkers_out); AFQ_NOTNULL(workspace);
    if (n_terms < 0) return fail(AFQ_E_INVALID_ARGUMENT, "n_terms=%d < 0", n_terms);
    Arena a(workspace, workspace_bytes);
    a.take<int>(64);  // status word: offset 0 of every workspace
    double2* V = a.take<double2>((size_t)chunk_size(d->n_walkers, n_chunks) * d->norb * d->norb);
    AFQ_TRY(check_ws(a, workspace_bytes));
    return trotter_chunked(d, n_terms, sqrt_dt, n_chunks, chol, exp_h1_half, (const double2*)walkers,
                           (const double2*)shifted_fields, (double2*)walkers_out, V, as_stream(stream));
}

int afq_orthogonalize(const afq_dims* d, const double* walkers, double* walkers_out, double* det_r, void* stream) {
    AFQ_TRY(check_dims(d, false));
    AFQ_NOTNULL(walkers); AFQ_NOTNULL(walkers_out);
    if (is_mixed(d->precision))
        return launch_cholqr2(d->n_walkers, d->norb, d->nocc, (const double2*)walkers, (double2*)walkers_out,
                              (double2*)det_r, as_stream(stream));
    return launch_qr(d->n_walkers, d->norb, d->nocc, (const double2*)walkers, (double2*)walkers_out,
                     (double2*)det_r, as_stream(stream));
}

size_t afq_sr_workspace(int32_t n_walkers) {
    Arena a;
    a.take<int>(64);  // status word: offset 0 of every workspace
    a.take<double>(sr_levels_size(n_walkers));
    a.take<int32_t>(n_walkers);
    a.take<double>(1);
    return a.used;
}

int afq_sr_indices(int32_t n_walkers, const double* weights, double zeta, int32_t* idx, double* cumsum,
                   void* workspace, size_t workspace_bytes, void* stream) {
    if (n_walkers < 1) return fail(AFQ_E_INVALID_ARGUMENT, "n_walkers=%d < 1", n_walkers);
    AFQ_NOTNULL(weights); AFQ_NOTNULL(idx); AFQ_NOTNULL(workspace);
    Arena a(workspace, workspace_bytes);
    a.take<int>(64);  // status word: offset 0 of every workspace
    double* lv = a.take<double>(sr_levels_size(n_walkers));
    AFQ_TRY(check_ws(a, workspace_bytes));
    return launch_sr_scan(n_walkers, weights, zeta, lv, idx, cumsum, nullptr, as_stream(stream));
}

int afq_stochastic_reconfiguration(const afq_dims* d, const double* weights, double zeta, const double* walkers,
                                   double* walkers_out, double* weights_out, int32_t* idx, void* workspace,
                                   size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_dims(d, false));
    AFQ_NOTNULL(weights); AFQ_NOTNULL(walkers); AFQ_NOTNULL(walkers_out); AFQ_NOTNULL(weights_out);
    AFQ_NOTNULL(workspace);
    if (walkers == walkers_out) return fail(AFQ_E_INVALID_ARGUMENT, "walkers_out must not alias walkers");
    Arena a(workspace, workspace_bytes);
    a.take<int>(64);  // status word: offset 0 of every workspace
    double* lv = a.take<double>(sr_levels_size(d->n_walkers));
    int32_t* id = a.take<int32_t>(d->n_walkers);
    double* avg = a.take<double>(1);
    AFQ_TRY(check_ws(a, workspace_bytes));
    cudaStream_t s = as_stream(stream);
    AFQ_TRY(launch_sr_scan(d->n_walkers, weights, zeta, lv, id, nullptr, avg, s));
    AFQ_TRY(launch_gather(d->n_walkers, (int64_t)d->norb * d->nocc, id, (const double2*)walkers,
                          (double2*)walkers_out, avg, weights_out, s));
    if (idx) AFQ_CUDA(cudaMemcpyAsync(idx, id, sizeof(int32_t) * d->n_walkers, cudaMemcpyDeviceToDevice, s));
    return AFQ_OK;
}

// ------------------------------------------------------------- step pieces
int afq_fill_normal(int64_t count, uint64_t seed, uint64_t counter, double* out, void* stream) {
    AFQ_NOTNULL(out);
    return launch_philox(count, seed, counter, 1, out, as_stream(stream));
}

int afq_fill_uniform(int64_t count, uint64_t seed, uint64_t counter, double* out, void* stream) {
    AFQ_NOTNULL(out);
    return launch_philox(count, seed, counter, 0, out, as_stream(stream));
}

int afq_field_shift(const afq_dims* d, double sqrt_dt, const double* fields, const double* force_bias,
                    const double* mf_shifts, double* shifted_fields, double* shift_term, double* fb_term,
                    void* stream) {
    AFQ_TRY(check_dims(d));
    AFQ_NOTNULL(fields); AFQ_NOTNULL(force_bias); AFQ_NOTNULL(mf_shifts); AFQ_NOTNULL(shifted_fields);
    AFQ_NOTNULL(shift_term); AFQ_NOTNULL(fb_term);
    return launch_field_shift(d->n_walkers, d->nchol, sqrt_dt, fields, (const double2*)force_bias,
                              (const double2*)mf_shifts, (double2*)shifted_fields, (double2*)shift_term,
                              (double2*)fb_term, as_stream(stream));
}

size_t afq_field_shift_lowp_bytes(int32_t n_walkers, int32_t nchol, int32_t sections) {
    if (n_walkers < 1 || nchol < 1 || (sections != 3 && sections != 6)) return 0;
    const size_t Kt = ((size_t)sections * nchol + 63) / 64 * 64;
    return 2 * (size_t)n_walkers * Kt * sizeof(__nv_bfloat16);
}

int afq_field_shift_lowp(int32_t n_walkers, int32_t nchol, int32_t sections, double sqrt_dt, const double* fields,
                         const float* force_bias_half, const double* mf_shifts, double* shift_term,
                         double* fb_term, void* split_out, size_t split_bytes, void* stream) {
    if (n_walkers < 1 || nchol < 1) return fail(AFQ_E_INVALID_ARGUMENT, "n_walkers=%d nchol=%d", n_walkers, nchol);
    if (sections != 3 && sections != 6) return fail(AFQ_E_INVALID_ARGUMENT, "sections=%d must be 3 or 6", sections);
    AFQ_NOTNULL(fields); AFQ_NOTNULL(force_bias_half); AFQ_NOTNULL(mf_shifts); AFQ_NOTNULL(shift_term);
    AFQ_NOTNULL(fb_term); AFQ_NOTNULL(split_out);
    if (split_bytes < afq_field_shift_lowp_bytes(n_walkers, nchol, sections))
        return fail(AFQ_E_WORKSPACE, "split_out holds %zu bytes, needs %zu", split_bytes,
                    afq_field_shift_lowp_bytes(n_walkers, nchol, sections));
    const int Kt = (sections * nchol + 63) / 64 * 64;
    return launch_field_shift_mixed(n_walkers, nchol, n_walkers, sqrt_dt, fields, force_bias_half, nchol,
                                    (const double2*)mf_shifts, (__nv_bfloat16*)split_out, nchol, Kt, sections,
                                    (double2*)shift_term, (double2*)fb_term, as_stream(stream));
}

int afq_weight_update(const afq_dims* d, const afq_params* p, const afq_problem* pb, const double* shift_term,
                      const double* fb_term, const double* overlaps_new, const afq_state* st, void* stream) {
    AFQ_TRY(check_dims(d, false));
    AFQ_TRY(check_params(p));
    if (!pb) return fail(AFQ_E_INVALID_ARGUMENT, "problem is NULL");
    AFQ_TRY(check_state(st));
    AFQ_NOTNULL(shift_term); AFQ_NOTNULL(fb_term); AFQ_NOTNULL(overlaps_new);
    return launch_weight_update(d->n_walkers, p, pb->sqrt_dt, pb->dt, make_double2(pb->h0_prop_re, pb->h0_prop_im),
                                (const double2*)shift_term, (const double2*)fb_term, (const double2*)overlaps_new,
                                st->weights, (double2*)st->overlaps, st->pop_control_ene_shift, st->e_estimate,
                                as_stream(stream));
}

int afq_block_measure(int32_t n_walkers, double dt, double shift_ema, const double* weights, const double* energy,
                      const double* e_estimate, double* pop_control_ene_shift, double* block_energy,
                      double* block_weight, void* stream) {
    if (n_walkers < 1) return fail(AFQ_E_INVALID_ARGUMENT, "n_walkers=%d < 1", n_walkers);
    if (!(dt > 0.0)) return fail(AFQ_E_INVALID_ARGUMENT, "dt=%g must be > 0", dt);
    AFQ_NOTNULL(weights); AFQ_NOTNULL(energy); AFQ_NOTNULL(e_estimate); AFQ_NOTNULL(pop_control_ene_shift);
    AFQ_NOTNULL(block_energy); AFQ_NOTNULL(block_weight);
    return launch_block_measure(n_walkers, dt, shift_ema, weights, (const double2*)energy, e_estimate,
                                pop_control_ene_shift, block_energy, block_weight, as_stream(stream));
}

// ----------------------------------------------------------- step / block
size_t afq_step_workspace(const afq_dims* d, int32_t n_chunks) {
    if (check_dims(d) != AFQ_OK) return 0;
    Arena a;
    layout_step(a, d, n_chunks);
    return a.used;
}

int afq_step(const afq_problem* pb, const afq_params* p, const afq_state* st, const double* fields, uint64_t seed,
             uint64_t counter, void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_problem(pb));
    AFQ_TRY(check_params(p));
    AFQ_TRY(check_state(st));
    AFQ_NOTNULL(workspace);
    Arena a(workspace, workspace_bytes);
    StepWS ws = layout_step(a, &pb->dims, p->n_chunks);
    AFQ_TRY(check_ws(a, workspace_bytes));
    return step_impl(pb, p, st, fields, seed, counter, ws, as_stream(stream));
}

size_t afq_block_workspace(const afq_dims* d, int32_t n_chunks) {
    if (check_dims(d) != AFQ_OK) return 0;
    Arena a;
    layout_block(a, d, n_chunks);
    return a.used;
}

int afq_block(const afq_problem* pb, const afq_params* p, const afq_state* st, const double* fields, double zeta,
              uint64_t seed, uint64_t counter, double* block_energy, double* block_weight, int32_t* sr_idx,
              void* workspace, size_t workspace_bytes, void* stream) {
    return afq_block_cv(pb, p, st, fields, zeta, seed, counter, block_energy, block_weight, sr_idx, nullptr,
                        workspace, workspace_bytes, stream);
}

int afq_block_cv(const afq_problem* pb, const afq_params* p, const afq_state* st, const double* fields, double zeta,
                 uint64_t seed, uint64_t counter, double* block_energy, double* block_weight, int32_t* sr_idx,
                 const afq_cv* cv, void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_problem(pb));
    AFQ_TRY(check_params(p));
    AFQ_TRY(check_state(st));
    AFQ_NOTNULL(block_energy); AFQ_NOTNULL(block_weight); AFQ_NOTNULL(workspace);
    const afq_dims* d = &pb->dims;
    const int cvmode = cv ? cv->mode : AFQ_CV_OFF;
    if (cvmode != AFQ_CV_OFF) {
        if (cvmode != AFQ_CV_RECORD && cvmode != AFQ_CV_ESTIMATE)
            return fail(AFQ_E_INVALID_ARGUMENT, "cv mode %d", cvmode);
        if (!is_mixed(d->precision)) return fail(AFQ_E_UNSUPPORTED, "the control variate needs a mixed precision");
        if (cvmode == AFQ_CV_RECORD) { AFQ_NOTNULL(cv->rec_features); AFQ_NOTNULL(cv->rec_exchange); }
        if (cvmode == AFQ_CV_ESTIMATE) {
            AFQ_NOTNULL(cv->net); AFQ_NOTNULL(cv->feat_shift); AFQ_NOTNULL(cv->feat_scale);
            if (cv->n_sample < 1) return fail(AFQ_E_INVALID_ARGUMENT, "cv n_sample=%d < 1", cv->n_sample);
            if (!mlp_shape_supported(AFQ_CV_FEATURES, cv->hidden))
                return fail(AFQ_E_INVALID_ARGUMENT, "cv hidden=%d (multiple of 32, <= 256)", cv->hidden);
        }
    }
    Arena a(workspace, workspace_bytes);
    BlockWS ws = layout_block(a, d, p->n_chunks);
    AFQ_TRY(check_ws(a, workspace_bytes));
    cudaStream_t s = as_stream(stream);
    const int W = d->n_walkers, n = d->norb, o = d->nocc, G = d->nchol;
    const size_t fstride = (size_t)W * G;
    // the block-end measurement reads the fp32 Green's function that the last
    // step's overlap pass writes (the QR leaves it unchanged): the three-section
    // form's energy, and either mixed form's control-variate measurement
    const bool green_kept = is_mixed(d->precision) && p->n_prop_steps > 0 &&
                            (cvmode != AFQ_CV_OFF || d->precision == AFQ_PREC_MIXED_FAST);
    // prop/blocks.py:38-51
    for (int st_i = 0; st_i < p->n_prop_steps; ++st_i) {
        // from the second step on, the previous overlap kernel left the force-bias operand
        const bool last = st_i + 1 == p->n_prop_steps;
        AFQ_TRY(step_impl(pb, p, st, fields ? fields + st_i * fstride : nullptr, seed, counter + st_i, ws.step, s,
                          st_i > 0, green_kept && last ? ws.green : nullptr));
        if (p->qr_every > 0 && (st_i + 1) % p->qr_every == 0 && st_i + 1 < p->n_prop_steps)
            AFQ_TRY(orthonormalize_refresh(pb, st, s, &ws.step, nullptr, nullptr, ws.step.ovl_new));
    }
    // prop/blocks.py:53-57, with the energy's Green's function from the same pass
    if (is_mixed(d->precision))
        AFQ_TRY(launch_split_c(n * o, (const double2*)pb->mo_coeff, ws.step.csplit, s));
    if (cvmode == AFQ_CV_OFF) {
        AFQ_TRY(orthonormalize_refresh(pb, st, s, nullptr, ws.green,
                                       is_mixed(d->precision) ? ws.step.csplit : nullptr, ws.step.ovl_new,
                                       green_kept, &ws.step));
        // prop/blocks.py:59-79
        AFQ_TRY(energy_impl(pb, st, ws, s, true));
        AFQ_PHASE("block_measure", s);
        AFQ_TRY(launch_block_measure(W, p->dt, p->shift_ema, st->weights, ws.energy, st->e_estimate,
                                     st->pop_control_ene_shift, block_energy, block_weight, s));
    } else {
        const LowpDims L = lowp_dims(d);
        Arena la((void*)pb->lowp, (size_t)-1);
        const LowpBufs lb = layout_lowp(la, d);
        double2* walk = (double2*)st->walkers;
        if (green_kept) {  // the Green's function and its force-bias operand are the last step's
            AFQ_TRY(orthonormalize_refresh(pb, st, s, &ws.step, nullptr, nullptr, ws.step.ovl_new));
        } else {
            { AFQ_PHASE("qr", s); AFQ_TRY(launch_cholqr2(W, n, o, walk, walk, nullptr, s)); }
            // overlaps, the Green's function and its force-bias operand in one pass; the GEMM gives c_g
            { AFQ_PHASE("green", s);
              AFQ_TRY(overlap_mixed(pb, walk, (double2*)st->overlaps, fb_split(d, ws.step), ws.green, ws.step, s)); }
        }
        { AFQ_PHASE("fb_gemm", s);
          AFQ_TRY(launch_tc_gemm_tn_drain(2 * W, G, L.Kt_F, ws.step.Ag, L.Kt_F, lb.Bf, L.Kt_F, ws.step.fbm, G,
                                          ws.step.status, s)); }
        const bool est = cvmode == AFQ_CV_ESTIMATE;
        { AFQ_PHASE("cv_features", s);
          AFQ_TRY(launch_cv_features(W, n, o, G, pb->h0, ws.green, (const double2*)pb->rot_h1, ws.step.fbm, G,
                                     (const double2*)st->overlaps, est ? cv->feat_shift : nullptr,
                                     est ? cv->feat_scale : nullptr, est ? ws.cv_feat : cv->rec_features,
                                     ws.cv_ebase, s)); }
        if (!est) {  // exact measurement, and the training data
            AFQ_TRY(energy_impl(pb, st, ws, s, true));
            AFQ_TRY(launch_cv_record(W, exch_chunks(d), (const double2*)ws.partial, cv->rec_exchange, s));
            AFQ_PHASE("block_measure", s);
            AFQ_TRY(launch_block_measure(W, p->dt, p->shift_ema, st->weights, ws.energy, st->e_estimate,
                                         st->pop_control_ene_shift, block_energy, block_weight, s));
        } else {
            { AFQ_PHASE("cv_network", s);
              AFQ_TRY(launch_mlp_forward(W, AFQ_CV_FEATURES, cv->hidden, (const __nv_bfloat16*)cv->net, ws.cv_feat,
                                         ws.cv_y, s)); }
            const int stride = cv->n_sample >= W ? 1 : W / cv->n_sample;
            const int m_max = (W + stride - 1) / stride;
            // the sample's offset: its own Philox stream (seed offset by a constant), this block's counter
            AFQ_TRY(launch_philox(1, seed ^ 0x9E3779B97F4A7C15ull, counter + p->n_prop_steps, 0, ws.cv_u, s));
            AFQ_TRY(launch_cv_pick(ws.cv_u, stride, ws.cv_off, s));
            const int We = energy_chunk(d), nch = exch_chunks(d);
            AFQ_PHASE("energy", s);
            for (int s0 = 0; s0 < m_max; s0 += We) {
                const int sc = m_max - s0 < We ? m_max - s0 : We;
                AFQ_TRY(launch_cv_green_rows(sc, s0, ws.cv_off, stride, W, n, o, L.Pe, ws.green, ws.Bg, L.S_E,
                                             L.Kt_E, L.sec, s));
                if (L.xf) {
                    AFQ_TRY(launch_tc_gemm_exchange(sc, G, L.Kt_E, ws.Bg, L.Kt_E, lb.Le, L.Kt_E, ws.xsum, ws.ctr,
                                                    ws.step.status, s, L.kd));
                    AFQ_TRY(launch_exchange_finish(sc, G, ws.xsum, ws.ctr,
                                                   (double2*)ws.partial + (size_t)s0 * nch * 2, s));
                    continue;
                }
                AFQ_TRY(launch_tc_gemm_tn_drain(2 * o * sc, G * o, L.Kt_E, ws.Bg, L.Kt_E, lb.Le, L.Kt_E, ws.F,
                                                (long long)G * o, ws.step.status, s));
                AFQ_TRY(launch_exchange_reduce(sc, G, o, ws.F, (long long)G * o,
                                               (double2*)ws.partial + (size_t)s0 * nch * 2, s));
            }
            AFQ_TRY(launch_cv_measure(W, p->dt, p->shift_ema, st->weights, ws.cv_ebase, ws.cv_y, cv->y_shift,
                                      cv->y_scale, m_max, stride, ws.cv_off, nch, (const double2*)ws.partial,
                                      st->e_estimate, st->pop_control_ene_shift, block_energy, block_weight,
                                      ws.energy, cv->stats, s));
        }
    }
    AFQ_PHASE("comb", s);
    // prop/blocks.py:81-92
    if (zeta < 0.0) {
        AFQ_TRY(launch_philox(1, seed, counter + p->n_prop_steps, 0, ws.zeta, s));
        AFQ_TRY(launch_sr_scan_dev(W, st->weights, ws.zeta, ws.levels, ws.idx, ws.avg, s));
    } else {
        AFQ_TRY(launch_sr_scan(W, st->weights, zeta, ws.levels, ws.idx, nullptr, ws.avg, s));
    }
    AFQ_CUDA(cudaMemcpyAsync(ws.wcopy, st->walkers, sizeof(double2) * (size_t)W * n * o, cudaMemcpyDeviceToDevice, s));
    AFQ_CUDA(cudaMemcpyAsync(ws.ocopy, st->overlaps, sizeof(double2) * (size_t)W, cudaMemcpyDeviceToDevice, s));
    AFQ_TRY(launch_gather(W, (int64_t)n * o, ws.idx, ws.wcopy, (double2*)st->walkers, ws.avg, st->weights, s));
    // overlaps of the copied walkers: a copy of the source walker's overlap is
    // bit-identical to recomputing det(C^H W)^2 on the copied data
    AFQ_TRY(launch_gather(W, 1, ws.idx, ws.ocopy, (double2*)st->overlaps, ws.avg, nullptr, s));
    if (sr_idx) AFQ_CUDA(cudaMemcpyAsync(sr_idx, ws.idx, sizeof(int32_t) * W, cudaMemcpyDeviceToDevice, s));
    return AFQ_OK;
}

// -------------------------------------------------------- taped block
}  // extern "C"

namespace afq {

int block_op_count(const afq_params* p) {
    int q = 0;
    if (p->qr_every > 0)
        for (int s = 0; s + 1 < p->n_prop_steps; ++s)
            if ((s + 1) % p->qr_every == 0) ++q;
    return p->n_prop_steps + q + 2;
}

size_t block_ws_bytes(const afq_dims* d, int n_chunks) { return afq_block_workspace(d, n_chunks); }

static int snap_state(const afq_dims* d, const afq_state* st, const BlockSnap* snap, int k, cudaStream_t s) {
    if (!snap) return AFQ_OK;
    const size_t W = d->n_walkers, no = (size_t)d->norb * d->nocc;
    AFQ_CUDA(cudaMemcpyAsync(snap->walkers + k * W * no, st->walkers, sizeof(double2) * W * no,
                             cudaMemcpyDeviceToDevice, s));
    AFQ_CUDA(cudaMemcpyAsync(snap->weights + k * W, st->weights, sizeof(double) * W, cudaMemcpyDeviceToDevice, s));
    AFQ_CUDA(cudaMemcpyAsync(snap->overlaps + k * W, st->overlaps, sizeof(double2) * W, cudaMemcpyDeviceToDevice,
                             s));
    AFQ_CUDA(cudaMemcpyAsync(snap->pop + k, st->pop_control_ene_shift, sizeof(double), cudaMemcpyDeviceToDevice, s));
    return AFQ_OK;
}

// The binary64 path of afq_block (fields and comb uniform from the Philox
// stream), with each operation's input state copied to snap.
int run_block_taped(const afq_problem* pb, const afq_params* p, const afq_state* st, uint64_t seed, uint64_t counter,
                    const int32_t* forced_idx, int32_t* idx_out, double* block_energy, double* block_weight,
                    const BlockSnap* snap, void* workspace, size_t workspace_bytes, cudaStream_t s) {
    const afq_dims* d = &pb->dims;
    if (is_mixed(d->precision)) return fail(AFQ_E_UNSUPPORTED, "the taped block runs the binary64 form");
    Arena a(workspace, workspace_bytes);
    BlockWS ws = layout_block(a, d, p->n_chunks);
    AFQ_TRY(check_ws(a, workspace_bytes));
    const int W = d->n_walkers, n = d->norb, o = d->nocc;
    int op = 0;
    for (int st_i = 0; st_i < p->n_prop_steps; ++st_i) {
        AFQ_TRY(snap_state(d, st, snap, op++, s));
        AFQ_TRY(step_impl(pb, p, st, nullptr, seed, counter + st_i, ws.step, s));
        if (snap && snap->V && chunk_size(W, p->n_chunks) == W)
            AFQ_CUDA(cudaMemcpyAsync(snap->V + (size_t)st_i * W * n * n, ws.step.V, sizeof(double2) * (size_t)W * n * n,
                                     cudaMemcpyDeviceToDevice, s));
        if (p->qr_every > 0 && (st_i + 1) % p->qr_every == 0 && st_i + 1 < p->n_prop_steps) {
            AFQ_TRY(snap_state(d, st, snap, op++, s));
            AFQ_TRY(orthonormalize_refresh(pb, st, s, &ws.step));
        }
    }
    AFQ_TRY(snap_state(d, st, snap, op++, s));
    AFQ_TRY(orthonormalize_refresh(pb, st, s, nullptr, ws.green, nullptr));
    AFQ_TRY(snap_state(d, st, snap, op++, s));
    AFQ_TRY(energy_impl(pb, st, ws, s, true));
    if (snap)
        AFQ_CUDA(cudaMemcpyAsync(snap->energy, ws.energy, sizeof(double2) * W, cudaMemcpyDeviceToDevice, s));
    AFQ_TRY(launch_block_measure(W, p->dt, p->shift_ema, st->weights, ws.energy, st->e_estimate,
                                 st->pop_control_ene_shift, block_energy, block_weight, s));
    AFQ_TRY(launch_philox(1, seed, counter + p->n_prop_steps, 0, ws.zeta, s));
    AFQ_TRY(launch_sr_scan_dev(W, st->weights, ws.zeta, ws.levels, ws.idx, ws.avg, s));
    if (forced_idx)
        AFQ_CUDA(cudaMemcpyAsync(ws.idx, forced_idx, sizeof(int32_t) * W, cudaMemcpyDeviceToDevice, s));
    AFQ_CUDA(cudaMemcpyAsync(ws.wcopy, st->walkers, sizeof(double2) * (size_t)W * n * o, cudaMemcpyDeviceToDevice, s));
    AFQ_CUDA(cudaMemcpyAsync(ws.ocopy, st->overlaps, sizeof(double2) * (size_t)W, cudaMemcpyDeviceToDevice, s));
    AFQ_TRY(launch_gather(W, (int64_t)n * o, ws.idx, ws.wcopy, (double2*)st->walkers, ws.avg, st->weights, s));
    AFQ_TRY(launch_gather(W, 1, ws.idx, ws.ocopy, (double2*)st->overlaps, ws.avg, nullptr, s));
    if (idx_out) AFQ_CUDA(cudaMemcpyAsync(idx_out, ws.idx, sizeof(int32_t) * W, cudaMemcpyDeviceToDevice, s));
    return AFQ_OK;
}

}  // namespace afq

extern "C" {

// ------------------------------------------------------------- block loop
size_t afq_run_blocks_workspace(const afq_dims* d, int32_t n_chunks) {
    const size_t b = afq_block_workspace(d, n_chunks);
    return b ? round_up(b, 256) + 256 : 0;
}

int afq_run_blocks(const afq_problem* pb, const afq_params* p, const afq_state* st, int32_t n_blocks, uint64_t seed,
                   uint64_t* counter_dev, double* energies, double* weights, void* workspace,
                   size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_problem(pb));
    AFQ_TRY(check_params(p));
    AFQ_TRY(check_state(st));
    AFQ_NOTNULL(counter_dev); AFQ_NOTNULL(energies); AFQ_NOTNULL(weights); AFQ_NOTNULL(workspace);
    if (n_blocks < 0) return fail(AFQ_E_INVALID_ARGUMENT, "n_blocks=%d < 0", n_blocks);
    const size_t need = afq_run_blocks_workspace(&pb->dims, p->n_chunks);
    if (!need || workspace_bytes < need)
        return fail(AFQ_E_WORKSPACE, "run workspace %zu < %zu bytes", workspace_bytes, need);
    const size_t bws = round_up(afq_block_workspace(&pb->dims, p->n_chunks), 256);
    double* slot = (double*)((char*)workspace + bws);  // e, w
    int* idx = (int*)(slot + 2);
    cudaStream_t s = as_stream(stream);
    if (n_blocks == 0) return AFQ_OK;
    const uint64_t inc = (uint64_t)p->n_prop_steps + 1;
    struct Base {  // the device counter for this thread's launches, reset on every exit
        Base(const uint64_t* c) { t_counter_base = c; }
        ~Base() { t_counter_base = nullptr; }
    } base(counter_dev);
    AFQ_CUDA(cudaMemsetAsync(idx, 0, sizeof(int), s));
    auto one = [&](cudaStream_t q) -> int {
        AFQ_TRY(afq_block_cv(pb, p, st, nullptr, -1.0, seed, 0, slot, slot + 1, nullptr, nullptr, workspace, bws,
                             q));
        return launch_run_record(slot, slot + 1, energies, weights, idx, counter_dev, inc, q);
    };
    // the first block runs as is (it also performs every one-time setup)
    AFQ_TRY(one(s));
    if (n_blocks == 1) return AFQ_OK;
    if (timing_enabled()) {  // per-phase events do not belong in a graph: plain launches
        for (int b = 1; b < n_blocks; ++b) AFQ_TRY(one(s));
        return AFQ_OK;
    }
    // the remaining blocks: one block captured into a CUDA graph, replayed
    cudaStream_t cs = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int rc = AFQ_OK;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev0, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev1, cudaEventDisableTiming) != cudaSuccess)
        rc = fail(AFQ_E_CUDA, "run_blocks: stream / event creation failed");
    if (rc == AFQ_OK && (cudaEventRecord(ev0, s) != cudaSuccess || cudaStreamWaitEvent(cs, ev0, 0) != cudaSuccess))
        rc = fail(AFQ_E_CUDA, "run_blocks: stream ordering failed");
    if (rc == AFQ_OK) {
        if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            rc = fail(AFQ_E_CUDA, "run_blocks: stream capture failed to start");
        } else {
            const int brc = one(cs);
            const cudaError_t ec = cudaStreamEndCapture(cs, &graph);
            if (brc != AFQ_OK) rc = brc;
            else if (ec != cudaSuccess || !graph) rc = fail(AFQ_E_CUDA, "run_blocks: capture failed (%s)", cudaGetErrorString(ec));
        }
    }
    if (rc == AFQ_OK && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
        rc = fail(AFQ_E_CUDA, "run_blocks: graph instantiation failed");
    for (int b = 1; rc == AFQ_OK && b < n_blocks; ++b)
        if (cudaGraphLaunch(exec, cs) != cudaSuccess) rc = fail(AFQ_E_CUDA, "run_blocks: graph launch failed");
    if (cs && ev1 && (cudaEventRecord(ev1, cs) != cudaSuccess || cudaStreamWaitEvent(s, ev1, 0) != cudaSuccess) &&
        rc == AFQ_OK)
        rc = fail(AFQ_E_CUDA, "run_blocks: stream ordering failed");
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (cs) cudaStreamDestroy(cs);  // destroyed once its work completes
    return rc;
}

// ---------------------------------------------------------------- network
size_t afq_mlp_param_count(int32_t n_features, int32_t hidden) {
    if (!mlp_shape_supported(n_features, hidden)) return 0;
    return mlp_param_count(n_features, hidden);
}

int afq_mlp_forward(int32_t batch, int32_t n_features, int32_t hidden, const void* params_bf16, const float* x,
                    float* y, void* stream) {
    if (!afq_mlp_param_count(n_features, hidden)) return fail(AFQ_E_INVALID_ARGUMENT, "mlp: F=%d H=%d", n_features, hidden);
    if (batch < 0) return fail(AFQ_E_INVALID_ARGUMENT, "mlp: batch %d < 0", batch);
    AFQ_NOTNULL(params_bf16); AFQ_NOTNULL(x); AFQ_NOTNULL(y);
    return launch_mlp_forward(batch, n_features, hidden, (const __nv_bfloat16*)params_bf16, x, y, as_stream(stream));
}

size_t afq_mlp_train_workspace(int32_t batch, int32_t n_features, int32_t hidden) {
    if (!afq_mlp_param_count(n_features, hidden) || batch < 1) return 0;
    return mlp_train_ws_floats(batch, n_features, hidden) * sizeof(float);
}

static int mlp_train_args(int32_t batch, int32_t n_features, int32_t hidden, const float* x, const float* target,
                          size_t workspace_bytes) {
    const size_t need = afq_mlp_train_workspace(batch, n_features, hidden);
    if (!need) return fail(AFQ_E_INVALID_ARGUMENT, "mlp: batch=%d F=%d H=%d", batch, n_features, hidden);
    if (workspace_bytes < need) return fail(AFQ_E_WORKSPACE, "mlp workspace %zu < %zu bytes", workspace_bytes, need);
    AFQ_NOTNULL(x); AFQ_NOTNULL(target);
    return AFQ_OK;
}

int afq_mlp_gradient(int32_t batch, int32_t n_features, int32_t hidden, const void* params_bf16, const float* x,
                     const float* target, float* grad, float* loss_out, void* workspace, size_t workspace_bytes,
                     void* stream) {
    AFQ_TRY(mlp_train_args(batch, n_features, hidden, x, target, workspace_bytes));
    AFQ_NOTNULL(params_bf16); AFQ_NOTNULL(grad); AFQ_NOTNULL(workspace);
    return launch_mlp_grad_adam(batch, n_features, hidden, (const __nv_bfloat16*)params_bf16, x, target,
                                (float*)workspace, grad, loss_out, nullptr, nullptr, nullptr, nullptr, 0.f, 1,
                                as_stream(stream));
}

int afq_mlp_train_step(int32_t batch, int32_t n_features, int32_t hidden, float* master, void* params_bf16,
                       float* adam_m, float* adam_v, const float* x, const float* target, float lr, int32_t step,
                       void* workspace, size_t workspace_bytes, float* loss_out, void* stream) {
    AFQ_TRY(mlp_train_args(batch, n_features, hidden, x, target, workspace_bytes));
    AFQ_NOTNULL(master); AFQ_NOTNULL(params_bf16); AFQ_NOTNULL(adam_m); AFQ_NOTNULL(adam_v); AFQ_NOTNULL(workspace);
    if (step < 1) return fail(AFQ_E_INVALID_ARGUMENT, "mlp: step %d < 1", step);
    return launch_mlp_grad_adam(batch, n_features, hidden, (const __nv_bfloat16*)params_bf16, x, target,
                                (float*)workspace, nullptr, loss_out, master, (__nv_bfloat16*)params_bf16, adam_m,
                                adam_v, lr, step, as_stream(stream));
}

int afq_mlp_sync(int32_t n_features, int32_t hidden, const float* master, void* params_bf16, void* stream) {
    const size_t P = afq_mlp_param_count(n_features, hidden);
    if (!P) return fail(AFQ_E_INVALID_ARGUMENT, "mlp: F=%d H=%d", n_features, hidden);
    AFQ_NOTNULL(master); AFQ_NOTNULL(params_bf16);
    return launch_mlp_sync_bf16(P, master, (__nv_bfloat16*)params_bf16, as_stream(stream));
}

}  // extern "C"
