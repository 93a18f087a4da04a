/*
 * afqmc_gb300.h -- C ABI of the GB300 phaseless-AFQMC step engine.
 *
 * Restricted walkers, RHF trial, Cholesky-factorised Hamiltonian.  Every
 * entry point replaces one call of the reference package
 * (ad_afqmc_prototype, a JAX program; citations are file:line inside that
 * project).  The reference has no native FFI of its own: its plug points are
 * Python callables (core/ops.py:11-90, prop/chol_afqmc_ops.py:45-50,
 * driver.py:39-47 block_fn), so these functions are what a ctypes / cffi /
 * torch-extension binding of that Python surface calls.
 *
 * Conventions
 *  - All array arguments are DEVICE pointers owned by the caller, C-contiguous.
 *    "complex" arrays are interleaved complex128 (re, im) passed as double*.
 *  - Walkers are (n_walkers, norb, nocc) complex128, as in walkers.py:64-68.
 *  - Every call is asynchronous on `stream` (a cudaStream_t passed as void*;
 *    NULL = legacy default stream) except the ones documented as set-up.
 *  - Hot calls allocate nothing: scratch comes from `workspace`, whose size
 *    the matching afq_*_workspace() query returns.  Too small -> AFQ_E_WORKSPACE.
 *  - Return 0 on success or a negative AFQ_E_* code; no call aborts, traps or
 *    throws across the ABI.  afq_last_error() gives a thread-local message.
 *  - Numerical trouble (zero overlap, overflowing importance weight) is
 *    absorbed the way the reference absorbs it (weights set to zero,
 *    prop/afqmc.py:127-134), not reported as an error.
 */
#ifndef AFQMC_GB300_H
#define AFQMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AFQ_ABI_VERSION 2

#define AFQ_OK 0
#define AFQ_E_INVALID_ARGUMENT (-1) /* bad shape, null pointer, bad value */
#define AFQ_E_UNSUPPORTED (-2)      /* size outside what the kernels handle */
#define AFQ_E_CUDA (-3)             /* a CUDA runtime call failed */
#define AFQ_E_WORKSPACE (-4)        /* workspace smaller than the query says */
#define AFQ_E_DEVICE_CHECK (-5)     /* a device-side bounded wait or check failed */

#define AFQ_PREC_FP64 0  /* every product in binary64 */
#define AFQ_PREC_MIXED 1 /* tensor-core / FP32 products, FP64 overlaps, QR, weights */
#define AFQ_PREC_MIXED_FAST 2 /* as MIXED with two-piece bf16 operands (~2^-17 products): half the GEMM work */

/* Sizes of one batch.  trial_is_real selects the real-trial fast path:
 * mo_coeff is still passed as complex128 but its imaginary parts must be 0,
 * and rot_chol is then real (G, o, n) float64 instead of complex. */
typedef struct afq_dims {
    int32_t n_walkers;
    int32_t norb;
    int32_t nocc;
    int32_t nchol;
    int32_t trial_is_real;
    int32_t precision; /* AFQ_PREC_* */
} afq_dims;

/* afqmc_params (prop/types.py:19-32) plus the in-block QR cadence. */
typedef struct afq_params {
    double dt;
    double pop_control_damping;
    double weight_floor;
    double weight_cap;
    double shift_ema;
    int32_t n_exp_terms;
    int32_t n_prop_steps;
    int32_t qr_every;  /* 0: orthonormalise only at block end (prop/blocks.py:53) */
    int32_t n_chunks;  /* walker chunks for the V workspace (walkers.py:94-166) */
} afq_params;

/* Hamiltonian, trial and the two contexts, all device pointers.
 * prop ctx = chol_afqmc_ctx (prop/chol_afqmc_ops.py:15-42),
 * meas ctx = rhf_meas_ctx (meas/rhf.py:133-138). */
typedef struct afq_problem {
    afq_dims dims;
    double h0;
    const double* chol;        /* (G, n, n) float64 */
    const double* mo_coeff;    /* (n, o) complex128 */
    double dt;
    double sqrt_dt;
    const double* exp_h1_half; /* (n, n) float64 */
    const double* mf_shifts;   /* (G,) complex128 */
    double h0_prop_re;
    double h0_prop_im;
    const double* rot_h1;      /* (o, n) complex128 */
    const double* rot_chol;    /* (G, o, n) float64 or complex128 */
    const void* lowp;          /* afq_prepare_lowp() output; NULL for FP64 */
} afq_problem;

/* prop_state (prop/types.py:10-16) without the rng key; device pointers. */
typedef struct afq_state {
    double* walkers;               /* (W, n, o) complex128 */
    double* weights;               /* (W,) float64 */
    double* overlaps;              /* (W,) complex128 */
    double* pop_control_ene_shift; /* (1,) float64 */
    double* e_estimate;            /* (1,) float64 */
} afq_state;

int afq_abi_version(void);
const char* afq_status_string(int status);
const char* afq_last_error(void);

/* ---- set-up (synchronises `stream`; allocates nothing) ------------------ */

/* _build_prop_ctx, prop/chol_afqmc_ops.py:77-103 (+ _mf_shifts :59-63,
 * _build_exp_h1_half_from_h1 :66-67).  rdm1 is complex (2, n, n) when
 * rdm1_spin_blocks = 1 (summed as at :53-56) or a total (n, n) when 0.
 * Outputs: exp_h1_half (n,n) f64, mf_shifts (G,) c128, h0_prop (1,) c128. */
size_t afq_build_prop_ctx_workspace(int32_t norb, int32_t nchol);
int afq_build_prop_ctx(int32_t norb, int32_t nchol, double h0, double dt,
                       const double* h1, const double* chol, const double* rdm1,
                       int32_t rdm1_spin_blocks, double* exp_h1_half, double* mf_shifts,
                       double* h0_prop, void* workspace, size_t workspace_bytes,
                       void* stream);

/* get_rdm1, trial/rhf.py:29-32: rdm1 (2, n, n) c128 = [C C^H, C C^H] of the
 * trial orbitals mo_coeff (n, o) c128. */
int afq_trial_rdm1(int32_t norb, int32_t nocc, const double* mo_coeff, double* rdm1, void* stream);

/* build_meas_ctx, meas/rhf.py:141-150.  rot_h1 (o,n) c128; rot_chol (G,o,n)
 * f64 when trial_is_real else c128. */
int afq_build_meas_ctx(int32_t norb, int32_t nocc, int32_t nchol, const double* h1,
                       const double* chol, const double* mo_coeff, int32_t trial_is_real,
                       double* rot_h1, double* rot_chol, void* stream);

/* Low-precision copies of chol / rot_chol for AFQ_PREC_MIXED / MIXED_FAST
 * (bf16 splits in six or three K sections, tensor-core operand order; the
 * layout depends on d->precision).  `out` must hold afq_lowp_bytes(). */
size_t afq_lowp_bytes(const afq_dims* d);
int afq_prepare_lowp(const afq_dims* d, const double* chol, const double* rot_chol,
                     void* out, size_t out_bytes, void* stream);

/* The tensor-core GEMM under the mixed-precision V-build and force bias
 * (prop/chol_afqmc_ops.py:70-74, meas/rhf.py:33): C (M x N, fp32, row stride
 * ldc) = A (M x K) . B (N x K)^T with bf16 A and B, row-major, K contiguous,
 * K a multiple of 64, lda / ldb multiples of 8, 16-byte aligned bases.
 * `err` (device int32, required) is set to 1 if a bounded pipeline wait
 * expired (the kernel then stops early instead of hanging).
 * accumulate: 0 = fp32 accumulation inside the tensor cores (truncating:
 * a sum of K positive terms drifts low by ~K/16 * 2^-25 relative);
 * d >= 1 = every d 64-wide K blocks form a fresh tensor-core partial,
 * summed in fp32 registers with round-to-nearest adds (the mixed step
 * uses d = 1). */
int afq_lowp_gemm_tn(int32_t M, int32_t N, int32_t K, const void* A, int64_t lda, const void* B,
                     int64_t ldb, float* C, int64_t ldc, int32_t* err, int32_t accumulate,
                     void* stream);

/* Device status word of a step / block / gradient workspace: synchronises
 * `stream`, copies the word to *status (0 = fine, AFQ_STATUS_* otherwise)
 * and clears it (and the non-finite walker count).  Returns
 * AFQ_E_DEVICE_CHECK when the word was set.  The first condition raised
 * since the last clear is the one reported. */
#define AFQ_STATUS_WAIT_EXPIRED 1 /* a bounded device-side wait expired */
#define AFQ_STATUS_SINGULAR 2     /* adjoint: a singular overlap matrix or QR factor R */
#define AFQ_STATUS_BAD_INDEX 3    /* adjoint: comb indices out of range or not non-decreasing */
#define AFQ_STATUS_NONFINITE 4    /* a walker's new overlap or weight was NaN or infinite */
int afq_workspace_status(void* workspace, int32_t* status, void* stream);
/* As afq_workspace_status, and *nonfinite receives how many walker updates
 * produced a NaN or infinite overlap or weight since the last clear.  Such a
 * walker propagates as in the reference (prop/afqmc.py:116-138: its NaN
 * weight passes the floor and cap and turns the mean weight NaN); the count
 * only reports it. */
int afq_workspace_counters(void* workspace, int32_t* status, int32_t* nonfinite, void* stream);

/* Bounded-wait self-test (no counterpart in the reference): one thread waits
 * on a fresh mbarrier with the same bounded wait the tensor-core pipelines
 * use, for at most limit_ns nanoseconds of the GPU's global timer.  With
 * arrive = 0 nothing ever arrives, the wait expires and *status (device
 * int32) is set to AFQ_STATUS_WAIT_EXPIRED; with arrive = 1 the thread
 * arrives first and *status is set to 0.  limit_ns must be in (0, 10 s]. */
int afq_selftest_wait(int64_t limit_ns, int32_t arrive, int32_t* status, void* stream);

/* ---- per-walker kernels, batched over walkers --------------------------- */

/* overlap_r: det(C^H W)^2.  meas/rhf.py:22-24 = trial/rhf.py:35-37. */
int afq_overlap(const afq_dims* d, const double* mo_coeff, const double* walkers,
                double* overlaps, void* stream);

/* _half_green_from_overlap_matrix: G_half = solve((C^H W)^T, W^T), (W,o,n)
 * c128 (meas/rhf.py:15-19).  `overlaps` (optional, may be NULL) receives
 * det(C^H W)^2 from the same factorisation. */
int afq_half_green(const afq_dims* d, const double* mo_coeff, const double* walkers,
                   double* green, double* overlaps, void* stream);

/* force_bias_kernel_r: 2 L~_flat vec(G_half), (W, G) c128 (meas/rhf.py:27-33). */
size_t afq_force_bias_workspace(const afq_dims* d);
int afq_force_bias(const afq_dims* d, const double* mo_coeff, const double* rot_chol,
                   const double* walkers, double* force_bias, void* workspace,
                   size_t workspace_bytes, void* stream);

/* energy_kernel_r: h0 + e1 + 2 sum_g c_g^2 - exc, (W,) c128 (meas/rhf.py:36-50). */
size_t afq_energy_workspace(const afq_dims* d);
int afq_energy(const afq_dims* d, double h0, const double* mo_coeff, const double* rot_h1,
               const double* rot_chol, const double* walkers, double* energy,
               void* workspace, size_t workspace_bytes, void* stream);

/* apply_trotter (restricted): E_half exp(i sqrt_dt V(x)) E_half W with a
 * n_terms Taylor series, V(x) = sum_g x_g L_g built from complex
 * shifted_fields (W, G).  prop/chol_afqmc_ops.py:173-183 (+ :70-74, :106-107,
 * :127-137, prop/utils.py:20-31).  walkers_out may equal walkers. */
size_t afq_apply_trotter_workspace(const afq_dims* d, int32_t n_chunks);
int afq_apply_trotter(const afq_dims* d, int32_t n_terms, double sqrt_dt, int32_t n_chunks,
                      const double* chol, const double* exp_h1_half, const double* walkers,
                      const double* shifted_fields, double* walkers_out, void* workspace,
                      size_t workspace_bytes, void* stream);

/* orthogonalize / orthonormalize (restricted): QR with diag(R) real >= 0
 * (walkers.py:169-211).  det_r (optional) receives prod diag(R) (W,) c128;
 * the restricted normalisation is det_r^2.  walkers_out may equal walkers.
 * d->precision FP64: Householder (as the reference's LAPACK QR); MIXED and
 * MIXED_FAST: CholeskyQR2, fp32 first Gram matrix, otherwise binary64 (the
 * same Q and R to ~cond(W) * 1e-16; the mixed block uses it). */
int afq_orthogonalize(const afq_dims* d, const double* walkers, double* walkers_out,
                      double* det_r, void* stream);

/* _sr_indices (walkers.py:233-240): comb indices (int32) and the inclusive
 * prefix sum of |w| (optional, may be NULL).  The prefix sum adds in the
 * association order of jax.lax.associative_scan (what jnp.cumsum lowers to):
 * an up-sweep of pairwise sums e'[k] = e[2k] + e[2k+1], recursively scanned,
 * then s[2k+1] = s'[k] and s[2k] = s'[k-1] + e[2k]; the search repeats
 * jnp.searchsorted's default probe sequence (ceil(log2(W+1)) halvings,
 * side='left').  Same inputs -> the same bits and indices as the reference. */
size_t afq_sr_workspace(int32_t n_walkers);
int afq_sr_indices(int32_t n_walkers, const double* weights, double zeta, int32_t* idx,
                   double* cumsum, void* workspace, size_t workspace_bytes, void* stream);

/* afq_sr_indices without a workspace.  No counterpart in the reference: it is
 * for callers that cannot give this library device memory -- a plug-in
 * inside a process whose runtime already reserved the GPU's memory for its own
 * pool (JAX does so by default), or a thin FFI binding with no device
 * allocator.  The scan's scratch is a file-scope device array of 1 MiB per GPU
 * (held until the process exits); at most 65536 walkers, larger calls return
 * AFQ_E_UNSUPPORTED.  All calls on a device share that array: calls that
 * overlap on the GPU race, so order them on one stream.  The first call on
 * each device looks the array up (cudaGetSymbolAddress) and should come
 * before any stream capture; the looked-up address is kept for the life of
 * the process, so do not call this again on a device after resetting it
 * (cudaDeviceReset).  Allocates nothing. */
int afq_sr_indices_static(int32_t n_walkers, const double* weights, double zeta, int32_t* idx,
                          double* cumsum, void* stream);

/* stochastic_reconfiguration (walkers.py:243-265): walkers_out[k] =
 * walkers[idx[k]], weights_out = sum|w| / W.  walkers_out must not alias
 * walkers.  idx (optional) receives the indices. */
int afq_stochastic_reconfiguration(const afq_dims* d, const double* weights, double zeta,
                                   const double* walkers, double* walkers_out,
                                   double* weights_out, int32_t* idx, void* workspace,
                                   size_t workspace_bytes, void* stream);

/* ---- the step pieces (prop/afqmc.py:86-138) ----------------------------- */

/* Philox4x32-10 (Salmon et al., SC'11) uniforms in [0, 1) with 53 random
 * bits, and normals by Box-Muller evaluated in fp32 from them (~1e-7
 * relative rounding); element i depends only on (seed, counter, i). */
int afq_fill_normal(int64_t count, uint64_t seed, uint64_t counter, double* out,
                    void* stream);
int afq_fill_uniform(int64_t count, uint64_t seed, uint64_t counter, double* out,
                     void* stream);

/* prop/afqmc.py:97-101: field shifts, shifted fields (W,G) c128 and the
 * per-walker shift_term, fb_term (W,) c128. */
int afq_field_shift(const afq_dims* d, double sqrt_dt, const double* fields,
                    const double* force_bias, const double* mf_shifts, double* shifted_fields,
                    double* shift_term, double* fb_term, void* stream);

/* The mixed forms' field shift (prop/afqmc.py:97-101, as afq_field_shift)
 * from the fp32 force bias the tensor-core GEMM gives: force_bias_half is
 * (2W, G) fp32, rows w = Re fb_w / 2 and W + w = Im fb_w / 2.  sections 6
 * (AFQ_PREC_MIXED) forms the shifts and the four weight sums in binary64;
 * sections 3 (AFQ_PREC_MIXED_FAST) forms them in fp32 (its operands carry 24
 * bits), sums each lane's terms in fp32 and the lanes in binary64.
 * shift_term, fb_term (W,) c128; split_out receives the shifted fields as
 * the V-build's bf16 split rows (afq_field_shift_lowp_bytes bytes). */
size_t afq_field_shift_lowp_bytes(int32_t n_walkers, int32_t nchol, int32_t sections);
int afq_field_shift_lowp(int32_t n_walkers, int32_t nchol, int32_t sections, double sqrt_dt,
                         const double* fields, const float* force_bias_half, const double* mf_shifts,
                         double* shift_term, double* fb_term, void* split_out, size_t split_bytes,
                         void* stream);

/* prop/afqmc.py:116-138: importance weights with the phaseless cut, floor and
 * cap, population-control shift.  Updates st->weights, st->overlaps (copied
 * from overlaps_new) and st->pop_control_ene_shift in place. */
int afq_weight_update(const afq_dims* d, const afq_params* p, const afq_problem* pb,
                      const double* shift_term, const double* fb_term,
                      const double* overlaps_new, const afq_state* st, void* stream);

/* prop/blocks.py:59-79: clip |Re E - e_est| > sqrt(2/dt) to e_est, weighted
 * block energy (w_sum == 0 -> e_est), shift <- (1-a) shift + a E_blk.
 * energy (W,) c128; block_energy, block_weight (1,) f64 outputs;
 * pop_control_ene_shift (1,) updated in place. */
int afq_block_measure(int32_t n_walkers, double dt, double shift_ema, const double* weights,
                      const double* energy, const double* e_estimate,
                      double* pop_control_ene_shift, double* block_energy, double* block_weight,
                      void* stream);

/* ---- fused step and block ------------------------------------------------ */

/* afqmc_step (prop/afqmc.py:74-147).  fields (W,G) f64 injected, or NULL to
 * draw them with afq_fill_normal(seed, counter). */
size_t afq_step_workspace(const afq_dims* d, int32_t n_chunks);
int afq_step(const afq_problem* pb, const afq_params* p, const afq_state* st,
             const double* fields, uint64_t seed, uint64_t counter, void* workspace,
             size_t workspace_bytes, void* stream);

/* afqmc_block (prop/blocks.py:22-95): n_prop_steps steps (with an extra
 * orthonormalisation after every qr_every-th step when qr_every > 0), QR,
 * mixed energy with clip, weighted block energy, shift EMA, comb
 * reconfiguration.  fields: (n_prop_steps, W, G) f64 or NULL (step s draws
 * with counter + s); zeta: the comb uniform, or a negative value to draw it
 * with afq_fill_uniform(seed, counter + n_prop_steps).  block_energy and
 * block_weight are device (1,) f64 outputs; sr_idx (optional) (W,) int32. */
size_t afq_block_workspace(const afq_dims* d, int32_t n_chunks);
int afq_block(const afq_problem* pb, const afq_params* p, const afq_state* st,
              const double* fields, double zeta, uint64_t seed, uint64_t counter,
              double* block_energy, double* block_weight, int32_t* sr_idx,
              void* workspace, size_t workspace_bytes, void* stream);

/* run_afqmc_energy's block loop (driver.py:22-38: a jitted scan of
 * block_fn over n_blocks) on the device: n_blocks afqmc_blocks with fields
 * and comb uniforms drawn from the Philox stream (seed, *counter_dev), the
 * device counter advancing by n_prop_steps + 1 per block, and block b's
 * energy and weight written to energies[b], weights[b] (device f64).  The
 * first block runs as is; the others replay a CUDA graph of one captured
 * block (plain launches while afq_timing is on).  The same stream as
 * afq_block with counter = *counter_dev gives the same results.
 * workspace: afq_run_blocks_workspace bytes. */
size_t afq_run_blocks_workspace(const afq_dims* d, int32_t n_chunks);
int afq_run_blocks(const afq_problem* pb, const afq_params* p, const afq_state* st, int32_t n_blocks,
                   uint64_t seed, uint64_t* counter_dev, double* energies, double* weights,
                   void* workspace, size_t workspace_bytes, void* stream);

/* ---- learned exchange control variate (no counterpart in the reference:
 * an engine form beside the plain measurement of prop/blocks.py:59-79) ----
 *
 * Per walker, features x (AFQ_CV_FEATURES floats) from the Coulomb vectors
 * c_g = tr(L~_g G_half^T) of the block-end Green's function: [0, 60) sums of
 * |c_g|^2 over 60 contiguous blocks of g, [60] Re sum_g c_g^2, [61] Im
 * sum_g c_g^2, [62] Re tr(rot_h1 G_half), [63] log|overlap|.  A network
 * (afq_mlp_*) predicts each walker's exchange energy X_w = sum_g tr(f_g f_g)
 * from them.  Modes of afq_block_cv:
 *   AFQ_CV_RECORD: the exact measurement, plus the raw features and the exact
 *     X_w of every walker (training data);
 *   AFQ_CV_ESTIMATE: X_w predicted for every walker, exact X_w for the walkers
 *     off + k * stride (stride = W / n_sample, off uniform in [0, stride) from
 *     the block's random stream), and the block energy
 *       sum_w w h(E_pred) + stride * sum_sampled w (h(E_exact) - h(E_pred))
 *     divided by sum_w w, h = the sqrt(2/dt) clip: unbiased for the exact
 *     block energy whatever the network predicts (every walker is sampled
 *     with probability 1 / stride).  Mixed precisions only. */
#define AFQ_CV_OFF 0
#define AFQ_CV_RECORD 1
#define AFQ_CV_ESTIMATE 2
#define AFQ_CV_FEATURES 64

typedef struct afq_cv {
    int32_t mode;            /* AFQ_CV_* */
    int32_t hidden;          /* network width (multiple of 32, <= 256) */
    int32_t n_sample;        /* ESTIMATE: walkers with exact exchange per block (>= 1) */
    int32_t pad_;
    const void* net;         /* ESTIMATE: bf16 parameters, afq_mlp_param_count entries */
    const float* feat_shift; /* ESTIMATE: network input = (x - shift) * scale, device (64,) */
    const float* feat_scale;
    double y_shift, y_scale; /* X_pred = y_shift + y_scale * network output */
    float* rec_features;     /* RECORD: device (W, 64) raw features */
    double* rec_exchange;    /* RECORD: device (W,) exact X_w */
    double* stats;           /* ESTIMATE, optional device (4,): sum w h(E_pred), stride * correction,
                                sum w, walkers sampled */
} afq_cv;

/* afq_block with the measurement chosen by cv (NULL or AFQ_CV_OFF: afq_block). */
int afq_block_cv(const afq_problem* pb, const afq_params* p, const afq_state* st,
                 const double* fields, double zeta, uint64_t seed, uint64_t counter,
                 double* block_energy, double* block_weight, int32_t* sr_idx, const afq_cv* cv,
                 void* workspace, size_t workspace_bytes, void* stream);

/* The network: F -> H -> H -> 1, GELU, bf16 weights.  Every product runs on
 * the tensor cores (mma.sync bf16, fp32 accumulation) with the fp32 operands
 * (inputs, activations, their gradients) as two bf16 pieces, so the sums are
 * fp32-accurate.  F a multiple of 16, H a multiple of 32 in [32, 256]
 * (afq_mlp_param_count returns 0 otherwise).  Parameters (bf16 copy and fp32
 * master, same layout): W1 (H x F), b1 (H), W2 (H x H), b2 (H), w3 (H), b3 (1). */
size_t afq_mlp_param_count(int32_t n_features, int32_t hidden);
/* y (B,) = network(x (B, F) fp32), all device. */
int afq_mlp_forward(int32_t batch, int32_t n_features, int32_t hidden, const void* params_bf16,
                    const float* x, float* y, void* stream);
/* Gradient of the loss mean (y - target)^2 / 2 over a batch with respect to
 * every parameter (fp32, P entries, device) at the bf16 parameters; the
 * batch's rows are split over CTAs of 32 whose partial gradients are added in
 * a fixed order (the same inputs give the same bits).  loss_out (optional,
 * device) receives the loss.  workspace: afq_mlp_train_workspace bytes. */
size_t afq_mlp_train_workspace(int32_t batch, int32_t n_features, int32_t hidden);
int afq_mlp_gradient(int32_t batch, int32_t n_features, int32_t hidden, const void* params_bf16,
                     const float* x, const float* target, float* grad, float* loss_out, void* workspace,
                     size_t workspace_bytes, void* stream);
/* One Adam step (beta 0.9 / 0.999, bias-corrected by `step` >= 1) with that
 * gradient: updates master, its bf16 copy and the moments m, v (two kernel
 * launches).  loss_out (optional, device) receives the batch loss before the
 * update. */
int afq_mlp_train_step(int32_t batch, int32_t n_features, int32_t hidden, float* master, void* params_bf16,
                       float* adam_m, float* adam_v, const float* x, const float* target, float lr,
                       int32_t step, void* workspace, size_t workspace_bytes, float* loss_out,
                       void* stream);
/* bf16 copy of the fp32 master parameters. */
int afq_mlp_sync(int32_t n_features, int32_t hidden, const float* master, void* params_bf16, void* stream);

/* ---- differentiated energy (no counterpart in the reference, which ships
 * no gradient of the energy) ----------------------------------------------
 *
 * dL/dh1 of a run of n_blocks binary64 blocks for any loss L of the block
 * energies and weights, by reverse-mode adjoint kernels; dL/dlam for
 * h1 + lam D is sum_ij dL/dh1[i,j] D[i,j].  The derivative is the pathwise
 * one that jax.grad of a wrapper around afqmc_block (prop/blocks.py:22-95)
 * gives on the same fields: the comb's indices (walkers.py:233-265), the
 * weight floor/cap (prop/afqmc.py:127-134) and the energy clip
 * (prop/blocks.py:59-66) are held at their values; the initial state is a
 * constant.  Fields and comb uniforms come from the Philox stream (seed,
 * counter + b (n_prop_steps + 1) + step) as in afq_run_blocks.  Binary64
 * form, real trial orbitals; the per-walker adjoint algebra sits in shared
 * memory: 32 norb nocc and 64 nocc^2 + 512 nocc bytes must each fit in
 * 227 KiB (nocc up to 52; norb nocc up to 7264, e.g. 200 x 36).
 *
 * afq_grad_forward runs the blocks like afq_block (state updated in place;
 * block b's energy and weight to block_energies[b], block_weights[b], its
 * comb indices to sr_idx[b W ...] when sr_idx is given), keeping in `tape`
 * the state every checkpoint_blocks blocks, the comb indices and the block
 * results.  sr_fixed (optional, n_blocks x W non-decreasing indices) replaces
 * the comb's own indices (finite differences of the same function).
 * afq_grad_backward replays each checkpoint segment and runs the adjoint
 * from energies_bar = dL/de_b, weights_bar = dL/dW_b (device, n_blocks) to
 * h1_bar (device n x n): pb, p, h1 (the h1 pb was built from), seed, counter,
 * n_blocks and checkpoint_blocks as in the forward.  The backward reads two
 * scalars back to the host (scaling of the Frechet derivative of expm).
 * A singular overlap matrix or unsorted indices set the workspace status.
 * Workspace: afq_grad_workspace(d, p, checkpoint_blocks) bytes for the
 * backward; the forward needs afq_grad_workspace(d, p, 0) bytes (a prefix
 * of the backward's layout). */
size_t afq_grad_tape_bytes(const afq_dims* d, int32_t n_blocks, int32_t checkpoint_blocks);
size_t afq_grad_workspace(const afq_dims* d, const afq_params* p, int32_t checkpoint_blocks);
int afq_grad_forward(const afq_problem* pb, const afq_params* p, const afq_state* st, int32_t n_blocks,
                     uint64_t seed, uint64_t counter, int32_t checkpoint_blocks, const int32_t* sr_fixed,
                     double* block_energies, double* block_weights, int32_t* sr_idx, void* tape,
                     size_t tape_bytes, void* workspace, size_t workspace_bytes, void* stream);
int afq_grad_backward(const afq_problem* pb, const afq_params* p, const double* h1, int32_t n_blocks,
                      uint64_t seed, uint64_t counter, int32_t checkpoint_blocks, const void* tape,
                      size_t tape_bytes, const double* energies_bar, const double* weights_bar, double* h1_bar,
                      void* workspace, size_t workspace_bytes, void* stream);

/* ---- unrestricted walkers (walker_kind "unrestricted" with the RHF trial:
 * meas/rhf.py:53-100, prop/chol_afqmc_ops.py:118-183, walkers.py:183-265) ---
 *
 * Walkers (2, W, n, o) complex128: all up-spin walkers, then all down-spin
 * walkers (the reference's tuple (w_up, w_dn) stored contiguously);
 * d->n_walkers = W pairs; binary64 form.  Overlap det(C^H W_up) det(C^H
 * W_dn); force bias L~ vec(G_up + G_dn); energy h0 + sum (G_up + G_dn) o
 * rot_h1 + [sum_g (c_up + c_dn)^2 - exc_up - exc_dn] / 2; Trotter with one
 * V_w for both spins; comb indices shared by both spins.  afq_orthogonalize
 * with n_walkers = 2W orthonormalises both spins.  Fields (W, G) as for
 * restricted walkers.  workspace: afq_u_workspace bytes for every call. */
size_t afq_u_workspace(const afq_dims* d, int32_t n_chunks);
int afq_overlap_u(const afq_dims* d, const double* mo_coeff, const double* walkers, double* overlaps,
                  void* workspace, size_t workspace_bytes, void* stream);
int afq_force_bias_u(const afq_dims* d, const double* mo_coeff, const double* rot_chol, const double* walkers,
                     double* force_bias, void* workspace, size_t workspace_bytes, void* stream);
int afq_energy_u(const afq_dims* d, double h0, const double* mo_coeff, const double* rot_h1,
                 const double* rot_chol, const double* walkers, double* energy, void* workspace,
                 size_t workspace_bytes, void* stream);
int afq_apply_trotter_u(const afq_dims* d, int32_t n_terms, double sqrt_dt, int32_t n_chunks,
                        const double* chol, const double* exp_h1_half, const double* walkers,
                        const double* shifted_fields, double* walkers_out, void* workspace,
                        size_t workspace_bytes, void* stream);
int afq_stochastic_reconfiguration_u(const afq_dims* d, const double* weights, double zeta,
                                     const double* walkers, double* walkers_out, double* weights_out,
                                     int32_t* idx, void* workspace, size_t workspace_bytes, void* stream);
int afq_step_u(const afq_problem* pb, const afq_params* p, const afq_state* st, const double* fields,
               uint64_t seed, uint64_t counter, void* workspace, size_t workspace_bytes, void* stream);
int afq_block_u(const afq_problem* pb, const afq_params* p, const afq_state* st, const double* fields,
                double zeta, uint64_t seed, uint64_t counter, double* block_energy, double* block_weight,
                int32_t* sr_idx, void* workspace, size_t workspace_bytes, void* stream);

/* ---- generalized walkers (walker_kind "generalized" with the RHF trial:
 * meas/rhf.py:103-130, prop/chol_afqmc_ops.py:141-197) ----------------------
 *
 * Walkers (W, 2n, 2o) complex128: the up block of rows over the down block;
 * d->norb = n, d->nocc = o (per spin), mo_coeff the RHF trial (n x o).
 * Overlap det(m), m = vstack(C^H W_top, C^H W_bot); force bias
 * L~ vec(G_uu + G_dd) of G_half = solve(m^T, W^T) (2o x 2n); Trotter: both
 * halves with the walker's V.  afq_orthogonalize and afq_stochastic_-
 * reconfiguration with dims (W, 2n, 2o) orthonormalise and reconfigure
 * them.  The reference has no generalized energy kernel.  Binary64 form.
 * workspace: afq_g_workspace bytes. */
size_t afq_g_workspace(const afq_dims* d, int32_t n_chunks);
int afq_overlap_g(const afq_dims* d, const double* mo_coeff, const double* walkers, double* overlaps,
                  void* workspace, size_t workspace_bytes, void* stream);
int afq_force_bias_g(const afq_dims* d, const double* mo_coeff, const double* rot_chol, const double* walkers,
                     double* force_bias, void* workspace, size_t workspace_bytes, void* stream);
int afq_apply_trotter_g(const afq_dims* d, int32_t n_terms, double sqrt_dt, int32_t n_chunks,
                        const double* chol, const double* exp_h1_half, const double* walkers,
                        const double* shifted_fields, double* walkers_out, void* workspace,
                        size_t workspace_bytes, void* stream);

/* ---- integrals (integrals.py:3-46) ---------------------------------------
 *
 * modified_cholesky: pivoted Cholesky vectors of the 4-fold symmetric ERI
 * matrix mat (size x size device f64, size = n (n + 1) / 2, pairs i >= j in
 * row-major triangle order), the reference's loop and stopping rule
 * (|residual pivot| > max_error), at most min(size, max_vectors) - 1 vectors
 * kept.  chol_out (device, max_vectors x n x n f64) receives the *nchol_out
 * vectors unpacked to symmetric n x n matrices.  Synchronises the stream
 * (the loop's exit is read back every 32 iterations).
 * workspace: afq_modified_cholesky_workspace bytes. */
size_t afq_modified_cholesky_workspace(int32_t size, int32_t max_vectors);
int afq_modified_cholesky(int32_t size, const double* mat, double max_error, int32_t max_vectors,
                          double* chol_out, int32_t* nchol_out, void* workspace, size_t workspace_bytes,
                          void* stream);

/* ---- tracing (no counterpart in the reference, which only times blocks
 * with time.perf_counter, driver.py:83-147) --------------------------------- */

/* Number of kernels this library has launched since it was loaded. */
long long afq_launch_count(void);
/* Process-wide switch: when on, the step and block record CUDA events
 * around each named phase on the launching stream.  Off by default. */
int afq_timing_enable(int on);
/* Waits for recorded events and writes "phase calls total_ms\n" lines of the
 * accumulated per-phase device time into buf. */
int afq_timing_report(char* buf, size_t len);
int afq_timing_reset(void);
/* Calibration (synchronises the device; allocates a small scratch buffer):
 * SIMT FMA throughput of the current GPU in TFLOP/s, binary64 when fp64 != 0
 * else binary32 -- the ceiling of the binary64 kernels' roofline. */
int afq_probe_fma_peak(int fp64, double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* AFQMC_GB300_H */
