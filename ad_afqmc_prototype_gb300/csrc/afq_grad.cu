// Differentiated energy (afq_grad_forward / afq_grad_backward): a run of
// binary64 blocks with its reverse-mode adjoint.  No counterpart in the
// reference (which ships no gradient); the derivative is the pathwise one
// that jax.grad of a wrapper around afqmc_block (prop/blocks.py:22-95) with
// respect to lam in h1 + lam D gives: comb indices, weight floor/cap and
// energy clip held at their values, the initial state constant.
//
// Memory: the forward keeps the state at every checkpoint_blocks-th block
// boundary, the comb indices and the block energies and weights (the tape).
// The backward walks the checkpoint segments from the last: it replays the
// segment's blocks from their checkpoint with every operation's input state
// saved (run_block_taped), then runs the operations' adjoints in reverse.
// Fields and comb uniforms are regenerated from the Philox stream, never
// stored.  dL/dE_half and the one-body energy term are accumulated over the
// run and turned into dL/dh1 at the end (launch_h1bar).
#include <utility>

#include "afq_internal.cuh"

using namespace afq;

namespace {

struct TapeLayout {
    double2* ck_walkers;  // n_ck x W n o
    double* ck_weights;   // n_ck x W
    double2* ck_overlaps; // n_ck x W
    double* ck_pop;       // n_ck
    double* e_est;        // 1
    int32_t* idx;         // n_blocks x W
    double* be;           // n_blocks
    double* bw;           // n_blocks
};

TapeLayout layout_tape(Arena& a, const afq_dims* d, int n_blocks, int ck) {
    const size_t W = d->n_walkers, no = (size_t)d->norb * d->nocc;
    const size_t nck = (n_blocks + ck - 1) / ck;
    TapeLayout t;
    t.ck_walkers = a.take<double2>(nck * W * no);
    t.ck_weights = a.take<double>(nck * W);
    t.ck_overlaps = a.take<double2>(nck * W);
    t.ck_pop = a.take<double>(nck);
    t.e_est = a.take<double>(1);
    t.idx = a.take<int32_t>((size_t)n_blocks * W);
    t.be = a.take<double>(n_blocks);
    t.bw = a.take<double>(n_blocks);
    return t;
}

// walkers per energy-adjoint product chunk: F (o x G o complex) <= 256 MiB
int grad_energy_chunk(const afq_dims* d) {
    const long long per = (long long)d->nocc * d->nchol * d->nocc * 16;
    long long wc = (256LL << 20) / (per > 0 ? per : 1);
    if (wc < 1) wc = 1;
    if (wc > d->n_walkers) wc = d->n_walkers;
    return (int)wc;
}

struct GradWS {
    int* status;
    void* block;
    size_t block_bytes;
    // replay state
    double2* walkers; double* weights; double2* overlaps; double* pop; double* e_est;
    double* be; double* bw;
    BlockSnap snap;  // ck blocks, n_ops slots each (energy: ck x W; V: ck x n_prop_steps when kept)
    bool keep_v;     // the replay keeps each step's V for the adjoint (no V-build recomputation)
    double2* zpart;  // split-K layers of the adjoint's FP64 GEMMs
    // adjoint state (two copies for the comb's scatter)
    double2 *wk, *wk2, *ob, *ob2;
    double *wb, *wb2, *pb, *wsum;
    // step
    double* fields; double2* green; double2* fb; double2* xs; double2* shift_term; double2* fb_term;
    double2* V; double2* terms; double2* w2; double2* tbar; double2* xtb; double2* gbar;
    double2* ovn_tot; double* fbt_bar; double2* shift_bar;
    // energy
    double2* cl; double2* y; double2* F; double2* Ft; double* ebar_w;
    // accumulators
    double* ebar_part; double2* sg_part; double* ebar; double2* sg;
    double* h1e; double* ftmp;
};

// The forward uses the first two regions only (status word and a block's workspace).
GradWS layout_grad_forward(Arena& a, const afq_dims* d, const afq_params* p) {
    GradWS g = {};
    g.status = a.take<int>(64);  // status word: offset 0 of every workspace
    g.block_bytes = block_ws_bytes(d, p->n_chunks);
    g.block = a.take<char>(g.block_bytes);
    return g;
}

GradWS layout_grad(Arena& a, const afq_dims* d, const afq_params* p, int ck) {
    const size_t W = d->n_walkers, n = d->norb, o = d->nocc, G = d->nchol, no = n * o;
    const size_t K = p->n_exp_terms > 0 ? p->n_exp_terms : 0;
    const size_t nops = block_op_count(p);
    const size_t ns = ebar_splits(d->n_walkers);
    const size_t wc = grad_energy_chunk(d);
    GradWS g = layout_grad_forward(a, d, p);
    g.walkers = a.take<double2>(W * no);
    g.weights = a.take<double>(W);
    g.overlaps = a.take<double2>(W);
    g.pop = a.take<double>(1);
    g.e_est = a.take<double>(1);
    g.be = a.take<double>(1);
    g.bw = a.take<double>(1);
    g.snap.walkers = a.take<double2>(ck * nops * W * no);
    g.snap.weights = a.take<double>(ck * nops * W);
    g.snap.overlaps = a.take<double2>(ck * nops * W);
    g.snap.pop = a.take<double>(ck * nops);
    g.snap.energy = a.take<double2>(ck * W);
    const size_t vbytes = (size_t)ck * p->n_prop_steps * W * n * n * sizeof(double2);
    const int wc1 = p->n_chunks <= 1 ? (int)W : (int)((W + p->n_chunks - 1) / p->n_chunks);
    g.keep_v = wc1 == (int)W && vbytes <= ((size_t)8 << 30);
    g.snap.V = g.keep_v ? a.take<double2>(vbytes / sizeof(double2)) : nullptr;
    {
        const size_t z1 = (size_t)zgemm_splits((int)W, (int)G, (int)(n * n)) * W * G;
        const size_t z2 = (size_t)zgemm_splits((int)W, (int)no, (int)G) * W * no;
        g.zpart = a.take<double2>(z1 > z2 ? z1 : z2);
    }
    g.wk = a.take<double2>(W * no);
    g.wk2 = a.take<double2>(W * no);
    g.ob = a.take<double2>(W);
    g.ob2 = a.take<double2>(W);
    g.wb = a.take<double>(W);
    g.wb2 = a.take<double>(W);
    g.pb = a.take<double>(1);
    g.wsum = a.take<double>(1);
    g.fields = a.take<double>(W * G);
    g.green = a.take<double2>(W * no);
    g.fb = a.take<double2>(W * G);
    g.xs = a.take<double2>(W * G);
    g.shift_term = a.take<double2>(W);
    g.fb_term = a.take<double2>(W);
    g.V = a.take<double2>(W * n * n);
    g.terms = a.take<double2>(W * (K > 0 ? K : 1) * no);
    g.w2 = a.take<double2>(W * no);
    g.tbar = a.take<double2>(W * (K + 1) * no);
    g.xtb = a.take<double2>(W * G);
    g.gbar = a.take<double2>(W * no);
    g.ovn_tot = a.take<double2>(W);
    g.fbt_bar = a.take<double>(W);
    g.shift_bar = a.take<double2>(W);
    g.cl = a.take<double2>(W * no);
    g.y = a.take<double2>(W * no);
    g.F = a.take<double2>(wc * o * G * o);
    g.Ft = a.take<double2>(wc * o * G * o);
    g.ebar_w = a.take<double>(W);
    g.ebar_part = a.take<double>(ns * n * n);
    g.sg_part = a.take<double2>(ns * no);
    g.ebar = a.take<double>(n * n);
    g.sg = a.take<double2>(no);
    g.h1e = a.take<double>(n * n);
    g.ftmp = a.take<double>(5 * 4 * n * n + 2);
    return g;
}

int check_grad(const afq_problem* pb, const afq_params* p, int n_blocks, int ck) {
    if (!pb || !p) return fail(AFQ_E_INVALID_ARGUMENT, "problem / params is NULL");
    const afq_dims* d = &pb->dims;
    if (d->precision != AFQ_PREC_FP64) return fail(AFQ_E_UNSUPPORTED, "the gradient runs the binary64 form");
    if (!d->trial_is_real) return fail(AFQ_E_UNSUPPORTED, "the gradient supports real trial orbitals");
    // per-walker adjoint algebra in shared memory: the Taylor adjoint holds two n x o complex
    // blocks, the overlap and QR adjoints four o x o blocks and 32 staged rows
    const size_t no = (size_t)d->norb * d->nocc, oo = (size_t)d->nocc * d->nocc;
    if (2 * no * sizeof(double2) > 227 * 1024 || (4 * oo + 32 * (size_t)d->nocc) * sizeof(double2) > 227 * 1024)
        return fail(AFQ_E_UNSUPPORTED, "the gradient needs 32 norb nocc <= 227 KiB and 64 nocc^2 + 512 nocc <= "
                    "227 KiB (norb %d, nocc %d)", d->norb, d->nocc);
    if (n_blocks < 1) return fail(AFQ_E_INVALID_ARGUMENT, "n_blocks=%d < 1", n_blocks);
    if (ck < 1) return fail(AFQ_E_INVALID_ARGUMENT, "checkpoint_blocks=%d < 1", ck);
    if (p->n_prop_steps < 1) return fail(AFQ_E_INVALID_ARGUMENT, "n_prop_steps=%d < 1", p->n_prop_steps);
    if (p->n_exp_terms < 0) return fail(AFQ_E_INVALID_ARGUMENT, "n_exp_terms=%d < 0", p->n_exp_terms);
    if (d->n_walkers > 65535) return fail(AFQ_E_UNSUPPORTED, "the gradient supports <= 65535 walkers");
    return AFQ_OK;
}

uint64_t block_counter(uint64_t counter, const afq_params* p, int b) {
    return counter + (uint64_t)b * (uint64_t)(p->n_prop_steps + 1);
}

struct Ctx {
    const afq_problem* pb;
    const afq_params* p;
    const GradWS* g;
    uint64_t seed;
    cudaStream_t s;
};

template <class T>
T* slot(T* base, size_t per, int k) { return base + (size_t)k * per; }

// Adjoint of step st_i of a block, whose input state is snapshot slot op.
int step_adjoint(const Ctx& c, const BlockSnap& sn, int op, int st_i, uint64_t counter) {
    const afq_problem* pb = c.pb;
    const afq_dims* d = &pb->dims;
    const GradWS& g = *c.g;
    const int W = d->n_walkers, n = d->norb, o = d->nocc, G = d->nchol, no = n * o, K = c.p->n_exp_terms;
    const double2* mo = (const double2*)pb->mo_coeff;
    cudaStream_t s = c.s;
    const double2* Wpre = slot(sn.walkers, (size_t)W * no, op);
    const double2* Wpost = slot(sn.walkers, (size_t)W * no, op + 1);
    // forward recomputation (the block's own kernels: the same fields, force bias and shifts)
    {
        AFQ_PHASE("adj_recompute", s);
        AFQ_TRY(launch_philox((int64_t)W * G, c.seed, counter, 1, g.fields, s));
        AFQ_TRY(launch_green(W, n, o, mo, 1, Wpre, nullptr, g.green, s));
        AFQ_TRY(launch_zgemm(W, G, no, 2.0, g.green, no, pb->rot_chol, no, false, true, g.fb, G, s));
        AFQ_TRY(launch_field_shift(W, G, pb->sqrt_dt, g.fields, g.fb, (const double2*)pb->mf_shifts, g.xs,
                                   g.shift_term, g.fb_term, s));
    }
    const double2* V = sn.V ? sn.V + (size_t)st_i * W * n * n : g.V;
    if (!sn.V) {
        AFQ_PHASE("adj_vbuild_gemm", s);
        AFQ_TRY(launch_zgemm(W, n * n, G, 1.0, g.xs, G, pb->chol, (int64_t)n * n, false, false, g.V,
                             (int64_t)n * n, s));
    }
    { AFQ_PHASE("adj_taylor_tape", s);
      AFQ_TRY(launch_taylor_tape(W, n, o, K, pb->sqrt_dt, pb->exp_h1_half, V, Wpre, g.terms, g.w2, s)); }
    AFQ_PHASE("adj_step_rest", s);
    // weights, population shift and overlap ratio
    AFQ_TRY(launch_weight_adj(W, c.p, pb->sqrt_dt, pb->dt, make_double2(pb->h0_prop_re, pb->h0_prop_im),
                              g.shift_term, g.fb_term, slot(sn.weights, W, op), slot(sn.overlaps, W, op),
                              sn.pop + op, slot(sn.weights, W, op + 1), slot(sn.overlaps, W, op + 1), g.wb, g.ob,
                              g.pb, g.ovn_tot, g.fbt_bar, g.shift_bar, s));
    // overlaps of the new walkers
    AFQ_TRY(launch_green_adj(W, n, o, mo, Wpost, nullptr, slot(sn.overlaps, W, op + 1), g.ovn_tot, g.wk, g.status,
                             s));
    // W' = E W2: dL/dE += Re W'b W2^H; Taylor reverse; W1 = E W: dL/dE += Re W1b W^H
    { AFQ_PHASE("adj_ebar", s); AFQ_TRY(launch_ebar(W, n, o, g.wk, no, g.w2, no, g.ebar_part, s)); }
    { AFQ_PHASE("adj_taylor", s);
      AFQ_TRY(launch_taylor_adj(W, n, o, K, pb->sqrt_dt, pb->exp_h1_half, V, g.wk, g.tbar, g.wk, s)); }
    { AFQ_PHASE("adj_ebar", s);
      AFQ_TRY(launch_ebar(W, n, o, g.tbar, (long long)(K + 1) * no, Wpre, no, g.ebar_part, s)); }
    // V = sum_g x~_g L_g: x~b = Vb . L^T
    { AFQ_PHASE("adj_vbar", s); AFQ_TRY(launch_vbar(W, n, o, K, pb->sqrt_dt, g.tbar, g.terms, g.V, s)); }
    { AFQ_PHASE("adj_xbar_gemm", s);
      AFQ_TRY(launch_zgemm_splitk(W, G, n * n, 1.0, g.V, (int64_t)n * n, pb->chol, (int64_t)n * n, false, true,
                                  g.xtb, g.zpart, s)); }
    // field shifts, then the force bias fb = 2 L~ vec(G_half)
    AFQ_TRY(launch_fs_adj(W, G, pb->sqrt_dt, g.fields, g.fb, (const double2*)pb->mf_shifts, g.fbt_bar, g.shift_bar,
                          g.xtb, s));
    AFQ_TRY(launch_zgemm_splitk(W, no, G, 2.0, g.xtb, G, pb->rot_chol, no, false, false, g.gbar, g.zpart, s));
    return launch_green_adj(W, n, o, mo, Wpre, g.gbar, nullptr, nullptr, g.wk, g.status, s);
}

// Adjoint of block b (its snapshots in sn; block energy at tape.be[b]).
int block_adjoint(const Ctx& c, const BlockSnap& sn, const TapeLayout& t, int b, uint64_t counter,
                  const double* eb_bar, const double* wb_bar, GradWS& g) {
    const afq_problem* pb = c.pb;
    const afq_params* p = c.p;
    const afq_dims* d = &pb->dims;
    const int W = d->n_walkers, n = d->norb, o = d->nocc, G = d->nchol, no = n * o;
    const int nops = block_op_count(p);
    const double2* mo = (const double2*)pb->mo_coeff;
    cudaStream_t s = c.s;
    const double2* Wm = slot(sn.walkers, (size_t)W * no, nops - 1);
    const double* wm = slot(sn.weights, W, nops - 1);
    const double2* om = slot(sn.overlaps, W, nops - 1);
    // comb: gather by the indices, weights sum|w| / N
    AFQ_TRY(launch_sr_adj(W, no, t.idx + (size_t)b * W, g.wk, g.ob, g.wb, wm, g.wsum, g.wk2, g.ob2, g.wb2, g.status,
                          s));
    std::swap(g.wk, g.wk2);
    std::swap(g.ob, g.ob2);
    std::swap(g.wb, g.wb2);
    AFQ_PHASE("adj_block_end", s);
    // measurement and population-shift EMA
    AFQ_TRY(launch_measure_adj(W, p->dt, p->shift_ema, wm, sn.energy, g.e_est, t.be + b, eb_bar + b, wb_bar + b,
                               g.pb, g.wb, g.ebar_w, s));
    // local energies -> G_half of the measured walkers
    AFQ_TRY(launch_green(W, n, o, mo, 1, Wm, nullptr, g.green, s));
    AFQ_TRY(launch_zgemm(W, G, no, 1.0, g.green, no, pb->rot_chol, no, false, true, g.xtb, G, s));   // c_g
    AFQ_TRY(launch_zgemm(W, no, G, 1.0, g.xtb, G, pb->rot_chol, no, false, false, g.cl, no, s));     // sum c_g L~_g
    const int wc = grad_energy_chunk(d);
    for (int w0 = 0; w0 < W; w0 += wc) {
        const int nw = W - w0 < wc ? W - w0 : wc;
        // F[(w, q), (g, p)] = f_g[p, q];  y[(w, p), j] = sum_{g, q} f_g[p, q] L~_g[q, j]
        AFQ_TRY(launch_zgemm(nw * o, G * o, n, 1.0, g.green + (size_t)w0 * no, n, pb->rot_chol, n, false, true, g.F,
                             (int64_t)G * o, s));
        AFQ_TRY(launch_block_transpose(nw, o, G, g.F, g.Ft, s));
        AFQ_TRY(launch_zgemm(nw * o, n, G * o, 1.0, g.Ft, (int64_t)G * o, pb->rot_chol, n, false, false,
                             g.y + (size_t)w0 * no, n, s));
    }
    AFQ_TRY(launch_energy_gbar(W, no, g.ebar_w, (const double2*)pb->rot_h1, g.cl, g.y, g.gbar, s));
    AFQ_TRY(launch_sg_accum(W, no, g.ebar_w, g.green, g.sg_part, s));
    AFQ_TRY(launch_green_adj(W, n, o, mo, Wm, g.gbar, om, g.ob, g.wk, g.status, s));
    AFQ_CUDA(cudaMemsetAsync(g.ob, 0, sizeof(double2) * W, s));
    // block-end QR
    AFQ_TRY(launch_qr_adj(W, n, o, slot(sn.walkers, (size_t)W * no, nops - 2), Wm, g.wk, g.wk, g.status, s));
    // steps and the QRs between them, in reverse
    int op = nops - 3;
    for (int st_i = p->n_prop_steps - 1; st_i >= 0; --st_i) {
        if (p->qr_every > 0 && (st_i + 1) % p->qr_every == 0 && st_i + 1 < p->n_prop_steps) {
            const double2* post = slot(sn.walkers, (size_t)W * no, op + 1);
            AFQ_TRY(launch_green_adj(W, n, o, mo, post, nullptr, slot(sn.overlaps, W, op + 1), g.ob, g.wk, g.status,
                                     s));
            AFQ_CUDA(cudaMemsetAsync(g.ob, 0, sizeof(double2) * W, s));
            AFQ_TRY(launch_qr_adj(W, n, o, slot(sn.walkers, (size_t)W * no, op), post, g.wk, g.wk, g.status, s));
            --op;
        }
        AFQ_TRY(step_adjoint(c, sn, op, st_i, counter + st_i));
        --op;
    }
    if (op != -1) return fail(AFQ_E_INVALID_ARGUMENT, "internal: block operations out of step (%d)", op);
    return AFQ_OK;
}

}  // namespace

size_t afq_grad_tape_bytes(const afq_dims* d, int32_t n_blocks, int32_t checkpoint_blocks) {
    if (!d || n_blocks < 1 || checkpoint_blocks < 1) return 0;
    Arena a;
    layout_tape(a, d, n_blocks, checkpoint_blocks);
    return a.used;
}

size_t afq_grad_workspace(const afq_dims* d, const afq_params* p, int32_t checkpoint_blocks) {
    if (!d || !p) return 0;
    Arena a;
    if (checkpoint_blocks < 1) layout_grad_forward(a, d, p);
    else layout_grad(a, d, p, checkpoint_blocks);
    return a.used;
}

int afq_grad_forward(const afq_problem* pb, const afq_params* p, const afq_state* st, int32_t n_blocks,
                     uint64_t seed, uint64_t counter, int32_t checkpoint_blocks, const int32_t* sr_fixed,
                     double* block_energies, double* block_weights, int32_t* sr_idx, void* tape,
                     size_t tape_bytes, void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_grad(pb, p, n_blocks, checkpoint_blocks));
    if (!st || !st->walkers || !st->weights || !st->overlaps || !st->pop_control_ene_shift || !st->e_estimate)
        return fail(AFQ_E_INVALID_ARGUMENT, "state has a NULL member");
    if (!block_energies || !block_weights || !tape || !workspace)
        return fail(AFQ_E_INVALID_ARGUMENT, "NULL output, tape or workspace");
    const afq_dims* d = &pb->dims;
    Arena ta(tape, tape_bytes);
    const TapeLayout t = layout_tape(ta, d, n_blocks, checkpoint_blocks);
    if (!ta.ok()) return fail(AFQ_E_WORKSPACE, "tape: %zu bytes < %zu", tape_bytes, ta.used);
    Arena a(workspace, workspace_bytes);
    GradWS g = layout_grad_forward(a, d, p);
    if (!a.ok()) return fail(AFQ_E_WORKSPACE, "workspace: %zu bytes < %zu", workspace_bytes, a.used);
    cudaStream_t s = as_stream(stream);
    const size_t W = d->n_walkers, no = (size_t)d->norb * d->nocc;
    AFQ_CUDA(cudaMemsetAsync(g.status, 0, sizeof(int), s));
    AFQ_CUDA(cudaMemcpyAsync(t.e_est, st->e_estimate, sizeof(double), cudaMemcpyDeviceToDevice, s));
    for (int b = 0; b < n_blocks; ++b) {
        if (b % checkpoint_blocks == 0) {
            const int k = b / checkpoint_blocks;
            AFQ_CUDA(cudaMemcpyAsync(t.ck_walkers + k * W * no, st->walkers, sizeof(double2) * W * no,
                                     cudaMemcpyDeviceToDevice, s));
            AFQ_CUDA(cudaMemcpyAsync(t.ck_weights + k * W, st->weights, sizeof(double) * W, cudaMemcpyDeviceToDevice,
                                     s));
            AFQ_CUDA(cudaMemcpyAsync(t.ck_overlaps + k * W, st->overlaps, sizeof(double2) * W,
                                     cudaMemcpyDeviceToDevice, s));
            AFQ_CUDA(cudaMemcpyAsync(t.ck_pop + k, st->pop_control_ene_shift, sizeof(double),
                                     cudaMemcpyDeviceToDevice, s));
        }
        AFQ_TRY(run_block_taped(pb, p, st, seed, block_counter(counter, p, b), sr_fixed ? sr_fixed + b * W : nullptr,
                                t.idx + b * W, t.be + b, t.bw + b, nullptr, g.block, g.block_bytes, s));
    }
    AFQ_CUDA(cudaMemcpyAsync(block_energies, t.be, sizeof(double) * n_blocks, cudaMemcpyDeviceToDevice, s));
    AFQ_CUDA(cudaMemcpyAsync(block_weights, t.bw, sizeof(double) * n_blocks, cudaMemcpyDeviceToDevice, s));
    if (sr_idx)
        AFQ_CUDA(cudaMemcpyAsync(sr_idx, t.idx, sizeof(int32_t) * W * n_blocks, cudaMemcpyDeviceToDevice, s));
    return AFQ_OK;
}

int afq_grad_backward(const afq_problem* pb, const afq_params* p, const double* h1, int32_t n_blocks,
                      uint64_t seed, uint64_t counter, int32_t checkpoint_blocks, const void* tape,
                      size_t tape_bytes, const double* energies_bar, const double* weights_bar, double* h1_bar,
                      void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_grad(pb, p, n_blocks, checkpoint_blocks));
    if (!h1 || !tape || !energies_bar || !weights_bar || !h1_bar || !workspace)
        return fail(AFQ_E_INVALID_ARGUMENT, "NULL argument");
    const afq_dims* d = &pb->dims;
    Arena ta((void*)tape, tape_bytes);
    const TapeLayout t = layout_tape(ta, d, n_blocks, checkpoint_blocks);
    if (!ta.ok()) return fail(AFQ_E_WORKSPACE, "tape: %zu bytes < %zu", tape_bytes, ta.used);
    Arena a(workspace, workspace_bytes);
    GradWS g = layout_grad(a, d, p, checkpoint_blocks);
    if (!a.ok()) return fail(AFQ_E_WORKSPACE, "workspace: %zu bytes < %zu", workspace_bytes, a.used);
    cudaStream_t s = as_stream(stream);
    const int W = d->n_walkers, n = d->norb, o = d->nocc, no = n * o;
    const int ck = checkpoint_blocks, nops = block_op_count(p), ns = ebar_splits(W);
    AFQ_CUDA(cudaMemsetAsync(g.status, 0, sizeof(int), s));
    AFQ_CUDA(cudaMemsetAsync(g.wk, 0, sizeof(double2) * W * no, s));
    AFQ_CUDA(cudaMemsetAsync(g.ob, 0, sizeof(double2) * W, s));
    AFQ_CUDA(cudaMemsetAsync(g.wb, 0, sizeof(double) * W, s));
    AFQ_CUDA(cudaMemsetAsync(g.pb, 0, sizeof(double), s));
    AFQ_CUDA(cudaMemsetAsync(g.ebar_part, 0, sizeof(double) * ns * n * n, s));
    AFQ_CUDA(cudaMemsetAsync(g.sg_part, 0, sizeof(double2) * ns * no, s));
    AFQ_CUDA(cudaMemcpyAsync(g.e_est, t.e_est, sizeof(double), cudaMemcpyDeviceToDevice, s));
    afq_state wst;
    wst.walkers = (double*)g.walkers;
    wst.weights = g.weights;
    wst.overlaps = (double*)g.overlaps;
    wst.pop_control_ene_shift = g.pop;
    wst.e_estimate = g.e_est;
    const Ctx c{pb, p, &g, seed, s};
    const int nseg = (n_blocks + ck - 1) / ck;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        AFQ_CUDA(cudaMemcpyAsync(g.walkers, t.ck_walkers + (size_t)seg * W * no, sizeof(double2) * W * no,
                                 cudaMemcpyDeviceToDevice, s));
        AFQ_CUDA(cudaMemcpyAsync(g.weights, t.ck_weights + (size_t)seg * W, sizeof(double) * W,
                                 cudaMemcpyDeviceToDevice, s));
        AFQ_CUDA(cudaMemcpyAsync(g.overlaps, t.ck_overlaps + (size_t)seg * W, sizeof(double2) * W,
                                 cudaMemcpyDeviceToDevice, s));
        AFQ_CUDA(cudaMemcpyAsync(g.pop, t.ck_pop + seg, sizeof(double), cudaMemcpyDeviceToDevice, s));
        const int b0 = seg * ck, b1 = b0 + ck < n_blocks ? b0 + ck : n_blocks;
        auto snap_of = [&](int b) {
            BlockSnap x;
            const size_t k = (size_t)(b - b0) * nops;
            x.walkers = g.snap.walkers + k * W * no;
            x.weights = g.snap.weights + k * W;
            x.overlaps = g.snap.overlaps + k * W;
            x.pop = g.snap.pop + k;
            x.energy = g.snap.energy + (size_t)(b - b0) * W;
            x.V = g.keep_v ? g.snap.V + (size_t)(b - b0) * p->n_prop_steps * W * n * n : nullptr;
            return x;
        };
        for (int b = b0; b < b1; ++b) {
            AFQ_PHASE("adj_replay", s);
            const BlockSnap x = snap_of(b);
            AFQ_TRY(run_block_taped(pb, p, &wst, seed, block_counter(counter, p, b), t.idx + (size_t)b * W, nullptr,
                                    g.be, g.bw, &x, g.block, g.block_bytes, s));
        }
        for (int b = b1 - 1; b >= b0; --b)
            AFQ_TRY(block_adjoint(c, snap_of(b), t, b, block_counter(counter, p, b), energies_bar, weights_bar, g));
    }
    AFQ_TRY(launch_sum_partials(n * n, ns, g.ebar_part, g.ebar, s));
    AFQ_TRY(launch_sum_partials(2 * no, ns, (const double*)g.sg_part, (double*)g.sg, s));
    AFQ_TRY(launch_h1_eff(n, d->nchol, h1, pb->chol, (const double2*)pb->mf_shifts, g.h1e, s));
    return launch_h1bar(n, o, pb->dt, g.h1e, g.ebar, (const double2*)pb->mo_coeff, g.sg, h1_bar, g.ftmp, s);
}
