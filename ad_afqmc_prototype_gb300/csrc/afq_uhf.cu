// Unrestricted and generalized walkers with the RHF trial: kernels and
// extern "C" entry points of the binary64 step and block (unrestricted) and
// of the overlap, force bias and Trotter step (generalized; the reference has
// no generalized energy kernel, so no block either).
//
// A walker is a pair (W_up, W_dn), each n x o (the RHF trial gives both
// spins nocc columns).  The engine stores the W pairs as one (2, W, n, o)
// complex128 array -- all up walkers, then all down walkers -- so the
// per-walker kernels of the restricted path (Green's function, Trotter, QR,
// energy partials) run on 2W spin-walkers.  What is new is the combination
// of the two spins (meas/rhf.py:53-100, prop/chol_afqmc_ops.py:118-183,
// walkers.py:183-265 of the reference):
//   overlap    det(C^H W_up) det(C^H W_dn)
//   force bias L~ vec(G_up + G_dn)
//   energy     h0 + sum (G_up + G_dn) o rot_h1
//              + [sum_g (c_up + c_dn)_g^2 - exc_up - exc_dn] / 2
//   Trotter    the same V_w on both spins
//   QR         per spin;  comb: one set of indices for both spins.
#include "afq_internal.cuh"

namespace afq {

// ov[w] = det_up[w] det_dn[w]
__global__ void k_spin_prod(int W, const double2* __restrict__ det, double2* __restrict__ ov) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w < W) ov[w] = cmul(det[w], det[W + w]);
}

// g[e] = G_up[e] + G_dn[e] over W o n entries
__global__ void k_spin_sum(long long count, const double2* __restrict__ green, double2* __restrict__ g) {
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < count;
         e += (long long)gridDim.x * blockDim.x)
        g[e] = cadd(green[e], green[count + e]);
}

// E_w from the spin-summed G (gsum), the Coulomb vectors c (2W x G: up rows,
// then down rows) and the exchange partials of the 2W spin-walkers; one
// warp per walker.
__global__ void k_energy_finish_u(int W, int on, int G, int nchunk, double h0, const double2* __restrict__ gsum,
                                  const double2* __restrict__ rot_h1, const double2* __restrict__ c,
                                  const double2* __restrict__ partial, double2* __restrict__ energy) {
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= W) return;
    double er = 0.0, ei = 0.0;
    for (int e = lane; e < on; e += 32) {
        const double2 p = cmul(gsum[(size_t)w * on + e], rot_h1[e]);
        er += p.x;
        ei += p.y;
    }
    double cr = 0.0, ci = 0.0;
    for (int g = lane; g < G; g += 32) {
        const double2 t = cadd(c[(size_t)w * G + g], c[(size_t)(W + w) * G + g]);
        const double2 t2 = cmul(t, t);
        cr += t2.x;
        ci += t2.y;
    }
    double xr = 0.0, xi = 0.0;
    for (int k = lane; k < nchunk; k += 32) {
        const double2 a = partial[((size_t)w * nchunk + k) * 2 + 1];
        const double2 b = partial[((size_t)(W + w) * nchunk + k) * 2 + 1];
        xr += a.x + b.x;
        xi += a.y + b.y;
    }
    er = warp_sum(er); ei = warp_sum(ei);
    cr = warp_sum(cr); ci = warp_sum(ci);
    xr = warp_sum(xr); xi = warp_sum(xi);
    if (lane == 0) energy[w] = make_double2(h0 + er + 0.5 * (cr - xr), ei + 0.5 * (ci - xi));
}

namespace {

int launch_spin_prod(int W, const double2* det, double2* ov, cudaStream_t s) {
    k_spin_prod<<<(W + 255) / 256, 256, 0, s>>>(W, det, ov);
    AFQ_LAUNCHED("k_spin_prod");
    return AFQ_OK;
}

int launch_spin_sum(long long count, const double2* green, double2* g, cudaStream_t s) {
    long long blocks = (count + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    k_spin_sum<<<(unsigned)blocks, 256, 0, s>>>(count, green, g);
    AFQ_LAUNCHED("k_spin_sum");
    return AFQ_OK;
}

int chunk_of(int W, int n_chunks) { return n_chunks <= 1 ? W : (W + n_chunks - 1) / n_chunks; }

struct UWS {
    int* status;
    double* fields;      // W G
    double2* green;      // 2W o n
    double2* gsum;       // W o n
    double2* fb;         // W G   (also the Coulomb vectors' first half)
    double2* c;          // 2W G
    double2* xs;         // W G
    double2 *shift_term, *fb_term, *det, *ov_new;  // W, W, 2W, W
    double2* V;          // Wc n n
    double* partial;     // energy partials of 2W spin-walkers
    double2* energy;     // W
    double* levels;
    int32_t* idx;
    double *avg, *zeta;
    double2* wcopy;      // 2W n o
    double2* ocopy;      // W
};

UWS layout_u(Arena& a, const afq_dims* d, int n_chunks) {
    const size_t W = d->n_walkers, n = d->norb, o = d->nocc, G = d->nchol, no = n * o;
    UWS u = {};
    u.status = a.take<int>(64);  // status word: offset 0 of every workspace
    u.fields = a.take<double>(W * G);
    u.green = a.take<double2>(2 * W * no);
    u.gsum = a.take<double2>(W * no);
    u.fb = a.take<double2>(W * G);
    u.c = a.take<double2>(2 * W * G);
    u.xs = a.take<double2>(W * G);
    u.shift_term = a.take<double2>(W);
    u.fb_term = a.take<double2>(W);
    u.det = a.take<double2>(2 * W);
    u.ov_new = a.take<double2>(W);
    u.V = a.take<double2>((size_t)chunk_of(d->n_walkers, n_chunks) * n * n);
    u.partial = (double*)a.take<double2>(energy_partial_count(2 * d->n_walkers, d->nocc, d->nchol));
    u.energy = a.take<double2>(W);
    u.levels = a.take<double>(sr_levels_size(d->n_walkers));
    u.idx = a.take<int32_t>(W);
    u.avg = a.take<double>(1);
    u.zeta = a.take<double>(1);
    u.wcopy = a.take<double2>(2 * W * no);
    u.ocopy = a.take<double2>(W);
    return u;
}

int check_u(const afq_dims* d) {
    if (!d) return fail(AFQ_E_INVALID_ARGUMENT, "dims is NULL");
    if (d->n_walkers < 1 || d->norb < 1 || d->nocc < 1 || d->nocc > d->norb || d->nchol < 1)
        return fail(AFQ_E_INVALID_ARGUMENT, "bad dims W=%d n=%d o=%d G=%d", d->n_walkers, d->norb, d->nocc,
                    d->nchol);
    if (d->precision != AFQ_PREC_FP64)
        return fail(AFQ_E_UNSUPPORTED, "unrestricted walkers run the binary64 form");
    if (2 * d->n_walkers > 65535) return fail(AFQ_E_UNSUPPORTED, "unrestricted walkers: W=%d > 32767", d->n_walkers);
    return AFQ_OK;
}

// overlaps (and optionally both spins' G_half) of the pairs
int overlap_u(const afq_dims* d, const double2* mo, const double2* walk, double2* ov, double2* green, const UWS& u,
              cudaStream_t s) {
    AFQ_TRY(launch_green_det(2 * d->n_walkers, d->norb, d->nocc, mo, d->trial_is_real, walk, u.det, green, s));
    return launch_spin_prod(d->n_walkers, u.det, ov, s);
}

// fb = L~ vec(G_up + G_dn) from both spins' G_half in u.green
int force_bias_u(const afq_dims* d, const double* rot_chol, const UWS& u, double2* fb, cudaStream_t s) {
    const int W = d->n_walkers, on = d->norb * d->nocc;
    AFQ_TRY(launch_spin_sum((long long)W * on, u.green, u.gsum, s));
    return launch_zgemm(W, d->nchol, on, 1.0, u.gsum, on, rot_chol, on, !d->trial_is_real, true, fb, d->nchol, s);
}

int trotter_u(const afq_dims* d, int n_terms, double sqrt_dt, int n_chunks, const double* chol, const double* E,
              const double2* win, const double2* xs, double2* wout, double2* V, cudaStream_t s) {
    const int W = d->n_walkers, n = d->norb, o = d->nocc, G = d->nchol;
    const size_t half = (size_t)W * n * o;
    const int Wc = chunk_of(W, n_chunks);
    for (int w0 = 0; w0 < W; w0 += Wc) {
        const int wc = W - w0 < Wc ? W - w0 : Wc;
        { AFQ_PHASE("vbuild_gemm", s);
          AFQ_TRY(launch_zgemm(wc, n * n, G, 1.0, xs + (size_t)w0 * G, G, chol, (int64_t)n * n, false, false, V,
                               (int64_t)n * n, s)); }
        AFQ_PHASE("trotter", s);
        for (int spin = 0; spin < 2; ++spin)
            AFQ_TRY(launch_trotter(wc, n, o, n_terms, sqrt_dt, E, V, win + spin * half + (size_t)w0 * n * o,
                                   wout + spin * half + (size_t)w0 * n * o, s));
    }
    return AFQ_OK;
}

// local energies of the pairs into u.energy; u.green must hold both spins' G_half
int energy_u(const afq_problem* pb, const UWS& u, cudaStream_t s) {
    const afq_dims* d = &pb->dims;
    const int W = d->n_walkers, n = d->norb, o = d->nocc, G = d->nchol, on = n * o;
    AFQ_PHASE("energy", s);
    AFQ_TRY(launch_spin_sum((long long)W * on, u.green, u.gsum, s));
    AFQ_TRY(launch_zgemm(2 * W, G, on, 1.0, u.green, on, pb->rot_chol, on, !d->trial_is_real, true, u.c, G, s));
    AFQ_TRY(launch_energy_partial(2 * W, n, o, G, u.green, pb->rot_chol, d->trial_is_real, u.partial, s));
    k_energy_finish_u<<<(W + 7) / 8, 256, 0, s>>>(W, on, G, energy_partial_chunks(o, G), pb->h0, u.gsum,
                                                  (const double2*)pb->rot_h1, u.c, (const double2*)u.partial,
                                                  u.energy);
    AFQ_LAUNCHED("k_energy_finish_u");
    return AFQ_OK;
}

int step_u(const afq_problem* pb, const afq_params* p, const afq_state* st, const double* fields, uint64_t seed,
           uint64_t counter, const UWS& u, cudaStream_t s) {
    const afq_dims* d = &pb->dims;
    const int W = d->n_walkers, G = d->nchol;
    const double2* mo = (const double2*)pb->mo_coeff;
    double2* walk = (double2*)st->walkers;
    if (!fields) {
        AFQ_PHASE("philox", s);
        AFQ_TRY(launch_philox((int64_t)W * G, seed, counter, 1, u.fields, s));
        fields = u.fields;
    }
    { AFQ_PHASE("green", s);
      AFQ_TRY(launch_green(2 * W, d->norb, d->nocc, mo, d->trial_is_real, walk, nullptr, u.green, s)); }
    { AFQ_PHASE("fb_gemm", s); AFQ_TRY(force_bias_u(d, pb->rot_chol, u, u.fb, s)); }
    { AFQ_PHASE("field_shift", s);
      AFQ_TRY(launch_field_shift(W, G, pb->sqrt_dt, fields, u.fb, (const double2*)pb->mf_shifts, u.xs, u.shift_term,
                                 u.fb_term, s)); }
    AFQ_TRY(trotter_u(d, p->n_exp_terms, pb->sqrt_dt, p->n_chunks, pb->chol, pb->exp_h1_half, walk, u.xs, walk, u.V,
                      s));
    { AFQ_PHASE("overlap", s); AFQ_TRY(overlap_u(d, mo, walk, u.ov_new, nullptr, u, s)); }
    AFQ_PHASE("weight_update", s);
    return launch_weight_update(W, p, pb->sqrt_dt, pb->dt, make_double2(pb->h0_prop_re, pb->h0_prop_im),
                                u.shift_term, u.fb_term, u.ov_new, st->weights, (double2*)st->overlaps,
                                st->pop_control_ene_shift, st->e_estimate, s, u.status);
}

// QR of both spins, then the pairs' overlaps (and G_half when green is given)
int orthonormalize_u(const afq_problem* pb, const afq_state* st, const UWS& u, double2* green, cudaStream_t s) {
    const afq_dims* d = &pb->dims;
    double2* walk = (double2*)st->walkers;
    { AFQ_PHASE("qr", s); AFQ_TRY(launch_qr(2 * d->n_walkers, d->norb, d->nocc, walk, walk, nullptr, s)); }
    AFQ_PHASE(green ? "green" : "overlap", s);
    return overlap_u(d, (const double2*)pb->mo_coeff, walk, (double2*)st->overlaps, green, u, s);
}

int check_problem_u(const afq_problem* pb) {
    if (!pb) return fail(AFQ_E_INVALID_ARGUMENT, "problem is NULL");
    AFQ_TRY(check_u(&pb->dims));
    if (!pb->chol || !pb->mo_coeff || !pb->exp_h1_half || !pb->mf_shifts || !pb->rot_h1 || !pb->rot_chol)
        return fail(AFQ_E_INVALID_ARGUMENT, "problem has a NULL member");
    if (!(pb->dt > 0.0)) return fail(AFQ_E_INVALID_ARGUMENT, "dt=%g must be > 0", pb->dt);
    return AFQ_OK;
}

int check_state_u(const afq_state* st) {
    if (!st || !st->walkers || !st->weights || !st->overlaps || !st->pop_control_ene_shift || !st->e_estimate)
        return fail(AFQ_E_INVALID_ARGUMENT, "state has a NULL member");
    return AFQ_OK;
}

// ---------------------------------------------------- generalized walkers
// A generalized walker is (2n x 2o): the up block of rows over the down
// block (meas/rhf.py:103-130).  With the block-diagonal trial
// C_g = [[C, 0], [0, C]], m = C_g^H W is the reference's vstack(C^H W_top,
// C^H W_bot), so the restricted Green's-function kernel at (2n, 2o) gives
// det(m) and G_half (2o x 2n).

__global__ void k_blockdiag_c(int n, int o, const double2* __restrict__ mo, double2* __restrict__ cg) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 4 * n * o) return;
    const int r = e / (2 * o), c = e % (2 * o);
    const bool top = r < n, left = c < o;
    cg[e] = top == left ? mo[(size_t)(top ? r : r - n) * o + (left ? c : c - o)] : make_double2(0.0, 0.0);
}

// g[w, a, j] = G[w, a, j] + G[w, o + a, n + j]  (the up-up plus down-down blocks of G_half)
__global__ void k_fold_g(int W, int n, int o, const double2* __restrict__ G, double2* __restrict__ g) {
    const long long total = (long long)W * o * n;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int w = (int)(e / ((long long)o * n));
        const int r = (int)(e % ((long long)o * n));
        const int a = r / n, j = r % n;
        const double2* Gw = G + (size_t)w * 4 * o * n;  // (2o x 2n)
        g[e] = cadd(Gw[(size_t)a * 2 * n + j], Gw[(size_t)(o + a) * 2 * n + n + j]);
    }
}

struct GWS {
    int* status;
    double2* cg;     // 2n x 2o
    double2* green;  // W x 2o x 2n
    double2* gsum;   // W x o x n
    double2* V;      // Wc x n x n
};

GWS layout_g(Arena& a, const afq_dims* d, int n_chunks) {
    const size_t W = d->n_walkers, n = d->norb, o = d->nocc;
    GWS g = {};
    g.status = a.take<int>(64);
    g.cg = a.take<double2>(4 * n * o);
    g.green = a.take<double2>(W * 4 * o * n);
    g.gsum = a.take<double2>(W * o * n);
    g.V = a.take<double2>((size_t)chunk_of(d->n_walkers, n_chunks) * n * n);
    return g;
}

int check_g(const afq_dims* d) {
    if (!d) return fail(AFQ_E_INVALID_ARGUMENT, "dims is NULL");
    if (d->n_walkers < 1 || d->norb < 1 || d->nocc < 1 || d->nocc > d->norb || d->nchol < 1)
        return fail(AFQ_E_INVALID_ARGUMENT, "bad dims W=%d n=%d o=%d G=%d", d->n_walkers, d->norb, d->nocc,
                    d->nchol);
    if (d->precision != AFQ_PREC_FP64) return fail(AFQ_E_UNSUPPORTED, "generalized walkers run the binary64 form");
    if (2 * d->nocc > 64) return fail(AFQ_E_UNSUPPORTED, "generalized walkers: 2 nocc = %d > 64", 2 * d->nocc);
    if (2 * d->n_walkers > 65535) return fail(AFQ_E_UNSUPPORTED, "generalized walkers: W=%d > 32767", d->n_walkers);
    return AFQ_OK;
}

int build_cg(const afq_dims* d, const double2* mo, const GWS& g, cudaStream_t s) {
    const int count = 4 * d->norb * d->nocc;
    k_blockdiag_c<<<(count + 255) / 256, 256, 0, s>>>(d->norb, d->nocc, mo, g.cg);
    AFQ_LAUNCHED("k_blockdiag_c");
    return AFQ_OK;
}

}  // namespace
}  // namespace afq

using namespace afq;

size_t afq_g_workspace(const afq_dims* d, int32_t n_chunks) {
    if (check_g(d) != AFQ_OK) return 0;
    Arena a;
    layout_g(a, d, n_chunks);
    return a.used;
}

int afq_overlap_g(const afq_dims* d, const double* mo_coeff, const double* walkers, double* overlaps,
                  void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_g(d));
    if (!mo_coeff || !walkers || !overlaps || !workspace) return fail(AFQ_E_INVALID_ARGUMENT, "NULL argument");
    Arena a(workspace, workspace_bytes);
    const GWS g = layout_g(a, d, 1);
    if (!a.ok()) return fail(AFQ_E_WORKSPACE, "workspace: %zu bytes < %zu", workspace_bytes, a.used);
    cudaStream_t s = as_stream(stream);
    AFQ_TRY(build_cg(d, (const double2*)mo_coeff, g, s));
    return launch_green_det(d->n_walkers, 2 * d->norb, 2 * d->nocc, g.cg, d->trial_is_real, (const double2*)walkers,
                            (double2*)overlaps, nullptr, s);
}

int afq_force_bias_g(const afq_dims* d, const double* mo_coeff, const double* rot_chol, const double* walkers,
                     double* force_bias, void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_g(d));
    if (!mo_coeff || !rot_chol || !walkers || !force_bias || !workspace)
        return fail(AFQ_E_INVALID_ARGUMENT, "NULL argument");
    Arena a(workspace, workspace_bytes);
    const GWS g = layout_g(a, d, 1);
    if (!a.ok()) return fail(AFQ_E_WORKSPACE, "workspace: %zu bytes < %zu", workspace_bytes, a.used);
    cudaStream_t s = as_stream(stream);
    const int W = d->n_walkers, n = d->norb, o = d->nocc, on = n * o;
    AFQ_TRY(build_cg(d, (const double2*)mo_coeff, g, s));
    AFQ_TRY(launch_green(W, 2 * n, 2 * o, g.cg, d->trial_is_real, (const double2*)walkers, nullptr, g.green, s));
    const long long total = (long long)W * on;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    k_fold_g<<<(unsigned)blocks, 256, 0, s>>>(W, n, o, g.green, g.gsum);
    AFQ_LAUNCHED("k_fold_g");
    return launch_zgemm(W, d->nchol, on, 1.0, g.gsum, on, rot_chol, on, !d->trial_is_real, true,
                        (double2*)force_bias, d->nchol, s);
}

int afq_apply_trotter_g(const afq_dims* d, int32_t n_terms, double sqrt_dt, int32_t n_chunks, const double* chol,
                        const double* exp_h1_half, const double* walkers, const double* shifted_fields,
                        double* walkers_out, void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_g(d));
    if (!chol || !exp_h1_half || !walkers || !shifted_fields || !walkers_out || !workspace)
        return fail(AFQ_E_INVALID_ARGUMENT, "NULL argument");
    if (n_terms < 0) return fail(AFQ_E_INVALID_ARGUMENT, "n_terms=%d < 0", n_terms);
    Arena a(workspace, workspace_bytes);
    const GWS g = layout_g(a, d, n_chunks);
    if (!a.ok()) return fail(AFQ_E_WORKSPACE, "workspace: %zu bytes < %zu", workspace_bytes, a.used);
    cudaStream_t s = as_stream(stream);
    const int W = d->n_walkers, n = d->norb, o = d->nocc, G = d->nchol;
    const int Wc = chunk_of(W, n_chunks);
    const double2* xs = (const double2*)shifted_fields;
    for (int w0 = 0; w0 < W; w0 += Wc) {
        const int wc = W - w0 < Wc ? W - w0 : Wc;
        AFQ_TRY(launch_zgemm(wc, n * n, G, 1.0, xs + (size_t)w0 * G, G, chol, (int64_t)n * n, false, false, g.V,
                             (int64_t)n * n, s));
        // the top and bottom n x 2o halves of each walker, both with the walker's V
        AFQ_TRY(launch_trotter(2 * wc, n, 2 * o, n_terms, sqrt_dt, exp_h1_half, g.V,
                               (const double2*)walkers + (size_t)w0 * 4 * n * o,
                               (double2*)walkers_out + (size_t)w0 * 4 * n * o, s, 2));
    }
    return AFQ_OK;
}

size_t afq_u_workspace(const afq_dims* d, int32_t n_chunks) {
    if (check_u(d) != AFQ_OK) return 0;
    Arena a;
    layout_u(a, d, n_chunks);
    return a.used;
}

int afq_overlap_u(const afq_dims* d, const double* mo_coeff, const double* walkers, double* overlaps,
                  void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_u(d));
    if (!mo_coeff || !walkers || !overlaps || !workspace) return fail(AFQ_E_INVALID_ARGUMENT, "NULL argument");
    Arena a(workspace, workspace_bytes);
    const UWS u = layout_u(a, d, 1);
    if (!a.ok()) return fail(AFQ_E_WORKSPACE, "workspace: %zu bytes < %zu", workspace_bytes, a.used);
    return overlap_u(d, (const double2*)mo_coeff, (const double2*)walkers, (double2*)overlaps, nullptr, u,
                     as_stream(stream));
}

int afq_force_bias_u(const afq_dims* d, const double* mo_coeff, const double* rot_chol, const double* walkers,
                     double* force_bias, void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_u(d));
    if (!mo_coeff || !rot_chol || !walkers || !force_bias || !workspace)
        return fail(AFQ_E_INVALID_ARGUMENT, "NULL argument");
    Arena a(workspace, workspace_bytes);
    const UWS u = layout_u(a, d, 1);
    if (!a.ok()) return fail(AFQ_E_WORKSPACE, "workspace: %zu bytes < %zu", workspace_bytes, a.used);
    cudaStream_t s = as_stream(stream);
    AFQ_TRY(launch_green(2 * d->n_walkers, d->norb, d->nocc, (const double2*)mo_coeff, d->trial_is_real,
                         (const double2*)walkers, nullptr, u.green, s));
    return force_bias_u(d, rot_chol, u, (double2*)force_bias, s);
}

int afq_energy_u(const afq_dims* d, double h0, const double* mo_coeff, const double* rot_h1, const double* rot_chol,
                 const double* walkers, double* energy, void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_u(d));
    if (!mo_coeff || !rot_h1 || !rot_chol || !walkers || !energy || !workspace)
        return fail(AFQ_E_INVALID_ARGUMENT, "NULL argument");
    Arena a(workspace, workspace_bytes);
    UWS u = layout_u(a, d, 1);
    if (!a.ok()) return fail(AFQ_E_WORKSPACE, "workspace: %zu bytes < %zu", workspace_bytes, a.used);
    cudaStream_t s = as_stream(stream);
    afq_problem pb = {};
    pb.dims = *d;
    pb.h0 = h0;
    pb.mo_coeff = mo_coeff;
    pb.rot_h1 = rot_h1;
    pb.rot_chol = rot_chol;
    AFQ_TRY(launch_green(2 * d->n_walkers, d->norb, d->nocc, (const double2*)mo_coeff, d->trial_is_real,
                         (const double2*)walkers, nullptr, u.green, s));
    u.energy = (double2*)energy;
    return energy_u(&pb, u, s);
}

int afq_apply_trotter_u(const afq_dims* d, int32_t n_terms, double sqrt_dt, int32_t n_chunks, const double* chol,
                        const double* exp_h1_half, const double* walkers, const double* shifted_fields,
                        double* walkers_out, void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_u(d));
    if (!chol || !exp_h1_half || !walkers || !shifted_fields || !walkers_out || !workspace)
        return fail(AFQ_E_INVALID_ARGUMENT, "NULL argument");
    if (n_terms < 0) return fail(AFQ_E_INVALID_ARGUMENT, "n_terms=%d < 0", n_terms);
    Arena a(workspace, workspace_bytes);
    const UWS u = layout_u(a, d, n_chunks);
    if (!a.ok()) return fail(AFQ_E_WORKSPACE, "workspace: %zu bytes < %zu", workspace_bytes, a.used);
    return trotter_u(d, n_terms, sqrt_dt, n_chunks, chol, exp_h1_half, (const double2*)walkers,
                     (const double2*)shifted_fields, (double2*)walkers_out, u.V, as_stream(stream));
}

int afq_stochastic_reconfiguration_u(const afq_dims* d, const double* weights, double zeta, const double* walkers,
                                     double* walkers_out, double* weights_out, int32_t* idx, void* workspace,
                                     size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_u(d));
    if (!weights || !walkers || !walkers_out || !weights_out || !workspace)
        return fail(AFQ_E_INVALID_ARGUMENT, "NULL argument");
    if (walkers == walkers_out) return fail(AFQ_E_INVALID_ARGUMENT, "walkers_out must not alias walkers");
    if (!(zeta >= 0.0 && zeta < 1.0)) return fail(AFQ_E_INVALID_ARGUMENT, "zeta=%g outside [0, 1)", zeta);
    Arena a(workspace, workspace_bytes);
    const UWS u = layout_u(a, d, 1);
    if (!a.ok()) return fail(AFQ_E_WORKSPACE, "workspace: %zu bytes < %zu", workspace_bytes, a.used);
    cudaStream_t s = as_stream(stream);
    const int W = d->n_walkers;
    const size_t half = (size_t)W * d->norb * d->nocc;
    AFQ_TRY(launch_sr_scan(W, weights, zeta, u.levels, u.idx, nullptr, u.avg, s));
    AFQ_TRY(launch_gather(W, (int64_t)d->norb * d->nocc, u.idx, (const double2*)walkers, (double2*)walkers_out,
                          u.avg, weights_out, s));
    AFQ_TRY(launch_gather(W, (int64_t)d->norb * d->nocc, u.idx, (const double2*)walkers + half,
                          (double2*)walkers_out + half, u.avg, nullptr, s));
    if (idx) AFQ_CUDA(cudaMemcpyAsync(idx, u.idx, sizeof(int32_t) * W, cudaMemcpyDeviceToDevice, s));
    return AFQ_OK;
}

int afq_step_u(const afq_problem* pb, const afq_params* p, const afq_state* st, const double* fields, uint64_t seed,
               uint64_t counter, void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_problem_u(pb));
    AFQ_TRY(check_state_u(st));
    if (!p || !workspace) return fail(AFQ_E_INVALID_ARGUMENT, "NULL params or workspace");
    Arena a(workspace, workspace_bytes);
    const UWS u = layout_u(a, &pb->dims, p->n_chunks);
    if (!a.ok()) return fail(AFQ_E_WORKSPACE, "workspace: %zu bytes < %zu", workspace_bytes, a.used);
    return step_u(pb, p, st, fields, seed, counter, u, as_stream(stream));
}

int afq_block_u(const afq_problem* pb, const afq_params* p, const afq_state* st, const double* fields, double zeta,
                uint64_t seed, uint64_t counter, double* block_energy, double* block_weight, int32_t* sr_idx,
                void* workspace, size_t workspace_bytes, void* stream) {
    AFQ_TRY(check_problem_u(pb));
    AFQ_TRY(check_state_u(st));
    if (!p || !workspace || !block_energy || !block_weight)
        return fail(AFQ_E_INVALID_ARGUMENT, "NULL params, outputs or workspace");
    Arena a(workspace, workspace_bytes);
    const UWS u = layout_u(a, &pb->dims, p->n_chunks);
    if (!a.ok()) return fail(AFQ_E_WORKSPACE, "workspace: %zu bytes < %zu", workspace_bytes, a.used);
    cudaStream_t s = as_stream(stream);
    const afq_dims* d = &pb->dims;
    const int W = d->n_walkers, G = d->nchol;
    const size_t half = (size_t)W * d->norb * d->nocc;
    // prop/blocks.py:38-57
    for (int i = 0; i < p->n_prop_steps; ++i) {
        AFQ_TRY(step_u(pb, p, st, fields ? fields + (size_t)i * W * G : nullptr, seed, counter + i, u, s));
        if (p->qr_every > 0 && (i + 1) % p->qr_every == 0 && i + 1 < p->n_prop_steps)
            AFQ_TRY(orthonormalize_u(pb, st, u, nullptr, s));
    }
    AFQ_TRY(orthonormalize_u(pb, st, u, u.green, s));
    // prop/blocks.py:59-79
    AFQ_TRY(energy_u(pb, u, s));
    AFQ_PHASE("block_measure", s);
    AFQ_TRY(launch_block_measure(W, p->dt, p->shift_ema, st->weights, u.energy, st->e_estimate,
                                 st->pop_control_ene_shift, block_energy, block_weight, s));
    // prop/blocks.py:81-92: one set of comb indices for both spins
    AFQ_PHASE("comb", s);
    if (zeta < 0.0) {
        AFQ_TRY(launch_philox(1, seed, counter + p->n_prop_steps, 0, u.zeta, s));
        AFQ_TRY(launch_sr_scan_dev(W, st->weights, u.zeta, u.levels, u.idx, u.avg, s));
    } else {
        AFQ_TRY(launch_sr_scan(W, st->weights, zeta, u.levels, u.idx, nullptr, u.avg, s));
    }
    AFQ_CUDA(cudaMemcpyAsync(u.wcopy, st->walkers, sizeof(double2) * 2 * half, cudaMemcpyDeviceToDevice, s));
    AFQ_CUDA(cudaMemcpyAsync(u.ocopy, st->overlaps, sizeof(double2) * W, cudaMemcpyDeviceToDevice, s));
    double2* walk = (double2*)st->walkers;
    const int64_t row = (int64_t)d->norb * d->nocc;
    AFQ_TRY(launch_gather(W, row, u.idx, u.wcopy, walk, u.avg, st->weights, s));
    AFQ_TRY(launch_gather(W, row, u.idx, u.wcopy + half, walk + half, u.avg, nullptr, s));
    AFQ_TRY(launch_gather(W, 1, u.idx, u.ocopy, (double2*)st->overlaps, u.avg, nullptr, s));
    if (sr_idx) AFQ_CUDA(cudaMemcpyAsync(sr_idx, u.idx, sizeof(int32_t) * W, cudaMemcpyDeviceToDevice, s));
    return AFQ_OK;
}
