// Unrestricted walkers with the RHF trial (walker_kind "unrestricted"):
// kernels and extern "C" entry points of the binary64 step and block.
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
                                st->pop_control_ene_shift, st->e_estimate, s);
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

}  // namespace
}  // namespace afq

using namespace afq;

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
