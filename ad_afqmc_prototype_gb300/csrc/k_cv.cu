// Control-variate measurement of the exchange energy (afq_block_cv).
//
// Features and the exact-except-exchange energy of every walker come from
// the block-end Green's function and its Coulomb vectors c_g =
// tr(L~_g G_half^T) (the force-bias GEMM's output; the force bias of
// meas/rhf.py:27-33 is 2 c_g):
//   E_base = h0 + 2 Re tr(rot_h1 G_half) + 2 Re sum_g c_g^2,   E = E_base - X,
//   X = sum_g tr(f_g f_g)   (meas/rhf.py:36-50).
// The estimator samples walkers off + k stride (off uniform in [0, stride))
// and corrects the network's prediction on them (Horvitz-Thompson weight
// stride), so the block energy is unbiased for the exact one.
#include "afq_internal.cuh"

namespace afq {

constexpr int CV_BLOCKS = AFQ_CV_FEATURES - 4;

// One warp per walker, eight walkers per CTA.  fbm: (2W, ldf) fp32 c_g,
// Re rows w, Im rows W + w.  shift / scale (optional):
// standardised features for the network; else raw features.
__global__ void __launch_bounds__(256) k_cv_features(int W, int n, int o, int G, double h0,
                                                     const double2* __restrict__ green,
                                                     const double2* __restrict__ rot_h1,
                                                     const float* __restrict__ fbm, long long ldf,
                                                     const double2* __restrict__ ovlp,
                                                     const float* __restrict__ shift,
                                                     const float* __restrict__ scale, float* __restrict__ feat,
                                                     double* __restrict__ ebase) {
    __shared__ float blk[8][CV_BLOCKS];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * 8 + wid;
    for (int e = lane; e < CV_BLOCKS; e += 32) blk[wid][e] = 0.f;
    __syncwarp();
    if (w >= W) return;  // whole warp
    double cr = 0.0, ci = 0.0;
    for (int g = lane; g < G; g += 32) {
        const float a = fbm[(size_t)w * ldf + g], b = fbm[(size_t)(W + w) * ldf + g];
        cr += (double)a * a - (double)b * b;
        ci += 2.0 * (double)a * b;
        atomicAdd(&blk[wid][(int)((long long)g * CV_BLOCKS / G)], a * a + b * b);
    }
    const double2* Gw = green + (size_t)w * o * n;
    double er = 0.0;
    for (int e = lane; e < o * n; e += 32) {
        const double2 gv = Gw[e], r = rot_h1[e];
        er += gv.x * r.x - gv.y * r.y;
    }
    cr = warp_sum(cr);
    ci = warp_sum(ci);
    er = warp_sum(er);
    __syncwarp();
    float* fw = feat + (size_t)w * AFQ_CV_FEATURES;
    for (int f = lane; f < AFQ_CV_FEATURES; f += 32) {
        float x;
        if (f < CV_BLOCKS) {
            x = blk[wid][f];
        } else if (f == CV_BLOCKS) {
            x = (float)cr;
        } else if (f == CV_BLOCKS + 1) {
            x = (float)ci;
        } else if (f == CV_BLOCKS + 2) {
            x = (float)er;
        } else {
            const double2 ov = ovlp[w];
            const double m = sqrt(ov.x * ov.x + ov.y * ov.y);
            x = m > 0.0 ? (float)log(m) : -700.f;
        }
        if (shift) x = (x - shift[f]) * scale[f];
        fw[f] = x;
    }
    if (lane == 0) ebase[w] = h0 + 2.0 * er + 2.0 * cr;
}

int launch_cv_features(int W, int n, int o, int G, double h0, const double2* green, const double2* rot_h1,
                       const float* fbm, long long ldf, const double2* ovlp, const float* shift, const float* scale,
                       float* feat, double* ebase, cudaStream_t s) {
    if (W <= 0) return AFQ_OK;
    k_cv_features<<<(W + 7) / 8, 256, 0, s>>>(W, n, o, G, h0, green, rot_h1, fbm, ldf, ovlp, shift, scale, feat,
                                              ebase);
    AFQ_LAUNCHED("k_cv_features");
    return AFQ_OK;
}

// The sample's offset from the block's uniform u: off = floor(u stride).
__global__ void k_cv_pick(const double* __restrict__ u, int stride, int* __restrict__ off) {
    int v = (int)(u[0] * (double)stride);
    off[0] = v < 0 ? 0 : (v >= stride ? stride - 1 : v);
}

int launch_cv_pick(const double* u, int stride, int* off, cudaStream_t s) {
    k_cv_pick<<<1, 1, 0, s>>>(u, stride, off);
    AFQ_LAUNCHED("k_cv_pick");
    return AFQ_OK;
}

// Energy-GEMM rows of sampled walkers s0 .. s0 + sc - 1 (walker off + s
// stride; rows of walkers past W are zero): row (s_local 2 + part) P + k
// holds split(G_part[w, k, :]) (zero for k >= o), as k_green_rows.
__global__ void k_cv_green_rows(int sc, int s0, const int* __restrict__ off, int stride, int W, int n, int o, int P,
                                const double2* __restrict__ green, __nv_bfloat16* __restrict__ dst, int S, int Kt,
                                int sec) {
    const long long rows = (long long)sc * P * 2;
    const long long total = rows * (long long)Kt;
    const int o0 = off[0];
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / Kt;
        const int kk = (int)(e % Kt);
        __nv_bfloat16* row = dst + r * Kt;
        const int k = (int)(r % P), part = (int)((r / P) % 2), sl = (int)(r / (2 * P));
        const int w = o0 + (s0 + sl) * stride;
        if (kk < S) {
            double x = 0.0;
            if (kk < n && w < W && k < o) {
                const double2 v = green[((size_t)w * o + k) * n + kk];
                x = part ? v.y : v.x;
            }
            split_store(row, S, kk, x, false, sec);
        } else if (kk >= sec * S) {
            row[kk] = __double2bfloat16(0.0);
        }
    }
}

int launch_cv_green_rows(int sc, int s0, const int* off, int stride, int W, int n, int o, int P, const double2* green,
                         __nv_bfloat16* dst, int S, int Kt, int sec, cudaStream_t s) {
    const long long total = (long long)sc * P * 2 * Kt;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    k_cv_green_rows<<<(unsigned)blocks, 256, 0, s>>>(sc, s0, off, stride, W, n, o, P, green, dst, S, Kt, sec);
    AFQ_LAUNCHED("k_cv_green_rows");
    return AFQ_OK;
}

// Exact exchange of every walker from the exchange partials (record mode).
__global__ void k_cv_record(int W, int nchunk, const double2* __restrict__ partial, double* __restrict__ xout) {
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= W) return;
    double x = 0.0;
    for (int c = lane; c < nchunk; c += 32) x += partial[((size_t)w * nchunk + c) * 2 + 1].x;
    x = warp_sum(x);
    if (lane == 0) xout[w] = x;
}

int launch_cv_record(int W, int nchunk, const double2* partial, double* xout, cudaStream_t s) {
    if (W <= 0) return AFQ_OK;
    k_cv_record<<<(W + 7) / 8, 256, 0, s>>>(W, nchunk, partial, xout);
    AFQ_LAUNCHED("k_cv_record");
    return AFQ_OK;
}

// Block measurement with the control variate (prop/blocks.py:59-79 with the
// network's exchange for every walker and the sampled correction); one CTA.
__global__ void __launch_bounds__(1024) k_cv_measure(int W, double dt, double alpha, const double* __restrict__ weights,
                                                     const double* __restrict__ ebase, const float* __restrict__ ynn,
                                                     double y_shift, double y_scale, int m_max, int stride,
                                                     const int* __restrict__ off, int nchunk,
                                                     const double2* __restrict__ partial,
                                                     const double* __restrict__ e_est, double* pop_shift,
                                                     double* block_energy, double* block_weight,
                                                     double2* __restrict__ energy, double* __restrict__ stats) {
    const double eref = e_est[0];
    const double thresh = sqrt(2.0 / dt);
    double sw = 0.0, swp = 0.0, corr = 0.0, cnt = 0.0;
    for (int w = threadIdx.x; w < W; w += blockDim.x) {
        double e = ebase[w] - (y_shift + y_scale * (double)ynn[w]);
        energy[w] = make_double2(e, 0.0);
        if (fabs(e - eref) > thresh) e = eref;
        const double wt = weights[w];
        sw += wt;
        swp += wt * e;
    }
    const int o0 = off[0];
    for (int sidx = threadIdx.x; sidx < m_max; sidx += blockDim.x) {
        const int w = o0 + sidx * stride;
        if (w >= W) continue;
        double x = 0.0;
        for (int c = 0; c < nchunk; ++c) x += partial[((size_t)sidx * nchunk + c) * 2 + 1].x;
        double ee = ebase[w] - x, ep = ebase[w] - (y_shift + y_scale * (double)ynn[w]);
        if (fabs(ee - eref) > thresh) ee = eref;
        if (fabs(ep - eref) > thresh) ep = eref;
        corr += weights[w] * (ee - ep);
        cnt += 1.0;
    }
    __shared__ double r[4][32];
    sw = warp_sum(sw); swp = warp_sum(swp); corr = warp_sum(corr); cnt = warp_sum(cnt);
    if ((threadIdx.x & 31) == 0) {
        r[0][threadIdx.x >> 5] = sw; r[1][threadIdx.x >> 5] = swp;
        r[2][threadIdx.x >> 5] = corr; r[3][threadIdx.x >> 5] = cnt;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const bool ok = threadIdx.x < (blockDim.x >> 5);
        double a = ok ? r[0][threadIdx.x] : 0.0, b = ok ? r[1][threadIdx.x] : 0.0;
        double c = ok ? r[2][threadIdx.x] : 0.0, d = ok ? r[3][threadIdx.x] : 0.0;
        a = warp_sum(a); b = warp_sum(b); c = warp_sum(c); d = warp_sum(d);
        if (threadIdx.x == 0) {
            const double num = b + (double)stride * c;
            double eb = num / (a == 0.0 ? 1.0 : a);
            if (a == 0.0) eb = eref;
            block_energy[0] = eb;
            block_weight[0] = a;
            pop_shift[0] = (1.0 - alpha) * pop_shift[0] + alpha * eb;
            if (stats) {
                stats[0] = b;
                stats[1] = (double)stride * c;
                stats[2] = a;
                stats[3] = d;
            }
        }
    }
}

int launch_cv_measure(int W, double dt, double alpha, const double* weights, const double* ebase, const float* ynn,
                      double y_shift, double y_scale, int m_max, int stride, const int* off, int nchunk,
                      const double2* partial, const double* e_est, double* pop_shift, double* block_energy,
                      double* block_weight, double2* energy, double* stats, cudaStream_t s) {
    k_cv_measure<<<1, 1024, 0, s>>>(W, dt, alpha, weights, ebase, ynn, y_shift, y_scale, m_max, stride, off, nchunk,
                                    partial, e_est, pop_shift, block_energy, block_weight, energy, stats);
    AFQ_LAUNCHED("k_cv_measure");
    return AFQ_OK;
}

}  // namespace afq
