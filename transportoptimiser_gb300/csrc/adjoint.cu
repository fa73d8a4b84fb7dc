// adjoint.cu - pathwise sensitivities of the controlled road valuation with
// the exercise policy frozen (no counterpart in the reference, which only
// estimates values).
//
// The frozen-policy model, per path p and year t = 0..Y-1, control c_{p,t}
// fixed (e.g. the optimal controls of a forward LSM pass):
//   exogenous processes (forwardPathKernel, SimulateGPU.cu:930-952)
//     U_{t+1} = U_t + theta (mu - U_t) dt + U_t sigma z_t + (e^{j_t} - 1) U_t J_t
//   unit profit (as the ROV's, SimulateGPU.cu:2375-2420)
//     pi_t = (unit_cost + sum_f fuel_f U_f - revenue sum_c ore_c U_{nF+c}) U_demand
//   PV = sum_t (1 + rrr dt / 100)^-t flows[c_t] pi_t
//   per species s: growth-rate mean g (mteKernel :691-701), migration with
//   the control's matrix M_c (survival exp(-crossings * hazard_c) inside),
//   corrected logistic growth x' = max(m (1 + gr (cap - m) / cap), 0) with
//   gr = g (1 + v z), and end population E_s = sum_k x_Y[k].
// Parameters theta (2U + 2S + C): reversion theta_u, volatility sigma_u,
// growth-rate mean mu_s (params[1]), growth variability v_s (params[7]),
// crossing hazard h_c (scales entry (k, l) of M_c by exp(-cross_lk dh_c)).
// Outputs: E[PV], E[E_s].
//
// Forward: PV per path (one thread per path) and the population recursion
// (one lane per path, states [patch][lane] in shared memory) with the
// states checkpointed every K years.  Backward (vector-Jacobian product):
// forward tangents for the scalar recursions (OU, growth-rate mean), and a
// reverse sweep for the patch populations: each K-year segment is
// recomputed from its checkpoint, then lambda_t = M_c^T (lambda_{t+1} .
// dF/dm) with the parameter terms accumulated on the way.  Per-path
// contributions are averaged in FP64.
#include <cmath>
#include <vector>

#include "to_internal.cuh"

namespace {

constexpr int kCk = 10;                 // checkpoint interval (years)

struct AdjArgs {
    int P, Y, S, C, U, NP, nF, Cm, demand_idx, road;
    float dt, rrr, unit_cost, unit_revenue;
    uint64_t seed;
    const float* theta;                 // [2U + 2S + C] device
    const float* uncert;                // [U][6]
    const float* flows;                 // [C]
    const float* fuel_costs;            // [nF]
    const int* fuel_idx;                // [nF]
    const float* ore_content;           // [Cm]
    const float* ore_sd;                // [Cm]
    const int* controls;                // [Y][P]
    const int* n_patches;               // [S]
    const float* params;                // [S][8]
    const float* init_pops;             // [S][NP]
    const float* caps;                  // [S][NP]
    const int* coo_off;                 // [S*C + 1] entries of matrix (s, c)
    const int* coo_k;                   // destination
    const int* coo_l;                   // source
    const float* coo_v;                 // value at the base hazards
    const float* coo_x;                 // crossings of the pair
    const float* base_h;                // [C] hazards the values were built with
    // tape
    float* ckpt;                        // [S][Y/K + 1][NP][P]
    float* seg;                         // [S][K][NP][P]
    float* gtab;                        // [S][Y][P] growth-rate mean used in year t
    float* gdot;                        // [S][Y][P] its derivative in mu_s
    double* pv;                         // [P]
    double* endp;                       // [S][P]
    double* gpath;                      // [P][ntheta] per-path vector-Jacobian products
    const float* gout;                  // [1 + S] output weights
};

__device__ __forceinline__ float th_theta(const AdjArgs& a, int u) { return a.theta[u]; }
__device__ __forceinline__ float th_sigma(const AdjArgs& a, int u) { return a.theta[a.U + u]; }
__device__ __forceinline__ float th_mu(const AdjArgs& a, int s) { return a.theta[2 * a.U + s]; }
__device__ __forceinline__ float th_v(const AdjArgs& a, int s) { return a.theta[2 * a.U + a.S + s]; }
__device__ __forceinline__ float th_h(const AdjArgs& a, int c) { return a.theta[2 * a.U + 2 * a.S + c]; }

__device__ __forceinline__ float ore_at(const AdjArgs& a, int p, int t, int c) {
    const long f = (long)c * a.Y * a.P + (long)p * a.Y + t;
    const float z = to_normal1(a.seed, TO_STREAM_ORE, (uint32_t)a.road, (uint32_t)(f >> 2), 0,
                               (uint32_t)(f & 3));
    return a.ore_content[c] + a.ore_sd[c] * z;
}

// OU paths with optional tangents (dU/dtheta_u, dU/dsigma_u) and the PV and
// its gradient.  mode 0: PV only; mode 1: gradient terms weighted by w.
__device__ void exog_path(const AdjArgs& a, int p, bool tangents, double* pv_out, float* gth,
                          float* gsg) {
    constexpr int UMAX = 8;
    float U[UMAX], dth[UMAX], dsg[UMAX];
    for (int u = 0; u < a.U; ++u) { U[u] = a.uncert[6 * u]; dth[u] = 0.0f; dsg[u] = 0.0f; gth[u] = 0.0f; gsg[u] = 0.0f; }
    double pv = 0.0;
    float disc = 1.0f;
    const float dfac = 1.0f / (1.0f + a.rrr * a.dt / 100.0f);   // rrr in percent, as the ROV
    for (int t = 0; t < a.Y; ++t) {
        // unit profit at U_t and its partials
        float uf = 0.0f, ore = 0.0f;
        float dpi_du[UMAX];
        for (int u = 0; u < a.U; ++u) dpi_du[u] = 0.0f;
        for (int f = 0; f < a.nF; ++f) uf = fmaf(a.fuel_costs[f], U[a.fuel_idx[f]], uf);
        float oc[UMAX];
        for (int c = 0; c < a.Cm; ++c) {
            oc[c] = ore_at(a, p, t, c);
            ore = fmaf(oc[c], U[a.nF + c], ore);
        }
        const float base = (a.unit_cost + uf) - a.unit_revenue * ore;
        const float dem = a.demand_idx >= 0 ? U[a.demand_idx] : 1.0f;
        const float pi = base * dem;
        const int ctl = a.controls[(size_t)t * a.P + p];
        const float w = disc * a.flows[ctl];
        pv += (double)(w * pi);
        if (tangents) {
            for (int f = 0; f < a.nF; ++f) dpi_du[a.fuel_idx[f]] += a.fuel_costs[f] * dem;
            for (int c = 0; c < a.Cm; ++c) dpi_du[a.nF + c] += -a.unit_revenue * oc[c] * dem;
            if (a.demand_idx >= 0) dpi_du[a.demand_idx] += base;
            for (int u = 0; u < a.U; ++u) {
                gth[u] += w * dpi_du[u] * dth[u];
                gsg[u] += w * dpi_du[u] * dsg[u];
            }
        }
        // advance the processes to t + 1
        for (int u = 0; u < a.U; ++u) {
            const float* up = a.uncert + 6 * u;
            const float uj = to_uniform1(a.seed, TO_STREAM_EX_JUMP, (uint32_t)a.road, p, t, u);
            const float zb = to_normal1(a.seed, TO_STREAM_EX_BROWNIAN, (uint32_t)a.road, p, t, u);
            const float zj = to_normal1(a.seed, TO_STREAM_EX_JUMPSIZE, (uint32_t)a.road, p, t, u);
            const float jump = (uj < up[5]) ? 1.0f : 0.0f;
            const float s4 = up[4] * up[4];
            const float jf = (to_expf(zj * up[4] - s4 / 2.0f) - 1.0f) * jump;
            const float th = th_theta(a, u), sg = th_sigma(a, u);
            const float cur = U[u];
            const float mult = 1.0f - th * a.dt + sg * zb + jf;
            if (tangents) {
                dth[u] = dth[u] * mult + (up[1] - cur) * a.dt;
                dsg[u] = dsg[u] * mult + cur * zb;
            }
            U[u] = cur + th * (up[1] - cur) * a.dt + cur * (zb * sg) + jf * cur;
        }
        disc *= dfac;
    }
    *pv_out = pv;
}

__global__ void k_adj_pv(AdjArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.P) return;
    float gth[8], gsg[8];
    double pv;
    exog_path(a, p, false, &pv, gth, gsg);
    a.pv[p] = pv;
}

__global__ void k_adj_pv_grad(AdjArgs a, int ntheta) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.P) return;
    float gth[8], gsg[8];
    double pv;
    exog_path(a, p, true, &pv, gth, gsg);
    const float w = a.gout[0];
    double* g = a.gpath + (size_t)p * ntheta;
    for (int u = 0; u < a.U; ++u) {
        g[u] = (double)(w * gth[u]);
        g[a.U + u] = (double)(w * gsg[u]);
    }
}

// growth-rate mean of species s in year t (updated before the year's
// growth) and its derivative in mu_s, for every year
__device__ void growth_means(const AdjArgs& a, int s, int p) {
    const float* sp = a.params + 8 * s;
    const float mu = th_mu(a, s);
    float g = sp[0], gd = 0.0f;
    for (int t = 0; t < a.Y; ++t) {
        const float uj = to_uniform1(a.seed, TO_STREAM_SP_JUMP, (uint32_t)a.road, p, t, s);
        const float zb = to_normal1(a.seed, TO_STREAM_SP_BROWNIAN, (uint32_t)a.road, p, t, s);
        const float zj = to_normal1(a.seed, TO_STREAM_SP_JUMPSIZE, (uint32_t)a.road, p, t, s);
        const float jump = (uj < sp[6]) ? 1.0f : 0.0f;
        const float s5 = sp[5] * sp[5];
        const float jf = (to_expf(zj * sp[5] - s5 / 2.0f) - 1.0f) * jump;
        const float mult = 1.0f - sp[4] * a.dt + zb * sp[2] + jf;
        gd = gd * mult + sp[4] * a.dt;
        g = g + sp[4] * (mu - g) * a.dt + g * (zb * sp[2]) + jf * g;
        a.gtab[((size_t)s * a.Y + t) * a.P + p] = g;
        a.gdot[((size_t)s * a.Y + t) * a.P + p] = gd;
    }
}

// migration m = M_c x for the lane's control (branch-free over controls)
__device__ __forceinline__ void migrate(const AdjArgs& a, int s, int ctl, int N, int TP,
                                        const float* x, float* m, const float* hscale) {
    const int lane = threadIdx.x;
    for (int k = 0; k < N; ++k) m[k * TP + lane] = 0.0f;
    for (int c = 0; c < a.C; ++c) {
        const float sel = (ctl == c) ? 1.0f : 0.0f;
        const float dh = hscale[c];
        const int e0 = a.coo_off[s * a.C + c], e1 = a.coo_off[s * a.C + c + 1];
        for (int e = e0; e < e1; ++e) {
            const int k = a.coo_k[e], l = a.coo_l[e];
            const float v = a.coo_v[e] * (dh == 0.0f ? 1.0f : to_expf(-a.coo_x[e] * dh)) * sel;
            m[k * TP + lane] = fmaf(v, x[l * TP + lane], m[k * TP + lane]);
        }
    }
}

__device__ __forceinline__ float growth_z(const AdjArgs& a, int s, int N, int p, int t, int k) {
    const int N4 = (N + 3) & ~3;
    float z[4];
    to_normal4(a.seed, TO_STREAM_GROWTH, (uint32_t)a.road, (uint32_t)p, t,
               (uint32_t)((s * N4) >> 2) + (uint32_t)(k >> 2), z);
    return z[k & 3];
}

// forward population recursion of one path tile; checkpoints every K years
// into ckpt (and, when seg_from >= 0, the states of years seg_from ..
// seg_from + K - 1 into seg)
__device__ void pop_forward(const AdjArgs& a, int s, int TP, float* x, float* m, int t_from,
                            int t_to, bool write_ckpt, bool write_seg, int seg_from,
                            const float* hscale) {
    const int lane = threadIdx.x, p = blockIdx.x * TP + lane;
    const int N = a.n_patches[s];
    const bool live = p < a.P;
    const int pp = live ? p : 0;
    const float v = th_v(a, s);
    const float* cp = a.caps + (size_t)s * a.NP;
    for (int t = t_from; t < t_to; ++t) {
        if (write_ckpt && t % kCk == 0 && live)
            for (int k = 0; k < N; ++k)
                a.ckpt[(((size_t)s * (a.Y / kCk + 1) + t / kCk) * a.NP + k) * a.P + p] = x[k * TP + lane];
        if (write_seg && live)
            for (int k = 0; k < N; ++k)
                a.seg[(((size_t)s * kCk + (t - seg_from)) * a.NP + k) * a.P + p] = x[k * TP + lane];
        const int ctl = live ? a.controls[(size_t)t * a.P + p] : 0;
        migrate(a, s, ctl, N, TP, x, m, hscale);
        const float g = a.gtab[((size_t)s * a.Y + t) * a.P + pp];
        for (int k = 0; k < N; ++k) {
            const float z = growth_z(a, s, N, pp, t, k);
            const float gr = fmaf(v * z, g, g);
            const float mv = m[k * TP + lane], c = cp[k];
            x[k * TP + lane] = fmaxf(mv * (1.0f + gr * (c - mv) / c), 0.0f);
        }
    }
}

// forward: end population per path and checkpoints
__global__ void k_adj_pop_fwd(AdjArgs a, int TP) {
    extern __shared__ float sm[];
    const int s = blockIdx.y, lane = threadIdx.x, p = blockIdx.x * TP + lane;
    const int N = a.n_patches[s];
    float* x = sm;                   // [N][TP]
    float* m = x + (size_t)N * TP;   // [N][TP]
    __shared__ float hscale[8];
    if (lane < a.C) hscale[lane] = th_h(a, lane) - a.base_h[lane];
    if (p < a.P) growth_means(a, s, p);
    const float* ip = a.init_pops + (size_t)s * a.NP;
    for (int k = 0; k < N; ++k) x[k * TP + lane] = ip[k];
    __syncthreads();
    pop_forward(a, s, TP, x, m, 0, a.Y, true, false, 0, hscale);
    if (p < a.P) {
        double e = 0.0;
        for (int k = 0; k < N; ++k) e += (double)x[k * TP + lane];
        a.endp[(size_t)s * a.P + p] = e;
    }
}

// backward: reverse sweep over the K-year segments
__global__ void k_adj_pop_bwd(AdjArgs a, int TP, int ntheta) {
    extern __shared__ float sm[];
    const int s = blockIdx.y, lane = threadIdx.x, p = blockIdx.x * TP + lane;
    // the sweep is linear in the species' output weight: a zero weight
    // contributes exactly zero (the per-path gradients start zeroed)
    if (a.gout[1 + s] == 0.0f) return;
    const int N = a.n_patches[s];
    const bool live = p < a.P;
    const int pp = live ? p : 0;
    float* x = sm;                       // [N][TP] state
    float* m = x + (size_t)N * TP;       // [N][TP] migrated state
    float* lam = m + (size_t)N * TP;     // [N][TP] adjoint of the state
    __shared__ float hscale[8];
    if (lane < a.C) hscale[lane] = th_h(a, lane) - a.base_h[lane];
    __syncthreads();
    const float v = th_v(a, s);
    const float* cp = a.caps + (size_t)s * a.NP;
    const float w = a.gout[1 + s];
    for (int k = 0; k < N; ++k) lam[k * TP + lane] = w;
    float g_mu = 0.0f, g_v = 0.0f, g_h[8];
    for (int c = 0; c < 8; ++c) g_h[c] = 0.0f;
    const int nseg = (a.Y + kCk - 1) / kCk;
    for (int sg = nseg - 1; sg >= 0; --sg) {
        const int t0 = sg * kCk, t1 = min(a.Y, t0 + kCk);
        // recompute the segment's states from its checkpoint
        for (int k = 0; k < N; ++k)
            x[k * TP + lane] = live ? a.ckpt[(((size_t)s * (a.Y / kCk + 1) + sg) * a.NP + k) * a.P + p] : 0.0f;
        pop_forward(a, s, TP, x, m, t0, t1, false, true, t0, hscale);
        for (int t = t1 - 1; t >= t0; --t) {
            // state x_t
            for (int k = 0; k < N; ++k)
                x[k * TP + lane] = live ? a.seg[(((size_t)s * kCk + (t - t0)) * a.NP + k) * a.P + p] : 0.0f;
            const int ctl = live ? a.controls[(size_t)t * a.P + p] : 0;
            migrate(a, s, ctl, N, TP, x, m, hscale);
            const float g = a.gtab[((size_t)s * a.Y + t) * a.P + pp];
            const float gd = a.gdot[((size_t)s * a.Y + t) * a.P + pp];
            // through the growth: mu_t = lambda * dF/dm (kept in m), params
            for (int k = 0; k < N; ++k) {
                const float z = growth_z(a, s, N, pp, t, k);
                const float gr = fmaf(v * z, g, g);
                const float mv = m[k * TP + lane], c = cp[k];
                const float f = mv * (1.0f + gr * (c - mv) / c);
                const float l = lam[k * TP + lane];
                float dfdm = 0.0f, dfdgr = 0.0f;
                if (f > 0.0f) {
                    dfdm = 1.0f + gr * (c - 2.0f * mv) / c;
                    dfdgr = mv * (c - mv) / c;
                }
                const float lg = l * dfdgr;
                g_v += lg * g * z;
                g_mu += lg * (1.0f + v * z) * gd;
                m[k * TP + lane] = l * dfdm;
            }
            // hazards and lambda_t = M_c^T mu_t
            for (int k = 0; k < N; ++k) lam[k * TP + lane] = 0.0f;
            for (int c = 0; c < a.C; ++c) {
                const float sel = (ctl == c) ? 1.0f : 0.0f;
                const float dh = hscale[c];
                const int e0 = a.coo_off[s * a.C + c], e1 = a.coo_off[s * a.C + c + 1];
                float gh = 0.0f;
                for (int e = e0; e < e1; ++e) {
                    const int k = a.coo_k[e], l = a.coo_l[e];
                    const float val = a.coo_v[e] * (dh == 0.0f ? 1.0f : to_expf(-a.coo_x[e] * dh)) * sel;
                    const float mu_k = m[k * TP + lane];
                    lam[l * TP + lane] = fmaf(val, mu_k, lam[l * TP + lane]);
                    gh = fmaf(-a.coo_x[e] * val * mu_k, x[l * TP + lane], gh);
                }
                g_h[c] += gh;
            }
        }
    }
    if (live) {
        double* gp = a.gpath + (size_t)p * ntheta;
        // species blocks are disjoint, so each species writes its own entries
        gp[2 * a.U + s] = (double)g_mu;
        gp[2 * a.U + a.S + s] = (double)g_v;
        for (int c = 0; c < a.C; ++c) atomicAdd(&gp[2 * a.U + 2 * a.S + c], (double)g_h[c]);
    }
}

// mean over paths of column j of a [P][ncol] array (FP64), one CTA per column
__global__ void k_col_mean(int P, int ncol, const double* __restrict__ v, double* out) {
    const int j = blockIdx.x;
    double s = 0.0;
    for (int p = threadIdx.x; p < P; p += blockDim.x) s += v[(size_t)p * ncol + j];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ double w[32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += w[i];
        out[j] = t / (double)P;
    }
}

int tile_paths(int N) { return N <= 128 ? 128 : (N <= 256 ? 64 : 32); }

}  // namespace

// ---- tape and C ABI ---------------------------------------------------------
struct to_tape_s {
    to_ctx ctx = nullptr;
    AdjArgs a;
    int ntheta = 0, nout = 0, maxN = 0;
    char* buf = nullptr;
    double* d_out = nullptr;            // [1 + S] forward outputs
    double* d_grad = nullptr;           // [ntheta] backward result
    double outputs[16];
};

extern "C" {

to_status to_adjoint_forward(to_ctx ctx, const to_adjoint_problem* pr, const double* theta,
                             double* outputs, to_tape* tape_out) {
    if (!ctx || !pr || !pr->rov || !theta || !outputs) return TO_ERR_INVALID;
    const to_rov_problem* rp = pr->rov;
    const int S = rp->n_species, C = rp->n_controls, U = rp->n_uncertainties;
    const int P = rp->n_paths, Y = rp->n_years;
    if (S <= 0 || S > 8 || C <= 0 || C > 8 || U < 0 || U > 8 || P <= 0 || Y <= 0 ||
        rp->n_commodities > 8 || !pr->controls || !pr->crossings || !pr->hazard)
        return TO_ERR_INVALID;
    const int ntheta = 2 * U + 2 * S + C;
    for (int i = 0; i < ntheta; ++i)
        if (!std::isfinite(theta[i])) return to_set_error(ctx, TO_ERR_NONFINITE, "theta %d", i);
    cudaSetDevice(ctx->device);
    int maxN = 4;
    for (int s = 0; s < S; ++s) {
        const int N = rp->species[s].n_patches;
        if (N <= 0 || N > 512) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "patches %d", N);
        if (N > maxN) maxN = N;
    }
    const int NP = (maxN + 3) & ~3;
    // COO lists of every (species, control) matrix with the pair's crossings
    std::vector<int> off(1, 0), kk, ll;
    std::vector<float> vv, xx;
    for (int s = 0; s < S; ++s) {
        const to_rov_species& sp = rp->species[s];
        const int N = sp.n_patches;
        for (int c = 0; c < C; ++c) {
            for (int k = 0; k < N; ++k)
                for (int l = 0; l < N; ++l) {
                    const float v = sp.mmm[((size_t)c * N + k) * N + l];
                    if (v == 0.0f) continue;
                    kk.push_back(k); ll.push_back(l); vv.push_back(v);
                    xx.push_back((float)pr->crossings[s][(size_t)l * N + k]);
                }
            off.push_back((int)kk.size());
        }
    }
    const size_t nnz = kk.size() > 0 ? kk.size() : 1;
    std::vector<int> np(S);
    std::vector<float> prm((size_t)S * 8), ip((size_t)S * NP, 0.0f), cpv((size_t)S * NP, 1.0f);
    for (int s = 0; s < S; ++s) {
        const to_rov_species& sp = rp->species[s];
        np[s] = sp.n_patches;
        for (int q = 0; q < 8; ++q) prm[(size_t)s * 8 + q] = sp.params[q];
        for (int k = 0; k < sp.n_patches; ++k) { ip[(size_t)s * NP + k] = sp.init_pops[k]; cpv[(size_t)s * NP + k] = sp.caps[k]; }
    }
    std::vector<float> th(ntheta), bh(C);
    for (int i = 0; i < ntheta; ++i) th[i] = (float)theta[i];
    for (int c = 0; c < C; ++c) bh[c] = (float)pr->hazard[c];
    // one allocation holds inputs and tape
    size_t bytes = 0;
    auto acc = [&](size_t b) { bytes += to_align256(b); };
    acc(ntheta * 4); acc((size_t)U * 24 + 4); acc(C * 4); acc(64); acc(64); acc(64); acc(64);
    acc((size_t)Y * P * 4); acc(S * 4); acc((size_t)S * 32); acc((size_t)S * NP * 4);
    acc((size_t)S * NP * 4); acc(off.size() * 4); acc(nnz * 4); acc(nnz * 4); acc(nnz * 4);
    acc(nnz * 4); acc(C * 4);
    acc((size_t)S * (Y / kCk + 1) * NP * P * 4); acc((size_t)S * kCk * NP * P * 4);
    acc((size_t)S * Y * P * 4); acc((size_t)S * Y * P * 4); acc((size_t)P * 8);
    acc((size_t)S * P * 8); acc((size_t)P * ntheta * 8); acc(64); acc(256); acc(256);
    to_tape t = new to_tape_s();
    t->ctx = ctx;
    cudaError_t e = cudaMalloc(&t->buf, bytes);
    if (e != cudaSuccess) { delete t; return to_check_cuda(ctx, e, "adjoint tape"); }
    char* q = t->buf;
    auto take = [&](size_t b) { char* r = q; q += to_align256(b); return r; };
    AdjArgs& a = t->a;
    memset(&a, 0, sizeof(a));
    a.P = P; a.Y = Y; a.S = S; a.C = C; a.U = U; a.NP = NP; a.nF = rp->n_fuels;
    a.Cm = rp->n_commodities; a.demand_idx = rp->demand_idx; a.road = rp->road;
    a.dt = rp->dt; a.rrr = rp->rrr; a.unit_cost = rp->unit_cost; a.unit_revenue = rp->unit_revenue;
    a.seed = rp->seed;
    float* d_th = (float*)take(ntheta * 4);
    float* d_unc = (float*)take((size_t)U * 24 + 4);
    float* d_fl = (float*)take(C * 4);
    float* d_fc = (float*)take(64); int* d_fi = (int*)take(64);
    float* d_oc = (float*)take(64); float* d_os = (float*)take(64);
    int* d_ctl = (int*)take((size_t)Y * P * 4);
    int* d_np = (int*)take(S * 4);
    float* d_prm = (float*)take((size_t)S * 32);
    float* d_ip = (float*)take((size_t)S * NP * 4);
    float* d_cp = (float*)take((size_t)S * NP * 4);
    int* d_off = (int*)take(off.size() * 4);
    int* d_k = (int*)take(nnz * 4); int* d_l = (int*)take(nnz * 4);
    float* d_v = (float*)take(nnz * 4); float* d_x = (float*)take(nnz * 4);
    float* d_bh = (float*)take(C * 4);
    a.ckpt = (float*)take((size_t)S * (Y / kCk + 1) * NP * P * 4);
    a.seg = (float*)take((size_t)S * kCk * NP * P * 4);
    a.gtab = (float*)take((size_t)S * Y * P * 4);
    a.gdot = (float*)take((size_t)S * Y * P * 4);
    a.pv = (double*)take((size_t)P * 8);
    a.endp = (double*)take((size_t)S * P * 8);
    a.gpath = (double*)take((size_t)P * ntheta * 8);
    float* d_gout = (float*)take(64);
    double* d_out = (double*)take(256);
    t->d_out = d_out;
    t->d_grad = (double*)take(256);
    a.theta = d_th; a.uncert = d_unc; a.flows = d_fl; a.fuel_costs = d_fc; a.fuel_idx = d_fi;
    a.ore_content = d_oc; a.ore_sd = d_os; a.controls = d_ctl; a.n_patches = d_np;
    a.params = d_prm; a.init_pops = d_ip; a.caps = d_cp; a.coo_off = d_off; a.coo_k = d_k;
    a.coo_l = d_l; a.coo_v = d_v; a.coo_x = d_x; a.base_h = d_bh; a.gout = d_gout;
    auto h2d = [&](void* d, const void* h, size_t b) {
        return b ? cudaMemcpyAsync(d, h, b, cudaMemcpyHostToDevice, ctx->stream) : cudaSuccess;
    };
    cudaError_t ce = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (ce == cudaSuccess) ce = x; };
    chk(h2d(d_th, th.data(), ntheta * 4));
    chk(h2d(d_unc, rp->uncert, (size_t)U * 24));
    chk(h2d(d_fl, rp->flows, C * 4));
    chk(h2d(d_fc, rp->fuel_costs, (size_t)rp->n_fuels * 4));
    chk(h2d(d_fi, rp->fuel_idx, (size_t)rp->n_fuels * 4));
    chk(h2d(d_oc, rp->ore_content, (size_t)rp->n_commodities * 4));
    chk(h2d(d_os, rp->ore_sd, (size_t)rp->n_commodities * 4));
    chk(h2d(d_ctl, pr->controls, (size_t)Y * P * 4));
    chk(h2d(d_np, np.data(), S * 4));
    chk(h2d(d_prm, prm.data(), prm.size() * 4));
    chk(h2d(d_ip, ip.data(), ip.size() * 4));
    chk(h2d(d_cp, cpv.data(), cpv.size() * 4));
    chk(h2d(d_off, off.data(), off.size() * 4));
    chk(h2d(d_k, kk.data(), kk.size() * 4));
    chk(h2d(d_l, ll.data(), ll.size() * 4));
    chk(h2d(d_v, vv.data(), vv.size() * 4));
    chk(h2d(d_x, xx.data(), xx.size() * 4));
    chk(h2d(d_bh, bh.data(), C * 4));
    if (ce != cudaSuccess) { cudaFree(t->buf); delete t; return to_check_cuda(ctx, ce, "adjoint inputs"); }
    t->ntheta = ntheta; t->nout = 1 + S; t->maxN = maxN;
    // forward
    k_adj_pv<<<(P + 127) / 128, 128, 0, ctx->stream>>>(a);
    const int TP = tile_paths(maxN);
    const size_t smf = (size_t)2 * maxN * TP * 4;
    cudaFuncSetAttribute(k_adj_pop_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smf);
    to_prof_begin(ctx, "adjoint_forward");
    k_adj_pop_fwd<<<dim3((P + TP - 1) / TP, S), TP, smf, ctx->stream>>>(a, TP);
    to_prof_end(ctx);
    k_col_mean<<<1, 256, 0, ctx->stream>>>(P, 1, a.pv, d_out);
    for (int s = 0; s < S; ++s)
        k_col_mean<<<1, 256, 0, ctx->stream>>>(P, 1, a.endp + (size_t)s * P, d_out + 1 + s);
    ctx->launches += 3 + S;
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(t->outputs, d_out, (size_t)(1 + S) * 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
    if (ce != cudaSuccess) { cudaFree(t->buf); delete t; return to_check_cuda(ctx, ce, "adjoint forward"); }
    for (int i = 0; i < 1 + S; ++i) outputs[i] = t->outputs[i];
    if (tape_out) *tape_out = t;
    else { cudaFree(t->buf); delete t; }
    return TO_OK;
}

to_status to_adjoint_backward(to_ctx ctx, to_tape t, const double* grad_outputs,
                              double* grad_theta) {
    if (!ctx || !t || !grad_outputs || !grad_theta || t->ctx != ctx) return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    AdjArgs& a = t->a;
    const int S = a.S, P = a.P, ntheta = t->ntheta;
    float go[16];
    for (int i = 0; i < 1 + S; ++i) go[i] = (float)grad_outputs[i];
    TO_CUDA(ctx, cudaMemcpyAsync(const_cast<float*>(a.gout), go, (size_t)(1 + S) * 4,
                                 cudaMemcpyHostToDevice, ctx->stream));
    TO_CUDA(ctx, cudaMemsetAsync(a.gpath, 0, (size_t)P * ntheta * 8, ctx->stream));
    if (grad_outputs[0] != 0.0) {           // the PV part is linear in its weight too
        k_adj_pv_grad<<<(P + 127) / 128, 128, 0, ctx->stream>>>(a, ntheta);
        TO_LAUNCHED(ctx);
    }
    const int TP = tile_paths(t->maxN);
    const size_t smb = (size_t)3 * t->maxN * TP * 4;
    TO_CUDA(ctx, cudaFuncSetAttribute(k_adj_pop_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smb));
    to_prof_begin(ctx, "adjoint_backward");
    k_adj_pop_bwd<<<dim3((P + TP - 1) / TP, S), TP, smb, ctx->stream>>>(a, TP, ntheta);
    to_prof_end(ctx);
    TO_LAUNCHED(ctx);
    std::vector<double> g(ntheta);
    double* d_g = t->d_grad;
    k_col_mean<<<ntheta, 256, 0, ctx->stream>>>(P, ntheta, a.gpath, d_g);
    TO_LAUNCHED(ctx);
    TO_CUDA(ctx, cudaMemcpyAsync(g.data(), d_g, (size_t)ntheta * 8, cudaMemcpyDeviceToHost,
                                 ctx->stream));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < ntheta; ++i) grad_theta[i] = g[i];
    return TO_OK;
}

to_status to_tape_destroy(to_tape t) {
    if (!t) return TO_OK;
    if (t->ctx) {
        cudaSetDevice(t->ctx->device);
        cudaStreamSynchronize(t->ctx->stream);
    }
    cudaFree(t->buf);
    delete t;
    return TO_OK;
}

}  // extern "C"
