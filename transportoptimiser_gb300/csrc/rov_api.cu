// rov_api.cu - host entry points of the ROV valuation and of kNN
// (include/transopt.h: to_simulate_rov, to_knn).
#include <cmath>
#include <cstring>
#include <vector>

#include "to_internal.cuh"
#include "to_rov.cuh"
#include "to_sparse.cuh"

namespace {
template <class T>
to_status up(to_ctx ctx, T* d, const T* h, size_t n) {
    if (n == 0) return TO_OK;
    TO_CUDA(ctx, cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    return TO_OK;
}
template <class T>
to_status down(to_ctx ctx, T* h, const T* d, size_t n) {
    if (n == 0) return TO_OK;
    TO_CUDA(ctx, cudaMemcpyAsync(h, d, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
    return TO_OK;
}
int k_rule(int n) {
    if (n <= 3) return 0;
    int k = (int)(10.0 * (std::log((double)n) + 1.0));
    return k < n ? k : n;
}
}  // namespace

extern "C" {

to_status to_simulate_rov(to_ctx ctx, const to_rov_problem* pr, to_rov_result* res) {
    if (!ctx || !pr || !res || pr->n_species <= 0 || pr->n_paths <= 0 ||
        pr->n_years < 3 || pr->n_controls <= 0 || pr->n_controls > TO_ROV_MAXC ||
        pr->dim_res < 2 || !pr->species || !pr->flows || pr->n_uncertainties < 0 ||
        (pr->n_uncertainties > 0 && !pr->uncert) || pr->n_fuels < 0 ||
        pr->n_commodities < 0 || pr->n_fuels + pr->n_commodities > pr->n_uncertainties)
        return TO_ERR_INVALID;
    const int S = pr->n_species, P = pr->n_paths, Y = pr->n_years, C = pr->n_controls;
    const int U = pr->n_uncertainties, R = pr->dim_res, d = S + 1;
    if (d > TO_LSM_MAXD) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "%d species", S);
    if (pr->sem == 0 && S != 1)
        return to_set_error(ctx, TO_ERR_UNSUPPORTED,
                            "reference semantics are defined for one species only");
    const int algo = pr->algo == 0 ? 4 : pr->algo;
    if (algo != 4 && algo != 6) return to_set_error(ctx, TO_ERR_INVALID, "algo %d", pr->algo);
    if (algo == 6 && (pr->sem != 1 || pr->migration == TO_MIG_SIMT_FP32 ||
                      pr->migration == TO_MIG_TC_3XTF32))
        return to_set_error(ctx, TO_ERR_UNSUPPORTED,
                            "ALGO6 is built for sem 1 with the sparse migration form");
    if (pr->demand_idx >= U) return TO_ERR_INVALID;
    for (int f = 0; f < pr->n_fuels; ++f)
        if (pr->fuel_idx[f] < 0 || pr->fuel_idx[f] >= U) return TO_ERR_INVALID;
    long Ql = 1;
    for (int j = 0; j < d; ++j) Ql *= R;
    if (Ql > (1L << 22)) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "grid %ld", Ql);
    const int Q = (int)Ql;
    cudaSetDevice(ctx->device);
    int maxN = 0;
    for (int s = 0; s < S; ++s) {
        const to_rov_species& sp = pr->species[s];
        if (sp.n_patches <= 0 || !sp.params || !sp.init_pops || !sp.caps || !sp.mmm)
            return TO_ERR_INVALID;
        maxN = sp.n_patches > maxN ? sp.n_patches : maxN;
        for (int k = 0; k < sp.n_patches; ++k)
            if (!std::isfinite(sp.init_pops[k]) || !(sp.caps[k] > 0.0f) ||
                !std::isfinite(sp.caps[k]))
                return to_set_error(ctx, TO_ERR_NONFINITE, "species %d patch %d", s, k);
    }
    for (int i = 0; i < 6 * U; ++i)
        if (!std::isfinite(pr->uncert[i])) return to_set_error(ctx, TO_ERR_NONFINITE, "uncert %d", i);
    const int NP = (maxN + 3) & ~3;
    if (NP > 1020) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "%d patches", maxN);
    std::vector<float> mmm((size_t)S * C * NP * NP, 0.0f), ip((size_t)S * NP, 0.0f),
        cp((size_t)S * NP, 1.0f), prm((size_t)S * 8);
    std::vector<int> np(S);
    for (int s = 0; s < S; ++s) {
        const to_rov_species& sp = pr->species[s];
        int N = sp.n_patches;
        np[s] = N;
        for (int k = 0; k < N; ++k) { ip[(size_t)s * NP + k] = sp.init_pops[k]; cp[(size_t)s * NP + k] = sp.caps[k]; }
        for (int c = 0; c < C; ++c)
            for (int k = 0; k < N; ++k)
                for (int l = 0; l < N; ++l)
                    mmm[(((size_t)s * C + c) * NP + k) * NP + l] = sp.mmm[((size_t)c * N + k) * N + l];
        for (int q = 0; q < 8; ++q) prm[(size_t)s * 8 + q] = sp.params[q];
    }
    const int kmax = k_rule(P) > 0 ? k_rule(P) : 1;
    if (kmax > TO_KNN_KMAX) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "k %d", kmax);
    const size_t blk = (size_t)R * d + 2 * (size_t)Q;
    size_t bytes = 0;
    auto acc = [&](size_t b) { bytes += to_align256(b); };
    acc(mmm.size() * 4); acc(ip.size() * 4); acc(cp.size() * 4); acc(prm.size() * 4); acc(S * 4);
    acc(C * 4); acc(6 * (size_t)(U > 0 ? U : 1) * 4); acc(16 * 4); acc(16 * 4); acc(16 * 4); acc(16 * 4);
    acc((size_t)Y * P * 4); acc((size_t)(U > 0 ? U : 1) * (Y + 1) * P * 4);
    acc((size_t)S * (Y + 1) * P * 4); acc((size_t)S * C * Y * P * 4);
    acc((size_t)C * d * P * 4); acc((size_t)C * d * P * 4); acc((size_t)C * P * 4);
    acc(C * 4); acc(C * 4); acc(d * 4); acc(d * 4);
    acc((size_t)C * d * P * 4); acc((size_t)C * P * 4);
    acc((size_t)C * (TO_KNN_GCELLS + 1) * 4); acc((size_t)C * sizeof(to_knn_grid));
    acc((size_t)C * Q * 4);
    const int lblocks = (P + 1023) / 1024;
    acc((size_t)C * lblocks * 4); acc((size_t)C * d * 2 * 4);
    const size_t nacc = (size_t)(d + 1) * (d + 2);
    acc(4); acc((size_t)C * Q * nacc * 4);
    acc((size_t)Y * C * blk * 4); acc((size_t)Y * P * 4); acc((size_t)Y * P * 4);
    acc((size_t)Y * P * 4); acc((size_t)Y * S * P * 4); acc(5 * 8);
    const int cap = NP * 64 < NP * NP ? NP * 64 : NP * NP;
    acc((size_t)S * C * (NP + 1) * 4); acc((size_t)S * C * cap * 2); acc((size_t)S * C * cap * 4);
    acc((size_t)S * C * 4);
    if (algo == 6) { acc((size_t)Y * S * NP * P * 4); acc((size_t)Y * S * P * 4); }
    TO_TRY(to_arena_reserve(ctx, bytes + 4096));
    TO_CUDA(ctx, cudaMemsetAsync(ctx->arena, 0, bytes, ctx->stream));
    to_rov_args a;
    memset(&a, 0, sizeof(a));
    a.P = P; a.Y = Y; a.S = S; a.C = C; a.U = U; a.R = R; a.Q = Q;
    a.nF = pr->n_fuels; a.Cm = pr->n_commodities; a.demand_idx = pr->demand_idx;
    a.sem = pr->sem; a.road = pr->road; a.dt = pr->dt; a.rrr = pr->rrr;
    a.unit_cost = pr->unit_cost; a.unit_revenue = pr->unit_revenue; a.scaling = 2.0f;
    a.seed = pr->seed; a.np = NP; a.ne = NP; a.kmax = kmax;
    a.algo = algo; a.k_mult = algo == 6 ? 3 : 10;
    float* d_mmm = to_arena_take<float>(ctx, mmm.size());
    float* d_ip = to_arena_take<float>(ctx, ip.size());
    float* d_cp = to_arena_take<float>(ctx, cp.size());
    float* d_prm = to_arena_take<float>(ctx, prm.size());
    int* d_np = to_arena_take<int>(ctx, S);
    float* d_flows = to_arena_take<float>(ctx, C);
    float* d_unc = to_arena_take<float>(ctx, 6 * (size_t)(U > 0 ? U : 1));
    float* d_fc = to_arena_take<float>(ctx, 16);
    int* d_fi = to_arena_take<int>(ctx, 16);
    float* d_oc = to_arena_take<float>(ctx, 16);
    float* d_os = to_arena_take<float>(ctx, 16);
    if (pr->n_fuels > 16 || pr->n_commodities > 16) return TO_ERR_UNSUPPORTED;
    a.controls = to_arena_take<int>(ctx, (size_t)Y * P);
    a.uRes = to_arena_take<float>(ctx, (size_t)(U > 0 ? U : 1) * (Y + 1) * P);
    a.totalPops = to_arena_take<float>(ctx, (size_t)S * (Y + 1) * P);
    a.aars = to_arena_take<float>(ctx, (size_t)S * C * Y * P);
    a.xraw = to_arena_take<float>(ctx, (size_t)C * d * P);
    a.xn = to_arena_take<float>(ctx, (size_t)C * d * P);
    a.yv = to_arena_take<float>(ctx, (size_t)C * P);
    a.npts = to_arena_take<int>(ctx, C);
    a.kc = to_arena_take<int>(ctx, C);
    a.gmin = to_arena_take<float>(ctx, d);
    a.gmax = to_arena_take<float>(ctx, d);
    a.gsx = to_arena_take<float>(ctx, (size_t)C * d * P);
    a.gsi = to_arena_take<int>(ctx, (size_t)C * P);
    a.gcell = to_arena_take<int>(ctx, (size_t)C * (TO_KNN_GCELLS + 1));
    a.ggrid = to_arena_take<to_knn_grid>(ctx, C);
    a.kth = to_arena_take<float>(ctx, (size_t)C * Q);
    a.lcnt = to_arena_take<int>(ctx, (size_t)C * lblocks);
    a.lkey = to_arena_take<unsigned>(ctx, (size_t)C * d * 2);
    a.lblocks = lblocks;
    if (algo == 6) {
        a.popsY = to_arena_take<float>(ctx, (size_t)Y * S * NP * P);
        a.gmY = to_arena_take<float>(ctx, (size_t)Y * S * P);
    }
    a.knn_next = to_arena_take<int>(ctx, 1);
    a.knn_acc = to_arena_take<float>(ctx, (size_t)C * Q * nacc);
    a.reg = to_arena_take<float>(ctx, (size_t)Y * C * blk);
    a.condExp = to_arena_take<float>(ctx, (size_t)Y * P);
    a.optCont = to_arena_take<int>(ctx, (size_t)Y * P);
    a.unitProfits = to_arena_take<float>(ctx, (size_t)Y * P);
    a.adjPops = to_arena_take<float>(ctx, (size_t)Y * S * P);
    a.stats = to_arena_take<double>(ctx, 5);
    to_csc csc;
    csc.ptr = to_arena_take<int>(ctx, (size_t)S * C * (NP + 1));
    csc.idx = to_arena_take<uint16_t>(ctx, (size_t)S * C * cap);
    csc.val = to_arena_take<float>(ctx, (size_t)S * C * cap);
    csc.nnz = to_arena_take<int>(ctx, (size_t)S * C);
    csc.cap = cap;
    csc.cap_smem = 0;
    if (!a.stats) return to_set_error(ctx, TO_ERR_ALLOC, "arena sizing");
    TO_TRY(up(ctx, d_mmm, mmm.data(), mmm.size()));
    TO_TRY(up(ctx, d_ip, ip.data(), ip.size()));
    TO_TRY(up(ctx, d_cp, cp.data(), cp.size()));
    TO_TRY(up(ctx, d_prm, prm.data(), prm.size()));
    TO_TRY(up(ctx, d_np, np.data(), np.size()));
    TO_TRY(up(ctx, d_flows, pr->flows, C));
    TO_TRY(up(ctx, d_unc, pr->uncert, 6 * (size_t)U));
    TO_TRY(up(ctx, d_fc, pr->fuel_costs, pr->n_fuels));
    TO_TRY(up(ctx, d_fi, pr->fuel_idx, pr->n_fuels));
    TO_TRY(up(ctx, d_oc, pr->ore_content, pr->n_commodities));
    TO_TRY(up(ctx, d_os, pr->ore_sd, pr->n_commodities));
    a.n_patches = d_np; a.params = d_prm; a.init_pops = d_ip; a.caps = d_cp;
    a.mmm = d_mmm; a.flows = d_flows; a.uncert = d_unc; a.fuel_costs = d_fc;
    a.fuel_idx = d_fi; a.ore_content = d_oc; a.ore_sd = d_os;
    bool sparse = false;
    if (pr->migration == TO_MIG_AUTO || pr->migration == TO_MIG_SPARSE_FP32) {
        TO_TRY(to_k::pack_csc(ctx, d_mmm, NP, C, d_np, S, csc));
        std::vector<int> nz((size_t)S * C);
        TO_CUDA(ctx, cudaMemcpyAsync(nz.data(), csc.nnz, nz.size() * sizeof(int),
                                     cudaMemcpyDeviceToHost, ctx->stream));
        TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        int mx = 0;
        bool ok = true;
        for (int v : nz) { if (v < 0) ok = false; mx = v > mx ? v : mx; }
        csc.cap_smem = (mx + 7) & ~7;
        sparse = ok && to_k::rov_sparse_smem(NP, C, csc.cap_smem) <= ctx->smem_optin;
        if (!sparse && (pr->migration == TO_MIG_SPARSE_FP32 || algo == 6))
            return to_set_error(ctx, TO_ERR_UNSUPPORTED, "matrices too dense for the sparse form");
    }
    TO_TRY(to_k::rov_run(ctx, a, sparse ? &csc : nullptr));
    double st[5];
    TO_TRY(down(ctx, st, a.stats, 5));
    std::vector<float> f;
    std::vector<int> iv;
    auto fetch_f = [&](double* out, const float* dptr, size_t n) -> to_status {
        if (!out) return TO_OK;
        f.resize(n);
        TO_TRY(down(ctx, f.data(), dptr, n));
        TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (size_t i = 0; i < n; ++i) out[i] = (double)f[i];
        return TO_OK;
    };
    TO_TRY(fetch_f(res->cond_exp, a.condExp, (size_t)Y * P));
    TO_TRY(fetch_f(res->unit_profits, a.unitProfits, (size_t)Y * P));
    TO_TRY(fetch_f(res->adj_pops, a.adjPops, (size_t)Y * S * P));
    TO_TRY(fetch_f(res->regression, a.reg, (size_t)Y * C * blk));
    if (res->opt_cont) TO_TRY(down(ctx, res->opt_cont, a.optCont, (size_t)Y * P));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    res->value = st[0];
    res->control = st[1];
    res->sd = st[2];
    res->se = st[3];
    res->n_best = (int)st[4];
    return TO_OK;
}

to_status to_knn(to_ctx ctx, const float* ref, int n, const float* query, int Q, int dim,
                 int k, float* dist, int* ind) {
    if (!ctx || !ref || !query || !dist || !ind || n <= 0 || Q <= 0 || dim <= 0 || k <= 0 ||
        k > n)
        return TO_ERR_INVALID;
    cudaSetDevice(ctx->device);
    TO_TRY(to_arena_reserve(ctx, to_align256((size_t)n * dim * 4) + to_align256((size_t)Q * dim * 4) +
                                 2 * to_align256((size_t)k * Q * 4)));
    float* d_ref = to_arena_take<float>(ctx, (size_t)n * dim);
    float* d_q = to_arena_take<float>(ctx, (size_t)Q * dim);
    float* d_dist = to_arena_take<float>(ctx, (size_t)k * Q);
    int* d_ind = to_arena_take<int>(ctx, (size_t)k * Q);
    TO_TRY(up(ctx, d_ref, ref, (size_t)n * dim));
    TO_TRY(up(ctx, d_q, query, (size_t)Q * dim));
    TO_TRY(to_k::knn(ctx, d_ref, n, d_q, Q, dim, k, d_dist, d_ind));
    TO_TRY(down(ctx, dist, d_dist, (size_t)k * Q));
    TO_TRY(down(ctx, ind, d_ind, (size_t)k * Q));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return TO_OK;
}

}  // extern "C"
