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
    return to_simulate_rov_batch(ctx, 1, pr, res);
}

to_status to_simulate_rov_batch(to_ctx ctx, int n_roads, const to_rov_problem* prs,
                                to_rov_result* results) {
    if (!ctx || !prs || !results || n_roads <= 0) return TO_ERR_INVALID;
    const to_rov_problem* pr = &prs[0];
    if (pr->n_species <= 0 || pr->n_paths <= 0 ||
        pr->n_years < 3 || pr->n_controls <= 0 || pr->n_controls > TO_ROV_MAXC ||
        pr->dim_res < 2 || !pr->species || !pr->flows || pr->n_uncertainties < 0 ||
        (pr->n_uncertainties > 0 && !pr->uncert) || pr->n_fuels < 0 ||
        pr->n_commodities < 0 || pr->n_fuels + pr->n_commodities > pr->n_uncertainties)
        return TO_ERR_INVALID;
    const int NR = n_roads;
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
    if (NR > 1) {
        // one batch: the same dimensions, processes, costs and seed; each
        // road brings its own species models and road id
        if (pr->sem != 1 || algo != 4 || P < 128 || pr->migration == TO_MIG_SIMT_FP32 ||
            pr->migration == TO_MIG_TC_3XTF32)
            return to_set_error(ctx, TO_ERR_UNSUPPORTED,
                                "batched roads: sem 1, ALGO4, sparse migration, >= 128 paths");
        for (int r = 1; r < NR; ++r) {
            const to_rov_problem& q = prs[r];
            bool same = q.n_species == S && q.n_paths == P && q.n_years == Y &&
                        q.n_controls == C && q.dim_res == R && q.n_uncertainties == U &&
                        q.n_fuels == pr->n_fuels && q.n_commodities == pr->n_commodities &&
                        q.unit_cost == pr->unit_cost && q.unit_revenue == pr->unit_revenue &&
                        q.dt == pr->dt && q.rrr == pr->rrr && q.demand_idx == pr->demand_idx &&
                        q.seed == pr->seed && q.sem == pr->sem && q.migration == pr->migration &&
                        (q.algo == 0 ? 4 : q.algo) == algo && q.species && q.flows;
            for (int c = 0; same && c < C; ++c) same = q.flows[c] == pr->flows[c];
            for (int i = 0; same && i < 6 * U; ++i) same = q.uncert[i] == pr->uncert[i];
            for (int f = 0; same && f < pr->n_fuels; ++f)
                same = q.fuel_costs[f] == pr->fuel_costs[f] && q.fuel_idx[f] == pr->fuel_idx[f];
            for (int c = 0; same && c < pr->n_commodities; ++c)
                same = q.ore_content[c] == pr->ore_content[c] && q.ore_sd[c] == pr->ore_sd[c];
            for (int s = 0; same && s < S; ++s)
                for (int k = 0; same && k < 8; ++k)
                    same = q.species[s].params && q.species[s].params[k] == pr->species[s].params[k];
            if (!same) return to_set_error(ctx, TO_ERR_INVALID, "road %d differs from road 0", r);
        }
    }
    if (pr->demand_idx >= U) return TO_ERR_INVALID;
    for (int f = 0; f < pr->n_fuels; ++f)
        if (pr->fuel_idx[f] < 0 || pr->fuel_idx[f] >= U) return TO_ERR_INVALID;
    long Ql = 1;
    for (int j = 0; j < d; ++j) Ql *= R;
    if (Ql > (1L << 22)) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "grid %ld", Ql);
    const int Q = (int)Ql;
    const long PTl = (long)NR * P;
    if (PTl > (1L << 30)) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "%ld paths", PTl);
    const int PT = (int)PTl, G = NR * C, RS = NR * S;
    cudaSetDevice(ctx->device);
    int maxN = 0;
    for (int r = 0; r < NR; ++r)
        for (int s = 0; s < S; ++s) {
            const to_rov_species& sp = prs[r].species[s];
            if (sp.n_patches <= 0 || !sp.params || !sp.init_pops || !sp.caps || !sp.mmm)
                return TO_ERR_INVALID;
            maxN = sp.n_patches > maxN ? sp.n_patches : maxN;
            for (int k = 0; k < sp.n_patches; ++k)
                if (!std::isfinite(sp.init_pops[k]) || !(sp.caps[k] > 0.0f) ||
                    !std::isfinite(sp.caps[k]))
                    return to_set_error(ctx, TO_ERR_NONFINITE, "road %d species %d patch %d",
                                        r, s, k);
        }
    for (int i = 0; i < 6 * U; ++i)
        if (!std::isfinite(pr->uncert[i])) return to_set_error(ctx, TO_ERR_NONFINITE, "uncert %d", i);
    const int NP = (maxN + 3) & ~3;
    if (NP > 1020) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "%d patches", maxN);
    std::vector<float> mmm((size_t)RS * C * NP * NP, 0.0f), ip((size_t)RS * NP, 0.0f),
        cp((size_t)RS * NP, 1.0f), prm((size_t)S * 8);
    std::vector<int> np(RS), rid(NR);
    for (int r = 0; r < NR; ++r) {
        rid[r] = prs[r].road;
        for (int s = 0; s < S; ++s) {
            const to_rov_species& sp = prs[r].species[s];
            const size_t rs = (size_t)r * S + s;
            int N = sp.n_patches;
            np[rs] = N;
            for (int k = 0; k < N; ++k) { ip[rs * NP + k] = sp.init_pops[k]; cp[rs * NP + k] = sp.caps[k]; }
            for (int c = 0; c < C; ++c)
                for (int k = 0; k < N; ++k)
                    for (int l = 0; l < N; ++l)
                        mmm[((rs * C + c) * NP + k) * NP + l] = sp.mmm[((size_t)c * N + k) * N + l];
        }
    }
    for (int s = 0; s < S; ++s)
        for (int q = 0; q < 8; ++q) prm[(size_t)s * 8 + q] = pr->species[s].params[q];
    const int kmax = k_rule(P) > 0 ? k_rule(P) : 1;
    if (kmax > TO_KNN_KMAX) return to_set_error(ctx, TO_ERR_UNSUPPORTED, "k %d", kmax);
    const size_t blk = (size_t)R * d + 2 * (size_t)Q;
    const int lblocks = (PT + 1023) / 1024;
    const size_t nacc = (size_t)(d + 1) * (d + 4) / 2;   // sums a query (doubles)
    const int cap = NP * 64 < NP * NP ? NP * 64 : NP * NP;
    size_t bytes = 0;
    auto acc = [&](size_t b) { bytes += to_align256(b); };
    acc(mmm.size() * 4); acc(ip.size() * 4); acc(cp.size() * 4); acc(prm.size() * 4); acc(RS * 4);
    acc(NR * 4);
    acc(C * 4); acc(6 * (size_t)(U > 0 ? U : 1) * 4); acc(16 * 4); acc(16 * 4); acc(16 * 4); acc(16 * 4);
    acc((size_t)Y * PT * 4); acc((size_t)(U > 0 ? U : 1) * (Y + 1) * PT * 4);
    acc((size_t)S * (Y + 1) * PT * 4); acc((size_t)S * C * Y * PT * 4);
    acc((size_t)G * d * P * 4); acc((size_t)G * d * P * 4); acc((size_t)G * P * 4);
    acc(G * 4); acc(G * 4); acc((size_t)NR * d * 4); acc((size_t)NR * d * 4);
    acc((size_t)NR * d * R * 4);
    acc((size_t)G * d * P * 4); acc((size_t)G * P * 4);
    acc((size_t)G * (TO_KNN_GCELLS + 1) * 4); acc((size_t)G * sizeof(to_knn_grid));
    acc((size_t)G * Q * 4);
    acc((size_t)G * lblocks * 4); acc((size_t)G * d * 2 * 4);
    acc(4); acc((size_t)G * Q * nacc * 8);
    acc((size_t)Y * G * blk * 4); acc((size_t)Y * PT * 4); acc((size_t)Y * PT * 4);
    acc((size_t)Y * PT * 4); acc((size_t)Y * S * PT * 4); acc((size_t)NR * 5 * 8);
    acc((size_t)RS * C * (NP + 1) * 4); acc((size_t)RS * C * cap * 2); acc((size_t)RS * C * cap * 4);
    acc((size_t)RS * C * 4);
    // union form of each road-species' C <= 3 matrices
    const int ucap = C <= 3 ? (C * cap < NP * NP ? C * cap : NP * NP) : 0;
    if (C <= 3) { acc((size_t)RS * ucap * 16); acc((size_t)RS * (NP + 1) * 4); acc((size_t)RS * 4); }
    if (algo == 6) { acc((size_t)Y * S * NP * P * 4); acc((size_t)Y * S * P * 4); }
    // regressions fitted only where the backward pass reads them, unless
    // the caller asks for the surfaces (corrected semantics, ALGO4)
    bool want_reg = false;
    for (int r = 0; r < NR; ++r) want_reg |= results[r].regression != nullptr;
    const bool touched = pr->sem == 1 && algo == 4 && !want_reg;
    if (touched) { acc((size_t)G * Q); acc((size_t)G * Q * 4); acc(4); }
    TO_TRY(to_arena_reserve(ctx, bytes + 4096));
    TO_CUDA(ctx, cudaMemsetAsync(ctx->arena, 0, bytes, ctx->stream));
    to_rov_args a;
    memset(&a, 0, sizeof(a));
    a.P = P; a.Y = Y; a.S = S; a.C = C; a.U = U; a.R = R; a.Q = Q;
    a.nr = NR; a.PT = PT; a.G = G;
    a.nF = pr->n_fuels; a.Cm = pr->n_commodities; a.demand_idx = pr->demand_idx;
    a.sem = pr->sem; a.road = pr->road; a.dt = pr->dt; a.rrr = pr->rrr;
    a.unit_cost = pr->unit_cost; a.unit_revenue = pr->unit_revenue; a.scaling = 2.0f;
    a.seed = pr->seed; a.np = NP; a.ne = NP; a.kmax = kmax; a.flags = ctx->d_flags;
    a.algo = algo; a.k_mult = algo == 6 ? 3 : 10;
    float* d_mmm = to_arena_take<float>(ctx, mmm.size());
    float* d_ip = to_arena_take<float>(ctx, ip.size());
    float* d_cp = to_arena_take<float>(ctx, cp.size());
    float* d_prm = to_arena_take<float>(ctx, prm.size());
    int* d_np = to_arena_take<int>(ctx, RS);
    int* d_rid = to_arena_take<int>(ctx, NR);
    float* d_flows = to_arena_take<float>(ctx, C);
    float* d_unc = to_arena_take<float>(ctx, 6 * (size_t)(U > 0 ? U : 1));
    float* d_fc = to_arena_take<float>(ctx, 16);
    int* d_fi = to_arena_take<int>(ctx, 16);
    float* d_oc = to_arena_take<float>(ctx, 16);
    float* d_os = to_arena_take<float>(ctx, 16);
    if (pr->n_fuels > 16 || pr->n_commodities > 16) return TO_ERR_UNSUPPORTED;
    a.controls = to_arena_take<int>(ctx, (size_t)Y * PT);
    a.uRes = to_arena_take<float>(ctx, (size_t)(U > 0 ? U : 1) * (Y + 1) * PT);
    a.totalPops = to_arena_take<float>(ctx, (size_t)S * (Y + 1) * PT);
    a.aars = to_arena_take<float>(ctx, (size_t)S * C * Y * PT);
    a.xraw = to_arena_take<float>(ctx, (size_t)G * d * P);
    a.xn = to_arena_take<float>(ctx, (size_t)G * d * P);
    a.yv = to_arena_take<float>(ctx, (size_t)G * P);
    a.npts = to_arena_take<int>(ctx, G);
    a.kc = to_arena_take<int>(ctx, G);
    a.gmin = to_arena_take<float>(ctx, (size_t)NR * d);
    a.gmax = to_arena_take<float>(ctx, (size_t)NR * d);
    a.qax = to_arena_take<float>(ctx, (size_t)NR * d * R);
    a.gsx = to_arena_take<float>(ctx, (size_t)G * d * P);
    a.gsi = to_arena_take<int>(ctx, (size_t)G * P);
    a.gcell = to_arena_take<int>(ctx, (size_t)G * (TO_KNN_GCELLS + 1));
    a.ggrid = to_arena_take<to_knn_grid>(ctx, G);
    a.kth = to_arena_take<float>(ctx, (size_t)G * Q);
    a.lcnt = to_arena_take<int>(ctx, (size_t)G * lblocks);
    a.lkey = to_arena_take<unsigned>(ctx, (size_t)G * d * 2);
    a.lblocks = lblocks;
    a.knn_next = to_arena_take<int>(ctx, 1);
    a.knn_acc = to_arena_take<double>(ctx, (size_t)G * Q * nacc);
    a.reg = to_arena_take<float>(ctx, (size_t)Y * G * blk);
    a.condExp = to_arena_take<float>(ctx, (size_t)Y * PT);
    a.optCont = to_arena_take<int>(ctx, (size_t)Y * PT);
    a.unitProfits = to_arena_take<float>(ctx, (size_t)Y * PT);
    a.adjPops = to_arena_take<float>(ctx, (size_t)Y * S * PT);
    a.stats = to_arena_take<double>(ctx, (size_t)NR * 5);
    to_csc csc;
    csc.ptr = to_arena_take<int>(ctx, (size_t)RS * C * (NP + 1));
    csc.idx = to_arena_take<uint16_t>(ctx, (size_t)RS * C * cap);
    csc.val = to_arena_take<float>(ctx, (size_t)RS * C * cap);
    csc.nnz = to_arena_take<int>(ctx, (size_t)RS * C);
    csc.cap = cap;
    csc.cap_smem = 0;
    csc.uent = nullptr; csc.uptr = nullptr; csc.unnz = nullptr; csc.ucap = 0; csc.ucap_smem = 0;
    if (C <= 3) {
        csc.uent = to_arena_take<int4>(ctx, (size_t)RS * ucap);
        csc.uptr = to_arena_take<int>(ctx, (size_t)RS * (NP + 1));
        csc.unnz = to_arena_take<int>(ctx, (size_t)RS);
        csc.ucap = ucap;
        if (!csc.unnz) return to_set_error(ctx, TO_ERR_ALLOC, "arena sizing");
    }
    if (algo == 6) {
        a.popsY = to_arena_take<float>(ctx, (size_t)Y * S * NP * P);
        a.gmY = to_arena_take<float>(ctx, (size_t)Y * S * P);
    }
    if (touched) {
        a.touched = 1;
        a.qmark = to_arena_take<unsigned char>(ctx, (size_t)G * Q);
        a.qlist = to_arena_take<int>(ctx, (size_t)G * Q);
        a.qcount = to_arena_take<int>(ctx, 1);
        if (!a.qcount) return to_set_error(ctx, TO_ERR_ALLOC, "arena sizing");
    }
    if (!csc.nnz || (algo == 6 && !a.gmY)) return to_set_error(ctx, TO_ERR_ALLOC, "arena sizing");
    TO_TRY(up(ctx, d_mmm, mmm.data(), mmm.size()));
    TO_TRY(up(ctx, d_ip, ip.data(), ip.size()));
    TO_TRY(up(ctx, d_cp, cp.data(), cp.size()));
    TO_TRY(up(ctx, d_prm, prm.data(), prm.size()));
    TO_TRY(up(ctx, d_np, np.data(), np.size()));
    TO_TRY(up(ctx, d_rid, rid.data(), rid.size()));
    TO_TRY(up(ctx, d_flows, pr->flows, C));
    TO_TRY(up(ctx, d_unc, pr->uncert, 6 * (size_t)U));
    TO_TRY(up(ctx, d_fc, pr->fuel_costs, pr->n_fuels));
    TO_TRY(up(ctx, d_fi, pr->fuel_idx, pr->n_fuels));
    TO_TRY(up(ctx, d_oc, pr->ore_content, pr->n_commodities));
    TO_TRY(up(ctx, d_os, pr->ore_sd, pr->n_commodities));
    a.n_patches = d_np; a.params = d_prm; a.init_pops = d_ip; a.caps = d_cp;
    a.mmm = d_mmm; a.flows = d_flows; a.uncert = d_unc; a.fuel_costs = d_fc;
    a.fuel_idx = d_fi; a.ore_content = d_oc; a.ore_sd = d_os; a.road_ids = d_rid;
    bool sparse = false;
    if (pr->migration == TO_MIG_AUTO || pr->migration == TO_MIG_SPARSE_FP32) {
        TO_TRY(to_k::pack_csc(ctx, d_mmm, NP, C, d_np, RS, csc));
        std::vector<int> nz((size_t)RS * C);
        TO_CUDA(ctx, cudaMemcpyAsync(nz.data(), csc.nnz, nz.size() * sizeof(int),
                                     cudaMemcpyDeviceToHost, ctx->stream));
        TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        int mx = 0;
        bool ok = true;
        for (int v : nz) { if (v < 0) ok = false; mx = v > mx ? v : mx; }
        csc.cap_smem = (mx + 7) & ~7;
        sparse = ok && to_k::rov_sparse_smem(NP, C, csc.cap_smem) <= ctx->smem_optin;
        if (ok && csc.uent) {
            // one list per destination for all controls (the forward pass's form)
            TO_TRY(to_k::union_csc(ctx, NP, C, d_np, RS, csc));
            std::vector<int> un((size_t)RS);
            TO_CUDA(ctx, cudaMemcpyAsync(un.data(), csc.unnz, un.size() * sizeof(int),
                                         cudaMemcpyDeviceToHost, ctx->stream));
            TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            int um = 0;
            bool uok = true;
            for (int v : un) { if (v < 0) uok = false; um = v > um ? v : um; }
            csc.ucap_smem = (um + 7) & ~7;
            if (!uok || to_k::rov_union_smem(NP, C, csc.ucap_smem) > ctx->smem_optin)
                csc.uent = nullptr;                   // the per-control form then
            else
                sparse = true;
        }
        if (!sparse && (pr->migration == TO_MIG_SPARSE_FP32 || algo == 6 || NR > 1))
            return to_set_error(ctx, TO_ERR_UNSUPPORTED, "matrices too dense for the sparse form");
    }
    TO_TRY(to_k::rov_run(ctx, a, sparse ? &csc : nullptr));
    std::vector<double> st((size_t)NR * 5);
    TO_TRY(down(ctx, st.data(), a.stats, (size_t)NR * 5));
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    TO_TRY(to_check_device_flags(ctx));
    // road-major device arrays -> each road's [Y][P] (or [Y][S][P]) output
    std::vector<float> f;
    std::vector<int> iv;
    auto fetch_rows = [&](int which, const float* dptr, size_t rows) -> to_status {
        bool any = false;
        for (int r = 0; r < NR; ++r) {
            double* o = which == 0 ? results[r].cond_exp
                      : which == 1 ? results[r].unit_profits : results[r].adj_pops;
            any |= o != nullptr;
        }
        if (!any) return TO_OK;
        f.resize(rows * PT);
        TO_TRY(down(ctx, f.data(), dptr, rows * PT));
        TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int r = 0; r < NR; ++r) {
            double* o = which == 0 ? results[r].cond_exp
                      : which == 1 ? results[r].unit_profits : results[r].adj_pops;
            if (!o) continue;
            for (size_t row = 0; row < rows; ++row)
                for (int p = 0; p < P; ++p)
                    o[row * P + p] = (double)f[row * PT + (size_t)r * P + p];
        }
        return TO_OK;
    };
    TO_TRY(fetch_rows(0, a.condExp, (size_t)Y));
    TO_TRY(fetch_rows(1, a.unitProfits, (size_t)Y));
    TO_TRY(fetch_rows(2, a.adjPops, (size_t)Y * S));
    bool want_oc = false;
    for (int r = 0; r < NR; ++r) want_oc |= results[r].opt_cont != nullptr;
    if (want_reg) {
        f.resize((size_t)Y * G * blk);
        TO_TRY(down(ctx, f.data(), a.reg, (size_t)Y * G * blk));
        TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int r = 0; r < NR; ++r) {
            double* o = results[r].regression;
            if (!o) continue;
            for (int t = 0; t < Y; ++t)
                for (size_t q = 0; q < (size_t)C * blk; ++q)
                    o[((size_t)t * C) * blk + q] = (double)f[((size_t)t * G + (size_t)r * C) * blk + q];
        }
    }
    if (want_oc) {
        iv.resize((size_t)Y * PT);
        TO_TRY(down(ctx, iv.data(), a.optCont, (size_t)Y * PT));
        TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int r = 0; r < NR; ++r) {
            int* o = results[r].opt_cont;
            if (!o) continue;
            for (int t = 0; t < Y; ++t)
                for (int p = 0; p < P; ++p) o[(size_t)t * P + p] = iv[(size_t)t * PT + (size_t)r * P + p];
        }
    }
    TO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int r = 0; r < NR; ++r) {
        const double* sr = st.data() + 5 * (size_t)r;
        results[r].value = sr[0];
        results[r].control = sr[1];
        results[r].sd = sr[2];
        results[r].se = sr[3];
        results[r].n_best = (int)sr[4];
    }
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
