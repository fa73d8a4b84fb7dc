// to_rov_dev.cuh - device pieces of the ROV valuation shared by the
// backward pass (rov.cu) and the ALGO6 path re-simulation (sparse_pop.cu):
// exogenous-process reads, unit profit, adjusted populations and the two
// decision rules.
#pragma once
#include "to_internal.cuh"
#include "to_lsm_math.h"
#include "to_rov.cuh"

namespace to_rovd {

__device__ __forceinline__ float ure(const to_rov_args& a, int p, int t, int u, int stride_y) {
    // value at the reference's flat index (p*stride_y + t)*U + u of its
    // [P][Y+1][U] array, read from the [U][Y+1][PT] layout (p: path of the
    // batch; the stride Y quirk only arises for one road)
    const int U = a.U, Y1 = a.Y + 1;
    long F = ((long)p * stride_y + t) * U + u;
    long per = (long)Y1 * U;
    int pp = (int)(F / per);
    long rem = F - (long)pp * per;
    int tt = (int)(rem / U), uu = (int)(rem - (long)tt * U);
    return a.uRes[((size_t)uu * Y1 + tt) * a.PT + pp];
}

__device__ __forceinline__ float ore_at(const to_rov_args& a, int p, int t, int c) {
    const int r = p / a.P, pl = p - r * a.P;      // road, path within it
    long f, gen;
    if (a.sem == 0) {
        f = ((long)pl * a.Y + t) * a.Cm + c;
        gen = f / ((long)a.Y * a.P);
    } else {
        gen = c;
        f = (long)c * a.Y * a.P + (long)pl * a.Y + t;
    }
    float z = to_normal1(a.seed, TO_STREAM_ORE, (uint32_t)a.road_ids[r], (uint32_t)(f >> 2), 0,
                         (uint32_t)(f & 3));
    return a.ore_content[gen] + a.ore_sd[gen] * z;
}

__device__ __forceinline__ float unit_profit(const to_rov_args& a, int p, int t,
                                             int fuel_stride_y, int ore_stride_y) {
    float uf = 0.0f, ore = 0.0f;
    for (int f = 0; f < a.nF; ++f)
        uf = fmaf(a.fuel_costs[f], ure(a, p, t, a.fuel_idx[f], fuel_stride_y), uf);
    for (int c = 0; c < a.Cm; ++c)
        ore = fmaf(ore_at(a, p, t, c), ure(a, p, t, a.nF + c, ore_stride_y), ore);
    float prof = (a.unit_cost + uf) - a.unit_revenue * ore;
    if (a.demand_idx >= 0)
        prof = prof * a.uRes[((size_t)a.demand_idx * (a.Y + 1) + t) * a.PT + p];
    return prof;
}

__device__ __forceinline__ float adj_pop(const to_rov_args& a, int p, int t, int s, int c) {
    return a.totalPops[((size_t)s * (a.Y + 1) + t) * a.PT + p] *
           a.aars[(((size_t)s * a.C + c) * a.Y + t) * a.PT + p];
}

__device__ __forceinline__ float threshold(const to_rov_args& a, int s) {
    return (a.sem == 0) ? a.params[a.S * s + 3] : a.params[8 * s + 3];
}


// Terminal-year decision (backwardInduction :2375-2463): the valid control
// with the least single-period payoff, payoffs capped at zero.  state holds
// the adjusted populations [C][S] and the unit profit at [S*C].
__device__ __forceinline__ void decide_terminal(const to_rov_args& a, const float* state,
                                                float& best, int& bc) {
    const int C = a.C, S = a.S;
    best = 0.0f;
    bc = 0;
    for (int c = 0; c < C; ++c) {
        bool valid = true;
        for (int s = 0; s < S; ++s)
            if (state[c * S + s] < threshold(a, s) && c > 0) { valid = false; break; }
        float pay = 0.0f;
        if (valid) {
            float v = a.flows[c] * state[S * C];
            pay = v > 0.0f ? 0.0f : v;
        }
        if (c == 0) best = pay;
        else if (valid && pay < best) { best = pay; bc = c; }
    }
}

// Interior-year decision (backwardInduction :2464-2776): current payoff plus
// the discounted regression value of year t (capped at zero), least wins;
// road r's regressions.
__device__ __forceinline__ void decide_interior(const to_rov_args& a, int t, int r,
                                                const float* state, float& best, int& bc) {
    const int C = a.C, S = a.S, d = S + 1, R = a.R;
    const float disc = 1.0f + a.rrr * a.dt / 100.0f;
    best = 0.0f;
    bc = 0;
    for (int c = 0; c < C; ++c) {
        bool valid = true;
        for (int s = 0; s < S; ++s)
            if (state[c * S + s] < threshold(a, s) && c > 0) { valid = false; break; }
        float pay = 0.0f;
        if (valid) {
            float cur = a.flows[c] * state[S * C];
            const float* rb = to_rov_reg_block(a, t, (size_t)r * C + c);
            float v = (a.sem == 0) ? to_lsm_interp_ref(rb, R, S, C, state)
                                   : to_lsm_interp(rb, R, S, state + c * S, state[S * C]);
            double ce = (double)(v / disc);
            if (ce > 0.0) ce = 0.0;
            pay = (float)((double)cur + ce);
        }
        if (c == 0) { best = pay; continue; }
        if (!valid) continue;
        bool better = (a.sem == 0) ? ((double)pay < 0.975 * (double)best) : (pay < best);
        if (better) { best = pay; bc = c; }
    }
}

}  // namespace to_rovd
