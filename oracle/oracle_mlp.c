/*
 * oracle_mlp.c - CPU restatement of the learned surrogate's forward and
 * backward passes (test infrastructure; the library's MLP kernels are in
 * transportoptimiser_gb300/csrc/mlp.cu).  The reference has no learned
 * surrogate, so this oracle follows the library's own definition: BF16
 * rounding (round to nearest even) of every value that feeds a
 * tensor-core GEMM, FP32 biases / ReLU / output layer, and FP64 sums where
 * the device sums in FP32 (the tensor-core accumulation order is not
 * specified, so agreement is to a tolerance, not bit for bit).
 */
#include "oracle_mlp.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum { IN = 16, HID = 128, OUT = 3 };
enum { OFF_W1 = 0, OFF_B1 = OFF_W1 + HID * IN, OFF_W2 = OFF_B1 + HID, OFF_B2 = OFF_W2 + HID * HID,
       OFF_W3 = OFF_B2 + HID, OFF_B3 = OFF_W3 + OUT * HID, NPARAM = OFF_B3 + OUT };

static int g_round = 1;
void or_mlp_set_rounding(int on) { g_round = on; }

float or_bf16(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7F800000u) == 0x7F800000u) {
        if (u & 0x007FFFFFu) u |= 0x00400000u;      /* quiet NaN */
        u &= 0xFFFF0000u;
    } else {
        u += 0x7FFFu + ((u >> 16) & 1u);
        u &= 0xFFFF0000u;
    }
    memcpy(&x, &u, 4);
    return x;
}

/* rounding point of the network (identity when rounding is switched off,
 * which the tests use to pin the backward formulas against autograd) */
static float rnd(float x) { return g_round ? or_bf16(x) : x; }

typedef struct {
    float w1[HID * IN], w2[HID * HID], w3[OUT * HID];
} bfw;

static void round_weights(const float* p, bfw* w) {
    for (int i = 0; i < HID * IN; ++i) w->w1[i] = rnd(p[OFF_W1 + i]);
    for (int i = 0; i < HID * HID; ++i) w->w2[i] = rnd(p[OFF_W2 + i]);
    for (int i = 0; i < OUT * HID; ++i) w->w3[i] = rnd(p[OFF_W3 + i]);
}

/* one row: activations needed by the backward pass */
static void fwd_row(const float* p, const bfw* w, const float* x, float* xb, float* a1, float* h1b,
                    float* a2, float* h2b, float* y) {
    for (int k = 0; k < IN; ++k) xb[k] = rnd(x[k]);
    for (int o = 0; o < HID; ++o) {
        double s = 0.0;
        for (int k = 0; k < IN; ++k) s += (double)xb[k] * w->w1[o * IN + k];
        a1[o] = (float)s + p[OFF_B1 + o];
        h1b[o] = rnd(a1[o] > 0.0f ? a1[o] : 0.0f);
    }
    for (int o = 0; o < HID; ++o) {
        double s = 0.0;
        for (int i = 0; i < HID; ++i) s += (double)h1b[i] * w->w2[o * HID + i];
        a2[o] = (float)s + p[OFF_B2 + o];
        h2b[o] = rnd(a2[o] > 0.0f ? a2[o] : 0.0f);
    }
    for (int q = 0; q < OUT; ++q) {
        float acc = 0.0f;
        for (int o = 0; o < HID; ++o) acc = acc + h2b[o] * w->w3[q * HID + o];
        y[q] = acc + p[OFF_B3 + q];
    }
}

void or_mlp_forward(const float* params, int n, const float* x, float* y) {
    bfw* w = (bfw*)malloc(sizeof(bfw));
    round_weights(params, w);
    float xb[IN], a1[HID], h1b[HID], a2[HID], h2b[HID];
    for (int r = 0; r < n; ++r) fwd_row(params, w, x + (size_t)r * IN, xb, a1, h1b, a2, h2b, y + (size_t)r * OUT);
    free(w);
}

void or_mlp_grad(const float* params, int n, const float* x, const float* t, double* grad,
                 double* loss) {
    bfw* w = (bfw*)malloc(sizeof(bfw));
    round_weights(params, w);
    memset(grad, 0, sizeof(double) * NPARAM);
    float xb[IN], a1[HID], h1b[HID], a2[HID], h2b[HID], y[OUT], dh2b[HID], dh1b[HID];
    const float inv = 1.0f / (3.0f * (float)n);
    double l = 0.0;
    for (int r = 0; r < n; ++r) {
        fwd_row(params, w, x + (size_t)r * IN, xb, a1, h1b, a2, h2b, y);
        float dy[OUT];
        for (int q = 0; q < OUT; ++q) {
            float d = y[q] - t[(size_t)r * OUT + q];
            l += (double)d * d;
            dy[q] = 2.0f * d * inv;
            grad[OFF_B3 + q] += dy[q];
            for (int o = 0; o < HID; ++o) grad[OFF_W3 + q * HID + o] += (double)dy[q] * h2b[o];
        }
        for (int o = 0; o < HID; ++o) {
            float g = (dy[0] * w->w3[o] + dy[1] * w->w3[HID + o]) + dy[2] * w->w3[2 * HID + o];
            dh2b[o] = rnd(a2[o] > 0.0f ? g : 0.0f);
            grad[OFF_B2 + o] += dh2b[o];
            for (int i = 0; i < HID; ++i) grad[OFF_W2 + o * HID + i] += (double)dh2b[o] * h1b[i];
        }
        for (int i = 0; i < HID; ++i) {
            double s = 0.0;
            for (int o = 0; o < HID; ++o) s += (double)dh2b[o] * w->w2[o * HID + i];
            dh1b[i] = rnd(a1[i] > 0.0f ? (float)s : 0.0f);
            grad[OFF_B1 + i] += dh1b[i];
            for (int k = 0; k < IN; ++k) grad[OFF_W1 + i * IN + k] += (double)dh1b[i] * xb[k];
        }
    }
    if (loss) *loss = l / (3.0 * n);
    free(w);
}
