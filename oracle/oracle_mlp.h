/* oracle_mlp.h - CPU restatement of the MLP surrogate (test infrastructure) */
#ifndef ORACLE_MLP_H
#define ORACLE_MLP_H
#ifdef __cplusplus
extern "C" {
#endif
float or_bf16(float x);
/* 1 (default): BF16 rounding at the device's rounding points; 0: none */
void or_mlp_set_rounding(int on);
void or_mlp_forward(const float* params, int n, const float* x, float* y);
/* gradient of mean((y - t)^2) (FP64 accumulation); loss = that mean */
void or_mlp_grad(const float* params, int n, const float* x, const float* t, double* grad,
                 double* loss);
#ifdef __cplusplus
}
#endif
#endif
