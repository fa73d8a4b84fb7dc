/* oracle_interp.h - CPU restatement of the surrogate evaluations (test infrastructure) */
#ifndef ORACLE_INTERP_H
#define ORACLE_INTERP_H
#ifdef __cplusplus
extern "C" {
#endif
/* fS / fP: float scratch of the surrogate and predictor sizes (mode 0) */
void or_interpolate_surrogate(int n, int d, int R, const double* S, const double* P, double* out,
                              int mode, float* fS, float* fP);
#ifdef __cplusplus
}
#endif
#endif
