/* oracle_sample.h - CPU restatement of the GA sample selection (test infrastructure) */
#ifndef ORACLE_SAMPLE_H
#define ORACLE_SAMPLE_H
#ifdef __cplusplus
extern "C" {
#endif
void or_select_samples(int n_cur, const double* cur, int nc, const double* cand, int d, int n,
                       int* sample);
#ifdef __cplusplus
}
#endif
#endif
