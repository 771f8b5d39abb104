/*
 * rmq_oracle.h -- CPU oracle (test infrastructure only; see rmq_oracle.c).
 */
#ifndef RMQ_ORACLE_H
#define RMQ_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* BASE: src/cpu_methods.h:6-77 restated (leftmost, strict `<`). */
int oracle_base_val(const float *A, int64_t n, const int32_t *Q, int64_t q, float *out, int nt);
int oracle_base_idx(const float *A, int64_t n, const int32_t *Q, int64_t q, int32_t *out, int nt);

/* RTX_blocks decomposition restated (src/rtx_kernels.cu:85-180, src/rtx.h:3-22). */
typedef struct oracle_blocks oracle_blocks_t;
oracle_blocks_t *oracle_blocks_build(const float *A, int64_t n, int64_t bs, int nt);
int oracle_blocks_query(const oracle_blocks_t *o, const int32_t *Q, int64_t q, float *val,
                        int32_t *idx, int nt);
void oracle_blocks_free(oracle_blocks_t *o);

int oracle_max_threads(void);

/* HRMQ (hrmq/RMQRMM64.cpp) restated: balanced-parentheses RMQ. strict = 0
 * resolves ties rightmost like HRMQ, strict = 1 leftmost like BASE. */
typedef struct hrmq_port hrmq_port_t;
hrmq_port_t *hrmq_port_build(const float *A, int64_t n, int strict, int nt);
int hrmq_port_query(const hrmq_port_t *h, const float *A, const int32_t *Q, int64_t q, float *val,
                    int32_t *idx, int nt);
int64_t hrmq_port_bytes(const hrmq_port_t *h);
void hrmq_port_free(hrmq_port_t *h);

#ifdef __cplusplus
}
#endif
#endif
