/*
 * Stand-in for the handful of BLIS declarations that convGemm's sources use.
 *
 * TEST INFRASTRUCTURE ONLY.  This header is written for this project from the
 * call sites in the reference (src/gemm_blis.c:29-35, src/gemm_blis.h:65-76,
 * 150-188, src/gemm_blis_B3A2C0_orig.c:241-243) so that the reference's own
 * loop nests, packers and epilogues compile unmodified and can serve as the
 * parity oracle.  It is not BLIS: the only micro-kernel behind it is a portable
 * FP32 loop with a sequential fused multiply-add per output element
 * (blis_shim.c), and the block sizes are the Skylake-X values quoted by the
 * reference (slides/slides.tex:156-160: MR=32, NR=12, MC=480, NC=3072, KC=384).
 */
#ifndef CONVGEMM_ORACLE_BLIS_SHIM_H
#define CONVGEMM_ORACLE_BLIS_SHIM_H

/* The reference relies on these coming in through blis.h (printf/exit in
 * gemm_blis.h:72-75, floor in gemm_blis.h:141, bool in gemm_blis.h:60,
 * omp_get_max_threads in convGemm.c:35). */
#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include <stdbool.h>
#include <string.h>
#include <math.h>
#include <omp.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int64_t dim_t;
typedef int64_t inc_t;

typedef enum { BLIS_FLOAT = 0, BLIS_DOUBLE = 1 } num_t;
typedef enum { BLIS_GEMM_UKR = 0 } l3ukr_t;
typedef enum { BLIS_KR = 0, BLIS_MR, BLIS_NR, BLIS_MC, BLIS_KC, BLIS_NC } bszid_t;
typedef enum { BLIS_NO_TRANSPOSE = 0, BLIS_TRANSPOSE = 1 } trans_t;

typedef struct {
    const void *next_a;
    const void *next_b;
} auxinfo_t;

typedef struct {
    dim_t mr, nr, mc, nc, kc;
} cntx_t;

/* ABI-4 micro-kernel signature (m, n, k first), as called at gemm_blis.h:70. */
typedef void (*sgemm_ukr_ft)(dim_t m, dim_t n, dim_t k, float *alpha, float *a, float *b,
                             float *beta, float *c, inc_t rs_c, inc_t cs_c,
                             auxinfo_t *data, cntx_t *cntx);

void bli_init(void);
cntx_t *bli_gks_query_cntx(void);
sgemm_ukr_ft bli_cntx_get_l3_vir_ukr_dt(num_t dt, l3ukr_t ukr, const cntx_t *cntx);
dim_t bli_cntx_get_blksz_def_dt(num_t dt, bszid_t bs, const cntx_t *cntx);
void bli_thread_set_num_threads(dim_t n);

static inline void bli_auxinfo_set_next_a(const void *p, auxinfo_t *aux) { aux->next_a = p; }
static inline void bli_auxinfo_set_next_b(const void *p, auxinfo_t *aux) { aux->next_b = p; }

/* Plain column-major SGEMM with general strides (used by the reference's tests,
 * tests/test_base.h:6-8). */
void bli_sgemm(trans_t transa, trans_t transb, dim_t m, dim_t n, dim_t k,
               float *alpha, float *a, inc_t rsa, inc_t csa,
               float *b, inc_t rsb, inc_t csb,
               float *beta, float *c, inc_t rsc, inc_t csc);

#ifdef __cplusplus
}
#endif

#endif
