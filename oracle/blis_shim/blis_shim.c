/*
 * Portable stand-in for the BLIS services that convGemm calls.
 *
 * TEST INFRASTRUCTURE ONLY: it exists so that the reference's own sources
 * (convGemm.c, gemm_blis*.c, im2row_nhwc.c, im2col_nchw.c) build here without
 * BLIS and produce the reference's results for the parity tests.
 *
 * Micro-kernel contract (fixed by the reference's packers, gemm_blis.c:40-142):
 *   Ac holds an MR-wide panel, element (i, p) at Ac[p*MR + i];
 *   Bc holds an NR-wide panel, element (p, j) at Bc[p*NR + j];
 *   C(i, j) at c[i*rs_c + j*cs_c] receives  beta*C + alpha*sum_p Ac(i,p)*Bc(p,j)
 * and, as in BLIS, beta == 0 overwrites C without reading it.  The sum is one
 * fused multiply-add chain per element, in increasing p, starting from +0.
 * This file is compiled without -ffast-math so that this order is kept.
 */
#include "blis/blis.h"

#define SHIM_MR 32
#define SHIM_NR 12
#define SHIM_MC 480
#define SHIM_NC 3072
#define SHIM_KC 384

static cntx_t shim_cntx = {SHIM_MR, SHIM_NR, SHIM_MC, SHIM_NC, SHIM_KC};

static void shim_sgemm_ukr(dim_t m, dim_t n, dim_t k, float *alpha, float *a, float *b,
                           float *beta, float *c, inc_t rs_c, inc_t cs_c,
                           auxinfo_t *data, cntx_t *cntx) {
    (void) data;
    (void) cntx;
    float acc[SHIM_NR][SHIM_MR];
    for (int j = 0; j < SHIM_NR; j++)
        for (int i = 0; i < SHIM_MR; i++) acc[j][i] = 0.0f;
    for (dim_t p = 0; p < k; p++) {
        const float *ap = a + p * SHIM_MR;
        const float *bp = b + p * SHIM_NR;
        for (int j = 0; j < SHIM_NR; j++) {
            const float bv = bp[j];
            for (int i = 0; i < SHIM_MR; i++) acc[j][i] = fmaf(ap[i], bv, acc[j][i]);
        }
    }
    const float al = *alpha, be = *beta;
    for (dim_t j = 0; j < n; j++)
        for (dim_t i = 0; i < m; i++) {
            const float ab = (al == 1.0f) ? acc[j][i] : al * acc[j][i];
            float *cp = c + i * rs_c + j * cs_c;
            if (be == 0.0f) *cp = ab;
            else if (be == 1.0f) *cp = *cp + ab;
            else *cp = fmaf(be, *cp, ab);
        }
}

void bli_init(void) {}

cntx_t *bli_gks_query_cntx(void) { return &shim_cntx; }

sgemm_ukr_ft bli_cntx_get_l3_vir_ukr_dt(num_t dt, l3ukr_t ukr, const cntx_t *cntx) {
    (void) dt;
    (void) ukr;
    (void) cntx;
    return shim_sgemm_ukr;
}

dim_t bli_cntx_get_blksz_def_dt(num_t dt, bszid_t bs, const cntx_t *cntx) {
    (void) dt;
    switch (bs) {
        case BLIS_MR: return cntx->mr;
        case BLIS_NR: return cntx->nr;
        case BLIS_MC: return cntx->mc;
        case BLIS_NC: return cntx->nc;
        case BLIS_KC: return cntx->kc;
        default: return 1;
    }
}

void bli_thread_set_num_threads(dim_t n) { omp_set_num_threads((int) n); }

/* C := beta*C + alpha*op(A)*op(B) with KC-blocked accumulation in the same
 * order as the reference's loop nests (first block scaled by beta, later
 * blocks added). */
void bli_sgemm(trans_t transa, trans_t transb, dim_t m, dim_t n, dim_t k,
               float *alpha, float *a, inc_t rsa, inc_t csa,
               float *b, inc_t rsb, inc_t csb,
               float *beta, float *c, inc_t rsc, inc_t csc) {
    #pragma omp parallel for
    for (dim_t j = 0; j < n; j++) {
        for (dim_t i = 0; i < m; i++) {
            float *cp = c + i * rsc + j * csc;
            for (dim_t pc = 0; pc < k || (pc == 0 && k == 0); pc += SHIM_KC) {
                dim_t kc = (k - pc < SHIM_KC) ? k - pc : SHIM_KC;
                float acc = 0.0f;
                for (dim_t p = pc; p < pc + kc; p++) {
                    float av = (transa == BLIS_TRANSPOSE) ? a[p * rsa + i * csa] : a[i * rsa + p * csa];
                    float bv = (transb == BLIS_TRANSPOSE) ? b[j * rsb + p * csb] : b[p * rsb + j * csb];
                    acc = fmaf(av, bv, acc);
                }
                const float ab = (*alpha == 1.0f) ? acc : *alpha * acc;
                const float be = (pc == 0) ? *beta : 1.0f;
                if (be == 0.0f) *cp = ab;
                else if (be == 1.0f) *cp = *cp + ab;
                else *cp = fmaf(be, *cp, ab);
                if (k == 0) break;
            }
        }
    }
}
