// Internal host-side interfaces between the library's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "../../include/convgemm_gpu.h"

struct cg_shape {
    int b, h, w, c, kn, kh, kw;
    int vpad, hpad, vstride, hstride, vdil, hdil;
};

static inline cg_shape cg_from_public(const convgemm_shape_t &s) {
    cg_shape r = {s.b, s.h, s.w, s.c, s.kn, s.kh, s.kw, s.vpad, s.hpad, s.vstride, s.hstride, s.vdil, s.hdil};
    return r;
}

struct cg_epi {
    const float *bias, *mean, *inv_std, *gamma, *beta;
    int relu;
};

// Records an error for convgemm_get_last_error(); returns the status.
convgemm_status_t cg_set_error(convgemm_status_t st, const char *fmt, ...);
convgemm_status_t cg_cuda_check(cudaError_t e, const char *what);

// FP32 launchers (cg_fp32.cu).  Inputs are validated by the caller.
cudaError_t cg_fp32_fwd(int nchw, const cg_shape &s, const float *w, const float *x, float *y,
                        const cg_epi &e, cudaStream_t st);
size_t cg_fp32_wgrad_ws_bytes(const cg_shape &s);
cudaError_t cg_fp32_wgrad(int nchw, const cg_shape &s, const float *dy, const float *x, float *dw,
                          float *ws, cudaStream_t st);
cudaError_t cg_fp32_dgrad(int nchw, const cg_shape &s, const float *w, const float *dy, float *dx,
                          int accumulate, cudaStream_t st);

// Fixed-order column sums of per-32-row-group statistics partials (bn_train.cu): the workspace
// holds the FP64 chunk sums, then the FP32 partials [ngroups][2][kn] the kernel writes (at
// workspace + the chunk bytes); out[c] = the sum of plane 0 over the groups, in FP32.
size_t cg_colsum_ws_bytes(long long ngroups, int kn);
cudaError_t cg_colsum_reduce(void *workspace, int ngroups, int kn, float *out, cudaStream_t st);
inline size_t cg_colsum_part_offset(long long ngroups, int kn) {
    return (size_t) ((ngroups + 255) / 256) * 2 * kn * 8;   // 256 groups per chunk (bn_train.cu)
}

// Device error word (set by bounded waits); defined in cg_runtime.cu.
int *cg_device_error_word();
// Counts one kernel launch made by the library (convgemm_launch_count).
void cg_note_launch();

// Explicit lowering helpers (cg_helpers.cu), device pointers.
cudaError_t cg_helper_im2row(float *rows, const float *in, int b, int h, int w, int c, int ho, int wo, int kh, int kw,
                             int vpad, int hpad, int vstr, int hstr, int vdil, int hdil, cudaStream_t st);
cudaError_t cg_helper_row2im(const float *rows, float *out, int b, int h, int w, int c, int ho, int wo, int kh, int kw,
                             int vpad, int hpad, int vstr, int hstr, int vdil, int hdil, cudaStream_t st);
cudaError_t cg_helper_im2col(float *cols, const float *in, int b, int c, int h, int w, int ho, int wo, int kh, int kw,
                             int vpad, int hpad, int vstr, int hstr, int vdil, int hdil, cudaStream_t st);
cudaError_t cg_helper_col2im(const float *cols, float *out, int b, int c, int h, int w, int ho, int wo, int kh, int kw,
                             int vpad, int hpad, int vstr, int hstr, int vdil, int hdil, cudaStream_t st);
cudaError_t cg_helper_transpose(int rows, int cols, const float *in, int ld, float beta, float *out, int kn, int ho,
                                int wo, int start_row, int start_col, cudaStream_t st);

bool cg_pdl_enabled();       // this host thread's setting (convgemm_set_pdl), default: the environment's
bool cg_pdl_env_enabled();   // false when the environment sets CONVGEMM_NO_PDL=1

// Programmatic dependent launch modes of cg_launch_ex.
enum CgPdl {
    CG_PDL_OFF = 0,      // plain launch (the weight-gradient kernels and their reductions)
    CG_PDL_THREAD = 1,   // as the calling thread's setting says (the persistent chain kernels)
};

// Launch, with programmatic stream serialization per `pdl` (CgPdl): the kernel must call
// tc::pdl_wait() before its first global memory access.  Counts the launch.
template <typename... KArgs, typename... Args>
cudaError_t cg_launch_ex(int pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                         Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = (pdl == CG_PDL_THREAD && cg_pdl_enabled()) ? 1 : 0;
    cg_note_launch();
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args &&>(args)...);
}

// Launch with programmatic stream serialization (the kernel must call
// tc::pdl_wait() before its first global memory access); plain launch when the
// environment sets CONVGEMM_NO_PDL=1.  Counts the launch.
// Weight-gradient splits as clusters (CONVGEMM_NO_WGRAD_CLUSTER=1 turns it off).
bool cg_wgrad_cluster_enabled();
template <typename... KArgs, typename... Args>
cudaError_t cg_launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                          Args &&...args) {
    return cg_launch_ex(CG_PDL_THREAD, kernel, grid, block, smem, st, static_cast<Args &&>(args)...);
}


