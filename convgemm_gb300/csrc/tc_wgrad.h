// Parameters of the BF16 tensor-core weight-gradient kernel.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include "cg_common.cuh"

struct TcWgradParams {
    const __nv_bfloat16 *x;   // NHWC [B][H][W][Cp]
    float *ws;                // [splits][Mext][Next] FP32 partial tiles
    int B, H, W, Cp, kh, kw, kn, Nx, P;
    int vstr, hstr, vpad, hpad, vdil, hdil;
    int nchunks, chunks_per_split;  // 64-pixel chunks of the reduction, per split
    FastDiv dcp, dwo, dho;
    int *err;
    int im2col;               // X by im2col-mode TMA (Cp % 64 == 0), else by cp.async gathers
    int x2d;                  // with im2col: X of a 1x1 stride-1 unpadded convolution is the matrix
                              // [P][Cp], loaded by tiled TMA (xmap 2-D, 64 x 64 boxes) instead
    // one split: the epilogue writes dW itself (no workspace, no reduction) in the
    // reference layout `layout` (0: [ci][kh][kw][co], 1: [co][ci][kh][kw]) of C channels
    float *dw;
    int direct, layout, C;
    // 2..8 splits as one thread-block cluster along z: the partial tiles meet in
    // distributed shared memory and the cluster writes dW (no workspace, no reduction launch)
    int cluster;
    // im2col path: one 64-pixel chunk per ring stage and twice the stages (else two chunks
    // per stage): the ring's stage count is a tuned choice
    int kb1;
    // im2col path with two chunks per stage: a second MMA-issuing warp takes the odd chunks into
    // a second accumulator (the epilogue adds the two)
    int iss2;
    // im2col path: chunks of 128 pixels (p.nchunks / chunks_per_split count them), one per stage
    int wide;
    // more splits than one cluster holds: `groups` clusters of `csize` splits per tile
    // (cluster dimension z = csize, splits = groups * csize).  Rank r of each cluster writes
    // its row slice of the cluster's sum to gws [tile][group][128][BN]; the last cluster to
    // arrive at counter [tile][r] adds the groups' slices in group order and writes dW, then
    // puts the counter back to zero.  groups = 0 or 1: one cluster per tile.
    int groups, csize;
    float *gws;
    unsigned *counters;       // mtiles * ntiles * csize words, zero between calls
    // dW of the NHWC API ([ci][kh][kw][co], kn % 4 == 0, Cp % 32 == 0) as a 3-D FP32 tensor
    // (co, tap, ci) with 32 x 1 x 32 boxes and 128-byte swizzle: the single-split epilogue and
    // the one-cluster reduction stage 32 x 32 blocks in shared memory and write them by TMA
    // CTA pairs (cluster x = 2, grid.x even): 256 x bn tiles (bn 128 / 256) through cta_group::2 MMAs,
    // 128-pixel chunks; no split clusters (several splits go to ws)
    int pair;
    int dw_tma;
    // with dw_tma and one cluster: the splits' partial tiles meet in ws ([tile][rank][32 x 32
    // blocks], 16-byte aligned) instead of distributed shared memory
    int xchg;
    CUtensorMap dwmap;
    // several splits, no cluster: the partial tiles go to ws by TMA, ws viewed as the FP32 tensor
    // (n, m, split) of extents (Next, Mext, splits), 32 x 32 x 1 boxes, 128-byte swizzle
    int ws_tma;
    CUtensorMap wsmap;
};

// xmap: im2col map of x (64 pixels x 64 channels per load), used when p.im2col.
cudaError_t tc_wgrad_launch(const TcWgradParams &p, const CUtensorMap &dymap, const CUtensorMap &xmap, int bn, int xa,
                            int mtiles, int ntiles, int splits, cudaStream_t st);
// Whether splits (2..8) can run as clusters for this tile width / operand side / stage form.
bool tc_wgrad_cluster_ok(int bn, int xa, int im2col, int splits, int kb1 = 0, int iss2 = 0, int wide = 0);
// Ring stages of the general weight-gradient kernel for a tile width and form.
int tc_wgrad_stages(int bn, int im2col, int kb1, int wide = 0, int pair = 0);
// Tile counters of the grouped cluster reduction on the current device: `n` consecutive
// zero words for one launch (a rotating range of a fixed device array; NULL if unavailable).
unsigned *tc_wgrad_counters(int n);
// Split groups of the two-pass reduction (0: one pass).  With many splits, the
// first pass sums each of G contiguous split ranges into planes that follow the
// split planes in the workspace, so the workspace holds splits + G planes.
int tc_wgrad_groups(int splits);
// ws: [splits + tc_wgrad_groups(splits)][Nx * kn] FP32.
cudaError_t tc_wgrad_reduce(float *ws, float *dw, int splits, int xa, int Nx, int kn, int C, int Cp, int kh, int kw,
                            int layout, cudaStream_t st);

// Bias gradient db[co] = sum_p dY[p][co] (BF16 dY [P][ld]), deterministic;
// part: tc_bias_grad_groups(P) * kn FP32 scratch.
int tc_bias_grad_groups(long long P);
cudaError_t tc_bias_grad(const void *dy, long long P, int kn, int ld, float *db, float *part, cudaStream_t st);
