// Parameters of the BF16 tensor-core implicit-GEMM convolution kernel.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "cg_common.cuh"

constexpr int TC_MAXCLS = 16;   // stride-phase classes (input gradient, strides up to 4x4)
constexpr int TC_MAXTAPS = 49;  // taps per class (7x7 filters)

// One dense implicit GEMM: its rows are the output pixels (b, j, jw) of a grid
// Hg x Wg, written to output pixel (oy0 + osy*j, ox0 + osx*jw); tap t reads the
// input pixel (j*isy + iby + toy[t], jw*isx + ibx + tox[t]).
struct TcClass {
    int Hg, Wg;
    int oy0, ox0, osy, osx;
    int isy, isx, iby, ibx;
    int ntaps;
    int kbeg;    // first K column of this class in the packed weights (multiple of 64)
    int ktiles;  // K / 64
    int mtiles;  // ceil(B*Hg*Wg / 128)
    int tile0;   // index of the class's first tile in the launch (classes' tiles are concatenated)
    int gbase;   // statistics form: the class's first 32-row group (classes' groups are concatenated)
    // im2col-mode TMA: first pixel of row j sits at (j*isy + lo_y, jw*isx + lo_x) in the gathered
    // tensor and tap t is the unsigned offset (toy[t] - mint_y, tox[t] - mint_x)
    int lo_y, lo_x, mint_y, mint_x;
    FastDiv dwg, dhg;
    int16_t toy[TC_MAXTAPS], tox[TC_MAXTAPS];
};

struct TcConvParams {
    const __nv_bfloat16 *in;   // gathered activation, NHWC [B][Hin][Win][Cin]
    __nv_bfloat16 *out;        // NHWC [B][Hout][Wout][Cout]
    const float *scale;        // per output channel, or NULL
    const float *shift;        // per output channel, or NULL
    int relu;
    const __nv_bfloat16 *mask;   // BF16 tensor laid out like out, or NULL: out = 0 where mask <= 0 (ReLU backward)
    int accum;                 // BF16 input gradient: out = out + acc (the old value read first; FP32 sum, one
                               // rounding), then the mask; 0: out overwritten
    float *stats;              // BF16 forward: per 32-row group g of the output pixels, [g][0][Cout] the sum
                               // and [g][1][Cout] the sum of squares of z = acc * scale + shift; or NULL
    int B, Hin, Win, Cin, Hout, Wout, Cout;
    FastDiv dcin;
    int *err;                  // device error word for timed-out waits
    int bn;                    // output channels per tile (64, 128, 256)
    int ntiles;                // tiles along the output channels
    int ntiles_total;          // all tiles of all classes; tile t of a class: m = t / ntiles, n = t % ntiles
    int epi_tma;               // output pixels are the GEMM rows in order: stage in SMEM, TMA store
    int im2col;                // A loaded by im2col-mode TMA (Cin % 64 == 0), else gathered by cp.async
    int cpb;                   // 64-channel chunks per tap (Cin / 64) on the im2col path
    int mode;                  // 0 BF16, 1 FP8-E4M3, 2 3xBF16 (FP32 output)
    int mt;                    // 128-row M tiles per tile (1, or 2 sharing each weight tile: BF16 im2col only)
    int ew;                    // epilogue warps: 4, or 8 (BF16 im2col, bn >= 128 or mt == 2, not bn 256 with mt 2)
    int kb1;                   // BF16 im2col, one M tile, four epilogue warps, bn 64 / 128: one K block per ring
                               // stage and twice the stages (8 / 6) instead of two blocks per stage (4 / 3)
    int ncls;
    TcClass cls[TC_MAXCLS];
};

constexpr int TC_MAXIM2COL = 4;  // classes that can use im2col-mode TMA in one launch

struct TcMaps {
    CUtensorMap a[TC_MAXIM2COL];    // im2col maps of the gathered tensor, one per class
    CUtensorMap alo[TC_MAXIM2COL];  // 3xBF16: maps of the low parts
    CUtensorMap wlo;                // 3xBF16: packed low parts of the weights
};

// wmap: packed weights [Cout][K] (box 64 x bn); omap: output [pixels][Cout] (box 64 x 128), used when epi_tma.
// Ring stages of the BF16 implicit-GEMM kernel form chosen by these settings.
int tc_conv_stages(int bn, int im2col, int mt, int ew, int kb1);
cudaError_t tc_conv_launch(const TcConvParams &p, const CUtensorMap &wmap, const CUtensorMap &omap,
                           const TcMaps &amaps, int grid, cudaStream_t st);
