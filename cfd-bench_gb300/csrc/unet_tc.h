// Tensor-core (tcgen05) 3x3x3 convolutions of the U-Net (unet_tc.cu).
#pragma once

namespace nusif {

// the volume and channel counts have a tcgen05 kernel: tiles of 128 cells
// cover whole x-rows (x <= 128 dividing 128, y a multiple of 128 / x) or
// 128-cell pieces of longer rows; 16-channel input groups; 16..96 outputs
bool tc_conv_supported(int X, int Y, int Z, int B, int N, int C0, int C1);

// out[cell][N] = act(sum over taps and input channels of in[cell + tap][c] *
// w[tap][N][c] + bias), zero padding; the input is the channel concat of two
// channels-last BF16 volumes s0 (C0) and s1 (C1, 0: none); w BF16
// [27][N][C0 + C1]; out BF16 or FP32; *err is set when a wait timed out.
// out_ch 1 (FP32 only): only channel 0 is stored, out[cell] (a 1-channel layer
// whose weights are padded to 16 rows); 0: all N channels
bool tc_conv(const void *s0, int C0, const void *s1, int C1, int B, int Z, int Y, int X,
    const void *w, int N, const float *bias, int relu, bool out_bf16, void *out, int *err,
    int out_ch = 0);

}  // namespace nusif
