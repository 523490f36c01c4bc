// fft_reg.cuh -- in-register radix-2 DFTs of length 2 ... 64 (sign +1) with compile-time
// twiddles, shared by the four-step transforms of the Green's function (fft32.cu) and of the
// adjoint (adjoint.cu).
#pragma once
#include "cplx.h"

namespace cqpi {

// shared-memory index of element x of a row padded by one element per 32 (conflict-free strides)
__device__ __forceinline__ int pad32(int x) { return x + (x >> 5); }

// e^{+2 pi i k / 64}, k = 0..63 (cos, sin rounded to float): twiddles of the register FFTs.
// Local constexpr tables: with k a compile-time constant (fully unrolled butterflies) the
// values become immediates, so no twiddle is loaded and trivial ones are skipped.
__device__ __forceinline__ float2 w64(int k)
{
    constexpr float re[64] = {
        1.000000000e+00f, 9.951847267e-01f, 9.807852804e-01f, 9.569403357e-01f, 9.238795325e-01f, 8.819212643e-01f, 8.314696123e-01f, 7.730104534e-01f,
        7.071067812e-01f, 6.343932842e-01f, 5.555702330e-01f, 4.713967368e-01f, 3.826834324e-01f, 2.902846773e-01f, 1.950903220e-01f, 9.801714033e-02f,
        6.123233996e-17f, -9.801714033e-02f, -1.950903220e-01f, -2.902846773e-01f, -3.826834324e-01f, -4.713967368e-01f, -5.555702330e-01f, -6.343932842e-01f,
        -7.071067812e-01f, -7.730104534e-01f, -8.314696123e-01f, -8.819212643e-01f, -9.238795325e-01f, -9.569403357e-01f, -9.807852804e-01f, -9.951847267e-01f,
        -1.000000000e+00f, -9.951847267e-01f, -9.807852804e-01f, -9.569403357e-01f, -9.238795325e-01f, -8.819212643e-01f, -8.314696123e-01f, -7.730104534e-01f,
        -7.071067812e-01f, -6.343932842e-01f, -5.555702330e-01f, -4.713967368e-01f, -3.826834324e-01f, -2.902846773e-01f, -1.950903220e-01f, -9.801714033e-02f,
        -1.836970199e-16f, 9.801714033e-02f, 1.950903220e-01f, 2.902846773e-01f, 3.826834324e-01f, 4.713967368e-01f, 5.555702330e-01f, 6.343932842e-01f,
        7.071067812e-01f, 7.730104534e-01f, 8.314696123e-01f, 8.819212643e-01f, 9.238795325e-01f, 9.569403357e-01f, 9.807852804e-01f, 9.951847267e-01f,
    };
    constexpr float im[64] = {
        0.000000000e+00f, 9.801714033e-02f, 1.950903220e-01f, 2.902846773e-01f, 3.826834324e-01f, 4.713967368e-01f, 5.555702330e-01f, 6.343932842e-01f,
        7.071067812e-01f, 7.730104534e-01f, 8.314696123e-01f, 8.819212643e-01f, 9.238795325e-01f, 9.569403357e-01f, 9.807852804e-01f, 9.951847267e-01f,
        1.000000000e+00f, 9.951847267e-01f, 9.807852804e-01f, 9.569403357e-01f, 9.238795325e-01f, 8.819212643e-01f, 8.314696123e-01f, 7.730104534e-01f,
        7.071067812e-01f, 6.343932842e-01f, 5.555702330e-01f, 4.713967368e-01f, 3.826834324e-01f, 2.902846773e-01f, 1.950903220e-01f, 9.801714033e-02f,
        1.224646799e-16f, -9.801714033e-02f, -1.950903220e-01f, -2.902846773e-01f, -3.826834324e-01f, -4.713967368e-01f, -5.555702330e-01f, -6.343932842e-01f,
        -7.071067812e-01f, -7.730104534e-01f, -8.314696123e-01f, -8.819212643e-01f, -9.238795325e-01f, -9.569403357e-01f, -9.807852804e-01f, -9.951847267e-01f,
        -1.000000000e+00f, -9.951847267e-01f, -9.807852804e-01f, -9.569403357e-01f, -9.238795325e-01f, -8.819212643e-01f, -8.314696123e-01f, -7.730104534e-01f,
        -7.071067812e-01f, -6.343932842e-01f, -5.555702330e-01f, -4.713967368e-01f, -3.826834324e-01f, -2.902846773e-01f, -1.950903220e-01f, -9.801714033e-02f,
    };
    return make_float2(re[k], im[k]);
}

// In-register radix-2 DFT of length L (sign +1), natural order in and out.
template <int L>
__device__ __forceinline__ void fft_reg(float2 (&x)[L])
{
    constexpr int LOG = (L == 2) ? 1 : (L == 4) ? 2 : (L == 8) ? 3 : (L == 16) ? 4 : (L == 32) ? 5 : 6;
#pragma unroll
    for (int i = 0; i < L; i++) {
        int j = 0;
#pragma unroll
        for (int bt = 0; bt < LOG; bt++) j |= ((i >> bt) & 1) << (LOG - 1 - bt);
        if (j > i) { const float2 t = x[i]; x[i] = x[j]; x[j] = t; }
    }
    // butterflies as one flat loop of constant trip count per stage, so that every index
    // is a compile-time constant and x stays in registers
#pragma unroll
    for (int s = 0; s < LOG; s++) {
#pragma unroll
        for (int t = 0; t < L / 2; t++) {
            const int hl = 1 << s;
            const int k = t & (hl - 1);
            const int i0 = ((t >> s) << (s + 1)) | k;
            const int widx = k * (64 >> (s + 1));   // < 32; 0: w = 1, 16: w = i
            const float2 y = x[i0 + hl];
            const float2 v = widx == 0 ? y : (widx == 16 ? make_float2(-y.y, y.x) : cmul(y, w64(widx)));
            const float2 u = x[i0];
            x[i0] = cadd(u, v);
            x[i0 + hl] = csub(u, v);
        }
    }
}

}  // namespace cqpi
