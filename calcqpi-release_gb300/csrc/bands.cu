// bands.cu -- H(k) build and batched FP64 Hermitian eigen-solve of every k-point.
//
// Replaces tmatrix::calchamiltonian (src/qpi.cc:454-475), which calls
// tightbind::setmatrix (src/tightbinding.cc:210-219) and gsl_eigen_hermv per
// k-point.  One thread owns one k-point; the b x b matrix and its eigenvectors
// live in registers (b is a template parameter padded up to B; up to 5 bands fully unrolled,
// 6 to 16 bands in local memory with the loops kept: bands_kernel_wide, the same body
// from bands_kernel.cuh).  The solver is
// cyclic complex Jacobi in FP64: G0(k) is invariant under eigenvector phase and
// ordering, so it matches any exact Hermitian eigensolver to rounding.
//
// Roofline: FP64-FLOP bound (GB300 FP64 is ~1/64 of FP32); once per run.  The sweeps start
// from FP32 Jacobi eigenvectors (see below), so most rotations run on the FP32 pipe.
#include <cstdlib>
#include <cstring>

#include "cqpi_internal.h"

namespace cqpi {

#define CQPI_BANDS_KERNEL bands_kernel
#define CQPI_BANDS_UNROLL _Pragma("unroll")
#include "bands_kernel.cuh"
#undef CQPI_BANDS_KERNEL
#undef CQPI_BANDS_UNROLL
#define CQPI_BANDS_KERNEL bands_kernel_wide
#define CQPI_BANDS_UNROLL _Pragma("unroll 1")
#include "bands_kernel.cuh"
#undef CQPI_BANDS_KERNEL
#undef CQPI_BANDS_UNROLL

// FP32 pre-diagonalisation before the FP64 sweeps (CQPI_BANDS_MIXED=0: FP64 throughout)
static int bands_mixed()
{
    const char *f = getenv("CQPI_BANDS_MIXED");
    return (f && !strcmp(f, "0")) ? 0 : 1;
}

template <int B>
static void launch_bands_t(cqpi_handle *h)
{
    const long long nk = (long long)h->kp * h->kp;
    const long long nthr = h->time_reversal ? (long long)(h->kp / 2 + 1) * h->kp : nk;
    const int tr = h->time_reversal ? 1 : 0, mixed = bands_mixed();
    // fully unrolled up to 5 bands; from 6 bands the loop-kept body (the unrolled 6-band copy
    // spilled 7 KB per thread: CJ eigen-solve 13.6 ms against 12.9 ms loop-kept)
    if constexpr (B <= 5)
        bands_kernel<B><<<cdiv(nthr, 128), 128, 0, h->stream>>>(h->b, h->kp, tr, h->scmax, h->efermi, h->npair_R,
                                                                h->d_pR, h->d_pPQ, h->d_eval, h->d_evec,
                                                                h->d_evec32, h->d_eval32, h->d_tw, mixed);
    else
        bands_kernel_wide<B><<<cdiv(nthr, 128), 128, 0, h->stream>>>(h->b, h->kp, tr, h->scmax, h->efermi,
                                                                     h->npair_R, h->d_pR, h->d_pPQ, h->d_eval,
                                                                     h->d_evec, h->d_evec32, h->d_eval32, h->d_tw,
                                                                     mixed);
    h->launches++;
}

void launch_bands(cqpi_handle *h)
{
    const int b = h->b;
    if (b <= 1) launch_bands_t<1>(h);
    else if (b <= 2) launch_bands_t<2>(h);
    else if (b <= 3) launch_bands_t<3>(h);
    else if (b <= 4) launch_bands_t<4>(h);
    else if (b <= 5) launch_bands_t<5>(h);
    else if (b <= 6) launch_bands_t<6>(h);
    else if (b <= 8) launch_bands_t<8>(h);
    else if (b <= 10) launch_bands_t<10>(h);
    else if (b <= 12) launch_bands_t<12>(h);
    else launch_bands_t<16>(h);
}

}  // namespace cqpi
