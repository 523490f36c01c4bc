// noalloc.cu -- cqpi_realspace_greens_noalloc: the pruned transform G0(k) -> G0(R) for
// callers that cannot allocate device memory.
//
// Some hosts of this library must not call cudaMalloc (or anything that allocates):
//  - code that enqueues work while a CUDA stream capture is active -- cudaMalloc is not
//    permitted inside a capture and would invalidate the graph being recorded;
//  - instrument-control and plugin hosts (e.g. a scanning-tunnelling-microscope
//    acquisition loop) that own a fixed device-memory budget allocated up front, because
//    cudaMalloc can synchronise the whole device and stall their real-time streams.
// For them this entry point computes, from a caller-owned device array of G0(k), the
// real-space box G0(R), R in [-rb, rb]^2, into a caller-owned device array.  The one
// intermediate it needs (the transform along k_y, bands^2 x kp x (2rb+1) complex
// doubles) lives in a fixed file-scope __device__ array of CQPI_NOALLOC_SCRATCH_BYTES
// (16 MiB), which every GPU that loads libcqpi.so holds until the process exits.
//
// Set-up: the first call on a device (with that device current) looks up the array's
// device address with cudaGetSymbolAddress and raises the kernels' shared-memory limit;
// make that first call before any stream capture begins.  No call allocates, frees or
// calls an allocating library routine.  All calls share the one scratch array and leave
// the last call's contents in it; nothing in it has to start at zero (every element that
// is read was written earlier by the same call), and calls whose GPU work overlaps (on
// different streams, or from different threads without ordering) race on it.
#include <cuda_runtime.h>
#include <mutex>

#include "../../include/cqpi.h"

namespace {

constexpr size_t kScratchElems = CQPI_NOALLOC_SCRATCH_BYTES / sizeof(double2);
static __device__ __align__(256) double2 g_noalloc_scratch[kScratchElems];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
bool g_setup_done[kMaxDevices] = {};
double2 *g_scratch_ptr[kMaxDevices] = {};

__device__ __forceinline__ double2 zmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ int rev_bits(int x, int bits) { return bits == 0 ? 0 : (int)(__brev((unsigned)x) >> (32 - bits)); }
__device__ __forceinline__ int mod_pos(int a, int m) { int r = a % m; return r < 0 ? r + m : r; }

// e^{+2 pi i t / kp} with the phase reduced exactly
__device__ __forceinline__ double2 twiddle(long long t, int kp)
{
    double s, c;
    sincospi(2.0 * (double)(t % kp) / (double)kp, &s, &c);
    return make_double2(c, s);
}

// In-place transform of x[0..kp) in shared memory (sign +1): radix-2 for powers of two,
// otherwise a direct DFT into y.  Returns the array that holds the result.
__device__ double2 *transform(double2 *x, double2 *y, int kp, int logkp)
{
    if (logkp >= 0) {
        for (int len = 2; len <= kp; len <<= 1) {
            const int hl = len >> 1;
            for (int t = threadIdx.x; t < (kp >> 1); t += blockDim.x) {
                const int kk = t % hl, idx = (t / hl) * len + kk;
                const double2 u = x[idx], v = zmul(x[idx + hl], twiddle((long long)kk * (kp / len), kp));
                x[idx] = make_double2(u.x + v.x, u.y + v.y);
                x[idx + hl] = make_double2(u.x - v.x, u.y - v.y);
            }
            __syncthreads();
        }
        return x;
    }
    for (int k = threadIdx.x; k < kp; k += blockDim.x) {
        double2 s = make_double2(0.0, 0.0);
        for (int n = 0; n < kp; n++) {
            const double2 v = zmul(x[n], twiddle((long long)n * k, kp));
            s.x += v.x;
            s.y += v.y;
        }
        y[k] = s;
    }
    __syncthreads();
    return y;
}

// pass 1: for each (i, plane), transform g0k[i][.][plane] along j, keep Y in [-rb, rb]
__global__ void noalloc_rows_kernel(int kp, int logkp, int nb, int rb, int bb, const double2 *__restrict__ g0k,
                                    double2 *__restrict__ half)
{
    extern __shared__ double2 buf[];
    const int i = blockIdx.x, pl = blockIdx.y;
    double2 *x = buf, *y = buf + kp;
    for (int j = threadIdx.x; j < kp; j += blockDim.x) {
        const double2 v = g0k[((size_t)i * kp + j) * bb + pl];
        x[logkp >= 0 ? rev_bits(j, logkp) : j] = v;
    }
    __syncthreads();
    const double2 *r = transform(x, y, kp, logkp);
    for (int yb = threadIdx.x; yb < nb; yb += blockDim.x) half[((size_t)pl * kp + i) * nb + yb] = r[mod_pos(yb - rb, kp)];
}

// pass 2: for each (column yb, plane), transform along i, keep X in [-rb, rb], scale kp^-2
__global__ void noalloc_cols_kernel(int kp, int logkp, int nb, int rb, int bb, double scale,
                                    const double2 *__restrict__ half, double2 *__restrict__ box)
{
    extern __shared__ double2 buf[];
    const int yb = blockIdx.x, pl = blockIdx.y;
    double2 *x = buf, *y = buf + kp;
    for (int i = threadIdx.x; i < kp; i += blockDim.x) {
        const double2 v = half[((size_t)pl * kp + i) * nb + yb];
        x[logkp >= 0 ? rev_bits(i, logkp) : i] = v;
    }
    __syncthreads();
    const double2 *r = transform(x, y, kp, logkp);
    for (int xb = threadIdx.x; xb < nb; xb += blockDim.x) {
        const double2 v = r[mod_pos(xb - rb, kp)];
        box[((size_t)xb * nb + yb) * bb + pl] = make_double2(v.x * scale, v.y * scale);
    }
}

int log2_exact(int v)
{
    if (v <= 0 || (v & (v - 1))) return -1;
    int l = 0;
    while ((1 << l) < v) l++;
    return l;
}

// Once per device, with that device current: the scratch array's device address and the
// kernels' shared-memory limit (2 * kp complex doubles, up to kp = 4096).
int setup_device(double2 **scratch)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return CQPI_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= kMaxDevices) return CQPI_ERR_NOT_SUPPORTED;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_setup_done[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) {
            cudaGetLastError();
            return CQPI_ERR_CUDA;
        }
        const int smem = (int)(2 * 4096 * sizeof(double2));
        if (cudaFuncSetAttribute(noalloc_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess ||
            cudaFuncSetAttribute(noalloc_cols_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) {
            cudaGetLastError();
            return CQPI_ERR_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<double2 *>(p);
        g_setup_done[dev] = true;
    }
    *scratch = g_scratch_ptr[dev];
    return CQPI_OK;
}

}  // namespace

extern "C" int cqpi_realspace_greens_noalloc(const double *g0k, int32_t kpoints, int32_t bands, int32_t rb, double *box,
                                             void *stream)
{
    if (!g0k || !box || kpoints < 1 || kpoints > 4096 || bands < 1 || bands > 16 || rb < 0) return CQPI_ERR_ARG;
    const size_t nb = 2 * (size_t)rb + 1, bb = (size_t)bands * bands;
    // the intermediate must fit the fixed scratch array: bands^2 * kpoints * (2*rb+1) <= 2^20
    if (bb * (size_t)kpoints * nb > kScratchElems) return CQPI_ERR_NOT_SUPPORTED;
    double2 *scratch = nullptr;
    const int rc = setup_device(&scratch);
    if (rc != CQPI_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int logkp = log2_exact(kpoints);
    const size_t smem = 2 * (size_t)kpoints * sizeof(double2);
    const int threads = kpoints >= 256 ? 256 : 64;
    noalloc_rows_kernel<<<dim3(kpoints, (unsigned)bb), threads, smem, s>>>(
        kpoints, logkp, (int)nb, rb, (int)bb, reinterpret_cast<const double2 *>(g0k), scratch);
    noalloc_cols_kernel<<<dim3((unsigned)nb, (unsigned)bb), threads, smem, s>>>(
        kpoints, logkp, (int)nb, rb, (int)bb, 1.0 / ((double)kpoints * kpoints), scratch, reinterpret_cast<double2 *>(box));
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CQPI_OK : CQPI_ERR_CUDA;
}
