// adjoint_mma.cu -- the contraction adjoint of the mixed handle on the tensor cores (warp-level
// mma.sync, split-fp16 x 3 with FP32 accumulation), up to 4 bands, one warp per site.
//
// The two products of the contraction adjoint (adjoint.cu, step 1) are small GEMMs with the
// orbital table Phi[q][t] (t = (d, o) window entry, q = sub-pixel) as the constant operand:
//   forward recompute   F[q][n] = sum_t Phi[q][t] Gw[t][n],   n = (operand u/s, band a, re/im)
//   window gradients    G[t][n] = sum_q Phi[q][t] X[q][n],    n = (band a, ubar re/im, sbar re/im)
// with Gw the site's window values G0(p+d)[o][a] (u) and G0(-p-d)[a][o] (s), and X the
// per-pixel ubar = -i W conj(T s), sbar = -i W conj(u^T T) formed in FP32 between the two.
// Each operand is scaled by a power of two into [2^13, 2^14] (Phi once per block, Gw and X
// per site) and split into fp16 hi + lo; hi*hi + hi*lo + lo*hi accumulate in FP32, as in the
// forward contraction (representation error 2^-22).  Phi's two fragment layouts (A of the
// forward, M = q; A of the gradient, M = t) are built once per block in shared memory in the
// per-lane register order of mma.m16n8k16, so each lane loads a fragment as one 16-byte read.
// Outputs are those of adj_contract_warp_kernel (same layouts), which stays for more than 4
// bands, more than 112 sub-pixels or 80 window entries, and the FP64 handle; the per-site M
// parts are FP32 here (adj_mreduce32_kernel sums them).
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "cplx.h"
#include "cqpi_internal.h"

namespace cqpi {

namespace {

constexpr int MQ = 7;    // q tiles of 16 (Q <= 112)
constexpr int KT = 5;    // t steps of 16 (W * mb <= 80)
constexpr int AM_WARPS = 12;
constexpr int ROWS = MQ * 16;   // rows of the per-warp buffer
// row stride of the per-warp buffer (floats): 16 values padded to 20, so that the fragment
// reads (lanes 2tg rows apart) and the row-per-lane float4 accesses hit distinct banks
constexpr int RS = 20;

__device__ __forceinline__ float pow2_scale_of(float mx)
{
    if (!(mx > 0.0f) || !(mx < 3.0e38f)) return 1.0f;
    int ex;
    frexpf(mx, &ex);
    return ldexpf(1.0f, 14 - ex);
}

__device__ __forceinline__ void split2(float v0, float v1, uint32_t &hi, uint32_t &lo)
{
    const __half2 h = __floats2half2_rn(v0, v1);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(v0 - hf.x, v1 - hf.y);
    hi = *reinterpret_cast<const uint32_t *>(&h);
    lo = *reinterpret_cast<const uint32_t *>(&l);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint4 &a, uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w), "r"(b0), "r"(b1));
}

// warp max of a non-negative float
__device__ __forceinline__ float warp_max(float v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

}  // namespace

template <int B>
__global__ void __launch_bounds__(32 * AM_WARPS, 1) adj_contract_mma_kernel(
    int b, int n, int os, int w, int Rb, int NB, int Q, int W, int nimp, int nmaps, int mb, int bs0,
    const float *__restrict__ phi,
    const float2 *__restrict__ box, const double2 *__restrict__ T, const float *__restrict__ wmap,
    float2 *__restrict__ Ub, float2 *__restrict__ Sb, float2 *__restrict__ Mp)
{
    extern __shared__ __align__(16) unsigned char am_sm[];
    // [tile][step][hi/lo][lane] uint4 fragments: forward A (M = q) and gradient A (M = t)
    uint4 *fA = reinterpret_cast<uint4 *>(am_sm);
    uint4 *gA = fA + MQ * KT * 2 * 32;
    float *wbuf = reinterpret_cast<float *>(gA + KT * MQ * 2 * 32);   // [warp][ROWS][RS]
    __shared__ float s_red[32];
    // window staging: offset (floats) of the complex entry (t, n pair) from the site's u or s base
    // point in the box (bit 30 set: the s operand), -1: zero (padding)
    __shared__ int s_off[KT * 16 * 8];
    const int Wmb = W * mb;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, tg = lane & 3;

    // ---- Phi's scale (max over the table) and its fragments
    float mx = 0.f;
    for (int i = tid; i < Q * Wmb; i += blockDim.x) mx = fmaxf(mx, fabsf(phi[i]));
    mx = warp_max(mx);
    if (lane == 0) s_red[warp] = mx;
    __syncthreads();
    if (tid < 32) {
        float v = tid < (int)(blockDim.x >> 5) ? s_red[tid] : 0.f;
        v = warp_max(v);
        if (tid == 0) s_red[31] = v;
    }
    __syncthreads();
    const float sA = pow2_scale_of(s_red[31]);
    auto ph = [&](int q, int t) { return (q < Q && t < Wmb) ? phi[(size_t)q * Wmb + t] * sA : 0.f; };
    // element (r, c) of lane register k of an m16n8k16 A fragment: r = g (+8 for odd pairs),
    // c = 2 tg (+8 for the second half), the pair (c, c+1) packed low-high
    for (int f = tid; f < (MQ * KT + KT * MQ) * 32; f += blockDim.x) {
        const bool grad = f >= MQ * KT * 32;
        const int ff = grad ? f - MQ * KT * 32 : f;
        const int tile = ff / (32 * (grad ? MQ : KT)), rest = ff - tile * 32 * (grad ? MQ : KT);
        const int step = rest >> 5, ln = rest & 31;
        const int lg = ln >> 2, lt = ln & 3;
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int r = lg + ((k & 1) ? 8 : 0), c = 2 * lt + ((k & 2) ? 8 : 0);
            const int m = tile * 16 + r, kk = step * 16 + c;
            // forward: A[q = m][t = kk]; gradient: A[t = m][q = kk]
            const float v0 = grad ? ph(kk, m) : ph(m, kk);
            const float v1 = grad ? ph(kk + 1, m) : ph(m, kk + 1);
            split2(v0, v1, hi[k], lo[k]);
        }
        uint4 *dst = grad ? gA + ((size_t)(tile * MQ + step) * 2) * 32 + ln : fA + ((size_t)(tile * KT + step) * 2) * 32 + ln;
        dst[0] = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        dst[32] = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    }
    {
        const int side_ = 2 * w + 1;
        for (int idx = tid; idx < KT * 16 * 8; idx += blockDim.x) {
            const int t = idx >> 3, nn = 2 * (idx & 7), ri = 0;
            int off = -1;
            if (t < Wmb && nn < 4 * b) {
                const int op = nn / (2 * b), a = (nn - op * 2 * b) >> 1;
                const int d = t / mb, o = bs0 + (t - d * mb);
                const int dx = d / side_ - w, dy = d % side_ - w;
                // u: G(p+d)[o][a] at ((px+dx+Rb) NB + py+dy+Rb) bb; s: G(-p-d)[a][o] at ((-px-dx+Rb) NB + ...)
                const int el = op == 0 ? o * b + a : a * b + o;
                const int rel = (op == 0 ? (dx * NB + dy) : -(dx * NB + dy)) * b * b + el;   // complex units
                off = ((rel * 2 + ri) & 0x3fffffff) | (op << 30);   // float units, two's complement in 30 bits
            }
            s_off[idx] = off;
        }
    }
    __syncthreads();

    // persistent: the block's warps take items (group of AM_WARPS sites, map ei) in turn, so the
    // fragments above are built once per block
    const int nsite = n * n, ngroup = (nsite + AM_WARPS - 1) / AM_WARPS;
    const int wn = n * os, bb = b * b, n2 = n >> 1;
    float *buf = wbuf + (size_t)warp * ROWS * RS;
    for (long long item = blockIdx.x; item < (long long)ngroup * nmaps; item += gridDim.x) {
        const int ei = (int)(item / ngroup), site0 = (int)(item - (long long)ei * ngroup) * AM_WARPS;
        const int site = site0 + warp;
        if (site < nsite) {
        const int e = ei / nimp;
        const int i = site / n, j = site % n;
        const int px = i - n2, py = j - n2;
        const float2 *boxe = box + (size_t)e * NB * NB * bb;
        const double2 *Te = T + (size_t)ei * bb;

        // ---- the site's window values, [t][n] with n = op*2b + 2a + re/im, staged in buf (rows t)
        float wmx = 0.f;
        const float *bf = reinterpret_cast<const float *>(boxe);
        const long long ub = 2LL * (((long long)(px + Rb) * NB + (py + Rb)) * bb);    // float units
        const long long sbs = 2LL * (((long long)(-px + Rb) * NB + (-py + Rb)) * bb);
        for (int idx = lane; idx < KT * 16 * 8; idx += 32) {
            const int off = s_off[idx];
            float2 v = make_float2(0.f, 0.f);
            if (off >= 0) {
                const int rel = ((off & 0x3fffffff) ^ 0x20000000) - 0x20000000;   // sign-extend 30 bits
                v = *reinterpret_cast<const float2 *>(bf + ((off >> 30) ? sbs : ub) + rel);
            }
            *reinterpret_cast<float2 *>(buf + (idx >> 3) * RS + 2 * (idx & 7)) = v;
            wmx = fmaxf(wmx, fmaxf(fabsf(v.x), fabsf(v.y)));
        }
        const float sG = pow2_scale_of(warp_max(wmx));
        __syncwarp();
        // B fragments of a k-step from buf (rows k): b0b1 = rows 2tg, 2tg+1 of column g, b2b3 = +8
        auto bfrag = [&](int k0, int nt, float sc, uint32_t &h0, uint32_t &l0, uint32_t &h1, uint32_t &l1) {
            const int col = nt * 8 + g;
            const float *r0 = buf + (size_t)(k0 + 2 * tg) * RS + col;
            split2(r0[0] * sc, r0[RS] * sc, h0, l0);
            split2(r0[8 * RS] * sc, r0[9 * RS] * sc, h1, l1);
        };
        // ---- forward recompute: F[q][n] for the 7 q tiles and 2 n tiles
        float F[MQ][2][4];
#pragma unroll
        for (int mt = 0; mt < MQ; mt++)
#pragma unroll
            for (int nt = 0; nt < 2; nt++)
#pragma unroll
                for (int c = 0; c < 4; c++) F[mt][nt][c] = 0.f;
#pragma unroll
        for (int ks = 0; ks < KT; ks++) {
#pragma unroll
            for (int nt = 0; nt < 2; nt++) {
                uint32_t h0, l0, h1, l1;
                bfrag(ks * 16, nt, sG, h0, l0, h1, l1);
#pragma unroll
                for (int mt = 0; mt < MQ; mt++) {
                    const uint4 ah = fA[((mt * KT + ks) * 2) * 32 + lane], al = fA[((mt * KT + ks) * 2 + 1) * 32 + lane];
                    mma16816(F[mt][nt], ah, h0, h1);
                    mma16816(F[mt][nt], ah, l0, l1);
                    mma16816(F[mt][nt], al, h0, h1);
                }
            }
        }
        __syncwarp();
        // u, s per pixel into buf rows q: D element (row g / g+8, cols 2tg, 2tg+1)
        const float invF = 1.f / (sA * sG);
#pragma unroll
        for (int mt = 0; mt < MQ; mt++)
#pragma unroll
            for (int nt = 0; nt < 2; nt++) {
                float *r0 = buf + (size_t)(mt * 16 + g) * RS + nt * 8 + 2 * tg;
                *reinterpret_cast<float2 *>(r0) = make_float2(F[mt][nt][0] * invF, F[mt][nt][1] * invF);
                *reinterpret_cast<float2 *>(r0 + 8 * RS) = make_float2(F[mt][nt][2] * invF, F[mt][nt][3] * invF);
            }
        __syncwarp();
        // ---- per pixel: ubar, sbar (in place, row q: n = 4a + {ubar re, im, sbar re, im}), M parts
        float mr[B][B], mi[B][B], Tr[B][B], Ti[B][B];   // T of this map in FP32, read once
#pragma unroll
        for (int a = 0; a < B; a++)
#pragma unroll
            for (int c = 0; c < B; c++) {
                mr[a][c] = 0.f;
                mi[a][c] = 0.f;
                const double2 t = (a < b && c < b) ? Te[a * b + c] : make_double2(0.0, 0.0);
                Tr[a][c] = (float)t.x;
                Ti[a][c] = (float)t.y;
            }
        float xmx = 0.f;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int q = lane + 32 * k;
            if (q >= ROWS) continue;
            float *row = buf + (size_t)q * RS;
            const bool qv = q < Q;
            const int qx = qv ? q / os : 0, qy = qv ? q % os : 0;
            const float W_ = qv ? wmap[((size_t)ei * wn + (size_t)j * os + qy) * wn + (size_t)i * os + qx] : 0.f;
            float rv[16];
#pragma unroll
            for (int c4 = 0; c4 < 4; c4++) {
                const float4 v = reinterpret_cast<const float4 *>(row)[c4];
                rv[4 * c4] = v.x; rv[4 * c4 + 1] = v.y; rv[4 * c4 + 2] = v.z; rv[4 * c4 + 3] = v.w;
            }
            float ur[B], ui[B], sr[B], si[B];
#pragma unroll
            for (int a = 0; a < B; a++) {
                ur[a] = rv[2 * a];
                ui[a] = rv[2 * a + 1];
                sr[a] = rv[(2 * B + 2 * a) & 15];
                si[a] = rv[(2 * B + 2 * a + 1) & 15];
                if (a >= b) { ur[a] = ui[a] = sr[a] = si[a] = 0.f; }
            }
            float x[16];
#pragma unroll
            for (int c = 0; c < 16; c++) x[c] = 0.f;
#pragma unroll
            for (int a = 0; a < B; a++) {
                if (a >= b) continue;
                float tsr = 0.f, tsi = 0.f, utr = 0.f, uti = 0.f;
#pragma unroll
                for (int c = 0; c < B; c++) {
                    if (c >= b) continue;
                    tsr += Tr[a][c] * sr[c] - Ti[a][c] * si[c];   // (T s)_a
                    tsi += Tr[a][c] * si[c] + Ti[a][c] * sr[c];
                    utr += ur[c] * Tr[c][a] - ui[c] * Ti[c][a];   // (u^T T)_a
                    uti += ur[c] * Ti[c][a] + ui[c] * Tr[c][a];
                    mr[a][c] += W_ * (ur[a] * sr[c] - ui[a] * si[c]);
                    mi[a][c] += W_ * (ur[a] * si[c] + ui[a] * sr[c]);
                }
                x[4 * a + 0] = -W_ * tsi;
                x[4 * a + 1] = -W_ * tsr;
                x[4 * a + 2] = -W_ * uti;
                x[4 * a + 3] = -W_ * utr;
            }
#pragma unroll
            for (int c4 = 0; c4 < 4; c4++)
                reinterpret_cast<float4 *>(row)[c4] = make_float4(x[4 * c4], x[4 * c4 + 1], x[4 * c4 + 2], x[4 * c4 + 3]);
#pragma unroll
            for (int c = 0; c < 16; c++) xmx = fmaxf(xmx, fabsf(x[c]));
        }
#pragma unroll
        for (int a = 0; a < B; a++)
#pragma unroll
            for (int c = 0; c < B; c++) {
                if (a >= b || c >= b) continue;
                // the warp sum in FP32 (4 pixels per lane, 32 lanes); FP32 parts per site
                float xr = mr[a][c], xi = mi[a][c];
                for (int o = 16; o > 0; o >>= 1) {
                    xr += __shfl_xor_sync(0xffffffffu, xr, o);
                    xi += __shfl_xor_sync(0xffffffffu, xi, o);
                }
                if (lane == 0) Mp[((size_t)ei * nsite + site) * bb + a * b + c] = make_float2(xr, xi);
            }
        const float sX = pow2_scale_of(warp_max(xmx));
        __syncwarp();
        // ---- window gradients G[t][n] for the 5 t tiles and 2 n tiles, k = q
        float G[KT][2][4];
#pragma unroll
        for (int mt = 0; mt < KT; mt++)
#pragma unroll
            for (int nt = 0; nt < 2; nt++)
#pragma unroll
                for (int c = 0; c < 4; c++) G[mt][nt][c] = 0.f;
#pragma unroll
        for (int ks = 0; ks < MQ; ks++) {
#pragma unroll
            for (int nt = 0; nt < 2; nt++) {
                uint32_t h0, l0, h1, l1;
                bfrag(ks * 16, nt, sX, h0, l0, h1, l1);
#pragma unroll
                for (int mt = 0; mt < KT; mt++) {
                    const uint4 ah = gA[((mt * MQ + ks) * 2) * 32 + lane], al = gA[((mt * MQ + ks) * 2 + 1) * 32 + lane];
                    mma16816(G[mt][nt], ah, h0, h1);
                    mma16816(G[mt][nt], ah, l0, l1);
                    mma16816(G[mt][nt], al, h0, h1);
                }
            }
        }
        // outputs: (row t = g / g+8, cols n = 2tg, 2tg+1) -> a = n / 4, (re, im) of ubar (n % 4 = 0)
        // or sbar (n % 4 = 2)
        const float invG = 1.f / (sA * sX);
#pragma unroll
        for (int mt = 0; mt < KT; mt++)
#pragma unroll
            for (int nt = 0; nt < 2; nt++)
#pragma unroll
                for (int hrow = 0; hrow < 2; hrow++) {
                    const int t = mt * 16 + g + 8 * hrow;
                    const int nn = nt * 8 + 2 * tg, a = nn >> 2;
                    if (t >= Wmb || a >= b) continue;
                    const float2 v = make_float2(G[mt][nt][2 * hrow] * invG, G[mt][nt][2 * hrow + 1] * invG);
                    const size_t idx = (((size_t)ei * Wmb + t) * b + a) * nsite + site;
                    if ((nn & 3) == 0) Ub[idx] = v;
                    else Sb[idx] = v;
                }
            __syncwarp();   // buf is reused by the warp's next site
        }
    }
}

static size_t mma_smem(const cqpi_handle *) { return 16 * (size_t)(2 * MQ * KT * 2 * 32) + 4 * (size_t)AM_WARPS * ROWS * RS; }

template <int B>
static bool launch_mma_t(cqpi_handle *h, int ne, const float *phi, const float2 *box, const float *wmap, float2 *Ub,
                         float2 *Sb, float2 *Mp)
{
    const size_t smem = mma_smem(h);
    if (cudaFuncSetAttribute(adj_contract_mma_kernel<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return false;
    const long long items = (long long)cdiv(h->n * h->n, AM_WARPS) * ne * h->nimp;
    const int grid = (int)std::min<long long>(items, (long long)h->num_sms);   // one block per SM (shared memory)
    adj_contract_mma_kernel<B><<<grid, 32 * AM_WARPS, smem, h->stream>>>(
        h->b, h->n, h->os, h->w, h->Rb, h->NB, h->Q, h->W, h->nimp, ne * h->nimp, h->mb, h->blk_start[0], phi, box,
        h->ws.T, wmap, Ub, Sb, Mp);
    return true;
}

// The tensor-core contraction adjoint (false: not applicable, the caller runs the CUDA-core
// kernel; CQPI_ADJ_MMA=0 forces that)
bool launch_adj_contract_mma(cqpi_handle *h, int ne, const float *phi, const float2 *box, const float *wmap,
                             float2 *Ub, float2 *Sb, float2 *Mp)
{
    const char *f = getenv("CQPI_ADJ_MMA");
    if ((f && !strcmp(f, "0")) || h->b > 4 || h->Q > MQ * 16 || h->W * h->mb > KT * 16 || mma_smem(h) > 227 * 1024)
        return false;
    switch (h->b) {
    case 1: return launch_mma_t<1>(h, ne, phi, box, wmap, Ub, Sb, Mp);
    case 2: return launch_mma_t<2>(h, ne, phi, box, wmap, Ub, Sb, Mp);
    case 3: return launch_mma_t<3>(h, ne, phi, box, wmap, Ub, Sb, Mp);
    default: return launch_mma_t<4>(h, ne, phi, box, wmap, Ub, Sb, Mp);
    }
}

}  // namespace cqpi
