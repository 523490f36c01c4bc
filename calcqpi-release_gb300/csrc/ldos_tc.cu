// ldos_tc.cu -- continuum LDOS contraction on the 5th-generation tensor cores (tcgen05).
//
// Replaces tmatrix::calcwannierldos (src/qpi.cc:876-950) / gpucalcwannierldos[spin]
// (src/qpicudakernel.cu:60-158) in the mixed-precision path.  With the factorisation
//   u_a(p,q) = sum_{d,o} phi_o(q,d) G0(p+d)[o][a],   s_c(p,q) = sum_{d,o} G0(-p-d)[c][o] phi_o(q,d)
//   rho(p,q) = -term1(q) - Im( sum_a u_a (T s)_a )
// the two window sums are GEMMs that share the real, constant A operand
// Phi[q][(d,o)] (M = oversamp^2 <= 128 rows, K = W*orbitals padded to 16):
//   D_u[q][(a,re/im,site)] = Phi x B_u,   D_s[q][(c,re/im,site)] = Phi x B_s,
// N = 2*bands*sites per tile.  Precision: split-FP16 x3 -- A and B are scaled by
// powers of two (A once per handle, B per energy from max|G0(R)|) and split into
// fp16 hi + lo; hi*hi + hi*lo + lo*hi are accumulated in FP32 in tensor memory
// (relative representation error ~2^-22; measured rel. error vs FP64 ~1e-7).
//
// Kernel organisation (persistent, 128 threads = 4 warps, one CTA owns TMEM
// columns for its accumulators):
//   - A (Phi hi/lo for every spin block) is copied once into shared memory in the
//     K-major, no-swizzle core-matrix layout (8 rows x 16 bytes per core matrix);
//   - per tile (energy, site row, TS consecutive sites) and spin block: all threads
//     gather the G0(R) window from the L2-resident FP32 box (im2col), scale, split and
//     store B_u / B_s hi/lo in the same layout; one thread issues the tcgen05.mma
//     chain and tcgen05.commit arrives on an mbarrier; every thread waits (bounded);
//   - epilogue: tcgen05.ld of the accumulators (warp w reads TMEM lanes 32w..32w+31,
//     lane = q row), T s and Im(u . Ts) in FP32, term1 in FP64, staging through
//     shared memory into coalesced row stores of the map.
// Every spin-wait is bounded; on time-out the CTA sets an error bit in *status,
// waits (bounded) for its in-flight MMAs, frees its tensor memory and returns.
// Roofline: tensor-pipe bound (see the bench's roofline object).
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "cplx.h"
#include "cqpi_internal.h"

namespace cqpi {

namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start address, leading-dimension byte
// offset (K direction between 16-byte core-matrix columns), stride byte offset
// (between 8-row groups), version 1, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor, kind::f16: D f32, A f16, B f16, both K-major, N>>3, M>>4.
__host__ __device__ __forceinline__ uint32_t idesc_f16(int M, int N)
{
    return (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(dtmem), "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

// Bounded wait for the given phase parity; false on time-out.  Each try_wait may suspend
// the thread for up to 1 us (it resumes as soon as the phase completes), so waiting warps
// do not take issue slots from the working ones; limit counts try_wait attempts.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, long long limit)
{
    for (long long it = 0; it < limit; it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mbar), "r"(parity), "r"(1000u)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// Four consecutive accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float &a, float &b, float &c, float &d)
{
    uint32_t r0, r1, r2, r3;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(taddr)
                 : "memory");
    a = __uint_as_float(r0); b = __uint_as_float(r1); c = __uint_as_float(r2); d = __uint_as_float(r3);
}

// Two consecutive accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld2(uint32_t taddr, float &a, float &b)
{
    uint32_t r0, r1;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];"
                 : "=r"(r0), "=r"(r1)
                 : "r"(taddr)
                 : "memory");
    a = __uint_as_float(r0); b = __uint_as_float(r1);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Power-of-two scale that maps max|x| to [2^13, 2^14].
__device__ __forceinline__ float pow2_scale(unsigned maxbits)
{
    const float mx = __uint_as_float(maxbits);
    if (!(mx > 0.0f) || !(mx < 3.0e38f)) return 1.0f;
    int ex;
    frexpf(mx, &ex);            // mx = f * 2^ex, f in [0.5, 1)
    return ldexpf(1.0f, 14 - ex);
}

// byte offset of element (row r, k) in a K-major no-swizzle operand with KP columns
__device__ __forceinline__ uint32_t core_off(int r, int kc, int sbo) { return (uint32_t)((r >> 3) * sbo + kc * 128 + (r & 7) * 16); }

}  // namespace tc

constexpr int TC_THREADS = 512;   // 16 warps; warps w, w+4, w+8, w+12 share TMEM lane quarter w%4

template <int B>
__global__ void __launch_bounds__(TC_THREADS, 1) ldos_tc_kernel(const __grid_constant__ TcParams p)
{
    using namespace tc;
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int bb = p.b * p.b, side = 2 * p.w + 1, n2 = p.n >> 1;
    const int sbo = p.KP * 16;                  // bytes per 8-row group (8 rows x KP halfs)
    const int kcs = p.KP >> 3;
    const int wx = p.TS + 2 * p.w;              // window extent in x (sites + halo)
    const int wfl = wx * side * bb * 2;         // floats per staged window
    // shared-memory carve-up (offsets in bytes, 16-byte aligned)
    unsigned char *smA = sm;
    unsigned char *smB = smA + (size_t)p.nblk * 2 * p.a_bytes;
    float *winU = reinterpret_cast<float *>(smB + 4 * (size_t)p.b_bytes);
    float *winS = winU + wfl + 4;               // +4: a zero slot used by padded k columns
    int *tblU = reinterpret_cast<int *>(winS + wfl + 4);
    int *tblS = tblU + p.nblk * p.KP;
    int *rowU = tblS + p.nblk * p.KP;           // per operand row n = (a, re/im, site): window base
    int *rowS = rowU + p.N;
    float *stage = reinterpret_cast<float *>(rowS + p.N);
    const int wt = p.TS * p.os;                 // staged tile width (pixels)
    const int sst = p.sst;                      // staging row stride, skewed against bank conflicts
    uint64_t *mbar = reinterpret_cast<uint64_t *>(stage + ((p.os * sst + 3) & ~3));
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 1);

    {   // A operands (Phi hi/lo of every spin block) -> shared memory, once
        const uint4 *src = p.Aimg;
        uint4 *dst = reinterpret_cast<uint4 *>(smA);
        const int nv = p.nblk * 2 * p.a_bytes / 16;
        for (int i = tid; i < nv; i += TC_THREADS) dst[i] = src[i];
    }
    // k -> float offset of G0(p+d)[o][.] in the u window and of G0(-p-d)[.][o] in the s
    // window, relative to a site's base; padded k point at the zero slot.
    for (int i = tid; i < p.nblk * p.KP; i += TC_THREADS) {
        const int blk = i / p.KP, k = i % p.KP;
        const int bs = blk ? p.bs1 : p.bs0;
        if (k < p.W * p.mb) {
            const int d = k / p.mb, o = bs + k % p.mb;
            const int dxw = d / side, dyw = d % side;   // dx + w, dy + w
            tblU[i] = 2 * ((dxw * side + dyw) * bb + o * p.b);
            tblS[i] = 2 * (((2 * p.w - dxw) * side + (2 * p.w - dyw)) * bb + o);
        } else {
            tblU[i] = -1;
            tblS[i] = -1;
        }
    }
    for (int nrow = tid; nrow < p.N; nrow += TC_THREADS) {
        const int ari = nrow / p.TS, sl = nrow % p.TS, a = ari >> 1, ri = ari & 1;
        rowU[nrow] = 2 * sl * side * bb + 2 * a + ri;
        rowS[nrow] = 2 * (p.TS - 1 - sl) * side * bb + 2 * a * p.b + ri;
    }
    if (tid < 4) { winU[wfl + tid] = 0.f; winS[wfl + tid] = 0.f; }
    if (tid == 0) {
        mbar_init(smem_u32(mbar), 1);
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(smem_u32(tmem_slot), p.tmem_cols);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = idesc_f16(128, p.N);
    uint32_t phase = 0;
    bool ok = true;

    const int ntiles = p.ne * p.n * p.ntx;
    const int lq = tid & 127;                 // TMEM lane = accumulator row = q = qy*os + qx
    const int qx = lq % p.os, qy = lq / p.os;
    const bool qvalid = lq < p.Q;
    const int sgrp = tid >> 7;                // warp group g takes the 4-site chunks g, g+4, ...
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;

    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const int e = t / (p.n * p.ntx);
        const int rr = t % (p.n * p.ntx);
        const int j = rr / p.ntx, i0 = (rr % p.ntx) * p.TS;
        const float sB = pow2_scale(p.gmax[e]);
        const float2 *boxe = p.box + (size_t)e * p.NB * p.NB * bb;
        const int py = j - n2, px0 = i0 - n2;

        // ---- stage the scaled G0 windows: u: X in [px0-w, px0+TS-1+w], Y in [py-w, py+w];
        //      s: X in [-px0-TS+1-w, -px0+w], Y in [-py-w, -py+w]  (zero outside the box)
        {
            // one warp per window x-row: for fixed X the Y range and all b^2 planes are a
            // contiguous segment of side*b^2 complex values in the box; Y always lies in
            // the box, X only leaves it for padded sites past the field of view
            const int rowlen = side * bb;
            for (int seg = warp; seg < 2 * wx; seg += TC_THREADS / 32) {
                const int which = seg >= wx, xl = which ? seg - wx : seg;
                const int X = which == 0 ? px0 - p.w + xl : -px0 - (p.TS - 1) - p.w + xl;
                const int Y0 = which == 0 ? py - p.w : -py - p.w;
                float *w = (which == 0 ? winU : winS) + 2 * xl * rowlen;
                const bool in = X >= -p.Rb && X <= p.Rb;
                const float2 *src = in ? boxe + ((size_t)(X + p.Rb) * p.NB + (Y0 + p.Rb)) * bb : boxe;
                for (int c = (tid & 31); c < rowlen; c += 32) {
                    const float2 v = in ? src[c] : make_float2(0.f, 0.f);
                    w[2 * c] = v.x * sB;
                    w[2 * c + 1] = v.y * sB;
                }
            }
        }
        __syncthreads();

        for (int blk = 0; blk < p.nblk && ok; blk++) {
            // ---- B operands from the windows: rows n = (a, re/im, site), 8 k per item
            const int *tU = tblU + blk * p.KP, *tS = tblS + blk * p.KP;
            // items (op, kc, nrow) with nrow fastest: a warp writes 32 consecutive 16-byte
            // operand rows (4 full core matrices), free of bank conflicts
            const int nitems = 2 * p.N * kcs;
            const float invN = 1.0f / (float)p.N;
            for (int it = tid; it < nitems; it += TC_THREADS) {
                int g = __float2int_rz(((float)it + 0.5f) * invN);   // it / N
                int nrow = it - g * p.N;
                if (nrow < 0) { g--; nrow += p.N; }
                if (nrow >= p.N) { g++; nrow -= p.N; }
                const int op = g >= kcs, kc = op ? g - kcs : g;
                const float *w = op ? winS : winU;
                const int *tb = op ? tS : tU;
                const int base = op ? rowS[nrow] : rowU[nrow];
                float v[8];
#pragma unroll
                for (int kk = 0; kk < 8; kk++) {
                    const int o = tb[kc * 8 + kk];
                    v[kk] = o >= 0 ? w[base + o] : 0.f;
                }
                uint32_t hw[4], lw[4];
#pragma unroll
                for (int kk = 0; kk < 4; kk++) {
                    const __half2 h = __floats2half2_rn(v[2 * kk], v[2 * kk + 1]);
                    const float2 hb = __half22float2(h);
                    const __half2 l = __floats2half2_rn(v[2 * kk] - hb.x, v[2 * kk + 1] - hb.y);
                    hw[kk] = *reinterpret_cast<const uint32_t *>(&h);
                    lw[kk] = *reinterpret_cast<const uint32_t *>(&l);
                }
                const uint32_t off = core_off(nrow, kc, sbo);
                *reinterpret_cast<uint4 *>(smB + (size_t)(op * 2 + 0) * p.b_bytes + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                *reinterpret_cast<uint4 *>(smB + (size_t)(op * 2 + 1) * p.b_bytes + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
            }
            fence_proxy_async();
            tc_fence_before();
            __syncthreads();
            if (tid == 0) {
                tc_fence_after();
                // descriptors of K-step 0; one K-step (16 halfs = 256 bytes) adds 256 >> 4 = 16
                const uint64_t aH = sdesc(smem_u32(smA + (size_t)(blk * 2 + 0) * p.a_bytes), 128, sbo);
                const uint64_t aL = sdesc(smem_u32(smA + (size_t)(blk * 2 + 1) * p.a_bytes), 128, sbo);
                const int nks = p.KP >> 4;
                for (int op = 0; op < 2; op++) {
                    const uint32_t d = tmem + (uint32_t)(blk * 2 * p.N + op * p.N);
                    const uint64_t bH = sdesc(smem_u32(smB + (size_t)(op * 2 + 0) * p.b_bytes), 128, sbo);
                    const uint64_t bL = sdesc(smem_u32(smB + (size_t)(op * 2 + 1) * p.b_bytes), 128, sbo);
                    for (int ks = 0; ks < nks; ks++) {
                        const uint64_t o = (uint64_t)(16 * ks);
                        mma_f16(d, aH + o, bH + o, idesc, ks > 0 ? 1u : 0u);
                        mma_f16(d, aH + o, bL + o, idesc, 1u);
                        mma_f16(d, aL + o, bH + o, idesc, 1u);
                    }
                }
                mma_commit(smem_u32(mbar));
            }
            const bool done = mbar_wait(smem_u32(mbar), phase, p.spin_limit);
            if (done) phase ^= 1u;
            if (__syncthreads_or(!done)) {
                ok = false;
                if (tid == 0) atomicOr(p.status, 2);
            }
        }
        if (!ok) break;
        tc_fence_after();

        // ---- epilogue: each warp group handles TS/4 sites of its lane quarter
        const float inv = p.inv_sA / sB;
        for (int imp = 0; imp < p.nimp; imp++) {
            const float2 *Te = p.T32 + ((size_t)e * p.nimp + imp) * bb;
            const float t1 = qvalid ? (float)p.term1[(size_t)e * p.Q + qx * p.os + qy] : 0.f;
            const float inv2 = inv * inv;
            for (int s0 = sgrp * 4; s0 < p.TS; s0 += 16) {
                float term2[4] = {0.f, 0.f, 0.f, 0.f};
                for (int blk = 0; blk < p.nblk; blk++) {
                    float ur[2 * B][4], sr[2 * B][4];
#pragma unroll
                    for (int ari = 0; ari < 2 * B; ari++) {
                        if (ari < 2 * p.b) {
                            const uint32_t cu = (uint32_t)(blk * 2 * p.N + ari * p.TS + s0);
                            tmem_ld4(tmem + lane_base + cu, ur[ari][0], ur[ari][1], ur[ari][2], ur[ari][3]);
                            tmem_ld4(tmem + lane_base + cu + (uint32_t)p.N, sr[ari][0], sr[ari][1], sr[ari][2], sr[ari][3]);
                        }
                    }
                    tmem_wait_ld();
#pragma unroll
                    for (int a = 0; a < B; a++) {
                        if (a >= p.b) continue;
                        float tsr[4] = {0.f, 0.f, 0.f, 0.f}, tsi[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                        for (int c = 0; c < B; c++) {
                            if (c >= p.b) continue;
                            const float2 tv = __ldg(Te + a * p.b + c);
#pragma unroll
                            for (int u = 0; u < 4; u++) {
                                tsr[u] += tv.x * sr[2 * c][u] - tv.y * sr[2 * c + 1][u];
                                tsi[u] += tv.x * sr[2 * c + 1][u] + tv.y * sr[2 * c][u];
                            }
                        }
#pragma unroll
                        for (int u = 0; u < 4; u++) term2[u] += ur[2 * a][u] * tsi[u] + ur[2 * a + 1][u] * tsr[u];
                    }
                }
                if (qvalid)
#pragma unroll
                    for (int u = 0; u < 4; u++)
                        stage[qy * sst + (s0 + u) * p.os + qx] = (-t1 - term2[u] * inv2) * p.scale;
            }
            __syncthreads();
            const int xbase = i0 * p.os;
            const int xend = min(wt, p.wn - xbase);
            const size_t rowbase = ((size_t)e * p.nimp + imp) * p.wn + (size_t)j * p.os;
            for (int yy = warp; yy < p.os; yy += TC_THREADS / 32) {
                float *dst = p.out + (rowbase + yy) * p.wn + xbase;
                for (int xx = (tid & 31); xx < xend; xx += 32) dst[xx] = stage[yy * sst + xx];
            }
            __syncthreads();
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }

    if (!ok) {
        // make sure no MMA of this CTA is still writing tensor memory before it is freed
        mbar_wait(smem_u32(mbar), phase, p.spin_limit);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, p.tmem_cols);
    }
}


// ---------------------------------------------------------------------------------
// Pipelined variant for one spin block (the non-spin case): tile t's MMAs run on the
// tensor cores while all warps do the epilogue of tile t-1 and build the B operand of
// tile t+1.  Two B buffers in shared memory, two accumulator sets in tensor memory,
// one mbarrier per accumulator set; the G0 windows of tile t+1 are fetched with
// cp.async (zero-fill outside the box) behind the epilogue.
__device__ __forceinline__ void cp_async8(uint32_t dst, const void *src, uint32_t src_bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// arrive on mbar when every earlier cp.async of this thread has landed (counted in the
// barrier's initial arrival count)
__device__ __forceinline__ void cp_async_mbar_arrive(uint32_t mbar)
{
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_n() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <int B>
__global__ void __launch_bounds__(TC_THREADS, 1) ldos_tc_pipe_kernel(const __grid_constant__ TcParams p)
{
    using namespace tc;
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int bb = p.b * p.b, side = 2 * p.w + 1, n2 = p.n >> 1;
    const int sbo = p.KP * 16;
    const int kcs = p.KP >> 3;
    const int wx = p.TS + 2 * p.w;
    const int rowlen = side * bb;
    const int wfl = wx * rowlen * 2;
    unsigned char *smA = sm;                                    // hi, lo
    unsigned char *smB = smA + 2 * (size_t)p.a_bytes;           // 2 buffers x (uH, uL, sH, sL)
    float *winU = reinterpret_cast<float *>(smB + 8 * (size_t)p.b_bytes);
    float *winS = winU + wfl + 4;
    int *tblU = reinterpret_cast<int *>(winS + wfl + 4);
    int *tblS = tblU + p.KP;
    int *rowU = tblS + p.KP;
    int *rowS = rowU + p.N;
    float *stage = reinterpret_cast<float *>(rowS + p.N);
    const int wt = p.TS * p.os, sst = p.sst;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(stage + ((p.os * sst + 3) & ~3));   // [2]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 2);

    {
        const uint4 *src = p.Aimg;
        uint4 *dst = reinterpret_cast<uint4 *>(smA);
        const int nv = 2 * p.a_bytes / 16;
        for (int i = tid; i < nv; i += TC_THREADS) dst[i] = src[i];
    }
    for (int k = tid; k < p.KP; k += TC_THREADS) {
        if (k < p.W * p.mb) {
            const int d = k / p.mb, o = p.bs0 + k % p.mb;
            const int dxw = d / side, dyw = d % side;
            tblU[k] = 2 * ((dxw * side + dyw) * bb + o * p.b);
            tblS[k] = 2 * (((2 * p.w - dxw) * side + (2 * p.w - dyw)) * bb + o);
        } else {
            tblU[k] = -(1 << 30);   // resolved below: points at the window's zero slot
            tblS[k] = -(1 << 30);
        }
    }
    for (int nrow = tid; nrow < p.N; nrow += TC_THREADS) {
        const int ari = nrow / p.TS, sl = nrow % p.TS, a = ari >> 1, ri = ari & 1;
        rowU[nrow] = 2 * sl * rowlen + 2 * a + ri;
        rowS[nrow] = 2 * (p.TS - 1 - sl) * rowlen + 2 * a * p.b + ri;
    }
    if (tid < 4) { winU[wfl + tid] = 0.f; winS[wfl + tid] = 0.f; }
    if (tid == 0) {
        mbar_init(smem_u32(&mbar[0]), 1);
        mbar_init(smem_u32(&mbar[1]), 1);
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(smem_u32(tmem_slot), p.tmem_cols);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = idesc_f16(128, p.N);
    const int ntiles = p.ne * p.n * p.ntx;
    const int lq = tid & 127;
    const int qx = lq % p.os, qy = lq / p.os;
    const bool qvalid = lq < p.Q;
    const int sgrp = tid >> 7;
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    const uint64_t aH = sdesc(smem_u32(smA), 128, sbo), aL = sdesc(smem_u32(smA + p.a_bytes), 128, sbo);

    // tile t -> (energy e, site row j, first site i0), computed once per tile by thread 0
    // of each warp would still divide; the decomposition is cheap enough done uniformly.
    const int per_e = p.n * p.ntx;
    auto tile_of = [&](int it, int &e, int &j, int &i0) {
        const int t = blockIdx.x + it * gridDim.x;
        if (t >= ntiles) return false;
        e = t / per_e;
        const int rr = t - e * per_e;
        j = rr / p.ntx;
        i0 = (rr - j * p.ntx) * p.TS;
        return true;
    };
    // cp.async the two G0 windows of a tile (unscaled; zero outside the box)
    auto fetch_windows = [&](int e, int j, int i0) {
        const float2 *boxe = p.box + (size_t)e * p.NB * p.NB * bb;
        const int py = j - n2, px0 = i0 - n2;
        for (int seg = warp; seg < 2 * wx; seg += TC_THREADS / 32) {
            const int which = seg >= wx, xl = which ? seg - wx : seg;
            const int X = which == 0 ? px0 - p.w + xl : -px0 - (p.TS - 1) - p.w + xl;
            const int Y0 = which == 0 ? py - p.w : -py - p.w;
            const bool in = X >= -p.Rb && X <= p.Rb;
            const float2 *src = in ? boxe + ((size_t)(X + p.Rb) * p.NB + (Y0 + p.Rb)) * bb : boxe;
            float *w = (which == 0 ? winU : winS) + 2 * xl * rowlen;
            for (int c = lane; c < rowlen; c += 32) cp_async8(smem_u32(w + 2 * c), in ? src + c : src, in ? 8u : 0u);
        }
        cp_async_commit();
    };
    // B operands of one tile from the windows into buffer bufi (scaled by sB, split hi/lo)
    auto build_b = [&](int bufi, float sB) {
        unsigned char *Bb = smB + (size_t)bufi * 4 * p.b_bytes;
        const int nitems = 2 * p.N * kcs;
        const float invN = 1.0f / (float)p.N;
        for (int it = tid; it < nitems; it += TC_THREADS) {
            int g = __float2int_rz(((float)it + 0.5f) * invN);
            int nrow = it - g * p.N;
            if (nrow < 0) { g--; nrow += p.N; }
            if (nrow >= p.N) { g++; nrow -= p.N; }
            const int op = g >= kcs, kc = op ? g - kcs : g;
            const float *w = op ? winS : winU;
            const int4 *tb4 = reinterpret_cast<const int4 *>((op ? tblS : tblU) + kc * 8);
            const int base = op ? rowS[nrow] : rowU[nrow];
            const int4 ta = tb4[0], tb = tb4[1];
            const int offs[8] = {ta.x, ta.y, ta.z, ta.w, tb.x, tb.y, tb.z, tb.w};
            float v[8];
#pragma unroll
            for (int kk = 0; kk < 8; kk++) {
                // padded k (negative table entry) reads the zero slot at float offset wfl
                const int o = offs[kk] < 0 ? wfl : base + offs[kk];
                v[kk] = w[o] * sB;
            }
            uint32_t hw[4], lw[4];
#pragma unroll
            for (int kk = 0; kk < 4; kk++) {
                const __half2 h = __floats2half2_rn(v[2 * kk], v[2 * kk + 1]);
                const float2 hb = __half22float2(h);
                const __half2 l = __floats2half2_rn(v[2 * kk] - hb.x, v[2 * kk + 1] - hb.y);
                hw[kk] = *reinterpret_cast<const uint32_t *>(&h);
                lw[kk] = *reinterpret_cast<const uint32_t *>(&l);
            }
            const uint32_t off = core_off(nrow, kc, sbo);
            *reinterpret_cast<uint4 *>(Bb + (size_t)(op * 2 + 0) * p.b_bytes + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
            *reinterpret_cast<uint4 *>(Bb + (size_t)(op * 2 + 1) * p.b_bytes + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
    };
    auto epilogue = [&](int accs, int e, int j, int i0, float sB) {
        const float inv = p.inv_sA / sB, inv2 = inv * inv;
        const uint32_t acc = tmem + (uint32_t)(accs * 2 * p.N);
        for (int imp = 0; imp < p.nimp; imp++) {
            const float2 *Te = p.T32 + ((size_t)e * p.nimp + imp) * bb;
            const float t1 = qvalid ? (float)p.term1[(size_t)e * p.Q + qx * p.os + qy] : 0.f;
            // sites per TMEM read: 4, or 2 for more than 4 bands (u and s of 4 sites would not
            // fit the 128-register cap of 512 threads: 322 bytes spilled at 6 bands)
            constexpr int SU = B > 4 ? 2 : 4;
            for (int s0 = sgrp * 4; s0 < p.TS; s0 += 16) {
#pragma unroll
                for (int hs = 0; hs < 4; hs += SU) {
                float ur[2 * B][SU], sr[2 * B][SU];
#pragma unroll
                for (int ari = 0; ari < 2 * B; ari++) {
                    if (ari < 2 * p.b) {
                        const uint32_t cu = (uint32_t)(ari * p.TS + s0 + hs);
                        if constexpr (SU == 4) {
                            tmem_ld4(acc + lane_base + cu, ur[ari][0], ur[ari][1], ur[ari][2], ur[ari][3]);
                            tmem_ld4(acc + lane_base + cu + (uint32_t)p.N, sr[ari][0], sr[ari][1], sr[ari][2], sr[ari][3]);
                        } else {
                            tmem_ld2(acc + lane_base + cu, ur[ari][0], ur[ari][1]);
                            tmem_ld2(acc + lane_base + cu + (uint32_t)p.N, sr[ari][0], sr[ari][1]);
                        }
                    }
                }
                tmem_wait_ld();
                float term2[SU];
#pragma unroll
                for (int u = 0; u < SU; u++) term2[u] = 0.f;
#pragma unroll
                for (int a = 0; a < B; a++) {
                    if (a >= p.b) continue;
                    float tsr[SU], tsi[SU];
#pragma unroll
                    for (int u = 0; u < SU; u++) tsr[u] = tsi[u] = 0.f;
#pragma unroll
                    for (int c = 0; c < B; c++) {
                        if (c >= p.b) continue;
                        const float2 tv = __ldg(Te + a * p.b + c);
#pragma unroll
                        for (int u = 0; u < SU; u++) {
                            tsr[u] += tv.x * sr[2 * c][u] - tv.y * sr[2 * c + 1][u];
                            tsi[u] += tv.x * sr[2 * c + 1][u] + tv.y * sr[2 * c][u];
                        }
                    }
#pragma unroll
                    for (int u = 0; u < SU; u++) term2[u] += ur[2 * a][u] * tsi[u] + ur[2 * a + 1][u] * tsr[u];
                }
                if (qvalid)
#pragma unroll
                    for (int u = 0; u < SU; u++)
                        stage[qy * sst + (s0 + hs + u) * p.os + qx] = (-t1 - term2[u] * inv2) * p.scale;
                }
            }
            __syncthreads();
            const int xbase = i0 * p.os;
            const int xend = min(wt, p.wn - xbase);
            const size_t rowbase = ((size_t)e * p.nimp + imp) * p.wn + (size_t)j * p.os;
            for (int yy = warp; yy < p.os; yy += TC_THREADS / 32) {
                float *dst = p.out + (rowbase + yy) * p.wn + xbase;
                for (int xx = lane; xx < xend; xx += 32) dst[xx] = stage[yy * sst + xx];
            }
            __syncthreads();
        }
    };

    bool ok = true;
    int e0, j0, i00;
    int issued = 0, waited = 0;
    float sB_cur = 1.f, sB_prev = 1.f;
    if (tile_of(0, e0, j0, i00)) {
        fetch_windows(e0, j0, i00);
        sB_cur = pow2_scale(p.gmax[e0]);
        cp_async_wait_all();
        __syncthreads();
        build_b(0, sB_cur);
        fence_proxy_async();
        __syncthreads();
    }
    int pe = 0, pj = 0, pi0 = 0;   // tile it-1
    for (int it = 0; ok; it++) {
        int e, j, i0;
        if (!tile_of(it, e, j, i0)) break;
        const int s = it & 1;
        if (tid == 0) {
            tc_fence_after();
            unsigned char *Bb = smB + (size_t)s * 4 * p.b_bytes;
            const int nks = p.KP >> 4;
            for (int op = 0; op < 2; op++) {
                const uint32_t d = tmem + (uint32_t)(s * 2 * p.N + op * p.N);
                const uint64_t bH = sdesc(smem_u32(Bb + (size_t)(op * 2 + 0) * p.b_bytes), 128, sbo);
                const uint64_t bL = sdesc(smem_u32(Bb + (size_t)(op * 2 + 1) * p.b_bytes), 128, sbo);
                for (int ks = 0; ks < nks; ks++) {
                    const uint64_t o = (uint64_t)(16 * ks);
                    mma_f16(d, aH + o, bH + o, idesc, ks > 0 ? 1u : 0u);
                    mma_f16(d, aH + o, bL + o, idesc, 1u);
                    mma_f16(d, aL + o, bH + o, idesc, 1u);
                }
            }
            mma_commit(smem_u32(&mbar[s]));
        }
        issued++;
        int ne_, nj, ni0;
        const bool has_next = tile_of(it + 1, ne_, nj, ni0);
        if (has_next) fetch_windows(ne_, nj, ni0);       // lands behind the epilogue
        if (it >= 1) {
            const int ps = (it - 1) & 1;
            const bool done = mbar_wait(smem_u32(&mbar[ps]), ((it - 1) >> 1) & 1, p.spin_limit);
            if (__syncthreads_or(!done)) {
                ok = false;
                if (tid == 0) atomicOr(p.status, 2);
                break;
            }
            waited++;
            tc_fence_after();
            epilogue(ps, pe, pj, pi0, sB_prev);
        }
        float sB_next = sB_cur;
        if (has_next) {
            sB_next = (ne_ == e) ? sB_cur : pow2_scale(p.gmax[ne_]);
            cp_async_wait_all();
            __syncthreads();
            build_b((it + 1) & 1, sB_next);
            fence_proxy_async();
        }
        pe = e; pj = j; pi0 = i0;
        sB_prev = sB_cur;
        sB_cur = sB_next;
        tc_fence_before();
        __syncthreads();
    }
    if (ok && issued > waited) {
        const int last = issued - 1, ps = last & 1;
        const bool done = mbar_wait(smem_u32(&mbar[ps]), (last >> 1) & 1, p.spin_limit);
        if (__syncthreads_or(!done)) {
            ok = false;
            if (tid == 0) atomicOr(p.status, 2);
        } else {
            waited++;
            tc_fence_after();
            epilogue(ps, pe, pj, pi0, sB_prev);
        }
    }
    if (!ok) {
        // bounded waits for every commit not yet observed, then free tensor memory
        for (int k = waited; k < issued; k++) mbar_wait(smem_u32(&mbar[k & 1]), (k >> 1) & 1, p.spin_limit);
    }
    cp_async_wait_all();
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, p.tmem_cols);
    }
}

// Direct-window variant (one spin block).  The B operands are not gathered per tile:
// the G0 windows of a tile -- for each of its EB energies the u window (X = px0-w ..
// px0+TS-1+w, Y = py-w .. py+w) and the s window (the point reflection, stored in reflected
// order) -- are split into fp16 hi/lo once and laid out as planes
//   [kchunk][operand u/s][energy][band, re/im][x][8 halfs],
// where a plane row (x) holds the (2w+1) x orbitals values of one X in K order
// r = dy*orbitals + o (zero padded to 8*NKC).  For a k-step at x-offset dx the B operand of
// 8 consecutive sites in every (operand, energy, band, re/im) plane is then 8 consecutive
// 16-byte rows -- one core matrix per plane -- and an MMA only moves its start address:
// SBO = one plane, LBO = one kchunk (all planes).  One MMA therefore covers both operands
// and all EB energies: N = 8 sites x 2 x EB x 2*bands (192 for 3 bands, 2 energies); the
// issue cost of tcgen05.mma barely depends on N, so wide MMAs are what makes this fast.
// The A operand (Phi) uses the matching K order k = dx * 8*NKC + r, from shared memory or
// (a_tmem) from tensor memory.
//
// Warp roles (18 warps), handing off through mbarriers only:
//   warps 0-7    epilogue: TMEM -> rho (two warps per TMEM lane quarter, warp % 4)
//   warps 8-16   producer: raw FP32 windows by cp.async pieces or one bulk copy per column
//                (raw_full[r]), fp16 split into a window buffer
//   warp 17      MMA issue (one elected lane)
//   win_full[b]  : window buffer b staged            (producer -> MMA)
//   win_empty[b] : MMAs reading buffer b completed    (tcgen05.commit -> producer)
//   acc_full[s]  : accumulator set s complete         (tcgen05.commit -> epilogue)
//   acc_empty[s] : epilogue finished reading set s    (epilogue -> MMA)
// Tile t uses window buffer and accumulator set t & 1, so staging of t+1, the MMAs of t and
// the epilogue of t-1 run concurrently.  Every wait is bounded; a time-out sets bit 1 of
// *status and every role leaves its loop (decisions inside a role are made uniform with a
// barrier reduction), then in-flight MMAs are awaited (bounded) and the tensor memory is
// freed.
// 9 producer warps: the C2 tile's 288 staging items (2 K chunks x 12 re/im plane pairs x 12
// columns) are then one per thread (measured: C2 contraction 6.26 -> 6.21 ms per job, CJ
// 34.3 -> 30.7 ms, against 8 warps converting single planes)
constexpr int TCW_EPI = 256;
constexpr int TCW_PROD = 288;
constexpr int TCW_THREADS = TCW_EPI + TCW_PROD + 32;

namespace tc {
template <int ID, int COUNT>
__device__ __forceinline__ void bar_sync_group() { asm volatile("bar.sync %0, %1;" ::"n"(ID), "n"(COUNT) : "memory"); }
template <int ID, int COUNT>
__device__ __forceinline__ bool bar_or_group(bool pred)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred pin, pout;\n\t"
        "setp.ne.u32 pin, %1, 0;\n\t"
        "bar.red.or.pred pout, %2, %3, pin;\n\t"
        "selp.u32 %0, 1, 0, pout;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)pred), "n"(ID), "n"(COUNT)
        : "memory");
    return r != 0;
}
__device__ __forceinline__ void mbar_arrive(uint32_t mbar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}
// arrive on mbar and add bytes of asynchronous copies to the current phase (the copies may
// land before this arrival: the transaction count may go negative meanwhile)
__device__ __forceinline__ void mbar_arrive_expect(uint32_t mbar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}
// bulk copy global -> shared of bytes (a multiple of 16; both addresses 16-byte aligned),
// completing its bytes on mbar
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t mbar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}
// D (+)= A x B with A read from tensor memory (lane m = row m, 16-bit K pairs per column)
__device__ __forceinline__ void mma_f16_ta(uint32_t dtmem, uint32_t atmem, uint64_t bd, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}"
        ::"r"(dtmem), "r"(atmem), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}
// eight consecutive 32-bit columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&v)[8])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};"
                 ::"r"(taddr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
}  // namespace tc

// JOS: the Josephson form (p.coff, p.tip); a template flag so that the LDOS epilogue keeps
// its register budget.  BULK: the first p.nbulk raw columns of a tile are fetched by bulk
// copies (instantiated for 3, 6 and 8 bands only; without it the producer carries no trace
// of them: measured 1.3% on the 3-band contraction).
template <int B, bool JOS, bool FOLD, bool BULK>
__global__ void __launch_bounds__(TCW_THREADS, 1) ldos_tcw_kernel(const __grid_constant__ TcParams p)
{
    using namespace tc;
    extern __shared__ __align__(1024) unsigned char sm[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int bb = p.b * p.b, side = 2 * p.w + 1, n2 = p.n >> 1;
    const int twob = 2 * p.b;
    const int NX = p.NX, NKC = p.NKC, TS = p.TS, EB = p.EB;
    const int rowlen = side * bb;                 // complex values per raw window column (one X)
    // raw column pitch (complex values): with bulk copies rowlen + 1 rounded up to even, so
    // that a column's copy can start at the 16-byte boundary at or below its first value;
    // else rowlen (an odd pitch spreads the converters' strided reads over more banks)
    const int cpf = (BULK && p.nbulk > 0) ? (rowlen + 2) & ~1 : rowlen;
    const int rawfl = NX * cpf * 2;               // floats per raw window
    const int ncol = 2 * EB * NX;                 // raw columns per tile: [op][energy][x]
    const int nval = side * p.mb;                 // K entries per window row that carry data
    const int sbo_a = p.KP * 16;
    const int NMMA = 8 * 2 * EB * twob;           // MMA N: 8 sites x (u, s) x EB energies x (band, re/im)
    const int setcols = p.H * NMMA;               // accumulator columns per set
    const int opcols = EB * twob * 8;             // column offset of the s operand inside a group
    const int nplanes = 2 * EB * twob;            // planes per kchunk
    unsigned char *smA = sm;                                                   // A hi, A lo (unless a_tmem)
    unsigned char *smW = smA + (p.a_tmem ? 0 : 2 * (size_t)p.a_bytes);         // [buffer][hi,lo] windows
    // raw windows: a ring of nraw buffers of [op][energy] windows, then a zero slot
    float *raw = reinterpret_cast<float *>(smW + 4 * (size_t)p.win_bytes);
    const int rawbuf = 2 * EB * rawfl;
    const int nraw = p.nraw;
    const int zslot = nraw * rawbuf;
    int *offR = reinterpret_cast<int *>(raw + zslot + 4);                      // [op][8*NKC] offsets in a raw column
    // epilogue constants of the current energy block: T [energy][impurity][b*b],
    // 1/(sA sB)^2 [energy], term1 [energy][q]
    float2 *cT = reinterpret_cast<float2 *>(offR + 2 * NKC * 8);
    float *cInv2 = reinterpret_cast<float *>(cT + EB * p.nimp * bb);
    float *cT1 = cInv2 + EB;
    float *cTip = cT1 + EB * 128;   // Josephson tip factor (re, im) [energy]
    // producer: float offset (0 or 2) of the first value of every raw column in its copy,
    // [raw buffer][op][energy][x], then the column table
    const size_t ct_off = ((size_t)(reinterpret_cast<unsigned char *>(cTip + 2 * EB) - sm) + 15) & ~(size_t)15;
    int *shTab = reinterpret_cast<int *>(sm + ct_off);
    // producer: source offset (float2 units, -1 outside the box) of every raw column of the
    // tile being fetched, [op][energy][x]
    long long *colTab = reinterpret_cast<long long *>(sm + ct_off + 4 * (size_t)nraw * ncol);
    const size_t mb_off = ct_off + 4 * (size_t)nraw * ncol + 8 * (size_t)ncol;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + mb_off);   // [9 + nraw]
    uint64_t *win_full = mbar, *win_empty = mbar + 2, *acc_full = mbar + 4, *acc_empty = mbar + 6;
    uint64_t *never = mbar + 8;    // fault injection: a barrier nothing arrives on
    uint64_t *raw_full = mbar + 9; // raw buffer r: its bulk copies landed
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mbar + 13);
    constexpr int NW = TCW_EPI + TCW_PROD;

    if (tid < NW) {
        if (!p.a_tmem) {
            const uint4 *src = p.Aimg;
            uint4 *dst = reinterpret_cast<uint4 *>(smA);
            const int nv = 2 * p.a_bytes / 16;
            for (int i = tid; i < nv; i += NW) dst[i] = src[i];
        }
        // K entry r = dy*orbitals + o of a window row -> float offset inside a raw column
        // (u: element [o][a] at Y-offset dy; s: element [a][o + coff] at the reflected
        // Y-offset, coff = bands/2 in the Josephson mode: the hole-block column)
        for (int i = tid; i < 2 * NKC * 8; i += NW) {
            const int op = i >= NKC * 8, r = i - op * NKC * 8;
            int v = -1;
            if (r < nval) {
                const int dyw = r / p.mb, o = p.bs0 + r % p.mb;
                v = op == 0 ? 2 * (dyw * bb + o * p.b) : 2 * ((2 * p.w - dyw) * bb + o + p.coff);
            }
            offR[i] = v;
        }
        if (tid < 4) raw[zslot + tid] = 0.f;
        for (int i = tid; i < nraw * ncol; i += NW) shTab[i] = 0;
    }
    if (tid == NW) {
        // acc_empty[s] completes when every epilogue warp has arrived
        // raw_full[r] (i >= 9) completes on one expect-tx arrival and every producer thread's
        // cp.async arrival
        for (int i = 0; i < 9 + nraw; i++)
            mbar_init(smem_u32(&mbar[i]), (i == 6 || i == 7) ? TCW_EPI / 32 : i >= 9 ? 1 + TCW_PROD : 1);
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(smem_u32(tmem_slot), p.tmem_cols);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    // A operand in tensor memory: columns [acol, acol + KP/2) hold Phi hi and the next KP/2
    // columns Phi lo; warps 0-3 write their lane quarter, row m = lane, from the image
    const uint32_t acol = (uint32_t)(2 * setcols);
    if (p.a_tmem && warp < 4) {
        const int m = warp * 32 + lane;
        const unsigned char *img = reinterpret_cast<const unsigned char *>(p.Aimg);
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        for (int hl = 0; hl < 2; hl++)
            for (int ks = 0; ks < (p.KP >> 4); ks++) {
                uint32_t v[8];
                for (int c = 0; c < 2; c++) {
                    const uint4 q = *reinterpret_cast<const uint4 *>(img + (size_t)hl * p.a_bytes + (size_t)(m >> 3) * sbo_a +
                                                                     (size_t)(2 * ks + c) * 128 + (m & 7) * 16);
                    v[4 * c + 0] = q.x; v[4 * c + 1] = q.y; v[4 * c + 2] = q.z; v[4 * c + 3] = q.w;
                }
                tmem_st8(trow + acol + (uint32_t)(hl * (p.KP >> 1) + ks * 8), v);
            }
        tmem_wait_st();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const int neb = (p.ne + EB - 1) / EB;
    const int ntiles = neb * p.n * p.ntx;
    // tile t -> (first energy e0, site row j, first site i0)
    auto tile_of = [&](int it, int &e0, int &j, int &i0) {
        const int t = blockIdx.x + it * gridDim.x;
        if (t >= ntiles) return false;
        const int per_e = p.n * p.ntx;
        const int eb = t / per_e;
        const int rr = t - eb * per_e;
        e0 = eb * EB;
        j = rr / p.ntx;
        i0 = (rr - j * p.ntx) * TS;
        return true;
    };

    if (warp == NW / 32) {
        // ---------------------------------------------------------------- MMA warp
        const uint32_t idesc = idesc_f16(128, NMMA);
        const uint64_t aH = sdesc(smem_u32(smA), 128, sbo_a), aL = sdesc(smem_u32(smA + p.a_bytes), 128, sbo_a);
        const uint32_t lbo_b = (uint32_t)(nplanes * NX * 16), sbo_b = (uint32_t)(NX * 16);
        int issued = 0;
        // fault injection (tests): wait on a barrier nothing arrives on; the bounded wait
        // runs out and every role takes the time-out path
        bool ok = !(p.stall && !mbar_wait(smem_u32(never), 0, p.spin_limit));
        for (int it = 0; ok; it++) {
            int e0, j, i0;
            if (!tile_of(it, e0, j, i0)) break;
            const int s = it & 1;
            if (!mbar_wait(smem_u32(&win_full[s]), (it >> 1) & 1, p.spin_limit) ||
                (it >= 2 && !mbar_wait(smem_u32(&acc_empty[s]), ((it - 2) >> 1) & 1, p.spin_limit))) {
                ok = false;
                break;
            }
            tc_fence_after();
            if (lane == 0) {
                const unsigned char *Wb = smW + (size_t)s * 2 * p.win_bytes;
                const uint64_t bH = sdesc(smem_u32(Wb), lbo_b, sbo_b);
                const uint64_t bL = sdesc(smem_u32(Wb + p.win_bytes), lbo_b, sbo_b);
                for (int g = 0; g < p.H; g++) {
                    const uint32_t d = tmem + (uint32_t)(s * setcols + g * NMMA);
                    uint32_t acc_flag = 0u;
                    for (int dxw = 0; dxw < side; dxw++)
                        for (int cp = 0; cp < (NKC >> 1); cp++) {
                            // descriptor address fields count 16-byte units
                            const uint64_t bo = (uint64_t)((2 * cp * nplanes) * NX + 8 * g + dxw);
                            if (p.a_tmem) {
                                // k-step (dxw, cp) = 16 K values = 8 columns of A
                                const uint32_t ac = tmem + acol + (uint32_t)((dxw * NKC + 2 * cp) * 4);
                                const uint32_t acl = ac + (uint32_t)(p.KP >> 1);
                                mma_f16_ta(d, ac, bH + bo, idesc, acc_flag);
                                mma_f16_ta(d, ac, bL + bo, idesc, 1u);
                                mma_f16_ta(d, acl, bH + bo, idesc, 1u);
                            } else {
                                const uint64_t ao = (uint64_t)((dxw * NKC + 2 * cp) * 8);
                                mma_f16(d, aH + ao, bH + bo, idesc, acc_flag);
                                mma_f16(d, aH + ao, bL + bo, idesc, 1u);
                                mma_f16(d, aL + ao, bH + bo, idesc, 1u);
                            }
                            acc_flag = 1u;
                        }
                }
                mma_commit(smem_u32(&acc_full[s]));
                mma_commit(smem_u32(&win_empty[s]));
            }
            __syncwarp();
            issued++;
        }
        if (!ok && lane == 0) atomicOr(p.status, 2);
        // the accumulator sets must be idle before the tensor memory is freed
        for (int k = issued > 2 ? issued - 2 : 0; k < issued; k++)
            mbar_wait(smem_u32(&acc_full[k & 1]), (k >> 1) & 1, p.spin_limit);
    } else if (warp >= TCW_EPI / 32) {
        // ---------------------------------------------------------------- producer
        const int ptid = tid - TCW_EPI;
        // staging items: the re and im plane rows (kchunk, operand, energy, band, x) of one
        // complex window column, converted together from 8-byte (re, im) loads; the first
        // three items of this thread are the same in every tile, so they are decomposed once.
        // cidx: the item's raw column [op][energy][x]
        const int nitems = NKC * (nplanes >> 1) * NX;
        auto item_of = [&](int it, int &rbase, int &toff, int &dst, int &eei, int &cidx) {
            const int pp = it / NX, xl = it - pp * NX;
            const int a = pp % p.b;
            const int rest = pp / p.b;
            const int ee = rest % EB;
            const int rest2 = rest / EB;
            const int op = rest2 & 1, kc = rest2 >> 1;
            const int plane = ((kc * 2 + op) * EB + ee) * twob + 2 * a;   // the re plane; im follows
            // the s operand reads its columns in reverse x order
            cidx = (op * EB + ee) * NX + (op ? NX - 1 - xl : xl);
            rbase = 2 * cidx * cpf + (op ? 2 * a * p.b : 2 * a);
            toff = op * NKC * 8 + kc * 8;
            dst = (plane * NX + xl) * 16;
            eei = op * EB + ee;   // operand and energy: the s operand may carry its own scale
        };
        int r0 = 0, t0 = 0, d0 = 0, q0 = 0, c0 = 0, r1 = 0, t1 = 0, d1 = 0, q1 = 0, c1 = 0;
        int r2 = 0, t2 = 0, d2 = 0, q2 = 0, c2 = 0;
        if (ptid < nitems) item_of(ptid, r0, t0, d0, q0, c0);
        if (ptid + TCW_PROD < nitems) item_of(ptid + TCW_PROD, r1, t1, d1, q1, c1);
        if (ptid + 2 * TCW_PROD < nitems) item_of(ptid + 2 * TCW_PROD, r2, t2, d2, q2, c2);
        // split scale of (operand, energy) qq = op * EB + ee: the s operand of the folded form is
        // T G0 with its own maximum
        auto scale_of = [&](int e0, int qq) {
            const bool sop = qq >= EB;
            const int e = e0 + (sop ? qq - EB : qq);
            if (e >= p.ne) return 1.f;
            return pow2_scale((sop && p.gmaxT) ? p.gmaxT[e] : p.gmax[e]);
        };
        // raw column ptid = (op, energy, x) of a tile, for threads ptid < ncol
        int my_op = 0, my_ee = 0, my_xl = 0;
        if (ptid < ncol) {
            const int w_ = ptid / NX;
            my_xl = ptid - w_ * NX;
            my_op = w_ / EB;
            my_ee = w_ - my_op * EB;
        }
        const uint32_t colbytes = (uint32_t)cpf * 8u;
        const long long sofs = FOLD ? (long long)(((uintptr_t)p.boxT - (uintptr_t)p.box) / sizeof(float2)) : 0LL;
        // column table of a tile: source offset (float2 units from p.box, -1 outside the box
        // and past the last energy) of every raw column (threads < ncol; read after a
        // producer barrier)
        auto column_table = [&](int e0, int j, int i0) {
            if (ptid < ncol) {
                const int py = j - n2, px0 = i0 - n2, e = e0 + my_ee;
                const int X = my_op == 0 ? px0 - p.w + my_xl : -px0 - (TS - 1) - p.w + my_xl;
                const int Y0 = my_op == 0 ? py - p.w : -py - p.w;
                const bool in = e < p.ne && X >= -p.Rb && X <= p.Rb;
                // the s columns of the folded form read T G0: offset of boxT from box (both
                // allocations 256-byte aligned, so the offset is even)
                const long long base = (FOLD && my_op == 1) ? sofs : 0LL;
                colTab[ptid] = in ? base + ((long long)e * p.NB * p.NB + (long long)(X + p.Rb) * p.NB + (Y0 + p.Rb)) * bb
                                  : -1LL;
            }
        };
        // copies: the first nbulk columns one bulk copy each (thread ptid < nbulk: cpf complex
        // values from the 16-byte boundary at or below the column's first value; the source
        // boxes have 16 bytes of slack at their end; zeros from p.zsrc), the rest as 8-byte
        // cp.async pieces (zero-filled), issued by every producer thread in column-major order
        // and advanced without divisions.  The bulk columns' shifts (0 or 2 floats) go to
        // shTab (the other entries stay 0).  With bulk copies raw_full[rb] completes on ptid
        // 0's arrival with the bulk bytes and every producer thread's cp.async arrival (noinc:
        // counted in the barrier's initial count); without, each fetch is one cp.async group
        // (measured: the 288 mbarrier arrivals per tile cost the 3-band contraction 7%).
        const int nbulk = BULK ? (p.nbulk < ncol ? p.nbulk : ncol) : 0;
        const int ncopy = (ncol - nbulk) * rowlen;
        const int col0 = nbulk + ptid / rowlen, pc0 = ptid % rowlen;
        const int dcol = TCW_PROD / rowlen, dpc = TCW_PROD - dcol * rowlen;
        auto fetch_raw = [&](int rb) {
            const uint32_t bar = smem_u32(&raw_full[rb]);
            float *rawb = raw + rb * rawbuf;
            if (nbulk > 0 && ptid == 0) mbar_arrive_expect(bar, (uint32_t)nbulk * colbytes);
            if (ptid < nbulk) {
                const long long so = colTab[ptid];
                const int sh = so >= 0 ? (int)(so & 1) : 0;
                const float2 *src = so >= 0 ? p.box + (so - sh) : p.zsrc;
                shTab[rb * ncol + ptid] = 2 * sh;
                bulk_load(smem_u32(rawb + 2 * ptid * cpf), src, colbytes, bar);
            }
            int col = col0, pc = pc0;
            for (int idx = ptid; idx < ncopy; idx += TCW_PROD) {
                const long long so = colTab[col];
                const float2 *src = so >= 0 ? p.box + so + pc : p.box;
                cp_async8(smem_u32(rawb + 2 * (col * cpf + pc)), src, so >= 0 ? 8u : 0u);
                col += dcol;
                pc += dpc;
                if (pc >= rowlen) { pc -= rowlen; col++; }
            }
            if (nbulk > 0) cp_async_mbar_arrive(bar);
            else cp_async_commit();
        };
        // raw windows -> scaled, split fp16 rows in window buffer Wb (hi) and Wb + win_bytes (lo):
        // the re row at dst, the im row one plane (NX rows) later; every raw offset is even, so
        // a (re, im) pair is one 8-byte load
        const float2 *raw2 = reinterpret_cast<const float2 *>(raw);
        auto split_row = [&](unsigned char *d, const float (&v)[8]) {
            uint32_t hw[4], lw[4];
#pragma unroll
            for (int kk = 0; kk < 4; kk++) {
                const __half2 hh = __floats2half2_rn(v[2 * kk], v[2 * kk + 1]);
                const float2 hb = __half22float2(hh);
                const __half2 ll = __floats2half2_rn(v[2 * kk] - hb.x, v[2 * kk + 1] - hb.y);
                hw[kk] = *reinterpret_cast<const uint32_t *>(&hh);
                lw[kk] = *reinterpret_cast<const uint32_t *>(&ll);
            }
            *reinterpret_cast<uint4 *>(d) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
            *reinterpret_cast<uint4 *>(d + p.win_bytes) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        };
        auto convert_item = [&](unsigned char *Wb, int rb, int rbase, int toff, int dst, float sB, int cidx) {
            const int4 *t4 = reinterpret_cast<const int4 *>(offR + toff);
            const int4 ta = t4[0], tb = t4[1];
            const int offs[8] = {ta.x, ta.y, ta.z, ta.w, tb.x, tb.y, tb.z, tb.w};
            const int cb = rb * rawbuf + rbase + (nbulk > 0 ? shTab[rb * ncol + cidx] : 0);
            float vr[8], vi[8];
#pragma unroll
            for (int kk = 0; kk < 8; kk++) {
                const float2 v = raw2[(offs[kk] < 0 ? zslot : cb + offs[kk]) >> 1];
                vr[kk] = v.x * sB;
                vi[kk] = v.y * sB;
            }
            split_row(Wb + dst, vr);
            split_row(Wb + dst + NX * 16, vi);
        };
        bool ok = true;
        int e0, j, i0;
        int se = -1;
        float sB0 = 1.f, sB1 = 1.f, sB2 = 1.f;
        // raw windows run nraw-1 tiles ahead; tile k uses raw buffer k % nraw, the
        // (k / nraw)-th phase of raw_full[k % nraw].  Every decision below is uniform over the
        // producer threads, so nfetch (tiles fetched) is the same in each.
        int nfetch = 0;
        for (int k = 0; k < nraw; k++) {
            int ke, kj, ki0;
            const bool has = tile_of(k, ke, kj, ki0);
            if (has) column_table(ke, kj, ki0);
            bar_sync_group<2, TCW_PROD>();
            if (k == nraw - 1) break;                 // its table is used by the first iteration
            if (has) {
                fetch_raw(k);
                nfetch++;
            } else if (nbulk == 0) {
                cp_async_commit();                    // one group per tile slot
            }
            bar_sync_group<2, TCW_PROD>();
        }
        int it = 0;
        for (;; it++) {
            if (!tile_of(it, e0, j, i0)) break;
            const int s = it & 1;
            // the tile nraw-1 ahead goes to the raw buffer last read by the previous
            // iteration's convert, which finished before that iteration's final barrier
            int ne_, nj, ni0;
            const int ahead = it + nraw - 1;
            if (tile_of(ahead, ne_, nj, ni0)) {   // table computed last iteration
                fetch_raw(ahead % nraw);
                nfetch++;
            } else if (nbulk == 0) {
                cp_async_commit();
            }
            const int rb = it % nraw;
            bool good = it < 2 || mbar_wait(smem_u32(&win_empty[s]), ((it - 2) >> 1) & 1, p.spin_limit);
            if (nbulk > 0) {
                good = good && mbar_wait(smem_u32(&raw_full[rb]), (it / nraw) & 1, p.spin_limit);
            } else {
                // all but the newest nraw-1 groups landed: this tile's windows
                if (nraw == 4) cp_async_wait_n<3>();
                else if (nraw == 3) cp_async_wait_n<2>();
                else cp_async_wait_n<1>();
            }
            // (this barrier also makes every thread's landed copies and the shift-table
            // writes of earlier fetches visible to the reads below)
            if (bar_or_group<2, TCW_PROD>(!good)) {
                ok = false;
                break;
            }
            if (e0 != se) {
                sB0 = scale_of(e0, q0);
                sB1 = scale_of(e0, q1);
                sB2 = scale_of(e0, q2);
                se = e0;
            }
            unsigned char *Wb = smW + (size_t)s * 2 * p.win_bytes;
            if (ptid < nitems) convert_item(Wb, rb, r0, t0, d0, sB0, c0);
            if (ptid + TCW_PROD < nitems) convert_item(Wb, rb, r1, t1, d1, sB1, c1);
            if (ptid + 2 * TCW_PROD < nitems) convert_item(Wb, rb, r2, t2, d2, sB2, c2);
            for (int k = ptid + 3 * TCW_PROD; k < nitems; k += TCW_PROD) {
                int rb_, to_, ds_, q_, c_;
                item_of(k, rb_, to_, ds_, q_, c_);
                convert_item(Wb, rb, rb_, to_, ds_, scale_of(e0, q_), c_);
            }
            // every copy of this iteration was issued before the barrier above, so the table
            // can now describe the tile fetched next iteration
            if (tile_of(ahead + 1, ne_, nj, ni0)) column_table(ne_, nj, ni0);
            fence_proxy_async();
            bar_sync_group<2, TCW_PROD>();           // buffer staged, raw buffer rb free
            if (ptid == 0) mbar_arrive(smem_u32(&win_full[s]));
        }
        if (!ok) {
            if (ptid == 0) atomicOr(p.status, 2);
            // bulk copies still in flight land before the block exits (bounded waits)
            if (nbulk > 0)
                for (int k = it; k < nfetch; k++) mbar_wait(smem_u32(&raw_full[k % nraw]), (k / nraw) & 1, p.spin_limit);
        }
        cp_async_commit();
        cp_async_wait_all();
    } else {
        // ---------------------------------------------------------------- epilogue
        const int lq = tid & 127;
        const int qx = lq % p.os, qy = lq / p.os;
        const bool qvalid = lq < p.Q;
        const int sub = warp >> 2;                                // 0, 1: the two warps of a lane quarter
        const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
        const int nb = B <= 4 ? B : p.b;                          // bands; a constant for B <= 4
        const int ncombo = EB * (TS >> 2);                        // (energy, 4-site group) pairs per tile
        constexpr bool jos = JOS;                                 // Josephson mode
        constexpr bool fold = FOLD;                               // T folded into the s operand
        // T, the scale and term1 of an energy block, loaded once per block (after every
        // epilogue warp has finished the previous block's tiles)
        auto load_block = [&](int e0) {
            bar_sync_group<1, TCW_EPI>();
            for (int i = tid; i < EB * p.nimp * bb; i += TCW_EPI) {
                const int e = e0 + i / (p.nimp * bb);
                cT[i] = e < p.ne ? p.T32[(size_t)e0 * p.nimp * bb + i] : make_float2(0.f, 0.f);
            }
            for (int i = tid; i < EB * 128; i += TCW_EPI) {
                const int ee = i >> 7, q = i & 127, e = e0 + ee;
                cT1[i] = (e < p.ne && q < p.Q) ? (float)p.term1[(size_t)e * p.Q + (q % p.os) * p.os + q / p.os] : 0.f;
            }
            if (tid < EB) {
                const int e = e0 + tid;
                const float inv = e < p.ne ? p.inv_sA / pow2_scale(p.gmax[e]) : 0.f;
                const float invs = (e < p.ne && p.gmaxT) ? p.inv_sA / pow2_scale(p.gmaxT[e]) : inv;
                cInv2[tid] = inv * invs;
                const double2 tp = (p.tip && e < p.ne) ? p.tip[e] : make_double2(0.0, 0.0);
                cTip[2 * tid] = (float)tp.x;
                cTip[2 * tid + 1] = (float)tp.y;
            }
            bar_sync_group<1, TCW_EPI>();
        };
        auto epilogue = [&](int accs, int e0, int j, int i0) {
            const uint32_t acc = tmem + (uint32_t)(accs * setcols);
            for (int imp = 0; imp < p.nimp; imp++) {
                for (int cmb = sub; cmb < ncombo; cmb += 2) {
                    const int ee = cmb / (TS >> 2), s0 = (cmb - ee * (TS >> 2)) * 4;
                    const int e = e0 + ee;
                    if (e >= p.ne) continue;
                    const float inv2 = cInv2[ee];
                    const float2 *Te = cT + (ee * p.nimp + imp) * bb;
                    const float t1 = cT1[ee * 128 + lq];
                    const uint32_t cb = (uint32_t)((s0 >> 3) * NMMA + ee * twob * 8 + (s0 & 7));
                    // sites per TMEM read: 4, or 2 for more than 4 bands (u and s of 4 sites
                    // would not fit the 96-register cap of 576 threads)
                    constexpr int SU = B > 4 ? 2 : 4;
#pragma unroll
                    for (int hs = 0; hs < 4; hs += SU) {
                    float ur[2 * B][SU], sr[2 * B][SU];
#pragma unroll
                    for (int ari = 0; ari < 2 * B; ari++) {
                        if (ari < 2 * nb) {
                            const uint32_t cu = cb + (uint32_t)(ari * 8 + hs);
                            if constexpr (SU == 4) {
                                tmem_ld4(acc + lane_base + cu, ur[ari][0], ur[ari][1], ur[ari][2], ur[ari][3]);
                                tmem_ld4(acc + lane_base + cu + (uint32_t)opcols, sr[ari][0], sr[ari][1], sr[ari][2], sr[ari][3]);
                            } else {
                                tmem_ld2(acc + lane_base + cu, ur[ari][0], ur[ari][1]);
                                tmem_ld2(acc + lane_base + cu + (uint32_t)opcols, sr[ari][0], sr[ari][1]);
                            }
                        }
                    }
                    tmem_wait_ld();
                    float term2[SU], term2r[SU];
#pragma unroll
                    for (int u = 0; u < SU; u++) term2[u] = term2r[u] = 0.f;
                    if (fold) {
                        // the s accumulators already hold (T s)_a
#pragma unroll
                        for (int a = 0; a < B; a++) {
                            if (a >= nb) continue;
#pragma unroll
                            for (int u = 0; u < SU; u++) {
                                term2[u] += ur[2 * a][u] * sr[2 * a + 1][u] + ur[2 * a + 1][u] * sr[2 * a][u];
                                if (jos) term2r[u] += ur[2 * a][u] * sr[2 * a][u] - ur[2 * a + 1][u] * sr[2 * a + 1][u];
                            }
                        }
                    }
#pragma unroll
                    for (int a = 0; a < B; a++) {
                        if (a >= nb || fold) continue;
                        float tsr[SU], tsi[SU];
#pragma unroll
                        for (int u = 0; u < SU; u++) tsr[u] = tsi[u] = 0.f;
#pragma unroll
                        for (int c = 0; c < B; c++) {
                            if (c >= nb) continue;
                            const float2 tv = Te[a * nb + c];
#pragma unroll
                            for (int u = 0; u < SU; u++) {
                                tsr[u] += tv.x * sr[2 * c][u] - tv.y * sr[2 * c + 1][u];
                                tsi[u] += tv.x * sr[2 * c + 1][u] + tv.y * sr[2 * c][u];
                            }
                        }
#pragma unroll
                        for (int u = 0; u < SU; u++) term2[u] += ur[2 * a][u] * tsi[u] + ur[2 * a + 1][u] * tsr[u];
                        if (jos) {
#pragma unroll
                            for (int u = 0; u < SU; u++) term2r[u] += ur[2 * a][u] * tsr[u] - ur[2 * a + 1][u] * tsi[u];
                        }
                    }
                    if (jos) {
                        // Im(tip * sum u T s) (tmatrix::calcwannierjosephson, src/qpi.cc:986-990)
                        const float tx = cTip[2 * ee], ty = cTip[2 * ee + 1];
#pragma unroll
                        for (int u = 0; u < SU; u++) term2[u] = tx * term2[u] + ty * term2r[u];
                    }
                    // pixel (qx, qy) of sites i0+s0+hs .. of row j, straight to the map
                    if (qvalid && p.fov) {
                        // map (e, imp) covers the centred fov x fov sites of the full field
                        const int mi = e * p.nimp + imp;
                        const int fv = p.fov[mi], f2 = fv >> 1;
                        const int jm = j - n2 + f2;
                        if (jm >= 0 && jm < fv) {
                            const size_t wm = (size_t)fv * p.os;
                            float *dst = p.out + p.fov_off[mi] + ((size_t)jm * p.os + qy) * wm + qx;
#pragma unroll
                            for (int u = 0; u < SU; u++) {
                                const int im = i0 + s0 + hs + u - n2 + f2;
                                if (im >= 0 && im < fv) dst[(size_t)im * p.os] = (-t1 - term2[u] * inv2) * p.scale;
                            }
                        }
                    } else if (qvalid) {
                        float *dst = p.out + ((((size_t)e * p.nimp + imp) * p.wn + (size_t)j * p.os + qy) * p.wn +
                                              (size_t)(i0 + s0) * p.os + qx);
                        const int xrem = p.wn - (i0 + s0) * p.os - qx;   // columns left in this map row
#pragma unroll
                        for (int u = 0; u < SU; u++)
                            if ((hs + u) * p.os < xrem) dst[(hs + u) * p.os] = (-t1 - term2[u] * inv2) * p.scale;
                    }
                    }
                }
            }
            // this warp's TMEM reads of the accumulator set are done: its arrival on
            // acc_empty (one per epilogue warp) hands the set back to the MMA warp
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&acc_empty[accs]));
        };
        // Epilogue warps run independently (no barrier per tile).  Every warp walks the same
        // tiles, so the barriers of the energy-block changes stay matched after a time-out:
        // from then on a warp skips the waits and the work but not the block changes.  The
        // time-out decision is made uniform within a warp (its TMEM loads are warp-wide).
        bool ok = true;
        int cur_e0 = -1;
        for (int it = 0;; it++) {
            int e0, j, i0;
            if (!tile_of(it, e0, j, i0)) break;
            if (e0 != cur_e0) {
                load_block(e0);
                cur_e0 = e0;
            }
            if (!ok) continue;
            const int s = it & 1;
            ok = __all_sync(0xffffffffu, mbar_wait(smem_u32(&acc_full[s]), (it >> 1) & 1, p.spin_limit));
            if (!ok) continue;
            tc_fence_after();
            epilogue(s, e0, j, i0);
        }
        if (!ok && lane == 0) atomicOr(p.status, 2);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, p.tmem_cols);
    }
}

__global__ void widen_kernel(const float *__restrict__ src, double *__restrict__ dst, size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (double)src[i];
}

void launch_widen(cqpi_handle *h, const float *src, double *dst, size_t n)
{
    const unsigned grid = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)h->num_sms * 8);
    widen_kernel<<<grid ? grid : 1, 256, 0, h->stream>>>(src, dst, n);
    h->launches++;
}

// ------------------------------------------------------------------ host side
bool tc_supported(const cqpi_handle *h) { return h->Q <= 128 && h->b <= CQPI_MAX_BANDS; }

void tc_plan(cqpi_handle *h)
{
    TcPlan &pl = h->tc;
    const int twob = 2 * h->b;
    // TS: multiple of 4 (4-site TMEM loads), N = TS*2b a multiple of 16
    int TS = 0;
    for (int t = 32; t >= 4; t -= 4)
        if ((t * twob) % 16 == 0 && t * twob <= 128) { TS = t; break; }
    if (!TS)
        for (int t = 32; t >= 4; t -= 4)
            if ((t * twob) % 16 == 0 && t * twob <= 256) { TS = t; break; }
    pl.TS = TS;
    pl.N = TS * twob;
    pl.KP = ((h->W * h->mb + 15) / 16) * 16;
    int cols = 2 * h->nblk * pl.N, tc = 32;
    while (tc < cols) tc <<= 1;
    pl.tmem_cols = tc;
    pl.a_bytes = 128 * pl.KP * 2;
    pl.b_bytes = pl.N * pl.KP * 2;
    const size_t wfl = (size_t)(TS + 2 * h->w) * (2 * h->w + 1) * h->b * h->b * 2;
    const int wt = TS * h->os;
    pl.sst = wt + ((h->os - wt) % 32 + 32) % 32;   // row r starts on bank r*os: conflict-free q writes
    pl.smem = (size_t)h->nblk * 2 * pl.a_bytes + 4 * (size_t)pl.b_bytes + 4 * (2 * (wfl + 4)) +
              4 * (size_t)(2 * h->nblk * pl.KP + 2 * pl.N) + 4 * (size_t)((h->os * pl.sst + 3) & ~3) + 64;
    pl.ok = TS > 0 && cols <= 512 && pl.smem <= 227 * 1024;
    // pipelined variant (one spin block): two B buffers, two accumulator sets
    int pcols = 32;
    while (pcols < 4 * pl.N) pcols <<= 1;
    pl.pipe_tmem_cols = pcols;
    pl.pipe_smem = 2 * (size_t)pl.a_bytes + 8 * (size_t)pl.b_bytes + 4 * (2 * (wfl + 4)) +
                   4 * (size_t)(2 * pl.KP + 2 * pl.N) + 4 * (size_t)((h->os * pl.sst + 3) & ~3) + 64;
    pl.pipe = pl.ok && h->nblk == 1 && 4 * pl.N <= 512 && pl.pipe_smem <= 227 * 1024;

    // direct-window variant: tiles of 8*H sites x EB energies; one MMA covers both operands
    // and all EB energies of an 8-site group (N = 32*b*EB <= 256).  The MMA count per
    // site-energy falls with EB only, so the default maximises EB, then H, with the deepest
    // raw-window ring that fits; cqpi_autotune times every valid shape instead.
    pl.win = false;
    for (int EB = 4; EB >= 1 && !pl.win; EB--)
        for (int H = 2; H >= 1 && !pl.win; H--)
            for (int nraw = 4; nraw >= 2 && !pl.win; nraw--) window_config(h, EB, H, nraw, pl);
}

// band counts whose direct-window kernel has a bulk-copy variant (templates B = 3, 6 and 8;
// for 3 bands only autotuning takes it: with many impurities per map the epilogue is the
// limit, and bulk copies leave it the issue slots of the producer's cp.async pieces)
static bool tcw_bulk_bands(int b) { return b == 3 || (b >= 5 && b <= 8); }

// Fill the direct-window fields of pl for EB energies x 8*H sites per tile and an nraw-deep
// raw-window ring; false if the shape does not fit (N <= 256, two accumulator sets in the
// 512 TMEM columns, shared memory with 16 KiB left for the per-impurity constants).
bool window_config(const cqpi_handle *h, int EB, int H, int nraw, TcPlan &pl)
{
    if (h->nblk != 1 || h->Q > 128) return false;
    const int twob = 2 * h->b, side = 2 * h->w + 1;
    const int NKC = 2 * ((side * h->mb + 15) / 16);
    const int KP = side * NKC * 8;
    const int N = 32 * h->b * EB;
    if (N > 256) return false;
    const int setcols = H * N;
    if (2 * setcols > 512) return false;
    const int NX = 8 * H + 2 * h->w;
    const bool a_tmem = 2 * setcols + KP <= 512;
    const int need = 2 * setcols + (a_tmem ? KP : 0);
    int wc = 32;
    while (wc < need) wc <<= 1;
    const int a_bytes = 128 * KP * 2;
    const int win_bytes = NKC * 2 * EB * twob * NX * 16;
    const int wwt = 8 * H * h->os;
    const int sst = wwt + ((h->os - wwt) % 32 + 32) % 32;
    // raw column pitch: side*b*b complex values + 1, rounded up to even (16-byte bulk copies)
    const size_t cpf = (size_t)((side * h->b * h->b + 2) & ~1);
    const size_t rawfl = (size_t)NX * cpf * 2;
    // shared memory with Phi in shared memory (the larger of the two layouts); the
    // per-impurity epilogue constants are added at launch.  After the constants: the
    // column shift table [nraw][2*EB*NX], the column table [2*EB*NX], 9 + nraw mbarriers and
    // the TMEM slot
    const size_t smem = 2 * (size_t)a_bytes + 4 * (size_t)win_bytes + 4 * (nraw * 2 * EB * rawfl + 4) +
                        4 * (size_t)(2 * NKC * 8) + 4 * (size_t)EB * (3 + 128) + 16 + 4 * (size_t)nraw * (2 * EB * NX) +
                        8 * (size_t)(2 * EB * NX) + 13 * 8 + 16;
    if (smem > 211 * 1024) return false;
    pl.wNKC = NKC; pl.wKP = KP; pl.w_a_bytes = a_bytes;
    pl.wNRAW = nraw; pl.wEB = EB; pl.wH = H; pl.wNX = NX; pl.w_win_bytes = win_bytes; pl.w_sst = sst;
    // bulk copies pay off for long raw columns (measured: 6-band columns of 1.4 KB fetched in
    // bulk cut the Josephson contraction by 16%; 3-band columns of 360 B ran 13% slower)
    pl.w_nbulk = (tcw_bulk_bands(h->b) && side * h->b * h->b * 8 >= 1024) ? 2 * EB * NX : 0;
    pl.w_a_tmem = a_tmem; pl.w_tmem_cols = wc; pl.w_smem = smem;
    pl.win = true;
    return true;
}

// Time every valid direct-window shape and raw-column fetch on the current energy batch
// (workspace already holds G0(R), T and term1 for ne energies) and keep the fastest.
// out: ne*nimp maps of scratch.
cudaError_t tc_autotune(cqpi_handle *h, int ne, float *out, float *best_ms, int *tried)
{
    TcPlan best = h->tc;
    float best_t = -1.f;
    int n = 0;
    cudaEvent_t e0, e1;
    cudaError_t err = cudaEventCreate(&e0);
    if (err != cudaSuccess) return err;
    err = cudaEventCreate(&e1);
    if (err != cudaSuccess) { cudaEventDestroy(e0); return err; }
    const TcPlan base = h->tc;
    for (int EB = 1; EB <= 4 && err == cudaSuccess; EB++)
        for (int H = 1; H <= 4 && err == cudaSuccess; H *= 2)
            for (int nraw = 2; nraw <= 4 && err == cudaSuccess; nraw++)
                for (int bulk = 0; bulk < (tcw_bulk_bands(h->b) ? 2 : 1) && err == cudaSuccess; bulk++) {
                    TcPlan pl = base;
                    if (!window_config(h, EB, H, nraw, pl)) continue;
                    // raw columns by cp.async only, or all by bulk copies
                    pl.w_nbulk = bulk ? 2 * EB * pl.wNX : 0;
                    h->tc = pl;
                    if (!tc_window_usable(h)) continue;
                    err = launch_ldos_tc(h, ne, out);                 // warm-up
                    if (err != cudaSuccess) break;
                    err = cudaEventRecord(e0, h->stream);
                    for (int r = 0; r < 3 && err == cudaSuccess; r++) err = launch_ldos_tc(h, ne, out);
                    if (err == cudaSuccess) err = cudaEventRecord(e1, h->stream);
                    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
                    float ms = 0.f;
                    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
                    if (err != cudaSuccess) break;
                    n++;
                    if (best_t < 0.f || ms < best_t) { best_t = ms; best = pl; }
                }
    h->tc = (best_t >= 0.f) ? best : base;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best_ms) *best_ms = best_t / 3.f;
    if (tried) *tried = n;
    return err;
}

// Phi hi/lo images for the direct-window variant: rows m = qy*os + qx, columns
// k = dx * 8*NKC + dy*orbitals + o (zero elsewhere); same power-of-two scale as tc_build_a.
void tc_build_a_window(cqpi_handle *h, const std::vector<double> &phi, std::vector<uint16_t> &img)
{
    const TcPlan &pl = h->tc;
    double mx = 0.0;
    for (double v : phi) mx = std::max(mx, std::fabs(v));
    int ex = 0;
    if (mx > 0) std::frexp(mx, &ex);
    const double sA = mx > 0 ? std::ldexp(1.0, 14 - ex) : 1.0;
    const size_t per = pl.w_a_bytes / 2;
    img.assign(2 * per, 0);
    const int sbo = pl.wKP * 16, side = 2 * h->w + 1;
    for (int qy = 0; qy < h->os; qy++)
        for (int qx = 0; qx < h->os; qx++) {
            const int m = qy * h->os + qx;
            for (int d = 0; d < h->W; d++) {
                const int dxw = d / side, dyw = d % side;
                for (int ol = 0; ol < h->mb; ol++) {
                    const double v = sA * phi[(((size_t)qx * h->os + qy) * h->W + d) * h->mb + ol];
                    const __half hi = __float2half_rn((float)v);
                    const __half lo = __float2half_rn((float)(v - (double)__half2float(hi)));
                    const int k = dxw * pl.wNKC * 8 + dyw * h->mb + ol;
                    const size_t off = ((size_t)(m >> 3) * sbo + (k >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2) / 2;
                    img[off] = __half_as_ushort(hi);
                    img[per + off] = __half_as_ushort(lo);
                }
            }
        }
}

// Phi hi/lo images in the operand layout: rows m = qy*os + qx, columns k = d*mb + ol.
void tc_build_a(cqpi_handle *h, const std::vector<double> &phi, std::vector<uint16_t> &img, float &inv_sA)
{
    const TcPlan &pl = h->tc;
    double mx = 0.0;
    for (double v : phi) mx = std::max(mx, std::fabs(v));
    int ex = 0;
    if (mx > 0) std::frexp(mx, &ex);
    const double sA = mx > 0 ? std::ldexp(1.0, 14 - ex) : 1.0;
    inv_sA = (float)(1.0 / sA);
    const size_t per = pl.a_bytes / 2;
    img.assign((size_t)h->nblk * 2 * per, 0);
    const int sbo = pl.KP * 16;
    for (int blk = 0; blk < h->nblk; blk++)
        for (int qy = 0; qy < h->os; qy++)
            for (int qx = 0; qx < h->os; qx++) {
                const int m = qy * h->os + qx;
                for (int d = 0; d < h->W; d++)
                    for (int ol = 0; ol < h->mb; ol++) {
                        const double v = sA * phi[((((size_t)blk * h->Q) + qx * h->os + qy) * h->W + d) * h->mb + ol];
                        const __half hi = __float2half_rn((float)v);
                        const __half lo = __float2half_rn((float)(v - (double)__half2float(hi)));
                        const int k = d * h->mb + ol;
                        const size_t off = ((size_t)(m >> 3) * sbo + (k >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2) / 2;
                        img[(size_t)(blk * 2 + 0) * per + off] = __half_as_ushort(hi);
                        img[(size_t)(blk * 2 + 1) * per + off] = __half_as_ushort(lo);
                    }
            }
}

// (T G0)(R)[a][o] = sum_c T[a][c] G0(R)[c][o] on the box, per energy, for one impurity: the
// s operand of the direct-window kernel with T folded in (its epilogue then only forms
// Im(sum_a u_a (T s)_a)).  FP32 (the operand is split from FP32 anyway); per-energy
// max |Re|,|Im| for the operand's split scale.
__global__ void __launch_bounds__(256) tfold_kernel(int b, long long npt, const float2 *__restrict__ box,
                                                    const float2 *__restrict__ T, float2 *__restrict__ boxT,
                                                    unsigned *__restrict__ gmaxT)
{
    const long long pt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int e = blockIdx.y, bb = b * b;
    float mx = 0.f;
    if (pt < npt) {
        const float2 *g = box + ((size_t)e * npt + pt) * bb;
        const float2 *Te = T + (size_t)e * bb;
        float2 *o = boxT + ((size_t)e * npt + pt) * bb;
        for (int a = 0; a < b; a++)
            for (int oc = 0; oc < b; oc++) {
                float sr = 0.f, si = 0.f;
                for (int c = 0; c < b; c++) {
                    const float2 t = Te[a * b + c];
                    const float2 v = g[c * b + oc];
                    sr += t.x * v.x - t.y * v.y;
                    si += t.x * v.y + t.y * v.x;
                }
                const float2 r = make_float2(sr, si);
                o[a * b + oc] = r;
                mx = fmaxf(mx, fmaxf(fabsf(r.x), fabsf(r.y)));
            }
    }
    for (int d = 16; d > 0; d >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, d));
    if ((threadIdx.x & 31) == 0 && mx > 0.f) atomicMax(gmaxT + e, __float_as_uint(mx));
}

template <int B, bool JOS, bool FOLD, bool BULK>
static cudaError_t launch_tcw_k(const TcParams &p, int grid, size_t smem, cudaStream_t st)
{
    cudaError_t err = cudaFuncSetAttribute(ldos_tcw_kernel<B, JOS, FOLD, BULK>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    ldos_tcw_kernel<B, JOS, FOLD, BULK><<<grid, TCW_THREADS, smem, st>>>(p);
    return cudaSuccess;
}
// bulk-copy variants exist for 3, 6 and 8 bands (p.nbulk is 0 for the other band counts)
template <int B, bool JOS, bool FOLD>
static cudaError_t launch_tcw(const TcParams &p, int grid, size_t smem, cudaStream_t st)
{
    if constexpr (B == 3 || B == 6 || B == 8) {
        if (p.nbulk > 0) return launch_tcw_k<B, JOS, FOLD, true>(p, grid, smem, st);
    }
    return launch_tcw_k<B, JOS, FOLD, false>(p, grid, smem, st);
}

template <int B>
static cudaError_t launch_tc_t(cqpi_handle *h, int ne, float *out, const int *fov, const long long *fov_off)
{
    const TcPlan &pl = h->tc;
    TcParams p = {};
    p.b = h->b; p.n = h->n; p.os = h->os; p.w = h->w; p.Rb = h->Rb; p.NB = h->NB; p.W = h->W;
    p.nblk = h->nblk; p.mb = h->mb; p.bs0 = h->blk_start[0]; p.bs1 = h->blk_start[1];
    p.TS = pl.TS; p.N = pl.N; p.KP = pl.KP; p.sst = pl.sst; p.Q = h->Q; p.nimp = h->nimp; p.ne = ne; p.wn = h->wn;
    p.ntx = (h->n + pl.TS - 1) / pl.TS;
    p.tmem_cols = pl.tmem_cols; p.a_bytes = pl.a_bytes; p.b_bytes = pl.b_bytes;
    p.inv_sA = h->tc_inv_sA;
    p.spin_limit = 1LL << 21;   // try_wait attempts (each suspends at most 1 us)
    // CQPI_TEST_STALL=1: the direct-window kernel waits on a barrier nothing arrives on,
    // with a short limit, to exercise the time-out path (tests only)
    const char *stall = getenv("CQPI_TEST_STALL");
    p.stall = (stall && !strcmp(stall, "1")) ? 1 : 0;
    if (p.stall) p.spin_limit = 256;
    p.box = h->ws.box32; p.T32 = h->ws.T32; p.term1 = h->ws.term1; p.gmax = h->ws.gmax;
    p.zsrc = box32_zeros(h);
    p.Aimg = reinterpret_cast<const uint4 *>(h->d_tc_a);
    p.out = out;
    p.scale = h->out_scale;
    p.fov = fov;
    p.fov_off = fov_off;
    p.status = h->d_status;
    p.coff = h->josephson ? h->b >> 1 : 0;
    p.tip = h->josephson ? h->jos_tip : nullptr;
    const char *force = getenv("CQPI_TC_PIPE");
    const bool pipe = pl.pipe && !(force && !strcmp(force, "0"));
    const char *fw = getenv("CQPI_TC_WINDOW");
    // the epilogue keeps T of every impurity of an energy block in shared memory
    const bool win_fits = pl.w_smem + 8 * (size_t)pl.wEB * h->nimp * h->b * h->b <= 227 * 1024;
    const bool win = pl.win && win_fits && h->d_tc_aw && !(fw && !strcmp(fw, "0")) && !(force && !strcmp(force, "0"));
    const long long ntiles = (long long)ne * h->n * p.ntx;
    cudaError_t err;
    if (fov && !win) return cudaErrorInvalidValue;   // per-map fields of view need the window kernel
    if (h->josephson && (!win || !h->jos_tip)) return cudaErrorInvalidValue;   // so does the Josephson form
    if (win) {
        // one impurity: T folded into the s operand (CQPI_TC_FOLD=0 keeps T in the epilogue)
        const char *ff = getenv("CQPI_TC_FOLD");
        // (not in the Josephson mode: its maps cancel more and keep T in the FP32 epilogue)
        if (h->nimp == 1 && !h->josephson && h->ws.boxT32 && !(ff && !strcmp(ff, "0"))) {
            const long long npt = (long long)h->NB * h->NB;
            err = cudaMemsetAsync(h->ws.gmaxT, 0, sizeof(unsigned) * ne, h->stream);
            if (err != cudaSuccess) return err;
            tfold_kernel<<<dim3(cdiv(npt, 256), ne), 256, 0, h->stream>>>(h->b, npt, h->ws.box32, h->ws.T32, h->ws.boxT32,
                                                                         h->ws.gmaxT);
            h->launches++;
            err = cudaGetLastError();
            if (err != cudaSuccess) return err;
            p.boxT = h->ws.boxT32;
            p.gmaxT = h->ws.gmaxT;
        }
        p.H = pl.wH; p.NX = pl.wNX; p.NKC = pl.wNKC; p.win_bytes = pl.w_win_bytes; p.EB = pl.wEB; p.nraw = pl.wNRAW;
        // CQPI_TC_NBULK=<n>: fetch the first n raw columns of a tile by bulk copies
        const char *fb = getenv("CQPI_TC_NBULK");
        p.nbulk = fb ? std::max(0, atoi(fb)) : pl.w_nbulk;
        if (!tcw_bulk_bands(h->b)) p.nbulk = 0;
        p.TS = 8 * pl.wH; p.KP = pl.wKP; p.a_bytes = pl.w_a_bytes; p.sst = pl.w_sst;
        p.ntx = (h->n + p.TS - 1) / p.TS;
        p.tmem_cols = pl.w_tmem_cols;
        const char *fa = getenv("CQPI_TC_ATMEM");
        p.a_tmem = pl.w_a_tmem && fa && !strcmp(fa, "1") ? 1 : 0;   // Phi in tensor memory: opt-in
        p.Aimg = reinterpret_cast<const uint4 *>(h->d_tc_aw);
        const size_t smem = pl.w_smem + 8 * (size_t)p.EB * h->nimp * h->b * h->b;
        const long long nt = (long long)((ne + p.EB - 1) / p.EB) * h->n * p.ntx;
        const int grid = (int)std::min<long long>(nt, (long long)h->num_sms);
        const bool fold = p.boxT != nullptr;
        if (h->josephson) {
            // Bogoliubov-de Gennes models have an even band count
            if constexpr (B % 2 == 0) {
                if (fold) err = launch_tcw<B, true, true>(p, grid, smem, h->stream);
                else err = launch_tcw<B, true, false>(p, grid, smem, h->stream);
            } else {
                return cudaErrorInvalidValue;
            }
        } else {
            if (fold) err = launch_tcw<B, false, true>(p, grid, smem, h->stream);
            else err = launch_tcw<B, false, false>(p, grid, smem, h->stream);
        }
        if (err != cudaSuccess) return err;
        h->launches++;
        return cudaGetLastError();
    }
    if (pipe) {
        p.tmem_cols = pl.pipe_tmem_cols;
        err = cudaFuncSetAttribute(ldos_tc_pipe_kernel<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.pipe_smem);
        if (err != cudaSuccess) return err;
        const int grid = (int)std::min<long long>(ntiles, (long long)h->num_sms);   // one CTA per SM (512 TMEM columns)
        ldos_tc_pipe_kernel<B><<<grid, TC_THREADS, pl.pipe_smem, h->stream>>>(p);
        h->launches++;
        return cudaGetLastError();
    }
    err = cudaFuncSetAttribute(ldos_tc_kernel<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem);
    if (err != cudaSuccess) return err;
    int per_sm = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ldos_tc_kernel<B>, TC_THREADS, pl.smem);
    if (err != cudaSuccess) return err;
    per_sm = std::max(1, std::min(per_sm, (int)(512 / pl.tmem_cols)));
    const int grid = (int)std::min<long long>(ntiles, (long long)h->num_sms * per_sm);
    ldos_tc_kernel<B><<<grid, TC_THREADS, pl.smem, h->stream>>>(p);
    h->launches++;
    return cudaGetLastError();
}

cudaError_t launch_ldos_tc(cqpi_handle *h, int ne, float *out, const int *fov, const long long *fov_off)
{
    const int b = h->b;
    if (b <= 1) return launch_tc_t<1>(h, ne, out, fov, fov_off);
    if (b <= 2) return launch_tc_t<2>(h, ne, out, fov, fov_off);
    if (b <= 3) return launch_tc_t<3>(h, ne, out, fov, fov_off);
    if (b <= 4) return launch_tc_t<4>(h, ne, out, fov, fov_off);
    if (b <= 6) return launch_tc_t<6>(h, ne, out, fov, fov_off);
    if (b <= 8) return launch_tc_t<8>(h, ne, out, fov, fov_off);
    if (b <= 10) return launch_tc_t<10>(h, ne, out, fov, fov_off);
    if (b <= 12) return launch_tc_t<12>(h, ne, out, fov, fov_off);
    return launch_tc_t<16>(h, ne, out, fov, fov_off);
}

bool tc_window_usable(const cqpi_handle *h)
{
    const char *force = getenv("CQPI_TC_PIPE");
    const char *fw = getenv("CQPI_TC_WINDOW");
    return h->use_tc && !h->list_mode && h->tc.win && h->d_tc_aw && !(fw && !strcmp(fw, "0")) && !(force && !strcmp(force, "0")) &&
           h->tc.w_smem + 8 * (size_t)h->tc.wEB * h->nimp * h->b * h->b <= 227 * 1024;
}

}  // namespace cqpi
