// greens.cu -- per-energy Green's function stages, FP64 (double2) and mixed (float2).
//
//  greens_k   G0(k,w) = sum_n U_n U_n^H / (w - e_n + i eta) for every k and every
//             energy of the batch; replaces tmatrix::setgreensfunction +
//             tightbind::calcgreensfunction (src/qpi.cc:478-486,
//             src/tightbinding.cc:282-289).  w - e_n is always formed in FP64 (the
//             pole distance needs it at small eta); the mixed path then works in FP32.
//             HBM-bound (reads the eigen cache, writes the G0(k) planes).
//  fft        G0(R) = kp^-2 sum_k G0(k) e^{+2 pi i k.R} on the pruned box
//             R in [-Rb, Rb]^2 only (Rb = lattice/2 + window); replaces the b^2
//             full FFTW transforms of tmatrix::calcrealspacegreensfunction
//             (src/qpi.cc:557-578).  Pass 1 transforms rows along j and keeps the
//             NB needed outputs, pass 2 transforms NB columns along i.  Radix-2 in
//             shared memory for power-of-two kp, a pruned direct DFT otherwise.
//  tmatrix    T = (1 - V G0(R=0))^-1 V in FP64 per energy and impurity
//             (tmatrix::setscatteringmatrix, src/qpi.cc:833-854).
//  term1      the site-independent part of the LDOS in FP64,
//             sum_{d1,d2,o1,o2} phi_o1(q,d1) phi_o2(q,d2) Im G0(d2-d1)[o2][o1]
//             (second accumulation of src/qpi.cc:921).
#include "cplx.h"
#include "cqpi_internal.h"

namespace cqpi {

// ------------------------------------------------------------------ G0(k,w)
// tr: only the planes o <= a, stored in the upper-triangle order (index o*b - o(o-1)/2 + a - o),
// np planes per energy; else all b^2 planes o*b + a
template <int B, class C>
__global__ void __launch_bounds__(256) greens_k_kernel(int b, long long nk, double eta, const double *__restrict__ energies,
                                                       const double *__restrict__ eval, const C *__restrict__ evec,
                                                       C *__restrict__ g0k, int tr)
{
    using R = typename real_of<C>::type;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    const int e = blockIdx.y;
    const double omega = energies[e];
    const int bb = b * b;
    C f[B];
#pragma unroll
    for (int n = 0; n < B; n++) {
        if (n < b) {
            const R dr = (R)(omega - eval[(size_t)n * nk + k]);   // FP64 difference, then rounded
            const R et = (R)eta;
            const R den = dr * dr + et * et;
            f[n].x = dr / den;
            f[n].y = -et / den;
        }
    }
    const int np = tr ? b * (b + 1) / 2 : bb;
    C *out = g0k + (size_t)e * np * nk + k;
#pragma unroll
    for (int o = 0; o < B; o++) {
        if (o >= b) continue;
        C x[B];
#pragma unroll
        for (int n = 0; n < B; n++)
            if (n < b) x[n] = cmul(evec[(size_t)(o * b + n) * nk + k], f[n]);
#pragma unroll
        for (int a = 0; a < B; a++) {
            if (a >= b || (tr && a < o)) continue;
            C s = cmake<C>(0.0, 0.0);
#pragma unroll
            for (int n = 0; n < B; n++) {
                if (n < b) {
                    const C u = evec[(size_t)(a * b + n) * nk + k];
                    s.x += x[n].x * u.x + x[n].y * u.y;   // x * conj(u)
                    s.y += x[n].y * u.x - x[n].x * u.y;
                }
            }
            const int pl = tr ? o * b - (o * (o - 1)) / 2 + (a - o) : o * b + a;
            out[(size_t)pl * nk] = s;
        }
    }
}

template <int B>
static void launch_greens_k_t(cqpi_handle *h, int ne, const double *d_energies)
{
    const long long nk = (long long)h->kp * h->kp;
    dim3 grid(cdiv(nk, 256), ne);
    if (h->precision == CQPI_PREC_FP64)
        greens_k_kernel<B, double2><<<grid, 256, 0, h->stream>>>(h->b, nk, h->eta, d_energies, h->d_eval, h->d_evec,
                                                                  h->ws.g0k, 0);
    else
        greens_k_kernel<B, float2><<<grid, 256, 0, h->stream>>>(h->b, nk, h->eta, d_energies, h->d_eval, h->d_evec32,
                                                                 h->ws.g0k32, g0k_reciprocity(h) ? 1 : 0);
    h->launches++;
}

void launch_greens_k(cqpi_handle *h, int ne, const double *d_energies)
{
    const int b = h->b;
    if (b <= 1) launch_greens_k_t<1>(h, ne, d_energies);
    else if (b <= 2) launch_greens_k_t<2>(h, ne, d_energies);
    else if (b <= 3) launch_greens_k_t<3>(h, ne, d_energies);
    else if (b <= 4) launch_greens_k_t<4>(h, ne, d_energies);
    else if (b <= 5) launch_greens_k_t<5>(h, ne, d_energies);
    else if (b <= 6) launch_greens_k_t<6>(h, ne, d_energies);
    else if (b <= 8) launch_greens_k_t<8>(h, ne, d_energies);
    else if (b <= 10) launch_greens_k_t<10>(h, ne, d_energies);
    else if (b <= 12) launch_greens_k_t<12>(h, ne, d_energies);
    else launch_greens_k_t<16>(h, ne, d_energies);
}

// ------------------------------------------------------------------ pruned 2D transform
__device__ __forceinline__ int bitrev(int x, int bits) { return bits == 0 ? 0 : (int)(__brev((unsigned)x) >> (32 - bits)); }
__device__ __forceinline__ int posmod(int a, int m) { int r = a % m; return r < 0 ? r + m : r; }

// Pass 1: rows (fixed i, plane, energy), transform along j, keep Y = yb - Rb for yb < NB.
template <class C>
__global__ void __launch_bounds__(256) fft_rows_kernel(int kp, int logkp, int NB, int Rb, int bb, long long nk,
                                                       const C *__restrict__ g0k, const C *__restrict__ tw,
                                                       C *__restrict__ half)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    const int i = blockIdx.x, pl = blockIdx.y, e = blockIdx.z;
    const C *src = g0k + ((size_t)e * bb + pl) * nk + (size_t)i * kp;
    C *dst = half + (((size_t)e * bb + pl) * kp + i) * NB;
    if (logkp >= 0) {
        for (int j = threadIdx.x; j < kp; j += blockDim.x) sm[bitrev(j, logkp)] = src[j];
        __syncthreads();
        for (int len = 2; len <= kp; len <<= 1) {
            const int hl = len >> 1, step = kp / len;
            for (int t = threadIdx.x; t < (kp >> 1); t += blockDim.x) {
                const int idx = (t / hl) * len + (t % hl);
                const C w = tw[(t % hl) * step];
                const C u = sm[idx], v = cmul(sm[idx + hl], w);
                sm[idx] = cadd(u, v);
                sm[idx + hl] = csub(u, v);
            }
            __syncthreads();
        }
        for (int yb = threadIdx.x; yb < NB; yb += blockDim.x) dst[yb] = sm[posmod(yb - Rb, kp)];
    } else {
        for (int j = threadIdx.x; j < kp; j += blockDim.x) sm[j] = src[j];
        __syncthreads();
        for (int yb = threadIdx.x; yb < NB; yb += blockDim.x) {
            const int ym = posmod(yb - Rb, kp);
            C s = cmake<C>(0.0, 0.0);
            for (int j = 0; j < kp; j++) s = cadd(s, cmul(sm[j], tw[(int)(((long long)j * ym) % kp)]));
            dst[yb] = s;
        }
    }
}

// Pass 2: NC adjacent columns yb (fixed plane, energy), transform along i, keep X = xb - Rb.
// Pass 2 also records max |Re|,|Im| of the box per energy (gmax, float bits; used to
// scale the tensor-core operands) when gmax is non-null.
__device__ __forceinline__ void track_max(unsigned *gmax, float v)
{
    v = fmaxf(v, 0.0f);
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v > 0.0f) atomicMax(gmax, __float_as_uint(v));
}

template <class C>
__global__ void __launch_bounds__(256) fft_cols_kernel(int kp, int logkp, int NB, int Rb, int bb, int NC, double scale,
                                                       const C *__restrict__ half, const C *__restrict__ tw,
                                                       C *__restrict__ box, unsigned *__restrict__ gmax)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    const int yb0 = blockIdx.x * NC, pl = blockIdx.y, e = blockIdx.z;
    const C *src = half + ((size_t)e * bb + pl) * (size_t)kp * NB;
    C *dst = box + (size_t)e * NB * NB * bb;
    const bool pow2 = logkp >= 0;
    for (int idx = threadIdx.x; idx < kp * NC; idx += blockDim.x) {
        const int i = idx / NC, c = idx % NC, yb = yb0 + c;
        const int pos = pow2 ? bitrev(i, logkp) : i;
        sm[pos * NC + c] = (yb < NB) ? src[(size_t)i * NB + yb] : cmake<C>(0.0, 0.0);
    }
    __syncthreads();
    if (pow2) {
        for (int len = 2; len <= kp; len <<= 1) {
            const int hl = len >> 1, step = kp / len;
            for (int t = threadIdx.x; t < (kp >> 1) * NC; t += blockDim.x) {
                const int c = t % NC, bt = t / NC;
                const int idx = (bt / hl) * len + (bt % hl);
                const C w = tw[(bt % hl) * step];
                const C u = sm[idx * NC + c], v = cmul(sm[(idx + hl) * NC + c], w);
                sm[idx * NC + c] = cadd(u, v);
                sm[(idx + hl) * NC + c] = csub(u, v);
            }
            __syncthreads();
        }
        float mx = 0.0f;
        const int lim = ((NB * NC + (int)blockDim.x - 1) / (int)blockDim.x) * (int)blockDim.x;
        for (int idx = threadIdx.x; idx < lim; idx += blockDim.x) {
            const int xb = idx / NC, c = idx % NC, yb = yb0 + c;
            if (idx < NB * NC && yb < NB) {
                const C v = cscale(sm[posmod(xb - Rb, kp) * NC + c], scale);
                dst[((size_t)xb * NB + yb) * bb + pl] = v;
                mx = fmaxf(mx, fmaxf(fabsf((float)v.x), fabsf((float)v.y)));
            }
        }
        if (gmax) track_max(gmax + e, mx);
    } else {
        for (int idx = threadIdx.x; idx < NB * NC; idx += blockDim.x) {
            const int xb = idx / NC, c = idx % NC, yb = yb0 + c;
            if (yb >= NB) continue;
            const int xm = posmod(xb - Rb, kp);
            C s = cmake<C>(0.0, 0.0);
            for (int i = 0; i < kp; i++) s = cadd(s, cmul(sm[i * NC + c], tw[(int)(((long long)i * xm) % kp)]));
            dst[((size_t)xb * NB + yb) * bb + pl] = cscale(s, scale);
        }
        if (gmax) {
            __syncthreads();
            float mx = 0.0f;
            const int lim = ((NB * NC + (int)blockDim.x - 1) / (int)blockDim.x) * (int)blockDim.x;
            for (int idx = threadIdx.x; idx < lim; idx += blockDim.x) {
                const int xb = idx / NC, c = idx % NC, yb = yb0 + c;
                if (idx < NB * NC && yb < NB) {
                    const C v = dst[((size_t)xb * NB + yb) * bb + pl];
                    mx = fmaxf(mx, fmaxf(fabsf((float)v.x), fabsf((float)v.y)));
                }
            }
            track_max(gmax + e, mx);
        }
    }
}

static int ilog2_exact(int v)
{
    if (v <= 0 || (v & (v - 1))) return -1;
    int l = 0;
    while ((1 << l) < v) l++;
    return l;
}

// Columns per CTA of pass 2: kp * NC complex values (<= 128 KiB) of shared memory.
static int fft_cols_per_block(int kp, size_t elem)
{
    int c = (int)((128 * 1024) / (elem * (size_t)kp));
    return c < 1 ? 1 : (c > 16 ? 16 : c);
}

cudaError_t configure_fft(cqpi_handle *h)
{
    const int kp = h->kp;
    cudaError_t e;
    e = cudaFuncSetAttribute(fft_rows_kernel<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(16 * kp));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(fft_cols_kernel<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(16 * kp * fft_cols_per_block(kp, 16)));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(fft_rows_kernel<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(8 * kp));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(fft_cols_kernel<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(8 * kp * fft_cols_per_block(kp, 8)));
}

template <class C>
static void launch_fft_t(cqpi_handle *h, int ne, const C *g0k, const C *tw, C *half, C *box, unsigned *gmax)
{
    const int kp = h->kp, bb = h->b * h->b, NB = h->NB;
    const long long nk = (long long)kp * kp;
    const int logkp = ilog2_exact(kp);
    const int thr = kp >= 512 ? 256 : (kp >= 64 ? 128 : 64);
    {
        dim3 grid(kp, bb, ne);
        fft_rows_kernel<C><<<grid, thr, sizeof(C) * kp, h->stream>>>(kp, logkp, NB, h->Rb, bb, nk, g0k, tw, half);
        h->launches++;
    }
    {
        const int NC = fft_cols_per_block(kp, sizeof(C));
        dim3 grid(cdiv(NB, NC), bb, ne);
        fft_cols_kernel<C><<<grid, 256, sizeof(C) * kp * NC, h->stream>>>(kp, logkp, NB, h->Rb, bb, NC,
                                                                         1.0 / ((double)kp * kp), half, tw, box, gmax);
        h->launches++;
    }
}

void launch_fft(cqpi_handle *h, int ne)
{
    if (h->precision == CQPI_PREC_FP64)
        launch_fft_t<double2>(h, ne, h->ws.g0k, h->d_tw, h->ws.half, h->ws.box, nullptr);
    else if (!launch_fft32_planes(h, ne))
        launch_fft_t<float2>(h, ne, h->ws.g0k32, h->d_tw32, h->ws.half32, h->ws.box32, h->ws.gmax);
}

// ------------------------------------------------------------------ T-matrix
template <class C>
__global__ void tmatrix_kernel(int b, int NB, int Rb, int nimp, int ne, const C *__restrict__ box,
                               const double2 *__restrict__ V, double2 *__restrict__ T, float2 *__restrict__ T32,
                               int *status)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= ne * nimp) return;
    const int e = id / nimp, imp = id % nimp;
    const int bb = b * b;
    const C *g = box + (((size_t)e * NB + Rb) * NB + Rb) * bb;
    const double2 *v = V + (size_t)imp * bb;
    double2 M[CQPI_MAX_BANDS * CQPI_MAX_BANDS], inv[CQPI_MAX_BANDS * CQPI_MAX_BANDS];
    for (int r = 0; r < b; r++)
        for (int c = 0; c < b; c++) {
            double2 s = make_double2(0.0, 0.0);
            for (int k = 0; k < b; k++) s = cadd(s, cmul(v[r * b + k], to_d2(g[k * b + c])));   // (V G0)_{rc}
            M[r * b + c] = make_double2((r == c ? 1.0 : 0.0) - s.x, -s.y);
            inv[r * b + c] = make_double2(r == c ? 1.0 : 0.0, 0.0);
        }
    bool singular = false;
    for (int c = 0; c < b; c++) {
        int piv = c;
        double best = -1.0;
        for (int r = c; r < b; r++) {
            double a = hypot(M[r * b + c].x, M[r * b + c].y);
            if (a > best) { best = a; piv = r; }
        }
        if (!(best > 0.0)) { singular = true; break; }
        if (piv != c)
            for (int k = 0; k < b; k++) {
                double2 t0 = M[c * b + k]; M[c * b + k] = M[piv * b + k]; M[piv * b + k] = t0;
                t0 = inv[c * b + k]; inv[c * b + k] = inv[piv * b + k]; inv[piv * b + k] = t0;
            }
        const double2 p = M[c * b + c];
        const double pd = p.x * p.x + p.y * p.y;
        for (int r = 0; r < b; r++) {
            if (r == c) continue;
            const double2 mm = M[r * b + c];
            const double2 f = make_double2((mm.x * p.x + mm.y * p.y) / pd, (mm.y * p.x - mm.x * p.y) / pd);
            for (int k = 0; k < b; k++) {
                M[r * b + k] = csub(M[r * b + k], cmul(f, M[c * b + k]));
                inv[r * b + k] = csub(inv[r * b + k], cmul(f, inv[c * b + k]));
            }
        }
    }
    double2 *out = T + (size_t)id * bb;
    float2 *out32 = T32 + (size_t)id * bb;
    if (singular) {
        atomicOr(status, 1);
        for (int k = 0; k < bb; k++) { out[k] = make_double2(0.0, 0.0); out32[k] = make_float2(0.f, 0.f); }
        return;
    }
    for (int r = 0; r < b; r++) {
        const double2 p = M[r * b + r];
        const double pd = p.x * p.x + p.y * p.y;
        for (int k = 0; k < b; k++) {
            const double2 x = inv[r * b + k];
            inv[r * b + k] = make_double2((x.x * p.x + x.y * p.y) / pd, (x.y * p.x - x.x * p.y) / pd);
        }
    }
    for (int r = 0; r < b; r++)
        for (int c = 0; c < b; c++) {
            double2 s = make_double2(0.0, 0.0);
            for (int k = 0; k < b; k++) s = cadd(s, cmul(inv[r * b + k], v[k * b + c]));
            out[r * b + c] = s;
            out32[r * b + c] = make_float2((float)s.x, (float)s.y);
        }
}

void launch_tmatrix(cqpi_handle *h, int ne)
{
    const int n = ne * h->nimp;
    if (h->precision == CQPI_PREC_FP64)
        tmatrix_kernel<double2><<<cdiv(n, 64), 64, 0, h->stream>>>(h->b, h->NB, h->Rb, h->nimp, ne, h->ws.box, h->d_V,
                                                                   h->ws.T, h->ws.T32, h->d_status);
    else
        tmatrix_kernel<float2><<<cdiv(n, 64), 64, 0, h->stream>>>(h->b, h->NB, h->Rb, h->nimp, ne, h->ws.box32, h->d_V,
                                                                  h->ws.T, h->ws.T32, h->d_status);
    h->launches++;
}

// ------------------------------------------------------------------ site-independent term
// term1(q) = sum_{d1,d2,o1,o2} phi_o1(q,d1) phi_o2(q,d2) Im G0(d2-d1)[o2][o1] per energy; in
// Josephson mode (tip != NULL, src/qpi.cc:986-990) the column is o1 + coff and the value
// Im(tip_e * G0(d2-d1)[o2][o1+coff]).
template <class C>
__global__ void __launch_bounds__(256) term1_kernel(int b, int NB, int Rb, int w, int Q, int W, int nblk, int mb, int bs0,
                                                    int bs1, int coff, const double2 *__restrict__ tip,
                                                    const double *__restrict__ phi, const C *__restrict__ box,
                                                    double *__restrict__ term1)
{
    const int q = blockIdx.x, e = blockIdx.y;
    const int bb = b * b, side = 2 * w + 1;
    const C *boxe = box + (size_t)e * NB * NB * bb;
    const double2 tp = tip ? tip[e] : make_double2(1.0, 0.0);
    double acc = 0.0;
    const int npair = nblk * W * W;
    for (int t = threadIdx.x; t < npair; t += blockDim.x) {
        const int blk = t / (W * W), d1 = (t / W) % W, d2 = t % W;
        const int bs = blk ? bs1 : bs0;
        const int rx = (d2 / side) - (d1 / side), ry = (d2 % side) - (d1 % side);
        const C *g = boxe + ((size_t)(rx + Rb) * NB + (ry + Rb)) * bb;
        const double *p1 = phi + (((size_t)blk * Q + q) * W + d1) * mb;
        const double *p2 = phi + (((size_t)blk * Q + q) * W + d2) * mb;
        for (int o1 = 0; o1 < mb; o1++) {
            const double f1 = p1[o1];
            if (f1 == 0.0) continue;
            for (int o2 = 0; o2 < mb; o2++) {
                const C v = g[(bs + o2) * b + (bs + o1 + coff)];
                const double im = tip ? tp.x * (double)v.y + tp.y * (double)v.x : (double)v.y;
                acc += f1 * p2[o2] * im;
            }
        }
    }
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) term1[(size_t)e * Q + q] = red[0];
}

template <class C>
static void launch_term1_t(cqpi_handle *h, int ne, const C *box, double *term1)
{
    dim3 grid(h->Q, ne);
    const double2 *tip = h->jos_tip;
    term1_kernel<C><<<grid, 256, 0, h->stream>>>(h->b, h->NB, h->Rb, h->w, h->Q, h->W, h->nblk, h->mb, h->blk_start[0],
                                                 h->blk_start[1], tip ? h->b >> 1 : 0, tip, h->d_phi, box, term1);
    h->launches++;
}

void launch_term1_ptr(cqpi_handle *h, int ne, const double2 *box, double *term1) { launch_term1_t(h, ne, box, term1); }

void launch_term1(cqpi_handle *h, int ne)
{
    if (h->precision == CQPI_PREC_FP64) launch_term1_t(h, ne, h->ws.box, h->ws.term1);
    else launch_term1_t(h, ne, h->ws.box32, h->ws.term1);
}

}  // namespace cqpi
