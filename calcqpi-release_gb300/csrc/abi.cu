// abi.cu -- the extern "C" boundary of libcqpi.so (declared in include/cqpi.h).
//
// Owns every device buffer of a handle, validates sizes against the reference's
// index domain, converts the reference's inputs (hopping list, orbital cache,
// scattering vector) into the engine's HBM layout and drives the per-energy
// stages in batches of energies on the handle's stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <utility>

#include "cqpi_internal.h"

using namespace cqpi;

namespace {

struct CudaError {
    cudaError_t code;
    const char *what;
};

#define CK(call)                                                   \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) throw CudaError{e_, #call};         \
    } while (0)

int fail(cqpi_handle *h, int code, const std::string &msg)
{
    if (h) h->err = msg;
    return code;
}

int cuda_fail(cqpi_handle *h, const CudaError &e)
{
    char buf[512];
    snprintf(buf, sizeof buf, "CUDA error %d (%s) in %s", (int)e.code, cudaGetErrorString(e.code), e.what);
    if (h) h->err = buf;
    return (e.code == cudaErrorMemoryAllocation) ? CQPI_ERR_ALLOC : CQPI_ERR_CUDA;
}

template <class T>
void dalloc(T **p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    CK(cudaMalloc((void **)p, sizeof(T) * count));
}

template <class T>
void dfree(T *&p)
{
    if (p) cudaFree(p);
    p = nullptr;
}

// Host -> device copy ordered on the handle's stream (which does not wait for the legacy
// default stream), complete when it returns, so that the host array may be reused at once and
// every later kernel on the stream sees the data.
template <class T>
void h2d_sync(cqpi_handle *h, T *dst, const T *src, size_t count)
{
    if (count == 0) return;
    CK(cudaMemcpyAsync(dst, src, sizeof(T) * count, cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
}

// Keep a device buffer of at least count elements, reallocating only when it must grow
// (cudaFree synchronises the device; repeated uploads of same-sized data avoid it).
template <class T>
void dreserve(T **p, size_t &cap, size_t count)
{
    if (*p && cap >= count) return;
    dfree(*p);
    cap = 0;
    dalloc(p, count);
    cap = count;
}

// H(k) = sum_R C(R) e^{i theta_R} with C(R) = tn(R) + ta(-R) (normal terms of R, conjugated
// terms of -R).  The eigen-solve builds it from pairs {R, -R}: C(R) e^{i th} + C(-R) e^{-i th}
// = P cos th + Q sin th with P = C(R) + C(-R), Q = i (C(R) - C(-R)) (R = 0: P = C(0), Q = 0).
void upload_pairs(cqpi_handle *h)
{
    const int nR = h->nR;
    const size_t bb = (size_t)h->b * h->b;
    std::map<std::pair<int, int>, int> idx;
    for (int r = 0; r < nR; r++) idx[std::make_pair(h->rt_R[2 * r], h->rt_R[2 * r + 1])] = r;
    auto C = [&](int r, size_t e, double2 &out) {   // C(R_r)[e]
        out = make_double2(h->rt_tn[2 * (r * bb + e)], h->rt_tn[2 * (r * bb + e) + 1]);
        auto it = idx.find(std::make_pair(-h->rt_R[2 * r], -h->rt_R[2 * r + 1]));
        if (it != idx.end()) {
            out.x += h->rt_ta[2 * (it->second * bb + e)];
            out.y += h->rt_ta[2 * (it->second * bb + e) + 1];
        }
    };
    std::vector<int32_t> pR;
    std::vector<double2> pq;
    std::vector<char> done(nR, 0);
    for (int r = 0; r < nR; r++) {
        if (done[r]) continue;
        const int rx = h->rt_R[2 * r], ry = h->rt_R[2 * r + 1];
        auto it = idx.find(std::make_pair(-rx, -ry));
        const int partner = (it != idx.end() && it->second != r) ? it->second : -1;
        done[r] = 1;
        if (partner >= 0) done[partner] = 1;
        pR.push_back(rx);
        pR.push_back(ry);
        const size_t base = pq.size();
        pq.resize(base + 2 * bb);
        for (size_t e = 0; e < bb; e++) {
            double2 c1, c2 = make_double2(0.0, 0.0);
            C(r, e, c1);
            if (partner >= 0) C(partner, e, c2);
            if (rx == 0 && ry == 0) {
                pq[base + e] = c1;
                pq[base + bb + e] = make_double2(0.0, 0.0);
            } else {
                pq[base + e] = make_double2(c1.x + c2.x, c1.y + c2.y);
                pq[base + bb + e] = make_double2(-(c1.y - c2.y), c1.x - c2.x);   // i (c1 - c2)
            }
        }
    }
    h->npair_R = (int)(pR.size() / 2);
    dreserve(&h->d_pR, h->cap_pR, std::max<size_t>(pR.size(), 2));
    dreserve(&h->d_pPQ, h->cap_pPQ, std::max<size_t>(pq.size(), 1));
    if (!pR.empty()) {
        CK(cudaMemcpyAsync(h->d_pR, pR.data(), sizeof(int32_t) * pR.size(), cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->d_pPQ, pq.data(), sizeof(double2) * pq.size(), cudaMemcpyHostToDevice, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));   // pageable temporaries
}

void free_workspace(cqpi_handle *h)
{
    dfree(h->ws.g0k);
    dfree(h->ws.half);
    dfree(h->ws.box);
    dfree(h->ws.T);
    dfree(h->ws.term1);
    dfree(h->ws.energies);
    dfree(h->ws.g0k32);
    dfree(h->ws.half32);
    dfree(h->ws.box32);
    dfree(h->ws.T32);
    dfree(h->ws.gmax);
    dfree(h->ws.boxT32);
    dfree(h->ws.gmaxT);
    h->ws.ebatch = 0;
}

void free_adj(cqpi_handle *h)
{
    dfree(h->adj.gbox);
    dfree(h->adj.M);
    dfree(h->adj.wsum);
    dfree(h->adj.gV);
    dfree(h->adj.A);
    dfree(h->adj.gk);
    dfree(h->adj.C);
    dfree(h->adj.gR);
    if (h->adj.win) cudaFree(h->adj.win);
    h->adj.win = nullptr;
    dfree(h->adj.Mp);
    dfree(h->adj.kt);
    h->adj.ebatch = 0;
}

void ensure_adj(cqpi_handle *h, int ebatch)
{
    if (h->adj.ebatch >= ebatch) return;
    free_adj(h);
    const size_t bb = (size_t)h->b * h->b, nk = (size_t)h->kp * h->kp;
    dalloc(&h->adj.gbox, ebatch * (size_t)h->NB * h->NB * bb);
    dalloc(&h->adj.M, ebatch * (size_t)std::max(h->nimp, 1) * bb);
    dalloc(&h->adj.wsum, ebatch * (size_t)h->Q);
    dalloc(&h->adj.gV, (size_t)std::max(h->nimp, 1) * bb);
    dalloc(&h->adj.A, bb * (size_t)h->NB * h->kp);
    // Gbar(k) of every energy of a batch in the handle's precision (at least one FP64 plane
    // set: Hbar(k) is written over it)
    const size_t gk_per_e = h->precision == CQPI_PREC_FP64 ? bb * nk : (bb * nk + 1) / 2;
    dalloc(&h->adj.gk, std::max(ebatch * gk_per_e, bb * nk));
    dalloc(&h->adj.C, bb * nk);
    dalloc(&h->adj.gR, (size_t)std::max(h->nR, 1) * 2 * bb);
    const size_t nsite = (size_t)h->n * h->n, nmap = ebatch * (size_t)std::max(h->nimp, 1);
    const size_t cs = h->precision == CQPI_PREC_FP64 ? sizeof(double2) : sizeof(float2);
    CK(cudaMalloc(&h->adj.win, 2 * cs * nmap * h->W * h->mb * h->b * nsite));
    dalloc(&h->adj.Mp, nmap * nsite * bb);
    const size_t span = 4 * (size_t)h->w + 1;
    dalloc(&h->adj.kt, span * span * h->mb * h->mb * h->Q);
    h->adj.ebatch = ebatch;
}

size_t bytes_per_energy(const cqpi_handle *h)
{
    const size_t bb = (size_t)h->b * h->b, nk = (size_t)h->kp * h->kp;
    const size_t cs = (h->precision == CQPI_PREC_FP64) ? 16 : 8;
    const size_t g0k = (h->use_fft32 && h->gmode == CQPI_GREEN_NORMAL) ? 0 : bb * nk;
    const size_t boxT = h->use_tc ? (size_t)h->NB * h->NB * bb : 0;   // T G0 box of the folded s operand
    return cs * (g0k + bb * (size_t)h->kp * h->NB + (size_t)h->NB * h->NB * bb + boxT) + 8 * (size_t)h->Q;
}

void ensure_workspace(cqpi_handle *h, int ebatch)
{
    if (h->ws.ebatch >= ebatch) return;
    free_workspace(h);
    free_adj(h);
    const size_t bb = (size_t)h->b * h->b, nk = (size_t)h->kp * h->kp;
    if (h->precision == CQPI_PREC_FP64) {
        dalloc(&h->ws.g0k, ebatch * bb * nk);
        dalloc(&h->ws.half, ebatch * bb * (size_t)h->kp * h->NB);
        dalloc(&h->ws.box, ebatch * (size_t)h->NB * h->NB * bb);
    } else {
        if (!h->use_fft32 || h->gmode != CQPI_GREEN_NORMAL) dalloc(&h->ws.g0k32, ebatch * bb * nk);
        dalloc(&h->ws.half32, ebatch * bb * (size_t)h->kp * h->NB);
        const size_t nbox = box32_boxes(h, ebatch), ncnt = box32_count(h, ebatch);
        dalloc(&h->ws.box32, ncnt);
        CK(cudaMemsetAsync(h->ws.box32 + nbox, 0, sizeof(float2) * (ncnt - nbox), h->stream));
        dalloc(&h->ws.gmax, ebatch);
        if (h->use_tc) {
            dalloc(&h->ws.boxT32, ncnt);
            dalloc(&h->ws.gmaxT, ebatch);
        }
    }
    dalloc(&h->ws.T, ebatch * (size_t)std::max(h->nimp, 1) * bb);
    dalloc(&h->ws.T32, ebatch * (size_t)std::max(h->nimp, 1) * bb);
    dalloc(&h->ws.term1, ebatch * (size_t)h->Q);
    dalloc(&h->ws.energies, ebatch);
    h->ws.ebatch = ebatch;
}

// The tensor-core contraction runs: mixed precision with a plan, no proximity list, and in the
// Josephson mode only through the direct-window kernel (one spin block), whose producer reads
// the hole-block columns and whose epilogue applies the tip factor; otherwise the CUDA-core
// kernels run.
bool tc_active(const cqpi_handle *h)
{
    return h->use_tc && !h->list_mode && (!h->josephson || tc_window_usable(h));
}

// The proximity-list contraction runs (threshold set; the Josephson mode ignores the list,
// as src/calcqpi.cc:705-709 does).
bool list_active(const cqpi_handle *h) { return h->list_mode && !h->josephson; }

// term1 of an energy batch: the list form or the full window form.
void do_term1(cqpi_handle *h, int ne)
{
    if (list_active(h))
        launch_term1_list(h, ne, h->precision == CQPI_PREC_FP64 ? (const void *)h->ws.box : (const void *)h->ws.box32,
                          h->ws.term1);
    else
        launch_term1(h, ne);
}

// tmp32: float buffer of ne*nimp maps used when only float64 maps are requested from the
// tensor-core contraction (which writes float32).
void launch_contraction(cqpi_handle *h, int ne, float *o32, double *o64, float *tmp32)
{
    if (list_active(h)) {
        if (h->precision == CQPI_PREC_FP64) launch_ldos_list(h, ne, h->ws.box, h->ws.T, h->ws.term1, o32, o64);
        else launch_ldos_list(h, ne, h->ws.box32, h->ws.T32, h->ws.term1, o32, o64);
    } else if (h->precision == CQPI_PREC_FP64) {
        launch_ldos_fp64(h, ne, h->ws.box, h->ws.T, h->ws.term1, o32, o64);
    } else if (tc_active(h)) {
        float *dst = o32 ? o32 : tmp32;
        CK(launch_ldos_tc(h, ne, dst));
        if (o64) launch_widen(h, dst, o64, (size_t)ne * h->nimp * h->wn * h->wn);
    } else {
        launch_ldos_fp32(h, ne, h->ws.box32, h->ws.T32, h->ws.term1, o32, o64);
    }
}

// energies per batch of a run with host outputs (CQPI_HOST_BATCH overrides)
int host_batch()
{
    const char *f = getenv("CQPI_HOST_BATCH");
    const int v = f ? atoi(f) : 0;
    return v > 0 ? v : 8;
}

int choose_batch(const cqpi_handle *h, int nE)
{
    const size_t budget = (size_t)16 << 30;   // workspace ceiling: 16 GiB of the 288 GB HBM
    size_t per = bytes_per_energy(h) + (size_t)h->nimp * h->wn * h->wn * 12;
    int eb = (int)std::max<size_t>(1, budget / std::max<size_t>(per, 1));
    eb = std::min(eb, 32);
    return std::max(1, std::min(eb, nE));
}

void check_launch()
{
    CK(cudaGetLastError());
}

// Device status word: bit 0 (1) a singular 1 - V G0(0), bit 1 (2) a bounded device wait
// that ran out (the kernel stopped early; its maps are incomplete).
int status_code(cqpi_handle *h, int st, const char *what)
{
    if (st & 2) return fail(h, CQPI_ERR_TIMEOUT, std::string("a device wait timed out in ") + what);
    if (st & 4) return fail(h, CQPI_ERR_NOT_CONVERGED, std::string("the surface / bulk decimation did not converge in ") + what);
    if (st & 1) return fail(h, CQPI_ERR_SINGULAR, std::string("1 - V G0(0) is singular at an energy of ") + what);
    return CQPI_OK;
}

int read_status(cqpi_handle *h)
{
    int st = 0;
    CK(cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (st) {
        int zero = 0;
        CK(cudaMemcpyAsync(h->d_status, &zero, sizeof(int), cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    return st;
}

// ---- asynchronous timing: pooled events and pending (stage, start, end) triples
int record(cqpi_handle *h)
{
    if (h->capturing) return -1;   // no timing events inside a captured graph
    int idx;
    if (!h->ev_free.empty()) {
        const cudaEvent_t e = h->ev_free.back();
        h->ev_free.pop_back();
        h->ev_pool.push_back(e);
    } else {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        h->ev_pool.push_back(e);
    }
    idx = (int)h->ev_pool.size() - 1;
    CK(cudaEventRecord(h->ev_pool[idx], h->stream));
    return idx;
}

void pend(cqpi_handle *h, int stage, int a, int b)
{
    if (a < 0 || b < 0) return;
    h->ev_pending.push_back(stage);
    h->ev_pending.push_back(a);
    h->ev_pending.push_back(b);
}

// Sum the pending stage intervals into stage_ms (totals since the previous query).
void collect_times(cqpi_handle *h)
{
    if (h->capturing) return;
    for (int i = 0; i < 5; i++) h->stage_ms[i] = 0.f;
    if (!h->ev_pool.empty()) CK(cudaEventSynchronize(h->ev_pool.back()));
    for (size_t i = 0; i + 2 < h->ev_pending.size(); i += 3) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, h->ev_pool[h->ev_pending[i + 1]], h->ev_pool[h->ev_pending[i + 2]]));
        h->stage_ms[h->ev_pending[i]] += ms;
        h->stage_ms[4] += ms;
    }
    for (cudaEvent_t e : h->ev_pool) h->ev_free.push_back(e);
    h->ev_pool.clear();
    h->ev_pending.clear();
}

void ensure_energies(cqpi_handle *h, int n)
{
    if (h->energies_cap >= n) return;
    dfree(h->d_energies_all);
    dfree(h->d_tip_all);
    if (h->h_energies_pinned) cudaFreeHost(h->h_energies_pinned);
    if (h->h_tip_pinned) cudaFreeHost(h->h_tip_pinned);
    h->h_energies_pinned = nullptr;
    h->h_tip_pinned = nullptr;
    h->energies_cap = 0;
    dalloc(&h->d_energies_all, (size_t)n);
    dalloc(&h->d_tip_all, (size_t)n);
    CK(cudaMallocHost((void **)&h->h_energies_pinned, sizeof(double) * n));
    CK(cudaMallocHost((void **)&h->h_tip_pinned, sizeof(double2) * n));
    h->energies_cap = n;
}

// The driver's Josephson tip factor (src/calcqpi.cc:705-708):
//   tip = (0, -sign(E) pi deltat) / sqrt((E + i etat)^2 - deltat^2)
// with the principal square root in the textbook careful form (t = sqrt((|x| + |z|)/2),
// the other part y / (2t)); sign(E) = copysign(1, E).
double2 josephson_tip(double energy, double deltat, double etat)
{
    const double zr = energy * energy - etat * etat - deltat * deltat, zi = 2.0 * energy * etat;
    double sr = 0.0, si = 0.0;
    if (zr != 0.0 || zi != 0.0) {
        const double t = std::sqrt(0.5 * (std::fabs(zr) + std::hypot(zr, zi)));
        if (zr >= 0.0) {
            sr = t;
            si = zi / (2.0 * t);
        } else {
            sr = std::fabs(zi) / (2.0 * t);
            si = std::copysign(t, zi);
        }
    }
    const double num = -std::copysign(1.0, energy) * M_PI * deltat;
    const double d = sr * sr + si * si;
    return make_double2(num * si / d, num * sr / d);
}

// Energies (and, in Josephson mode, their tip factors) of a call to the device, through the
// page-locked mirrors, on the handle's stream.
void upload_energies(cqpi_handle *h, const double *energies, int n)
{
    memcpy(h->h_energies_pinned, energies, sizeof(double) * n);
    CK(cudaMemcpyAsync(h->d_energies_all, h->h_energies_pinned, sizeof(double) * n, cudaMemcpyHostToDevice,
                       h->stream));
    if (h->josephson) {
        for (int i = 0; i < n; i++) h->h_tip_pinned[i] = josephson_tip(energies[i], h->jos_deltat, h->jos_etat);
        CK(cudaMemcpyAsync(h->d_tip_all, h->h_tip_pinned, sizeof(double2) * n, cudaMemcpyHostToDevice, h->stream));
    }
}

void ensure_fov(cqpi_handle *h, size_t n)
{
    if (h->fov_cap >= n) return;
    dfree(h->d_fov);
    dfree(h->d_fov_off);
    if (h->h_fov_pinned) cudaFreeHost(h->h_fov_pinned);
    if (h->h_off_pinned) cudaFreeHost(h->h_off_pinned);
    h->h_fov_pinned = nullptr;
    h->h_off_pinned = nullptr;
    h->fov_cap = 0;
    dalloc(&h->d_fov, n);
    dalloc(&h->d_fov_off, n);
    CK(cudaMallocHost((void **)&h->h_fov_pinned, sizeof(int) * n));
    CK(cudaMallocHost((void **)&h->h_off_pinned, sizeof(long long) * n));
    h->fov_cap = n;
}

void ensure_copy_stream(cqpi_handle *h)
{
    if (h->copy_stream) return;
    CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    for (int i = 0; i < 2; i++) {
        CK(cudaEventCreateWithFlags(&h->ev_comp[i], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&h->ev_copy[i], cudaEventDisableTiming));
    }
}

void ensure_stage32(cqpi_handle *h, size_t n)
{
    if (h->stage_cap32 >= n) return;
    dfree(h->stage32);
    h->stage_cap32 = 0;
    dalloc(&h->stage32, n);
    h->stage_cap32 = n;
}

void ensure_stage64(cqpi_handle *h, size_t n)
{
    if (h->stage_cap64 >= n) return;
    dfree(h->stage64);
    h->stage_cap64 = 0;
    dalloc(&h->stage64, n);
    h->stage_cap64 = n;
}

// ---- spin-degenerate reduction (see cqpi_handle::sr_*)
bool spin_model_reducible(const cqpi_handle *h)
{
    if (!h->spin || h->nblk != 2 || h->b != 2 * h->mb || h->blk_start[1] != h->mb) return false;
    const int b = h->b, mb = h->mb;
    // diagonal: -efermi for p < scmax, +efermi otherwise; the two blocks must agree
    for (int p = 0; p < mb; p++)
        if ((p < h->scmax) != (p + mb < h->scmax)) return false;
    const size_t bb = (size_t)b * b;
    for (int r = 0; r < h->nR; r++)
        for (int p = 0; p < b; p++)
            for (int q = 0; q < b; q++) {
                const size_t e = ((size_t)r * bb + (size_t)p * b + q) * 2;
                const bool cross = (p < mb) != (q < mb);
                for (int c = 0; c < 2; c++) {
                    const double vn = h->rt_tn[e + c], va = h->rt_ta[e + c];
                    if (cross) {
                        if (vn != 0.0 || va != 0.0) return false;
                    } else if (p < mb) {
                        const size_t e2 = ((size_t)r * bb + (size_t)(p + mb) * b + (q + mb)) * 2;
                        if (vn != h->rt_tn[e2 + c] || va != h->rt_ta[e2 + c]) return false;
                    }
                }
            }
    return true;
}

void sr_drop(cqpi_handle *h)
{
    if (h->sr_sub) cqpi_destroy(h->sr_sub);
    h->sr_sub = nullptr;
    h->sr_stale = true;
}

bool sr_active(const cqpi_handle *h)
{
    const char *f = getenv("CQPI_SPIN_REDUCE");
    return h->sr_model && h->sr_orb && h->sr_v && !h->josephson && !h->list_mode && h->gmode == CQPI_GREEN_NORMAL &&
           !(f && !strcmp(f, "0"));
}

// Create (or re-create) the mb-band handle of the reduction; shares this handle's stream.
int sr_prepare(cqpi_handle *h)
{
    if (h->sr_sub && !h->sr_stale) return CQPI_OK;
    sr_drop(h);
    const int b = h->b, mb = h->mb;
    const size_t bb = (size_t)b * b;
    std::vector<int32_t> R, orb;
    std::vector<double> t;
    std::vector<uint8_t> anti;
    for (int r = 0; r < h->nR; r++)
        for (int p = 0; p < mb; p++)
            for (int q = 0; q < mb; q++)
                for (int a = 0; a < 2; a++) {
                    const std::vector<double> &src = a ? h->rt_ta : h->rt_tn;
                    const size_t e = ((size_t)r * bb + (size_t)p * b + q) * 2;
                    if (src[e] == 0.0 && src[e + 1] == 0.0) continue;
                    R.push_back(h->rt_R[2 * r]);
                    R.push_back(h->rt_R[2 * r + 1]);
                    R.push_back(0);
                    orb.push_back(p);
                    orb.push_back(q);
                    t.push_back(src[e]);
                    t.push_back(src[e + 1]);
                    anti.push_back((uint8_t)a);
                }
    cqpi_model m;
    m.bands = mb;
    m.scmaxbands = std::min(h->scmax, mb);
    m.efermi = h->efermi;
    m.nhops = (int64_t)t.size() / 2;
    m.R = R.data();
    m.orb = orb.data();
    m.t = t.data();
    m.anti = anti.data();
    cqpi_params prm;
    prm.lattice = h->n;
    prm.kpoints = h->kp;
    prm.oversamp = h->os;
    prm.window = h->w;
    prm.maxband = mb;
    prm.spin = 0;
    prm.eta = h->eta;
    prm.precision = h->precision;
    cqpi_handle *sub = nullptr;
    int rc = cqpi_create(&m, &prm, &sub);
    if (rc != CQPI_OK) return fail(h, rc, "spin-block reduction: internal handle");
    cudaStreamDestroy(sub->stream);
    sub->stream = h->stream;
    sub->owns_stream = false;
    sub->out_scale = 2.0f;    // two identical spin blocks
    rc = cqpi_set_orbitals(sub, h->sr_wf.data(), mb, h->sr_side, h->sr_zero.data());
    if (rc == CQPI_OK) rc = cqpi_set_impurities(sub, h->sr_V.data(), h->sr_nimp);
    if (rc != CQPI_OK) {
        h->err = sub->err;
        cqpi_destroy(sub);
        return rc;
    }
    h->sr_sub = sub;
    h->sr_stale = false;
    return CQPI_OK;
}

int sr_forward(cqpi_handle *h, int rc)
{
    if (rc != CQPI_OK && h->sr_sub) h->err = h->sr_sub->err;
    return rc;
}

// Device hopping sets of the surface / bulk Green's function: surface in-plane (the surface
// model's R_z = 0 terms, or the model's), bulk in-plane (R_z = 0), bulk coupling (R_z < 0)
// (tightbind::setmatrix with kzdepinplane / kzdepoutofplane, src/tightbinding.cc:184-207).
void upload_surface_terms(cqpi_handle *h)
{
    std::vector<int4> ti;
    std::vector<double2> tt;
    std::vector<int> an;
    SurfaceTerms &S = h->surf;
    const size_t nm = h->hop_r.size();
    auto model_set = [&](bool inplane) {
        for (size_t i = 0; i < nm; i++)
            if (inplane ? h->hop_rz[i] == 0 : h->hop_rz[i] < 0) {
                ti.push_back(make_int4(h->hop_rx[i], h->hop_ry[i], h->hop_o1[i], h->hop_o2[i]));
                tt.push_back(make_double2(h->hop_t[2 * i], h->hop_t[2 * i + 1]));
                an.push_back(h->hop_anti[i]);
            }
    };
    S.off_s = 0;
    if (h->surf_own_model) {
        for (size_t i = 0; i < h->surf_anti.size(); i++)
            if (h->surf_R[3 * i + 2] == 0) {
                ti.push_back(make_int4(h->surf_R[3 * i], h->surf_R[3 * i + 1], h->surf_orb[2 * i], h->surf_orb[2 * i + 1]));
                tt.push_back(make_double2(h->surf_t[2 * i], h->surf_t[2 * i + 1]));
                an.push_back(h->surf_anti[i]);
            }
    } else {
        model_set(true);
    }
    S.ns = (int)ti.size();
    S.off_b = (int)ti.size();
    model_set(true);
    S.nb = (int)ti.size() - S.off_b;
    S.off_o = (int)ti.size();
    model_set(false);
    S.no = (int)ti.size() - S.off_o;
    if (ti.empty()) {
        ti.push_back(make_int4(0, 0, 0, 0));
        tt.push_back(make_double2(0.0, 0.0));
        an.push_back(0);
    }
    dreserve(&S.d_i, S.cap_i, ti.size());
    dreserve(&S.d_t, S.cap_t, tt.size());
    dreserve(&S.d_anti, S.cap_anti, an.size());
    CK(cudaMemcpyAsync(S.d_i, ti.data(), sizeof(int4) * ti.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(S.d_t, tt.data(), sizeof(double2) * tt.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(S.d_anti, an.data(), sizeof(int) * an.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));   // pageable temporaries
    if (!S.d_mats) dalloc(&S.d_mats, (size_t)3 * h->kp * h->kp * h->b * h->b);
}

// The k-space data of the current Green's function: the eigen cache, or in the surface /
// bulk modes the per-k in-plane and coupling matrices.
void do_bands(cqpi_handle *h)
{
    if (h->gmode != CQPI_GREEN_NORMAL) {
        upload_surface_terms(h);
        launch_surface_mats(h);
    } else {
        launch_bands(h);
    }
    check_launch();
    h->bands_ready = true;
}

// G0(k) -> G0(R) box -> T -> term1 for ne energies already in ws.energies.
void do_greens(cqpi_handle *h, int ne, const double *d_energies)
{
    if (h->gmode != CQPI_GREEN_NORMAL) {
        launch_greens_surface(h, ne, d_energies);
        check_launch();
        launch_fft(h, ne);
        check_launch();
        return;
    }
    if (h->use_fft32) {
        launch_greens_fft32(h, ne, d_energies);
        check_launch();
        return;
    }
    launch_greens_k(h, ne, d_energies);
    check_launch();
    launch_fft(h, ne);
    check_launch();
}

struct ListEnt {
    int d1, q, d2, o1, o2;
    double f;
};

// A proximity list on the device, CSR by (d1, q) with the list order kept inside every
// segment; pairs = the (o1, o2) the list uses.
int upload_list(cqpi_handle *h, const std::vector<ListEnt> &ents)
{
    const int b = h->b;
    std::vector<int> pidx((size_t)b * b, -1);
    std::vector<int2> pairs;
    for (const ListEnt &e : ents) {
        if (e.o1 < 0 || e.o2 < 0 || e.o1 >= b || e.o2 >= b)
            return fail(h, CQPI_ERR_ARG, "a proximity-list orbital is outside the band count");
        int &p = pidx[(size_t)e.o1 * b + e.o2];
        if (p < 0) {
            p = (int)pairs.size();
            pairs.push_back(make_int2(e.o1, e.o2));
        }
    }
    const int npair = std::max<int>(1, (int)pairs.size());
    if (pairs.empty()) pairs.push_back(make_int2(0, 0));
    const size_t nseg = (size_t)h->W * h->Q;
    std::vector<int> off(nseg + 1, 0), u(std::max<size_t>(ents.size(), 1), 0);
    std::vector<double> f(std::max<size_t>(ents.size(), 1), 0.0);
    for (const ListEnt &e : ents) off[(size_t)e.d1 * h->Q + e.q + 1]++;
    for (size_t k = 0; k < nseg; k++) off[k + 1] += off[k];
    std::vector<int> pos(off.begin(), off.end() - 1);
    for (const ListEnt &e : ents) {
        const int s = pos[(size_t)e.d1 * h->Q + e.q]++;
        u[s] = e.d2 * npair + pidx[(size_t)e.o1 * b + e.o2];
        f[s] = e.f;
    }
    std::vector<float> f32(f.begin(), f.end());
    h->list_npair = npair;
    h->list_count = (int64_t)ents.size();
    if (list_smem_bytes(h, true) > 227 * 1024)   // the FP64 form (also the seam's)
        return fail(h, CQPI_ERR_NOT_SUPPORTED, "proximity list: window, bands and pairs exceed the shared memory of a block");
    dfree(h->surf.d_i);
    dfree(h->surf.d_t);
    dfree(h->surf.d_anti);
    dfree(h->surf.d_mats);
    dfree(h->d_list_off);
    dfree(h->d_list_u);
    dfree(h->d_list_f);
    dfree(h->d_list_f32);
    dfree(h->d_list_pair);
    dalloc(&h->d_list_off, off.size());
    dalloc(&h->d_list_u, u.size());
    dalloc(&h->d_list_f, f.size());
    dalloc(&h->d_list_f32, f32.size());
    dalloc(&h->d_list_pair, pairs.size());
    h2d_sync(h, h->d_list_off, off.data(), off.size());
    h2d_sync(h, h->d_list_u, u.data(), u.size());
    h2d_sync(h, h->d_list_f, f.data(), f.size());
    h2d_sync(h, h->d_list_f32, f32.data(), f32.size());
    h2d_sync(h, h->d_list_pair, pairs.data(), pairs.size());
    CK(configure_list(h));
    return CQPI_OK;
}

// mkthresholdlist (src/qpi.cc:139-253) over the handle's orbitals: the entries (d1, d2, q,
// o1, o2, f) with |f| = |phi_o1 phi_o2| > threshold * max phi^2, in the maxband / spin form
// (orbitals 0 .. maxband-1, or both spin blocks of maxband/2) or the spinarr form (orbitals
// of equal non-zero label).
int build_list(cqpi_handle *h)
{
    const int wins = 2 * h->w + 1, os = h->os, xs = os * wins, norb = h->wf_norb;
    double maxval = 0.0;
    for (size_t k = 0; k < h->wf_host.size(); k++) maxval = std::max(maxval, h->wf_host[k] * h->wf_host[k]);
    const double thr = h->list_threshold * maxval;
    std::vector<ListEnt> ents;
    auto wfv = [&](int o, int x, int y) { return h->wf_host[((size_t)o * xs + x) * xs + y]; };
    auto push = [&](int xn1, int yn1, int xn2, int yn2, int i, int j, int o1, int o2) {
        const int x = i + (wins - 1) * os, y = j + (wins - 1) * os;
        const double f = wfv(o1, x - xn1 * os, y - yn1 * os) * wfv(o2, x - xn2 * os, y - yn2 * os);
        if (std::fabs(f) > thr) ents.push_back({xn1 * wins + yn1, i * os + j, xn2 * wins + yn2, o1, o2, f});
    };
    const int maxband = h->m, spinbands = maxband >> 1;
    for (int xn1 = 0; xn1 < wins; xn1++)
        for (int yn1 = 0; yn1 < wins; yn1++)
            for (int xn2 = 0; xn2 < wins; xn2++)
                for (int yn2 = 0; yn2 < wins; yn2++) {
                    if (h->list_use_spinarr) {
                        for (int o1 = 0; o1 < norb; o1++) {
                            if (!h->list_spinarr[o1]) continue;
                            for (int o2 = 0; o2 < norb; o2++) {
                                if (h->list_spinarr[o1] != h->list_spinarr[o2]) continue;
                                for (int i = 0; i < os; i++)
                                    for (int j = 0; j < os; j++) push(xn1, yn1, xn2, yn2, i, j, o1, o2);
                            }
                        }
                    } else if (h->spin) {
                        for (int o1 = 0; o1 < spinbands; o1++)
                            for (int o2 = 0; o2 < spinbands; o2++)
                                for (int i = 0; i < os; i++)
                                    for (int j = 0; j < os; j++) {
                                        push(xn1, yn1, xn2, yn2, i, j, o1, o2);
                                        push(xn1, yn1, xn2, yn2, i, j, spinbands + o1, spinbands + o2);
                                    }
                    } else {
                        for (int o1 = 0; o1 < maxband; o1++)
                            for (int o2 = 0; o2 < maxband; o2++)
                                for (int i = 0; i < os; i++)
                                    for (int j = 0; j < os; j++) push(xn1, yn1, xn2, yn2, i, j, o1, o2);
                    }
                }
    return upload_list(h, ents);
}

}  // namespace

extern "C" {

const char *cqpi_version(void) { return "cqpi-gb300 0.1 (sm_103a)"; }

const char *cqpi_status_string(int s)
{
    switch (s) {
    case CQPI_OK: return "ok";
    case CQPI_ERR_ARG: return "invalid argument";
    case CQPI_ERR_CUDA: return "CUDA error";
    case CQPI_ERR_ALLOC: return "allocation failed";
    case CQPI_ERR_DOMAIN: return "sizes outside the reference's index domain";
    case CQPI_ERR_SINGULAR: return "1 - V G0(0) is singular";
    case CQPI_ERR_STATE: return "call order violated";
    case CQPI_ERR_NOT_SUPPORTED: return "not supported";
    case CQPI_ERR_NO_DEVICE: return "no CUDA device";
    case CQPI_ERR_TIMEOUT: return "a bounded device wait timed out";
    case CQPI_ERR_NOT_CONVERGED: return "the surface / bulk decimation did not converge";
    }
    return "unknown status";
}

const char *cqpi_last_error(const cqpi_handle *h) { return h ? h->err.c_str() : "null handle"; }

int cqpi_create(const cqpi_model *model, const cqpi_params *p, cqpi_handle **out)
{
    if (!out) return CQPI_ERR_ARG;
    *out = nullptr;
    if (!model || !p) return CQPI_ERR_ARG;
    const int b = model->bands;
    if (b < 1 || b > CQPI_MAX_BANDS) return CQPI_ERR_ARG;
    if (model->nhops < 0 || (model->nhops > 0 && (!model->R || !model->orb || !model->t))) return CQPI_ERR_ARG;
    if (p->lattice < 1 || p->kpoints < 1 || p->oversamp < 1 || p->window < 0) return CQPI_ERR_ARG;
    if (p->kpoints > 8192) return CQPI_ERR_NOT_SUPPORTED;
    if (p->maxband < 1 || p->maxband > b) return CQPI_ERR_ARG;
    if (!(p->eta == p->eta)) return CQPI_ERR_ARG;   // NaN
    if (p->precision != CQPI_PREC_FP64 && p->precision != CQPI_PREC_MIXED) return CQPI_ERR_ARG;
    for (int64_t i = 0; i < model->nhops; i++) {
        if (model->orb[2 * i] < 0 || model->orb[2 * i] >= b || model->orb[2 * i + 1] < 0 || model->orb[2 * i + 1] >= b)
            return CQPI_ERR_ARG;
    }
    // The reference forms G0 indices with unsigned arithmetic, e.g.
    // (kpoints + ipos + nni2) % kpoints (src/qpi.cc:901,907,921).  They equal the
    // mathematical R mod kp when lattice/2 + window <= kp and 2*window <= kp, and
    // always when kp is a power of two (2^64 is then a multiple of kp).
    const int n2 = p->lattice >> 1;
    const bool pow2 = (p->kpoints & (p->kpoints - 1)) == 0;
    if (!pow2 && (n2 + p->window > p->kpoints || 2 * p->window > p->kpoints)) return CQPI_ERR_DOMAIN;
    // Wide output indices are 32-bit inside kernels.
    const long long wn = (long long)p->lattice * p->oversamp;
    if (wn > 46340 || (long long)p->kpoints * p->kpoints > (1LL << 31)) return CQPI_ERR_NOT_SUPPORTED;

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return CQPI_ERR_NO_DEVICE;
    }

    cqpi_handle *h = new (std::nothrow) cqpi_handle();
    if (!h) return CQPI_ERR_ALLOC;
    try {
        CK(cudaGetDevice(&h->device));
        CK(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device));
        CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        for (auto &e : h->ev) CK(cudaEventCreate(&e));
        h->b = b;
        h->scmax = model->scmaxbands;
        h->efermi = model->efermi;
        h->n = p->lattice;
        h->kp = p->kpoints;
        h->os = p->oversamp;
        h->w = p->window;
        h->m = p->maxband;
        h->spin = p->spin ? 1 : 0;
        h->eta = p->eta;
        h->precision = p->precision;
        h->Rb = std::max(n2 + h->w, 2 * h->w);
        h->NB = 2 * h->Rb + 1;
        h->W = (2 * h->w + 1) * (2 * h->w + 1);
        h->Q = h->os * h->os;
        h->wn = (int)wn;
        if (h->spin) {
            // spin mode pairs orbitals inside [0, m/2) and [m/2, 2*(m/2)) (src/qpi.cc:924-940)
            h->nblk = 2;
            h->mb = h->m >> 1;
            h->blk_start[0] = 0;
            h->blk_start[1] = h->mb;
        } else {
            h->nblk = 1;
            h->mb = h->m;
        }

        // unique in-plane R with summed normal / conjugated (anti) hopping matrices; kz = 0
        std::map<std::pair<int, int>, int> idx;
        std::vector<int32_t> Rv;
        std::vector<double> tn, ta;
        const size_t bb = (size_t)b * b;
        for (int64_t i = 0; i < model->nhops; i++) {
            auto key = std::make_pair(model->R[3 * i], model->R[3 * i + 1]);
            auto it = idx.find(key);
            int r;
            if (it == idx.end()) {
                r = (int)idx.size();
                idx[key] = r;
                Rv.push_back(key.first);
                Rv.push_back(key.second);
                tn.resize(tn.size() + 2 * bb, 0.0);
                ta.resize(ta.size() + 2 * bb, 0.0);
            } else {
                r = it->second;
            }
            const size_t e = (size_t)r * bb + (size_t)model->orb[2 * i] * b + model->orb[2 * i + 1];
            const bool anti = model->anti && model->anti[i];
            std::vector<double> &dst = anti ? ta : tn;
            dst[2 * e] += model->t[2 * i];
            dst[2 * e + 1] += model->t[2 * i + 1];
            h->hop_r.push_back(r);
            h->hop_rx.push_back(model->R[3 * i]);
            h->hop_ry.push_back(model->R[3 * i + 1]);
            h->hop_rz.push_back(model->R[3 * i + 2]);
            h->hop_t.push_back(model->t[2 * i]);
            h->hop_t.push_back(model->t[2 * i + 1]);
            h->hop_o1.push_back(model->orb[2 * i]);
            h->hop_o2.push_back(model->orb[2 * i + 1]);
            h->hop_anti.push_back(anti ? 1 : 0);
        }
        h->nR = (int)idx.size();
        h->rt_tn = tn;
        h->rt_ta = ta;
        h->rt_R = Rv;
        // real hoppings: H(-k) = conj(H(k)), the eigen-solve covers half the k-grid
        // (CQPI_TIME_REVERSAL=0 solves every k-point)
        {
            bool real = true;
            for (size_t q = 1; q < tn.size(); q += 2) real = real && tn[q] == 0.0 && ta[q] == 0.0;
            const char *f = getenv("CQPI_TIME_REVERSAL");
            h->time_reversal = real && !(f && !strcmp(f, "0"));
        }
        dalloc(&h->d_R, Rv.size());
        dalloc(&h->d_tn, tn.size());
        dalloc(&h->d_ta, ta.size());
        if (h->nR) {
            h2d_sync(h, h->d_R, Rv.data(), Rv.size());
            h2d_sync(h, h->d_tn, tn.data(), tn.size());
            h2d_sync(h, h->d_ta, ta.data(), ta.size());
        }
        upload_pairs(h);
        // twiddles e^{+2 pi i t / kp}
        std::vector<double2> tw(h->kp);
        for (int t = 0; t < h->kp; t++) {
            double s, c;
            sincospi(2.0 * t / h->kp, &s, &c);
            tw[t] = make_double2(c, s);
        }
        dalloc(&h->d_tw, h->kp);
        h2d_sync(h, h->d_tw, tw.data(), (size_t)h->kp);
        const size_t nk = (size_t)h->kp * h->kp;
        dalloc(&h->d_eval, nk * b);
        dalloc(&h->d_evec, nk * bb);
        if (h->precision == CQPI_PREC_MIXED) {
            dalloc(&h->d_evec32, nk * bb);
            dalloc(&h->d_eval32, nk * b);
            std::vector<float2> tw32(h->kp);
            for (int t = 0; t < h->kp; t++) tw32[t] = make_float2((float)tw[t].x, (float)tw[t].y);
            dalloc(&h->d_tw32, h->kp);
            h2d_sync(h, h->d_tw32, tw32.data(), (size_t)h->kp);
        }
        dalloc(&h->d_status, 1);
        CK(cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
        // default scattering: phase (1,0) on every band (src/qpi.h:99)
        h->nimp = 1;
        std::vector<double2> V(bb, make_double2(0.0, 0.0));
        for (int i = 0; i < b; i++) V[(size_t)i * b + i] = make_double2(1.0, 0.0);
        dalloc(&h->d_V, bb);
        h2d_sync(h, h->d_V, V.data(), bb);
        // the transform kernels keep whole rows / column tiles in shared memory
        CK(configure_fft(h));
        // tensor-core contraction for the mixed path (CUDA-core FP32 kernel otherwise);
        // CQPI_CONTRACTION=fp32 selects the CUDA-core kernel explicitly
        // fused G0(k) + row transform for up to 4 bands (all b^2 planes of a k-point are
        // built from registers); more bands go through G0(k) planes in HBM and the separate
        // transforms, which read the eigen cache once per energy instead of once per plane group
        if (h->precision == CQPI_PREC_MIXED && fft32_supported(h)) {
            const char *f = getenv("CQPI_GREENS");
            h->use_fft32 = b <= 4 && !(f && !strcmp(f, "unfused"));
            if (f && !strcmp(f, "fused")) h->use_fft32 = true;
            CK(configure_fft32(h));
        }
        if (h->precision == CQPI_PREC_MIXED && tc_supported(h)) {
            tc_plan(h);
            const char *force = getenv("CQPI_CONTRACTION");
            h->use_tc = h->tc.ok && !(force && !strcmp(force, "fp32"));
        }
        h->sr_model = spin_model_reducible(h);
    } catch (const CudaError &e) {
        int rc = cuda_fail(h, e);
        cqpi_destroy(h);
        return rc;
    } catch (const std::bad_alloc &) {
        cqpi_destroy(h);
        return CQPI_ERR_ALLOC;
    }
    *out = h;
    return CQPI_OK;
}

int cqpi_destroy(cqpi_handle *h)
{
    if (!h) return CQPI_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_workspace(h);
    free_adj(h);
    dfree(h->d_fov);
    dfree(h->d_fov_off);
    if (h->h_fov_pinned) cudaFreeHost(h->h_fov_pinned);
    if (h->h_off_pinned) cudaFreeHost(h->h_off_pinned);
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    dfree(h->d_R);
    dfree(h->d_tn);
    dfree(h->d_ta);
    dfree(h->d_pR);
    dfree(h->d_pPQ);
    dfree(h->d_tw);
    dfree(h->d_tw32);
    dfree(h->d_eval);
    dfree(h->d_evec);
    dfree(h->d_evec32);
    dfree(h->d_eval32);
    dfree(h->d_phi);
    dfree(h->d_phi32);
    dfree(h->d_tc_a);
    dfree(h->d_tc_aw);
    dfree(h->d_seam_box);
    dfree(h->d_seam_T);
    dfree(h->d_seam_term1);
    dfree(h->d_seam_tip);
    dfree(h->d_list_off);
    dfree(h->d_list_u);
    dfree(h->d_list_f);
    dfree(h->d_list_f32);
    dfree(h->d_list_pair);
    dfree(h->d_V);
    dfree(h->d_status);
    dfree(h->d_seam_ldos);
    for (auto &e : h->ev)
        if (e) cudaEventDestroy(e);
    for (auto e : h->ev_pool) cudaEventDestroy(e);
    for (auto e : h->ev_free) cudaEventDestroy(e);
    dfree(h->d_energies_all);
    dfree(h->d_tip_all);
    if (h->h_energies_pinned) cudaFreeHost(h->h_energies_pinned);
    if (h->h_tip_pinned) cudaFreeHost(h->h_tip_pinned);
    dfree(h->stage32);
    dfree(h->stage64);
    sr_drop(h);
    if (h->copy_stream) {
        cudaStreamDestroy(h->copy_stream);
        for (int i = 0; i < 2; i++) {
            cudaEventDestroy(h->ev_comp[i]);
            cudaEventDestroy(h->ev_copy[i]);
        }
    }
    if (h->stream && h->owns_stream) cudaStreamDestroy(h->stream);
    cudaGetLastError();
    delete h;
    return CQPI_OK;
}

int cqpi_set_orbitals(cqpi_handle *h, const double *wf, int32_t norb, int32_t side, const uint8_t *is_zero)
{
    if (!h || !wf) return fail(h, CQPI_ERR_ARG, "null argument");
    if (side != (2 * h->w + 1) * h->os) return fail(h, CQPI_ERR_ARG, "orbital side must be (2*window+1)*oversamp");
    const int need = h->spin ? 2 * h->mb : h->m;
    if (norb < need) return fail(h, CQPI_ERR_ARG, "fewer orbitals than maxband");
    // phi[blk][q][d][ol] = wf[o](w*os + qx - dx*os, w*os + qy - dy*os)  (src/qpi.cc:912-918)
    const int side1 = 2 * h->w + 1;
    std::vector<double> phi((size_t)h->nblk * h->Q * h->W * h->mb, 0.0);
    for (int blk = 0; blk < h->nblk; blk++)
        for (int qx = 0; qx < h->os; qx++)
            for (int qy = 0; qy < h->os; qy++)
                for (int d = 0; d < h->W; d++) {
                    const int dx = d / side1 - h->w, dy = d % side1 - h->w;
                    const int ix = h->w * h->os + qx - dx * h->os, iy = h->w * h->os + qy - dy * h->os;
                    for (int ol = 0; ol < h->mb; ol++) {
                        const int o = h->blk_start[blk] + ol;
                        double v = 0.0;
                        if (!(is_zero && is_zero[o])) v = wf[((size_t)o * side + ix) * side + iy];
                        phi[((((size_t)blk * h->Q) + qx * h->os + qy) * h->W + d) * h->mb + ol] = v;
                    }
                }
    try {
        // the stream may still read the previous images: uploads are ordered on it
        dreserve(&h->d_phi, h->cap_phi, phi.size());
        CK(cudaMemcpyAsync(h->d_phi, phi.data(), sizeof(double) * phi.size(), cudaMemcpyHostToDevice, h->stream));
        std::vector<float> phi32(phi.begin(), phi.end());
        dreserve(&h->d_phi32, h->cap_phi32, phi32.size());
        CK(cudaMemcpyAsync(h->d_phi32, phi32.data(), sizeof(float) * phi32.size(), cudaMemcpyHostToDevice, h->stream));
        std::vector<uint16_t> img, imgw;
        if (h->use_tc) {
            tc_build_a(h, phi, img, h->tc_inv_sA);
            dreserve(&h->d_tc_a, h->cap_tc_a, img.size());
            CK(cudaMemcpyAsync(h->d_tc_a, img.data(), sizeof(uint16_t) * img.size(), cudaMemcpyHostToDevice, h->stream));
            if (h->tc.win) {
                tc_build_a_window(h, phi, imgw);
                dreserve(&h->d_tc_aw, h->cap_tc_aw, imgw.size());
                CK(cudaMemcpyAsync(h->d_tc_aw, imgw.data(), sizeof(uint16_t) * imgw.size(), cudaMemcpyHostToDevice,
                                   h->stream));
            }
        }
        CK(cudaStreamSynchronize(h->stream));   // the host vectors are pageable temporaries
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    h->orbitals_ready = true;
    // host copy for the proximity list (zero orbitals as zeros, src/wannierfunctions.cc)
    {
        const size_t n2 = (size_t)side * side;
        h->wf_host.assign(wf, wf + (size_t)norb * n2);
        h->wf_norb = norb;
        if (is_zero)
            for (int o = 0; o < norb; o++)
                if (is_zero[o]) std::fill(h->wf_host.begin() + o * n2, h->wf_host.begin() + (o + 1) * n2, 0.0);
    }
    if (h->list_mode && h->list_from_orbitals) {
        try {
            const int rc = build_list(h);
            if (rc != CQPI_OK) return rc;
        } catch (const CudaError &e) {
            return cuda_fail(h, e);
        }
    }
    // spin reduction: the two spin blocks carry the same orbitals
    h->sr_orb = false;
    if (h->spin && h->nblk == 2 && norb >= 2 * h->mb) {
        const size_t n2 = (size_t)side * side;
        bool same = true;
        for (int o = 0; o < h->mb && same; o++) {
            const bool z0 = is_zero && is_zero[o], z1 = is_zero && is_zero[o + h->mb];
            same = z0 == z1 && (z0 || std::equal(wf + o * n2, wf + (o + 1) * n2, wf + (o + h->mb) * n2));
        }
        if (same) {
            h->sr_orb = true;
            h->sr_side = side;
            h->sr_wf.assign(wf, wf + (size_t)h->mb * n2);
            h->sr_zero.assign(h->mb, 0);
            for (int o = 0; o < h->mb; o++) h->sr_zero[o] = (is_zero && is_zero[o]) ? 1 : 0;
            if (h->sr_sub) {
                const int rc = cqpi_set_orbitals(h->sr_sub, h->sr_wf.data(), h->mb, side, h->sr_zero.data());
                if (rc != CQPI_OK) sr_drop(h);
            }
        }
    }
    return CQPI_OK;
}

int cqpi_set_impurities(cqpi_handle *h, const double *V, int32_t nimp)
{
    if (!h || !V || nimp < 1) return fail(h, CQPI_ERR_ARG, "invalid impurity list");
    const size_t bb = (size_t)h->b * h->b;
    try {
        dfree(h->d_V);
        dalloc(&h->d_V, bb * nimp);
        h2d_sync(h, h->d_V, reinterpret_cast<const double2 *>(V), bb * nimp);
        if (nimp > h->nimp) {
            free_workspace(h);
            free_adj(h);
        }
        h->nimp = nimp;
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    // spin reduction: every V is block diagonal with two equal blocks
    h->sr_v = false;
    if (h->spin && h->nblk == 2 && h->b == 2 * h->mb) {
        const int b = h->b, mb = h->mb;
        bool ok = true;
        std::vector<double> half((size_t)nimp * mb * mb * 2);
        for (int i = 0; i < nimp && ok; i++)
            for (int p = 0; p < b && ok; p++)
                for (int q = 0; q < b && ok; q++) {
                    const double *v = V + (((size_t)i * b + p) * b + q) * 2;
                    if ((p < mb) != (q < mb)) {
                        ok = v[0] == 0.0 && v[1] == 0.0;
                    } else if (p < mb) {
                        const double *v2 = V + (((size_t)i * b + p + mb) * b + q + mb) * 2;
                        ok = v[0] == v2[0] && v[1] == v2[1];
                        half[(((size_t)i * mb + p) * mb + q) * 2] = v[0];
                        half[(((size_t)i * mb + p) * mb + q) * 2 + 1] = v[1];
                    }
                }
        if (ok) {
            h->sr_v = true;
            h->sr_V.swap(half);
            h->sr_nimp = nimp;
            if (h->sr_sub && cqpi_set_impurities(h->sr_sub, h->sr_V.data(), nimp) != CQPI_OK) sr_drop(h);
        }
    }
    return CQPI_OK;
}

int cqpi_set_scattering(cqpi_handle *h, const double *vscat)
{
    if (!h || !vscat) return fail(h, CQPI_ERR_ARG, "null argument");
    const int b = h->b;
    std::vector<double> V((size_t)2 * b * b, 0.0);
    for (int i = 0; i < b; i++) {
        V[2 * ((size_t)i * b + i)] = vscat[2 * i];
        V[2 * ((size_t)i * b + i) + 1] = vscat[2 * i + 1];
    }
    return cqpi_set_impurities(h, V.data(), 1);
}

int cqpi_solve_bands(cqpi_handle *h)
{
    if (!h) return CQPI_ERR_ARG;
    if (sr_active(h)) {
        const int rc = sr_prepare(h);
        if (rc != CQPI_OK) return rc;
        h->sr_sub->capturing = h->capturing;
        return sr_forward(h, cqpi_solve_bands(h->sr_sub));
    }
    try {
        const int a = record(h);
        do_bands(h);
        pend(h, 0, a, record(h));
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

int cqpi_run(cqpi_handle *h, const double *energies, int32_t nE, float *maps32, double *maps64, int32_t on_device)
{
    if (!h) return CQPI_ERR_ARG;
    if (sr_active(h) && h->orbitals_ready) {
        const int rc = sr_prepare(h);
        if (rc != CQPI_OK) return rc;
        h->sr_sub->capturing = h->capturing;
        return sr_forward(h, cqpi_run(h->sr_sub, energies, nE, maps32, maps64, on_device));
    }
    if (nE < 0 || (nE > 0 && !energies)) return fail(h, CQPI_ERR_ARG, "invalid energy list");
    if (!h->orbitals_ready) return fail(h, CQPI_ERR_STATE, "cqpi_set_orbitals has not been called");
    if (nE == 0) return CQPI_OK;
    const size_t mapn = (size_t)h->wn * h->wn;
    const size_t per_e = (size_t)h->nimp * mapn;
    try {
        // host outputs: the device-to-host copy (~0.2 TB/s, against ~7 TB/s of HBM) of a batch can
        // start only when the batch is complete, so batches of a few energies keep the copy of the
        // last one short while the copies of the others run behind the computation
        const int eb = on_device ? choose_batch(h, nE) : std::min(choose_batch(h, nE), host_batch());
        if (h->capturing && (h->ws.ebatch < eb || h->energies_cap < nE || !on_device || !h->bands_ready))
            return fail(h, CQPI_ERR_STATE, "capture needs device outputs, solved bands and buffers of an earlier identical call");
        ensure_workspace(h, eb);
        ensure_energies(h, nE);
        if (h->ev_pool.size() > 2048) collect_times(h);   // bounded event pool when nobody queries
        // host outputs (and float64-only requests on the tensor-core path) go through
        // device staging buffers kept by the handle; host outputs use two staging slots and
        // a copy stream, so the copy of batch k overlaps the computation of batch k+1
        const int nslot = on_device ? 1 : 2;
        const size_t slot_n = (size_t)eb * per_e;
        const bool need32 = (!on_device && maps32) || (tc_active(h) && !maps32);
        if (need32) ensure_stage32(h, nslot * slot_n);
        if (!on_device && maps64) ensure_stage64(h, nslot * slot_n);
        if (!on_device) ensure_copy_stream(h);
        upload_energies(h, energies, nE);
        if (!h->bands_ready) {
            const int a = record(h);
            do_bands(h);
            pend(h, 0, a, record(h));
        }
        for (int e0 = 0, bi = 0, ne = 0; e0 < nE; e0 += ne, bi++) {
            ne = std::min(eb, nE - e0);
            const int slot = bi % nslot;
            const double *den = h->d_energies_all + e0;
            h->jos_tip = h->josephson ? h->d_tip_all + e0 : nullptr;
            float *s32 = need32 ? h->stage32 + slot * slot_n : nullptr;
            double *s64 = (!on_device && maps64) ? h->stage64 + slot * slot_n : nullptr;
            float *tmp32 = need32 ? s32 : nullptr;
            // the slot's previous contents (batch bi - 2) must have reached the host
            if (!on_device && bi >= 2) CK(cudaStreamWaitEvent(h->stream, h->ev_copy[slot], 0));
            if (h->ws.gmax) CK(cudaMemsetAsync(h->ws.gmax, 0, sizeof(unsigned) * ne, h->stream));
            const int t0 = record(h);
            do_greens(h, ne, den);
            const int t1 = record(h);
            launch_tmatrix(h, ne);
            check_launch();
            do_term1(h, ne);
            check_launch();
            const int t2 = record(h);
            float *o32 = maps32 ? (on_device ? maps32 + (size_t)e0 * per_e : s32) : nullptr;
            double *o64 = maps64 ? (on_device ? maps64 + (size_t)e0 * per_e : s64) : nullptr;
            launch_contraction(h, ne, o32, o64, tmp32);
            check_launch();
            const int t3 = record(h);
            pend(h, 1, t0, t1);
            pend(h, 2, t1, t2);
            pend(h, 3, t2, t3);
            if (!on_device) {
                CK(cudaEventRecord(h->ev_comp[slot], h->stream));
                CK(cudaStreamWaitEvent(h->copy_stream, h->ev_comp[slot], 0));
                if (maps32)
                    CK(cudaMemcpyAsync(maps32 + (size_t)e0 * per_e, s32, sizeof(float) * ne * per_e,
                                       cudaMemcpyDeviceToHost, h->copy_stream));
                if (maps64)
                    CK(cudaMemcpyAsync(maps64 + (size_t)e0 * per_e, s64, sizeof(double) * ne * per_e,
                                       cudaMemcpyDeviceToHost, h->copy_stream));
                CK(cudaEventRecord(h->ev_copy[slot], h->copy_stream));
            }
        }
        h->jos_tip = nullptr;
        h->status_pending = true;
        if (!on_device) {
            CK(cudaStreamSynchronize(h->copy_stream));
            CK(cudaStreamSynchronize(h->stream));
            h->status_pending = false;
            if (const int st = read_status(h)) return status_code(h, st, "the batch");
        }
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

int cqpi_run_fov(cqpi_handle *h, const double *energies, int32_t nE, const int32_t *fov, float *maps, int32_t on_device)
{
    if (!h) return CQPI_ERR_ARG;
    if (sr_active(h) && h->orbitals_ready) {
        const int rc = sr_prepare(h);
        if (rc != CQPI_OK) return rc;
        h->sr_sub->capturing = h->capturing;
        return sr_forward(h, cqpi_run_fov(h->sr_sub, energies, nE, fov, maps, on_device));
    }
    if (nE < 0 || (nE > 0 && (!energies || !fov || !maps))) return fail(h, CQPI_ERR_ARG, "invalid energies, fields of view or maps");
    if (!h->orbitals_ready) return fail(h, CQPI_ERR_STATE, "cqpi_set_orbitals has not been called");
    if (!on_device) return fail(h, CQPI_ERR_NOT_SUPPORTED, "cqpi_run_fov writes device memory (on_device = 1)");
    if (!tc_window_usable(h))
        return fail(h, CQPI_ERR_NOT_SUPPORTED, "per-map fields of view need the mixed-precision direct-window contraction");
    if (nE == 0) return CQPI_OK;
    const size_t nmap = (size_t)nE * h->nimp;
    for (size_t k = 0; k < nmap; k++)
        if (fov[k] < 1 || fov[k] > h->n) return fail(h, CQPI_ERR_ARG, "field of view outside 1..lattice");
    try {
        const int eb = choose_batch(h, nE);
        if (h->capturing && (h->ws.ebatch < eb || h->energies_cap < nE || h->fov_cap < nmap))
            return fail(h, CQPI_ERR_STATE, "buffers must be allocated before capture: run the same call once first");
        ensure_workspace(h, eb);
        ensure_energies(h, nE);
        ensure_fov(h, nmap);
        long long off = 0;
        for (size_t k = 0; k < nmap; k++) {
            h->h_fov_pinned[k] = fov[k];
            h->h_off_pinned[k] = off;
            off += (long long)fov[k] * h->os * fov[k] * h->os;
        }
        upload_energies(h, energies, nE);
        CK(cudaMemcpyAsync(h->d_fov, h->h_fov_pinned, sizeof(int) * nmap, cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->d_fov_off, h->h_off_pinned, sizeof(long long) * nmap, cudaMemcpyHostToDevice, h->stream));
        if (!h->bands_ready) {
            if (h->capturing) return fail(h, CQPI_ERR_STATE, "solve the bands before capture");
            const int a = record(h);
            do_bands(h);
            pend(h, 0, a, record(h));
        }
        for (int e0 = 0; e0 < nE; e0 += eb) {
            const int ne = std::min(eb, nE - e0);
            const double *den = h->d_energies_all + e0;
            h->jos_tip = h->josephson ? h->d_tip_all + e0 : nullptr;
            if (h->ws.gmax) CK(cudaMemsetAsync(h->ws.gmax, 0, sizeof(unsigned) * ne, h->stream));
            const int t0 = record(h);
            do_greens(h, ne, den);
            const int t1 = record(h);
            launch_tmatrix(h, ne);
            check_launch();
            do_term1(h, ne);
            check_launch();
            const int t2 = record(h);
            CK(launch_ldos_tc(h, ne, maps, h->d_fov + (size_t)e0 * h->nimp, h->d_fov_off + (size_t)e0 * h->nimp));
            const int t3 = record(h);
            pend(h, 1, t0, t1);
            pend(h, 2, t1, t2);
            pend(h, 3, t2, t3);
        }
        h->jos_tip = nullptr;
        h->status_pending = true;
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

int cqpi_autotune(cqpi_handle *h, const double *energies, int32_t nE, float *best_ms, int32_t *tried)
{
    if (!h) return CQPI_ERR_ARG;
    if (nE < 1 || !energies) return fail(h, CQPI_ERR_ARG, "invalid energy list");
    if (!h->orbitals_ready) return fail(h, CQPI_ERR_STATE, "cqpi_set_orbitals has not been called");
    if (h->capturing) return fail(h, CQPI_ERR_STATE, "not during a capture");
    if (sr_active(h)) {
        const int rc = sr_prepare(h);
        if (rc != CQPI_OK) return rc;
        return sr_forward(h, cqpi_autotune(h->sr_sub, energies, nE, best_ms, tried));
    }
    if (!tc_window_usable(h)) return fail(h, CQPI_ERR_NOT_SUPPORTED, "autotuning covers the direct-window tensor-core contraction");
    try {
        const int ne = choose_batch(h, nE);
        const size_t per_e = (size_t)h->nimp * h->wn * h->wn;
        ensure_workspace(h, ne);
        ensure_energies(h, nE);
        ensure_stage32(h, (size_t)ne * per_e);
        upload_energies(h, energies, ne);
        h->jos_tip = h->josephson ? h->d_tip_all : nullptr;
        if (!h->bands_ready) do_bands(h);
        if (h->ws.gmax) CK(cudaMemsetAsync(h->ws.gmax, 0, sizeof(unsigned) * ne, h->stream));
        do_greens(h, ne, h->d_energies_all);
        launch_tmatrix(h, ne);
        do_term1(h, ne);
        check_launch();
        float ms = 0.f;
        int n = 0;
        const cudaError_t te = tc_autotune(h, ne, h->stage32, &ms, &n);
        h->jos_tip = nullptr;
        CK(te);
        if (best_ms) *best_ms = ms;
        if (tried) *tried = n;
        if (const int st = read_status(h)) return status_code(h, st, "autotuning");
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

int cqpi_graph_begin(cqpi_handle *h)
{
    if (!h) return CQPI_ERR_ARG;
    if (h->capturing) return fail(h, CQPI_ERR_STATE, "capture already active");
    try {
        collect_times(h);
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    h->capturing = true;
    h->graph_kernels = h->launches;
    h->graph_kernels_sub = h->sr_sub ? h->sr_sub->launches : 0;
    return CQPI_OK;
}

int cqpi_graph_end(cqpi_handle *h)
{
    if (!h) return CQPI_ERR_ARG;
    if (!h->capturing) return fail(h, CQPI_ERR_STATE, "no capture active");
    h->capturing = false;
    int64_t sub_delta = 0;
    if (h->sr_sub) {
        h->sr_sub->capturing = false;
        sub_delta = h->sr_sub->launches - h->graph_kernels_sub;
        h->sr_sub->launches -= sub_delta;                 // captured, not yet run
    }
    h->graph_kernels = h->launches - h->graph_kernels;   // kernels per replay
    h->launches -= h->graph_kernels;                      // captured, not yet run
    h->graph_kernels += sub_delta;
    try {
        cudaGraph_t g = nullptr;
        CK(cudaStreamEndCapture(h->stream, &g));
        if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
        if (h->graph) cudaGraphDestroy(h->graph);
        h->graph = g;
        h->graph_exec = nullptr;
        CK(cudaGraphInstantiate(&h->graph_exec, g, 0));
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

int cqpi_graph_launch(cqpi_handle *h)
{
    if (!h) return CQPI_ERR_ARG;
    if (!h->graph_exec) return fail(h, CQPI_ERR_STATE, "no captured graph");
    try {
        CK(cudaGraphLaunch(h->graph_exec, h->stream));
        h->launches += h->graph_kernels;
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    h->status_pending = true;
    return CQPI_OK;
}

int cqpi_set_hoppings(cqpi_handle *h, const double *t)
{
    if (!h || !t) return CQPI_ERR_ARG;
    const size_t bb = (size_t)h->b * h->b;
    std::vector<double> tn(h->rt_tn.size(), 0.0), ta(h->rt_ta.size(), 0.0);
    for (size_t i = 0; i < h->hop_r.size(); i++) {
        if (!(t[2 * i] == t[2 * i]) || !(t[2 * i + 1] == t[2 * i + 1])) return fail(h, CQPI_ERR_ARG, "NaN hopping");
        const size_t e = (size_t)h->hop_r[i] * bb + (size_t)h->hop_o1[i] * h->b + h->hop_o2[i];
        std::vector<double> &dst = h->hop_anti[i] ? ta : tn;
        dst[2 * e] += t[2 * i];
        dst[2 * e + 1] += t[2 * i + 1];
    }
    bool real = true;
    for (size_t q = 1; q < tn.size(); q += 2) real = real && tn[q] == 0.0 && ta[q] == 0.0;
    const char *f = getenv("CQPI_TIME_REVERSAL");
    try {
        if (!tn.empty()) {
            CK(cudaMemcpyAsync(h->d_tn, tn.data(), sizeof(double) * tn.size(), cudaMemcpyHostToDevice, h->stream));
            CK(cudaMemcpyAsync(h->d_ta, ta.data(), sizeof(double) * ta.size(), cudaMemcpyHostToDevice, h->stream));
            CK(cudaStreamSynchronize(h->stream));
        }
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    h->rt_tn.swap(tn);
    h->rt_ta.swap(ta);
    h->hop_t.assign(t, t + 2 * h->hop_r.size());
    try {
        upload_pairs(h);
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    h->time_reversal = real && !(f && !strcmp(f, "0"));
    h->bands_ready = false;
    h->sr_model = spin_model_reducible(h);
    sr_drop(h);
    return CQPI_OK;
}

int cqpi_adjoint(cqpi_handle *h, const double *energies, int32_t nE, const float *dL_dmaps, int32_t on_device,
                 double *dL_dt, double *dL_dV)
{
    if (!h) return CQPI_ERR_ARG;
    if (nE < 0 || (nE > 0 && (!energies || !dL_dmaps))) return fail(h, CQPI_ERR_ARG, "invalid energies or map gradient");
    if (!h->orbitals_ready) return fail(h, CQPI_ERR_STATE, "cqpi_set_orbitals has not been called");
    if (h->josephson) return fail(h, CQPI_ERR_NOT_SUPPORTED, "adjoint: Josephson mode is not supported");
    if (h->list_mode) return fail(h, CQPI_ERR_NOT_SUPPORTED, "adjoint: the proximity-list form is not supported");
    if (h->gmode != CQPI_GREEN_NORMAL)
        return fail(h, CQPI_ERR_NOT_SUPPORTED, "adjoint: surface / bulk Green's functions are not supported");
    if (h->nblk != 1) return fail(h, CQPI_ERR_NOT_SUPPORTED, "adjoint: spin blocks are not supported");
    if (h->kp & (h->kp - 1)) return fail(h, CQPI_ERR_NOT_SUPPORTED, "adjoint: kpoints must be a power of two");
    if (h->Q > 128) return fail(h, CQPI_ERR_NOT_SUPPORTED, "adjoint: oversamp^2 must be <= 128");
    const size_t bb = (size_t)h->b * h->b, nk = (size_t)h->kp * h->kp;
    const size_t mapn = (size_t)h->wn * h->wn, per_e = (size_t)h->nimp * mapn;
    const int nhops = (int)h->hop_r.size();
    try {
        // energies per batch: also bounded by the stored window gradients of every site
        // (2 x W x orbitals x bands complex values per site and map) within 8 GiB
        const size_t win_map = 2 * (h->precision == CQPI_PREC_FP64 ? 16 : 8) * (size_t)h->W * h->mb * h->b *
                               (size_t)h->n * h->n * (size_t)std::max(h->nimp, 1);
        const size_t gk_e = (h->precision == CQPI_PREC_FP64 ? 16 : 8) * (size_t)h->b * h->b * h->kp * h->kp;
        const int eb = std::max(1, std::min(choose_batch(h, std::max(nE, 1)), (int)(((size_t)12 << 30) / (win_map + gk_e))));
        ensure_workspace(h, eb);
        ensure_adj(h, eb);
        ensure_energies(h, std::max(nE, 1));
        if (!on_device && nE > 0) ensure_stage32(h, (size_t)eb * per_e);
        CK(cudaMemsetAsync(h->adj.C, 0, sizeof(double2) * bb * nk, h->stream));
        CK(cudaMemsetAsync(h->adj.gR, 0, sizeof(double2) * (size_t)std::max(h->nR, 1) * 2 * bb, h->stream));
        CK(cudaMemsetAsync(h->adj.gV, 0, sizeof(double2) * (size_t)std::max(h->nimp, 1) * bb, h->stream));
        if (nE > 0) {
            memcpy(h->h_energies_pinned, energies, sizeof(double) * nE);
            CK(cudaMemcpyAsync(h->d_energies_all, h->h_energies_pinned, sizeof(double) * nE, cudaMemcpyHostToDevice,
                               h->stream));
        }
        if (!h->bands_ready) do_bands(h);
        for (int e0 = 0; e0 < nE; e0 += eb) {
            const int ne = std::min(eb, nE - e0);
            const double *den = h->d_energies_all + e0;
            if (h->ws.gmax) CK(cudaMemsetAsync(h->ws.gmax, 0, sizeof(unsigned) * ne, h->stream));
            CK(cudaMemsetAsync(h->adj.gbox, 0, sizeof(double2) * ne * (size_t)h->NB * h->NB * bb, h->stream));
            CK(cudaMemsetAsync(h->adj.M, 0, sizeof(double2) * ne * (size_t)h->nimp * bb, h->stream));
            CK(cudaMemsetAsync(h->adj.wsum, 0, sizeof(double) * ne * (size_t)h->Q, h->stream));
            const float *wm = dL_dmaps + (size_t)e0 * per_e;
            if (!on_device) {
                CK(cudaMemcpyAsync(h->stage32, wm, sizeof(float) * ne * per_e, cudaMemcpyHostToDevice, h->stream));
                wm = h->stage32;
            }
            do_greens(h, ne, den);
            launch_tmatrix(h, ne);
            check_launch();
            launch_adj_energy_batch(h, ne, wm, h->adj);
            check_launch();
            for (int e = 0; e < ne; e++) {
                launch_adj_kspace(h, e, h->adj);
                check_launch();
            }
            launch_adj_kacc(h, ne, den, h->adj);
            check_launch();
        }
        launch_adj_hoppings(h, h->adj);
        check_launch();
        std::vector<double2> gR((size_t)std::max(h->nR, 1) * 2 * bb), gV((size_t)std::max(h->nimp, 1) * bb);
        CK(cudaMemcpyAsync(gR.data(), h->adj.gR, sizeof(double2) * gR.size(), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(gV.data(), h->adj.gV, sizeof(double2) * gV.size(), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (const int st = read_status(h)) return status_code(h, st, "the batch");
        if (dL_dt)
            for (int i = 0; i < nhops; i++) {
                const double2 g = gR[((size_t)h->hop_r[i] * 2 + h->hop_anti[i]) * bb + (size_t)h->hop_o1[i] * h->b + h->hop_o2[i]];
                dL_dt[2 * i] = g.x;
                dL_dt[2 * i + 1] = g.y;
            }
        if (dL_dV)
            for (size_t k = 0; k < (size_t)h->nimp * bb; k++) {
                dL_dV[2 * k] = gV[k].x;
                dL_dV[2 * k + 1] = gV[k].y;
            }
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

int cqpi_get_bands(cqpi_handle *h, double *eval, double *evec)
{
    if (!h) return CQPI_ERR_ARG;
    if (h->gmode != CQPI_GREEN_NORMAL) return fail(h, CQPI_ERR_NOT_SUPPORTED, "no eigen cache in the surface / bulk modes");
    const size_t nk = (size_t)h->kp * h->kp, b = h->b, bb = b * b;
    try {
        if (!h->bands_ready) do_bands(h);
        CK(cudaStreamSynchronize(h->stream));
        if (eval) {
            std::vector<double> t(nk * b);
            CK(cudaMemcpyAsync(t.data(), h->d_eval, sizeof(double) * t.size(), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            for (size_t k = 0; k < nk; k++)
                for (size_t n = 0; n < b; n++) eval[k * b + n] = t[n * nk + k];
        }
        if (evec) {
            std::vector<double2> t(nk * bb);
            CK(cudaMemcpyAsync(t.data(), h->d_evec, sizeof(double2) * t.size(), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            for (size_t k = 0; k < nk; k++)
                for (size_t e = 0; e < bb; e++) {
                    evec[2 * (k * bb + e)] = t[e * nk + k].x;
                    evec[2 * (k * bb + e) + 1] = t[e * nk + k].y;
                }
        }
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

int cqpi_get_greens_box(cqpi_handle *h, double energy, double *box, int32_t *rb)
{
    if (!h) return CQPI_ERR_ARG;
    if (rb) *rb = h->Rb;
    if (!box) return CQPI_OK;
    try {
        ensure_workspace(h, 1);
        if (!h->bands_ready) do_bands(h);
        CK(cudaMemcpyAsync(h->ws.energies, &energy, sizeof(double), cudaMemcpyHostToDevice, h->stream));
        if (h->ws.gmax) CK(cudaMemsetAsync(h->ws.gmax, 0, sizeof(unsigned), h->stream));
        do_greens(h, 1, h->ws.energies);
        const size_t cnt = (size_t)h->NB * h->NB * h->b * h->b;
        if (h->precision == CQPI_PREC_FP64) {
            CK(cudaMemcpyAsync(box, h->ws.box, sizeof(double2) * cnt, cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
        } else {
            std::vector<float2> t(cnt);
            CK(cudaMemcpyAsync(t.data(), h->ws.box32, sizeof(float2) * cnt, cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            for (size_t i = 0; i < cnt; i++) { box[2 * i] = t[i].x; box[2 * i + 1] = t[i].y; }
        }
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

int cqpi_get_tmatrix(cqpi_handle *h, double energy, double *T)
{
    if (!h || !T) return CQPI_ERR_ARG;
    try {
        ensure_workspace(h, 1);
        if (!h->bands_ready) do_bands(h);
        CK(cudaMemcpyAsync(h->ws.energies, &energy, sizeof(double), cudaMemcpyHostToDevice, h->stream));
        do_greens(h, 1, h->ws.energies);
        launch_tmatrix(h, 1);
        check_launch();
        CK(cudaMemcpyAsync(T, h->ws.T, sizeof(double2) * h->b * h->b, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (const int st = read_status(h)) return status_code(h, st, "the call");
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

// One energy through the FP64 contraction with a given T-matrix and full G0(R) grid; tip
// selects the Josephson form (tmatrix::calcwannierjosephson) when not NULL.
static int seam_contract(cqpi_handle *h, const double *T, const double *g0r, const double *tip, bool list)
{
    if (!h || !T || !g0r) return fail(h, CQPI_ERR_ARG, "null argument");
    if (!h->orbitals_ready) return fail(h, CQPI_ERR_STATE, "cqpi_set_orbitals has not been called");
    const size_t bb = (size_t)h->b * h->b, kp = h->kp;
    // pick the pruned box out of the full grid: box[R+Rb] = g0r[R mod kp]
    std::vector<double2> box((size_t)h->NB * h->NB * bb);
    for (int xb = 0; xb < h->NB; xb++) {
        const size_t X = (size_t)(((xb - h->Rb) % h->kp + h->kp) % h->kp);
        for (int yb = 0; yb < h->NB; yb++) {
            const size_t Y = (size_t)(((yb - h->Rb) % h->kp + h->kp) % h->kp);
            memcpy(&box[((size_t)xb * h->NB + yb) * bb], g0r + 2 * ((X * kp + Y) * bb), sizeof(double2) * bb);
        }
    }
    try {
        if (!h->d_seam_ldos) {
            dalloc(&h->d_seam_ldos, (size_t)h->wn * h->wn);
            dalloc(&h->d_seam_box, box.size());
            dalloc(&h->d_seam_T, bb);
            dalloc(&h->d_seam_term1, (size_t)h->Q);
            dalloc(&h->d_seam_tip, 1);
        }
        CK(cudaMemcpyAsync(h->d_seam_box, box.data(), sizeof(double2) * box.size(), cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->d_seam_T, T, sizeof(double2) * bb, cudaMemcpyHostToDevice, h->stream));
        if (tip) CK(cudaMemcpyAsync(h->d_seam_tip, tip, sizeof(double2), cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));   // 'box' is a pageable temporary
        const int saved = h->nimp;
        h->nimp = 1;
        h->jos_tip = tip ? h->d_seam_tip : nullptr;
        const int saved_prec = h->precision;
        h->precision = CQPI_PREC_FP64;   // the seam is FP64 on every handle
        if (list) {
            launch_term1_list(h, 1, h->d_seam_box, h->d_seam_term1);
            check_launch();
            launch_ldos_list(h, 1, h->d_seam_box, h->d_seam_T, h->d_seam_term1, nullptr, h->d_seam_ldos);
        } else {
            launch_term1_ptr(h, 1, h->d_seam_box, h->d_seam_term1);
            check_launch();
            launch_ldos_fp64(h, 1, h->d_seam_box, h->d_seam_T, h->d_seam_term1, nullptr, h->d_seam_ldos);
        }
        h->precision = saved_prec;
        h->jos_tip = nullptr;
        h->nimp = saved;
        check_launch();
        h->seam_pending = true;
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

int cqpi_wannierldos(cqpi_handle *h, const double *T, const double *g0r)
{
    if (h && h->josephson) return fail(h, CQPI_ERR_STATE, "Josephson mode is on: use cqpi_wannierjosephson");
    if (h && h->list_mode) return fail(h, CQPI_ERR_STATE, "a proximity list is set: use cqpi_wannierldoslist");
    return seam_contract(h, T, g0r, nullptr, false);
}

int cqpi_wannierldoslist(cqpi_handle *h, const double *T, const double *g0r)
{
    if (!h) return CQPI_ERR_ARG;
    if (!h->list_mode) return fail(h, CQPI_ERR_STATE, "cqpi_set_threshold has not been called");
    return seam_contract(h, T, g0r, nullptr, true);
}

int cqpi_set_list(cqpi_handle *h, int64_t nent, const int32_t *ent, const double *factor)
{
    if (!h) return CQPI_ERR_ARG;
    if (h->capturing) return fail(h, CQPI_ERR_STATE, "not during a capture");
    if (nent < 0 || (nent > 0 && (!ent || !factor))) return fail(h, CQPI_ERR_ARG, "invalid proximity list");
    if (h->Q > 512) return fail(h, CQPI_ERR_NOT_SUPPORTED, "proximity list: oversamp^2 must be <= 512");
    if (nent > (int64_t)1 << 30) return fail(h, CQPI_ERR_NOT_SUPPORTED, "proximity list longer than 2^30 entries");
    const int wins = 2 * h->w + 1;
    const int64_t nlist = (int64_t)wins * wins * wins * wins;
    std::vector<ListEnt> ents((size_t)nent);
    for (int64_t k = 0; k < nent; k++) {
        const int32_t *e = ent + 5 * k;
        if (e[0] < 0 || e[0] >= nlist || e[1] < 0 || e[1] >= h->os || e[2] < 0 || e[2] >= h->os)
            return fail(h, CQPI_ERR_ARG, "proximity-list entry outside the window or the sub-pixel grid");
        const int L = e[0], xn1 = L / (wins * wins * wins), yn1 = (L / (wins * wins)) % wins;
        const int xn2 = (L / wins) % wins, yn2 = L % wins;
        ents[(size_t)k] = {xn1 * wins + yn1, e[1] * h->os + e[2], xn2 * wins + yn2, e[3], e[4], factor[k]};
    }
    h->list_mode = true;
    h->list_from_orbitals = false;
    try {
        const int rc = upload_list(h, ents);
        if (rc != CQPI_OK) {
            h->list_mode = false;
            return rc;
        }
    } catch (const CudaError &e) {
        h->list_mode = false;
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

int cqpi_set_threshold(cqpi_handle *h, double threshold, const int32_t *spinarr, int32_t nspinarr, int64_t *count)
{
    if (!h) return CQPI_ERR_ARG;
    if (h->capturing) return fail(h, CQPI_ERR_STATE, "not during a capture");
    if (threshold != threshold) {   // NaN: the full window sum (the reference's default)
        h->list_mode = false;
        if (count) *count = 0;
        return CQPI_OK;
    }
    if (!h->orbitals_ready) return fail(h, CQPI_ERR_STATE, "cqpi_set_orbitals has not been called");
    if (h->Q > 512) return fail(h, CQPI_ERR_NOT_SUPPORTED, "proximity list: oversamp^2 must be <= 512");
    if (nspinarr < 0 || (nspinarr > 0 && !spinarr)) return fail(h, CQPI_ERR_ARG, "invalid spinarr");
    h->list_threshold = threshold;
    h->list_use_spinarr = spinarr != nullptr;
    // spinarr.resize(orbitals, 0) (src/qpi.cc:217)
    h->list_spinarr.assign(h->wf_norb, 0);
    for (int i = 0; i < std::min<int>(nspinarr, h->wf_norb); i++) h->list_spinarr[i] = spinarr[i];
    h->list_mode = true;
    h->list_from_orbitals = true;
    try {
        const int rc = build_list(h);
        if (rc != CQPI_OK) {
            h->list_mode = false;
            return rc;
        }
    } catch (const CudaError &e) {
        h->list_mode = false;
        return cuda_fail(h, e);
    }
    if (count) *count = h->list_count;
    return CQPI_OK;
}

int cqpi_wannierjosephson(cqpi_handle *h, const double *T, const double *g0r, const double *tip)
{
    if (!h || !tip) return fail(h, CQPI_ERR_ARG, "null argument");
    if (!h->josephson) return fail(h, CQPI_ERR_STATE, "cqpi_set_josephson has not been called");
    return seam_contract(h, T, g0r, tip, false);
}

int cqpi_set_greens(cqpi_handle *h, int32_t mode, double epserr, const cqpi_model *smodel)
{
    if (!h) return CQPI_ERR_ARG;
    if (h->capturing) return fail(h, CQPI_ERR_STATE, "not during a capture");
    if (mode != CQPI_GREEN_NORMAL && mode != CQPI_GREEN_SURFACE && mode != CQPI_GREEN_BULK)
        return fail(h, CQPI_ERR_ARG, "unknown Green's function mode");
    if (mode != CQPI_GREEN_NORMAL) {
        if (!(epserr > 0.0)) return fail(h, CQPI_ERR_ARG, "epserr must be positive");
        if (h->b > 8) return fail(h, CQPI_ERR_NOT_SUPPORTED, "surface / bulk Green's functions: at most 8 bands");
        if (smodel) {
            if (smodel->bands != h->b) return fail(h, CQPI_ERR_ARG, "the surface model must have the model's band count");
            if (smodel->nhops < 0 || (smodel->nhops > 0 && (!smodel->R || !smodel->orb || !smodel->t)))
                return fail(h, CQPI_ERR_ARG, "invalid surface model");
            for (int64_t i = 0; i < smodel->nhops; i++)
                if (smodel->orb[2 * i] < 0 || smodel->orb[2 * i] >= h->b || smodel->orb[2 * i + 1] < 0 ||
                    smodel->orb[2 * i + 1] >= h->b)
                    return fail(h, CQPI_ERR_ARG, "surface model orbital index out of range");
        }
    }
    const int old = h->gmode;
    h->gmode = mode;
    h->epserr = epserr;
    h->surf_own_model = mode != CQPI_GREEN_NORMAL && smodel != nullptr;
    h->surf_R.clear();
    h->surf_orb.clear();
    h->surf_t.clear();
    h->surf_anti.clear();
    if (h->surf_own_model) {
        h->surf_R.assign(smodel->R, smodel->R + 3 * smodel->nhops);
        h->surf_orb.assign(smodel->orb, smodel->orb + 2 * smodel->nhops);
        h->surf_t.assign(smodel->t, smodel->t + 2 * smodel->nhops);
        for (int64_t i = 0; i < smodel->nhops; i++) h->surf_anti.push_back(smodel->anti && smodel->anti[i] ? 1 : 0);
    }
    // the k-space data and the G0(k) buffers depend on the mode
    h->bands_ready = false;
    if ((old == CQPI_GREEN_NORMAL) != (mode == CQPI_GREEN_NORMAL)) {
        free_workspace(h);
        free_adj(h);
    }
    sr_drop(h);
    return CQPI_OK;
}

// Spectral function / unfolded spectral function of all energies into host maps [nE][n][n].
static int spectral(cqpi_handle *h, int kind, const double *energies, int32_t nE, int32_t maxband, const double *pos,
                    const double *pre, float *maps32, double *maps64)
{
    if (!h) return CQPI_ERR_ARG;
    if (nE < 0 || (nE > 0 && !energies)) return fail(h, CQPI_ERR_ARG, "invalid energy list");
    if (maxband < 1 || maxband > h->b) return fail(h, CQPI_ERR_ARG, "maxband outside 1..bands");
    if (kind == 1 && (!pos || !pre)) return fail(h, CQPI_ERR_ARG, "uspf needs orbital positions and prefactors");
    // tmatrix::calcspf computes nothing unless the k-grid is the lattice (src/qpi.cc:670)
    if (kind == 0 && h->kp != h->n) return fail(h, CQPI_ERR_ARG, "output=spf needs kpoints = lattice");
    if (h->capturing) return fail(h, CQPI_ERR_STATE, "not during a capture");
    if (nE == 0) return CQPI_OK;
    const size_t mapn = (size_t)h->n * h->n;
    double *d_pp = nullptr;
    try {
        ensure_energies(h, nE);
        upload_energies(h, energies, nE);
        ensure_stage64(h, (size_t)nE * mapn);
        if (!h->bands_ready) do_bands(h);
        const int mb = kind == 1 ? maxband : 0;
        std::vector<double> pp(3 * (size_t)std::max(mb, 1), 0.0);
        for (int i = 0; i < mb; i++) {
            pp[2 * i] = pos[2 * i];
            pp[2 * i + 1] = pos[2 * i + 1];
            pp[2 * (size_t)mb + i] = pre[i];
        }
        dalloc(&d_pp, pp.size());
        CK(cudaMemcpyAsync(d_pp, pp.data(), sizeof(double) * pp.size(), cudaMemcpyHostToDevice, h->stream));
        if (h->gmode == CQPI_GREEN_NORMAL) {
            launch_spectral(h, kind, nE, 0, h->d_energies_all, maxband, d_pp, d_pp + 2 * mb, h->stage64);
            check_launch();
        } else {
            const int eb = choose_batch(h, nE);
            ensure_workspace(h, eb);
            for (int e0 = 0; e0 < nE; e0 += eb) {
                const int ne = std::min(eb, nE - e0);
                launch_greens_surface(h, ne, h->d_energies_all + e0);
                check_launch();
                launch_spectral(h, kind, ne, e0, h->d_energies_all + e0, maxband, d_pp, d_pp + 2 * mb, h->stage64);
                check_launch();
            }
        }
        std::vector<double> host((size_t)nE * mapn);
        CK(cudaMemcpyAsync(host.data(), h->stage64, sizeof(double) * host.size(), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        dfree(d_pp);
        d_pp = nullptr;
        if (maps64) std::copy(host.begin(), host.end(), maps64);
        if (maps32)
            for (size_t i = 0; i < host.size(); i++) maps32[i] = (float)host[i];
        if (const int st = read_status(h)) return status_code(h, st, "the spectral function");
    } catch (const CudaError &e) {
        if (d_pp) cudaFree(d_pp);
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

int cqpi_spf(cqpi_handle *h, const double *energies, int32_t nE, int32_t maxband, float *maps32, double *maps64)
{
    return spectral(h, 0, energies, nE, maxband, nullptr, nullptr, maps32, maps64);
}

int cqpi_uspf(cqpi_handle *h, const double *energies, int32_t nE, int32_t maxband, const double *pos,
              const double *prearr, float *maps32, double *maps64)
{
    return spectral(h, 1, energies, nE, maxband, pos, prearr, maps32, maps64);
}

int cqpi_dos(cqpi_handle *h, const double *energies, int32_t nE, int32_t maxband, double *dos)
{
    if (!h) return CQPI_ERR_ARG;
    if (nE < 0 || (nE > 0 && (!energies || !dos))) return fail(h, CQPI_ERR_ARG, "invalid energies or output");
    if (maxband < 1 || maxband > h->b) return fail(h, CQPI_ERR_ARG, "maxband outside 1..bands");
    if (h->capturing) return fail(h, CQPI_ERR_STATE, "not during a capture");
    if (nE == 0) return CQPI_OK;
    try {
        const int eb = choose_batch(h, nE);
        ensure_workspace(h, eb);
        ensure_energies(h, nE);
        ensure_stage64(h, (size_t)nE);
        upload_energies(h, energies, nE);
        if (!h->bands_ready) do_bands(h);
        for (int e0 = 0; e0 < nE; e0 += eb) {
            const int ne = std::min(eb, nE - e0);
            if (h->ws.gmax) CK(cudaMemsetAsync(h->ws.gmax, 0, sizeof(unsigned) * ne, h->stream));
            do_greens(h, ne, h->d_energies_all + e0);
            launch_dos(h, ne, maxband, h->stage64 + e0);
            check_launch();
        }
        CK(cudaMemcpyAsync(dos, h->stage64, sizeof(double) * nE, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (const int st = read_status(h)) return status_code(h, st, "the density of states");
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

int cqpi_set_josephson(cqpi_handle *h, int32_t enable, double deltat, double etat)
{
    if (!h) return CQPI_ERR_ARG;
    if (h->capturing) return fail(h, CQPI_ERR_STATE, "not during a capture");
    h->jos_tip = nullptr;
    if (!enable) {
        h->josephson = false;
        return CQPI_OK;
    }
    if (!(deltat == deltat) || !(etat == etat)) return fail(h, CQPI_ERR_ARG, "deltat and etat must be numbers");
    // the reference's Josephson sum runs over the particle block, orbitals 0 .. bands/2 - 1,
    // and reads the hole-block columns o + bands/2 (src/qpi.cc:956,986)
    if (h->b < 2 || (h->b & 1)) return fail(h, CQPI_ERR_ARG, "Josephson mode needs a Bogoliubov-de Gennes model (even band count)");
    if (h->m != (h->b >> 1))
        return fail(h, CQPI_ERR_ARG, "Josephson mode needs maxband = bands/2 (the particle block)");
    h->josephson = true;
    h->jos_deltat = deltat;
    h->jos_etat = etat;
    return CQPI_OK;
}

int cqpi_retrieve_result(cqpi_handle *h, double *ldos)
{
    if (!h || !ldos) return fail(h, CQPI_ERR_ARG, "null argument");
    if (!h->seam_pending) return fail(h, CQPI_ERR_STATE, "cqpi_wannierldos has not been called");
    try {
        CK(cudaMemcpyAsync(ldos, h->d_seam_ldos, sizeof(double) * h->wn * h->wn, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    return CQPI_OK;
}

int cqpi_get_stream(cqpi_handle *h, void **stream)
{
    if (!h || !stream) return CQPI_ERR_ARG;
    *stream = (void *)h->stream;
    return CQPI_OK;
}

int cqpi_synchronize(cqpi_handle *h)
{
    if (!h) return CQPI_ERR_ARG;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, CudaError{e, "cudaStreamSynchronize"});
    if (h->status_pending) {
        h->status_pending = false;
        try {
            if (const int st = read_status(h)) return status_code(h, st, "a run");
        } catch (const CudaError &ce) {
            return cuda_fail(h, ce);
        }
    }
    if (h->sr_sub) return sr_forward(h, cqpi_synchronize(h->sr_sub));
    return CQPI_OK;
}

int cqpi_kernel_launches(const cqpi_handle *h, int64_t *count)
{
    if (!h || !count) return CQPI_ERR_ARG;
    *count = h->launches + (h->sr_sub ? h->sr_sub->launches : 0);
    return CQPI_OK;
}

int cqpi_contraction_kind(const cqpi_handle *h, int32_t *kind)
{
    if (!h || !kind) return CQPI_ERR_ARG;
    const cqpi_handle *k = (sr_active(h) && h->sr_sub) ? h->sr_sub : h;
    *kind = (k->precision == CQPI_PREC_FP64) ? 0 : (tc_active(k) ? 2 : 1);
    return CQPI_OK;
}

int cqpi_stage_times(cqpi_handle *h, float *ms5)
{
    if (!h || !ms5) return CQPI_ERR_ARG;
    try {
        collect_times(h);
    } catch (const CudaError &e) {
        return cuda_fail(h, e);
    }
    for (int i = 0; i < 5; i++) ms5[i] = h->stage_ms[i];
    if (h->sr_sub) {
        float sub[5];
        const int rc = cqpi_stage_times(h->sr_sub, sub);
        if (rc != CQPI_OK) return sr_forward(h, rc);
        for (int i = 0; i < 5; i++) ms5[i] += sub[i];
    }
    return CQPI_OK;
}

}  // extern "C"
