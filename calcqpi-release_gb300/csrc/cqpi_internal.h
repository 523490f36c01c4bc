// cqpi_internal.h -- shared declarations of the GB300 continuum-LDOS engine.
//
// Data layout in HBM (one handle):
//   bands     eval [b][nk] f64, evec [b*b][nk] f64x2 (o*b+n), nk = kp*kp, k = i*kp + j
//   greens    g0k  [E][b*b][nk] complex (SoA planes, plane = o*b+a)
//             half [E][b*b][kp][NB] complex: transform along j done, pruned to Y in box
//             box  [E][NB][NB][b*b] complex: G0(R) for R in [-Rb, Rb]^2 (box index R+Rb)
//   T         [E][nimp][b*b] f64x2
//   term1     [E][os*os] f64 (site-independent part of the LDOS)
//   phi       [nblk][os*os][W][mb] f64: phi_o(q,d) = wf[o](w*os+qx-dx*os, w*os+qy-dy*os)
//   maps      [E][nimp][wn][wn] f32 and/or f64, x fastest
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/cqpi.h"

#define CQPI_MAX_BANDS 16

namespace cqpi {

// Unique in-plane lattice vectors with their summed hopping matrices: H(k) adds
// tn[R] e^{+i theta} + ta[R] e^{-i theta}, theta = 2 pi k.R (anti terms conjugated).
struct RTerms {
    std::vector<int32_t> R;     // [nR][2]
    std::vector<double> tn, ta; // [nR][b*b][2]
};

// Launch plan of the tcgen05 contraction (ldos_tc.cu).
struct TcPlan {
    bool ok = false;
    int TS = 0;          // sites per tile (multiple of 4)
    int N = 0;           // MMA N = 2*bands*TS (multiple of 16, <= 256)
    int KP = 0;          // K padded to a multiple of 16
    int tmem_cols = 0;   // power of two >= 2*nblk*N
    int a_bytes = 0, b_bytes = 0;
    int sst = 0;         // staging row stride (floats)
    size_t smem = 0;
    bool pipe = false;   // pipelined variant usable (one spin block)
    int pipe_tmem_cols = 0;
    size_t pipe_smem = 0;
    // direct-window variant (one spin block): the staged fp16 G0 windows are the B operand
    bool win = false;
    int wH = 0;          // 8-site groups per tile (sites per tile = 8*wH)
    int wEB = 0;         // energies per tile
    int wNRAW = 0;       // raw-window ring depth (fetches run wNRAW-1 tiles ahead)
    int wNX = 0;         // window width in sites (8*wH + 2*window)
    int w_nbulk = 0;     // raw columns per tile fetched by bulk copies, the rest by cp.async
    int wNKC = 0;        // 8-element K chunks per window row (even)
    int wKP = 0;         // A columns: (2*window+1) * wNKC * 8
    int w_a_bytes = 0, w_win_bytes = 0, w_sst = 0, w_tmem_cols = 0;
    bool w_a_tmem = false;   // Phi fits in the tensor-memory columns left by the accumulators
    size_t w_smem = 0;
};

struct TcParams {
    int b, n, os, w, Rb, NB, W, nblk, mb, bs0, bs1;
    int TS, N, KP, Q, nimp, ne, wn, ntx, sst;
    int tmem_cols, a_bytes, b_bytes;
    int H, NX, NKC, win_bytes, EB, nraw;   // direct-window variant
    int nbulk;                   // direct-window variant: raw columns fetched by bulk copies (the rest by cp.async)
    int a_tmem;                  // direct-window variant: Phi operand held in tensor memory
    int stall;                   // fault injection: wait on a barrier nothing arrives on
    int coff;                    // Josephson mode: column offset of the s operand (bands/2), else 0
    const double2 *tip;          // Josephson mode: tip factor per energy of the batch, else NULL
    float inv_sA;
    float scale;                 // factor of every map value
    long long spin_limit;
    const float2 *box;
    const float2 *T32;
    const double *term1;
    const unsigned *gmax;
    const float2 *boxT;          // direct-window variant, one impurity: (T G0)(R) per energy for the s
    const unsigned *gmaxT;       // operand (T folded out of the epilogue) and its max |Re|,|Im|; else NULL
    const float2 *zsrc;          // direct-window variant: 16-byte aligned zeros, at least one raw column
    const uint4 *Aimg;
    float *out;
    const int *fov;              // direct-window variant: per-map field of view (sites per side) or NULL
    const long long *fov_off;    // and the float offset of every map in out
    int *status;
};

// Buffers of the adjoint (adjoint.cu), kept by the handle between calls.
struct AdjWorkspace {
    int ebatch = 0;
    double2 *gbox = nullptr;   // [E][NB][NB][b*b]  dL/dG0(R) (box)
    double2 *M = nullptr;      // [E][nimp][b*b]    sum W u s^T
    double *wsum = nullptr;    // [E][Q]            sum_p W
    double2 *gV = nullptr;     // [nimp][b*b]       dL/dV
    double2 *A = nullptr;      // [b*b][NB][kp]     column pass of the box -> k transform
    double2 *gk = nullptr;     // [E][b*b][nk]      dL/dG0(k) per energy of a batch (in the handle's
                               // precision), then [b*b][nk] dL/dH(k) (FP64)
    double2 *C = nullptr;      // [b*b][nk]         eigenbasis accumulator over energies
    double2 *gR = nullptr;     // [nR][2][b*b]      dL/dtn, dL/dta per unique R
    void *win = nullptr;       // [2][E][nimp][W*mb][b][n*n] window gradients of every site (u, s;
                               // float2 for the mixed handle, double2 for the FP64 handle)
    double2 *Mp = nullptr;     // [E][nimp][n*n][b*b] per-site parts of M
    double *kt = nullptr;      // [(4w+1)^2][mb*mb][Q] the term1 kernel of the orbitals
};

// Hopping terms of the surface / bulk Green's function on the device: three sets (surface
// in-plane, bulk in-plane, bulk R_z < 0) packed one after the other, and the k-dependent
// matrices eps_s, eps_b, alpha [3][kp*kp][b*b] built from them.
struct SurfaceTerms {
    int ns = 0, nb = 0, no = 0, off_s = 0, off_b = 0, off_o = 0;
    int4 *d_i = nullptr;        // (rx, ry, o1, o2)
    double2 *d_t = nullptr;     // amplitudes
    int *d_anti = nullptr;
    size_t cap_i = 0, cap_t = 0, cap_anti = 0;
    double2 *d_mats = nullptr;
};

struct Workspace {
    int ebatch = 0;
    double2 *g0k = nullptr;
    double2 *half = nullptr;
    double2 *box = nullptr;
    double2 *T = nullptr;
    double *term1 = nullptr;
    double *energies = nullptr;
    float2 *g0k32 = nullptr;
    float2 *half32 = nullptr;
    float2 *box32 = nullptr;
    float2 *T32 = nullptr;
    unsigned *gmax = nullptr;   // per energy: bits of max |Re|,|Im| of the FP32 box
    float2 *boxT32 = nullptr;   // per energy: T G0(R) on the box (one impurity, tensor-core path)
    unsigned *gmaxT = nullptr;  // per energy: bits of max |Re|,|Im| of boxT32
};

}  // namespace cqpi

struct cqpi_handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    // model
    int b = 0, scmax = 0;
    double efermi = 0.0;
    int nR = 0;
    int32_t *d_R = nullptr;
    double *d_tn = nullptr, *d_ta = nullptr;
    // {R, -R} pairs of the H(k) build: R [np][2], then P and Q [np][2][b*b] (see upload_pairs)
    int npair_R = 0;
    int32_t *d_pR = nullptr;
    double2 *d_pPQ = nullptr;
    size_t cap_pR = 0, cap_pPQ = 0;
    // parameters
    int n = 0, kp = 0, os = 0, w = 0, m = 0, spin = 0, precision = 0;
    double eta = 0.0;
    int Rb = 0, NB = 0, W = 0, Q = 0, wn = 0, nblk = 1, mb = 0;
    int blk_start[2] = {0, 0};
    // eigen cache
    double *d_eval = nullptr;
    double2 *d_evec = nullptr;
    float2 *d_evec32 = nullptr;   // FP32 copy for the mixed path
    float2 *d_eval32 = nullptr;   // eigenvalues as float pairs (hi, lo) for the mixed path
    bool time_reversal = false;   // every hopping is real: H(-k) = conj(H(k))
    bool bands_ready = false;
    // twiddles e^{+2 pi i t / kp}
    double2 *d_tw = nullptr;
    float2 *d_tw32 = nullptr;
    // orbitals
    double *d_phi = nullptr;
    float *d_phi32 = nullptr;
    bool orbitals_ready = false;
    // fused FP32 G0(k) + pruned FFT (mixed path, power-of-two k-grid)
    bool use_fft32 = false;
    // tcgen05 contraction
    bool use_tc = false;
    cqpi::TcPlan tc;
    uint16_t *d_tc_a = nullptr;   // Phi hi/lo operand images
    uint16_t *d_tc_aw = nullptr;  // Phi hi/lo images in the direct-window K order
    float tc_inv_sA = 1.0f;
    size_t cap_phi = 0, cap_phi32 = 0, cap_tc_a = 0, cap_tc_aw = 0;   // element capacities of the four images
    int num_sms = 0;
    // impurities
    int nimp = 0;
    double2 *d_V = nullptr;   // [nimp][b*b]
    // workspace
    cqpi::Workspace ws;
    cqpi::AdjWorkspace adj;
    int *d_status = nullptr;
    // per-map fields of view (cqpi_run_fov): device copies and page-locked staging
    int *d_fov = nullptr;
    long long *d_fov_off = nullptr;
    int *h_fov_pinned = nullptr;
    long long *h_off_pinned = nullptr;
    size_t fov_cap = 0;
    // CUDA graph capture of the handle's stream (cqpi_graph_begin / end / launch)
    bool capturing = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int64_t graph_kernels = 0;   // kernels of one replay
    int64_t graph_kernels_sub = 0;
    // model hopping terms as given to cqpi_create (for cqpi_set_hoppings / cqpi_adjoint):
    // unique-R index, orbital pair and conjugation flag of every term
    std::vector<int> hop_r, hop_o1, hop_o2, hop_anti;
    std::vector<double> rt_tn, rt_ta;   // host copies of the summed matrices [nR][b*b][2]
    std::vector<int32_t> rt_R;          // [nR][2]
    // spin-degenerate reduction: with spin blocks [0, mb) and [mb, 2mb) that do not couple
    // (hoppings and V) and are identical (hoppings, diagonal, orbitals, V), G0 and T are
    // block diagonal with equal blocks and every map is exactly twice the map of the mb-band
    // problem, which an internal handle (sharing this stream) computes
    bool sr_model = false, sr_orb = false, sr_v = false, sr_stale = true;
    cqpi_handle *sr_sub = nullptr;
    std::vector<double> sr_wf, sr_V;
    std::vector<uint8_t> sr_zero;
    int sr_side = 0, sr_nimp = 0;
    bool owns_stream = true;
    float out_scale = 1.0f;             // factor applied to every map value
    // Josephson mode (tmatrix::calcwannierjosephson): tip gap and broadening, per-energy tip
    // factors on the device and their page-locked mirror, and the tip factors of the energy
    // batch being launched (read by the term1 and contraction launchers; NULL otherwise)
    bool josephson = false;
    double jos_deltat = 0.001, jos_etat = 0.0;
    double2 *d_tip_all = nullptr, *h_tip_pinned = nullptr;
    const double2 *jos_tip = nullptr;
    double2 *d_seam_tip = nullptr;
    // surface / bulk Green's function: mode, tolerance, the surface model's in-plane terms
    // (host; empty = the model itself) and the device terms and matrices
    int gmode = 0;
    double epserr = 1e-5;
    bool surf_own_model = false;
    std::vector<int32_t> surf_R, surf_orb;
    std::vector<double> surf_t;
    std::vector<uint8_t> surf_anti;
    std::vector<int32_t> hop_rx, hop_ry, hop_rz;   // R of every model term
    std::vector<double> hop_t;                     // current amplitudes of the model terms
    cqpi::SurfaceTerms surf;
    // proximity-list form of the wannier mode (threshold keyword, mkthresholdlist +
    // tmatrix::calcwannierldos(os, w, flaglist)): host copy of the orbitals the list is built
    // from, the list's parameters, and the list on the device, CSR by (d1, q): entry s holds
    // u = d2 * npair + pair index and the factor f; pairs are the (o1, o2) the list uses
    std::vector<double> wf_host;
    int wf_norb = 0;
    bool list_mode = false;
    double list_threshold = 0.0;
    std::vector<int32_t> list_spinarr;
    bool list_use_spinarr = false;
    bool list_from_orbitals = true;     // built by cqpi_set_threshold (rebuilt with the orbitals)
    int list_npair = 0;
    int64_t list_count = 0;
    int *d_list_off = nullptr, *d_list_u = nullptr;
    double *d_list_f = nullptr;
    float *d_list_f32 = nullptr;
    int2 *d_list_pair = nullptr;
    // narrow seam (always FP64)
    double *d_seam_ldos = nullptr;
    double2 *d_seam_box = nullptr, *d_seam_T = nullptr;
    double *d_seam_term1 = nullptr;
    bool seam_pending = false;
    // accounting
    int64_t launches = 0;
    float stage_ms[5] = {0, 0, 0, 0, 0};
    cudaEvent_t ev[8] = {};
    // asynchronous runs: pooled timing events, pending (stage, start, end) triples,
    // all-energies buffer with a page-locked host mirror, host-output staging
    std::vector<cudaEvent_t> ev_pool, ev_free;
    std::vector<int> ev_pending;               // triples: stage, start index, end index into ev_pool
    double *d_energies_all = nullptr, *h_energies_pinned = nullptr;
    int energies_cap = 0;
    float *stage32 = nullptr;
    double *stage64 = nullptr;
    // host outputs: copy stream and per-slot events (computation done / copy done)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_comp[2] = {}, ev_copy[2] = {};
    size_t stage_cap32 = 0, stage_cap64 = 0;
    bool status_pending = false;
    std::string err;
};

namespace cqpi {

// bands.cu
void launch_bands(cqpi_handle *h);
// greens.cu
void launch_greens_k(cqpi_handle *h, int ne, const double *d_energies);
void launch_fft(cqpi_handle *h, int ne);
cudaError_t configure_fft(cqpi_handle *h);
void launch_tmatrix(cqpi_handle *h, int ne);
void launch_term1(cqpi_handle *h, int ne);
void launch_term1_ptr(cqpi_handle *h, int ne, const double2 *box, double *term1);
// ldos.cu
void launch_ldos_fp64(cqpi_handle *h, int ne, const double2 *box, const double2 *T, const double *term1,
                      float *out32, double *out64);
void launch_ldos_fp32(cqpi_handle *h, int ne, const float2 *box, const float2 *T, const double *term1,
                      float *out32, double *out64);
// fft32.cu
bool fft32_supported(const cqpi_handle *h);
cudaError_t configure_fft32(cqpi_handle *h);
void launch_greens_fft32(cqpi_handle *h, int ne, const double *d_energies);
bool launch_fft32_planes(cqpi_handle *h, int ne);
bool g0k_reciprocity(const cqpi_handle *h);   // G0(k) planes of the unfused path: upper triangle only
// adjoint_mma.cu: the mixed handle's contraction adjoint on the tensor cores (false: not applicable)
bool launch_adj_contract_mma(cqpi_handle *h, int ne, const float *phi, const float2 *box, const float *wmap,
                             float2 *Ub, float2 *Sb, float2 *Mp);
// ldos_tc.cu
bool tc_supported(const cqpi_handle *h);
void tc_plan(cqpi_handle *h);
void tc_build_a(cqpi_handle *h, const std::vector<double> &phi, std::vector<uint16_t> &img, float &inv_sA);
void tc_build_a_window(cqpi_handle *h, const std::vector<double> &phi, std::vector<uint16_t> &img);
// adjoint.cu
void launch_adj_energy_batch(cqpi_handle *h, int ne, const float *wmap, AdjWorkspace &aw);
void launch_adj_kspace(cqpi_handle *h, int e, AdjWorkspace &aw);
void launch_adj_kacc(cqpi_handle *h, int ne, const double *omegas, AdjWorkspace &aw);
void launch_adj_hoppings(cqpi_handle *h, AdjWorkspace &aw);
// surface.cu
void launch_surface_mats(cqpi_handle *h);
void launch_greens_surface(cqpi_handle *h, int ne, const double *d_energies);
// spectral.cu
void launch_spectral(cqpi_handle *h, int kind, int ne, int e_base, const double *d_energies, int maxband,
                     const double *d_pos, const double *d_pre, double *out);
void launch_dos(cqpi_handle *h, int ne, int maxband, double *dos);
// ldos_list.cu
size_t list_smem_bytes(const cqpi_handle *h, bool fp64);
cudaError_t configure_list(cqpi_handle *h);
void launch_term1_list(cqpi_handle *h, int ne, const void *box, double *term1);
void launch_ldos_list(cqpi_handle *h, int ne, const void *box, const void *T, const double *term1, float *o32,
                      double *o64);
cudaError_t launch_ldos_tc(cqpi_handle *h, int ne, float *out, const int *fov = nullptr,
                           const long long *fov_off = nullptr);
bool tc_window_usable(const cqpi_handle *h);   // the direct-window kernel runs (per-map FOV support)
// The FP32 box buffers (box32, boxT32) carry a tail after their ebatch boxes: slack for the
// contraction's 16-byte-aligned bulk copies, which may read 16 bytes past a window column,
// and (box32) zeros from the first 16-byte boundary after the boxes, NB*b*b + 8 complex
// values long, the source of the raw columns outside the box (at least one column).
inline size_t box32_boxes(const cqpi_handle *h, int ebatch) { return (size_t)ebatch * h->NB * h->NB * h->b * h->b; }
inline size_t box32_count(const cqpi_handle *h, int ebatch) { return box32_boxes(h, ebatch) + 2 + (size_t)h->NB * h->b * h->b + 8; }
inline const float2 *box32_zeros(const cqpi_handle *h) { return h->ws.box32 + ((box32_boxes(h, h->ws.ebatch) + 1) & ~(size_t)1); }
bool window_config(const cqpi_handle *h, int EB, int H, int nraw, TcPlan &pl);
cudaError_t tc_autotune(cqpi_handle *h, int ne, float *out, float *best_ms, int *tried);
void launch_widen(cqpi_handle *h, const float *src, double *dst, size_t n);

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace cqpi
