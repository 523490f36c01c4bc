/*
 * cqpi.h -- C ABI of the GB300 continuum-LDOS engine (libcqpi.so).
 *
 * The engine computes CalcQPI's "Wannier mode" quasiparticle-interference maps
 * (output=wannier, green=normal) on one NVIDIA GB300 (sm_103a):
 *   H(k) -> Hermitian eigen-solve -> G0(k,w) -> G0(R,w) -> T-matrix -> LDOS map.
 * Reference path: gpwahl/calcqpi-release, src/qpi.cc:454-950 driven by
 * src/calcqpi.cc:655-783.
 *
 * Conventions (identical to the reference's):
 *  - hoppings: R[h][3] int32 (lattice units), orb[h][2] int32 0-based (o1,o2),
 *    t[h][2] double (re,im) already divided by the _hr.dat degeneracy, anti[h]
 *    (conjugated phase, BdG hole block; src/tightbinding.h:128-135).
 *  - H(k)_{o1 o2} = -efermi*d (o<scmaxbands) / +efermi*d (otherwise)
 *                   + sum_h t_h exp(+-2 pi i k.R_h)     (src/tightbinding.cc:210-219)
 *  - k-grid x_i = i/kp (i <= kp/2) else (i-kp)/kp       (src/qpi.cc:465-466)
 *  - G0(k) = sum_n U_n U_n^H / (w - e_n + i eta)        (src/tightbinding.cc:282-289)
 *  - G0(R) = kp^-2 sum_k G0(k) exp(+2 pi i k.R)         (src/qpi.cc:557-578)
 *  - T = (1 - V G0(R=0))^-1 V                           (src/qpi.cc:833-854)
 *  - orbitals wf[o][ix][iy], side (2*window+1)*oversamp (src/wannierfunctions.cc:433-442)
 *  - maps are float32 (or float64) [layer][y][x], x = site_i*oversamp + sub_x,
 *    the IDL file order of src/idl.cc:78-97.
 * Complex numbers are interleaved (re, im) doubles.  All entry points return a
 * status code (CQPI_OK == 0); none exits or aborts.  Calls on one handle are not
 * thread-safe; distinct handles may be used from distinct threads.
 */
#ifndef CQPI_H
#define CQPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CQPI_OK 0
#define CQPI_ERR_ARG 1          /* invalid argument / size */
#define CQPI_ERR_CUDA 2         /* CUDA runtime error (message in cqpi_last_error) */
#define CQPI_ERR_ALLOC 3        /* device or host allocation failed */
#define CQPI_ERR_DOMAIN 4       /* sizes outside the reference's index domain */
#define CQPI_ERR_SINGULAR 5     /* 1 - V G0(0) singular at some energy */
#define CQPI_ERR_STATE 6        /* call order violated (e.g. no orbitals set) */
#define CQPI_ERR_NOT_SUPPORTED 7
#define CQPI_ERR_NO_DEVICE 8    /* no CUDA device visible */
#define CQPI_ERR_TIMEOUT 9      /* a bounded device wait ran out; the kernel stopped early */
#define CQPI_ERR_NOT_CONVERGED 10 /* the surface / bulk decimation did not reach epserr */

#define CQPI_PREC_FP64 0        /* every stage in FP64 */
#define CQPI_PREC_MIXED 1       /* FP64: eigen-solve, T-matrix, term1; FP32: G0(k) and both
                                   passes of the k-sum transform (pole distances from float
                                   pairs); tensor-core contraction (split-FP16 x3, FP32
                                   accumulation).  Maps within 1e-6 of the FP64 path. */

/* Green's function of cqpi_set_greens (the green keyword, src/calcqpi.cc:129,206-209) */
#define CQPI_GREEN_NORMAL 0     /* G0(k) from the eigen cache */
#define CQPI_GREEN_SURFACE 1    /* surface Green's function of a layered model */
#define CQPI_GREEN_BULK 2       /* bulk Green's function of a layered model */

typedef struct cqpi_handle cqpi_handle;

typedef struct {
    int32_t bands;        /* b = num_wann */
    int32_t scmaxbands;   /* diagonal sign switch (b, or b/2 for scmodel) */
    double efermi;        /* 'fermi' keyword */
    int64_t nhops;
    const int32_t *R;     /* [nhops][3] */
    const int32_t *orb;   /* [nhops][2], 0-based */
    const double *t;      /* [nhops][2] */
    const uint8_t *anti;  /* [nhops], may be NULL (all 0) */
} cqpi_model;

typedef struct {
    int32_t lattice;      /* n: sites per side ('lattice') */
    int32_t kpoints;      /* kp ('kpoints', defaults to lattice in the CLI) */
    int32_t oversamp;     /* os ('oversamp') */
    int32_t window;       /* w ('window') */
    int32_t maxband;      /* m: orbitals carrying a Wannier function (b, or b/2 for scmodel) */
    int32_t spin;         /* 'spin': pair orbitals only inside spin half-blocks */
    double eta;           /* 'eta' */
    int32_t precision;    /* CQPI_PREC_FP64 or CQPI_PREC_MIXED */
} cqpi_params;

/* ---- lifetime ------------------------------------------------------------
 * Replaces tmatrix::tmatrix (src/qpi.h:96-106) + CudaQPI::CudaQPI
 * (src/qpicudakernel.cu:395-429): validates sizes, uploads the model, creates
 * the handle's CUDA stream and owns all device memory. */
int cqpi_create(const cqpi_model *model, const cqpi_params *params, cqpi_handle **out);
/* Replaces tmatrix::~tmatrix / CudaQPI::~CudaQPI.  NULL is accepted. */
int cqpi_destroy(cqpi_handle *h);
/* Human-readable message of the last failing call on this handle. */
const char *cqpi_last_error(const cqpi_handle *h);
const char *cqpi_status_string(int status);
const char *cqpi_version(void);

/* ---- inputs ----------------------------------------------------------------
 * Orbital cache, replaces the wf upload of CudaQPI::CudaQPI
 * (src/qpicudakernel.cu:412-416) and the iszero() skips of src/qpi.cc:915-940.
 * wf: [norb][side][side] doubles, norb >= maxband, side == (2w+1)*oversamp;
 * is_zero: [norb] flags (NULL = none) for padded 'z' orbitals. */
int cqpi_set_orbitals(cqpi_handle *h, const double *wf, int32_t norb, int32_t side, const uint8_t *is_zero);
/* Diagonal scattering potential, replaces tmatrix::setscatteringphase
 * (src/qpi.h:107-130): vscat [bands][2].  Sets one impurity. */
int cqpi_set_scattering(cqpi_handle *h, const double *vscat);
/* Extension (C4 workloads): nimp full b x b potentials V[imp][b][b][2]; each
 * impurity gives its own map.  Diagonal V reproduces cqpi_set_scattering. */
int cqpi_set_impurities(cqpi_handle *h, const double *V, int32_t nimp);

/* ---- compute ---------------------------------------------------------------
 * H(k) build + FP64 Hermitian eigen-solve of every k-point, cached on the device.
 * Replaces tmatrix::calchamiltonian (src/qpi.cc:454-475).  Asynchronous on the
 * handle's stream; cqpi_run calls it lazily when the cache is empty, as
 * tmatrix::setgreensfunction does (src/qpi.cc:479-480). */
int cqpi_solve_bands(cqpi_handle *h);
/* All energies -> maps.  Replaces, per energy, setgreensfunction +
 * calcrealspacegreensfunction + calcwannierldos + ldos2idl
 * (src/calcqpi.cc:690-756).  maps32 / maps64: [nE][nimp][wn][wn] (either may be
 * NULL), wn = lattice*oversamp.  on_device != 0: the pointers are device memory
 * and the call returns after enqueueing (cqpi_synchronize waits and reports a
 * singular T-matrix); otherwise they are host memory and the call returns when they
 * are filled. */
int cqpi_run(cqpi_handle *h, const double *energies, int32_t nE, float *maps32, double *maps64, int32_t on_device);

/* Batched maps with a field of view per map (extension: the reference has one field of
 * view per run).  fov[nE][nimp]: sites per side of map (energy, impurity), 1..lattice,
 * centred like the full field (a crop of cqpi_run's map); maps: device memory, maps
 * packed in (energy, impurity) order, map k (fov f) is (f*oversamp)^2 floats, rows of
 * f*oversamp, starting after the maps before it.  Asynchronous (on_device must be 1);
 * needs the mixed-precision tensor-core contraction, else CQPI_ERR_NOT_SUPPORTED. */
int cqpi_run_fov(cqpi_handle *h, const double *energies, int32_t nE, const int32_t *fov, float *maps, int32_t on_device);
/* Tile-shape autotuner of the tensor-core contraction (extension): runs the Green's function
 * stages for the first batch of the given energies, times every valid tile shape (energies per
 * tile, sites per tile, raw-window ring depth) of the direct-window kernel on it and keeps the
 * fastest for this handle.  best_ms / tried (may be NULL): time of one batch with the chosen
 * shape, number of shapes timed. */
int cqpi_autotune(cqpi_handle *h, const double *energies, int32_t nE, float *best_ms, int32_t *tried);
/* CUDA graph of the handle's stream: begin / end capture around on-device calls
 * (cqpi_run / cqpi_run_fov with on_device = 1, after one identical un-captured call so
 * that every buffer exists), then launch the captured batch as one graph. */
int cqpi_graph_begin(cqpi_handle *h);
int cqpi_graph_end(cqpi_handle *h);
int cqpi_graph_launch(cqpi_handle *h);

/* ---- k-space outputs (output=spf|uspf, dosfile) ------------------------------------
 * Host maps [nE][lattice][lattice] in IDL order (either pointer may be NULL); synchronous.
 * cqpi_spf: tmatrix::calcspf(maxband) (src/qpi.cc:659-683), -sum_{l<maxband} Im G0(k)_ll on
 * the k-grid shifted by kp/2; needs kpoints = lattice (the driver sets it for output=spf,
 * src/calcqpi.cc:333-334), else CQPI_ERR_ARG.
 * cqpi_uspf: tmatrix::calcuspf (src/qpi.cc:735-775), unfolded with the orbital positions
 * pos[maxband][2] (lattice units) and prefactors prearr[maxband]; spin handles sum the two
 * blocks of maxband/2 orbitals.
 * cqpi_dos: tmatrix::calcdos after the real-space transform (src/qpi.cc:856-862, the dosfile
 * loop src/calcqpi.cc:336-391): dos[e] = -sum_{i<maxband} Im G0(R=0)_ii.
 * All three follow the handle's Green's function (normal, surface, bulk). */
int cqpi_spf(cqpi_handle *h, const double *energies, int32_t nE, int32_t maxband, float *maps32, double *maps64);
int cqpi_uspf(cqpi_handle *h, const double *energies, int32_t nE, int32_t maxband, const double *pos,
              const double *prearr, float *maps32, double *maps64);
int cqpi_dos(cqpi_handle *h, const double *energies, int32_t nE, int32_t maxband, double *dos);

/* ---- surface / bulk Green's function (green=surface|bulk, stbfile, epserr;
 * tmatrix::calcsurfacegreensfunction, src/qpi.cc:488-554) -----------------------------
 * mode CQPI_GREEN_SURFACE / CQPI_GREEN_BULK replaces G0(k) by the decimation over the
 * layers of the model: the terms with R_z = 0 are the in-plane Hamiltonian, those with
 * R_z < 0 the coupling to the next layer (principal-layer form); surface_model (NULL = the
 * model itself; same band count) supplies the in-plane terms of the surface layer; the
 * iteration stops when the Frobenius norms of both couplings are <= epserr (at most 200
 * doublings; else the run returns CQPI_ERR_NOT_CONVERGED).  CQPI_GREEN_NORMAL returns to
 * the eigen-based G0.  Up to 8 bands; cqpi_adjoint and cqpi_get_bands return
 * CQPI_ERR_NOT_SUPPORTED in these modes. */
int cqpi_set_greens(cqpi_handle *h, int32_t mode, double epserr, const cqpi_model *surface_model);

/* ---- Josephson mode (output=josephson, src/calcqpi.cc:225,451-460,705-709) -----------
 * enable != 0 switches cqpi_run to the Josephson contraction of
 * tmatrix::calcwannierjosephson (src/qpi.cc:953-1033): the sum runs over the particle-block
 * orbitals 0 .. bands/2 - 1, reads the hole-block column o + bands/2 of G0 and T G0, and
 * every map is -Im(tip(E) * ...) with the driver's per-energy tip factor
 *   tip(E) = (0, -sign(E) pi deltat) / sqrt((E + i etat)^2 - deltat^2).
 * Needs an even band count and maxband = bands/2 (CQPI_ERR_ARG otherwise); the driver's
 * defaults are deltat = 0.001 and etat = eta.  In this mode the mixed path contracts on the
 * tensor cores (direct-window kernel, one spin block) or else on FP32 CUDA cores;
 * cqpi_adjoint returns CQPI_ERR_NOT_SUPPORTED.  enable = 0 returns to the LDOS (wannier)
 * mode. */
int cqpi_set_josephson(cqpi_handle *h, int32_t enable, double deltat, double etat);

/* ---- proximity list (threshold keyword, src/calcqpi.cc:238,619-635,700-701) -----------
 * threshold = NaN: the full window sum (default).  Otherwise builds the reference's list
 * (mkthresholdlist, src/qpi.cc:139-253) from the orbitals of the last cqpi_set_orbitals call
 * (and rebuilds it on every later one): the (sub-pixel, d1, d2, o1, o2) terms whose factor
 * |phi_o1 phi_o2| exceeds threshold * max phi^2 -- orbitals 0 .. maxband-1 (spin: both
 * blocks of maxband/2), or, with spinarr (nspinarr labels, padded with 0 to the orbital
 * count), the orbital pairs of equal non-zero label -- and cqpi_run then sums only those
 * (tmatrix::calcwannierldos(os, w, flaglist)).  *count (may be NULL) receives the entry
 * count.  oversamp^2 <= 512.  The Josephson mode ignores the list (as the reference's
 * driver); cqpi_run_fov, cqpi_autotune and cqpi_adjoint return CQPI_ERR_NOT_SUPPORTED while
 * it is set. */
int cqpi_set_threshold(cqpi_handle *h, double threshold, const int32_t *spinarr, int32_t nspinarr, int64_t *count);
/* An explicit proximity list, as the reference's list-mode GPU backend receives it
 * (CudaQPI(..., flaglist&), src/qpicudakernel.cu:431-487): nent entries ent[k][5] =
 * (list, i, j, o1, o2) with list = ((xn1*wins + yn1)*wins + xn2)*wins + yn2, wins = 2w+1
 * (flags[xn1][yn1][xn2][yn2]), sub-pixel (i, j) and orbitals o1, o2 < bands, and factor[k].
 * Replaces any list; kept when the orbitals change.  cqpi_set_threshold(NaN) clears it. */
int cqpi_set_list(cqpi_handle *h, int64_t nent, const int32_t *ent, const double *factor);

/* ---- differentiation (extension: the reference computes no derivatives) -----
 * New hopping amplitudes for the terms of the model given to cqpi_create (same order,
 * same R / orbitals / conjugation flags): t[nhops][2].  The eigen cache is rebuilt by
 * the next run or adjoint call. */
int cqpi_set_hoppings(cqpi_handle *h, const double *t);
/* Reverse-mode derivative of cqpi_run: given dL_dmaps = dL/drho in the maps32 layout
 * [nE][nimp][wn][wn] (device memory if on_device != 0, else host), writes
 *   dL_dt[nhops][2] = (dL/dRe t, dL/dIm t) for every hopping term of the model, and
 *   dL_dV[nimp][b][b][2] = (dL/dRe V, dL/dIm V) for every impurity matrix entry.
 * G0(k), G0(R) and T are recomputed per energy from the eigen cache; the call returns
 * when the gradients are filled.  One spin block, kpoints a power of two, oversamp^2
 * <= 128; otherwise CQPI_ERR_NOT_SUPPORTED.  Either output may be NULL. */
int cqpi_adjoint(cqpi_handle *h, const double *energies, int32_t nE, const float *dL_dmaps, int32_t on_device,
                 double *dL_dt, double *dL_dV);

/* ---- narrow seam (GPUQPI, include/gpuqpi.h:18-32) ------------------------
 * GPUQPI::wannierldos(scat, g0): host T-matrix T[b][b][2] and host real-space
 * Green's function g0r[kp][kp][b][b][2] (the reference's g0 after
 * calcrealspacegreensfunction); asynchronous like src/qpicudakernel.cu:577-598. */
int cqpi_wannierldos(cqpi_handle *h, const double *T, const double *g0r);
/* GPUQPI::wannierjosephson(scat, g0, tip) (include/gpuqpi.h:24, src/qpicudakernel.cu:600-620):
 * the Josephson form of the same contraction
 * (tmatrix::calcwannierjosephson, src/qpi.cc:953-1033) with the tip factor tip[2] of the
 * energy; needs cqpi_set_josephson(h, 1, ...) first (CQPI_ERR_STATE otherwise), as
 * cqpi_wannierldos needs it off. */
int cqpi_wannierjosephson(cqpi_handle *h, const double *T, const double *g0r, const double *tip);
/* GPUQPI::wannierldoslist(scat, g0) (include/gpuqpi.h:25, src/qpicudakernel.cu:624-636): the
 * proximity-list form (tmatrix::calcwannierldos(os, w, flaglist), src/qpi.cc:1085-1134) with
 * the list of cqpi_set_threshold; CQPI_ERR_STATE without one. */
int cqpi_wannierldoslist(cqpi_handle *h, const double *T, const double *g0r);
/* GPUQPI::retrieveResult(double*) (src/qpicudakernel.cu:690-704): waits and
 * copies the last map, ldos[y][x] float64 (= the reference's ldos[x][y]). */
int cqpi_retrieve_result(cqpi_handle *h, double *ldos);

/* ---- stage access (parity tests, debugging) ----------------------------- */
/* Eigen cache: eval[kp*kp][b], evec[kp*kp][b][b][2] (component o of vector n at [o][n]). */
int cqpi_get_bands(cqpi_handle *h, double *eval, double *evec);
/* G0(R) on the pruned box R in [-Rb, Rb]^2 at one energy: box[(X+Rb)][(Y+Rb)][b][b][2];
 * *rb receives Rb (pass box = NULL to query it). */
int cqpi_get_greens_box(cqpi_handle *h, double energy, double *box, int32_t *rb);
/* T-matrix of impurity 0 at one energy: T[b][b][2]. */
int cqpi_get_tmatrix(cqpi_handle *h, double energy, double *T);

/* ---- runtime -------------------------------------------------------------- */
int cqpi_get_stream(cqpi_handle *h, void **stream);   /* cudaStream_t of the handle */
int cqpi_synchronize(cqpi_handle *h);
/* Kernels this handle has launched since creation (all of them are the engine's own). */
int cqpi_kernel_launches(const cqpi_handle *h, int64_t *count);
/* Device time (ms) per stage, summed over every cqpi_solve_bands / cqpi_run since the
 * previous query (waits for them), measured with CUDA events on the handle's stream:
 * [0] bands, [1] G0(k)+FFT, [2] T-matrix + term1, [3] contraction, [4] total. */
int cqpi_stage_times(cqpi_handle *h, float *ms5);

/* ---- entry point that allocates nothing ------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory:
 * code running while a CUDA stream capture is active (cudaMalloc is not permitted there)
 * and hosts that pre-allocate a fixed device-memory budget and must not let a driver
 * allocation synchronise the device (e.g. a real-time instrument-control loop).
 * Input: the caller-owned device array g0k[kpoints][kpoints][bands][bands][2], G0 of one
 * energy at k = (i, j) / kpoints (index i, j in 0 .. kpoints-1; an index above
 * kpoints/2 stands for i - kpoints), orbital pair (o1, o2), interleaved (re, im) doubles.
 * Output: the caller-owned device array box[2rb+1][2rb+1][bands][bands][2] with, at
 * [X + rb][Y + rb][o1][o2],
 *     G0(R)[o1][o2] = kpoints^-2 sum_{i,j} g0k[i][j][o1][o2] e^{+2 pi i (i X + j Y) / kpoints}
 * for R = (X, Y) in [-rb, rb]^2 (the only real-space values the LDOS contraction reads),
 * in FP64, asynchronously on 'stream' (a cudaStream_t; NULL = default stream).
 * Limits: kpoints <= 4096, bands <= 16, and bands^2 * kpoints * (2rb+1) complex doubles
 * must fit the fixed scratch array of CQPI_NOALLOC_SCRATCH_BYTES -- larger requests
 * return CQPI_ERR_NOT_SUPPORTED.  The array is a file-scope __device__ variable held by
 * every GPU that loads the library until exit; the first call on a device looks up its
 * address (make it before any stream capture).  Calls share the array, so calls whose
 * GPU work overlaps race on it.  No call allocates or frees memory. */
#define CQPI_NOALLOC_SCRATCH_BYTES ((size_t)16 << 20)
int cqpi_realspace_greens_noalloc(const double *g0k, int32_t kpoints, int32_t bands, int32_t rb, double *box,
                                  void *stream);

/* Contraction kernel the handle runs: 0 = FP64 CUDA cores, 1 = FP32 CUDA cores,
 * 2 = tcgen05 tensor cores (split-FP16 x3). */
int cqpi_contraction_kind(const cqpi_handle *h, int32_t *kind);
/* Diagnostic: measured CUDA-core FMA throughput of the current device in TFLOP/s
 * (kind 0: FP64 DFMA, kind 1: FP32 FFMA), the roofline denominator of the engine's
 * CUDA-core kernels.  No counterpart in the reference. */
int cqpi_measure_fma_peak(int32_t kind, double *tflops);

#ifdef __cplusplus
}
#endif
#endif
