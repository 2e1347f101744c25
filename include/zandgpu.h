/*
 * zandgpu.h -- C ABI of libzandgpu.so, the GB300 (sm_103a) engine for the
 * auxiliary-mode-expansion (AME) propagation of Zandpack's `zand` driver.
 *
 * Conventions
 *   - complex numbers are interleaved (re, im) doubles, as numpy complex128;
 *   - every function returns a zg_status; zg_last_error() gives the message of
 *     the last failure on the calling thread;
 *   - host pointers are plain host memory (pageable or pinned); device pointers
 *     are CUDA device memory of the current device;
 *   - no function throws across the ABI.
 *
 * Which reference interface each entry point replaces is cited per function
 * (paths inside the Zandpack repository).
 */
#ifndef ZANDGPU_H
#define ZANDGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  ZG_OK = 0,
  ZG_EINVAL = 1,     /* bad argument or shape (the reference raises AssertionError) */
  ZG_ENOMEM = 2,     /* device allocation failed */
  ZG_ECUDA = 3,      /* CUDA runtime error */
  ZG_ETIMEOUT = 4,   /* a bounded device-side wait gave up */
  ZG_ENONFINITE = 5  /* the error norm is NaN or infinite */
} zg_status;

enum { ZG_PREC_F64 = 0, ZG_PREC_MIXED = 1 };
enum { ZG_DH_NONE = 0, ZG_DH_MATRIX = 1, ZG_DH_HUBBARD = 2 };
#define ZG_MAX_LEADS 16
#define ZG_MAX_STAGES 13

const char* zg_last_error(void);
int zg_version(void);
/* Number of kernels this library has launched since it was loaded. */
long long zg_launch_count(void);

/* ------------------------------------------------------------------------
 * Compact layout of one propagation (host arrays, copied at creation).
 * Built by zandpack_gb300.layout.CompactLayout from the reference's Arrays/
 * (Zandpack/mpi/zand:113-124,568-664; Zandpack/Writer.py:61-151).
 * Mode order: sourced modes by lead, then source-free modes by lead.
 * ---------------------------------------------------------------------- */
typedef struct {
  int32_t n;           /* orbitals (NO) */
  int32_t n_leads;     /* NL */
  int32_t n_modes;     /* N: live auxiliary modes */
  int32_t n_sourced;   /* Ns: modes with diff_GGP_GLP or diff_GGM_GLM nonzero */
  int32_t nc;          /* coupling columns per lead (padded) */
  double hbar;         /* eV fs */
  const int32_t* mode_lead;   /* [N] */
  const int64_t* s_start;     /* [NL+1] sourced rows of lead a: [s_start[a], s_start[a+1]) */
  const int64_t* f_start;     /* [NL+1] free rows of lead a (absolute mode index) */
  const int32_t* lead_cols;   /* [NL*nc] orbital of coupling column k of lead a */
  const int32_t* colmap;      /* [NL*n] coupling column of orbital j in lead a, or -1 */
  const double* H0;           /* [n*n] complex */
  const double* Xp;           /* [N] complex: Xpp of the mode */
  const double* Xm;           /* [N] complex: Xpm of the mode */
  const double* GLP;          /* [N] complex */
  const double* dGP;          /* [N] complex: diff_GGP_GLP */
  const double* dGM;          /* [N] complex: diff_GGM_GLM */
  const double* XI;           /* [N*nc] complex: xi on the lead's columns */
  const double* IXI;          /* [N*nc] complex: Ixi on orbidx_alpha, else 0 */
  const double* XIS;          /* [N*nc] complex: xi/hbar^2 on orbidx_Ixi_all_nonzero, else 0 */
  const double* XIT2;         /* [N*nc] complex: xi on orbidx_xi_nonzero, else 0 */
} zg_layout;

typedef struct zg_traj zg_traj;

/* One trajectory: constants, the RK_N+1 state slots (k_0..k_{RK_N-1}, y) and
 * scratch on the device.  Replaces the per-rank arrays of SIGMA()/Worker()
 * (Zandpack/mpi/zand:200-290,498-690).  precision: ZG_PREC_F64 or ZG_PREC_MIXED. */
int zg_traj_create(int device, const zg_layout* layout, int precision, zg_traj** out);
int zg_traj_destroy(zg_traj* t);
/* out[0..7] = n, NL, N, Ns, Nf, nc, state size (complex elements), stages */
int zg_traj_info(const zg_traj* t, int64_t* out);
/* The cudaStream_t all work of the trajectory is issued on (for events). */
void* zg_traj_stream(const zg_traj* t);

/* Butcher tableau (Zandpack/mpi_RK4pars_dev.py:118-149 layout): A[s], B[s*(s+1)]
 * (column s multiplies the stored y), CT[s], CH[s+1].  Entries of B outside
 * idxholder[i] must be given as 0.  DOP54 is preloaded. */
int zg_set_tableau(zg_traj* t, int stages, const double* A, const double* B,
                   const double* CT, const double* CH);

/* State slots: slot 0..stages-1 = k_i (the SIGS/PSIS/OMGS[i] arrays), slot
 * `stages` = y (SIGS[-1] etc.).  Flat compact vector of `state size` complex. */
int zg_set_state(zg_traj* t, int slot, const double* host);
int zg_get_state(zg_traj* t, int slot, double* host);
/* y = (sigma, psi = 0, Omega = 0): the reference's initial state
 * (Zandpack/mpi/zand:536-538) from the n*n sigma alone. */
int zg_set_sigma(zg_traj* t, const double* sigma);

/* Stage input Y_i = sum_{j in idxholder[i]} B[i,j] Y_j (Y_stages = y); for
 * i = 0 the input is y itself.  Replaces the MM / step_*_forward_nb stage
 * combination (Zandpack/mpi/zand:306-313,722-735; Zandpack/func_step_forward.py:16-139). */
int zg_stage_input(zg_traj* t, int stage);
/* Download sigma of the current stage input (n*n complex), for a host dH(t, sigma). */
int zg_get_stage_sigma(zg_traj* t, double* host);
/* Upload the dH(t, sigma) matrix (n*n complex) that ZG_DH_MATRIX adds to H0. */
int zg_set_dH(zg_traj* t, const double* host);
/* dissipator(ts, sigma) of the coming zg_rhs calls (n*n complex), entering k_sigma
 * as - hbar * dissipator (Zandpack/mpi/zand:343); NULL switches it off.  The
 * reference evaluates it at every stage: set it before each zg_rhs.  zg_attempt
 * and the graph path refuse to run while one is set. */
int zg_set_dissipator(zg_traj* t, const double* host);

/* Non-orthogonal basis: the equations of the reference's nozand
 * (Zandpack/mpi/nozand:259-320, :456-500, :1003-1290) for sigma' =
 * S^-1/2 sigma S^-1/2 and psi' (rows S^-1/2 psi).  The trajectory's layout
 * must already hold the nozand constants: H0 = H0' (S^1/2 H_Ortho S^1/2), XI
 * and IXI from xi' (rows S^1/2 xi) and Ixi' (rows Ixi S^1/2).  Sm1 = S^-1
 * (n*n complex), C0 = the constant term S^-1 (GL_P xi') of every compact mode
 * row (N*n complex, computed from the full xi').  Then every stage uses
 * S^-1 H(t) in place of H(t) (the Hubbard term enters as S^-1 diag(u), an
 * uploaded dH matrix is multiplied by S^-1 on the device), the lead terms of
 * sigma become (P S^-1 + h.c.)/hbar, and psi gains S^-1 (Omega xi'/hbar^2)
 * and C0 in place of the coupling-column terms.  Sm1 = NULL returns to the
 * orthogonal equations.  The steady-state entry points refuse a trajectory
 * in this mode. */
int zg_set_overlap(zg_traj* t, const double* Sm1, const double* C0);

/* k_stage = h f(ts, Y_stage): the stage body of zand (Zandpack/mpi/zand:318-387
 * master, :713-809 worker).  delta[NL] = bias(ts, a); dH_mode selects
 * H(t) = H0 (+ uploaded dH | + hubbard_U*diag(Re sigma_ii - 0.5)).  If
 * currents != NULL, the lead currents Re Tr(PI_a)/hbar of this stage input
 * are written there (:368-378). */
int zg_rhs(zg_traj* t, int stage, double ts, double h, const double* delta,
           int dH_mode, double hubbard_U, double* currents);

/* err2[0..2] = TERR2_sig, TERR2_psi, TERR2_omg of the k slots
 * (Zandpack/mpi_funcs.py:247-252; Zandpack/func_step_forward.py:39-53,75-91,141-159). */
int zg_error_norm2(zg_traj* t, double* err2);

/* y <- sum_j CH_j Y_j (step_fourth_*, Zandpack/mpi_funcs.py:254-259). */
int zg_step_fourth(zg_traj* t);

/* Analytic lead biases evaluated inside the library: Delta_a(t) = w[a] V(t) with
 *   ZG_BIAS_ZERO: V = 0;  ZG_BIAS_EXP_RAMP: V0 (1 - exp(-t/tau));
 *   ZG_BIAS_GAUSS: V0 exp(-(t-tc)^2 / (2 sigma^2));  ZG_BIAS_SIN: V0 sin(2 pi f t);
 *   ZG_BIAS_STEP: V0 for t > 0, else 0;  ZG_BIAS_BOX: V0 (tanh(t/tau) - tanh((t-tc)/tau))/2.
 * The +V/2, -V/2 split of make_constant_bias (Zandpack/Pulses.py:81-88) is
 * w = {0.5, -0.5, 0, ...}; box_pulse is Zandpack/Pulses.py:72-74. */
enum { ZG_BIAS_ZERO = 0, ZG_BIAS_EXP_RAMP = 1, ZG_BIAS_GAUSS = 2, ZG_BIAS_SIN = 3, ZG_BIAS_STEP = 4,
       ZG_BIAS_BOX = 5 };
typedef struct {
  int32_t kind;
  double V0, tau, tc, sigma, f;
  double w[ZG_MAX_LEADS];
} zg_bias;

/* One attempt of the zand controller (Zandpack/mpi/zand:301-430) with
 * library-evaluated bias and dH (dH_mode ZG_DH_NONE or ZG_DH_HUBBARD):
 * all stages from the stored y at time *t with step *h, the error norm,
 * accept iff TE < eps; on acceptance y is updated and *t advances by the new
 * step size; *h becomes 0.9 h (eps/TE)^(1/5) either way.  currents (may be
 * NULL) receives the stage-0 lead currents.  One host call per attempt. */
int zg_attempt(zg_traj* t, double* time, double* h, double eps, const zg_bias* bias, int dH_mode,
               double hubbard_U, double* TE, int* accepted, double* currents);
/* Download sigma (n*n complex) of a state slot; the DM the reference records
 * after every accepted step (Zandpack/mpi/zand:428-430). */
int zg_get_sigma(zg_traj* t, int slot, double* host);

/* Steady state (Zandpack/cmdtools/psinought:180-451), on an FP64 trajectory
 * whose y holds the fixed density matrix (zg_set_sigma).  The stationary psi
 * solves k_psi(sigma, psi, Omega(psi)) = 0 where Omega(psi) solves
 * dOmega/dt = 0; a Krylov solver on the caller's side drives:
 *   zg_stationary_setup: stage time, lead biases, dH mode, and the eigenpairs
 *     (V: n*n complex, columns; lam: n) of H = H0 + dH used by the
 *     preconditioner;
 *   zg_stationary_apply: kpsi = k_psi(psi) with h = 1 (affine in psi); psi and
 *     kpsi are N*n complex device arrays (compact layout); afterwards y holds
 *     (sigma, psi, Omega(psi));
 *   zg_stationary_precond: out = i hbar r_m (H^T - X+_m - Delta)^{-1} per mode
 *     row m, the inverse of k_psi's dominant term. */
int zg_stationary_setup(zg_traj* t, double ts, const double* delta, int dH_mode, double hubbard_U, const double* V,
                        const double* lam);
int zg_stationary_apply(zg_traj* t, const double* psi_dev, double* kpsi_dev);
int zg_stationary_precond(zg_traj* t, const double* r_dev, double* out_dev);

/* Graph-launched attempts.  The same attempt as zg_attempt, with the
 * controller (t, h, TE, accept, next step size) kept on the device and the
 * whole attempt captured once as a CUDA graph, so that a run of attempts needs
 * one graph launch each and one host synchronisation per batch of attempts.
 * Once t >= t1 (or a non-finite error norm) the trajectory is done and further
 * launched attempts change nothing.  Replaces the host loop of
 * Zandpack/mpi/zand:301-430 for analytic biases. */
#define ZG_GRAPH_MAX_BATCH 256
typedef struct {
  double t;       /* time at the start of the attempt */
  double h;       /* step size of the attempt */
  double TE;      /* error norm */
  double h_next;  /* 0.9 h (eps/TE)^(1/5) */
  int32_t accepted;
  int32_t status; /* ZG_OK or ZG_ENONFINITE */
  double J[ZG_MAX_LEADS]; /* stage-0 lead currents */
} zg_attempt_rec;
/* Capture the attempt graph for this bias and dH mode (ZG_DH_NONE or
 * ZG_DH_HUBBARD).  zg_set_tableau and a change of zg_profile drop the graph;
 * the next zg_graph_run captures it again.  With profiling on, the regions of
 * the last attempt of each batch are accumulated. */
int zg_graph_prepare(zg_traj* t, const zg_bias* bias, int dH_mode, double hubbard_U);
/* Set the device controller: time, step size, tolerance and end time. */
int zg_graph_set(zg_traj* t, double time, double h, double eps, double t1);
/* Launch `count` (<= ZG_GRAPH_MAX_BATCH) attempts back to back, then
 * synchronise once.  recs (may be NULL) receives one record per attempt that
 * ran before the trajectory was done, *nrec their number; time, h and done
 * (each may be NULL) the controller after the batch. */
int zg_graph_run(zg_traj* t, int count, zg_attempt_rec* recs, int* nrec, double* time, double* h, int* done);

/* Which kernels compute the mixed path's small products (the PI partials,
 * Omega xi, xi sigma^T) and dOmega/dt:
 *   ZG_IMPL_SIMT         FP32 SIMT kernels for both (dOmega/dt on the
 *                        trajectory's second stream);
 *   ZG_IMPL_TC_PRODUCTS  the products on the tensor cores, dOmega/dt SIMT on
 *                        the second stream;
 *   ZG_IMPL_TC_ALL       both in one tensor-core launch;
 *   ZG_IMPL_TC_SPLIT     the products on the tensor cores, dOmega/dt as a
 *                        second tensor-core launch (tiles of 32 complex
 *                        columns whatever n_c) on the second stream.
 * zg_set_impl selects one (ZG_EINVAL when the trajectory's shapes do not
 * allow it; the FP64 path ignores it); zg_get_impl reads the current choice
 * and, in *avail, a bit mask of the implementations the trajectory supports.
 * The second stream (H(t) sigma, and dOmega/dt unless ZG_IMPL_TC_ALL) forks
 * off before psi H(t)^T (ZG_SCHED_EARLY, the default: faster on every
 * workload measured) or after it (ZG_SCHED_LATE): zg_set_schedule /
 * zg_get_schedule.
 * zg_tune times one right-hand side of every supported implementation under
 * both schedules (CUDA events, `reps` evaluations each, after one untimed
 * evaluation) on the current state, keeps the fastest and returns it as
 * *best = impl + ZG_IMPL_COUNT * schedule, and the milliseconds per
 * evaluation of each in ms[ZG_IMPL_COUNT * ZG_SCHED_COUNT] (same index, -1
 * where not supported).  It overwrites k slot 0 and drops a captured attempt
 * graph.
 * These replace no reference interface: they choose among this library's
 * kernels for the reference's Q_np / Omega stage terms
 * (Zandpack/mpi/zand:91-110,770-809). */
enum { ZG_IMPL_SIMT = 0, ZG_IMPL_TC_PRODUCTS = 1, ZG_IMPL_TC_ALL = 2, ZG_IMPL_TC_SPLIT = 3, ZG_IMPL_COUNT = 4 };
enum { ZG_SCHED_LATE = 0, ZG_SCHED_EARLY = 1, ZG_SCHED_COUNT = 2 };
int zg_set_impl(zg_traj* t, int impl);
int zg_get_impl(const zg_traj* t, int* impl, int* avail);
int zg_set_schedule(zg_traj* t, int sched);
int zg_get_schedule(const zg_traj* t, int* sched);
int zg_tune(zg_traj* t, int reps, int* best, double* ms);

/* Measurement.  With profiling on, CUDA events on the trajectory's stream
 * bracket each region; zg_profile_read returns accumulated milliseconds and
 * counts per region (indices ZG_PROF_*).  zg_profile(t, 1) also resets them. */
enum { ZG_PROF_GEMM = 0, ZG_PROF_OMEGA = 1, ZG_PROF_FINAL = 2, ZG_PROF_COMBINE = 3, ZG_PROF_ERROR = 4,
       ZG_PROF_UPDATE = 5, ZG_PROF_RHS = 6, ZG_PROF_PREP = 7, ZG_PROF_SMALL = 8, ZG_PROF_GEMM2 = 9,
       ZG_PROF_REGIONS = 10 };
int zg_profile(zg_traj* t, int enable);
int zg_profile_read(zg_traj* t, double* ms, long long* count);
/* Live FP64 and FP32 FMA throughput of `device` in GFLOP/s (out[0], out[1]). */
int zg_measure_peaks(int device, double* out);
/* Live FP64 tensor-core (mma.sync m8n8k4, DMMA) throughput of `device` in
 * GFLOP/s, beside the DFMA rate of zg_measure_peaks: the FP64 path's GEMMs
 * run on DFMA, and this probe records whether DMMA would be faster. */
int zg_measure_fp64_mma(int device, double* gflops);

/* ------------------------------------------------------------------------
 * Tensor-core building blocks of the mixed-precision path (device pointers).
 * ---------------------------------------------------------------------- */
/* hi = x rounded to TF32 (nearest, ties away), lo = (x - hi) rounded to TF32. */
int zg_split_tf32(const float* x, float* hi, float* lo, int64_t n, void* stream);
/* D (M x N, row-major fp32) = (Ah + Al)(Bh + Bl)^T minus the Al.Bl^T term, on
 * tcgen05 tensor cores; A is M x K, B is N x K, row-major, TF32-exact values;
 * K % 4 == 0, N % 32 == 0.  Synchronises the stream; ZG_ETIMEOUT if a bounded
 * device-side wait gave up. */
int zg_gemm_tf32x3(const float* Ah, const float* Al, const float* Bh, const float* Bl, float* D,
                   int M, int N, int K, void* stream);
/* Self-test of the bounded device-side waits: one thread waits, with the
 * GEMM's wait helper and a budget of `budget_cycles` SM clocks, on an
 * mbarrier that nothing completes.  Returns ZG_ETIMEOUT when the wait gave
 * up and reported it (the expected outcome; the context stays usable),
 * ZG_OK if it did not. */
int zg_wait_selftest(int device, long long budget_cycles);

/* ------------------------------------------------------------------------
 * Stateless array kernels on caller device buffers (complex128), the
 * numba/numpy kernels of Zandpack/func_step_forward.py and mpi_funcs.py.
 * Y holds `nslots` arrays of `count` complex elements, `slot_stride`
 * complex elements apart.  stream: a cudaStream_t (NULL = default stream).
 * ---------------------------------------------------------------------- */
/* out = sum_{j in idx} b[j] Y[j]  (step_{sig,psi,omg}_forward_nb(Y, b, out, idx), :16-109) */
int zg_combine_c128(const double* Y, int64_t slot_stride, int nslots, const double* b,
                    const int32_t* idx, int nidx, double* out, int64_t count, void* stream);
/* *result = sum_e |sum_j ct[j] Y[j][e]|^2  (TERR2_*_nb, :39-53; TERR2_*, mpi_funcs.py:247-252).
 * Uses a device scratch buffer of partial sums that it allocates stream-ordered. */
int zg_terr2_c128(const double* Y, int64_t slot_stride, int nslots, const double* ct,
                  int64_t count, double* result, void* stream);
/* Same result as zg_terr2_c128, for callers that must not allocate device
 * memory while they run (for example a serving loop that reserved all of HBM
 * up front, or a host whose device memory is owned by another allocator).
 * No counterpart in the reference.  The partial sums live in a static 8 KiB
 * device array (1024 doubles) inside the library.  The reduction's grid is
 * capped at 608 blocks, so it never needs more than 609 of those doubles and
 * every count the allocating entry point accepts fits; the size check before
 * the launch (ZG_EINVAL on an oversize request) can therefore not trigger
 * with the present grid cap.  Calls share the array: calls that overlap on
 * the GPU race and must be serialised.  The first call on a device looks up
 * the array's device address (with that device current) and caches it for
 * the life of the process; the cached address does not survive a
 * cudaDeviceReset, so a program that resets the device must not call this
 * entry point afterwards.  Like zg_terr2_c128 it copies the result to host
 * memory and synchronises `stream`, so it must not be called while that
 * stream is being captured into a CUDA graph. */
int zg_terr2_c128_noalloc(const double* Y, int64_t slot_stride, int nslots, const double* ct,
                          int64_t count, double* result, void* stream);
/* Y[nslots-1] = sum_j ch[j] Y[j]  (step_fourth_*, mpi_funcs.py:254-259) */
int zg_step_fourth_c128(double* Y, int64_t slot_stride, int nslots, const double* ch,
                        int64_t count, void* stream);
/* The Omega stage combination that leaves Fermi x Fermi blocks untouched
 * (step_omg_forward_nb_fermi_opti(Y, b, out, idx, fp_loc, fp_all),
 * Zandpack/func_step_forward.py:112-139): a slot has shape7 = (nk, NL, NX,
 * NOT, NL, NX, NOT); out[e] = sum_{j in idx} b[j] Y[j][e] except where
 * fp_loc[x] and fp_all[x'] are both nonzero (x = axis 2, x' = axis 5), where
 * out is not written.  fp_loc (NX bytes) and fp_all (NX bytes) are device
 * arrays. */
int zg_combine_fermi_skip_c128(const double* Y, int64_t slot_stride, int nslots, const double* b,
                               const int32_t* idx, int nidx, double* out, const int64_t* shape7,
                               const uint8_t* fp_loc, const uint8_t* fp_all, void* stream);
/* The diagonal term of dOmega/dt (OuterSubtraction_hard_opti(A, B, C, out),
 * Zandpack/mpi_funcs.py:91-102): with shape7 = (nk, na, nx, noT, NA, NX, NO)
 * the shape of C and out, out[k,a,x,c,a',x',:] += (A[k,a,x,0] - B[k,a',x',0])
 * * C[k,a,x,c,a',x',:].  A is (nk, na, nx, lda_c) and B (nk, NA, NX, ldb_c),
 * all contiguous complex128 device arrays. */
int zg_outer_subtraction_c128(const double* A, int lda_c, const double* B, int ldb_c, const double* C,
                              double* out, const int64_t* shape7, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ZANDGPU_H */
