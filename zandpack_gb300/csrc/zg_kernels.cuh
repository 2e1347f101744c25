// Kernel declarations and launch descriptors shared by the runtime and the
// kernel translation units.
#pragma once
#include "zg_common.cuh"

#include <cuda.h>

#include <atomic>

namespace zg {

// kernels launched by this library since load (all threads)
extern std::atomic<long long> g_launches;
// kernels launched (or captured into a graph) by the calling thread
extern thread_local long long t_launches;
inline void count_launch() {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  ++t_launches;
}

// ------------------------------------------------ tensor-core GEMM (3xTF32)
// D (M x N, fp32, row stride ldd) = (Ah + Al)(Bh + Bl)^T without Al.Bl^T;
// A is M x K, B is N x K, row-major; values are exact TF32 numbers.
struct TcGemm {
  CUtensorMap Ah, Al, Bh, Bl;
  float* D;
  long long ldd;
  int M, N, K, BN, BK;
  int* err;  // device int, nonzero after a timed-out wait
};
int make_tmap_f32(CUtensorMap* map, const float* base, int64_t rows, int64_t cols, int64_t ld, int box_rows,
                  int box_k);
int tc_gemm_prepare(TcGemm& g, const float* Ah, const float* Al, const float* Bh, const float* Bl, int64_t lda,
                    int64_t ldb, float* D, int64_t ldd, int M, int N, int K, int* err);
int tc_gemm_launch(const TcGemm& g, cudaStream_t s);
// hi = rna_tf32(x), lo = rna_tf32(x - hi)
int launch_split_tf32(const float* x, float* hi, float* lo, int64_t n, cudaStream_t s);

// ------------------------------------------------------ flat kernels (FP64)
// out[e] = sum_t c[t] * Y[idx[t]][e]   (Y slots `stride` complex apart)
int launch_combine_c128(const double2* Y, int64_t stride, const CombineCoefs& cf, double2* out,
                        int64_t count, cudaStream_t s);
// Y[last][e] = sum_t c[t] * Y[idx[t]][e], in place (last is one of the idx)
// gate (device int, may be null): the update is skipped when *gate == 0
int launch_step_fourth_c128(double2* Y, int64_t stride, int last, const CombineCoefs& cf,
                            int64_t count, cudaStream_t s, const int* gate = nullptr);
// partial[b] for b < nblocks: block sums of |sum_t c[t] Y[idx[t]][e]|^2 over e in [begin, end)
int terr2_nblocks(int64_t count);
int launch_terr2_partials_c128(const double2* Y, int64_t stride, const CombineCoefs& cf,
                               int64_t begin, int64_t end, double* partial, int nblocks, cudaStream_t s);
// out[j] = sum of partial[j*nblocks .. (j+1)*nblocks), j < nseg (fixed order)
int launch_reduce_partials(const double* partial, int nblocks, int nseg, double* out, cudaStream_t s);

// --------------------------------------------------- flat kernels (mixed)
// Offsets of the mixed-precision stage buffer (complex64 units): sigma (n x n),
// psi hi and lo parts (N x np each, zero beyond column n), Omega (OmA | OmB).
struct MixedLayout {
  int64_t n, N, np;
  int64_t off_psi, off_omA, S;            // flat state offsets
  int64_t st_psih, st_psil, st_om, st_S;  // stage buffer offsets / size
  int64_t plane;  // psi hi and lo are planar: N x np real parts, then N x np imaginary parts (floats)
};
// stage = y32 + sum_t c[t] K[idx[t]] in FP32, psi written as TF32 hi/lo parts
int launch_stage_input_mixed(const float2* y32, const float2* K, int64_t stride, const CombineCoefs& cf,
                             const MixedLayout& ml, float2* stage, cudaStream_t s);
// FP64 block sums of |sum_t c[t] K[idx[t]][e]|^2 (inner sum in FP32)
int launch_terr2_partials_mixed(const float2* K, int64_t stride, const CombineCoefs& cf, int64_t begin, int64_t end,
                                double* partial, int nblocks, cudaStream_t s);
// y64 += sum_t c[t] K[idx[t]] (increment in FP32, addition in FP64); y32 = fl32(y64)
int launch_update_mixed(double2* y64, float2* y32, const float2* K, int64_t stride, const CombineCoefs& cf,
                        int64_t count, cudaStream_t s, const int* gate = nullptr);
int launch_f64_to_f32(const double2* a, float2* b, int64_t count, cudaStream_t s);
int launch_f32_to_f64(const float2* a, double2* b, int64_t count, cudaStream_t s);

// ------------------------------------------------ SIMT complex GEMM batch
// C = alpha * opA(A [+ A2]) opB(B) + beta * C ; opA: 0 = A[m*lda+k], 1 = A[k*lda+m];
// opB: 0 = B[k*ldb+n], 1 = B[n*ldb+k], 2 = conj(B[n*ldb+k]).  K = 0 writes beta*C.
template <typename T>
struct GemmProb {
  using C = typename cx<T>::t;
  const C* A;
  const C* A2;  // optional second part of A (hi/lo split operands), same layout
  const C* B;
  C* Cm;
  int M, N, K;
  int opA, opB;
  int tile_begin, tiles_n, tiles_mn;
  int ksplit, kchunk;  // split-K: ksplit partial products of kchunk, summed in a fixed order
  int64_t planeA;      // 0: A interleaved complex; > 0: A planar, imaginary part planeA reals after the real
  int64_t ws_off;      // offset of this problem's partials in the workspace
  int64_t lda, ldb, ldc;
  C alpha, beta;
};
#define ZG_MAX_GEMM 32
template <typename T>
struct GemmBatch {
  int nprob;
  int total_tiles;
  int bn;                 // tile width chosen by the planner (32 or 64)
  int want_bn;            // 32: 128x32 tiles whatever the widths (0: the planner chooses)
  typename cx<T>::t* ws;  // split-K workspace
  GemmProb<T> p[ZG_MAX_GEMM];
};
// Chooses split-K factors (enough CTAs for the device) and workspace offsets;
// returns the workspace size in complex elements.
template <typename T>
int64_t plan_zgemm_batch(GemmBatch<T>& b);
// Launches the batch (after planning with the same shapes); problems with
// ksplit > 1 need beta == 0 and a workspace of plan_zgemm_batch() elements.
template <typename T>
int launch_zgemm_batch(GemmBatch<T>& b, int64_t ws_capacity, cudaStream_t s);

// ------------------------------------------------------------ RHS helpers
struct StageParams {
  double h, ts, hbar;
  double delta[ZG_MAX_LEADS];
  // derived once per stage by whoever writes the above (derive_params), so
  // that no kernel thread divides in FP64 (a slow pipe on this GPU)
  double h_hb, inv_hb, h_hb2;  // h/hbar, 1/hbar, h/hbar^2
  float fh, fhbar, fh_hb, finv_hb, fh_hb2;
  float fdelta[ZG_MAX_LEADS];
};
__host__ __device__ inline void derive_params(StageParams& p) {
  p.h_hb = p.h / p.hbar;
  p.inv_hb = 1.0 / p.hbar;
  p.h_hb2 = p.h / (p.hbar * p.hbar);
  p.fh = (float)p.h;
  p.fhbar = (float)p.hbar;
  p.fh_hb = (float)p.h_hb;
  p.finv_hb = (float)p.inv_hb;
  p.fh_hb2 = (float)p.h_hb2;
  for (int a = 0; a < ZG_MAX_LEADS; ++a) p.fdelta[a] = (float)p.delta[a];
}

// ------------------------------------------------ device-side controller
// State of the zand controller kept on the device, so that one attempt runs
// as one CUDA graph without host round trips.
struct DevCtl {
  double t, h, eps, t1;
  double TE, hnew;
  int accepted, done, status, attempts, naccepted;
  int skip;   // this attempt started after the trajectory was done: changes nothing
  int rec_n;  // records written since the batch began
  int pad;
};
// Delta_a(t) of an analytic bias (zg_bias), host and device
__host__ __device__ inline double zg_bias_value(const zg_bias& b, double t, int a) {
  double V = 0.0;
  switch (b.kind) {
    case ZG_BIAS_EXP_RAMP: V = b.V0 * (1.0 - exp(-t / b.tau)); break;
    case ZG_BIAS_GAUSS: V = b.V0 * exp(-(t - b.tc) * (t - b.tc) / (2.0 * b.sigma * b.sigma)); break;
    case ZG_BIAS_SIN: V = b.V0 * sin(2.0 * 3.14159265358979323846 * b.f * t); break;
    case ZG_BIAS_STEP: V = t > 0.0 ? b.V0 : 0.0; break;
    case ZG_BIAS_BOX: V = b.V0 * (tanh(t / b.tau) - tanh((t - b.tc) / b.tau)) / 2.0; break;
    default: V = 0.0;
  }
  return b.w[a] * V;
}
// *out = p (stage parameters given by the host)
int launch_set_params(const StageParams& p, StageParams* out, cudaStream_t s);
// *out = h, ts = t + A_i h, hbar, delta[a] = bias(ts, a) from the device controller
int launch_stage_prologue(const DevCtl* ctl, const zg_bias& b, double A_i, double hbar, StageParams* out,
                          cudaStream_t s);
// the same for all stages of an attempt at once: out[i] from A[i], i < nst
struct StageNodes {
  double A[ZG_MAX_STAGES];
};
int launch_stage_prologues(const DevCtl* ctl, const zg_bias& b, const StageNodes& A, int nst, double hbar,
                           StageParams* out, cudaStream_t s);
// TE = sqrt(err[0]+err[1]+err[2]); accepted = TE < eps; hnew = 0.9 h (eps/TE)^(1/5);
// an attempt that starts after done is skipped (accepted = 0)
int launch_control(const double* err3, DevCtl* ctl, cudaStream_t s);
// after the (gated) update: records the attempt (recs[rec_n], stage-0 currents
// J[0..L)), then on acceptance t += hnew; always h = hnew; done = t >= t1
int launch_advance(DevCtl* ctl, const double* J, int L, zg_attempt_rec* recs, int cap, cudaStream_t s);

template <typename T>
struct RhsDev {  // device pointers and sizes of one trajectory
  using C = typename cx<T>::t;
  int n, L, N, Ns, Nf, nc;
  const int* mode_lead;
  const int* lead_cols;
  const int* colmap;
  int nu;             // orbitals that are a coupling column of some lead
  const int* ucols;   // [nu] those orbitals, ascending
  const int* umap;    // [n] position in ucols, or -1
  const C *Xp, *Xm, *GLP, *dGP, *XI, *U, *V;
};

struct OmTile {
  int row0, nrows;      // absolute mode rows
  int col0, ncols;      // local column within the block
  int a, b;             // row lead, column lead
  int blk;              // 0: OmA (columns are sourced modes), 1: OmB (free modes)
  int term1, term2;     // which source products apply
};

// sigC[a][i][k] = sig[i][C_a[k]], G[m][a][k] = (psi + psi_lo)[m][C_a[k]];
// plane > 0: psi (and psi_lo) planar, imaginary parts plane reals after the real parts
template <typename T>
int launch_gathers(const RhsDev<T>& d, const typename cx<T>::t* sig, const typename cx<T>::t* psi,
                   const typename cx<T>::t* psi_lo, int64_t ldpsi, typename cx<T>::t* sigC, typename cx<T>::t* G,
                   cudaStream_t s, int64_t plane = 0);
// k_sig without the lead terms, then the lead terms (P + P^H)/hbar added to
// the rows and columns of the coupling orbitals only (where P is nonzero).
// dis (may be null): the n x n FP64 dissipator of this stage, entering as - hbar * dis
template <typename T>
// tmode 0: T interleaved complex (row stride ldT complex); planar (row stride
// ldT reals, imaginary columns npl further): 1 = T = [Tr | Ti] (real H),
// 2 = rows [Hr sigma_r | Hr sigma_i] then, npl rows further, [Hi sigma_r | Hi sigma_i]
// W (may be null; non-orthogonal basis): the n x n product P S^-1, whose
// (h/hbar^2)(W + W^H) replaces the lead terms (Pc is then not read)
int launch_sigma_finalize(const RhsDev<T>& d, const StageParams* p, const typename cx<T>::t* Tm, int64_t ldT,
                          const typename cx<T>::t* Pc, const double2* dis, typename cx<T>::t* ksig, cudaStream_t s,
                          int tmode = 0, int npl = 0, const typename cx<T>::t* W = nullptr, bool leads = true);
template <typename T>
int launch_currents(const RhsDev<T>& d, const StageParams* p, const typename cx<T>::t* Pc, double* J, cudaStream_t s);
template <typename T>
// plane > 0: psi planar (see launch_gathers).  rmode 0: R1 interleaved complex
// (row stride ldR1 complex); planar R1 (row stride ldR1 reals, rows of the
// real parts of psi, then N rows of the imaginary parts): 1 = columns H_r
// (real H), 2 = columns [H_r | H_i] with H_i npl columns further
int launch_psi_finalize(const RhsDev<T>& d, const StageParams* p, const typename cx<T>::t* psi,
                        const typename cx<T>::t* psi_lo, int64_t ldpsi, const typename cx<T>::t* R1, int64_t ldR1,
                        const typename cx<T>::t* R2, const typename cx<T>::t* ZA, const typename cx<T>::t* ZB,
                        typename cx<T>::t* kpsi, cudaStream_t s, int64_t plane = 0, int rmode = 0, int npl = 0,
                        const typename cx<T>::t* R3 = nullptr, const typename cx<T>::t* C0 = nullptr);
// R3 and C0 (non-orthogonal basis, both N x n): the Omega xi term already
// multiplied by S^-1 and the constant S^-1 (GL_P xi'), added in place of the
// coupling-column terms (ZA, ZB and GL_P XI are then not read).
// Non-orthogonal basis: Qcat (n x L nc) = the two row classes of Pc summed per
// lead; Zcat (N x L nc) = ZA + ZB per lead; K operands of W = Qcat SmR and
// R3 = Zcat SmT
template <typename T>
int launch_nonorth_gather(const RhsDev<T>& d, const typename cx<T>::t* Pc, const typename cx<T>::t* ZA,
                          const typename cx<T>::t* ZB, typename cx<T>::t* Qcat, typename cx<T>::t* Zcat,
                          cudaStream_t s);
// stationary != 0: writes the Omega of dOmega/dt = 0, i hbar S / (X+ + D_a - X- - D_b),
// instead of the stage derivative (the input Omega is not read)
template <typename T>
int launch_omega(const RhsDev<T>& d, const StageParams* p, const OmTile* tiles, int ntiles, const typename cx<T>::t* G,
                 const typename cx<T>::t* omA_in, const typename cx<T>::t* omB_in, typename cx<T>::t* omA_out,
                 typename cx<T>::t* omB_out, cudaStream_t s, int stationary = 0);
// steady-state preconditioner middle: W[m][k] *= i hbar / (lam_k - X+_m - Delta_lead(m))
int launch_stationary_scale(int N, int n, const double2* Xp, const int* mode_lead, const double* delta,
                            const double* lam, double hbar, double2* W, cudaStream_t s);

// H(t) = H0 + dH (FP64 path).  Sm1 (may be null; non-orthogonal basis): H0
// and dH already carry the factor S^-1 and the Hubbard term enters as
// S^-1 diag(U (sigma_jj - 0.5)), i.e. column j of S^-1 scaled
int launch_build_ht(int n, const double2* H0, const double2* sig, const double2* dH, int dH_mode, double U,
                    double2* Ht, cudaStream_t s, const double2* Sm1 = nullptr);
// Mixed path operands of the two tensor-core GEMMs, TF32 hi/lo parts:
//   Ht (n x np complex = n x 2np real)             A of  T = H(t) sigma
//   BH (2np x 2np real embedding of H(t)^T form)    B of  R1 = psi H(t)^T
//   BS (2np x 2np real embedding of sigma)          B of  T
// Planar TF32 hi/lo operands of the two tensor-core GEMMs (np x np blocks):
//   Ht rows [0, np): Re H(t), rows [np, 2 np): Im H(t)          (K = column)
//   BS rows [0, np): Re sigma^T, rows [np, 2 np): Im sigma^T    (K = row of sigma)
// h_part: 0 = all of Ht, 1 = its diagonal only (off-diagonal entries already
// hold H0), 2 = leave it; BS is always rebuilt.  Padding is zero.
// Sm1: as for launch_build_ht (needs h_part 0 with the Hubbard term)
int launch_build_operands_mixed(int n, int np, const double2* H0, const float2* sig32, const double2* dH, int dH_mode,
                                double U, int h_part, float* Hth, float* Htl, float* BSh, float* BSl, cudaStream_t s,
                                const double2* Sm1 = nullptr);
// the lead terms of k_sigma (after launch_sigma_finalize(..., leads = false);
// Pc = null: none) and the psi finalisation of a mixed stage in one launch,
// for planar psi hi/lo and planar R1 (final_mixed_ok)
bool final_mixed_ok(const RhsDev<float>& d, const float2* psi, const float2* psi_lo, int64_t ldpsi, const float2* R1,
                    int64_t ldR1, int64_t plane, int rmode, int npl);
int launch_final_mixed(const RhsDev<float>& d, const StageParams* p, const float2* Pc, float2* ksig,
                       const float2* psi, const float2* psi_lo, int64_t ldpsi, const float2* R1, int64_t ldR1,
                       const float2* R2, const float2* ZA, const float2* ZB, float2* kpsi, int64_t plane, int rmode,
                       int npl, const float2* R3, const float2* C0, cudaStream_t s);
// k_sigma with its lead terms and the psi finalisation in one launch (no dissipator)
int launch_final_all_mixed(const RhsDev<float>& d, const StageParams* p, const float2* Tm, int64_t ldT, int tmode,
                           const float2* W, const float2* Pc, float2* ksig, const float2* psi, const float2* psi_lo,
                           int64_t ldpsi, const float2* R1, int64_t ldR1, const float2* R2, const float2* ZA,
                           const float2* ZB, float2* kpsi, int64_t plane, int rmode, int npl, const float2* R3,
                           const float2* C0, cudaStream_t s);
// launch_build_operands_mixed and launch_gathers<float> of a mixed stage in one launch
// Per-stage operands of the tensor-core products (zg_tcx.cu) written by the
// stage's gathers: the embedded sigma columns of the xi sigma^T product, and
// the psi gathers of the Omega sources as A rows (Gt, [lead][mode]) and as
// embedded conjugate B' rows (Gc, [lead][2 mode + 0/1]); TF32 hi/lo, rows of
// ldx floats.  Null pointers: not written.
struct TcxOperands {
  float *sigEh = nullptr, *sigEl = nullptr, *Gth = nullptr, *Gtl = nullptr, *Gch = nullptr, *Gcl = nullptr;
  int ldx = 0;
};
int launch_prep_mixed(int n, int np, const double2* H0, const float2* sig32, const double2* dH, int dH_mode,
                      double U, int h_part, float* Hth, float* Htl, float* BSh, float* BSl, const double2* Sm1,
                      const RhsDev<float>& d, const float2* psih, const float2* psil, int64_t ldpsi, float2* sigC,
                      float2* G, int64_t plane, cudaStream_t s, const TcxOperands& op = TcxOperands());
// Lead currents in FP64 from the FP64 state: J_a = 2 Re sum_{m in a} sum_k psi[m][C_a[k]] IXI[m][k] / hbar^2
// row ranges per lead: sourced rows [s[a], s[a+1]), free rows [f[a], f[a+1])
struct CurRows {
  int64_t s[ZG_MAX_LEADS + 1];
  int64_t f[ZG_MAX_LEADS + 1];
};
// part: L x 64 doubles of scratch
int launch_currents64(int n, int L, int nc, const CurRows& rows, const int* lead_cols, const double2* psi,
                      const double2* IXI, double hbar, double* part, double* J, cudaStream_t s);

// out[0] = FP64 FMA rate, out[1] = FP32 FMA rate, GFLOP/s (2 flops per FMA)
int measure_dmma(double* gflops);
int measure_peaks(double* out);

}  // namespace zg
