// Kernel declarations and launch descriptors shared by the runtime and the
// kernel translation units.
#pragma once
#include "zg_common.cuh"

#include <cuda.h>

#include <atomic>

namespace zg {

// kernels launched by this library since load (all threads)
extern std::atomic<long long> g_launches;

// ------------------------------------------------ tensor-core GEMM (3xTF32)
// D (M x N, fp32, row stride ldd) = (Ah + Al)(Bh + Bl)^T without Al.Bl^T;
// A is M x K, B is N x K, row-major; values are exact TF32 numbers.
struct TcGemm {
  CUtensorMap Ah, Al, Bh, Bl;
  float* D;
  long long ldd;
  int M, N, K, BN;
  int* err;  // device int, nonzero after a timed-out wait
};
int make_tmap_f32(CUtensorMap* map, const float* base, int64_t rows, int64_t cols, int64_t ld, int box_rows);
int tc_gemm_prepare(TcGemm& g, const float* Ah, const float* Al, const float* Bh, const float* Bl, int64_t lda,
                    int64_t ldb, float* D, int64_t ldd, int M, int N, int K, int* err);
int tc_gemm_launch(const TcGemm& g, cudaStream_t s);
// hi = rna_tf32(x), lo = rna_tf32(x - hi)
int launch_split_tf32(const float* x, float* hi, float* lo, int64_t n, cudaStream_t s);

// ------------------------------------------------------------ flat kernels
// out[e] = sum_t c[t] * Y[idx[t]][e]   (Y slots `stride` complex apart)
int launch_combine_c128(const double2* Y, int64_t stride, const CombineCoefs& cf, double2* out,
                        int64_t count, cudaStream_t s);
// Y[last][e] = sum_t c[t] * Y[idx[t]][e], in place (last is one of the idx)
int launch_step_fourth_c128(double2* Y, int64_t stride, int last, const CombineCoefs& cf,
                            int64_t count, cudaStream_t s);
// partial[b] for b < nblocks: block sums of |sum_t c[t] Y[idx[t]][e]|^2 over e in [begin, end)
int terr2_nblocks(int64_t count);
int launch_terr2_partials_c128(const double2* Y, int64_t stride, const CombineCoefs& cf,
                               int64_t begin, int64_t end, double* partial, int nblocks, cudaStream_t s);
// out[j] = sum of partial[j*nblocks .. (j+1)*nblocks), j < nseg (fixed order)
int launch_reduce_partials(const double* partial, int nblocks, int nseg, double* out, cudaStream_t s);

// ------------------------------------------------------------ FP64 GEMM
// C = alpha * opA(A) opB(B) + beta * C ; opA: 0 = A[m*lda+k], 1 = A[k*lda+m];
// opB: 0 = B[k*ldb+n], 1 = B[n*ldb+k], 2 = conj(B[n*ldb+k]).  K = 0 writes beta*C.
struct GemmProb {
  const double2* A;
  const double2* B;
  double2* C;
  int M, N, K;
  int opA, opB;
  int tile_begin, tiles_n;
  int64_t lda, ldb, ldc;
  double2 alpha, beta;
};
#define ZG_MAX_GEMM 32
struct GemmBatch {
  int nprob;
  int total_tiles;
  GemmProb p[ZG_MAX_GEMM];
};
// fills tile_begin/tiles_n/total_tiles and launches
int launch_zgemm_batch(GemmBatch& b, cudaStream_t s);

// ------------------------------------------------------------ RHS helpers
struct StageParams {
  double h, ts, hbar;
  double delta[ZG_MAX_LEADS];
};

struct RhsDev {  // device pointers and sizes of one trajectory
  int n, L, N, Ns, Nf, nc;
  int64_t off_psi, off_omA, off_omB, S;
  const int* mode_lead;
  const int* lead_cols;
  const int* colmap;
  const double2 *H0, *Xp, *Xm, *GLP, *dGP, *XI, *U, *V;
};

struct OmTile {
  int row0, nrows;      // absolute mode rows
  int col0, ncols;      // local column within the block
  int a, b;             // row lead, column lead
  int blk;              // 0: OmA (columns are sourced modes), 1: OmB (free modes)
  int term1, term2;     // which source products apply
};

int launch_build_ht(const RhsDev& d, const double2* sig, const double2* dH, int dH_mode, double U,
                    double2* Ht, cudaStream_t s);
int launch_gathers(const RhsDev& d, const double2* sig, const double2* psi, double2* sigC, double2* G,
                   cudaStream_t s);
int launch_sigma_finalize(const RhsDev& d, const StageParams& p, const double2* T, const double2* Pc,
                          double2* ksig, double* currents, cudaStream_t s);
int launch_psi_finalize(const RhsDev& d, const StageParams& p, const double2* psi, const double2* R2,
                        const double2* ZA, const double2* ZB, double2* kpsi, cudaStream_t s);
// out[0] = FP64 FMA rate, out[1] = FP32 FMA rate, GFLOP/s (2 flops per FMA)
int measure_peaks(double* out);

int launch_omega(const RhsDev& d, const StageParams& p, const OmTile* tiles, int ntiles, const double2* G,
                 const double2* yin, double2* kout, cudaStream_t s);

}  // namespace zg
