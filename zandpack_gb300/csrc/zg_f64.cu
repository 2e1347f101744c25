// FP64 kernels of the AME right-hand side and the Runge-Kutta bookkeeping.
//
// Everything here computes in IEEE double.  On GB300 the FP64 pipe delivers
// about 1 TFLOP/s, so these kernels are bound by DFMA issue, not by HBM; they
// are the accuracy reference of the device path (the plain FP64 GPU path).
#include <atomic>

#include "zg_kernels.cuh"

namespace zg {

std::atomic<long long> g_launches{0};

// =================================================================== flat
// One thread handles one complex element per grid-stride iteration; the
// coefficient list is uniform (kernel parameter), loads are 16-byte double2.
__global__ void __launch_bounds__(256) k_combine(const double2* __restrict__ Y, int64_t stride, CombineCoefs cf,
                                                 double2* __restrict__ out, int64_t count) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    double2 acc = make_double2(0.0, 0.0);
    for (int t = 0; t < cf.n; ++t) {
      double2 v = Y[cf.idx[t] * stride + e];
      acc.x = fma(cf.c[t], v.x, acc.x);
      acc.y = fma(cf.c[t], v.y, acc.y);
    }
    out[e] = acc;
  }
}

int launch_combine_c128(const double2* Y, int64_t stride, const CombineCoefs& cf, double2* out,
                        int64_t count, cudaStream_t s) {
  if (count <= 0) return ZG_OK;
  k_combine<<<grid_for(count, 256, 152 * 16), 256, 0, s>>>(Y, stride, cf, out, count);
  ZG_CHECK_LAUNCH();
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return ZG_OK;
}

__global__ void __launch_bounds__(256) k_step_fourth(double2* Y, int64_t stride, int last, CombineCoefs cf,
                                                     int64_t count) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count;
       e += (int64_t)gridDim.x * blockDim.x) {
    double2 acc = make_double2(0.0, 0.0);
    for (int t = 0; t < cf.n; ++t) {
      double2 v = Y[cf.idx[t] * stride + e];
      acc.x = fma(cf.c[t], v.x, acc.x);
      acc.y = fma(cf.c[t], v.y, acc.y);
    }
    Y[last * stride + e] = acc;  // every read of element e happened above
  }
}

int launch_step_fourth_c128(double2* Y, int64_t stride, int last, const CombineCoefs& cf, int64_t count,
                            cudaStream_t s) {
  if (count <= 0) return ZG_OK;
  k_step_fourth<<<grid_for(count, 256, 152 * 16), 256, 0, s>>>(Y, stride, last, cf, count);
  ZG_CHECK_LAUNCH();
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return ZG_OK;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block sum of 256 threads; result valid in thread 0
__device__ __forceinline__ double block_sum256(double v) {
  __shared__ double red[8];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = threadIdx.x < 8 ? red[threadIdx.x] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(256) k_terr2(const double2* __restrict__ Y, int64_t stride, CombineCoefs cf,
                                               int64_t begin, int64_t end, double* __restrict__ partial) {
  double s = 0.0;
  for (int64_t e = begin + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < end;
       e += (int64_t)gridDim.x * blockDim.x) {
    double2 acc = make_double2(0.0, 0.0);
    for (int t = 0; t < cf.n; ++t) {
      double2 v = Y[cf.idx[t] * stride + e];
      acc.x = fma(cf.c[t], v.x, acc.x);
      acc.y = fma(cf.c[t], v.y, acc.y);
    }
    s = fma(acc.x, acc.x, s);
    s = fma(acc.y, acc.y, s);
  }
  s = block_sum256(s);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

int terr2_nblocks(int64_t count) { return grid_for(count, 256, 152 * 4); }

int launch_terr2_partials_c128(const double2* Y, int64_t stride, const CombineCoefs& cf, int64_t begin,
                               int64_t end, double* partial, int nblocks, cudaStream_t s) {
  k_terr2<<<nblocks, 256, 0, s>>>(Y, stride, cf, begin, end, partial);
  ZG_CHECK_LAUNCH();
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return ZG_OK;
}

__global__ void __launch_bounds__(256) k_reduce_partials(const double* __restrict__ partial, int nblocks,
                                                         double* __restrict__ out) {
  const double* p = partial + (int64_t)blockIdx.x * nblocks;
  double s = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) s += p[i];
  s = block_sum256(s);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

int launch_reduce_partials(const double* partial, int nblocks, int nseg, double* out, cudaStream_t s) {
  k_reduce_partials<<<nseg, 256, 0, s>>>(partial, nblocks, out);
  ZG_CHECK_LAUNCH();
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return ZG_OK;
}

// =================================================================== GEMM
// 64x64 output tile per 256-thread block, K staged 8 at a time in shared
// memory; thread (tx, ty) owns rows ty+16i and columns tx+16j (i, j < 4).
#define ZT 64
#define ZK 8

__device__ __forceinline__ double2 load_opA(const GemmProb& P, int m, int k) {
  if (m >= P.M || k >= P.K) return make_double2(0.0, 0.0);
  return P.opA == 0 ? P.A[(int64_t)m * P.lda + k] : P.A[(int64_t)k * P.lda + m];
}
__device__ __forceinline__ double2 load_opB(const GemmProb& P, int k, int n) {
  if (n >= P.N || k >= P.K) return make_double2(0.0, 0.0);
  if (P.opB == 0) return P.B[(int64_t)k * P.ldb + n];
  double2 v = P.B[(int64_t)n * P.ldb + k];
  return P.opB == 2 ? cconj(v) : v;
}

__global__ void __launch_bounds__(256) k_zgemm(const __grid_constant__ GemmBatch batch) {
  const int tile = blockIdx.x;
  int pi = 0;
  while (pi + 1 < batch.nprob && tile >= batch.p[pi + 1].tile_begin) ++pi;
  const GemmProb& P = batch.p[pi];
  const int lt = tile - P.tile_begin;
  const int m0 = (lt / P.tiles_n) * ZT, n0 = (lt % P.tiles_n) * ZT;
  __shared__ double2 As[ZK][ZT];
  __shared__ double2 Bs[ZK][ZT];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_double2(0.0, 0.0);
  for (int k0 = 0; k0 < P.K; k0 += ZK) {
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int idx = tid + 256 * r;
      int m, k, n;
      if (P.opA == 0) { m = idx >> 3; k = idx & 7; } else { m = idx & 63; k = idx >> 6; }
      As[k][m] = load_opA(P, m0 + m, k0 + k);
      if (P.opB == 0) { n = idx & 63; k = idx >> 6; } else { n = idx >> 3; k = idx & 7; }
      Bs[k][n] = load_opB(P, k0 + k, n0 + n);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < ZK; ++kk) {
      double2 a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) cfma(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
  const bool use_beta = (P.beta.x != 0.0 || P.beta.y != 0.0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty + 16 * i;
    if (m >= P.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx + 16 * j;
      if (n >= P.N) continue;
      double2* c = P.C + (int64_t)m * P.ldc + n;
      double2 v = cmul(P.alpha, acc[i][j]);
      if (use_beta) v = cadd(v, cmul(P.beta, *c));
      *c = v;
    }
  }
}

int launch_zgemm_batch(GemmBatch& b, cudaStream_t s) {
  ZG_REQUIRE(b.nprob > 0 && b.nprob <= ZG_MAX_GEMM, "gemm batch size %d out of range", b.nprob);
  int tiles = 0;
  for (int i = 0; i < b.nprob; ++i) {
    GemmProb& P = b.p[i];
    ZG_REQUIRE(P.M >= 0 && P.N >= 0 && P.K >= 0, "negative gemm extent");
    int tm = (P.M + ZT - 1) / ZT, tn = (P.N + ZT - 1) / ZT;
    P.tiles_n = tn > 0 ? tn : 1;
    P.tile_begin = tiles;
    tiles += tm * tn;
  }
  b.total_tiles = tiles;
  if (tiles == 0) return ZG_OK;
  k_zgemm<<<tiles, 256, 0, s>>>(b);
  ZG_CHECK_LAUNCH();
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return ZG_OK;
}

// ============================================================ RHS helpers
// Ht = H0 + dH, dH = uploaded matrix or U*diag(Re sigma_ii - 0.5)
__global__ void k_build_ht(const RhsDev d, const double2* __restrict__ sig, const double2* __restrict__ dH,
                           int dH_mode, double U, double2* __restrict__ Ht) {
  const int64_t nn = (int64_t)d.n * d.n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
    double2 v = d.H0[e];
    if (dH_mode == ZG_DH_MATRIX) v = cadd(v, dH[e]);
    const int i = (int)(e / d.n), j = (int)(e % d.n);
    if (dH_mode == ZG_DH_HUBBARD && i == j) v.x += U * (sig[e].x - 0.5);
    Ht[e] = v;
  }
}

int launch_build_ht(const RhsDev& d, const double2* sig, const double2* dH, int dH_mode, double U, double2* Ht,
                    cudaStream_t s) {
  int64_t nn = (int64_t)d.n * d.n;
  k_build_ht<<<grid_for(nn, 256, 152 * 8), 256, 0, s>>>(d, sig, dH, dH_mode, U, Ht);
  ZG_CHECK_LAUNCH();
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return ZG_OK;
}

// sigC[a][i][k] = sig[i][C_a[k]]  and  G[m][a][k] = psi[m][C_a[k]]
__global__ void k_gathers(const RhsDev d, const double2* __restrict__ sig, const double2* __restrict__ psi,
                          double2* __restrict__ sigC, double2* __restrict__ G) {
  const int64_t ns = (int64_t)d.L * d.n * d.nc;
  const int64_t ng = (int64_t)d.N * d.L * d.nc;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ns + ng;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (e < ns) {
      const int k = (int)(e % d.nc);
      const int64_t r = e / d.nc;
      const int i = (int)(r % d.n), a = (int)(r / d.n);
      sigC[e] = sig[(int64_t)i * d.n + d.lead_cols[a * d.nc + k]];
    } else {
      const int64_t g = e - ns;
      const int k = (int)(g % d.nc);
      const int64_t r = g / d.nc;
      const int a = (int)(r % d.L);
      const int64_t m = r / d.L;
      G[g] = psi[m * d.n + d.lead_cols[a * d.nc + k]];
    }
  }
}

int launch_gathers(const RhsDev& d, const double2* sig, const double2* psi, double2* sigC, double2* G,
                   cudaStream_t s) {
  int64_t tot = (int64_t)d.L * d.n * d.nc + (int64_t)d.N * d.L * d.nc;
  k_gathers<<<grid_for(tot, 256, 152 * 8), 256, 0, s>>>(d, sig, psi, sigC, G);
  ZG_CHECK_LAUNCH();
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return ZG_OK;
}

// P_full[i][j] = sum over (class, lead a) of Pc[class][a][i][colmap[a][j]]
__device__ __forceinline__ double2 p_full(const RhsDev& d, const double2* Pc, int i, int j) {
  double2 v = make_double2(0.0, 0.0);
  for (int a = 0; a < d.L; ++a) {
    const int k = d.colmap[a * d.n + j];
    if (k < 0) continue;
#pragma unroll
    for (int cls = 0; cls < 2; ++cls) v = cadd(v, Pc[((int64_t)(cls * d.L + a) * d.n + i) * d.nc + k]);
  }
  return v;
}

// k_sig = (h/hbar) (-i (T - T^H) + (P + P^H)/hbar), T = H(t) sigma  (Zandpack/mpi/zand:340-387)
__global__ void k_sigma_finalize(const RhsDev d, const StageParams p, const double2* __restrict__ T,
                                 const double2* __restrict__ Pc, double2* __restrict__ ksig) {
  const int64_t nn = (int64_t)d.n * d.n;
  const double ih = 1.0 / p.hbar;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / d.n), j = (int)(e % d.n);
    const double2 tij = T[e], tji = T[(int64_t)j * d.n + i];
    const double2 pij = p_full(d, Pc, i, j), pji = p_full(d, Pc, j, i);
    // -i (tij - conj(tji)) = (tij.y + tji.y, -(tij.x - tji.x))
    double2 v = make_double2(tij.y + tji.y, -(tij.x - tji.x));
    v.x += (pij.x + pji.x) * ih;
    v.y += (pij.y - pji.y) * ih;
    ksig[e] = cscale(v, p.h * ih);
  }
}

// J_a = 2 Re Tr(P_a) / hbar^2 = Re Tr(PI_a)/hbar  (Zandpack/mpi/zand:368-378)
__global__ void k_currents(const RhsDev d, const StageParams p, const double2* __restrict__ Pc,
                           double* __restrict__ J) {
  const int a = blockIdx.x;
  double s = 0.0;
  for (int k = threadIdx.x; k < d.nc; k += blockDim.x) {
    const int i = d.lead_cols[a * d.nc + k];
#pragma unroll
    for (int cls = 0; cls < 2; ++cls) s += Pc[((int64_t)(cls * d.L + a) * d.n + i) * d.nc + k].x;
  }
  s = block_sum256(s);
  if (threadIdx.x == 0) J[a] = 2.0 * s / (p.hbar * p.hbar);
}

int launch_sigma_finalize(const RhsDev& d, const StageParams& p, const double2* T, const double2* Pc,
                          double2* ksig, double* currents, cudaStream_t s) {
  int64_t nn = (int64_t)d.n * d.n;
  k_sigma_finalize<<<grid_for(nn, 256, 152 * 8), 256, 0, s>>>(d, p, T, Pc, ksig);
  ZG_CHECK_LAUNCH();
  g_launches.fetch_add(1, std::memory_order_relaxed);
  if (currents) {
    k_currents<<<d.L, 256, 0, s>>>(d, p, Pc, currents);
    ZG_CHECK_LAUNCH();
  g_launches.fetch_add(1, std::memory_order_relaxed);
  }
  return ZG_OK;
}

// k_psi = -i h [ R1/hbar - (X+ + Delta)/hbar psi + dGP R2 + Z(Omega xi) + GL_P xi ]
// with R1 = psi H^T already in kpsi  (Zandpack/mpi/zand:745-778)
__global__ void k_psi_finalize(const RhsDev d, const StageParams p, const double2* __restrict__ psi,
                               const double2* __restrict__ R2, const double2* __restrict__ ZA,
                               const double2* __restrict__ ZB, double2* __restrict__ kpsi) {
  const int64_t tot = (int64_t)d.N * d.n;
  const double ih = 1.0 / p.hbar;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = e / d.n;
    const int i = (int)(e % d.n);
    const int a = d.mode_lead[m];
    double2 xp = d.Xp[m];
    xp.x += p.delta[a];
    double2 v = cscale(kpsi[e], ih);
    v = csub(v, cscale(cmul(xp, psi[e]), ih));
    if (m < d.Ns) v = cadd(v, cmul(d.dGP[m], R2[m * d.n + i]));
    for (int b = 0; b < d.L; ++b) {
      const int k = d.colmap[b * d.n + i];
      if (k < 0) continue;
      v = cadd(v, ZA[((int64_t)b * d.N + m) * d.nc + k]);
      if (m < d.Ns) v = cadd(v, ZB[((int64_t)b * d.Ns + m) * d.nc + k]);
    }
    const int ka = d.colmap[a * d.n + i];
    if (ka >= 0) v = cadd(v, cmul(d.GLP[m], d.XI[m * d.nc + ka]));
    // (-i h) v = (h v.y, -h v.x)
    kpsi[e] = make_double2(p.h * v.y, -p.h * v.x);
  }
}

int launch_psi_finalize(const RhsDev& d, const StageParams& p, const double2* psi, const double2* R2,
                        const double2* ZA, const double2* ZB, double2* kpsi, cudaStream_t s) {
  int64_t tot = (int64_t)d.N * d.n;
  k_psi_finalize<<<grid_for(tot, 256, 152 * 16), 256, 0, s>>>(d, p, psi, R2, ZA, ZB, kpsi);
  ZG_CHECK_LAUNCH();
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return ZG_OK;
}

// Omega stage derivative on one 64x64 tile whose rows belong to lead a and
// columns to lead b (Zandpack/mpi/zand:782-809):
//   k[m,l] = h sum_k G[m][b][k] U[l][k]              (term1, U = dGM * IXI)
//          + h sum_k V[m][k] conj(G[l][a][k])        (term2, V = dGP * XIT2)
//          + (i h/hbar)(X+_m + D_a - X-_l - D_b) Omega[m,l]
__global__ void __launch_bounds__(256) k_omega(const RhsDev d, const StageParams p, const OmTile* __restrict__ tiles,
                                               const double2* __restrict__ G, const double2* __restrict__ yin,
                                               double2* __restrict__ kout) {
  const OmTile t = tiles[blockIdx.x];
  __shared__ double2 As[ZK][ZT];
  __shared__ double2 Bs[ZK][ZT];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int nc = d.nc;
  const int colmode0 = (t.blk == 0 ? 0 : d.Ns) + t.col0;  // absolute mode of local column col0
  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = make_double2(0.0, 0.0);
  const int kbeg = t.term1 ? 0 : nc, kend = t.term2 ? 2 * nc : nc;
  for (int k0 = kbeg; k0 < kend; k0 += ZK) {
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int idx = tid + 256 * r;
      const int rr = idx >> 3, kk = idx & 7;
      const int k = k0 + kk;
      double2 av = make_double2(0.0, 0.0), bv = make_double2(0.0, 0.0);
      if (k < kend) {
        if (rr < t.nrows) {
          const int64_t m = t.row0 + rr;
          av = k < nc ? G[(m * d.L + t.b) * nc + k] : d.V[m * nc + (k - nc)];
        }
        if (rr < t.ncols) {
          const int64_t l = colmode0 + rr;
          bv = k < nc ? d.U[l * nc + k] : cconj(G[(l * d.L + t.a) * nc + (k - nc)]);
        }
      }
      As[kk][rr] = av;
      Bs[kk][rr] = bv;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < ZK; ++kk) {
      double2 a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) cfma(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
  const double sc = p.h / p.hbar;
  const int64_t ld = t.blk == 0 ? d.Ns : d.Nf;
  const int64_t base = t.blk == 0 ? d.off_omA : d.off_omB;
  const double da = p.delta[t.a], db = p.delta[t.b];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = ty + 16 * i;
    if (r >= t.nrows) continue;
    const int64_t m = t.row0 + r;
    double2 xp = d.Xp[m];
    xp.x += da;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = tx + 16 * j;
      if (c >= t.ncols) continue;
      const int64_t l = colmode0 + c;
      double2 xm = d.Xm[l];
      xm.x += db;
      const int64_t e = base + m * ld + (t.col0 + c);
      const double2 dx = csub(xp, xm);
      const double2 om = yin[e];
      const double2 dd = cmul(dx, om);           // (X+ - X-) Omega
      // (i h/hbar) dd = sc * (-dd.y, dd.x)
      double2 v = cscale(acc[i][j], p.h);
      v.x -= sc * dd.y;
      v.y += sc * dd.x;
      kout[e] = v;
    }
  }
}

int launch_omega(const RhsDev& d, const StageParams& p, const OmTile* tiles, int ntiles, const double2* G,
                 const double2* yin, double2* kout, cudaStream_t s) {
  if (ntiles == 0) return ZG_OK;
  k_omega<<<ntiles, 256, 0, s>>>(d, p, tiles, G, yin, kout);
  ZG_CHECK_LAUNCH();
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return ZG_OK;
}

}  // namespace zg

namespace zg {

// ------------------------------------------------------------ peak probes
// Independent FMA chains per thread; the result store is never taken but keeps
// the chains live.
template <typename T>
__global__ void __launch_bounds__(256) k_fma_peak(T* out, T a, T b, int iters) {
  T x0 = (T)threadIdx.x * (T)1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
    x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)1.2345) out[0] = s;
}

int measure_peaks(double* out) {
  int dev = 0, sms = 0;
  ZG_CHECK_CUDA(cudaGetDevice(&dev));
  ZG_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double* d = nullptr;
  ZG_CHECK_CUDA(cudaMalloc(&d, 16));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, thr = 256;
  for (int which = 0; which < 2; ++which) {
    const int iters = which == 0 ? 2048 : 65536;
    double best = 0.0;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0);
      if (which == 0) k_fma_peak<double><<<blocks, thr>>>(d, 0.999, 1e-3, iters);
      else k_fma_peak<float><<<blocks, thr>>>((float*)d, 0.999f, 1e-3f, iters);
      cudaEventRecord(e1);
      cudaError_t err = cudaEventSynchronize(e1);
      if (err != cudaSuccess) { cudaFree(d); set_error("peak probe: %s", cudaGetErrorString(err)); return ZG_ECUDA; }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      double gf = 2.0 * 8.0 * iters * (double)blocks * thr / (ms * 1e6);
      best = gf > best ? gf : best;
    }
    out[which] = best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  ZG_CHECK_LAUNCH();
  return ZG_OK;
}

}  // namespace zg
