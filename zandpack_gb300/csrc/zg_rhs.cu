// Right-hand-side kernels of the AME equations (Zandpack/mpi/zand:318-387
// sigma, :745-778 psi, :782-809 Omega), templated on the real type: double
// for the FP64 path, float for the mixed-precision path (whose two large
// products run on the tensor cores, zg_tc.cu).
#include "zg_kernels.cuh"

namespace zg {

#define GRID_STRIDE(e, count) \
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (count); e += (int64_t)gridDim.x * blockDim.x)

// Stage parameters as the kernels read them: the scalars in registers, the
// per-lead biases through a pointer (a dynamically indexed copy of the whole
// struct would live in local memory).
struct StageScalars {
  double h, ts, hbar, h_hb, inv_hb, h_hb2;
  float fh, fhbar, fh_hb, finv_hb, fh_hb2;
  const double* delta;
  const float* fdelta;
};
__device__ __forceinline__ StageScalars load_params(const StageParams* __restrict__ pp) {
  StageScalars s;
  s.h = pp->h;
  s.ts = pp->ts;
  s.hbar = pp->hbar;
  s.h_hb = pp->h_hb;
  s.inv_hb = pp->inv_hb;
  s.h_hb2 = pp->h_hb2;
  s.fh = pp->fh;
  s.fhbar = pp->fhbar;
  s.fh_hb = pp->fh_hb;
  s.finv_hb = pp->finv_hb;
  s.fh_hb2 = pp->fh_hb2;
  s.delta = pp->delta;
  s.fdelta = pp->fdelta;
  return s;
}
// the stage scalar of the kernel's real type: the FP64 value or its FP32 copy
template <typename T>
__device__ __forceinline__ T pv(double d, float f);
template <>
__device__ __forceinline__ double pv<double>(double d, float) { return d; }
template <>
__device__ __forceinline__ float pv<float>(double, float f) { return f; }

template <typename T>
__device__ __forceinline__ typename cx<T>::t czero() {
  return cx<T>::make((T)0, (T)0);
}

// =================================================================== GEMM
// Output tile of BM x BN complex per 256-thread block, K staged 8 at a time
// in shared memory; TX = BN/4 threads along N, TY = 256/TX along M, thread
// (tx, ty) owns rows ty+TY*i and columns tx+TX*j (i, j < 4).  BN = 64 gives
// 64x64 tiles; BN = 32 gives 128x32 tiles for the products whose N is the
// coupling width (n_c <= 32), which would leave half of a 64-wide tile idle.
#define ZK 8

// Raw operand loads: nothing consumes the loaded values until they are stored
// to shared memory a K stage later (the hi + lo sum and the conjugation of
// opB = 2 happen there), so the loads stay in flight behind the compute.
template <typename T>
__device__ __forceinline__ void load_opA(const GemmProb<T>& P, int m, int k, typename cx<T>::t& v,
                                         typename cx<T>::t& v2) {
  v = czero<T>();
  v2 = czero<T>();
  if (m >= P.M || k >= P.K) return;
  const int64_t o = P.opA == 0 ? (int64_t)m * P.lda + k : (int64_t)k * P.lda + m;
  if (P.planeA) {  // planar A: real part at element index o, imaginary part planeA reals further
    const T* a = reinterpret_cast<const T*>(P.A);
    v = cx<T>::make(a[o], a[o + P.planeA]);
    if (P.A2) {
      const T* a2 = reinterpret_cast<const T*>(P.A2);
      v2 = cx<T>::make(a2[o], a2[o + P.planeA]);
    }
    return;
  }
  v = P.A[o];
  if (P.A2) v2 = P.A2[o];
}
template <typename T>
__device__ __forceinline__ typename cx<T>::t load_opB(const GemmProb<T>& P, int k, int n) {
  if (n >= P.N || k >= P.K) return czero<T>();
  return P.opB == 0 ? P.B[(int64_t)k * P.ldb + n] : P.B[(int64_t)n * P.ldb + k];
}

// FP32: K staged 8 at a time under a 3-blocks-per-SM register budget (80
// registers; 16 at a time needed 144 registers, one block per SM)
template <typename T, int BN>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1) k_zgemm(const __grid_constant__ GemmBatch<T> batch) {
  using C = typename cx<T>::t;
  constexpr int TX = BN / 4, TY = 256 / TX, BM = 4 * TY;
  const int tile = blockIdx.x;
  int pi = 0;
  while (pi + 1 < batch.nprob && tile >= batch.p[pi + 1].tile_begin) ++pi;
  const GemmProb<T>& P = batch.p[pi];
  const int ltk = tile - P.tile_begin;
  const int split = ltk / P.tiles_mn, lt = ltk % P.tiles_mn;
  const int m0 = (lt / P.tiles_n) * BM, n0 = (lt % P.tiles_n) * BN;
  const int kb0 = split * P.kchunk;
  const int kb1 = min(P.K, kb0 + P.kchunk);
  // K staged ZKG at a time; the next stage's global loads are issued into
  // registers before the current stage is computed, hiding their latency
  constexpr int ZKG = sizeof(T) == 4 ? 8 : 16, RA = BM * ZKG / 256, RB = BN * ZKG / 256;
  // rows padded by one element: K-contiguous operands are stored column-wise
  // (ZKG threads with consecutive k, same m), which without padding would hit
  // one bank ZKG times
  __shared__ C As[ZKG][BM + 1];
  __shared__ C Bs[ZKG][BN + 1];
  const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
  C acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = czero<T>();
  // element r of this thread's share of a K stage (recomputed, not kept in registers)
#define ZG_AM(r) (P.opA == 0 ? ((tid + 256 * (r)) / ZKG) : ((tid + 256 * (r)) % BM))
#define ZG_AK(r) (P.opA == 0 ? ((tid + 256 * (r)) % ZKG) : ((tid + 256 * (r)) / BM))
#define ZG_BN(r) (P.opB == 0 ? ((tid + 256 * (r)) % BN) : ((tid + 256 * (r)) / ZKG))
#define ZG_BK(r) (P.opB == 0 ? ((tid + 256 * (r)) / BN) : ((tid + 256 * (r)) % ZKG))
  C ra[RA], ra2[RA], rb[RB];
  const bool conjB = P.opB == 2;
#pragma unroll
  for (int r = 0; r < RA; ++r) {
    if (kb0 + ZG_AK(r) < kb1) {
      load_opA(P, m0 + ZG_AM(r), kb0 + ZG_AK(r), ra[r], ra2[r]);
    } else {
      ra[r] = czero<T>();
      ra2[r] = czero<T>();
    }
  }
#pragma unroll
  for (int r = 0; r < RB; ++r) rb[r] = kb0 + ZG_BK(r) < kb1 ? load_opB(P, kb0 + ZG_BK(r), n0 + ZG_BN(r)) : czero<T>();
  for (int k0 = kb0; k0 < kb1; k0 += ZKG) {
#pragma unroll
    for (int r = 0; r < RA; ++r) As[ZG_AK(r)][ZG_AM(r)] = cadd(ra[r], ra2[r]);
#pragma unroll
    for (int r = 0; r < RB; ++r) Bs[ZG_BK(r)][ZG_BN(r)] = conjB ? cconj(rb[r]) : rb[r];
    __syncthreads();
    const int k1 = k0 + ZKG;
    if (k1 < kb1) {
#pragma unroll
      for (int r = 0; r < RA; ++r) {
        if (k1 + ZG_AK(r) < kb1) {
          load_opA(P, m0 + ZG_AM(r), k1 + ZG_AK(r), ra[r], ra2[r]);
        } else {
          ra[r] = czero<T>();
          ra2[r] = czero<T>();
        }
      }
#pragma unroll
      for (int r = 0; r < RB; ++r) rb[r] = k1 + ZG_BK(r) < kb1 ? load_opB(P, k1 + ZG_BK(r), n0 + ZG_BN(r)) : czero<T>();
    }
#pragma unroll
    for (int kk = 0; kk < ZKG; ++kk) {
      C a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + TY * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + TX * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) cfma(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
  const bool use_beta = (P.beta.x != (T)0 || P.beta.y != (T)0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty + TY * i;
    if (m >= P.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx + TX * j;
      if (n >= P.N) continue;
      if (P.ksplit > 1) {  // partial product of this K chunk, reduced later in split order
        batch.ws[P.ws_off + ((int64_t)split * P.M + m) * P.N + n] = acc[i][j];
        continue;
      }
      C* c = P.Cm + (int64_t)m * P.ldc + n;
      C v = cmul(P.alpha, acc[i][j]);
      if (use_beta) v = cadd(v, cmul(P.beta, *c));
      *c = v;
    }
  }
#undef ZG_AM
#undef ZG_AK
#undef ZG_BN
#undef ZG_BK
}

// C = alpha * sum over splits of the partials, splits added in order.  The
// output elements of all split problems form one index space (problem after
// problem), so every problem is reduced by the whole grid at once.
template <typename T>
__global__ void k_zgemm_reduce(const __grid_constant__ GemmBatch<T> batch, int64_t total) {
  using C = typename cx<T>::t;
  GRID_STRIDE(g, total) {
    int64_t e = g;
    int pi = 0;
    for (; pi < batch.nprob; ++pi) {
      const GemmProb<T>& P = batch.p[pi];
      if (P.ksplit <= 1) continue;
      const int64_t mn = (int64_t)P.M * P.N;
      if (e < mn) break;
      e -= mn;
    }
    const GemmProb<T>& P = batch.p[pi];
    const int64_t mn = (int64_t)P.M * P.N;
    const C* src = batch.ws + P.ws_off + e;
    C v = czero<T>();
    // four partials loaded together, added in split order
    int sp = 0;
    for (; sp + 4 <= P.ksplit; sp += 4) {
      const C v0 = src[sp * mn], v1 = src[(sp + 1) * mn], v2 = src[(sp + 2) * mn], v3 = src[(sp + 3) * mn];
      v = cadd(cadd(cadd(cadd(v, v0), v1), v2), v3);
    }
    for (; sp < P.ksplit; ++sp) v = cadd(v, src[sp * mn]);
    P.Cm[(e / P.N) * P.ldc + (e % P.N)] = cmul(P.alpha, v);
  }
}

template <typename T>
int64_t plan_zgemm_batch(GemmBatch<T>& b) {
  // tile width: 32 when every problem is at most 32 wide
  int maxN = 0;
  for (int i = 0; i < b.nprob; ++i) maxN = b.p[i].N > maxN ? b.p[i].N : maxN;
  b.bn = b.want_bn == 32 || maxN <= 32 ? 32 : 64;
  const int BN = b.bn, BM = 4 * (256 / (BN / 4));
  // A problem with few output tiles and a long K would serialise on a handful
  // of CTAs (the batch is then less than one wave, and its longest tile sets
  // the time): split its K into chunks of >= KMIN until it has ~TARGET CTAs.
  // FP32 tiles are cheap per K, so their chunks are shorter than FP64's.
  const int64_t target = sizeof(T) == 4 ? 4 * 152 : 2 * 152;
  const int KMIN = sizeof(T) == 4 ? 128 : 256;
  int tiles = 0;
  int64_t ws = 0;
  for (int i = 0; i < b.nprob; ++i) {
    GemmProb<T>& P = b.p[i];
    const int tm = (P.M + BM - 1) / BM, tn = (P.N + BN - 1) / BN;
    P.tiles_n = tn > 0 ? tn : 1;
    P.tiles_mn = tm * tn > 0 ? tm * tn : 1;
    P.ksplit = 1;
    P.kchunk = P.K > 0 ? P.K : 1;
    P.ws_off = 0;
    const bool plain_beta = P.beta.x == (T)0 && P.beta.y == (T)0;
    if (plain_beta && P.K >= 2 * KMIN && tm * tn > 0 && tm * tn < target) {
      int want = (int)((target + tm * tn - 1) / (tm * tn));
      int maxs = P.K / KMIN;  // at least KMIN of K per split
      int ks = want < maxs ? want : maxs;
      if (ks > 1) {
        int chunk = (P.K + ks - 1) / ks;
        chunk = (chunk + ZK - 1) / ZK * ZK;
        P.kchunk = chunk;
        P.ksplit = (P.K + chunk - 1) / chunk;
        P.ws_off = ws;
        ws += (int64_t)P.ksplit * P.M * P.N;
      }
    }
    P.tile_begin = tiles;
    tiles += (tm * tn) * P.ksplit;
  }
  b.total_tiles = tiles;
  return ws;
}

template <typename T>
int launch_zgemm_batch(GemmBatch<T>& b, int64_t ws_capacity, cudaStream_t s) {
  ZG_REQUIRE(b.nprob > 0 && b.nprob <= ZG_MAX_GEMM, "gemm batch size %d out of range", b.nprob);
  for (int i = 0; i < b.nprob; ++i)
    ZG_REQUIRE(b.p[i].M >= 0 && b.p[i].N >= 0 && b.p[i].K >= 0, "negative gemm extent");
  const int64_t need = plan_zgemm_batch<T>(b);
  ZG_REQUIRE(need <= ws_capacity && (need == 0 || b.ws), "split-K workspace too small (%lld > %lld)",
             (long long)need, (long long)ws_capacity);
  if (b.total_tiles == 0) return ZG_OK;
  if (b.bn == 32)
    k_zgemm<T, 32><<<b.total_tiles, 256, 0, s>>>(b);
  else
    k_zgemm<T, 64><<<b.total_tiles, 256, 0, s>>>(b);
  ZG_CHECK_LAUNCH();
  count_launch();
  if (need > 0) {
    int64_t total = 0;
    for (int i = 0; i < b.nprob; ++i)
      if (b.p[i].ksplit > 1) total += (int64_t)b.p[i].M * b.p[i].N;
    k_zgemm_reduce<T><<<grid_for(total, 256, 152 * 8), 256, 0, s>>>(b, total);
    ZG_CHECK_LAUNCH();
    count_launch();
  }
  return ZG_OK;
}

// ============================================================ RHS helpers
// gather elements e = first, first + stride, ... of sigC and G
template <typename T>
__device__ __forceinline__ void gathers_job(const RhsDev<T>& d, const typename cx<T>::t* __restrict__ sig,
                                            const typename cx<T>::t* __restrict__ psi,
                                            const typename cx<T>::t* __restrict__ psi_lo, int64_t ldpsi,
                                            typename cx<T>::t* __restrict__ sigC, typename cx<T>::t* __restrict__ G,
                                            int64_t plane, int64_t first, int64_t stride,
                                            const TcxOperands op = TcxOperands()) {
  float* __restrict__ sigEh = op.sigEh;
  float* __restrict__ sigEl = op.sigEl;
  const int ldx = op.ldx;
  const int64_t ns = (int64_t)d.L * d.n * d.nc;
  const int64_t ng = (int64_t)d.N * d.L * d.nc;
  for (int64_t e = first; e < ns + ng; e += stride) {
    if (e < ns) {
      const int k = (int)(e % d.nc);
      const int64_t r = e / d.nc;
      const int i = (int)(r % d.n), a = (int)(r / d.n);
      const typename cx<T>::t v = sig[(int64_t)i * d.n + d.lead_cols[a * d.nc + k]];
      sigC[e] = v;
      if (sigEh) {
        // B' of the xi sigma^T product on the tensor cores: rows 2i, 2i+1 of
        // lead a hold (Re, -Im) and (Im, Re) of sigma[i][C_a[k]], TF32 hi/lo
        const float x = (float)v.x, y = (float)v.y;
        uint32_t hx, hy, lx, ly;
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hx) : "f"(x));
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hy) : "f"(y));
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lx) : "f"(x - __uint_as_float(hx)));
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(ly) : "f"(y - __uint_as_float(hy)));
        const int64_t o0 = ((int64_t)a * 2 * d.n + 2 * i) * ldx + 2 * k, o1 = o0 + ldx;
        sigEh[o0] = __uint_as_float(hx);
        sigEh[o0 + 1] = -__uint_as_float(hy);
        sigEh[o1] = __uint_as_float(hy);
        sigEh[o1 + 1] = __uint_as_float(hx);
        sigEl[o0] = __uint_as_float(lx);
        sigEl[o0 + 1] = -__uint_as_float(ly);
        sigEl[o1] = __uint_as_float(ly);
        sigEl[o1 + 1] = __uint_as_float(lx);
      }
    } else {
      const int64_t g = e - ns;
      const int k = (int)(g % d.nc);
      const int64_t r = g / d.nc;
      const int a = (int)(r % d.L);
      const int64_t m = r / d.L;
      const int64_t o = m * ldpsi + d.lead_cols[a * d.nc + k];
      typename cx<T>::t v;
      if (plane) {  // planar psi: real parts, imaginary parts plane reals further
        const T* ph = reinterpret_cast<const T*>(psi);
        v = cx<T>::make(ph[o], ph[o + plane]);
        if (psi_lo) {
          const T* pl = reinterpret_cast<const T*>(psi_lo);
          v = cadd(v, cx<T>::make(pl[o], pl[o + plane]));
          if (op.Gth) {
            // the Omega sources on the tensor cores: A rows (psi on lead a's
            // columns) and the embedded conjugate B' rows (Re, Im) / (-Im, Re),
            // from the TF32 hi/lo parts of psi as they are
            const float hr = (float)ph[o], hi = (float)ph[o + plane], lr = (float)pl[o], li = (float)pl[o + plane];
            const int64_t ot = ((int64_t)a * d.N + m) * ldx + 2 * k;
            op.Gth[ot] = hr; op.Gth[ot + 1] = hi;
            op.Gtl[ot] = lr; op.Gtl[ot + 1] = li;
            const int64_t oc = ((int64_t)a * 2 * d.N + 2 * m) * ldx + 2 * k, oc1 = oc + ldx;
            op.Gch[oc] = hr; op.Gch[oc + 1] = hi; op.Gch[oc1] = -hi; op.Gch[oc1 + 1] = hr;
            op.Gcl[oc] = lr; op.Gcl[oc + 1] = li; op.Gcl[oc1] = -li; op.Gcl[oc1 + 1] = lr;
          }
        }
      } else {
        v = psi[o];
        if (psi_lo) v = cadd(v, psi_lo[o]);
      }
      G[g] = v;
    }
  }
}

template <typename T>
__global__ void k_gathers(const RhsDev<T> d, const typename cx<T>::t* __restrict__ sig,
                          const typename cx<T>::t* __restrict__ psi, const typename cx<T>::t* __restrict__ psi_lo,
                          int64_t ldpsi, typename cx<T>::t* __restrict__ sigC, typename cx<T>::t* __restrict__ G,
                          int64_t plane) {
  gathers_job<T>(d, sig, psi, psi_lo, ldpsi, sigC, G, plane, blockIdx.x * (int64_t)blockDim.x + threadIdx.x,
                 (int64_t)gridDim.x * blockDim.x);
}

template <typename T>
int launch_gathers(const RhsDev<T>& d, const typename cx<T>::t* sig, const typename cx<T>::t* psi,
                   const typename cx<T>::t* psi_lo, int64_t ldpsi, typename cx<T>::t* sigC, typename cx<T>::t* G,
                   cudaStream_t s, int64_t plane) {
  int64_t tot = (int64_t)d.L * d.n * d.nc + (int64_t)d.N * d.L * d.nc;
  k_gathers<T><<<grid_for(tot, 256, 152 * 8), 256, 0, s>>>(d, sig, psi, psi_lo, ldpsi, sigC, G, plane);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

// P_full[i][j] = sum over (class, lead a) of Pc[class][a][i][colmap[a][j]]
template <typename T>
__device__ __forceinline__ typename cx<T>::t p_full(const RhsDev<T>& d, const typename cx<T>::t* Pc, int i, int j) {
  typename cx<T>::t v = czero<T>();
  for (int a = 0; a < d.L; ++a) {
    const int k = d.colmap[a * d.n + j];
    if (k < 0) continue;
#pragma unroll
    for (int cls = 0; cls < 2; ++cls) v = cadd(v, Pc[((int64_t)(cls * d.L + a) * d.n + i) * d.nc + k]);
  }
  return v;
}

// k_sig = (h/hbar) (-i (T - T^H) + (P + P^H)/hbar), T = H(t) sigma  (Zandpack/mpi/zand:340-387)
// Pass 1: the commutator (and the dissipator) for every element, one 32 x 32
// block per CTA with the transposed block of T staged through shared memory
// so that both reads of T are row-contiguous.
// element (i, j) of T = H(t) sigma in the layouts of launch_sigma_finalize
template <typename T>
__device__ __forceinline__ typename cx<T>::t load_T(const typename cx<T>::t* Tm, int64_t ldT, int tmode, int npl, int i,
                                                    int j) {
  if (tmode == 0) return Tm[(int64_t)i * ldT + j];
  const T* f = reinterpret_cast<const T*>(Tm);
  const int64_t r = (int64_t)i * ldT;
  if (tmode == 1) return cx<T>::make(f[r + j], f[r + npl + j]);
  const int64_t r2 = (int64_t)(npl + i) * ldT;  // rows of Im H
  return cx<T>::make(f[r + j] - f[r2 + npl + j], f[r + npl + j] + f[r2 + j]);
}

// DIS: a dissipator is set (a template parameter: a runtime branch would be
// if-converted into predicated FP64 multiplies issued for every element)
// One 32 x 32 block (bx, by) of k_sigma by 256 threads (tx < 32, ty < 8).
// Pc (may be null): the lead terms (h/hbar^2)(P + P^H) added here to the
// elements in a coupling row or column, after the scaling, as the separate
// lead pass adds them.
template <typename T, bool DIS>
__device__ __forceinline__ void sigma_tile_job(int bx, int by, int tx, int ty, const RhsDev<T>& d,
                                               const StageScalars& p, const typename cx<T>::t* __restrict__ Tm,
                                               int64_t ldT, const double2* __restrict__ dis,
                                               typename cx<T>::t* __restrict__ ksig, int tmode, int npl,
                                               const typename cx<T>::t* __restrict__ W,
                                               const typename cx<T>::t* __restrict__ Pc) {
  using C = typename cx<T>::t;
  __shared__ C tile[32][33];   // tile[r][c] = T[j0 + r][i0 + c]
  __shared__ C wtile[32][33];  // the same of W (non-orthogonal basis)
  const T sc = pv<T>(p.h_hb, p.fh_hb);
  const T fw = pv<T>(p.h_hb2, p.fh_hb2);
  const int n = d.n;
  const int i0 = by * 32, j0 = bx * 32;
  for (int r = ty; r < 32; r += 8) {
    const int j = j0 + r, i = i0 + tx;
    const bool in = j < n && i < n;
    tile[r][tx] = in ? load_T<T>(Tm, ldT, tmode, npl, j, i) : czero<T>();
    if (W) wtile[r][tx] = in ? W[(int64_t)j * n + i] : czero<T>();
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + r, j = j0 + tx;
    if (i >= n || j >= n) continue;
    const C tij = load_T<T>(Tm, ldT, tmode, npl, i, j);
    const C tji = tile[tx][r];
    // -i (tij - conj(tji)) = (tij.y + tji.y, -(tij.x - tji.x))
    C v = cx<T>::make(tij.y + tji.y, -(tij.x - tji.x));
    const int64_t e = (int64_t)i * n + j;
    if (DIS) {  // - hbar * dissipator(ts, sigma)  (Zandpack/mpi/zand:343)
      const double2 q = dis[e];
      v.x -= (T)(p.hbar * q.x);
      v.y -= (T)(p.hbar * q.y);
    }
    v = cscale(v, sc);
    if (W) {  // (h/hbar^2)(P S^-1 + (P S^-1)^H)  (Zandpack/mpi/nozand:489-499)
      const C wij = W[e], wji = wtile[tx][r];
      v.x += fw * (wij.x + wji.x);
      v.y += fw * (wij.y - wji.y);
    } else if (Pc && (d.umap[i] >= 0 || d.umap[j] >= 0)) {
      const C pij = p_full(d, Pc, i, j), pji = p_full(d, Pc, j, i);
      v.x += fw * (pij.x + pji.x);
      v.y += fw * (pij.y - pji.y);
    }
    ksig[e] = v;
  }
}

template <typename T, bool DIS>
__global__ void __launch_bounds__(256) k_sigma_finalize(const RhsDev<T> d, const StageParams* __restrict__ pp,
                                                        const typename cx<T>::t* __restrict__ Tm, int64_t ldT,
                                                        const double2* __restrict__ dis,
                                                        typename cx<T>::t* __restrict__ ksig, int tmode, int npl,
                                                        const typename cx<T>::t* __restrict__ W) {
  const StageScalars p = load_params(pp);
  sigma_tile_job<T, DIS>(blockIdx.x, blockIdx.y, threadIdx.x, threadIdx.y, d, p, Tm, ldT, dis, ksig, tmode, npl, W,
                         nullptr);
}

// Pass 2: + (h/hbar^2)(P + P^H) on the elements (i, j) with i or j a coupling
// orbital, each element once: columns j in U for every row i, then rows i in U
// for the columns j not in U.
template <typename T>
__device__ __forceinline__ void sigma_leads_job(const RhsDev<T>& d, const StageScalars& p,
                                                const typename cx<T>::t* __restrict__ Pc,
                                                typename cx<T>::t* __restrict__ ksig, int64_t first, int64_t stride) {
  using C = typename cx<T>::t;
  const T f = pv<T>(p.h_hb2, p.fh_hb2);
  const int n = d.n, nu = d.nu;
  const int64_t half = (int64_t)nu * n;
  for (int64_t q = first; q < 2 * half; q += stride) {
    int i, j;
    if (q < half) {
      i = (int)(q / nu);
      j = d.ucols[q - (int64_t)i * nu];
    } else {
      const int64_t q2 = q - half;
      const int u = (int)(q2 / n);
      j = (int)(q2 - (int64_t)u * n);
      if (d.umap[j] >= 0) continue;  // done in the column pass
      i = d.ucols[u];
    }
    const C pij = p_full(d, Pc, i, j), pji = p_full(d, Pc, j, i);
    const int64_t e = (int64_t)i * n + j;
    C v = ksig[e];
    v.x += f * (pij.x + pji.x);
    v.y += f * (pij.y - pji.y);
    ksig[e] = v;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_sigma_leads(const RhsDev<T> d, const StageParams* __restrict__ pp,
                                                     const typename cx<T>::t* __restrict__ Pc,
                                                     typename cx<T>::t* __restrict__ ksig) {
  const StageScalars p = load_params(pp);
  sigma_leads_job<T>(d, p, Pc, ksig, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

template <typename T>
int launch_sigma_finalize(const RhsDev<T>& d, const StageParams* p, const typename cx<T>::t* Tm, int64_t ldT,
                          const typename cx<T>::t* Pc, const double2* dis, typename cx<T>::t* ksig, cudaStream_t s,
                          int tmode, int npl, const typename cx<T>::t* W, bool leads) {
  ZG_REQUIRE(tmode >= 0 && tmode <= 2, "bad T layout %d", tmode);
  const int nb = (d.n + 31) / 32;
  if (dis)
    k_sigma_finalize<T, true><<<dim3(nb, nb), dim3(32, 8), 0, s>>>(d, p, Tm, ldT, dis, ksig, tmode, npl, W);
  else
    k_sigma_finalize<T, false><<<dim3(nb, nb), dim3(32, 8), 0, s>>>(d, p, Tm, ldT, dis, ksig, tmode, npl, W);
  ZG_CHECK_LAUNCH();
  count_launch();
  if (d.nu > 0 && !W && leads) {
    const int64_t tot = 2 * (int64_t)d.nu * d.n;
    k_sigma_leads<T><<<grid_for(tot, 256, 152 * 8), 256, 0, s>>>(d, p, Pc, ksig);
    ZG_CHECK_LAUNCH();
    count_launch();
  }
  return ZG_OK;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double block_sum256_d(double v) {
  __shared__ double red[8];
  v = warp_sum_d(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = threadIdx.x < 8 ? red[threadIdx.x] : 0.0;
    r = warp_sum_d(r);
  }
  __syncthreads();
  return r;
}

// J_a = 2 Re Tr(P_a) / hbar^2 = Re Tr(PI_a)/hbar  (Zandpack/mpi/zand:368-378)
template <typename T>
__global__ void k_currents(const RhsDev<T> d, const StageParams* __restrict__ pp, const typename cx<T>::t* __restrict__ Pc,
                           double* __restrict__ J) {
  const StageScalars p = load_params(pp);
  const int a = blockIdx.x;
  double s = 0.0;
  for (int k = threadIdx.x; k < d.nc; k += blockDim.x) {
    const int i = d.lead_cols[a * d.nc + k];
#pragma unroll
    for (int cls = 0; cls < 2; ++cls) s += (double)Pc[((int64_t)(cls * d.L + a) * d.n + i) * d.nc + k].x;
  }
  s = block_sum256_d(s);
  if (threadIdx.x == 0) J[a] = 2.0 * s / (p.hbar * p.hbar);
}

template <typename T>
int launch_currents(const RhsDev<T>& d, const StageParams* p, const typename cx<T>::t* Pc, double* J, cudaStream_t s) {
  k_currents<T><<<d.L, 256, 0, s>>>(d, p, Pc, J);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

// J_a from the FP64 state: 2 Re sum_{m in lead a} sum_k psi[m][C_a[k]] IXI[m][k] / hbar^2.
// Grid (CUR_CHUNKS, L): chunk c of lead a sums a strided share of the lead's
// (row, k) pairs; the chunks of a lead are then added in a fixed order.
#define CUR_CHUNKS 64
__global__ void __launch_bounds__(256) k_currents64_part(int n, int nc, CurRows rows,
                                                         const int* __restrict__ lead_cols,
                                                         const double2* __restrict__ psi,
                                                         const double2* __restrict__ IXI, double* __restrict__ part) {
  const int a = blockIdx.y;
  const int64_t s0 = rows.s[a], ns = rows.s[a + 1] - s0;
  const int64_t f0 = rows.f[a], nf = rows.f[a + 1] - f0;
  const int64_t tot = (ns + nf) * nc;
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / nc;
    const int k = (int)(e % nc);
    const int64_t m = r < ns ? s0 + r : f0 + (r - ns);
    const double2 ps = psi[m * n + lead_cols[a * nc + k]];
    const double2 ix = IXI[m * nc + k];
    s += ps.x * ix.x - ps.y * ix.y;
  }
  s = block_sum256_d(s);
  if (threadIdx.x == 0) part[a * CUR_CHUNKS + blockIdx.x] = s;
}

__global__ void k_currents64_final(const double* __restrict__ part, double hbar, double* __restrict__ J) {
  if (threadIdx.x != 0) return;
  const int a = blockIdx.x;
  double s = 0.0;
  for (int c = 0; c < CUR_CHUNKS; ++c) s += part[a * CUR_CHUNKS + c];
  J[a] = 2.0 * s / (hbar * hbar);
}

int launch_currents64(int n, int L, int nc, const CurRows& rows, const int* lead_cols, const double2* psi,
                      const double2* IXI, double hbar, double* part, double* J, cudaStream_t s) {
  k_currents64_part<<<dim3(CUR_CHUNKS, L), 256, 0, s>>>(n, nc, rows, lead_cols, psi, IXI, part);
  ZG_CHECK_LAUNCH();
  count_launch();
  k_currents64_final<<<L, 32, 0, s>>>(part, hbar, J);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

// k_psi = -i h [ R1/hbar - (X+ + Delta)/hbar psi + dGP R2 + Z(Omega xi) + GL_P xi ]
// with R1 = psi H^T  (Zandpack/mpi/zand:745-778).
// One block per mode row at a time: the row's constants are uniform, and its
// coupling-column terms (ZA, ZB rows of every lead, XI row) are staged in
// shared memory, so the per-element work is four streaming loads plus the
// column map.  R1 may alias kpsi (the FP64 path finalises in place).
template <typename T>
__global__ void __launch_bounds__(256) k_psi_finalize(const RhsDev<T> d, const StageParams* __restrict__ pp, const typename cx<T>::t* __restrict__ psi,
                               const typename cx<T>::t* __restrict__ psi_lo, int64_t ldpsi,
                               const typename cx<T>::t* R1, int64_t ldR1, const typename cx<T>::t* __restrict__ R2,
                               const typename cx<T>::t* __restrict__ ZA, const typename cx<T>::t* __restrict__ ZB,
                               typename cx<T>::t* kpsi, int64_t plane, int rmode, int npl,
                               const typename cx<T>::t* __restrict__ R3, const typename cx<T>::t* __restrict__ C0) {
  using C = typename cx<T>::t;
  extern __shared__ __align__(16) unsigned char psi_smem[];
  C* sZ = reinterpret_cast<C*>(psi_smem);  // [L][nc]: ZA + ZB of this row
  C* sX = sZ + d.L * d.nc;                 // [nc]: GL_P xi of this row on its lead's columns
  const StageScalars p = load_params(pp);
  const T ih = pv<T>(p.inv_hb, p.finv_hb);
  const T h = pv<T>(p.h, p.fh);
  const int n = d.n, nc = d.nc, L = d.L;
  for (int m = blockIdx.x; m < d.N; m += gridDim.x) {
    const bool src = m < d.Ns;
    const int a = d.mode_lead[m];
    const C glp = d.GLP[m];
    if (!R3) {
      for (int q = threadIdx.x; q < L * nc; q += blockDim.x) {
        const int b = q / nc, k = q - b * nc;
        C z = ZA[((int64_t)b * d.N + m) * nc + k];
        if (src) z = cadd(z, ZB[((int64_t)b * d.Ns + m) * nc + k]);
        sZ[q] = z;
      }
      for (int q = threadIdx.x; q < nc; q += blockDim.x) sX[q] = cmul(glp, d.XI[(int64_t)m * nc + q]);
    }
    C xp = d.Xp[m];
    xp.x += pv<T>(p.delta[a], p.fdelta[a]);
    const C dgp = src ? d.dGP[m] : czero<T>();
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      C ps, pl, r1;
      const int64_t o = (int64_t)m * ldpsi + i;
      if (plane) {
        const T* ph = reinterpret_cast<const T*>(psi);
        ps = cx<T>::make(ph[o], ph[o + plane]);
        if (psi_lo) {
          const T* plo = reinterpret_cast<const T*>(psi_lo);
          pl = cx<T>::make(plo[o], plo[o + plane]);
        } else {
          pl = czero<T>();
        }
      } else {
        ps = psi[o];
        pl = psi_lo ? psi_lo[o] : czero<T>();
      }
      if (rmode == 0) {
        r1 = R1[(int64_t)m * ldR1 + i];
      } else {
        // planar R1: rows (Re psi) m and (Im psi) N + m; columns H_r, then H_i npl further
        const T* f = reinterpret_cast<const T*>(R1);
        const int64_t a0 = (int64_t)m * ldR1 + i, a1 = (int64_t)(d.N + m) * ldR1 + i;
        r1 = rmode == 1 ? cx<T>::make(f[a0], f[a1])
                        : cx<T>::make(f[a0] - f[a1 + npl], f[a0 + npl] + f[a1]);
      }
      const C r2 = src ? R2[(int64_t)m * n + i] : czero<T>();
      ps = cadd(ps, pl);
      C v = cscale(r1, ih);
      v = csub(v, cscale(cmul(xp, ps), ih));
      v = cadd(v, cmul(dgp, r2));
      if (R3) {  // S^-1 (Omega xi'/hbar^2) + S^-1 (GL_P xi')  (Zandpack/mpi/nozand:1003,1208-1210)
        const int64_t e = (int64_t)m * n + i;
        v = cadd(v, cadd(R3[e], C0[e]));
      } else {
        for (int b = 0; b < L; ++b) {
          const int k = d.colmap[b * n + i];
          if (k >= 0) {
            v = cadd(v, sZ[b * nc + k]);
            if (b == a) v = cadd(v, sX[k]);
          }
        }
      }
      // (-i h) v = (h v.y, -h v.x)
      kpsi[(int64_t)m * n + i] = cx<T>::make(h * v.y, -h * v.x);
    }
    __syncthreads();
  }
}

// Mixed path, planar psi hi/lo and planar R1, n a multiple of V: one thread
// per (row, V consecutive columns), no shared memory and no block barriers,
// 8-byte (V = 2) loads of the planar operands.  The terms are added in the
// order of k_psi_finalize, so both give the same bits.
template <int V>
struct fvec {
  float v[V];
};
template <int V>
__device__ __forceinline__ fvec<V> ldv(const float* p) {
  fvec<V> r;
  if constexpr (V == 2) {
    const float2 t = __ldg(reinterpret_cast<const float2*>(p));
    r.v[0] = t.x;
    r.v[1] = t.y;
  } else {
    const float4 t = __ldg(reinterpret_cast<const float4*>(p));
    r.v[0] = t.x;
    r.v[1] = t.y;
    r.v[2] = t.z;
    r.v[3] = t.w;
  }
  return r;
}

template <int RMODE, int V>
__device__ __forceinline__ void psi_v4_job(const RhsDev<float>& d, const StageScalars& p, const float* __restrict__ ph,
                                           const float* __restrict__ pl, int64_t ldpsi, int64_t plane,
                                           const float* __restrict__ R1, int64_t ldR1, int npl,
                                           const float2* __restrict__ R2, const float2* __restrict__ ZA,
                                           const float2* __restrict__ ZB, float2* __restrict__ kpsi,
                                           const float2* __restrict__ R3, const float2* __restrict__ C0,
                                           int64_t first, int64_t stride) {
  const float ih = p.finv_hb;
  const float h = p.fh;
  const int n = d.n, nq = n / V, nc = d.nc, L = d.L;
  const int64_t total = (int64_t)d.N * nq;
  for (int64_t q = first; q < total; q += stride) {
    const int m = (int)(q / nq);
    const int i0 = (int)(q - (int64_t)m * nq) * V;
    const bool src = m < d.Ns;
    const int a = d.mode_lead[m];
    float2 xp = d.Xp[m];
    xp.x += p.fdelta[a];
    const float2 dgp = src ? d.dGP[m] : czero<float>();
    const int64_t o = (int64_t)m * ldpsi + i0;
    const fvec<V> pr = ldv<V>(ph + o), pim = ldv<V>(ph + o + plane);
    const fvec<V> lr = ldv<V>(pl + o), lim = ldv<V>(pl + o + plane);
    const int64_t a0 = (int64_t)m * ldR1 + i0, a1 = (int64_t)(d.N + m) * ldR1 + i0;
    fvec<V> r1r = ldv<V>(R1 + a0), r1i, r1x, r1y;
    if (RMODE == 1) {
      r1i = ldv<V>(R1 + a1);
    } else {  // columns [H_r | H_i]: (f[a0] - f[a1 + npl], f[a0 + npl] + f[a1])
      r1x = ldv<V>(R1 + a1 + npl);
      r1i = ldv<V>(R1 + a0 + npl);
      r1y = ldv<V>(R1 + a1);
    }
    const int64_t e0 = (int64_t)m * n + i0;
#pragma unroll
    for (int j = 0; j < V; ++j) {
      const float2 r2 = src ? R2[e0 + j] : czero<float>();
      float2 ps = make_float2(pr.v[j], pim.v[j]);
      const float2 pz = make_float2(lr.v[j], lim.v[j]);
      const float2 r1 = RMODE == 1 ? make_float2(r1r.v[j], r1i.v[j])
                                   : make_float2(r1r.v[j] - r1x.v[j], r1i.v[j] + r1y.v[j]);
      ps = cadd(ps, pz);
      float2 v = cscale(r1, ih);
      v = csub(v, cscale(cmul(xp, ps), ih));
      v = cadd(v, cmul(dgp, r2));
      const int i = i0 + j;
      if (R3) {
        v = cadd(v, cadd(R3[e0 + j], C0[e0 + j]));
      } else if (d.umap[i] >= 0) {  // a coupling orbital of some lead
        for (int b = 0; b < L; ++b) {
          const int k = d.colmap[b * n + i];
          if (k >= 0) {
            float2 z = ZA[((int64_t)b * d.N + m) * nc + k];
            if (src) z = cadd(z, ZB[((int64_t)b * d.Ns + m) * nc + k]);
            v = cadd(v, z);
            if (b == a) v = cadd(v, cmul(d.GLP[m], d.XI[(int64_t)m * nc + k]));
          }
        }
      }
      kpsi[e0 + j] = make_float2(h * v.y, -h * v.x);
    }
  }
}

template <int RMODE, int V>
__global__ void __launch_bounds__(256) k_psi_finalize_v4(const RhsDev<float> d, const StageParams* __restrict__ pp,
                                                         const float* __restrict__ ph, const float* __restrict__ pl,
                                                         int64_t ldpsi, int64_t plane, const float* __restrict__ R1,
                                                         int64_t ldR1, int npl, const float2* __restrict__ R2,
                                                         const float2* __restrict__ ZA, const float2* __restrict__ ZB,
                                                         float2* __restrict__ kpsi, const float2* __restrict__ R3,
                                                         const float2* __restrict__ C0) {
  const StageScalars p = load_params(pp);
  psi_v4_job<RMODE, V>(d, p, ph, pl, ldpsi, plane, R1, ldR1, npl, R2, ZA, ZB, kpsi, R3, C0,
                       blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

// The lead terms of k_sigma (blocks [0, nbl), after k_sigma_finalize) and the
// psi finalisation (the other blocks) of a mixed stage in one launch.
template <int RMODE, int V>
__global__ void __launch_bounds__(256) k_final_mixed(const RhsDev<float> d, const StageParams* __restrict__ pp,
                                                     int nbl, const float2* __restrict__ Pc, float2* __restrict__ ksig,
                                                     const float* __restrict__ ph, const float* __restrict__ pl,
                                                     int64_t ldpsi, int64_t plane, const float* __restrict__ R1,
                                                     int64_t ldR1, int npl, const float2* __restrict__ R2,
                                                     const float2* __restrict__ ZA, const float2* __restrict__ ZB,
                                                     float2* __restrict__ kpsi, const float2* __restrict__ R3,
                                                     const float2* __restrict__ C0) {
  const StageScalars p = load_params(pp);
  if ((int)blockIdx.x < nbl)
    sigma_leads_job<float>(d, p, Pc, ksig, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)nbl * blockDim.x);
  else
    psi_v4_job<RMODE, V>(d, p, ph, pl, ldpsi, plane, R1, ldR1, npl, R2, ZA, ZB, kpsi, R3, C0,
                         (blockIdx.x - nbl) * (int64_t)blockDim.x + threadIdx.x,
                         (int64_t)(gridDim.x - nbl) * blockDim.x);
}

constexpr int kPsiV = 2;  // columns per thread of k_psi_finalize_v4

template <typename T>
static bool psi_v4_ok(const RhsDev<T>& d, const void* psi, const void* psi_lo, int64_t ldpsi, const void* R1,
                      int64_t ldR1, int64_t plane, int rmode, int npl) {
  if (sizeof(T) != 4 || !plane || !psi_lo || (rmode != 1 && rmode != 2)) return false;
  if (d.n % kPsiV || ldpsi % kPsiV || plane % kPsiV || ldR1 % kPsiV || npl % kPsiV) return false;
  auto al = [](const void* q) { return ((uintptr_t)q & (4 * kPsiV - 1)) == 0; };
  return al(psi) && al(psi_lo) && al(R1);
}

bool final_mixed_ok(const RhsDev<float>& d, const float2* psi, const float2* psi_lo, int64_t ldpsi, const float2* R1,
                    int64_t ldR1, int64_t plane, int rmode, int npl) {
  return psi_v4_ok<float>(d, psi, psi_lo, ldpsi, R1, ldR1, plane, rmode, npl);
}

// The whole mixed finalisation in one launch: k_sigma with its lead terms
// (blocks [0, nb*nb), 32 x 32 tiles) and the psi finalisation (the other
// blocks); no dissipator.
template <int RMODE, int V>
__global__ void __launch_bounds__(256) k_final_all_mixed(const RhsDev<float> d, const StageParams* __restrict__ pp,
                                                         int nb, const float2* __restrict__ Tm, int64_t ldT, int tmode,
                                                         const float2* __restrict__ W, const float2* __restrict__ Pc,
                                                         float2* __restrict__ ksig, const float* __restrict__ ph,
                                                         const float* __restrict__ pl, int64_t ldpsi, int64_t plane,
                                                         const float* __restrict__ R1, int64_t ldR1, int npl,
                                                         const float2* __restrict__ R2, const float2* __restrict__ ZA,
                                                         const float2* __restrict__ ZB, float2* __restrict__ kpsi,
                                                         const float2* __restrict__ R3, const float2* __restrict__ C0) {
  const StageScalars p = load_params(pp);
  const int ntb = nb * nb;
  if ((int)blockIdx.x < ntb)
    sigma_tile_job<float, false>(blockIdx.x % nb, blockIdx.x / nb, threadIdx.x & 31, threadIdx.x >> 5, d, p, Tm, ldT,
                                 nullptr, ksig, tmode, npl, W, Pc);
  else
    psi_v4_job<RMODE, V>(d, p, ph, pl, ldpsi, plane, R1, ldR1, npl, R2, ZA, ZB, kpsi, R3, C0,
                         (blockIdx.x - ntb) * (int64_t)blockDim.x + threadIdx.x,
                         (int64_t)(gridDim.x - ntb) * blockDim.x);
}

int launch_final_all_mixed(const RhsDev<float>& d, const StageParams* p, const float2* Tm, int64_t ldT, int tmode,
                           const float2* W, const float2* Pc, float2* ksig, const float2* psi, const float2* psi_lo,
                           int64_t ldpsi, const float2* R1, int64_t ldR1, const float2* R2, const float2* ZA,
                           const float2* ZB, float2* kpsi, int64_t plane, int rmode, int npl, const float2* R3,
                           const float2* C0, cudaStream_t s) {
  ZG_REQUIRE(final_mixed_ok(d, psi, psi_lo, ldpsi, R1, ldR1, plane, rmode, npl), "operands not in the planar form");
  ZG_REQUIRE((R3 == nullptr) == (C0 == nullptr), "R3 and C0 come together");
  ZG_REQUIRE(tmode == 1 || tmode == 2, "planar T expected");
  const int nb = (d.n + 31) / 32;
  const int64_t total = (int64_t)d.N * (d.n / kPsiV);
  const int grid = nb * nb + grid_for(total, 256, 152 * 16);
  const float* ph = reinterpret_cast<const float*>(psi);
  const float* plo = reinterpret_cast<const float*>(psi_lo);
  const float* r1 = reinterpret_cast<const float*>(R1);
  const float2* P = d.nu > 0 && !W ? Pc : nullptr;
  if (rmode == 1)
    k_final_all_mixed<1, kPsiV><<<grid, 256, 0, s>>>(d, p, nb, Tm, ldT, tmode, W, P, ksig, ph, plo, ldpsi, plane, r1,
                                                     ldR1, npl, R2, ZA, ZB, kpsi, R3, C0);
  else
    k_final_all_mixed<2, kPsiV><<<grid, 256, 0, s>>>(d, p, nb, Tm, ldT, tmode, W, P, ksig, ph, plo, ldpsi, plane, r1,
                                                     ldR1, npl, R2, ZA, ZB, kpsi, R3, C0);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

int launch_final_mixed(const RhsDev<float>& d, const StageParams* p, const float2* Pc, float2* ksig,
                       const float2* psi, const float2* psi_lo, int64_t ldpsi, const float2* R1, int64_t ldR1,
                       const float2* R2, const float2* ZA, const float2* ZB, float2* kpsi, int64_t plane, int rmode,
                       int npl, const float2* R3, const float2* C0, cudaStream_t s) {
  ZG_REQUIRE(final_mixed_ok(d, psi, psi_lo, ldpsi, R1, ldR1, plane, rmode, npl), "operands not in the planar form");
  ZG_REQUIRE((R3 == nullptr) == (C0 == nullptr), "R3 and C0 come together");
  const int64_t tl = Pc && d.nu > 0 ? 2 * (int64_t)d.nu * d.n : 0;
  const int nbl = tl ? grid_for(tl, 256, 256) : 0;
  const int64_t total = (int64_t)d.N * (d.n / kPsiV);
  const int grid = nbl + grid_for(total, 256, 152 * 16);
  const float* ph = reinterpret_cast<const float*>(psi);
  const float* plo = reinterpret_cast<const float*>(psi_lo);
  const float* r1 = reinterpret_cast<const float*>(R1);
  if (rmode == 1)
    k_final_mixed<1, kPsiV><<<grid, 256, 0, s>>>(d, p, nbl, Pc, ksig, ph, plo, ldpsi, plane, r1, ldR1, npl, R2, ZA,
                                                 ZB, kpsi, R3, C0);
  else
    k_final_mixed<2, kPsiV><<<grid, 256, 0, s>>>(d, p, nbl, Pc, ksig, ph, plo, ldpsi, plane, r1, ldR1, npl, R2, ZA,
                                                 ZB, kpsi, R3, C0);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

template <typename T>
int launch_psi_finalize(const RhsDev<T>& d, const StageParams* p, const typename cx<T>::t* psi,
                        const typename cx<T>::t* psi_lo, int64_t ldpsi, const typename cx<T>::t* R1, int64_t ldR1,
                        const typename cx<T>::t* R2, const typename cx<T>::t* ZA, const typename cx<T>::t* ZB,
                        typename cx<T>::t* kpsi, cudaStream_t s, int64_t plane, int rmode, int npl,
                        const typename cx<T>::t* R3, const typename cx<T>::t* C0) {
  if (d.N == 0) return ZG_OK;
  ZG_REQUIRE(rmode >= 0 && rmode <= 2, "bad R1 layout %d", rmode);
  ZG_REQUIRE((R3 == nullptr) == (C0 == nullptr), "R3 and C0 come together");
  if constexpr (sizeof(T) == 4) {
    if (psi_v4_ok(d, psi, psi_lo, ldpsi, R1, ldR1, plane, rmode, npl)) {
      const int64_t total = (int64_t)d.N * (d.n / kPsiV);
      const int grid = grid_for(total, 256, 152 * 16);
      const float* ph = reinterpret_cast<const float*>(psi);
      const float* plo = reinterpret_cast<const float*>(psi_lo);
      const float* r1 = reinterpret_cast<const float*>(R1);
      if (rmode == 1)
        k_psi_finalize_v4<1, kPsiV><<<grid, 256, 0, s>>>(d, p, ph, plo, ldpsi, plane, r1, ldR1, npl, R2, ZA, ZB, kpsi,
                                                         R3, C0);
      else
        k_psi_finalize_v4<2, kPsiV><<<grid, 256, 0, s>>>(d, p, ph, plo, ldpsi, plane, r1, ldR1, npl, R2, ZA, ZB, kpsi,
                                                         R3, C0);
      ZG_CHECK_LAUNCH();
      count_launch();
      return ZG_OK;
    }
  }
  const size_t smem = R3 ? 0 : (size_t)(d.L + 1) * d.nc * sizeof(typename cx<T>::t);
  ZG_REQUIRE(smem <= 48 * 1024, "coupling width too large for the psi finalisation (%zu B)", smem);
  const int grid = d.N < 152 * 8 ? d.N : 152 * 8;
  k_psi_finalize<T><<<grid, 256, smem, s>>>(d, p, psi, psi_lo, ldpsi, R1, ldR1, R2, ZA, ZB, kpsi, plane, rmode, npl,
                                            R3, C0);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

// Non-orthogonal basis: K-concatenated operands of the two S^-1 products,
//   Qcat[i][a nc + k] = Pc[sourced rows of a][i][k] + Pc[free rows of a][i][k]   (n x L nc)
//   Zcat[m][b nc + k] = ZA[b][m][k] + (m sourced ? ZB[b][m][k] : 0)              (N x L nc)
template <typename T>
__global__ void k_nonorth_gather(const RhsDev<T> d, const typename cx<T>::t* __restrict__ Pc,
                                 const typename cx<T>::t* __restrict__ ZA, const typename cx<T>::t* __restrict__ ZB,
                                 typename cx<T>::t* __restrict__ Qcat, typename cx<T>::t* __restrict__ Zcat) {
  using C = typename cx<T>::t;
  const int64_t W = (int64_t)d.L * d.nc;
  const int64_t nq = (int64_t)d.n * W, tot = nq + (int64_t)d.N * W;
  GRID_STRIDE(q, tot) {
    if (q < nq) {
      const int64_t i = q / W, r = q - i * W;
      const int64_t a = r / d.nc, k = r - a * d.nc;
      const C p0 = Pc[((0 * d.L + a) * d.n + i) * d.nc + k];
      const C p1 = Pc[((1 * d.L + a) * d.n + i) * d.nc + k];
      Qcat[q] = cadd(p0, p1);
    } else {
      const int64_t q2 = q - nq;
      const int64_t m = q2 / W, r = q2 - m * W;
      const int64_t b = r / d.nc, k = r - b * d.nc;
      C z = ZA[(b * d.N + m) * d.nc + k];
      if (m < d.Ns) z = cadd(z, ZB[(b * d.Ns + m) * d.nc + k]);
      Zcat[q2] = z;
    }
  }
}

template <typename T>
int launch_nonorth_gather(const RhsDev<T>& d, const typename cx<T>::t* Pc, const typename cx<T>::t* ZA,
                          const typename cx<T>::t* ZB, typename cx<T>::t* Qcat, typename cx<T>::t* Zcat,
                          cudaStream_t s) {
  const int64_t tot = ((int64_t)d.n + d.N) * d.L * d.nc;
  k_nonorth_gather<T><<<grid_for(tot, 256, 152 * 8), 256, 0, s>>>(d, Pc, ZA, ZB, Qcat, Zcat);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

// Omega stage derivative on one 64x64 tile whose rows belong to lead a and
// columns to lead b (Zandpack/mpi/zand:782-809):
//   k[m,l] = h sum_k G[m][b][k] U[l][k]              (term1, U = dGM * IXI)
//          + h sum_k V[m][k] conj(G[l][a][k])        (term2, V = dGP * XIT2)
//          + (i h/hbar)(X+_m + D_a - X-_l - D_b) Omega[m,l]
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1) k_omega(const RhsDev<T> d, const StageParams* __restrict__ pp, const OmTile* __restrict__ tiles,
                                               const typename cx<T>::t* __restrict__ G,
                                               const typename cx<T>::t* __restrict__ omA_in,
                                               const typename cx<T>::t* __restrict__ omB_in,
                                               typename cx<T>::t* __restrict__ omA_out,
                                               typename cx<T>::t* __restrict__ omB_out, int stationary) {
  const StageScalars p = load_params(pp);
  using C = typename cx<T>::t;
  const OmTile t = tiles[blockIdx.x];
  // K (the 2 n_c source terms) staged ZKO at a time, next stage prefetched into registers
  constexpr int ZKO = 16, RO = 64 * ZKO / 256;
  // padded rows: stores run along k (column-wise), which would otherwise hit one bank
  __shared__ C As[ZKO][64 + 1];
  __shared__ C Bs[ZKO][64 + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int nc = d.nc;
  const int colmode0 = (t.blk == 0 ? 0 : d.Ns) + t.col0;  // absolute mode of local column col0
  C acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = czero<T>();
  const int kbeg = t.term1 ? 0 : nc, kend = t.term2 ? 2 * nc : nc;
  const int64_t ld = t.blk == 0 ? d.Ns : d.Nf;
  const C* in = t.blk == 0 ? omA_in : omB_in;
  // FP32: the Omega tile of the diagonal term is copied to shared memory
  // (cp.async) while the source products run, instead of being waited for in
  // the epilogue
  extern __shared__ __align__(16) unsigned char om_smem[];
  C* Os = reinterpret_cast<C*>(om_smem);  // [64][64], FP32 only
  if (sizeof(T) == 4 && !stationary) {
    for (int q = tid; q < 64 * 64; q += 256) {
      const int r = q >> 6, c = q & 63;
      if (r < t.nrows && c < t.ncols) {
        const C* src = in + (int64_t)(t.row0 + r) * ld + t.col0 + c;
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(Os + q);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  C ra[RO], rb[RO];
  // operands of K index k for local row/column rr (zero outside the tile and K range)
#define ZG_OMEGA_FETCH(k0)                                                                  \
  _Pragma("unroll") for (int r = 0; r < RO; ++r) {                                          \
    const int idx = tid + 256 * r;                                                          \
    const int rr = idx / ZKO, k = (k0) + idx % ZKO;                                         \
    C av = czero<T>(), bv = czero<T>();                                                     \
    if (k < kend) {                                                                         \
      if (rr < t.nrows) {                                                                   \
        const int64_t m = t.row0 + rr;                                                      \
        av = k < nc ? G[(m * d.L + t.b) * nc + k] : d.V[m * nc + (k - nc)];                 \
      }                                                                                     \
      if (rr < t.ncols) {                                                                   \
        const int64_t l = colmode0 + rr;                                                    \
        bv = k < nc ? d.U[l * nc + k] : G[(l * d.L + t.a) * nc + (k - nc)];                 \
      }                                                                                     \
    }                                                                                       \
    ra[r] = av;                                                                             \
    rb[r] = bv;                                                                             \
  }
  ZG_OMEGA_FETCH(kbeg)
  for (int k0 = kbeg; k0 < kend; k0 += ZKO) {
#pragma unroll
    for (int r = 0; r < RO; ++r) {
      const int idx = tid + 256 * r;
      As[idx % ZKO][idx / ZKO] = ra[r];
      // K indices >= n_c take conj(G) (the second source term), conjugated here
      // rather than at the load so that the load is not waited for
      Bs[idx % ZKO][idx / ZKO] = k0 + idx % ZKO >= nc ? cconj(rb[r]) : rb[r];
    }
    __syncthreads();
    if (k0 + ZKO < kend) {
      ZG_OMEGA_FETCH(k0 + ZKO)
    }
#pragma unroll
    for (int kk = 0; kk < ZKO; ++kk) {
      C a[4], b[4];
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
  if (sizeof(T) == 4 && !stationary) {
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
  }
  const T sc = pv<T>(p.h_hb, p.fh_hb);
  const T h = pv<T>(p.h, p.fh);
  C* out = t.blk == 0 ? omA_out : omB_out;
  const T da = pv<T>(p.delta[t.a], p.fdelta[t.a]), db = pv<T>(p.delta[t.b], p.fdelta[t.b]);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = ty + 16 * i;
    if (r >= t.nrows) continue;
    const int64_t m = t.row0 + r;
    C xp = d.Xp[m];
    xp.x += da;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = tx + 16 * j;
      if (c >= t.ncols) continue;
      const int64_t l = colmode0 + c;
      C xm = d.Xm[l];
      xm.x += db;
      const int64_t e = m * ld + (t.col0 + c);
      if (stationary) {
        // dOmega/dt = 0: Omega = i hbar S / (X+ + D_a - X- - D_b)  (Zandpack/cmdtools/psinought:443-451)
        const C q = cdiv(acc[i][j], csub(xp, xm));
        out[e] = cx<T>::make(-pv<T>(p.hbar, p.fhbar) * q.y, pv<T>(p.hbar, p.fhbar) * q.x);
        continue;
      }
      const C om = sizeof(T) == 4 ? Os[r * 64 + c] : in[e];
      const C dd = cmul(csub(xp, xm), om);  // (X+ - X-) Omega
      // (i h/hbar) dd = sc * (-dd.y, dd.x)
      C v = cscale(acc[i][j], h);
      v.x -= sc * dd.y;
      v.y += sc * dd.x;
      out[e] = v;
    }
  }
#undef ZG_OMEGA_FETCH
}

template <typename T>
int launch_omega(const RhsDev<T>& d, const StageParams* p, const OmTile* tiles, int ntiles, const typename cx<T>::t* G,
                 const typename cx<T>::t* omA_in, const typename cx<T>::t* omB_in, typename cx<T>::t* omA_out,
                 typename cx<T>::t* omB_out, cudaStream_t s, int stationary) {
  if (ntiles == 0) return ZG_OK;
  const int smem = sizeof(T) == 4 ? 64 * 64 * (int)sizeof(typename cx<T>::t) : 0;
  if (smem > 0) {
    static std::atomic<bool> configured[64];
    int dev = 0;
    ZG_CHECK_CUDA(cudaGetDevice(&dev));
    if (dev < 64 && !configured[dev].load()) {
      ZG_CHECK_CUDA(cudaFuncSetAttribute(k_omega<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      configured[dev] = true;
    }
  }
  k_omega<T><<<ntiles, 256, smem, s>>>(d, p, tiles, G, omA_in, omB_in, omA_out, omB_out, stationary);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

// ========================================================= H(t), operands
// Ht = H0 + dH, dH = uploaded matrix or U*diag(Re sigma_ii - 0.5)
__global__ void k_build_ht(int n, const double2* __restrict__ H0, const double2* __restrict__ sig,
                           const double2* __restrict__ dH, int dH_mode, double U, double2* __restrict__ Ht,
                           const double2* __restrict__ Sm1) {
  const int64_t nn = (int64_t)n * n;
  GRID_STRIDE(e, nn) {
    double2 v = H0[e];
    if (dH_mode == ZG_DH_MATRIX) v = cadd(v, dH[e]);
    const int i = (int)(e / n), j = (int)(e % n);
    if (dH_mode == ZG_DH_HUBBARD) {
      if (Sm1) {  // S^-1 diag(u): column j of S^-1 times u_j (Zandpack/mpi/nozand:1075-1083)
        const double u = U * (sig[(int64_t)j * n + j].x - 0.5);
        v.x += Sm1[e].x * u;
        v.y += Sm1[e].y * u;
      } else if (i == j) {
        v.x += U * (sig[e].x - 0.5);
      }
    }
    Ht[e] = v;
  }
}

int launch_build_ht(int n, const double2* H0, const double2* sig, const double2* dH, int dH_mode, double U,
                    double2* Ht, cudaStream_t s, const double2* Sm1) {
  int64_t nn = (int64_t)n * n;
  k_build_ht<<<grid_for(nn, 256, 152 * 8), 256, 0, s>>>(n, H0, sig, dH, dH_mode, U, Ht, Sm1);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

__device__ __forceinline__ void split_tf32_r(float v, float& hi, float& lo) {
  uint32_t h, l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
  const float r = v - __uint_as_float(h);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(r));
  hi = __uint_as_float(h);
  lo = __uint_as_float(l);
}

// H(t) element (r, c) in FP64 (r, c < n)
__device__ __forceinline__ double2 ht_element(int n, int r, int c, const double2* __restrict__ H0,
                                              const float2* __restrict__ sig32, const double2* __restrict__ dH,
                                              int dH_mode, double U, const double2* __restrict__ Sm1) {
  double2 v = H0[(int64_t)r * n + c];
  if (dH_mode == ZG_DH_MATRIX) v = cadd(v, dH[(int64_t)r * n + c]);
  if (dH_mode == ZG_DH_HUBBARD) {
    if (Sm1) {  // column c of S^-1 scaled by the Hubbard term of orbital c
      const double u = U * ((double)sig32[(int64_t)c * n + c].x - 0.5);
      const double2 sv = Sm1[(int64_t)r * n + c];
      v.x += sv.x * u;
      v.y += sv.y * u;
    } else if (r == c) {
      v.x += U * ((double)sig32[(int64_t)r * n + r].x - 0.5);
    }
  }
  return v;
}

__device__ __forceinline__ void put_split(float* __restrict__ hi, float* __restrict__ lo, int64_t o, int64_t off,
                                          float re, float im) {
  float a, b;
  split_tf32_r(re, a, b);
  hi[o] = a;
  lo[o] = b;
  split_tf32_r(im, a, b);
  hi[off + o] = a;
  lo[off + o] = b;
}

// Planar TF32 hi/lo operands of the two tensor-core GEMMs (np x np blocks):
// Ht rows [0, np) = Re H(t), rows [np, 2 np) = Im H(t); BS rows [0, np) =
// Re sigma^T, rows [np, 2 np) = Im sigma^T.  One 32x32 tile per block: sigma
// is read along its rows and transposed through shared memory.  HP (the
// H(t) part): 0 = every entry, 1 = the diagonal only (the blocks on the
// diagonal), 2 = none.  Padding (r or c >= n) is written as zero.
template <int HP>
__device__ __forceinline__ void operands_tile(int bx, int by, int n, int np, const double2* __restrict__ H0,
                                              const float2* __restrict__ sig32, const double2* __restrict__ dH,
                                              int dH_mode, double U, float* __restrict__ Hth,
                                              float* __restrict__ Htl, float* __restrict__ BSh,
                                              float* __restrict__ BSl, const double2* __restrict__ Sm1) {
  __shared__ float2 tile[32][33];  // tile[k][j] = sigma[c0 + k][r0 + j]
  const int64_t nn = (int64_t)np * np;
  const int r0 = by * 32, c0 = bx * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int k = ty; k < 32; k += 8) {
    const int row = c0 + k, col = r0 + tx;
    tile[k][tx] = (row < n && col < n) ? sig32[(int64_t)row * n + col] : czero<float>();
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int r = r0 + k, c = c0 + tx;
    if (r >= np || c >= np) continue;
    const int64_t o = (int64_t)r * np + c;
    const float2 sv = tile[tx][k];  // sigma[c][r]: row r of BS, K index c
    put_split(BSh, BSl, o, nn, sv.x, sv.y);
    if (HP == 0 || (HP == 1 && r == c)) {
      float hr = 0.f, hi = 0.f;
      if (r < n && c < n) {
        const double2 v = ht_element(n, r, c, H0, sig32, dH, dH_mode, U, Sm1);
        hr = (float)v.x;
        hi = (float)v.y;
      }
      put_split(Hth, Htl, o, nn, hr, hi);
    }
  }
}

template <int HP>
__global__ void __launch_bounds__(256) k_build_operands_mixed(int n, int np, const double2* __restrict__ H0,
                                                              const float2* __restrict__ sig32,
                                                              const double2* __restrict__ dH, int dH_mode, double U,
                                                              float* __restrict__ Hth, float* __restrict__ Htl,
                                                              float* __restrict__ BSh, float* __restrict__ BSl,
                                                              const double2* __restrict__ Sm1) {
  operands_tile<HP>(blockIdx.x, blockIdx.y, n, np, H0, sig32, dH, dH_mode, U, Hth, Htl, BSh, BSl, Sm1);
}

// The operand tiles (blocks [0, nb*nb)) and the gathers of the Omega and
// xi sigma^T products (the remaining blocks) of a mixed stage in one launch.
template <int HP>
__global__ void __launch_bounds__(256) k_prep_mixed(int n, int np, int nb, const double2* __restrict__ H0,
                                                    const float2* __restrict__ sig32, const double2* __restrict__ dH,
                                                    int dH_mode, double U, float* __restrict__ Hth,
                                                    float* __restrict__ Htl, float* __restrict__ BSh,
                                                    float* __restrict__ BSl, const double2* __restrict__ Sm1,
                                                    const RhsDev<float> d, const float2* __restrict__ psih,
                                                    const float2* __restrict__ psil, int64_t ldpsi,
                                                    float2* __restrict__ sigC, float2* __restrict__ G,
                                                    int64_t plane, const TcxOperands op) {
  const int ntb = nb * nb;
  if ((int)blockIdx.x < ntb) {
    operands_tile<HP>(blockIdx.x % nb, blockIdx.x / nb, n, np, H0, sig32, dH, dH_mode, U, Hth, Htl, BSh, BSl, Sm1);
  } else {
    const int tid = threadIdx.y * 32 + threadIdx.x;
    gathers_job<float>(d, sig32, psih, psil, ldpsi, sigC, G, plane, (int64_t)(blockIdx.x - ntb) * 256 + tid,
                       (int64_t)(gridDim.x - ntb) * 256, op);
  }
}

int launch_prep_mixed(int n, int np, const double2* H0, const float2* sig32, const double2* dH, int dH_mode,
                      double U, int h_part, float* Hth, float* Htl, float* BSh, float* BSl, const double2* Sm1,
                      const RhsDev<float>& d, const float2* psih, const float2* psil, int64_t ldpsi, float2* sigC,
                      float2* G, int64_t plane, cudaStream_t s, const TcxOperands& op) {
  ZG_REQUIRE(h_part >= 0 && h_part <= 2, "bad operand part %d", h_part);
  ZG_REQUIRE(!(Sm1 && dH_mode == ZG_DH_HUBBARD && h_part == 1), "the overlap's Hubbard term changes every entry");
  const int nb = (np + 31) / 32;
  const int64_t tot = (int64_t)d.L * d.n * d.nc + (int64_t)d.N * d.L * d.nc;
  const int gb = grid_for(tot, 256, 152 * 4);
  const dim3 grid(nb * nb + gb), block(32, 8);
  if (h_part == 0)
    k_prep_mixed<0><<<grid, block, 0, s>>>(n, np, nb, H0, sig32, dH, dH_mode, U, Hth, Htl, BSh, BSl, Sm1, d, psih,
                                           psil, ldpsi, sigC, G, plane, op);
  else if (h_part == 1)
    k_prep_mixed<1><<<grid, block, 0, s>>>(n, np, nb, H0, sig32, dH, dH_mode, U, Hth, Htl, BSh, BSl, Sm1, d, psih,
                                           psil, ldpsi, sigC, G, plane, op);
  else
    k_prep_mixed<2><<<grid, block, 0, s>>>(n, np, nb, H0, sig32, dH, dH_mode, U, Hth, Htl, BSh, BSl, Sm1, d, psih,
                                           psil, ldpsi, sigC, G, plane, op);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

int launch_build_operands_mixed(int n, int np, const double2* H0, const float2* sig32, const double2* dH, int dH_mode,
                                double U, int h_part, float* Hth, float* Htl, float* BSh, float* BSl, cudaStream_t s,
                                const double2* Sm1) {
  ZG_REQUIRE(h_part >= 0 && h_part <= 2, "bad operand part %d", h_part);
  ZG_REQUIRE(!(Sm1 && dH_mode == ZG_DH_HUBBARD && h_part == 1), "the overlap's Hubbard term changes every entry");
  const int nb = (np + 31) / 32;
  const dim3 grid(nb, nb), block(32, 8);
  if (h_part == 0)
    k_build_operands_mixed<0><<<grid, block, 0, s>>>(n, np, H0, sig32, dH, dH_mode, U, Hth, Htl, BSh, BSl, Sm1);
  else if (h_part == 1)
    k_build_operands_mixed<1><<<grid, block, 0, s>>>(n, np, H0, sig32, dH, dH_mode, U, Hth, Htl, BSh, BSl, Sm1);
  else
    k_build_operands_mixed<2><<<grid, block, 0, s>>>(n, np, H0, sig32, dH, dH_mode, U, Hth, Htl, BSh, BSl, Sm1);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

// W[m][k] *= i hbar / (lam_k - x_m), x_m = X+_m + Delta_{lead(m)}: the middle of
// the steady-state preconditioner  r -> i hbar r (H^T - x_m)^{-1}
__global__ void k_stationary_scale(int N, int n, const double2* __restrict__ Xp, const int* __restrict__ mode_lead,
                                   const double* __restrict__ delta, const double* __restrict__ lam, double hbar,
                                   double2* __restrict__ W) {
  const int64_t tot = (int64_t)N * n;
  GRID_STRIDE(e, tot) {
    const int m = (int)(e / n), k = (int)(e % n);
    double2 x = Xp[m];
    x.x += delta[mode_lead[m]];
    const double2 den = make_double2(lam[k] - x.x, -x.y);
    const double2 q = cdiv(W[e], den);
    W[e] = make_double2(-hbar * q.y, hbar * q.x);
  }
}

int launch_stationary_scale(int N, int n, const double2* Xp, const int* mode_lead, const double* delta,
                            const double* lam, double hbar, double2* W, cudaStream_t s) {
  const int64_t tot = (int64_t)N * n;
  if (tot == 0) return ZG_OK;
  k_stationary_scale<<<grid_for(tot, 256, 152 * 8), 256, 0, s>>>(N, n, Xp, mode_lead, delta, lam, hbar, W);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

// ----------------------------------------------------------- instantiate
#define ZG_INST(T)                                                                                                   \
  template int64_t plan_zgemm_batch<T>(GemmBatch<T>&);                                                               \
  template int launch_zgemm_batch<T>(GemmBatch<T>&, int64_t, cudaStream_t);                                         \
  template int launch_gathers<T>(const RhsDev<T>&, const cx<T>::t*, const cx<T>::t*, const cx<T>::t*, int64_t,      \
                                 cx<T>::t*, cx<T>::t*, cudaStream_t, int64_t);                                        \
  template int launch_sigma_finalize<T>(const RhsDev<T>&, const StageParams*, const cx<T>::t*, int64_t,              \
                                        const cx<T>::t*, const double2*, cx<T>::t*, cudaStream_t, int, int,           \
                                        const cx<T>::t*, bool);                                                      \
  template int launch_currents<T>(const RhsDev<T>&, const StageParams*, const cx<T>::t*, double*, cudaStream_t);     \
  template int launch_psi_finalize<T>(const RhsDev<T>&, const StageParams*, const cx<T>::t*, const cx<T>::t*,        \
                                      int64_t, const cx<T>::t*, int64_t, const cx<T>::t*, const cx<T>::t*,           \
                                      const cx<T>::t*, cx<T>::t*, cudaStream_t, int64_t, int, int, const cx<T>::t*,  \
                                      const cx<T>::t*);                                                              \
  template int launch_nonorth_gather<T>(const RhsDev<T>&, const cx<T>::t*, const cx<T>::t*, const cx<T>::t*,         \
                                        cx<T>::t*, cx<T>::t*, cudaStream_t);                                         \
  template int launch_omega<T>(const RhsDev<T>&, const StageParams*, const OmTile*, int, const cx<T>::t*,            \
                               const cx<T>::t*, const cx<T>::t*, cx<T>::t*, cx<T>::t*, cudaStream_t, int);
ZG_INST(double)
ZG_INST(float)

}  // namespace zg
