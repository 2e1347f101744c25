// Tensor-core GEMM for the mixed-precision path: D = A * B^T in FP32 from
// split-TF32 operands on the 5th-generation tensor cores (tcgen05).
//
//   D[m][n] = sum_k (Ahi + Alo)[m][k] (Bhi + Blo)[n][k]
//           ~ Ahi.Bhi^T + Ahi.Blo^T + Alo.Bhi^T          ("3xTF32")
//
// A is M x K and B is N x K, both row-major with K contiguous (K-major), FP32
// arrays whose values are exact TF32 numbers (zg_split_tf32 produces them).
// Complex products are real GEMMs on planar operands (the real-part rows,
// then the imaginary-part rows; k_build_operands_mixed and the stage input in
// zg_rhs.cu / zg_flat.cu write them), so this kernel only sees real matrices.
//
// One CTA computes a BM x BN tile (BM = 128 TMEM lanes, BN = 256 or 128 fp32
// columns) with NDW = 4 * BN / 64 drain warps followed by two more warps:
//   * warp NDW, one elected thread: streams K blocks of Ahi, Alo, Bhi, Blo
//     with TMA (cp.async.bulk.tensor) into a STAGES-deep ring of shared-memory
//     buffers.  BN = 256: four stages of 16 floats along K (64-byte rows,
//     SWIZZLE_64B); BN = 128: three stages of 32 floats (SWIZZLE_128B);
//   * warp NDW + 1, one elected thread: owns the TMEM allocation and issues
//     tcgen05.mma (kind::tf32, M = 128, N = BN, K = 8) for the three products
//     of every K block into one of NACC = 512 / BN TMEM accumulator buffers
//     (all 512 columns), committing to the ring stage's "empty" barrier and,
//     after each K = TC_BK group, to the TMEM buffer's "full" barrier;
//   * warps 0 .. NDW-1: read each K = TC_BK group's partial sum from TMEM
//     (tcgen05.ld 32x32b; warp w takes TMEM lane quarter w % 4 and the 64
//     columns w / 4), add it into FP32 registers and release the buffer.
// The tensor core truncates inside its accumulation, so a single accumulator
// over K = 2048 drifts by ~1e-5 relative; per-group partials (TC_BK = 32
// floats) summed with round-to-nearest keep the product within 2e-6.  Groups
// of 64 are 2.5% faster at n = 1024, but their truncation bias accumulates
// along a trajectory: over 10 fs of the n = 1024 lattice (269 steps) the
// mixed path's sigma drifts from the FP64 one by 3.1e-7 and its currents by
// 1.5e-6, against 1.8e-7 and 6.1e-7 with groups of 32.
// Every wait on an mbarrier is bounded by a clock64 budget; on timeout the
// thread records an error code in *err and stops issuing, the MMA thread
// waits for its own MMAs, the producer for its copies in flight, and TMEM is
// freed before the CTA exits.
#include <cudaTypedefs.h>

#include "zg_tc_ptx.cuh"

namespace zg {

// Self-test of the bounded wait: one thread waits on an mbarrier that
// nothing arrives on, with the wait helper of the GEMM and a short budget.
// The wait must give up, record `code` and return; nothing else is in flight.
__global__ void k_wait_selftest(int* err, long long budget, int code) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  const uint32_t b = smem_u32(&bar);
  mbar_init(b, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  mbar_wait_budget(b, 0, err, code, budget);
}

// BK: K elements per shared-memory stage (32 or 16); a TMEM accumulation
// group always spans K = TC_BK (KPG stages), so the drain granularity and hence
// the accuracy do not depend on BK.
template <int BN, int STAGES, int BK>
struct TcCfg {
  static constexpr int A_BYTES = TC_BM * BK * 4;      // 16 KB at BK = 32
  static constexpr int B_BYTES = BN * BK * 4;         // 32 KB at BN = 256, BK = 32
  static constexpr int KPG = TC_BK / BK;              // stages per accumulation group
  static constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
  static constexpr int BAR_OFF = STAGES * STAGE_BYTES;
  static constexpr int SMEM = BAR_OFF + 256 + 1024;  // barriers, TMEM slot, alignment slack
  static constexpr int NACC = 512 / BN;               // accumulator buffers: all 512 TMEM columns
  static constexpr uint32_t TMEM_COLS = NACC * BN;
  static constexpr int DCOLS = 64;                    // columns of one drain warp
  static constexpr int NDW = 4 * BN / DCOLS;          // drain warps (four TMEM lane quarters)
  static constexpr int THREADS = 32 * (NDW + 2);      // + TMA warp + MMA warp
  // SMEM > 114 KB keeps one CTA per SM, so the 512-column allocation never waits
  static_assert(SMEM > 116 * 1024, "one CTA per SM is required by the full TMEM allocation");
  static_assert(NACC >= 2 && (NACC & (NACC - 1)) == 0, "accumulator buffer count");
};

// Warp roles (32 * (NDW + 2) threads): warps 0..NDW-1 drain the accumulators
// (TMEM lane quarter = warp % 4, 64-column part = warp / 4), warp NDW lane 0
// loads with TMA, warp NDW+1 lane 0 issues MMAs and that warp owns the TMEM
// allocation.  Each K group of TC_BK is accumulated alone in one of NACC TMEM
// buffers and added into FP32 registers (round to nearest), so the tensor
// core's truncating accumulation never spans more than 12 instructions.
template <int BN, int STAGES, int BK>
__global__ void __launch_bounds__(TcCfg<BN, STAGES, BK>::THREADS, 1)
    k_gemm_tf32x3(const __grid_constant__ CUtensorMap mAh, const __grid_constant__ CUtensorMap mAl,
                  const __grid_constant__ CUtensorMap mBh, const __grid_constant__ CUtensorMap mBl, float* __restrict__ D,
                  int M, int N, int K, long long ldd, int* err) {
  using C = TcCfg<BN, STAGES, BK>;
  constexpr int NACC = C::NACC, NDW = C::NDW, KPG = C::KPG;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t pad = (1024u - (raw & 1023u)) & 1023u;
  uint8_t* smem = smem_raw + pad;
  const uint32_t sbase = raw + pad;
  const uint32_t bar_full = sbase + C::BAR_OFF;        // STAGES x 8 B
  const uint32_t bar_empty = bar_full + 8 * STAGES;    // STAGES x 8 B
  const uint32_t bar_tfull = bar_empty + 8 * STAGES;   // NACC x 8 B
  const uint32_t bar_tempty = bar_tfull + 8 * NACC;    // NACC x 8 B
  const uint32_t bar_done = bar_tempty + 8 * NACC;     // 8 B
  uint32_t* tmem_slot = (uint32_t*)(smem + C::BAR_OFF + 16 * STAGES + 16 * NACC + 8);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * BN;
  const int nk = (K + BK - 1) / BK;       // shared-memory stages of BK
  const int ng = (nk + KPG - 1) / KPG;    // TMEM accumulation groups of K = TC_BK

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(bar_full + 8 * s, 1);
      mbar_init(bar_empty + 8 * s, 1);
    }
    for (int b = 0; b < NACC; ++b) {
      mbar_init(bar_tfull + 8 * b, 1);
      mbar_init(bar_tempty + 8 * b, 32 * NDW);  // every thread of the drain warps
    }
    mbar_init(bar_done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == NDW + 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(C::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == NDW) {
    if (lane == 0) {
      // ---------------- TMA producer
      int issued[STAGES];
      for (int s = 0; s < STAGES; ++s) issued[s] = 0;
      bool ok = true;
      for (int kb = 0; kb < nk && ok; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (uint32_t)(kb / STAGES) & 1u;
        ok = mbar_wait(bar_empty + 8 * s, ph ^ 1u, err, 1);
        if (!ok) break;
        const uint32_t st = sbase + s * C::STAGE_BYTES;
        mbar_expect_tx(bar_full + 8 * s, C::STAGE_BYTES);
        const int kx = kb * BK;
        tma_load_2d(st, &mAh, bar_full + 8 * s, kx, m0);
        tma_load_2d(st + C::A_BYTES, &mAl, bar_full + 8 * s, kx, m0);
        tma_load_2d(st + 2 * C::A_BYTES, &mBh, bar_full + 8 * s, kx, n0);
        tma_load_2d(st + 2 * C::A_BYTES + C::B_BYTES, &mBl, bar_full + 8 * s, kx, n0);
        issued[s] = kb / STAGES + 1;
      }
      if (!ok) {
        // wait (bounded) for the copies already in flight before leaving
        for (int s = 0; s < STAGES; ++s)
          if (issued[s] > 0) mbar_wait(bar_full + 8 * s, (uint32_t)(issued[s] - 1) & 1u, err, 4);
      }
    }
  } else if (warp == NDW + 1) {
    if (lane == 0) {
      // ---------------- MMA issuer
      constexpr uint32_t idesc = idesc_tf32(TC_BM, BN);
      bool ok = true;
      for (int g = 0; g < ng && ok; ++g) {
        const int b = g % NACC;
        if (!mbar_wait(bar_tempty + 8 * b, ((uint32_t)(g / NACC) & 1u) ^ 1u, err, 5)) break;
        const uint32_t d = tmem + (uint32_t)(b * BN);
        for (int q = 0; q < KPG; ++q) {
          const int kb = g * KPG + q;
          if (kb >= nk) break;
          const int s = kb % STAGES;
          const uint32_t ph = (uint32_t)(kb / STAGES) & 1u;
          if (!mbar_wait(bar_full + 8 * s, ph, err, 2)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t st = sbase + s * C::STAGE_BYTES;
          const uint32_t aH = st, aL = st + C::A_BYTES, bH = st + 2 * C::A_BYTES, bL = bH + C::B_BYTES;
#pragma unroll
          for (int j = 0; j < BK / 8; ++j) {
            const uint32_t off = j * 32;  // 8 tf32 = 32 bytes along K inside the swizzle row
            const uint32_t first = (q == 0 && j == 0) ? 0u : 1u;
            umma_tf32(d, umma_desc_k<BK>(aH + off), umma_desc_k<BK>(bH + off), idesc, first);
            umma_tf32(d, umma_desc_k<BK>(aH + off), umma_desc_k<BK>(bL + off), idesc, 1u);
            umma_tf32(d, umma_desc_k<BK>(aL + off), umma_desc_k<BK>(bH + off), idesc, 1u);
          }
          umma_commit(bar_empty + 8 * s);  // frees the smem buffer once these MMAs have read it
        }
        if (!ok) break;
        umma_commit(bar_tfull + 8 * b);  // hands the group's K = TC_BK sum to the drain warps
      }
      umma_commit(bar_done);
      mbar_wait(bar_done, 0, err, 6);  // every MMA issued above has completed
    }
  } else {
    // ---------------- drain warps: row m0 + 32*(warp%4) + lane, columns part*DCOLS ...
    const int quarter = warp & 3, part = warp >> 2;
    float acc[C::DCOLS];
#pragma unroll
    for (int i = 0; i < C::DCOLS; ++i) acc[i] = 0.f;
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    bool ok = true;
    for (int g = 0; g < ng; ++g) {
      const int b = g % NACC;
      ok = __all_sync(0xffffffffu, mbar_wait(bar_tfull + 8 * b, (uint32_t)(g / NACC) & 1u, err, 3));
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t t0 = tmem + lane_base + (uint32_t)(b * BN + part * C::DCOLS);
      // 32-column loads where registers allow (BN = 128: 320 threads), else 16
      constexpr int LDW = C::THREADS <= 320 ? 32 : 16;
#pragma unroll
      for (int c = 0; c < C::DCOLS; c += LDW) {
        uint32_t r0[LDW];
        if constexpr (LDW == 32) {
          TC_LD32(r0, t0 + c);
        } else {
          TC_LD16(r0, t0 + c);
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int i = 0; i < LDW; ++i) acc[c + i] += __uint_as_float(r0[i]);
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(bar_tempty + 8 * b);
    }
    const int row = m0 + quarter * 32 + lane;
    const int c0 = n0 + part * C::DCOLS;
    if (ok && row < M) {
      float* dst = D + (long long)row * ldd + c0;
      if (c0 + C::DCOLS <= N && (((uintptr_t)dst) & 15) == 0) {
#pragma unroll
        for (int i = 0; i < C::DCOLS; i += 4)
          *(float4*)(dst + i) = make_float4(acc[i], acc[i + 1], acc[i + 2], acc[i + 3]);
      } else {
#pragma unroll
        for (int i = 0; i < C::DCOLS; ++i)
          if (c0 + i < N) dst[i] = acc[i];
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == NDW + 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------- host side
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

static int tmap_encode_fn() {
  if (g_encode) return ZG_OK;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  ZG_CHECK_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
  if (fn == nullptr || q != cudaDriverEntryPointSuccess) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return ZG_ECUDA;
  }
  g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  return ZG_OK;
}

// rows x cols fp32 row-major (cols contiguous, row stride ld elements), box = box_k x box_rows,
// swizzled to match the tcgen05 descriptor of a box_k-float row (128 B or 64 B)
int make_tmap_f32(CUtensorMap* map, const float* base, int64_t rows, int64_t cols, int64_t ld, int box_rows,
                  int box_k) {
  ZG_TRY(tmap_encode_fn());
  ZG_REQUIRE(((uintptr_t)base & 15) == 0, "TMA base address must be 16-byte aligned");
  ZG_REQUIRE((ld * 4) % 16 == 0, "TMA row stride must be a multiple of 16 bytes");
  ZG_REQUIRE(rows > 0 && cols > 0, "empty TMA tensor");
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 4)};
  ZG_REQUIRE(box_k == 32 || box_k == 16, "TMA box of 16 or 32 floats along K");
  cuuint32_t box[2] = {(cuuint32_t)box_k, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE,
                        box_k == 32 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d) for %lld x %lld, ld %lld", (int)r, (long long)rows,
              (long long)cols, (long long)ld);
    return ZG_ECUDA;
  }
  return ZG_OK;
}

int make_tmap_f32_box(CUtensorMap* map, const float* base, int64_t rows, int64_t cols, int64_t ld, int box_rows,
                      int box_cols, bool swizzle128) {
  ZG_TRY(tmap_encode_fn());
  ZG_REQUIRE(((uintptr_t)base & 15) == 0, "TMA base address must be 16-byte aligned");
  ZG_REQUIRE((ld * 4) % 16 == 0, "TMA row stride must be a multiple of 16 bytes");
  ZG_REQUIRE(rows > 0 && cols > 0, "empty TMA tensor");
  ZG_REQUIRE(box_rows >= 1 && box_rows <= 256 && box_cols >= 4 && box_cols <= 256 && box_cols % 4 == 0,
             "TMA box %d x %d out of range", box_cols, box_rows);
  ZG_REQUIRE(!swizzle128 || box_cols == 32, "the 128-byte swizzle needs 32-float rows");
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 4)};
  cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE,
                        swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d) for %lld x %lld, ld %lld, box %d x %d", (int)r, (long long)rows,
              (long long)cols, (long long)ld, box_cols, box_rows);
    return ZG_ECUDA;
  }
  return ZG_OK;
}

template <int BN, int STAGES, int BK>
static int launch_tc(const TcGemm& g, cudaStream_t s) {
  using C = TcCfg<BN, STAGES, BK>;
  static std::atomic<bool> configured[64];
  int dev = 0;
  ZG_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && !configured[dev].load()) {
    ZG_CHECK_CUDA(
        cudaFuncSetAttribute(k_gemm_tf32x3<BN, STAGES, BK>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
    configured[dev] = true;
  }
  dim3 grid((g.N + BN - 1) / BN, (g.M + TC_BM - 1) / TC_BM);
  k_gemm_tf32x3<BN, STAGES, BK><<<grid, C::THREADS, C::SMEM, s>>>(g.Ah, g.Al, g.Bh, g.Bl, g.D, g.M, g.N, g.K,
                                                                  g.ldd, g.err);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

int tc_gemm_prepare(TcGemm& g, const float* Ah, const float* Al, const float* Bh, const float* Bl, int64_t lda,
                    int64_t ldb, float* D, int64_t ldd, int M, int N, int K, int* err) {
  ZG_REQUIRE(M > 0 && N > 0 && K > 0, "empty tensor-core GEMM");
  ZG_REQUIRE(N % 32 == 0, "tensor-core GEMM needs N a multiple of 32 (got %d)", N);
  // 256-wide tiles halve the shared-memory operand traffic per MMA (the
  // 128 x 128 x 8 MMA reads 8 KB of operands for 262 kflop) when there are
  // enough of them to fill the GPU; otherwise 128-wide tiles
  const int64_t tiles256 = (int64_t)((M + TC_BM - 1) / TC_BM) * ((N + 255) / 256);
  g.BN = tiles256 >= 152 ? 256 : 128;
  // 256-wide tiles take 16-float K stages: four 48 KB ring stages instead of
  // two 96 KB ones (measured 15 % faster at 4480 x 2048 x 2048); 128-wide
  // tiles keep three 64 KB stages of 32 floats (six 32 KB stages were slower)
  g.BK = g.BN == 256 ? 16 : 32;
  ZG_TRY(make_tmap_f32(&g.Ah, Ah, M, K, lda, TC_BM, g.BK));
  ZG_TRY(make_tmap_f32(&g.Al, Al, M, K, lda, TC_BM, g.BK));
  ZG_TRY(make_tmap_f32(&g.Bh, Bh, N, K, ldb, g.BN, g.BK));
  ZG_TRY(make_tmap_f32(&g.Bl, Bl, N, K, ldb, g.BN, g.BK));
  g.D = D; g.ldd = ldd; g.M = M; g.N = N; g.K = K; g.err = err;
  return ZG_OK;
}

int tc_gemm_launch(const TcGemm& g, cudaStream_t s) {
  return g.BN == 256 ? launch_tc<256, 4, 16>(g, s) : launch_tc<128, 3, 32>(g, s);
}

// hi = rna_tf32(x), lo = rna_tf32(x - hi)
__global__ void k_split_tf32(const float* __restrict__ x, float* __restrict__ hi, float* __restrict__ lo, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float v = x[i];
    uint32_t h, l;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(v));
    const float r = v - __uint_as_float(h);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(r));
    hi[i] = __uint_as_float(h);
    lo[i] = __uint_as_float(l);
  }
}

int launch_split_tf32(const float* x, float* hi, float* lo, int64_t n, cudaStream_t s) {
  if (n <= 0) return ZG_OK;
  k_split_tf32<<<grid_for(n, 256, 152 * 8), 256, 0, s>>>(x, hi, lo, n);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

}  // namespace zg

using namespace zg;

extern "C" int zg_split_tf32(const float* x, float* hi, float* lo, int64_t n, void* stream) {
  ZG_REQUIRE(n >= 0 && (n == 0 || (x && hi && lo)), "bad arguments");
  return launch_split_tf32(x, hi, lo, n, (cudaStream_t)stream);
}

extern "C" int zg_gemm_tf32x3(const float* Ah, const float* Al, const float* Bh, const float* Bl, float* D, int M,
                              int N, int K, void* stream) {
  ZG_REQUIRE(Ah && Al && Bh && Bl && D, "null argument");
  ZG_REQUIRE(K % 4 == 0, "K must be a multiple of 4 (16-byte rows for TMA)");
  cudaStream_t s = (cudaStream_t)stream;
  int* err = nullptr;
  ZG_CHECK_CUDA(cudaMallocAsync((void**)&err, sizeof(int), s));
  ZG_CHECK_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
  TcGemm g;
  int st = tc_gemm_prepare(g, Ah, Al, Bh, Bl, K, K, D, N, M, N, K, err);
  if (st == ZG_OK) st = tc_gemm_launch(g, s);
  int herr = 0;
  cudaError_t e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(err, s);
  if (st != ZG_OK) return st;
  if (e != cudaSuccess) { set_error("%s", cudaGetErrorString(e)); return ZG_ECUDA; }
  ZG_CHECK_CUDA(cudaStreamSynchronize(s));
  if (herr != 0) {
    set_error("tensor-core GEMM wait timed out (code %d)", herr);
    return ZG_ETIMEOUT;
  }
  return ZG_OK;
}

extern "C" int zg_wait_selftest(int device, long long budget_cycles) {
  ZG_REQUIRE(budget_cycles > 0 && budget_cycles <= 4LL * 1000 * 1000 * 1000, "budget out of range");
  ZG_CHECK_CUDA(cudaSetDevice(device));
  int* err = nullptr;
  ZG_CHECK_CUDA(cudaMalloc((void**)&err, sizeof(int)));
  cudaError_t e = cudaMemset(err, 0, sizeof(int));
  if (e == cudaSuccess) {
    k_wait_selftest<<<1, 32>>>(err, budget_cycles, 7);
    count_launch();
    e = cudaGetLastError();
  }
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(err);
  if (e != cudaSuccess) {
    set_error("%s", cudaGetErrorString(e));
    return ZG_ECUDA;
  }
  if (herr != 0) {
    set_error("bounded wait gave up as intended (code %d)", herr);
    return ZG_ETIMEOUT;
  }
  return ZG_OK;
}
