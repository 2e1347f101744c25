// Complex products of the mixed-precision right-hand side on the tcgen05
// tensor cores: the PI partials psi^T IXI (Zandpack/mpi/zand:91-110,363-366),
// the Omega xi products (:770-778), the xi sigma^T rows (:760-768) and,
// optionally, the Omega derivative (:782-809: its two rank-n_c source terms
// as products, the diagonal term in the epilogue).
//
// Every product is C = A B^T with complex A (M x K) and B (Nc x K).  On the
// tensor core it is the real GEMM
//
//   D (M x 2Nc) = A' (M x 2K) B'^T,   A'[m][2k], A'[m][2k+1] = Re, Im A[m][k]
//   B'[2c][2k] = Re B[c][k],   B'[2c][2k+1] = -Im B[c][k]
//   B'[2c+1][2k] = Im B[c][k], B'[2c+1][2k+1] = Re B[c][k]
//
// so that D[m][2c], D[m][2c+1] = Re, Im C[m][c]: A' is the interleaved
// complex storage itself and D is the interleaved complex result.  Products
// are 3xTF32 (Ahi.Bhi + Ahi.Blo + Alo.Bhi) with FP32 accumulation, each K
// block of 32 floats accumulated alone in TMEM and added into FP32 registers
// with round-to-nearest (the tensor core truncates inside its accumulation).
//
// The A operand reaches shared memory in one of three forms (per problem):
//   0: hi and lo parts, K-major (constants split once);
//   1: raw FP32, K-major (the Omega blocks of the stage input): converter
//      warps split each element into hi and lo in place;
//   2: the planar TF32 hi/lo parts of psi (rows = modes, columns = orbitals),
//      loaded as 16-mode x 128-orbital boxes: converter warps transpose and
//      interleave them into K-major A' rows (one orbital per row), so the
//      reduction over modes needs no transposed copy of psi in HBM.
// B' always arrives pre-split (constants, or built by the stage's operand
// kernel).
//
// One persistent CTA per SM claims work items (problem, 128-row tile,
// BN-column tile, K chunk) from a global counter, most expensive first, so
// that the CTAs finish together whatever the items cost; the producer claims
// and passes each item to the other roles through a small queue in shared
// memory.  Warp roles:
//   warp 0      one thread: claims items, TMA loads into a ring of 2 to 4
//               stages (as many as shared memory holds);
//   warp 1      one thread: tcgen05.mma issue, owns the TMEM allocation (up
//               to 8 accumulators of BN columns);
//   warps 2-5   converters (forms 1 and 2; form 0 passes through);
//   warps 6..   drain: TMEM -> registers, per-item sums, epilogue.
// Split-K items write FP32 partial tiles; the last drain warp to finish a
// 32-row slice of a tile (an atomic counter per slice) adds the partials in a
// fixed order and writes the result, so results are deterministic whichever
// CTA computed which item.  Waits on mbarriers are bounded like those of the
// 3xTF32 GEMM (zg_tc.cu): on timeout the error code is recorded, in-flight
// copies and MMAs are waited for (bounded) and TMEM is freed.
#include <vector>

#include "zg_tc_ptx.cuh"
#include "zg_tcx.cuh"

namespace zg {

template <int BN, bool OMG>
struct TcxCfg {
  static constexpr int A_BYTES = 128 * 32 * 4;   // one 128 x 32-float K-major tile
  static constexpr int RAW_BYTES = 4 * 16 * 128 * 4;  // four 16-mode x 128-orbital planes (form 2)
  static constexpr int B_BYTES = BN * 32 * 4;
  // stage: A region (A hi | A lo; the raw tile of form 1 and the planes of
  // form 2 land here and are converted in place) | B hi | B lo
  static constexpr int OFF_AL = A_BYTES, OFF_BH = 2 * A_BYTES, OFF_BL = OFF_BH + B_BYTES;
  static constexpr int STAGE_BYTES = OFF_BL + B_BYTES;
  // TMEM accumulator buffers of BN columns: as many as fit in the 512
  // columns (at most 8), so that the MMAs run ahead while the drain warps
  // finish an item's epilogue
  static constexpr int NACC = 512 / BN < 8 ? 512 / BN : 8;
  // columns per drain warp: 32 for the BN = 64 kernel with Omega blocks, whose
  // epilogues (the Omega derivative of every tile) then have eight warps
  static constexpr int DCOLS = (OMG && BN == 64) ? 32 : (BN % 64 == 0 ? 64 : 32);
  static constexpr int NDW = 4 * (BN / DCOLS);
  // epilogue staging: per drain warp a 32-row x 32-float tile (rows padded to
  // 36 floats), so that global loads and stores run along rows; and the Omega
  // tile of an item with epilogue 1 (128 rows x BN floats)
  static constexpr int STG_LD = 36;
  static constexpr int STG_WARP_FLOATS = 32 * STG_LD;
  static constexpr int STG_BYTES = NDW * STG_WARP_FLOATS * 4;
  static constexpr int OMT_BYTES = 128 * BN * 4;
  static constexpr int LIMIT = 232448 - 1024;  // dynamic shared memory less the alignment slack
  // barriers and the TMEM address (first 264 bytes), then at byte 320 the
  // item queue: QLEN "full" and "empty" barriers and the item numbers
  static constexpr int BAR_AREA = 512;
  static constexpr int QLEN = 8;
  static constexpr int fit(int stages, bool stg, bool omt) {
    return stages * STAGE_BYTES + BAR_AREA + (stg ? STG_BYTES : 0) + (omt ? OMT_BYTES : 0) <= LIMIT;
  }
  // the deepest ring that fits with staging and the Omega tile, else with
  // staging alone, else two stages with what fits
  // (OMG: the kernel of batches with Omega blocks; without them the room of
  // the Omega tile can hold another stage)
  static constexpr int STAGES = fit(4, true, OMG) ? 4 : fit(3, true, OMG) ? 3 : fit(3, true, false) ? 3 : 2;
  static constexpr bool STAGED = fit(STAGES, true, false);
  static constexpr bool HAS_OMT = OMG && STAGED && fit(STAGES, true, true);
  static constexpr int BAR_OFF = STAGES * STAGE_BYTES;
  static constexpr int STG_OFF = BAR_OFF + BAR_AREA;
  static constexpr int OMT_OFF = STG_OFF + (STAGED ? STG_BYTES : 0);
  static constexpr int SMEM = OMT_OFF + (HAS_OMT ? OMT_BYTES : 0) + 1024;
  static constexpr uint32_t TMEM_COLS = NACC * BN <= 256 ? (NACC * BN <= 128 ? 128 : 256) : 512;
  static constexpr int NCONV = 4;
  static constexpr int W_DRAIN = 2 + NCONV;
  static constexpr int THREADS = 32 * (W_DRAIN + NDW);
  static_assert(BN % 32 == 0 && BN >= 32 && BN <= 256, "BN");
  static_assert(SMEM <= 232448, "shared memory");
  static_assert(STAGES <= 4 && 24 * STAGES + 16 * NACC + 12 <= 240, "barrier area");
};

struct TcxItem {
  int prob, tm, tn, split;
};

__device__ __forceinline__ TcxItem tcx_item(const TcxBatch& b, int w) {
  // the last problem whose first item is <= w (binary search: each probe is
  // a dependent load from the parameter space)
  int lo = 0, hi = b.nprob - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (b.p[mid].item_begin <= w) lo = mid;
    else hi = mid - 1;
  }
  const int p = lo;
  const TcxProb& P = b.p[p];
  int r = w - P.item_begin;
  TcxItem it;
  it.prob = p;
  it.split = r % P.nsplit;
  r /= P.nsplit;
  it.tn = r % P.tiles_n;
  it.tm = r / P.tiles_n;
  return it;
}

// K blocks (of 32 floats) of an item
__device__ __forceinline__ void tcx_kblocks(const TcxProb& P, int split, int& kb0, int& nkb) {
  const int total = P.K / 32;
  const int per = P.kchunk / 32;
  kb0 = split * per;
  nkb = min(per, total - kb0);
}

__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t h;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  return h;
}

template <int BN, bool OMG>
__global__ void __launch_bounds__(TcxCfg<BN, OMG>::THREADS, 1) k_tcx(const __grid_constant__ TcxBatch batch) {
  using C = TcxCfg<BN, OMG>;
  constexpr int STAGES = C::STAGES, NACC = C::NACC, NDW = C::NDW;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t pad = (1024u - (raw & 1023u)) & 1023u;
  uint8_t* smem = smem_raw + pad;
  const uint32_t sbase = raw + pad;
  const uint32_t bar_full = sbase + C::BAR_OFF;        // STAGES: TMA landed
  const uint32_t bar_conv = bar_full + 8 * STAGES;     // STAGES: converters done
  const uint32_t bar_empty = bar_conv + 8 * STAGES;    // STAGES: MMAs read the stage
  const uint32_t bar_tfull = bar_empty + 8 * STAGES;   // NACC
  const uint32_t bar_tempty = bar_tfull + 8 * NACC;    // NACC
  const uint32_t bar_done = bar_tempty + 8 * NACC;
  const uint32_t bar_omt_full = sbase + C::BAR_OFF + 240;   // the Omega tile landed
  const uint32_t bar_omt_empty = sbase + C::BAR_OFF + 248;  // the drain warps read it
  const uint32_t bar_cread = sbase + C::BAR_OFF + 256;      // converters read a form-2 stage
  const uint32_t bar_qfull = sbase + C::BAR_OFF + 320;      // QLEN: the producer wrote an item number
  const uint32_t bar_qempty = bar_qfull + 8 * C::QLEN;      // QLEN: every role read it
  volatile int* q_ids = reinterpret_cast<volatile int*>(smem + C::BAR_OFF + 320 + 16 * C::QLEN);
  uint32_t* tmem_slot = (uint32_t*)(smem + C::BAR_OFF + 24 * STAGES + 16 * NACC + 8);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int* err = batch.err;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(bar_full + 8 * s, 1);
      mbar_init(bar_conv + 8 * s, C::NCONV);  // lane 0 of each converter warp
      mbar_init(bar_empty + 8 * s, 1);
    }
    for (int b = 0; b < NACC; ++b) {
      mbar_init(bar_tfull + 8 * b, 1);
      mbar_init(bar_tempty + 8 * b, NDW);  // lane 0 of each drain warp
    }
    mbar_init(bar_done, 1);
    mbar_init(bar_omt_full, 1);
    mbar_init(bar_omt_empty, NDW);
    mbar_init(bar_cread, C::NCONV);
    for (int q = 0; q < C::QLEN; ++q) {
      mbar_init(bar_qfull + 8 * q, 1);
      mbar_init(bar_qempty + 8 * q, 1 + C::NCONV + NDW);  // MMA thread, lane 0 of each warp
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(C::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // the descriptors of every map the problems read, into the descriptor
    // cache (one problem per lane, so that the reads of the problem table
    // from the parameter space overlap)
    for (int i = lane; i < batch.nprob; i += 32) {
      const TcxProb& P = batch.p[i];
      const int ids[5] = {P.mapA, P.mapB, P.kseg < P.K ? P.mapA2 : -1, P.kseg < P.K ? P.mapB2 : -1, P.om_map};
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        if (ids[j] < 0 || ids[j] >= ZG_TCX_MAPS) continue;
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&batch.maps[ids[j]]) : "memory");
        if (j < 4 && ids[j] + 1 < ZG_TCX_MAPS)
          asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&batch.maps[ids[j] + 1]) : "memory");
      }
    }
    __syncwarp();
    if (lane == 0) {
      // ---------------- TMA producer
      int issued[STAGES];
      for (int s = 0; s < STAGES; ++s) issued[s] = 0;
      bool ok = true;
      int kb_global = 0;
      // CTA c starts with item c.  With many short items per CTA (ahead2) it
      // also starts with item gridDim.x + c and claims each further item when
      // it starts on the item two places before it, so that the atomic's
      // round trip is hidden even behind short items; otherwise it claims the
      // next item three K blocks before the current one ends, so that no CTA
      // holds a long item it is far from starting.  claim[0] counts the
      // claims past the first (1 + ahead2) gridDim.x items
      const int G = (int)gridDim.x;
      const int base = batch.ahead2 ? 2 * G : G;
      int idx = blockIdx.x, idx_next = G + blockIdx.x;
      for (int seq = 0; ok; ++seq) {
        // pass the claimed item on once the queue has room (-1: none left)
        const int slot = seq % C::QLEN;
        ok = mbar_wait(bar_qempty + 8 * slot, ((uint32_t)(seq / C::QLEN) & 1u) ^ 1u, err, 22);
        if (!ok) break;
        const int w = idx < batch.nitems ? (int)batch.items[idx] : -1;
        if (batch.ahead2) {
          idx = idx_next;
          if (w >= 0) idx_next = base + atomicAdd(batch.claim, 1);
        }
        q_ids[slot] = w;
        mbar_arrive(bar_qfull + 8 * slot);
        if (w < 0) break;
        const TcxItem it = tcx_item(batch, w);
        const TcxProb& P = batch.p[it.prob];
        int kb0, nkb;
        tcx_kblocks(P, it.split, kb0, nkb);
        for (int q = 0; q < nkb; ++q, ++kb_global) {
          const int s = kb_global % STAGES;
          const uint32_t ph = (uint32_t)(kb_global / STAGES) & 1u;
          ok = mbar_wait(bar_empty + 8 * s, ph ^ 1u, err, 11);
          if (!ok) break;
          if (!batch.ahead2 && q == max(0, nkb - 3)) idx = base + atomicAdd(batch.claim, 1);
          const uint32_t st = sbase + s * C::STAGE_BYTES;
          const uint32_t fb = bar_full + 8 * s;
          const int kx = (kb0 + q) * 32;  // K float offset inside the problem
          const bool seg2 = kx >= P.kseg;
          const int bytes_a = P.amode == 0 || seg2 ? 2 * C::A_BYTES : P.amode == 1 ? C::A_BYTES : C::RAW_BYTES;
          mbar_expect_tx(fb, bytes_a + 2 * C::B_BYTES);
          const CUtensorMap* mA = &batch.maps[seg2 ? P.mapA2 : P.mapA];
          if (seg2) {
            const int k2 = kx - P.kseg;
            tma_load_2d(st, mA, fb, k2, P.a_row0_2 + it.tm * 128);
            tma_load_2d(st + C::OFF_AL, mA + 1, fb, k2, P.a_row0_2 + it.tm * 128);
          } else if (P.amode == 0) {
            tma_load_2d(st, mA, fb, P.a_k0 + kx, P.a_row0 + it.tm * 128);
            tma_load_2d(st + C::OFF_AL, mA + 1, fb, P.a_k0 + kx, P.a_row0 + it.tm * 128);
          } else if (P.amode == 1) {
            tma_load_2d(st, mA, fb, P.a_k0 + kx, P.a_row0 + it.tm * 128);
          } else {
            // planes: rows = modes (16 per K block), columns = 128 orbitals
            const int x = P.a_row0 + it.tm * 128, mode = (P.a_k0 + kx) / 2;
            const uint32_t rb = st;  // the A region; converted in place
            tma_load_2d(rb, mA, fb, x, mode);
            tma_load_2d(rb + 8192, mA, fb, x, P.a_plane + mode);
            tma_load_2d(rb + 16384, mA + 1, fb, x, mode);
            tma_load_2d(rb + 24576, mA + 1, fb, x, P.a_plane + mode);
          }
          const CUtensorMap* mB = &batch.maps[seg2 ? P.mapB2 : P.mapB];
          const int bx = seg2 ? kx - P.kseg : P.b_k0 + kx;
          const int by = (seg2 ? P.b_row0_2 : P.b_row0) + it.tn * BN;
          tma_load_2d(st + C::OFF_BH, mB, fb, bx, by);
          tma_load_2d(st + C::OFF_BL, mB + 1, fb, bx, by);
          issued[s] = kb_global / STAGES + 1;
        }
      }
      if (!ok) {
        for (int s = 0; s < STAGES; ++s)
          if (issued[s] > 0) mbar_wait(bar_full + 8 * s, (uint32_t)(issued[s] - 1) & 1u, err, 14);
      }
      // this CTA claims no more; the last CTA to get here zeroes the counters
      // for the next launch (every claim of every CTA precedes its count)
      __threadfence();
      if (atomicAdd(batch.claim + 1, 1) == (int)gridDim.x - 1) {
        __threadfence();
        atomicExch(batch.claim, 0);
        atomicExch(batch.claim + 1, 0);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer: one TMEM buffer per K block
      constexpr uint32_t idesc = idesc_tf32(128, BN);
      bool ok = true;
      int kb_global = 0;
      for (int seq = 0; ok; ++seq) {
        const int slot = seq % C::QLEN;
        ok = mbar_wait(bar_qfull + 8 * slot, (uint32_t)(seq / C::QLEN) & 1u, err, 23);
        if (!ok) break;
        const int w = q_ids[slot];
        mbar_arrive(bar_qempty + 8 * slot);
        if (w < 0) break;
        const TcxItem it = tcx_item(batch, w);
        const TcxProb& P = batch.p[it.prob];
        int kb0, nkb;
        tcx_kblocks(P, it.split, kb0, nkb);
        for (int q = 0; q < nkb; ++q, ++kb_global) {
          const int b = kb_global % NACC;
          if (!mbar_wait(bar_tempty + 8 * b, ((uint32_t)(kb_global / NACC) & 1u) ^ 1u, err, 15)) {
            ok = false;
            break;
          }
          const int s = kb_global % STAGES;
          if (!mbar_wait(bar_conv + 8 * s, (uint32_t)(kb_global / STAGES) & 1u, err, 12)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t st = sbase + s * C::STAGE_BYTES;
          const uint32_t aH = st, aL = st + C::OFF_AL, bH = st + C::OFF_BH, bL = st + C::OFF_BL;
          const uint32_t d = tmem + (uint32_t)(b * BN);
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const uint32_t off = j * 32;
            umma_tf32(d, umma_desc_k<32>(aH + off), umma_desc_k<32>(bH + off), idesc, j == 0 ? 0u : 1u);
            umma_tf32(d, umma_desc_k<32>(aH + off), umma_desc_k<32>(bL + off), idesc, 1u);
            umma_tf32(d, umma_desc_k<32>(aL + off), umma_desc_k<32>(bH + off), idesc, 1u);
          }
          umma_commit(bar_empty + 8 * s);
          umma_commit(bar_tfull + 8 * b);
        }
      }
      umma_commit(bar_done);
      mbar_wait(bar_done, 0, err, 16);
    }
  } else if (warp < C::W_DRAIN) {
    // ---------------- converters (128 threads)
    const int ct = threadIdx.x - 64;
    bool ok = true;
    int kb_global = 0;
    int nform2 = 0;  // form-2 stages converted (phase of bar_cread)
    for (int seq = 0; ok; ++seq) {
      const int slot = seq % C::QLEN;
      ok = __all_sync(0xffffffffu, mbar_wait(bar_qfull + 8 * slot, (uint32_t)(seq / C::QLEN) & 1u, err, 24));
      if (!ok) break;
      const int w = q_ids[slot];
      __syncwarp();
      if (lane == 0) mbar_arrive(bar_qempty + 8 * slot);
      if (w < 0) break;
      const TcxItem it = tcx_item(batch, w);
      const TcxProb& P = batch.p[it.prob];
      int kb0, nkb;
      tcx_kblocks(P, it.split, kb0, nkb);
      for (int q = 0; q < nkb; ++q, ++kb_global) {
        const int s = kb_global % STAGES;
        ok = __all_sync(0xffffffffu, mbar_wait(bar_full + 8 * s, (uint32_t)(kb_global / STAGES) & 1u, err, 13));
        if (!ok) break;
        uint8_t* st = smem + s * C::STAGE_BYTES;
        const int amode = (kb0 + q) * 32 >= P.kseg ? 0 : P.amode;
        if (amode == 1) {
          // split in place: A hi overwrites the raw tile, A lo goes to its own tile
          float4* ah = reinterpret_cast<float4*>(st);
          float4* al = reinterpret_cast<float4*>(st + C::OFF_AL);
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int c = ct + 128 * j;
            const float4 v = ah[c];
            float4 h, l;
            h.x = __uint_as_float(tf32_rna(v.x)); l.x = __uint_as_float(tf32_rna(v.x - h.x));
            h.y = __uint_as_float(tf32_rna(v.y)); l.y = __uint_as_float(tf32_rna(v.y - h.y));
            h.z = __uint_as_float(tf32_rna(v.z)); l.z = __uint_as_float(tf32_rna(v.z - h.z));
            h.w = __uint_as_float(tf32_rna(v.w)); l.w = __uint_as_float(tf32_rna(v.w - h.w));
            ah[c] = h;
            al[c] = l;
          }
        } else if (amode == 2) {
          // row ct of A' (orbital ct of the tile): modes 0..15 as (re, im)
          // pairs, 128-byte rows in the SWIZZLE_128B pattern (16-byte chunk c
          // of row r at chunk c ^ (r % 8)).  The planes occupy the same 32 KB:
          // every converter thread reads its values first, all of them meet at
          // an mbarrier (bounded wait), then the rows are written in place.
          const float* rp = reinterpret_cast<const float*>(st);
          float4 v[2][8];
#pragma unroll
          for (int part = 0; part < 2; ++part) {  // 0: hi, 1: lo
            const float* re = rp + part * 4096;
            const float* im = re + 2048;
#pragma unroll
            for (int c = 0; c < 8; ++c)
              v[part][c] = make_float4(re[(2 * c) * 128 + ct], im[(2 * c) * 128 + ct], re[(2 * c + 1) * 128 + ct],
                                       im[(2 * c + 1) * 128 + ct]);
          }
          __syncwarp();
          if (lane == 0) mbar_arrive(bar_cread);
          ok = __all_sync(0xffffffffu, mbar_wait(bar_cread, (uint32_t)nform2 & 1u, err, 21));
          ++nform2;
          if (!ok) break;
#pragma unroll
          for (int part = 0; part < 2; ++part) {
            uint8_t* dst = st + (part ? C::OFF_AL : 0) + ct * 128;
#pragma unroll
            for (int c = 0; c < 8; ++c) *reinterpret_cast<float4*>(dst + ((c ^ (ct & 7)) << 4)) = v[part][c];
          }
        }
        // generic-proxy writes to shared memory, read next by the tensor core
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(bar_conv + 8 * s);
      }
    }
  } else {
    // ---------------- drain warps: TMEM lane quarter (warp % 4), columns part * DCOLS
    const int dw = warp - C::W_DRAIN;
    const int quarter = warp & 3, part = dw >> 2;
    const int row_in_tile = quarter * 32 + lane;
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    float acc[C::DCOLS];
    bool ok = true;
    int kb_global = 0;
    int nom = 0;             // Omega tiles prefetched so far (all drain threads count them)
    bool omt_pending = false;  // lane 0 of drain warp 0: a tile load not yet waited for
    for (int seq = 0; ok; ++seq) {
      const int slot = seq % C::QLEN;
      ok = __all_sync(0xffffffffu, mbar_wait(bar_qfull + 8 * slot, (uint32_t)(seq / C::QLEN) & 1u, err, 25));
      if (!ok) break;
      const int w = q_ids[slot];
      __syncwarp();
      if (lane == 0) mbar_arrive(bar_qempty + 8 * slot);
      if (w < 0) break;
      const TcxItem it = tcx_item(batch, w);
      const TcxProb& P = batch.p[it.prob];
      int kb0, nkb;
      tcx_kblocks(P, it.split, kb0, nkb);
      const bool omt = C::HAS_OMT && P.epi == 1 && P.om_map >= 0;
      if (omt && dw == 0 && lane == 0) {
        // the block of Omega_in for this tile, loaded while its MMAs run; the
        // buffer is free once every drain thread has read the previous tile
        bool free_ok = nom == 0 || mbar_wait(bar_omt_empty, (uint32_t)(nom - 1) & 1u, err, 18);
        if (free_ok) {
          mbar_expect_tx(bar_omt_full, C::OMT_BYTES);
          tma_load_2d(sbase + C::OMT_OFF, &batch.maps[P.om_map], bar_omt_full, P.om_x0 + it.tn * BN,
                      P.om_y0 + it.tm * 128);
          omt_pending = true;
        }
      }
#pragma unroll
      for (int i = 0; i < C::DCOLS; ++i) acc[i] = 0.f;
      for (int q = 0; q < nkb; ++q, ++kb_global) {
        const int b = kb_global % NACC;
        ok = __all_sync(0xffffffffu, mbar_wait(bar_tfull + 8 * b, (uint32_t)(kb_global / NACC) & 1u, err, 17));
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t t0 = tmem + lane_base + (uint32_t)(b * BN + part * C::DCOLS);
#pragma unroll
        for (int c = 0; c < C::DCOLS; c += 32) {
          uint32_t r0[32];
          TC_LD32(r0, t0 + c);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int i = 0; i < 32; ++i) acc[c + i] += __uint_as_float(r0[i]);
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(bar_tempty + 8 * b);
      }
      if (!ok) break;
      // ---- epilogue of the item
      const int row = it.tm * 128 + row_in_tile;
      const int col0 = it.tn * BN + part * C::DCOLS;
      if constexpr (C::STAGED) {
        {
          // split K: this item's partial tile goes to its slot of the scratch
          // (row-major 128 x BN), written through the staging like the result
          const int tile = it.tm * P.tiles_n + it.tn;
          const bool part_out = P.epi == 0 && P.nsplit > 1;
          float* ws_tile = part_out ? P.ws + (long long)tile * P.nsplit * (128 * BN) : nullptr;
          float* ws_mine = part_out ? ws_tile + (long long)it.split * (128 * BN) : nullptr;
          // 32 columns at a time through the warp's staging tile: lane r writes
          // its row, then each pass stores two rows of 16 complex columns
          float* stg = reinterpret_cast<float*>(smem + C::STG_OFF) + dw * C::STG_WARP_FLOATS;
          const int rs = lane >> 4, cs = lane & 15;
          const float* omt_s = reinterpret_cast<const float*>(smem + C::OMT_OFF);
          float fh = 0.f, fhh = 0.f;
          float2 xp_own = make_float2(0.f, 0.f), xmv[C::DCOLS / 32];
          if (P.epi == 1) {
            // X+ of this lane's row (shared across lanes below) and X- of its
            // column in each 32-column chunk, loaded once per item
            const StageParams* pp = batch.params;
            fh = pp->fh;
            fhh = pp->fh_hb;
            if (row < P.M) xp_own = batch.Xp[P.row_mode0 + row];
            xp_own.x += pp->fdelta[P.la];
            const float db = pp->fdelta[P.lb];
#pragma unroll
            for (int ch = 0; ch < C::DCOLS / 32; ++ch) {
              const int col = (col0 >> 1) + ch * 16 + cs;
              xmv[ch] = 2 * col < P.Nv ? batch.Xm[P.col_mode0 + col] : make_float2(0.f, 0.f);
              xmv[ch].x += db;
            }
            if (omt) {
              ok = __all_sync(0xffffffffu, mbar_wait(bar_omt_full, (uint32_t)nom & 1u, err, 19));
              if (!ok) break;
              if (dw == 0 && lane == 0) omt_pending = false;
            }
          }
#pragma unroll
          for (int ch = 0; ch < C::DCOLS / 32; ++ch) {
            float4* wv = reinterpret_cast<float4*>(stg + lane * C::STG_LD);
#pragma unroll
            for (int j = 0; j < 8; ++j)
              wv[j] = make_float4(acc[32 * ch + 4 * j], acc[32 * ch + 4 * j + 1], acc[32 * ch + 4 * j + 2],
                                  acc[32 * ch + 4 * j + 3]);
            __syncwarp();
            const int col = (col0 >> 1) + ch * 16 + cs;  // complex column
#pragma unroll 4
            for (int itr = 0; itr < 16; ++itr) {
              const int rr = itr * 2 + rs;
              const int r = it.tm * 128 + quarter * 32 + rr;
              const float2 v = *reinterpret_cast<const float2*>(stg + rr * C::STG_LD + 2 * cs);
              const float2 xp = make_float2(__shfl_sync(0xffffffffu, xp_own.x, rr),
                                            __shfl_sync(0xffffffffu, xp_own.y, rr));
              if (r < P.M && 2 * col < P.Nv) {
                if (P.epi == 1) {
                  // the Omega derivative (Zandpack/mpi/zand:782-809; the diagonal
                  // term is Zandpack/mpi_funcs.py:91-102):
                  // h (sources) + (i h/hbar)(X+ - X-) Omega
                  const float2 dx = make_float2(xp.x - xmv[ch].x, xp.y - xmv[ch].y);
                  const float2 om =
                      omt ? *reinterpret_cast<const float2*>(omt_s + (quarter * 32 + rr) * BN +
                                                             2 * (col - it.tn * (BN / 2)))
                          : P.om_in[(long long)r * P.ld_om + col];
                  const float2 dd = make_float2(dx.x * om.x - dx.y * om.y, dx.x * om.y + dx.y * om.x);
                  batch.om_out_base[P.om_out_off + (long long)r * P.ld_om + col] =
                      make_float2(v.x * fh - fhh * dd.y, v.y * fh + fhh * dd.x);
                } else if (part_out) {
                  __stcg(reinterpret_cast<float2*>(ws_mine + (quarter * 32 + rr) * BN + 2 * (col - it.tn * (BN / 2))),
                         v);
                } else {
                  *reinterpret_cast<float2*>(P.D + (long long)r * P.ldd + 2 * col) = v;
                }
              }
            }
            __syncwarp();
          }
          if (omt) {
            __syncwarp();
            if (lane == 0) mbar_arrive(bar_omt_empty);
            ++nom;
          }
          if (part_out) {
            // the warp that completes this 32-row slice last (one counter per
            // slice; one release fence before the count, one acquire after)
            // adds the partials in split order and writes the result
            const int slice = tile * NDW + dw;
            __syncwarp();
            int prev = 0;
            if (lane == 0) {
              __threadfence();
              prev = atomicAdd(P.counters + slice, 1);
              if (prev == P.nsplit - 1) __threadfence();
            }
            prev = __shfl_sync(0xffffffffu, prev, 0);
            if (prev == P.nsplit - 1) {
              // the 16 row pairs of a 32-column chunk in flight at once, one
              // split after the other (partials added in split order)
#pragma unroll 1
              for (int ch = 0; ch < C::DCOLS / 32; ++ch) {
                const int col = (col0 >> 1) + ch * 16 + cs;
                const int lc = 2 * (col - it.tn * (BN / 2));
                const float* src = ws_tile + (quarter * 32 + rs) * BN + lc;
                float2 sum[16];
#pragma unroll
                for (int itr = 0; itr < 16; ++itr)
                  sum[itr] = __ldcg(reinterpret_cast<const float2*>(src + itr * 2 * BN));
                for (int sp = 1; sp < P.nsplit; ++sp) {
                  const float* sps = src + (long long)sp * (128 * BN);
                  float2 q[16];
#pragma unroll
                  for (int itr = 0; itr < 16; ++itr) q[itr] = __ldcg(reinterpret_cast<const float2*>(sps + itr * 2 * BN));
#pragma unroll
                  for (int itr = 0; itr < 16; ++itr) {
                    sum[itr].x += q[itr].x;
                    sum[itr].y += q[itr].y;
                  }
                }
#pragma unroll
                for (int itr = 0; itr < 16; ++itr) {
                  const int r = it.tm * 128 + quarter * 32 + itr * 2 + rs;
                  if (r < P.M && 2 * col < P.Nv)
                    *reinterpret_cast<float2*>(P.D + (long long)r * P.ldd + 2 * col) = sum[itr];
                }
              }
              __syncwarp();
              if (lane == 0) P.counters[slice] = 0;  // ready for the next launch
            }
          }
          continue;
        }
      }
      if (P.epi == 1) {
        // the Omega derivative (Zandpack/mpi/zand:782-809; the diagonal term
        // is Zandpack/mpi_funcs.py:91-102): h (sources) + (i h/hbar)(X+ - X-) Omega
        if (row < P.M) {
          const StageParams* pp = batch.params;
          const float h = pp->fh, sc = pp->fh_hb;
          const int m = P.row_mode0 + row;
          float2 xp = batch.Xp[m];
          xp.x += pp->fdelta[P.la];
          const float db = pp->fdelta[P.lb];
          const float2* in = P.om_in + (long long)row * P.ld_om;
          float2* out = batch.om_out_base + P.om_out_off + (long long)row * P.ld_om;
#pragma unroll
          for (int c2 = 0; c2 < C::DCOLS / 2; ++c2) {
            const int col = (col0 >> 1) + c2;
            if (2 * col >= P.Nv) continue;
            float2 xm = batch.Xm[P.col_mode0 + col];
            xm.x += db;
            const float2 dx = make_float2(xp.x - xm.x, xp.y - xm.y);
            const float2 om = in[col];
            const float2 dd = make_float2(dx.x * om.x - dx.y * om.y, dx.x * om.y + dx.y * om.x);
            out[col] = make_float2(acc[2 * c2] * h - sc * dd.y, acc[2 * c2 + 1] * h + sc * dd.x);
          }
        }
        continue;
      }
      if (P.nsplit == 1) {
        if (row < P.M) {
          float* dst = P.D + (long long)row * P.ldd + col0;
#pragma unroll
          for (int i = 0; i < C::DCOLS; ++i)
            if (col0 + i < P.Nv) dst[i] = acc[i];
        }
        continue;
      }
      // split K: every drain warp writes its 32-row slice of the partial tile;
      // the warp that completes a slice last (one counter per slice) adds the
      // partials in split order and writes the result
      const int tile = it.tm * P.tiles_n + it.tn;
      const int slice = tile * NDW + dw;
      const long long tile_ws = (long long)tile * P.nsplit * (128 * BN);
      const long long my = (long long)row_in_tile * BN + part * C::DCOLS;
      float* wsp = P.ws + tile_ws + (long long)it.split * (128 * BN) + my;
#pragma unroll
      for (int i = 0; i < C::DCOLS; i += 4)
        __stcg(reinterpret_cast<float4*>(wsp + i), make_float4(acc[i], acc[i + 1], acc[i + 2], acc[i + 3]));
      __syncwarp();
      int prev = 0;
      if (lane == 0) {
        __threadfence();
        prev = atomicAdd(P.counters + slice, 1);
        if (prev == P.nsplit - 1) __threadfence();
      }
      prev = __shfl_sync(0xffffffffu, prev, 0);
      if (prev == P.nsplit - 1) {
        if (row < P.M) {
          // every load of one partial slice in flight at once
          const float* src = P.ws + tile_ws + my;
          float4 sum[C::DCOLS / 4];
#pragma unroll
          for (int i = 0; i < C::DCOLS / 4; ++i) sum[i] = __ldcg(reinterpret_cast<const float4*>(src) + i);
          for (int sp = 1; sp < P.nsplit; ++sp) {
            const float4* q = reinterpret_cast<const float4*>(src + (long long)sp * (128 * BN));
            float4 v[C::DCOLS / 4];
#pragma unroll
            for (int i = 0; i < C::DCOLS / 4; ++i) v[i] = __ldcg(q + i);
#pragma unroll
            for (int i = 0; i < C::DCOLS / 4; ++i) {
              sum[i].x += v[i].x; sum[i].y += v[i].y; sum[i].z += v[i].z; sum[i].w += v[i].w;
            }
          }
          float* dst = P.D + (long long)row * P.ldd + col0;
#pragma unroll
          for (int i = 0; i < C::DCOLS / 4; ++i) {
            const float sv[4] = {sum[i].x, sum[i].y, sum[i].z, sum[i].w};
#pragma unroll
            for (int e = 0; e < 4; ++e)
              if (col0 + 4 * i + e < P.Nv) dst[4 * i + e] = sv[e];
          }
        }
        __syncwarp();
        if (lane == 0) P.counters[slice] = 0;  // ready for the next launch
      }
    }
    // a tile load still in flight (only after a timed-out wait): wait for it
    if (omt_pending) mbar_wait(bar_omt_full, (uint32_t)nom & 1u, err, 20);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------- host side
int make_tmap_f32_box(CUtensorMap* map, const float* base, int64_t rows, int64_t cols, int64_t ld, int box_rows,
                      int box_cols, bool swizzle128);

template <int BN, bool OMG>
static int launch_tcx_bn(const TcxBatch& b, int grid, cudaStream_t s) {
  using C = TcxCfg<BN, OMG>;
  static std::atomic<bool> configured[64];
  int dev = 0;
  ZG_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 64 && !configured[dev].load()) {
    ZG_CHECK_CUDA(cudaFuncSetAttribute(k_tcx<BN, OMG>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
    configured[dev] = true;
  }
  k_tcx<BN, OMG><<<grid, C::THREADS, C::SMEM, s>>>(b);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

int tcx_map(TcxBatch& b, int i, const void* base, int64_t rows, int64_t cols, int64_t ld, int box_rows,
            int box_cols, bool swizzle128) {
  ZG_REQUIRE(i >= 0 && i < ZG_TCX_MAPS, "tensor map index %d", i);
  ZG_TRY(make_tmap_f32_box(&b.maps[i], (const float*)base, rows, cols, ld, box_rows, box_cols, swizzle128));
  b.box_cols[i] = box_cols;
  b.box_rows[i] = box_rows;
  return ZG_OK;
}

int tcx_validate(const TcxBatch& b) {
  ZG_REQUIRE(b.nprob > 0 && b.nprob <= ZG_TCX_PROBS, "problem count %d", b.nprob);
  ZG_REQUIRE(b.nitems > 0 && b.nitems <= ZG_TCX_ITEMS, "item count %d", b.nitems);
  ZG_REQUIRE(tcx_bn_for(b.bn) == b.bn, "no kernel for BN %d", b.bn);
  auto has = [&](int m, int cols, int rows) {
    return m >= 0 && m + 1 < ZG_TCX_MAPS + 1 && b.box_cols[m] == cols && b.box_rows[m] == rows;
  };
  int items = 0;
  for (int i = 0; i < b.nprob; ++i) {
    const TcxProb& P = b.p[i];
    ZG_REQUIRE(P.K > 0 && P.K % 32 == 0 && P.kseg >= 0 && P.kseg <= P.K && P.kseg % 32 == 0,
               "problem %d: K %d, split point %d", i, P.K, P.kseg);
    ZG_REQUIRE(P.kchunk > 0 && P.kchunk % 32 == 0 && P.nsplit == (P.K + P.kchunk - 1) / P.kchunk,
               "problem %d: K chunk %d, %d splits", i, P.kchunk, P.nsplit);
    ZG_REQUIRE(P.tiles_m > 0 && P.tiles_n > 0 && P.M > 0 && P.M <= 128 * P.tiles_m && P.Nv > 0 &&
                   P.Nv <= b.bn * P.tiles_n,
               "problem %d: tiles", i);
    ZG_REQUIRE(P.item_begin == items, "problem %d: item range", i);
    items += P.tiles_m * P.tiles_n * P.nsplit;
    if (P.kseg > 0) {
      if (P.amode == 2)
        ZG_REQUIRE(has(P.mapA, 128, 16) && has(P.mapA + 1, 128, 16), "problem %d: planar A maps", i);
      else if (P.amode == 1)
        ZG_REQUIRE(has(P.mapA, 32, 128), "problem %d: raw A map", i);
      else
        ZG_REQUIRE(P.amode == 0 && has(P.mapA, 32, 128) && has(P.mapA + 1, 32, 128), "problem %d: A maps", i);
      ZG_REQUIRE(has(P.mapB, 32, b.bn) && has(P.mapB + 1, 32, b.bn), "problem %d: B maps", i);
      ZG_REQUIRE(P.a_k0 % 32 == 0 && P.b_k0 % 32 == 0, "problem %d: K offsets", i);
    }
    if (P.kseg < P.K) {
      ZG_REQUIRE(has(P.mapA2, 32, 128) && has(P.mapA2 + 1, 32, 128), "problem %d: second A maps", i);
      ZG_REQUIRE(has(P.mapB2, 32, b.bn) && has(P.mapB2 + 1, 32, b.bn), "problem %d: second B maps", i);
    }
    if (P.epi == 1) {
      ZG_REQUIRE(P.nsplit == 1 && P.om_in && b.params && b.Xp && b.Xm && P.ld_om > 0, "problem %d: Omega epilogue", i);
      if (P.om_map >= 0)
        ZG_REQUIRE(tcx_has_omega_tile(b.bn) && P.om_map < ZG_TCX_MAPS && b.box_cols[P.om_map] == b.bn &&
                       b.box_rows[P.om_map] == 128 && P.om_x0 % 4 == 0 && P.om_x0 >= 0 && P.om_y0 >= 0,
                   "problem %d: Omega tile map", i);
    } else {
      ZG_REQUIRE(P.D && P.ldd >= P.Nv, "problem %d: output", i);
      ZG_REQUIRE(P.nsplit == 1 || (P.ws && P.counters), "problem %d: split-K scratch", i);
    }
  }
  ZG_REQUIRE(items == b.nitems, "item total %d, table %d", items, b.nitems);
  ZG_REQUIRE(b.claim != nullptr, "item claim counters");
  // the claim order is a permutation of the items
  std::vector<char> seen(b.nitems, 0);
  for (int w = 0; w < b.nitems; ++w) {
    ZG_REQUIRE(b.items[w] < b.nitems && !seen[b.items[w]], "item %d in the claim order", w);
    seen[b.items[w]] = 1;
  }
  return ZG_OK;
}

bool tcx_has_omega_tile(int bn) {
  switch (bn) {
    case 32: return TcxCfg<32, true>::HAS_OMT;
    case 64: return TcxCfg<64, true>::HAS_OMT;
    case 128: return TcxCfg<128, true>::HAS_OMT;
    case 192: return TcxCfg<192, true>::HAS_OMT;
    default: return false;
  }
}

int tcx_bn_for(int ncols) {
  if (ncols <= 32) return 32;
  if (ncols <= 64) return 64;
  if (ncols <= 128) return 128;
  if (ncols <= 192) return 192;
  return 0;
}

int tcx_launch(const TcxBatch& b, int grid, cudaStream_t s) {
  if (b.nitems == 0) return ZG_OK;
  bool om = false;  // Omega blocks in the batch: the kernel with room for their tiles
  for (int i = 0; i < b.nprob; ++i) om = om || b.p[i].epi == 1;
  switch (b.bn * 2 + (om ? 1 : 0)) {
    case 64: return launch_tcx_bn<32, false>(b, grid, s);
    case 65: return launch_tcx_bn<32, true>(b, grid, s);
    case 128: return launch_tcx_bn<64, false>(b, grid, s);
    case 129: return launch_tcx_bn<64, true>(b, grid, s);
    case 256: return launch_tcx_bn<128, false>(b, grid, s);
    case 257: return launch_tcx_bn<128, true>(b, grid, s);
    case 384: return launch_tcx_bn<192, false>(b, grid, s);
    case 385: return launch_tcx_bn<192, true>(b, grid, s);
    default: set_error("complex tensor-core product: no kernel for %d columns", b.bn); return ZG_EINVAL;
  }
}

}  // namespace zg
