// Problem table of the complex tensor-core products (zg_tcx.cu).
#pragma once
#include <cuda.h>

#include "zg_kernels.cuh"

namespace zg {

#define ZG_TCX_MAPS 20
#define ZG_TCX_PROBS (5 * ZG_MAX_LEADS)

// One complex product D (M x Nv real columns, row stride ldd floats) =
// A' B'^T over K floats (a multiple of 32), in items of kchunk floats.
struct TcxProb {
  int amode;          // 0: A hi/lo (maps mapA, mapA+1); 1: raw FP32 A (map mapA); 2: planar psi hi/lo planes
  int mapA, mapB;     // tensor-map indices (B: hi at mapB, lo at mapB + 1)
  int a_row0;         // forms 0/1: first A row; form 2: first orbital (x coordinate)
  int a_k0;           // first K float of A (form 2: 2 x the first mode)
  int a_plane;        // form 2: row offset of the imaginary plane
  int b_row0, b_k0;   // first row and K float of B'
  int M, Nv, K, kchunk, nsplit, tiles_m, tiles_n;
  int item_begin;     // first work item of this problem
  float* D;
  long long ldd;
  float* ws;          // split-K partial tiles (nsplit > 1): [tile][split][128][BN]
  int* counters;      // one per 32-row slice of a tile and drain warp, zero between launches
  // a second operand pair for the K floats from kseg on (form 0 only):
  // A from map mapA2 at row a_row0_2, B' from map mapB2 at row b_row0_2,
  // both from K float 0
  int kseg, mapA2, mapB2, a_row0_2, b_row0_2;
  // epi 1: the Omega derivative of a block of Omega instead of a plain store:
  // out = h D + (i h/hbar)(X+_m + delta_la - X-_l - delta_lb) Omega_in, with
  // D = the source terms, row m = row_mode0 + row, column l = col_mode0 + col
  // (complex columns), Omega_in at om_in and out at om_out_base + om_out_off,
  // both with row stride ld_om complex
  int epi, ld_om, row_mode0, col_mode0, la, lb;
  const float2* om_in;
  long long om_out_off;
  // epi 1: the block of Omega_in is prefetched into shared memory with TMA
  // through map om_map (box BN floats x 128 rows, no swizzle) from float
  // column om_x0 and row om_y0 of that map; om_map < 0: read from om_in
  int om_map, om_x0, om_y0;
};

#define ZG_TCX_ITEMS 6144
#define ZG_TCX_GRID 160

struct TcxBatch {
  CUtensorMap maps[ZG_TCX_MAPS];
  TcxProb p[ZG_TCX_PROBS];
  // work items in the order CTAs claim them (most expensive first, ordered on
  // the host; item w is decoded against p[].item_begin).  CTA c starts with
  // item c (and c + gridDim.x when ahead2) and claims each further one near
  // the end of the previous one (two items ahead when ahead2): claim[0]
  // counts those claims and claim[1] the CTAs that are done; the last CTA
  // zeroes both, so they are zero between launches
  unsigned short items[ZG_TCX_ITEMS];
  int* claim;
  int nprob, nitems, bn, ahead2;
  int* err;
  // epilogue 1: stage parameters, X+ and X- of the modes (complex64), output base
  const StageParams* params;
  const float2* Xp;
  const float2* Xm;
  float2* om_out_base;
  // box of each tensor map (columns x rows; 0: map not set), for tcx_validate
  int box_cols[ZG_TCX_MAPS], box_rows[ZG_TCX_MAPS];
};
// the batch is the kernel's __grid_constant__ parameter
static_assert(sizeof(TcxBatch) <= 32764, "kernel parameter space");

// BN of the kernel for products with `ncols` real output columns per tile
// (0 when none fits)
int tcx_bn_for(int ncols);
// drain warps per tile of the BN kernels, the larger of the two kinds (split-K
// counters per tile)
inline int tcx_ndw(int bn) { return bn == 64 ? 8 : 4 * (bn / (bn % 64 == 0 ? 64 : 32)); }
// whether the BN kernel prefetches Omega tiles into shared memory (it fits)
bool tcx_has_omega_tile(int bn);
int tcx_launch(const TcxBatch& b, int grid, cudaStream_t s);
// tensor map `i` of a batch over a rows x cols fp32 array (row stride ld),
// with its box recorded for tcx_validate
int tcx_map(TcxBatch& b, int i, const void* base, int64_t rows, int64_t cols, int64_t ld, int box_rows,
            int box_cols, bool swizzle128);
// host checks before any launch: every map a problem reads is set and has the
// box the kernel expects for its role (so the expected transaction bytes
// match the copies), K split points and chunks are whole K blocks, split-K
// problems have their scratch, and the item lists are consistent
int tcx_validate(const TcxBatch& b);
// rows x cols fp32 row-major (row stride ld floats); box = box_cols x box_rows;
// swizzle128: the 128-byte swizzle of a 32-float K-major row, else no swizzle
int make_tmap_f32_box(CUtensorMap* map, const float* base, int64_t rows, int64_t cols, int64_t ld, int box_rows,
                      int box_cols, bool swizzle128);

}  // namespace zg
