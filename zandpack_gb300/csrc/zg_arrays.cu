// Array kernels behind two more names the reference's drivers import, on
// caller device buffers (complex128):
//
//   * the stage combination of Omega that leaves the Fermi x Fermi blocks
//     alone (step_omg_forward_nb_fermi_opti, Zandpack/func_step_forward.py:
//     112-139): out[e] = sum_t b_t Y[idx_t][e] for every element e whose row
//     pole x (axis 3 of a slot) and column pole x' (axis 6) are not both
//     Fermi poles; those elements of out are not written;
//   * the diagonal term of dOmega/dt (OuterSubtraction_hard_opti,
//     Zandpack/mpi_funcs.py:91-102): out[k,a,x,c,a',x',:] +=
//     (A[k,a,x,0] - B[k,a',x',0]) * C[k,a,x,c,a',x',:].
//
// Both are streaming kernels (HBM-bound): one grid-stride pass over the
// elements, the index decomposition done once per element.
#include "zg_kernels.cuh"

namespace zg {

#define GRID_STRIDE(e, count) \
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (count); e += (int64_t)gridDim.x * blockDim.x)

// slot shape (n2, n3, n4, n5, n6, n7, n8) = (k, a, x, c, a', x', c'); inner = n5*n6*n7*n8
__global__ void __launch_bounds__(256) k_combine_fermi_skip(const double2* __restrict__ Y, int64_t stride,
                                                            CombineCoefs cf, double2* __restrict__ out, int64_t count,
                                                            int n4, int64_t inner, int n7, int n8,
                                                            const uint8_t* __restrict__ fp_loc,
                                                            const uint8_t* __restrict__ fp_all) {
  GRID_STRIDE(e, count) {
    const int y = (int)((e / n8) % n7);
    const int l = (int)((e / inner) % n4);
    if (fp_loc[l] && fp_all[y]) continue;
    double2 acc = make_double2(0.0, 0.0);
    for (int t = 0; t < cf.n; ++t) {
      const double2 v = Y[cf.idx[t] * stride + e];
      acc.x = fma(cf.c[t], v.x, acc.x);
      acc.y = fma(cf.c[t], v.y, acc.y);
    }
    out[e] = acc;
  }
}

// out and C: (nk, na, nx, noT, NA, NX, NO); A: (nk, na, nx, lda_c); B: (nk, NA, NX, ldb_c)
__global__ void __launch_bounds__(256) k_outer_subtraction(const double2* __restrict__ A, const double2* __restrict__ B,
                                                           const double2* __restrict__ C, double2* __restrict__ out,
                                                           int64_t count, int na, int nx, int noT, int NA, int NX,
                                                           int NO, int lda_c, int ldb_c) {
  GRID_STRIDE(e, count) {
    int64_t r = e / NO;
    const int xx = (int)(r % NX); r /= NX;
    const int aa = (int)(r % NA); r /= NA;
    r /= noT;  // c
    const int x = (int)(r % nx); r /= nx;
    const int a = (int)(r % na); r /= na;
    const int64_t k = r;
    const double2 av = A[((k * na + a) * nx + x) * lda_c];
    const double2 bv = B[((k * NA + aa) * NX + xx) * ldb_c];
    const double2 d = make_double2(av.x - bv.x, av.y - bv.y);
    const double2 c = C[e];
    double2 o = out[e];
    o.x += d.x * c.x - d.y * c.y;
    o.y += d.x * c.y + d.y * c.x;
    out[e] = o;
  }
}

}  // namespace zg

using namespace zg;

extern "C" int zg_combine_fermi_skip_c128(const double* Y, int64_t slot_stride, int nslots, const double* b,
                                          const int32_t* idx, int nidx, double* out, const int64_t* shape7,
                                          const uint8_t* fp_loc, const uint8_t* fp_all, void* stream) {
  ZG_REQUIRE(b && shape7 && fp_loc && fp_all, "null argument");
  int64_t count = 1;
  for (int d = 0; d < 7; ++d) {
    ZG_REQUIRE(shape7[d] >= 0 && shape7[d] < (1LL << 31), "bad extent %lld on axis %d", (long long)shape7[d], d);
    count *= shape7[d];
  }
  ZG_REQUIRE(slot_stride >= count && (count == 0 || (Y && out)), "bad arguments");
  ZG_REQUIRE(nidx >= 0 && nidx <= ZG_MAX_STAGES + 1, "too many terms (%d)", nidx);
  if (count == 0) return ZG_OK;
  CombineCoefs cf;
  cf.n = 0;
  for (int t = 0; t < nidx; ++t) {
    const int j = idx[t];
    ZG_REQUIRE(j >= 0 && j < nslots, "index %d out of range", j);
    cf.idx[cf.n] = j;
    cf.c[cf.n] = b[j];
    ++cf.n;
  }
  // fp_loc (shape7[2] bytes) and fp_all (shape7[5] bytes) are device arrays
  const int64_t inner = shape7[3] * shape7[4] * shape7[5] * shape7[6];
  cudaStream_t s = (cudaStream_t)stream;
  k_combine_fermi_skip<<<grid_for(count, 256, 152 * 16), 256, 0, s>>>(
      (const double2*)Y, slot_stride, cf, (double2*)out, count, (int)shape7[2], inner, (int)shape7[5],
      (int)shape7[6], fp_loc, fp_all);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}

extern "C" int zg_outer_subtraction_c128(const double* A, int lda_c, const double* B, int ldb_c, const double* C,
                                         double* out, const int64_t* shape7, void* stream) {
  ZG_REQUIRE(shape7, "null argument");
  int64_t count = 1;
  for (int d = 0; d < 7; ++d) {
    ZG_REQUIRE(shape7[d] >= 0 && shape7[d] < (1LL << 31), "bad extent %lld on axis %d", (long long)shape7[d], d);
    count *= shape7[d];
  }
  if (count == 0) return ZG_OK;
  ZG_REQUIRE(A && B && C && out && lda_c >= 1 && ldb_c >= 1, "bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  k_outer_subtraction<<<grid_for(count, 256, 152 * 16), 256, 0, s>>>(
      (const double2*)A, (const double2*)B, (const double2*)C, (double2*)out, count, (int)shape7[1],
      (int)shape7[2], (int)shape7[3], (int)shape7[4], (int)shape7[5], (int)shape7[6], lda_c, ldb_c);
  ZG_CHECK_LAUNCH();
  count_launch();
  return ZG_OK;
}
