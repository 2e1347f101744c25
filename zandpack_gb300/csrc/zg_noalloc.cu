// Error norm of caller arrays without any device allocation.
//
// zg_terr2_c128 takes the buffer for its block partial sums from the
// stream-ordered allocator on every call.  Some callers of this library must
// not allocate device memory once they are running: a serving loop that has
// divided all of HBM among trajectory states at start-up, or a host program
// whose device memory belongs to another allocator.  For them an allocation
// in the middle of a time step could fail, or wait on work that has nothing
// to do with the call.  zg_terr2_c128_noalloc computes the same quantity with
// its partial sums in a fixed array that is part of the library image.
//
// The array is 1024 doubles (8 KiB) of static device memory on every GPU that
// loads the library, held until the process exits.  The reduction writes at
// most one partial per block of its grid (never more than 608 blocks) plus the
// result, so every size the allocating entry point accepts fits; the size is
// still checked before any launch and an oversize request is refused with
// ZG_EINVAL.
//
// All calls share the array.  Each call writes every word it later reads, so
// nothing has to start at zero, but two calls that run at the same time on
// the GPU (different streams, or different host threads) overwrite each
// other's partial sums and return wrong results: serialise them.
#include <mutex>

#include "zg_kernels.cuh"

namespace zg {

#define ZG_NOALLOC_SCRATCH_DOUBLES 1024
#define ZG_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_scratch[ZG_NOALLOC_SCRATCH_DOUBLES];

static std::mutex g_noalloc_mutex;
static double* g_noalloc_addr[ZG_NOALLOC_MAX_DEVICES] = {};

// Device address of the static scratch array on the current device.  The name
// g_noalloc_scratch in host code is only a host-side stand-in, so the address
// is looked up once per device (with that device current) and cached for the
// life of the process.  The cache does not survive cudaDeviceReset (the module
// is loaded again afterwards and the array may move): a program that resets
// the device must not call zg_terr2_c128_noalloc after the reset.
static int noalloc_scratch(double** out) {
  int dev = 0;
  ZG_CHECK_CUDA(cudaGetDevice(&dev));
  ZG_REQUIRE(dev >= 0 && dev < ZG_NOALLOC_MAX_DEVICES, "device %d beyond the %d supported", dev,
             ZG_NOALLOC_MAX_DEVICES);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_addr[dev] == nullptr) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_error("cudaGetSymbolAddress of the error-norm scratch failed on device %d: %s", dev,
                cudaGetErrorString(e));
      return ZG_ECUDA;
    }
    g_noalloc_addr[dev] = (double*)p;
  }
  *out = g_noalloc_addr[dev];
  return ZG_OK;
}

}  // namespace zg

using namespace zg;

extern "C" int zg_terr2_c128_noalloc(const double* Y, int64_t slot_stride, int nslots, const double* ct,
                                     int64_t count, double* result, void* stream) {
  ZG_REQUIRE(ct && result && count >= 0 && slot_stride >= count && (count == 0 || Y), "bad arguments");
  ZG_REQUIRE(nslots >= 1 && nslots <= ZG_MAX_STAGES + 1, "nslots %d out of range", nslots);
  CombineCoefs cf;
  cf.n = nslots;
  for (int j = 0; j < nslots; ++j) {
    cf.idx[j] = j;
    cf.c[j] = ct[j];
  }
  const int nb = terr2_nblocks(count);
  ZG_REQUIRE(nb + 1 <= ZG_NOALLOC_SCRATCH_DOUBLES,
             "error norm needs %d scratch doubles, the static array holds %d", nb + 1, ZG_NOALLOC_SCRATCH_DOUBLES);
  double* scratch = nullptr;
  ZG_TRY(noalloc_scratch(&scratch));
  cudaStream_t s = (cudaStream_t)stream;
  ZG_TRY(launch_terr2_partials_c128((const double2*)Y, slot_stride, cf, 0, count, scratch, nb, s));
  ZG_TRY(launch_reduce_partials(scratch, nb, 1, scratch + nb, s));
  ZG_CHECK_CUDA(cudaMemcpyAsync(result, scratch + nb, sizeof(double), cudaMemcpyDeviceToHost, s));
  ZG_CHECK_CUDA(cudaStreamSynchronize(s));
  return ZG_OK;
}
