// Host runtime of libzandgpu: trajectory objects (device constants, the
// Runge-Kutta state slots, scratch), the per-stage launch sequence of the AME
// right-hand side in the FP64 and the mixed-precision form, and the
// extern "C" entry points declared in zandgpu.h.
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include <math.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <mutex>
#include <vector>

#include "zg_kernels.cuh"
#include "zg_tcx.cuh"

namespace zg {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

// Device memory of trajectories comes from one stream-ordered pool per device
// that keeps freed memory for the next trajectory: creating and destroying
// trajectories (the serving loop) then neither maps memory nor synchronises
// the device, as cudaMalloc/cudaFree would.  The pool is trimmed when the
// device's last trajectory is destroyed.
#define ZG_MAX_DEVICES 64
static std::mutex g_pool_mu;
static cudaMemPool_t g_pool[ZG_MAX_DEVICES] = {};
static int g_live[ZG_MAX_DEVICES] = {};

static int pool_for(int dev, cudaMemPool_t* out) {
  ZG_REQUIRE(dev >= 0 && dev < ZG_MAX_DEVICES, "device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (!g_pool[dev]) {
    cudaMemPoolProps props;
    memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    ZG_CHECK_CUDA(cudaMemPoolCreate(&g_pool[dev], &props));
    uint64_t keep = UINT64_MAX;
    ZG_CHECK_CUDA(cudaMemPoolSetAttribute(g_pool[dev], cudaMemPoolAttrReleaseThreshold, &keep));
  }
  *out = g_pool[dev];
  return ZG_OK;
}

// Pinned host blocks of the controller mirrors, recycled through a free list
// (cudaMallocHost/cudaFreeHost are slow and serialise concurrent threads).
static std::mutex g_pinned_mu;
static std::vector<void*> g_pinned_free;
static int pinned_get(size_t bytes, void** out) {
  {
    std::lock_guard<std::mutex> lk(g_pinned_mu);
    if (!g_pinned_free.empty()) {
      *out = g_pinned_free.back();
      g_pinned_free.pop_back();
      return ZG_OK;
    }
  }
  if (cudaMallocHost(out, bytes) != cudaSuccess) {
    set_error("pinned host allocation of %zu bytes failed", bytes);
    return ZG_ENOMEM;
  }
  return ZG_OK;
}
static void pinned_put(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_pinned_mu);
  g_pinned_free.push_back(p);
}

}  // namespace zg
struct zg_traj;
namespace zg {
static cudaStream_t traj_stream(const zg_traj* t);
static int traj_device(const zg_traj* t);

template <class T>
static int dalloc(const zg_traj* t, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaMemPool_t pool;
  ZG_TRY(pool_for(traj_device(t), &pool));
  cudaError_t e = cudaMallocFromPoolAsync((void**)p, count * sizeof(T), pool, traj_stream(t));
  if (e != cudaSuccess) {
    *p = nullptr;
    set_error("device allocation of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? ZG_ENOMEM : ZG_ECUDA;
  }
  return ZG_OK;
}

template <class T>
static int upload(T* dst, const void* src, size_t count, cudaStream_t s) {
  if (count == 0) return ZG_OK;
  ZG_CHECK_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyHostToDevice, s));
  return ZG_OK;
}

}  // namespace zg

using namespace zg;

// DOP54 (Zandpack/mpi_RK4pars_dev.py:118-149): A, B (column 7 = stored y), CT = b5 - b4, CH = [b5, 1]
static const double kDopA[7] = {0, 1. / 5, 3. / 10, 4. / 5, 8. / 9, 1, 1};
static const double kDopB[7][8] = {
    {0, 0, 0, 0, 0, 0, 0, 0},
    {1. / 5, 0, 0, 0, 0, 0, 0, 1},
    {3. / 40, 9. / 40, 0, 0, 0, 0, 0, 1},
    {44. / 45, -56. / 15, 32. / 9, 0, 0, 0, 0, 1},
    {19372. / 6561, -25360. / 2187, 64448. / 6561, -212. / 729, 0, 0, 0, 1},
    {9017. / 3168, -355. / 33, 46732. / 5247, 49. / 176, -5103. / 18656, 0, 0, 1},
    {35. / 384, 0, 500. / 1113, 125. / 192, -2187. / 6784, 11. / 84, 0, 1}};
static const double kB5[7] = {35. / 384, 0, 500. / 1113, 125. / 192, -2187. / 6784, 11. / 84, 0};
static const double kB4[7] = {5179. / 57600, 0, 7571. / 16695, 393. / 640, -92097. / 339200, 187. / 2100, 1. / 40};

// one pinned host block per trajectory: controller mirror, currents, error flag, attempt records
static const size_t kPinJ = (sizeof(DevCtl) + 63) / 64 * 64;
static const size_t kPinErr = kPinJ + (ZG_MAX_LEADS * sizeof(double) + 63) / 64 * 64;
static const size_t kPinRecs = kPinErr + 64;
static const size_t kPinnedBytes = kPinRecs + ZG_GRAPH_MAX_BATCH * sizeof(zg_attempt_rec);

struct zg_traj {
  int dev = 0;
  int precision = ZG_PREC_F64;
  cudaStream_t stream = nullptr;
  // mixed path: the H sigma tensor-core GEMM and the Omega derivative run on a
  // second stream while the SIMT products run on the first (fork and join
  // events; both are captured into the attempt graph as dependencies)
  cudaStream_t stream2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int n = 0, L = 0, N = 0, Ns = 0, Nf = 0, nc = 0;
  double hbar = 0;
  int64_t off_psi = 0, off_omA = 0, off_omB = 0, S = 0;
  std::vector<int64_t> s_start, f_start;
  // tableau
  int stages = 0;
  std::vector<double> A, B, CT, CH;  // B: stages x (stages+1)
  // device constants (FP64)
  double2 *H0 = nullptr, *Xp = nullptr, *Xm = nullptr, *GLP = nullptr, *dGP = nullptr, *XI = nullptr,
          *IXI = nullptr, *XIS = nullptr, *U = nullptr, *V = nullptr;
  int *mode_lead = nullptr, *lead_cols = nullptr, *colmap = nullptr;
  int *ucols = nullptr, *umap = nullptr;  // coupling orbitals of any lead
  int nu = 0;
  OmTile* tiles = nullptr;
  int ntiles = 0;
  // FP64 path: (stages+1) slots of S complex128, slot `stages` is y.
  // Mixed path: one FP64 slot (y) here, k slots in K32.
  double2* Y = nullptr;
  int y_slots = 0;
  double2* Ystage = nullptr;
  const double2* cur_in = nullptr;
  // FP64 scratch
  double2 *Ht = nullptr, *dH = nullptr, *T = nullptr, *Pc = nullptr, *sigC = nullptr, *G = nullptr, *R2 = nullptr,
          *ZA = nullptr, *ZB = nullptr;
  double *J = nullptr, *Jpart = nullptr, *partial = nullptr, *err = nullptr;
  int nblk_err = 0;
  bool dH_set = false;
  // mixed path: the H(t) tensor-core operands hold H0's off-diagonal entries
  // (built once; only the diagonal then changes with the Hubbard term)
  bool h_offdiag_ready = false;
  int h_diag_mode = -1;  // dH mode of the diagonal currently in the operands
  double2* dis = nullptr;  // dissipator of the coming stages (zg_set_dissipator)
  bool dis_on = false;
  // steady state (zg_stationary_*): eigenpairs of H, stage parameters, scratch
  double2 *st_V = nullptr, *st_Vc = nullptr, *st_W = nullptr;
  double* st_lam = nullptr;
  double* st_delta = nullptr;  // device copy of the lead biases
  StageParams st_p;
  int st_mode = ZG_DH_NONE;
  double st_U = 0.0;
  bool st_ready = false;
  // non-orthogonal basis (zg_set_overlap): S^-1, S^-1 H0, S^-1 dH, the
  // S^-1 rows/columns at the coupling orbitals (K operands of the two S^-1
  // products), the constant psi term, and the products' scratch
  bool nonorth = false;
  bool h0_real_orth = false;  // H0 itself is real (h0_real then also covers S^-1)
  bool sm1_real = false;
  bool dH_raw_real = false;
  std::vector<int> lead_cols_h, colmap_h;
  double2 *Sm1 = nullptr, *Hn0 = nullptr, *dHn = nullptr, *SmR = nullptr, *SmT = nullptr, *C0 = nullptr;
  double2 *Qcat = nullptr, *Wn = nullptr, *Zcat = nullptr, *R3 = nullptr;
  float2 *SmR32 = nullptr, *SmT32 = nullptr, *C0_32 = nullptr, *Qcat32 = nullptr, *Wn32 = nullptr,
         *Zcat32 = nullptr, *R3_32 = nullptr;
  // ---- mixed path
  int np = 0;  // n padded to a multiple of 16
  MixedLayout ml;
  float2 *Xp32 = nullptr, *Xm32 = nullptr, *GLP32 = nullptr, *dGP32 = nullptr, *XI32 = nullptr, *XIS32 = nullptr,
         *IXI32 = nullptr, *U32 = nullptr, *V32 = nullptr;
  float2 *y32 = nullptr, *K32 = nullptr, *stage32 = nullptr;
  int k_slots = 0;
  // mixed-path tensor-core operands, planar (real part rows, then imaginary
  // part rows np further), TF32 hi/lo: H(t) (A of H sigma, B of psi H^T) and
  // the transposed sigma (B of H sigma)
  float *Hth = nullptr, *Htl = nullptr, *BSh = nullptr, *BSl = nullptr;
  bool h0_real = false;   // H0 has no imaginary part
  bool dH_real = false;   // the uploaded dH matrix has no imaginary part
  TcGemm gTc, gR1c;       // complex H(t) forms of the two products (gT, gR1: real H(t))
  float2 *T32 = nullptr, *R1p = nullptr, *Pc32 = nullptr, *sigC32 = nullptr, *G32 = nullptr, *R2_32 = nullptr,
         *ZA32 = nullptr, *ZB32 = nullptr;
  double2 *conv64 = nullptr, *sig64 = nullptr;
  int* tc_err = nullptr;
  double2* ws64 = nullptr;
  float2* ws32 = nullptr;
  int64_t ws64_cap = 0, ws32_cap = 0;
  TcGemm gT, gR1;
  // mixed path: the PI partials, Omega xi and xi sigma^T products on the
  // tensor cores (zg_tcx.cu): problem table, the B' operand stack and the A
  // operand of xi sigma^T (constants, TF32 hi/lo), the per-stage B' of
  // xi sigma^T (embedded sigma columns, written by the operand kernel),
  // split-K partials and slice counters
  bool tcx_on = false;
  TcxBatch* tcx = nullptr;      // the products alone
  TcxBatch* tcx_all = nullptr;  // the products and the Omega derivative
  TcxBatch* tcx_om = nullptr;   // the Omega derivative alone, 64-column tiles
  int* tcx_claim = nullptr;     // item claim counters of the three batches
  int tcx_grid_all = 0, tcx_grid_om = 0;
  int prod_impl = 0;            // ZG_IMPL_*: which kernels compute the products and dOmega/dt
  int sched = ZG_SCHED_EARLY;   // ZG_SCHED_*: where the second stream forks off
  TcxOperands tcx_ops;
  // the Omega derivative in the same batch (epilogue 1 of zg_tcx.cu): the
  // constant operands U' (embedded) and V (TF32 hi/lo), and the per-stage psi
  // gathers Gt (A rows) and Gc (embedded conjugate B' rows)
  bool tco_on = false;
  float *Uh = nullptr, *Ul = nullptr, *Vh = nullptr, *Vl = nullptr, *Gth = nullptr, *Gtl = nullptr, *Gch = nullptr,
        *Gcl = nullptr;
  int tcx_grid = 0, ldx = 0;
  float *tcxBh = nullptr, *tcxBl = nullptr, *XIh = nullptr, *XIl = nullptr, *sigEh = nullptr, *sigEl = nullptr,
        *tcx_ws = nullptr;
  int* tcx_cnt = nullptr;
  // stage parameters read by the RHS kernels, and the device-side controller
  StageParams* d_params = nullptr;
  DevCtl* ctl = nullptr;
  DevCtl* ctl_host = nullptr;  // pinned mirror, written by the attempt graph
  double* J_host = nullptr;    // pinned
  int* tcerr_host = nullptr;   // pinned
  zg_attempt_rec* d_recs = nullptr;     // ZG_GRAPH_MAX_BATCH records of the current batch
  zg_attempt_rec* recs_host = nullptr;  // pinned
  bool capturing = false;
  bool counted = false;  // included in the live trajectories of its device
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  long long graph_kernels = 0;  // kernels of this library in one launch of the graph
  bool g_prepared = false;      // bias and dH mode of the graph are set
  zg_bias gbias;
  int g_dH_mode = ZG_DH_NONE;
  double g_U = 0.0;
  // event pairs recorded inside the attempt graph (region, begin, end)
  std::vector<int> gprof_r;
  std::vector<cudaEvent_t> gprof_b, gprof_e;
  // profiling: CUDA event pairs on `stream` around each region, collected at host syncs
  struct Prof {
    bool on = false;
    static const int RING = 64;
    cudaEvent_t b[ZG_PROF_REGIONS][RING], e[ZG_PROF_REGIONS][RING];
    int pending[ZG_PROF_REGIONS] = {};
    double ms[ZG_PROF_REGIONS] = {};
    long long cnt[ZG_PROF_REGIONS] = {};
    bool created = false;
  } prof;

  template <typename R>
  RhsDev<R> dev_view() const;
  double2* slot(int i) const { return Y + (int64_t)i * S; }
  float2* kslot(int i) const { return K32 + (int64_t)i * S; }
};

template <>
RhsDev<double> zg_traj::dev_view<double>() const {
  RhsDev<double> d;
  d.n = n; d.L = L; d.N = N; d.Ns = Ns; d.Nf = Nf; d.nc = nc;
  d.mode_lead = mode_lead; d.lead_cols = lead_cols; d.colmap = colmap;
  d.nu = nu; d.ucols = ucols; d.umap = umap;
  d.Xp = Xp; d.Xm = Xm; d.GLP = GLP; d.dGP = dGP; d.XI = XI; d.U = U; d.V = V;
  return d;
}
template <>
RhsDev<float> zg_traj::dev_view<float>() const {
  RhsDev<float> d;
  d.n = n; d.L = L; d.N = N; d.Ns = Ns; d.Nf = Nf; d.nc = nc;
  d.mode_lead = mode_lead; d.lead_cols = lead_cols; d.colmap = colmap;
  d.nu = nu; d.ucols = ucols; d.umap = umap;
  d.Xp = Xp32; d.Xm = Xm32; d.GLP = GLP32; d.dGP = dGP32; d.XI = XI32; d.U = U32; d.V = V32;
  return d;
}

namespace zg {
static cudaStream_t traj_stream(const zg_traj* t) { return t->stream; }
static int traj_device(const zg_traj* t) { return t->dev; }
}  // namespace zg

// ---------------------------------------------------------------- profiling
static void prof_collect(zg_traj* t) {
  auto& P = t->prof;
  if (!P.created) return;
  for (int r = 0; r < ZG_PROF_REGIONS; ++r) {
    for (int i = 0; i < P.pending[r]; ++i) {
      float ms = 0.f;
      if (cudaEventSynchronize(P.e[r][i]) == cudaSuccess && cudaEventElapsedTime(&ms, P.b[r][i], P.e[r][i]) == cudaSuccess) {
        P.ms[r] += ms;
        P.cnt[r] += 1;
      }
    }
    P.pending[r] = 0;
  }
}
// region r begins / ends on stream st (default: the trajectory's stream)
static void prof_begin(zg_traj* t, int r, cudaStream_t st = nullptr) {
  auto& P = t->prof;
  if (!P.on) return;
  if (!st) st = t->stream;
  if (t->capturing) {  // event record nodes inside the attempt graph
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
    t->gprof_r.push_back(r);
    t->gprof_b.push_back(e);
    return;
  }
  if (P.pending[r] == P.RING) prof_collect(t);
  cudaEventRecord(P.b[r][P.pending[r]], st);
}
static void prof_end(zg_traj* t, int r, cudaStream_t st = nullptr) {
  auto& P = t->prof;
  if (!P.on) return;
  if (!st) st = t->stream;
  if (t->capturing) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
    // pair with the latest unmatched begin of this region
    t->gprof_e.resize(t->gprof_b.size(), nullptr);
    for (size_t i = t->gprof_b.size(); i-- > 0;)
      if (t->gprof_r[i] == r && t->gprof_e[i] == nullptr) {
        t->gprof_e[i] = e;
        break;
      }
    return;
  }
  cudaEventRecord(P.e[r][P.pending[r]], st);
  P.pending[r] += 1;
}
// after a replay of the attempt graph: accumulate the regions it recorded
static void graph_prof_collect(zg_traj* t) {
  auto& P = t->prof;
  if (!P.on) return;
  for (size_t i = 0; i < t->gprof_b.size(); ++i) {
    if (i >= t->gprof_e.size() || !t->gprof_e[i]) continue;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, t->gprof_b[i], t->gprof_e[i]) == cudaSuccess) {
      P.ms[t->gprof_r[i]] += ms;
      P.cnt[t->gprof_r[i]] += 1;
    }
  }
}

static void drop_graph(zg_traj* t) {
  if (t->gexec) cudaGraphExecDestroy(t->gexec);
  if (t->graph) cudaGraphDestroy(t->graph);
  t->gexec = nullptr;
  t->graph = nullptr;
  t->graph_kernels = 0;
  for (auto e : t->gprof_b) cudaEventDestroy(e);
  for (auto e : t->gprof_e)
    if (e) cudaEventDestroy(e);
  t->gprof_r.clear();
  t->gprof_b.clear();
  t->gprof_e.clear();
}

// stream-ordered release of a trajectory buffer back to the pool
static void dfree(zg_traj* t, void* p) {
  if (p) cudaFreeAsync(p, t->stream);
}

static void free_traj(zg_traj* t) {
  if (!t) return;
  drop_graph(t);
  pinned_put(t->ctl_host);  // one block: ctl_host, J_host, tcerr_host, recs_host
  dfree(t, t->d_recs);
  dfree(t, t->d_params);
  dfree(t, t->ctl);
  if (t->prof.created)
    for (int r = 0; r < ZG_PROF_REGIONS; ++r)
      for (int i = 0; i < t->prof.RING; ++i) {
        cudaEventDestroy(t->prof.b[r][i]);
        cudaEventDestroy(t->prof.e[r][i]);
      }
  void* ptrs[] = {t->H0, t->Xp, t->Xm, t->GLP, t->dGP, t->XI, t->IXI, t->XIS, t->U, t->V, t->mode_lead,
                  t->lead_cols, t->colmap, t->tiles, t->Y, t->Ystage, t->Ht, t->dH, t->T, t->Pc, t->sigC,
                  t->G, t->R2, t->ZA, t->ZB, t->J, t->Jpart, t->partial, t->err, t->Xp32, t->Xm32, t->GLP32,
                  t->dGP32,
                  t->XI32, t->XIS32, t->IXI32, t->U32, t->V32, t->y32, t->K32, t->stage32, t->Hth, t->Htl,
                  t->BSh, t->BSl, t->T32, t->R1p, t->Pc32, t->sigC32, t->G32, t->R2_32, t->ZA32, t->ZB32,
                  t->conv64, t->sig64, t->tc_err, t->ws64, t->ws32, t->dis, t->ucols, t->umap,
                  t->st_V, t->st_Vc, t->st_W, t->st_lam, t->st_delta,
                  t->Sm1, t->Hn0, t->dHn, t->SmR, t->SmT, t->C0, t->Qcat, t->Wn, t->Zcat, t->R3,
                  t->SmR32, t->SmT32, t->C0_32, t->Qcat32, t->Wn32, t->Zcat32, t->R3_32,
                  t->tcxBh, t->tcxBl, t->XIh, t->XIl, t->sigEh, t->sigEl, t->tcx_ws, t->tcx_cnt, t->tcx_claim,
                  t->Uh, t->Ul, t->Vh, t->Vl, t->Gth, t->Gtl, t->Gch, t->Gcl};
  for (void* p : ptrs) dfree(t, p);
  delete t->tcx;
  delete t->tcx_all;
  delete t->tcx_om;
  if (t->stream2) {
    cudaStreamSynchronize(t->stream2);
    cudaStreamDestroy(t->stream2);
  }
  if (t->ev_fork) cudaEventDestroy(t->ev_fork);
  if (t->ev_join) cudaEventDestroy(t->ev_join);
  if (t->stream) {
    cudaStreamSynchronize(t->stream);
    cudaStreamDestroy(t->stream);
    bool trim = false;
    {
      std::lock_guard<std::mutex> lk(g_pool_mu);
      if (t->counted && --g_live[t->dev] == 0) trim = true;
    }
    cudaMemPool_t pool;
    if (trim && pool_for(t->dev, &pool) == ZG_OK) cudaMemPoolTrimTo(pool, 0);
  }
  delete t;
}

static int alloc_state(zg_traj* t, int stages) {
  const bool mixed = t->precision == ZG_PREC_MIXED;
  const int yslots = mixed ? 1 : stages + 1;
  if (!t->Y || t->y_slots != yslots) {
    dfree(t, t->Y);
    t->Y = nullptr;
    ZG_TRY(dalloc(t, &t->Y, (size_t)yslots * t->S));
    t->y_slots = yslots;
    ZG_CHECK_CUDA(cudaMemsetAsync(t->Y, 0, (size_t)yslots * t->S * sizeof(double2), t->stream));
  }
  if (mixed && (!t->K32 || t->k_slots != stages)) {
    dfree(t, t->K32);
    t->K32 = nullptr;
    ZG_TRY(dalloc(t, &t->K32, (size_t)stages * t->S));
    t->k_slots = stages;
    ZG_CHECK_CUDA(cudaMemsetAsync(t->K32, 0, (size_t)stages * t->S * sizeof(float2), t->stream));
  }
  return ZG_OK;
}

// y slot index inside Y: FP64 path keeps it after the k slots, mixed keeps only y
static double2* y64(const zg_traj* t) { return t->precision == ZG_PREC_MIXED ? t->Y : t->slot(t->stages); }

static int set_tableau_impl(zg_traj* t, int stages, const double* A, const double* B, const double* CT,
                            const double* CH) {
  ZG_REQUIRE(stages >= 1 && stages <= ZG_MAX_STAGES, "stages=%d out of range", stages);
  if (t->precision == ZG_PREC_MIXED) {
    // the mixed path applies y with weight 1 implicitly
    ZG_REQUIRE(CH[stages] == 1.0, "mixed precision needs CH[stages] == 1");
    for (int i = 1; i < stages; ++i) ZG_REQUIRE(B[(size_t)i * (stages + 1) + stages] == 1.0, "mixed precision needs B[i][stages] == 1");
  }
  t->stages = stages;
  t->A.assign(A, A + stages);
  t->B.assign(B, B + (size_t)stages * (stages + 1));
  t->CT.assign(CT, CT + stages);
  t->CH.assign(CH, CH + stages + 1);
  return alloc_state(t, stages);
}

// Tiles of the Omega derivative: rows of one (class, lead) range against
// columns of one lead's sourced (OmA) or free (OmB) modes.
static void build_tiles(zg_traj* t, std::vector<OmTile>& out) {
  const int TS = 64;
  auto add = [&](int r0, int r1, int c0, int c1, int a, int b, int blk, int term1, int term2) {
    for (int r = r0; r < r1; r += TS)
      for (int c = c0; c < c1; c += TS) {
        OmTile x;
        x.row0 = r; x.nrows = std::min(TS, r1 - r);
        x.col0 = c; x.ncols = std::min(TS, c1 - c);
        x.a = a; x.b = b; x.blk = blk; x.term1 = term1; x.term2 = term2;
        out.push_back(x);
      }
  };
  for (int a = 0; a < t->L; ++a)
    for (int b = 0; b < t->L; ++b) {
      // OmA: columns = sourced modes of lead b (local column == mode index)
      int c0 = (int)t->s_start[b], c1 = (int)t->s_start[b + 1];
      add((int)t->s_start[a], (int)t->s_start[a + 1], c0, c1, a, b, 0, 1, 1);
      add((int)t->f_start[a], (int)t->f_start[a + 1], c0, c1, a, b, 0, 1, 0);
      // OmB: rows = sourced modes of lead a, columns = free modes of lead b
      add((int)t->s_start[a], (int)t->s_start[a + 1], (int)(t->f_start[b] - t->Ns), (int)(t->f_start[b + 1] - t->Ns),
          a, b, 1, 0, 1);
    }
}

// sizes the split-K workspaces from the fixed GEMM shapes of the trajectory
static int presize_workspaces(zg_traj* t);

static void to_f32(const double2* a, float2* b, size_t n) {
  for (size_t i = 0; i < n; ++i) b[i] = make_float2((float)a[i].x, (float)a[i].y);
}

// The products of the mixed stage that run on the tensor cores (zg_tcx.cu):
// PI partials (A = the planar psi parts, transposed in shared memory), the
// Omega xi products (A = the raw Omega blocks of the stage input) and the
// xi sigma^T rows (A = xi, B' = the embedded sigma columns of the lead).  The
// B' operands of the first two kinds are constants: the real embedding of
// IXI (PI) and XIS (Omega xi) over each problem's mode range, zero outside it,
// stacked along K.  Leaves t->tcx_on false (the SIMT batch then runs) when a
// shape does not suit TMA (odd block widths, misaligned blocks) or the
// coupling width exceeds the kernels.
static int build_tcx(zg_traj* t, const zg_layout* Lo, const std::vector<double2>& U, const std::vector<double2>& V) {
  const int64_t n = t->n, N = t->N, Ns = t->Ns, Nf = t->Nf, L = t->L, nc = t->nc, np = t->np;
  const int bn = tcx_bn_for((int)(2 * nc));
  const MixedLayout& ml = t->ml;
  const float* psih = (const float*)(t->stage32 + ml.st_psih);
  const float* psil = (const float*)(t->stage32 + ml.st_psil);
  const float* omA = (const float*)(t->stage32 + ml.st_om);
  const float* omB = omA + 2 * N * Ns;
  auto al16 = [](const void* q) { return ((uintptr_t)q & 15) == 0; };
  if (bn == 0 || Ns % 2 || Nf % 2 || !al16(omA) || !al16(omB) || Ns == 0) return ZG_OK;
  cudaStream_t s = t->stream;
  const int ndw = tcx_ndw(bn);
  std::unique_ptr<TcxBatch> B(new TcxBatch());
  memset(B.get(), 0, sizeof(TcxBatch));
  // ---- B' stack of the PI and Omega xi problems
  struct Blk { int kind, a, cls; int64_t r0, r1, q0, q1, koff; };  // kind 0 PI, 1 ZA, 2 ZB
  std::vector<Blk> blk;
  int64_t kstack = 0;
  auto add = [&](int kind, int a, int cls, int64_t r0, int64_t r1) {
    if (r1 <= r0) return;
    Blk b;
    b.kind = kind; b.a = a; b.cls = cls; b.r0 = r0; b.r1 = r1;
    b.q0 = r0 / 16 * 16;
    b.q1 = (r1 + 15) / 16 * 16;
    b.koff = kstack;
    kstack += 2 * (b.q1 - b.q0);
    blk.push_back(b);
  };
  for (int a = 0; a < L; ++a) {
    add(0, a, 0, t->s_start[a], t->s_start[a + 1]);
    add(0, a, 1, t->f_start[a], t->f_start[a + 1]);
  }
  for (int b = 0; b < L; ++b) add(1, b, 0, t->s_start[b], t->s_start[b + 1]);
  for (int b = 0; b < L; ++b) add(2, b, 0, t->f_start[b] - Ns, t->f_start[b + 1] - Ns);
  if ((int)blk.size() + L > ZG_TCX_PROBS || kstack == 0) return ZG_OK;
  std::vector<float> Bh((size_t)bn * kstack, 0.f);
  const double2* IXI = (const double2*)Lo->IXI;
  const double2* XIS = (const double2*)Lo->XIS;
  const double2* XI = (const double2*)Lo->XI;
  for (const Blk& b : blk) {
    const double2* val = b.kind == 0 ? IXI : XIS;
    for (int64_t r = b.r0; r < b.r1; ++r) {
      const int64_t m = b.kind == 2 ? r + Ns : r;  // OmB columns are free modes
      const int64_t j = b.koff + 2 * (r - b.q0);
      for (int64_t k = 0; k < nc; ++k) {
        const double2 v = val[m * nc + k];
        Bh[(size_t)(2 * k) * kstack + j] = (float)v.x;
        Bh[(size_t)(2 * k) * kstack + j + 1] = (float)-v.y;
        Bh[(size_t)(2 * k + 1) * kstack + j] = (float)v.y;
        Bh[(size_t)(2 * k + 1) * kstack + j + 1] = (float)v.x;
      }
    }
  }
  ZG_TRY(dalloc(t, &t->tcxBh, Bh.size()));
  ZG_TRY(dalloc(t, &t->tcxBl, Bh.size()));
  ZG_CHECK_CUDA(cudaMemcpyAsync(t->tcxBl, Bh.data(), Bh.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  ZG_TRY(launch_split_tf32(t->tcxBl, t->tcxBh, t->tcxBl, (int64_t)Bh.size(), s));
  // ---- A of xi sigma^T (xi, interleaved) and the per-stage B' (embedded sigma columns)
  const int ldx = (int)((2 * nc + 31) / 32 * 32);
  t->ldx = ldx;
  std::vector<float> Xh((size_t)N * ldx, 0.f);
  for (int64_t m = 0; m < N; ++m)
    for (int64_t k = 0; k < nc; ++k) {
      Xh[(size_t)m * ldx + 2 * k] = (float)XI[m * nc + k].x;
      Xh[(size_t)m * ldx + 2 * k + 1] = (float)XI[m * nc + k].y;
    }
  ZG_TRY(dalloc(t, &t->XIh, Xh.size()));
  ZG_TRY(dalloc(t, &t->XIl, Xh.size()));
  ZG_CHECK_CUDA(cudaMemcpyAsync(t->XIl, Xh.data(), Xh.size() * sizeof(float), cudaMemcpyHostToDevice, s));
  ZG_TRY(launch_split_tf32(t->XIl, t->XIh, t->XIl, (int64_t)Xh.size(), s));
  const int64_t nE = L * 2 * n * ldx;
  ZG_TRY(dalloc(t, &t->sigEh, nE));
  ZG_TRY(dalloc(t, &t->sigEl, nE));
  ZG_CHECK_CUDA(cudaMemsetAsync(t->sigEh, 0, nE * sizeof(float), s));
  ZG_CHECK_CUDA(cudaMemsetAsync(t->sigEl, 0, nE * sizeof(float), s));
  // products that get no problem keep zero blocks (an empty class or lead)
  ZG_CHECK_CUDA(cudaMemsetAsync(t->Pc32, 0, 2 * L * n * nc * sizeof(float2), s));
  ZG_CHECK_CUDA(cudaMemsetAsync(t->ZA32, 0, L * N * nc * sizeof(float2), s));
  ZG_CHECK_CUDA(cudaMemsetAsync(t->ZB32, 0, L * std::max<int64_t>(Ns, 1) * nc * sizeof(float2), s));
  // ---- tensor maps
  CUtensorMap* mp = B->maps;
  ZG_TRY(tcx_map(*B, 0, psih, 2 * N, np, np, 16, 128, false));
  ZG_TRY(tcx_map(*B, 1, psil, 2 * N, np, np, 16, 128, false));
  ZG_TRY(tcx_map(*B, 2, omA, N, 2 * Ns, 2 * Ns, 128, 32, true));
  if (Nf > 0) ZG_TRY(tcx_map(*B, 3, omB, Ns, 2 * Nf, 2 * Nf, 128, 32, true));
  ZG_TRY(tcx_map(*B, 4, t->XIh, N, 2 * nc, ldx, 128, 32, true));
  ZG_TRY(tcx_map(*B, 5, t->XIl, N, 2 * nc, ldx, 128, 32, true));
  ZG_TRY(tcx_map(*B, 6, t->tcxBh, bn, kstack, kstack, bn, 32, true));
  ZG_TRY(tcx_map(*B, 7, t->tcxBl, bn, kstack, kstack, bn, 32, true));
  ZG_TRY(tcx_map(*B, 8, t->sigEh, L * 2 * n, 2 * nc, ldx, bn, 32, true));
  ZG_TRY(tcx_map(*B, 9, t->sigEl, L * 2 * n, 2 * nc, ldx, bn, 32, true));
  // ---- problems (K chunks set below, once the total work is known)
  std::vector<TcxProb> probs;
  for (const Blk& b : blk) {
    TcxProb P;
    memset(&P, 0, sizeof(P));
    P.mapB = 6;
    P.b_row0 = 0;
    P.b_k0 = (int)b.koff;
    P.a_k0 = (int)(2 * b.q0);
    P.K = (int)(2 * (b.q1 - b.q0));
    P.kseg = P.K;  // one operand pair
    P.om_map = -1;
    P.Nv = (int)(2 * nc);
    P.ldd = 2 * nc;
    P.tiles_n = 1;
    if (b.kind == 0) {
      P.amode = 2; P.mapA = 0; P.a_row0 = 0; P.a_plane = (int)N; P.M = (int)n;
      P.D = (float*)(t->Pc32 + ((int64_t)(b.cls * L + b.a) * n) * nc);
    } else if (b.kind == 1) {
      P.amode = 1; P.mapA = 2; P.M = (int)N;
      P.D = (float*)(t->ZA32 + (int64_t)b.a * N * nc);
    } else {
      P.amode = 1; P.mapA = 3; P.M = (int)Ns;
      P.D = (float*)(t->ZB32 + (int64_t)b.a * Ns * nc);
    }
    P.tiles_m = (P.M + 127) / 128;
    probs.push_back(P);
  }
  for (int a = 0; a < L; ++a) {
    const int64_t r0 = t->s_start[a], r1 = t->s_start[a + 1];
    if (r1 <= r0) continue;
    TcxProb P;
    memset(&P, 0, sizeof(P));
    P.amode = 0; P.mapA = 4; P.mapB = 8;
    P.a_row0 = (int)r0; P.a_k0 = 0;
    P.b_row0 = (int)(a * 2 * n); P.b_k0 = 0;
    P.M = (int)(r1 - r0); P.Nv = (int)(2 * n);
    P.K = ldx;
    P.kseg = P.K;
    P.om_map = -1;
    P.tiles_m = (P.M + 127) / 128;
    P.tiles_n = (int)((2 * n + bn - 1) / bn);
    P.D = (float*)(t->R2_32 + r0 * n);
    P.ldd = 2 * n;
    probs.push_back(P);
  }
  // ---- the Omega derivative: one problem per block of Omega (rows of one
  // class and lead a, columns of lead b) in tiles of 128 rows x bn/2 complex
  // columns.  Source terms (Zandpack/mpi/zand:784-801) as two K segments of
  // n_c complex:
  //   term 1 (OmA blocks): psi[m] on lead b's columns . U[l]   (U = dGM Ixi)
  //   term 2 (sourced rows): V[m] . conj(psi[l] on lead a's columns)
  // (A rows Gt[b][m] and V[m]; B' rows the embeddings of U and of conj psi),
  // the diagonal term in the kernel's epilogue.
  bool omega_tc = (int)probs.size() + 3 * L * L <= ZG_TCX_PROBS;
  std::vector<int> om_tile_map;  // per Omega problem: its tile map when tiles are prefetched
  if (omega_tc) {
    std::vector<float> Vf((size_t)N * ldx, 0.f), Uf((size_t)2 * N * ldx, 0.f);
    for (int64_t m = 0; m < N; ++m)
      for (int64_t k = 0; k < nc; ++k) {
        const double2 v = V[m * nc + k], u = U[m * nc + k];
        Vf[(size_t)m * ldx + 2 * k] = (float)v.x;
        Vf[(size_t)m * ldx + 2 * k + 1] = (float)v.y;
        Uf[(size_t)(2 * m) * ldx + 2 * k] = (float)u.x;
        Uf[(size_t)(2 * m) * ldx + 2 * k + 1] = (float)-u.y;
        Uf[(size_t)(2 * m + 1) * ldx + 2 * k] = (float)u.y;
        Uf[(size_t)(2 * m + 1) * ldx + 2 * k + 1] = (float)u.x;
      }
    ZG_TRY(dalloc(t, &t->Vh, Vf.size()));
    ZG_TRY(dalloc(t, &t->Vl, Vf.size()));
    ZG_TRY(dalloc(t, &t->Uh, Uf.size()));
    ZG_TRY(dalloc(t, &t->Ul, Uf.size()));
    ZG_CHECK_CUDA(cudaMemcpyAsync(t->Vl, Vf.data(), Vf.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    ZG_CHECK_CUDA(cudaMemcpyAsync(t->Ul, Uf.data(), Uf.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    ZG_TRY(launch_split_tf32(t->Vl, t->Vh, t->Vl, (int64_t)Vf.size(), s));
    ZG_TRY(launch_split_tf32(t->Ul, t->Uh, t->Ul, (int64_t)Uf.size(), s));
    const int64_t ng = L * N * ldx, nG = L * 2 * N * ldx;
    ZG_TRY(dalloc(t, &t->Gth, ng));
    ZG_TRY(dalloc(t, &t->Gtl, ng));
    ZG_TRY(dalloc(t, &t->Gch, nG));
    ZG_TRY(dalloc(t, &t->Gcl, nG));
    for (float* q : {t->Gth, t->Gtl}) ZG_CHECK_CUDA(cudaMemsetAsync(q, 0, ng * sizeof(float), s));
    for (float* q : {t->Gch, t->Gcl}) ZG_CHECK_CUDA(cudaMemsetAsync(q, 0, nG * sizeof(float), s));
    ZG_TRY(tcx_map(*B, 10, t->Gth, L * N, 2 * nc, ldx, 128, 32, true));
    ZG_TRY(tcx_map(*B, 11, t->Gtl, L * N, 2 * nc, ldx, 128, 32, true));
    ZG_TRY(tcx_map(*B, 12, t->Uh, 2 * N, 2 * nc, ldx, bn, 32, true));
    ZG_TRY(tcx_map(*B, 13, t->Ul, 2 * N, 2 * nc, ldx, bn, 32, true));
    ZG_TRY(tcx_map(*B, 14, t->Vh, N, 2 * nc, ldx, 128, 32, true));
    ZG_TRY(tcx_map(*B, 15, t->Vl, N, 2 * nc, ldx, 128, 32, true));
    ZG_TRY(tcx_map(*B, 16, t->Gch, L * 2 * N, 2 * nc, ldx, bn, 32, true));
    ZG_TRY(tcx_map(*B, 17, t->Gcl, L * 2 * N, 2 * nc, ldx, bn, 32, true));
    const float2* oA = t->stage32 + ml.st_om;
    const float2* oB = oA + N * Ns;
    // blocks of Omega_in prefetched by the kernel (when its shared memory has room)
    const bool tiles_ok = tcx_has_omega_tile(bn);
    if (tiles_ok) {
      ZG_TRY(tcx_map(*B, 18, oA, N, 2 * Ns, 2 * Ns, 128, bn, false));
      if (Nf > 0) ZG_TRY(tcx_map(*B, 19, oB, Ns, 2 * Nf, 2 * Nf, 128, bn, false));
    }
    // kind 0: OmA rows sourced of a (both terms); 1: OmA rows free of a (term 1);
    // 2: OmB rows sourced of a, columns free of b (term 2)
    for (int a = 0; a < L; ++a)
      for (int b = 0; b < L; ++b)
        for (int kind = 0; kind < 3; ++kind) {
          const int64_t r0 = kind == 1 ? t->f_start[a] : t->s_start[a];
          const int64_t r1 = kind == 1 ? t->f_start[a + 1] : t->s_start[a + 1];
          const int64_t c0 = kind == 2 ? t->f_start[b] : t->s_start[b];
          const int64_t c1 = kind == 2 ? t->f_start[b + 1] : t->s_start[b + 1];
          if (r1 <= r0 || c1 <= c0) continue;
          TcxProb P;
          memset(&P, 0, sizeof(P));
          P.amode = 0;
          P.epi = 1;
          P.M = (int)(r1 - r0);
          P.Nv = (int)(2 * (c1 - c0));
          P.tiles_m = (int)((r1 - r0 + 127) / 128);
          P.tiles_n = (int)((2 * (c1 - c0) + bn - 1) / bn);
          P.mapA = 10; P.a_row0 = (int)(b * N + r0); P.a_k0 = 0;  // term 1: Gt[b][m]
          P.mapB = 12; P.b_row0 = (int)(2 * c0); P.b_k0 = 0;       // U' rows 2l
          P.mapA2 = 14; P.a_row0_2 = (int)r0;                      // term 2: V[m]
          P.mapB2 = 16; P.b_row0_2 = (int)(a * 2 * N + 2 * c0);    // Gc[a] rows 2l
          if (kind == 0) { P.kseg = ldx; P.K = 2 * ldx; }
          else if (kind == 1) { P.kseg = ldx; P.K = ldx; }
          else { P.kseg = 0; P.K = ldx; }
          P.ld_om = (int)(kind == 2 ? Nf : Ns);
          const int64_t lc0 = kind == 2 ? c0 - Ns : c0;  // local column in OmA / OmB
          P.om_in = (kind == 2 ? oB : oA) + r0 * P.ld_om + lc0;
          P.om_out_off = (kind == 2 ? t->off_omB : t->off_omA) + r0 * P.ld_om + lc0;
          P.row_mode0 = (int)r0;
          P.col_mode0 = (int)c0;
          P.la = a;
          P.lb = b;
          // TMA needs the block's first float column on a 16-byte boundary
          om_tile_map.push_back(lc0 % 2 == 0 ? (kind == 2 ? 19 : 18) : -1);
          P.om_map = tiles_ok ? om_tile_map.back() : -1;
          P.om_x0 = (int)(2 * lc0);
          P.om_y0 = (int)r0;
          probs.push_back(P);
        }
  }
  int sms = 0;
  ZG_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, t->dev));
  const int grid = std::max(1, std::min(sms, ZG_TCX_GRID));
  // K chunks: at most about the average work of a CTA over the products
  // (measured at n=1024 against half and a third of it: the fewer split-K
  // partials outweigh the coarser balance, which the CTAs' run-time claims
  // of the items, most expensive first, keep close); each problem's K is cut
  // into equal chunks (the same chunks in both batches below, so that they
  // share the split-K scratch)
  int64_t total_kb = 0;
  for (const TcxProb& P : probs)
    if (P.epi == 0) total_kb += (int64_t)P.tiles_m * P.tiles_n * (P.K / 32);
  const int chunk_kb0 = (int)std::min<int64_t>(64, std::max<int64_t>(8, (total_kb + grid - 1) / grid));
  int chunk_kb = chunk_kb0;
  for (;;) {
    int items = 0;
    for (TcxProb& P : probs) {
      const int kb = P.K / 32;
      const int ns = (kb + chunk_kb - 1) / chunk_kb;
      P.kchunk = P.epi == 1 ? P.K : 32 * ((kb + ns - 1) / ns);  // Omega blocks: whole K per tile
      P.nsplit = (P.K + P.kchunk - 1) / P.kchunk;
      if (P.epi == 0) items += P.tiles_m * P.tiles_n * P.nsplit;
    }
    if (items <= ZG_TCX_ITEMS) break;
    if (chunk_kb >= 1024) return ZG_OK;  // too many tiles for the item table: the SIMT kernels run
    chunk_kb *= 2;
  }
  // the batch with the Omega blocks too needs its items in the table as well
  if (omega_tc) {
    int all = 0;
    for (const TcxProb& P : probs) all += P.tiles_m * P.tiles_n * P.nsplit;
    if (all > ZG_TCX_ITEMS) omega_tc = false;
  }
  // split-K scratch and slice counters of the products (shared by both batches)
  int64_t ws_need = 0, cnt_need = 0;
  std::vector<int64_t> ws_off, cnt_off;
  for (const TcxProb& P : probs) {
    if (P.epi == 1) {
      ws_off.push_back(-1);
      cnt_off.push_back(-1);
      continue;
    }
    ws_off.push_back(P.nsplit > 1 ? ws_need : -1);
    if (P.nsplit > 1) ws_need += (int64_t)P.tiles_m * P.tiles_n * P.nsplit * 128 * bn;
    cnt_off.push_back(cnt_need);
    cnt_need += (int64_t)P.tiles_m * P.tiles_n * ndw;
  }
  if (ws_need > 0) ZG_TRY(dalloc(t, &t->tcx_ws, ws_need));
  ZG_TRY(dalloc(t, &t->tcx_cnt, std::max<int64_t>(cnt_need, 1)));
  ZG_CHECK_CUDA(cudaMemsetAsync(t->tcx_cnt, 0, std::max<int64_t>(cnt_need, 1) * sizeof(int), s));
  for (size_t i = 0; i < probs.size(); ++i) {
    probs[i].ws = ws_off[i] >= 0 ? t->tcx_ws + ws_off[i] : nullptr;
    probs[i].counters = cnt_off[i] >= 0 ? t->tcx_cnt + cnt_off[i] : nullptr;
  }
  B->params = t->d_params;
  B->Xp = t->Xp32;
  B->Xm = t->Xm32;
  B->bn = bn;
  B->err = t->tc_err;
  // one batch with the products alone, one with the products and the Omega
  // blocks: the problem list, item numbering and the longest-first item lists
  // CTAs claim items at run time, most expensive first; the estimate is the
  // item's traffic through shared memory in KB: per K block the A tile (raw
  // FP32 Omega: 16 KB; hi and lo parts or the four psi planes: 32 KB) and B'
  // hi and lo (bn / 4 KB), then the stored tile (bn / 2 KB) and, for split
  // K, the partial re-read by the reduction, for an Omega tile its block of
  // Omega_in
  auto item_cost = [&](const TcxProb& P, int split) -> int64_t {
    const int64_t nkb = std::min(P.kchunk, P.K - split * P.kchunk) / 32;
    const int64_t tile = bn / 2;
    return nkb * ((P.amode == 1 ? 16 : 32) + bn / 4) + tile * (1 + (P.nsplit > 1) + (P.epi == 1));
  };
  // two claim counters per batch, zero between launches
  ZG_TRY(dalloc(t, &t->tcx_claim, 6));
  ZG_CHECK_CUDA(cudaMemsetAsync(t->tcx_claim, 0, 6 * sizeof(int), s));
  auto finish = [&](TcxBatch& Bt, bool with_omega, int* claim, int* grid_used) -> int {
    int np_ = 0, items = 0;
    std::vector<int64_t> cost;
    for (const TcxProb& P0 : probs) {
      if (P0.epi == 1 && !with_omega) continue;
      TcxProb P = P0;
      P.item_begin = items;
      items += P.tiles_m * P.tiles_n * P.nsplit;
      for (int w = 0; w < P.tiles_m * P.tiles_n * P.nsplit; ++w) cost.push_back(item_cost(P, w % P.nsplit));
      Bt.p[np_++] = P;
    }
    Bt.nprob = np_;
    Bt.nitems = items;
    std::vector<int> order(items);
    for (int i = 0; i < items; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
    for (int i = 0; i < items; ++i) Bt.items[i] = (unsigned short)order[i];
    Bt.claim = claim;
    *grid_used = std::min(grid, items);
    // many items per CTA (the Omega tiles are short): claim two items ahead
    Bt.ahead2 = items >= 6 * *grid_used ? 1 : 0;
    return tcx_validate(Bt);
  };
  std::unique_ptr<TcxBatch> Bm, Bo;
  if (omega_tc) {
    Bm.reset(new TcxBatch(*B));
    ZG_TRY(finish(*Bm, true, t->tcx_claim + 2, &t->tcx_grid_all));
    // dOmega/dt alone in tiles of 128 rows x 32 complex columns, whatever
    // the products' width, for the second stream (ZG_IMPL_TC_SPLIT): the
    // Omega blocks' tile width does not depend on n_c.  Wider tiles (64 or
    // 96 complex columns) when the narrow ones overflow the item table
    int bo = 0;
    for (int cand : {64, 128, 192}) {
      int64_t it = 0;
      for (const TcxProb& P0 : probs)
        if (P0.epi == 1) it += (int64_t)P0.tiles_m * ((P0.Nv + cand - 1) / cand);
      if (it <= ZG_TCX_ITEMS) {
        bo = cand;
        break;
      }
    }
    if (bo == 0) bo = 192;  // no width fits: the batch is not built below
    Bo.reset(new TcxBatch());
    memset(Bo.get(), 0, sizeof(TcxBatch));
    const float2* oA = t->stage32 + ml.st_om;
    const float2* oB = oA + N * Ns;
    ZG_TRY(tcx_map(*Bo, 10, t->Gth, L * N, 2 * nc, ldx, 128, 32, true));
    ZG_TRY(tcx_map(*Bo, 11, t->Gtl, L * N, 2 * nc, ldx, 128, 32, true));
    ZG_TRY(tcx_map(*Bo, 12, t->Uh, 2 * N, 2 * nc, ldx, bo, 32, true));
    ZG_TRY(tcx_map(*Bo, 13, t->Ul, 2 * N, 2 * nc, ldx, bo, 32, true));
    ZG_TRY(tcx_map(*Bo, 14, t->Vh, N, 2 * nc, ldx, 128, 32, true));
    ZG_TRY(tcx_map(*Bo, 15, t->Vl, N, 2 * nc, ldx, 128, 32, true));
    ZG_TRY(tcx_map(*Bo, 16, t->Gch, L * 2 * N, 2 * nc, ldx, bo, 32, true));
    ZG_TRY(tcx_map(*Bo, 17, t->Gcl, L * 2 * N, 2 * nc, ldx, bo, 32, true));
    const bool bo_tiles = tcx_has_omega_tile(bo);
    if (bo_tiles) {
      ZG_TRY(tcx_map(*Bo, 18, oA, N, 2 * Ns, 2 * Ns, 128, bo, false));
      if (Nf > 0) ZG_TRY(tcx_map(*Bo, 19, oB, Ns, 2 * Nf, 2 * Nf, 128, bo, false));
    }
    int np_ = 0, items = 0, om_i = 0;
    std::vector<int64_t> cost;
    for (const TcxProb& P0 : probs) {
      if (P0.epi != 1) continue;
      TcxProb P = P0;
      P.tiles_n = (P.Nv + bo - 1) / bo;
      P.om_map = bo_tiles ? om_tile_map[om_i] : -1;
      ++om_i;
      P.item_begin = items;
      items += P.tiles_m * P.tiles_n;
      for (int w = 0; w < P.tiles_m * P.tiles_n; ++w) cost.push_back((P.K / 32) * (32 + bo / 4) + bo);
      Bo->p[np_++] = P;
    }
    if (items > 0 && items <= ZG_TCX_ITEMS) {
      Bo->nprob = np_;
      Bo->nitems = items;
      Bo->bn = bo;
      Bo->err = t->tc_err;
      Bo->params = t->d_params;
      Bo->Xp = t->Xp32;
      Bo->Xm = t->Xm32;
      std::vector<int> order(items);
      for (int i = 0; i < items; ++i) order[i] = i;
      std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
      for (int i = 0; i < items; ++i) Bo->items[i] = (unsigned short)order[i];
      Bo->claim = t->tcx_claim + 4;
      t->tcx_grid_om = std::min(grid, items);
      Bo->ahead2 = items >= 6 * t->tcx_grid_om ? 1 : 0;
      ZG_TRY(tcx_validate(*Bo));
    } else {
      Bo.reset();
    }
  }
  ZG_TRY(finish(*B, false, t->tcx_claim, &t->tcx_grid));
  t->tcx = B.release();
  t->tcx_all = Bm.release();
  t->tcx_om = Bo.release();
  t->tcx_on = true;
  t->prod_impl = ZG_IMPL_TC_PRODUCTS;
  t->tcx_ops.sigEh = t->sigEh;
  t->tcx_ops.sigEl = t->sigEl;
  t->tcx_ops.ldx = ldx;
  if (omega_tc) t->tco_on = true;
  return ZG_OK;
}

static int create_mixed(zg_traj* t, const zg_layout* Lo, const std::vector<double2>& U, const std::vector<double2>& V) {
  const int64_t n = t->n, N = t->N, Ns = t->Ns, Nf = t->Nf, L = t->L, nc = t->nc;
  const int64_t np = (n + 15) / 16 * 16;
  t->np = (int)np;
  MixedLayout& ml = t->ml;
  ml.n = n; ml.N = N; ml.np = np;
  ml.off_psi = t->off_psi; ml.off_omA = t->off_omA; ml.S = t->S;
  ml.st_psih = n * n;
  ml.st_psil = ml.st_psih + N * np;
  ml.st_om = ml.st_psil + N * np;
  ml.st_S = ml.st_om + N * Ns + Ns * Nf;
  ml.plane = N * np;  // psi hi and lo are stored planar: real rows, then imaginary rows
  {
    bool real = true;
    for (int64_t e = 0; e < n * n && real; ++e) real = Lo->H0[2 * e + 1] == 0.0;
    t->h0_real = real;
    t->h0_real_orth = real;
  }
  cudaStream_t s = t->stream;
  // host copies stay alive until the stream synchronisation at the end
  std::vector<std::vector<float2>> keep;
  auto up32 = [&](float2** dst, const double* src, size_t cnt) -> int {
    keep.emplace_back(cnt);
    to_f32((const double2*)src, keep.back().data(), cnt);
    ZG_TRY(dalloc(t, dst, cnt));
    ZG_CHECK_CUDA(cudaMemcpyAsync(*dst, keep.back().data(), cnt * sizeof(float2), cudaMemcpyHostToDevice, s));
    return ZG_OK;
  };
  ZG_TRY(up32(&t->Xp32, Lo->Xp, N));
  ZG_TRY(up32(&t->Xm32, Lo->Xm, N));
  ZG_TRY(up32(&t->GLP32, Lo->GLP, N));
  ZG_TRY(up32(&t->dGP32, Lo->dGP, N));
  ZG_TRY(up32(&t->XI32, Lo->XI, N * nc));
  ZG_TRY(up32(&t->XIS32, Lo->XIS, N * nc));
  ZG_TRY(up32(&t->IXI32, Lo->IXI, N * nc));
  ZG_TRY(up32(&t->U32, (const double*)U.data(), N * nc));
  ZG_TRY(up32(&t->V32, (const double*)V.data(), N * nc));
  ZG_TRY(dalloc(t, &t->y32, t->S));
  ZG_TRY(dalloc(t, &t->stage32, ml.st_S));
  ZG_CHECK_CUDA(cudaMemsetAsync(t->stage32, 0, ml.st_S * sizeof(float2), s));  // psi padding columns stay zero
  ZG_TRY(dalloc(t, &t->Hth, 2 * np * np)); ZG_TRY(dalloc(t, &t->Htl, 2 * np * np));
  ZG_TRY(dalloc(t, &t->BSh, 2 * np * np)); ZG_TRY(dalloc(t, &t->BSl, 2 * np * np));
  ZG_CHECK_CUDA(cudaMemsetAsync(t->Hth, 0, 2 * np * np * sizeof(float), s));
  ZG_CHECK_CUDA(cudaMemsetAsync(t->Htl, 0, 2 * np * np * sizeof(float), s));
  ZG_TRY(dalloc(t, &t->T32, 2 * np * np)); ZG_TRY(dalloc(t, &t->R1p, N * 2 * np));
  ZG_TRY(dalloc(t, &t->Pc32, 2 * L * n * nc)); ZG_TRY(dalloc(t, &t->sigC32, L * n * nc)); ZG_TRY(dalloc(t, &t->G32, N * L * nc));
  ZG_TRY(dalloc(t, &t->R2_32, std::max<int64_t>(Ns, 1) * n));
  ZG_TRY(dalloc(t, &t->ZA32, L * N * nc)); ZG_TRY(dalloc(t, &t->ZB32, L * std::max<int64_t>(Ns, 1) * nc));
  ZG_TRY(dalloc(t, &t->sig64, n * n));
  ZG_TRY(dalloc(t, &t->tc_err, 1));
  ZG_CHECK_CUDA(cudaMemsetAsync(t->tc_err, 0, sizeof(int), s));
  // Tensor maps of the two tensor-core GEMMs (fixed buffers), planar operands
  // with K = np, every output row 2 np floats wide:
  //   psi H^T:  A = psi (2N rows: real, imaginary), B = H rows (real H: the
  //             real part, nb32 rows; complex H: 2 np rows, real then imaginary)
  //   H sigma:  A = H rows (real H: n rows; complex H: 2 np), B = sigma^T
  //             (2 np rows: real part columns, imaginary part columns)
  const float* psih = (const float*)(t->stage32 + ml.st_psih);
  const float* psil = (const float*)(t->stage32 + ml.st_psil);
  const int64_t nb32 = (n + 31) / 32 * 32;  // <= 2 np; rows n.. of H are zero
  ZG_TRY(tc_gemm_prepare(t->gT, t->Hth, t->Htl, t->BSh, t->BSl, np, np, (float*)t->T32, 2 * np, (int)n,
                         (int)(2 * np), (int)np, t->tc_err));
  ZG_TRY(tc_gemm_prepare(t->gTc, t->Hth, t->Htl, t->BSh, t->BSl, np, np, (float*)t->T32, 2 * np, (int)(2 * np),
                         (int)(2 * np), (int)np, t->tc_err));
  ZG_TRY(tc_gemm_prepare(t->gR1, psih, psil, t->Hth, t->Htl, np, np, (float*)t->R1p, 2 * np, (int)(2 * N),
                         (int)nb32, (int)np, t->tc_err));
  ZG_TRY(tc_gemm_prepare(t->gR1c, psih, psil, t->Hth, t->Htl, np, np, (float*)t->R1p, 2 * np, (int)(2 * N),
                         (int)(2 * np), (int)np, t->tc_err));
  if (getenv("ZG_SIMT_PRODUCTS") == nullptr) {
    ZG_TRY(build_tcx(t, Lo, U, V));
  }
  ZG_CHECK_CUDA(cudaStreamSynchronize(s));
  return ZG_OK;
}

extern "C" {

const char* zg_last_error(void) { return g_err; }
int zg_version(void) { return 101; }
long long zg_launch_count(void) { return g_launches.load(); }
void* zg_traj_stream(const zg_traj* t) { return t ? (void*)t->stream : nullptr; }

int zg_traj_create(int device, const zg_layout* Lo, int precision, zg_traj** out) {
  ZG_REQUIRE(out && Lo, "null argument");
  *out = nullptr;
  ZG_REQUIRE(precision == ZG_PREC_F64 || precision == ZG_PREC_MIXED, "unknown precision mode %d", precision);
  ZG_REQUIRE(Lo->n > 0 && Lo->n_leads > 0 && Lo->n_leads <= ZG_MAX_LEADS && Lo->n_modes > 0 &&
                 Lo->n_sourced >= 0 && Lo->n_sourced <= Lo->n_modes && Lo->nc > 0,
             "bad layout sizes");
  ZG_REQUIRE(Lo->hbar > 0, "hbar must be positive");
  ZG_REQUIRE(device >= 0 && device < ZG_MAX_DEVICES, "device %d out of range", device);
  ZG_CHECK_CUDA(cudaSetDevice(device));
  zg_traj* t = new zg_traj();
  t->dev = device;
  t->precision = precision;
  t->n = Lo->n; t->L = Lo->n_leads; t->N = Lo->n_modes; t->Ns = Lo->n_sourced; t->Nf = t->N - t->Ns; t->nc = Lo->nc;
  t->hbar = Lo->hbar;
  const int64_t n = t->n, N = t->N, Ns = t->Ns, L = t->L, nc = t->nc;
  t->off_psi = n * n;
  t->off_omA = t->off_psi + N * n;
  t->off_omB = t->off_omA + N * Ns;
  t->S = t->off_omB + Ns * t->Nf;
  t->s_start.assign(Lo->s_start, Lo->s_start + L + 1);
  t->f_start.assign(Lo->f_start, Lo->f_start + L + 1);
  int st = ZG_OK;
#define ZG_STEP(x)  \
  do {              \
    st = (x);       \
    if (st != ZG_OK) { free_traj(t); return st; } \
  } while (0)
  // validate row ranges
  bool ok = t->s_start[0] == 0 && t->s_start[L] == Ns && t->f_start[0] == Ns && t->f_start[L] == N;
  for (int a = 0; a < L && ok; ++a) ok = t->s_start[a] <= t->s_start[a + 1] && t->f_start[a] <= t->f_start[a + 1];
  if (!ok) { free_traj(t); set_error("s_start/f_start do not partition the modes"); return ZG_EINVAL; }
  for (int64_t m = 0; m < N; ++m) {
    int a = Lo->mode_lead[m];
    bool in = a >= 0 && a < L &&
              ((m < Ns) ? (m >= t->s_start[a] && m < t->s_start[a + 1]) : (m >= t->f_start[a] && m < t->f_start[a + 1]));
    if (!in) { free_traj(t); set_error("mode_lead inconsistent with row ranges at mode %lld", (long long)m); return ZG_EINVAL; }
  }
  for (int64_t i = 0; i < L * nc; ++i)
    if (Lo->lead_cols[i] < 0 || Lo->lead_cols[i] >= n) { free_traj(t); set_error("lead_cols out of range"); return ZG_EINVAL; }
  for (int64_t i = 0; i < L * n; ++i)
    if (Lo->colmap[i] < -1 || Lo->colmap[i] >= nc) { free_traj(t); set_error("colmap out of range"); return ZG_EINVAL; }
  if (cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess) {
    free_traj(t); set_error("cudaStreamCreate failed"); return ZG_ECUDA;
  }
  if (precision == ZG_PREC_MIXED &&
      (cudaStreamCreateWithFlags(&t->stream2, cudaStreamNonBlocking) != cudaSuccess ||
       cudaEventCreateWithFlags(&t->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&t->ev_join, cudaEventDisableTiming) != cudaSuccess)) {
    free_traj(t); set_error("second stream or events could not be created"); return ZG_ECUDA;
  }
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    ++g_live[t->dev];
    t->counted = true;
  }
  ZG_STEP(dalloc(t, &t->H0, n * n));
  ZG_STEP(dalloc(t, &t->Xp, N)); ZG_STEP(dalloc(t, &t->Xm, N)); ZG_STEP(dalloc(t, &t->GLP, N)); ZG_STEP(dalloc(t, &t->dGP, N));
  ZG_STEP(dalloc(t, &t->XI, N * nc)); ZG_STEP(dalloc(t, &t->IXI, N * nc)); ZG_STEP(dalloc(t, &t->XIS, N * nc));
  ZG_STEP(dalloc(t, &t->U, N * nc)); ZG_STEP(dalloc(t, &t->V, N * nc));
  ZG_STEP(dalloc(t, &t->mode_lead, N)); ZG_STEP(dalloc(t, &t->lead_cols, L * nc)); ZG_STEP(dalloc(t, &t->colmap, L * n));
  ZG_STEP(upload<double2>(t->H0, Lo->H0, n * n, t->stream));
  ZG_STEP(upload<double2>(t->Xp, Lo->Xp, N, t->stream));
  ZG_STEP(upload<double2>(t->Xm, Lo->Xm, N, t->stream));
  ZG_STEP(upload<double2>(t->GLP, Lo->GLP, N, t->stream));
  ZG_STEP(upload<double2>(t->dGP, Lo->dGP, N, t->stream));
  ZG_STEP(upload<double2>(t->XI, Lo->XI, N * nc, t->stream));
  ZG_STEP(upload<double2>(t->IXI, Lo->IXI, N * nc, t->stream));
  ZG_STEP(upload<double2>(t->XIS, Lo->XIS, N * nc, t->stream));
  ZG_STEP(upload<int>(t->mode_lead, Lo->mode_lead, N, t->stream));
  ZG_STEP(upload<int>(t->lead_cols, Lo->lead_cols, L * nc, t->stream));
  ZG_STEP(upload<int>(t->colmap, Lo->colmap, L * n, t->stream));
  t->lead_cols_h.assign(Lo->lead_cols, Lo->lead_cols + L * nc);
  t->colmap_h.assign(Lo->colmap, Lo->colmap + L * n);
  // orbitals that are a coupling column of some lead: the only rows and
  // columns where the lead terms of the sigma equation are nonzero
  std::vector<int> ucols_h, umap_h(n, -1);
  for (int64_t j = 0; j < n; ++j) {
    bool in = false;
    for (int64_t a = 0; a < L; ++a) in = in || Lo->colmap[a * n + j] >= 0;
    if (in) {
      umap_h[j] = (int)ucols_h.size();
      ucols_h.push_back((int)j);
    }
  }
  t->nu = (int)ucols_h.size();
  ZG_STEP(dalloc(t, &t->ucols, std::max<size_t>(ucols_h.size(), 1)));
  ZG_STEP(dalloc(t, &t->umap, n));
  if (t->nu > 0) ZG_STEP(upload<int>(t->ucols, ucols_h.data(), ucols_h.size(), t->stream));
  ZG_STEP(upload<int>(t->umap, umap_h.data(), n, t->stream));
  // U = dGM * IXI (per column mode), V = dGP * XIT2 (per row mode)
  std::vector<double2> U(N * nc), V(N * nc);
  {
    const double2* dGM = (const double2*)Lo->dGM;
    const double2* dGP = (const double2*)Lo->dGP;
    const double2* IXI = (const double2*)Lo->IXI;
    const double2* XIT2 = (const double2*)Lo->XIT2;
    for (int64_t m = 0; m < N; ++m)
      for (int64_t k = 0; k < nc; ++k) {
        U[m * nc + k] = cmul(dGM[m], IXI[m * nc + k]);
        V[m * nc + k] = cmul(dGP[m], XIT2[m * nc + k]);
      }
  }
  ZG_STEP(upload<double2>(t->U, U.data(), N * nc, t->stream));
  ZG_STEP(upload<double2>(t->V, V.data(), N * nc, t->stream));
  std::vector<OmTile> tiles;
  build_tiles(t, tiles);
  t->ntiles = (int)tiles.size();
  ZG_STEP(dalloc(t, &t->tiles, tiles.size()));
  ZG_STEP(upload<OmTile>(t->tiles, tiles.data(), tiles.size(), t->stream));
  ZG_STEP(dalloc(t, &t->dH, n * n));
  ZG_STEP(dalloc(t, &t->J, L));
  ZG_STEP(dalloc(t, &t->Jpart, L * 64));
  ZG_STEP(dalloc(t, &t->d_params, ZG_MAX_STAGES));  // one per stage in the attempt graph
  ZG_STEP(dalloc(t, &t->ctl, 1));
  ZG_STEP(dalloc(t, &t->d_recs, ZG_GRAPH_MAX_BATCH));
  {
    void* blk = nullptr;
    ZG_STEP(pinned_get(kPinnedBytes, &blk));
    char* b = (char*)blk;
    t->ctl_host = (DevCtl*)b;
    t->J_host = (double*)(b + kPinJ);
    t->tcerr_host = (int*)(b + kPinErr);
    t->recs_host = (zg_attempt_rec*)(b + kPinRecs);
  }
  memset(t->ctl_host, 0, sizeof(DevCtl));
  *t->tcerr_host = 0;
  ZG_CHECK_CUDA(cudaMemsetAsync(t->ctl, 0, sizeof(DevCtl), t->stream));
  t->nblk_err = terr2_nblocks(t->S);
  ZG_STEP(dalloc(t, &t->partial, 3 * (size_t)t->nblk_err));
  ZG_STEP(dalloc(t, &t->err, 3));
  if (precision == ZG_PREC_F64) {
    ZG_STEP(dalloc(t, &t->Ystage, t->S));
    ZG_STEP(dalloc(t, &t->Ht, n * n)); ZG_STEP(dalloc(t, &t->T, n * n));
    ZG_STEP(dalloc(t, &t->Pc, 2 * L * n * nc)); ZG_STEP(dalloc(t, &t->sigC, L * n * nc)); ZG_STEP(dalloc(t, &t->G, N * L * nc));
    ZG_STEP(dalloc(t, &t->R2, std::max<int64_t>(Ns, 1) * n));
    ZG_STEP(dalloc(t, &t->ZA, L * N * nc)); ZG_STEP(dalloc(t, &t->ZB, L * std::max<int64_t>(Ns, 1) * nc));
  } else {
    ZG_STEP(create_mixed(t, Lo, U, V));
  }
  {
    double B[7 * 8], CT[7], CH[8];
    for (int i = 0; i < 7; ++i)
      for (int j = 0; j < 8; ++j) B[i * 8 + j] = kDopB[i][j];
    for (int j = 0; j < 7; ++j) { CT[j] = kB5[j] - kB4[j]; CH[j] = kB5[j]; }
    CH[7] = 1.0;
    ZG_STEP(set_tableau_impl(t, 7, kDopA, B, CT, CH));
  }
  ZG_STEP(presize_workspaces(t));
  t->cur_in = y64(t);
  if (precision == ZG_PREC_MIXED) ZG_STEP(launch_f64_to_f32(t->Y, t->y32, t->S, t->stream));
  // host vectors above must outlive their asynchronous copies
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
#undef ZG_STEP
  *out = t;
  return ZG_OK;
}

int zg_traj_destroy(zg_traj* t) {
  if (!t) return ZG_OK;
  cudaSetDevice(t->dev);
  if (t->stream) cudaStreamSynchronize(t->stream);
  free_traj(t);
  return ZG_OK;
}

int zg_traj_info(const zg_traj* t, int64_t* out) {
  ZG_REQUIRE(t && out, "null argument");
  out[0] = t->n; out[1] = t->L; out[2] = t->N; out[3] = t->Ns; out[4] = t->Nf; out[5] = t->nc; out[6] = t->S;
  out[7] = t->stages;
  return ZG_OK;
}

int zg_set_tableau(zg_traj* t, int stages, const double* A, const double* B, const double* CT, const double* CH) {
  ZG_REQUIRE(t && A && B && CT && CH, "null argument");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  drop_graph(t);  // the captured attempt holds the old coefficients and slots
  ZG_TRY(set_tableau_impl(t, stages, A, B, CT, CH));
  t->cur_in = y64(t);
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  return ZG_OK;
}

static int ensure_conv64(zg_traj* t) {
  if (!t->conv64) ZG_TRY(dalloc(t, &t->conv64, t->S));
  return ZG_OK;
}

int zg_set_state(zg_traj* t, int slot, const double* host) {
  ZG_REQUIRE(t && host, "null argument");
  ZG_REQUIRE(slot >= 0 && slot <= t->stages, "slot %d out of range", slot);
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  const size_t bytes = t->S * sizeof(double2);
  if (t->precision == ZG_PREC_F64) {
    ZG_CHECK_CUDA(cudaMemcpyAsync(t->slot(slot), host, bytes, cudaMemcpyHostToDevice, t->stream));
  } else if (slot == t->stages) {
    ZG_CHECK_CUDA(cudaMemcpyAsync(t->Y, host, bytes, cudaMemcpyHostToDevice, t->stream));
    ZG_TRY(launch_f64_to_f32(t->Y, t->y32, t->S, t->stream));
  } else {
    ZG_TRY(ensure_conv64(t));
    ZG_CHECK_CUDA(cudaMemcpyAsync(t->conv64, host, bytes, cudaMemcpyHostToDevice, t->stream));
    ZG_TRY(launch_f64_to_f32(t->conv64, t->kslot(slot), t->S, t->stream));
  }
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  return ZG_OK;
}

int zg_set_sigma(zg_traj* t, const double* sigma) {
  ZG_REQUIRE(t && sigma, "null argument");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  double2* y = y64(t);
  ZG_CHECK_CUDA(cudaMemsetAsync(y, 0, t->S * sizeof(double2), t->stream));
  ZG_CHECK_CUDA(cudaMemcpyAsync(y, sigma, (size_t)t->n * t->n * sizeof(double2), cudaMemcpyHostToDevice, t->stream));
  if (t->precision == ZG_PREC_MIXED) ZG_TRY(launch_f64_to_f32(t->Y, t->y32, t->S, t->stream));
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  return ZG_OK;
}

int zg_get_state(zg_traj* t, int slot, double* host) {
  ZG_REQUIRE(t && host, "null argument");
  ZG_REQUIRE(slot >= 0 && slot <= t->stages, "slot %d out of range", slot);
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  const size_t bytes = t->S * sizeof(double2);
  const double2* src;
  if (t->precision == ZG_PREC_F64) {
    src = t->slot(slot);
  } else if (slot == t->stages) {
    src = t->Y;
  } else {
    ZG_TRY(ensure_conv64(t));
    ZG_TRY(launch_f32_to_f64(t->kslot(slot), t->conv64, t->S, t->stream));
    src = t->conv64;
  }
  ZG_CHECK_CUDA(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, t->stream));
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  return ZG_OK;
}

int zg_stage_input(zg_traj* t, int stage) {
  ZG_REQUIRE(t, "null argument");
  ZG_REQUIRE(stage >= 0 && stage < t->stages, "stage %d out of range", stage);
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  CombineCoefs cf;
  cf.n = 0;
  if (t->precision == ZG_PREC_F64) {
    if (stage == 0) {
      t->cur_in = t->slot(t->stages);
      return ZG_OK;
    }
    for (int j = 0; j <= t->stages; ++j) {
      double b = t->B[(size_t)stage * (t->stages + 1) + j];
      if (b != 0.0) { cf.idx[cf.n] = j; cf.c[cf.n] = b; ++cf.n; }
    }
    prof_begin(t, ZG_PROF_COMBINE);
    ZG_TRY(launch_combine_c128(t->Y, t->S, cf, t->Ystage, t->S, t->stream));
    prof_end(t, ZG_PROF_COMBINE);
    t->cur_in = t->Ystage;
    return ZG_OK;
  }
  // mixed: y32 + sum over k slots (y enters with weight B[i][stages] == 1)
  if (stage > 0)
    for (int j = 0; j < t->stages; ++j) {
      double b = t->B[(size_t)stage * (t->stages + 1) + j];
      if (b != 0.0) { cf.idx[cf.n] = j; cf.c[cf.n] = b; ++cf.n; }
    }
  prof_begin(t, ZG_PROF_COMBINE);
  ZG_TRY(launch_stage_input_mixed(t->y32, t->K32, t->S, cf, t->ml, t->stage32, t->stream));
  prof_end(t, ZG_PROF_COMBINE);
  t->cur_in = nullptr;
  return ZG_OK;
}

int zg_get_stage_sigma(zg_traj* t, double* host) {
  ZG_REQUIRE(t && host, "null argument");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  const double2* src = t->cur_in;
  if (t->precision == ZG_PREC_MIXED) {
    ZG_TRY(launch_f32_to_f64(t->stage32, t->sig64, (int64_t)t->n * t->n, t->stream));
    src = t->sig64;
  }
  ZG_CHECK_CUDA(cudaMemcpyAsync(host, src, (size_t)t->n * t->n * sizeof(double2), cudaMemcpyDeviceToHost, t->stream));
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  return ZG_OK;
}

static int sm1_times(zg_traj* t, const double2* X, double2* out);

int zg_set_dH(zg_traj* t, const double* host) {
  ZG_REQUIRE(t && host, "null argument");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  {
    bool real = true;
    for (int64_t e = 0; e < (int64_t)t->n * t->n && real; ++e) real = host[2 * e + 1] == 0.0;
    t->dH_raw_real = real;
    t->dH_real = real && (!t->nonorth || t->sm1_real);
  }
  ZG_CHECK_CUDA(cudaMemcpyAsync(t->dH, host, (size_t)t->n * t->n * sizeof(double2), cudaMemcpyHostToDevice,
                                t->stream));
  if (t->nonorth) ZG_TRY(sm1_times(t, t->dH, t->dHn));  // the stages add S^-1 dH
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  t->dH_set = true;
  return ZG_OK;
}

int zg_set_dissipator(zg_traj* t, const double* host) {
  ZG_REQUIRE(t, "null argument");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  if (!host) {
    t->dis_on = false;
    return ZG_OK;
  }
  if (!t->dis) ZG_TRY(dalloc(t, &t->dis, (size_t)t->n * t->n));
  ZG_CHECK_CUDA(cudaMemcpyAsync(t->dis, host, (size_t)t->n * t->n * sizeof(double2), cudaMemcpyHostToDevice,
                                t->stream));
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  t->dis_on = true;
  return ZG_OK;
}

static void gemm_prob_f64(std::vector<GemmProb<double>>& v, const double2* A, int64_t lda, int opA, const double2* B,
                          int64_t ldb, int opB, double2* C, int64_t ldc, int M, int N, int K) {
  GemmProb<double> P;
  P.A = A; P.A2 = nullptr; P.B = B; P.Cm = C; P.M = M; P.N = N; P.K = K; P.opA = opA; P.opB = opB;
  P.planeA = 0;
  P.lda = lda; P.ldb = ldb; P.ldc = ldc;
  P.alpha = make_double2(1.0, 0.0); P.beta = make_double2(0.0, 0.0);
  P.tile_begin = 0; P.tiles_n = 1;
  v.push_back(P);
}
// planeA > 0: A (and A2) are planar, element (r, c) = (A_f[i], A_f[i + planeA]) with i
// the element index, A_f the floats at A
static void gemm_prob_f32(std::vector<GemmProb<float>>& v, const float2* A, const float2* A2, int64_t lda, int opA,
                          const float2* B, int64_t ldb, int opB, float2* C, int64_t ldc, int M, int N, int K,
                          int64_t planeA = 0) {
  GemmProb<float> P;
  P.A = A; P.A2 = A2; P.B = B; P.Cm = C; P.M = M; P.N = N; P.K = K; P.opA = opA; P.opB = opB;
  P.planeA = planeA;
  P.lda = lda; P.ldb = ldb; P.ldc = ldc;
  P.alpha = make_float2(1.f, 0.f); P.beta = make_float2(0.f, 0.f);
  P.tile_begin = 0; P.tiles_n = 1;
  v.push_back(P);
}

}  // extern "C"

// split-K workspace of one precision, sized when the trajectory is created
// (plan_only pass); a later call that needs more (never, for fixed shapes)
// grows it outside of graph capture
template <typename R>
static int run_batches(zg_traj* t, std::vector<GemmProb<R>>& all, typename cx<R>::t** ws, int64_t* cap,
                       cudaStream_t s, bool plan_only) {
  // problems at most 32 wide (the n_c-wide products), and wide ones with a
  // short K (the xi sigma^T rows, K = n_c), run with 128x32 tiles in one
  // launch; the rest with 64x64 tiles
  auto narrow_p = [](const GemmProb<R>& P) { return P.N <= 32 || P.K <= 64; };
  std::vector<GemmProb<R>> probs;
  for (int pass = 0; pass < 2; ++pass)
    for (const auto& P : all)
      if (narrow_p(P) == (pass == 0)) probs.push_back(P);
  size_t narrow = 0;
  for (const auto& P : all) narrow += narrow_p(P);
  for (size_t b0 = 0; b0 < probs.size();) {
    GemmBatch<R> batch;
    const bool nar = b0 < narrow;
    batch.want_bn = nar ? 32 : 0;
    const size_t end = nar ? narrow : probs.size();
    batch.nprob = (int)std::min<size_t>(ZG_MAX_GEMM, end - b0);
    for (int i = 0; i < batch.nprob; ++i) batch.p[i] = probs[b0 + i];
    b0 += batch.nprob;
    const int64_t need = plan_zgemm_batch<R>(batch);
    if (need > *cap) {
      ZG_REQUIRE(!t->capturing, "split-K workspace must be sized before graph capture");
      ZG_CHECK_CUDA(cudaStreamSynchronize(s));
      dfree(t, *ws);
      *ws = nullptr;
      *cap = 0;
      ZG_TRY(dalloc(t, ws, need));
      *cap = need;
    }
    batch.ws = *ws;
    if (!plan_only) ZG_TRY(launch_zgemm_batch<R>(batch, *cap, s));
  }
  return ZG_OK;
}

extern "C" {

// p: device pointer to the stage parameters.  plan_only: build the GEMM
// problem list and size the split-K workspace, launch nothing.
static int rhs_f64(zg_traj* t, int stage, const StageParams* p, int dH_mode, double hubbard_U, bool want_J,
                   bool plan_only = false) {
  const RhsDev<double> d = t->dev_view<double>();
  const double2* in = plan_only ? t->slot(t->stages) : t->cur_in;
  const double2* sig = in;
  const double2* psi = in + t->off_psi;
  double2* out = t->slot(stage);
  cudaStream_t s = t->stream;
  const int64_t n = t->n, N = t->N, Ns = t->Ns, Nf = t->Nf, L = t->L, nc = t->nc;
  if (!plan_only) {
    prof_begin(t, ZG_PROF_PREP);
    if (t->nonorth)  // S^-1 H(t) (Zandpack/mpi/nozand:1075-1085)
      ZG_TRY(launch_build_ht((int)n, t->Hn0, sig, t->dHn, dH_mode, hubbard_U, t->Ht, s, t->Sm1));
    else
      ZG_TRY(launch_build_ht((int)n, t->H0, sig, t->dH, dH_mode, hubbard_U, t->Ht, s));
    ZG_TRY(launch_gathers<double>(d, sig, psi, nullptr, n, t->sigC, t->G, s));
    prof_end(t, ZG_PROF_PREP);
  }
  std::vector<GemmProb<double>> probs;
  // T = H(t) sigma ; R1 = psi H(t)^T into k_psi
  gemm_prob_f64(probs, t->Ht, n, 0, sig, n, 0, t->T, n, (int)n, (int)n, (int)n);
  gemm_prob_f64(probs, psi, n, 0, t->Ht, n, 1, out + t->off_psi, n, (int)N, (int)n, (int)n);
  for (int a = 0; a < L; ++a) {
    // PI partials: Pc[cls][a] = psi[rows]^T IXI[rows]
    int64_t r0 = t->s_start[a], r1 = t->s_start[a + 1];
    gemm_prob_f64(probs, psi + r0 * n, n, 1, t->IXI + r0 * nc, nc, 0, t->Pc + ((0 * L + a) * n) * nc, nc, (int)n,
                  (int)nc, (int)(r1 - r0));
    r0 = t->f_start[a]; r1 = t->f_start[a + 1];
    gemm_prob_f64(probs, psi + r0 * n, n, 1, t->IXI + r0 * nc, nc, 0, t->Pc + ((1 * L + a) * n) * nc, nc, (int)n,
                  (int)nc, (int)(r1 - r0));
    // R2 rows of lead a: XI[rows] sigC_a^T
    r0 = t->s_start[a]; r1 = t->s_start[a + 1];
    if (r1 > r0)
      gemm_prob_f64(probs, t->XI + r0 * nc, nc, 0, t->sigC + a * n * nc, nc, 1, t->R2 + r0 * n, n, (int)(r1 - r0),
                    (int)n, (int)nc);
    // Omega xi: ZA[a] = OmA[:, sourced of a] XIS[sourced of a]; ZB[a] = OmB[:, free of a] XIS[free of a]
    gemm_prob_f64(probs, in + t->off_omA + r0, Ns, 0, t->XIS + r0 * nc, nc, 0, t->ZA + a * N * nc, nc, (int)N,
                  (int)nc, (int)(r1 - r0));
    r0 = t->f_start[a]; r1 = t->f_start[a + 1];
    if (Ns > 0)
      gemm_prob_f64(probs, in + t->off_omB + (r0 - Ns), Nf, 0, t->XIS + r0 * nc, nc, 0, t->ZB + a * Ns * nc, nc,
                    (int)Ns, (int)nc, (int)(r1 - r0));
  }
  // non-orthogonal basis: W = P S^-1 and R3 = S^-1 (Omega xi'/hbar^2), K = L nc
  std::vector<GemmProb<double>> probs2;
  if (t->nonorth) {
    const int64_t K = L * nc;
    gemm_prob_f64(probs2, t->Qcat, K, 0, t->SmR, n, 0, t->Wn, n, (int)n, (int)n, (int)K);
    gemm_prob_f64(probs2, t->Zcat, K, 0, t->SmT, n, 0, t->R3, n, (int)N, (int)n, (int)K);
  }
  if (plan_only) {
    ZG_TRY(run_batches<double>(t, probs, &t->ws64, &t->ws64_cap, s, true));
    return run_batches<double>(t, probs2, &t->ws64, &t->ws64_cap, s, true);
  }
  prof_begin(t, ZG_PROF_GEMM);
  ZG_TRY(run_batches<double>(t, probs, &t->ws64, &t->ws64_cap, s, false));
  if (t->nonorth) {
    ZG_TRY(launch_nonorth_gather<double>(d, t->Pc, t->ZA, t->ZB, t->Qcat, t->Zcat, s));
    ZG_TRY(run_batches<double>(t, probs2, &t->ws64, &t->ws64_cap, s, false));
  }
  prof_end(t, ZG_PROF_GEMM);
  prof_begin(t, ZG_PROF_FINAL);
  ZG_TRY(launch_sigma_finalize<double>(d, p, t->T, n, t->Pc, t->dis_on ? t->dis : nullptr, out, s, 0, 0,
                                       t->nonorth ? t->Wn : nullptr));
  if (want_J) ZG_TRY(launch_currents<double>(d, p, t->Pc, t->J, s));
  ZG_TRY(launch_psi_finalize<double>(d, p, psi, nullptr, n, out + t->off_psi, n, t->R2, t->ZA, t->ZB,
                                     out + t->off_psi, s, 0, 0, 0, t->nonorth ? t->R3 : nullptr,
                                     t->nonorth ? t->C0 : nullptr));
  prof_end(t, ZG_PROF_FINAL);
  prof_begin(t, ZG_PROF_OMEGA);
  ZG_TRY(launch_omega<double>(d, p, t->tiles, t->ntiles, t->G, in + t->off_omA, in + t->off_omB, out + t->off_omA,
                              out + t->off_omB, s));
  prof_end(t, ZG_PROF_OMEGA);
  return ZG_OK;
}

static int rhs_mixed(zg_traj* t, int stage, const StageParams* p, int dH_mode, double hubbard_U, bool want_J,
                     bool plan_only = false) {
  const RhsDev<float> d = t->dev_view<float>();
  const MixedLayout& ml = t->ml;
  const float2* sig = t->stage32;
  // psi hi and lo, planar: real parts (N x np floats), then imaginary parts
  const float* psih_f = (const float*)(t->stage32 + ml.st_psih);
  const float* psil_f = (const float*)(t->stage32 + ml.st_psil);
  const bool hreal = t->h0_real && (dH_mode != ZG_DH_MATRIX || t->dH_real);
  const TcGemm& gR1 = hreal ? t->gR1 : t->gR1c;
  const TcGemm& gT = hreal ? t->gT : t->gTc;
  const float2* omA = t->stage32 + ml.st_om;
  const float2* omB = omA + (int64_t)t->N * t->Ns;
  float2* out = t->kslot(stage);
  cudaStream_t s = t->stream;
  const int64_t n = t->n, N = t->N, Ns = t->Ns, Nf = t->Nf, L = t->L, nc = t->nc, np = t->np;
  const int impl = t->prod_impl;
  if (!plan_only) {
    prof_begin(t, ZG_PROF_PREP);
    // H(t) = H0 + dH changes only on the diagonal unless dH is a full matrix
    int h_part = 0;
    if (dH_mode == ZG_DH_MATRIX || (t->nonorth && dH_mode == ZG_DH_HUBBARD)) {
      // a full matrix, or S^-1 diag(u): every entry changes
      t->h_offdiag_ready = false;
    } else if (t->h_offdiag_ready) {
      h_part = dH_mode == ZG_DH_HUBBARD || t->h_diag_mode != dH_mode ? 1 : 2;
    } else {
      t->h_offdiag_ready = true;
    }
    t->h_diag_mode = dH_mode;
    // operands of the tensor-core kernels the chosen implementation runs
    TcxOperands ops;
    if (impl >= ZG_IMPL_TC_PRODUCTS) {
      ops.sigEh = t->tcx_ops.sigEh;
      ops.sigEl = t->tcx_ops.sigEl;
      ops.ldx = t->tcx_ops.ldx;
    }
    if (impl == ZG_IMPL_TC_ALL || impl == ZG_IMPL_TC_SPLIT) {
      ops.Gth = t->Gth; ops.Gtl = t->Gtl; ops.Gch = t->Gch; ops.Gcl = t->Gcl;
    }
    ZG_TRY(launch_prep_mixed((int)n, (int)np, t->nonorth ? t->Hn0 : t->H0, sig, t->nonorth ? t->dHn : t->dH, dH_mode,
                             hubbard_U, h_part, t->Hth, t->Htl, t->BSh, t->BSl, t->nonorth ? t->Sm1 : nullptr, d,
                             (const float2*)psih_f, (const float2*)psil_f, np, t->sigC32, t->G32, ml.plane, s, ops));
    prof_end(t, ZG_PROF_PREP);
    // fork: T = H(t) sigma (tensor cores) and then the Omega derivative run on
    // the second stream, beside psi H(t)^T and the products (ZG_SCHED_EARLY)
    // or beside the products alone (ZG_SCHED_LATE)
    cudaStream_t s2 = t->stream2;
    if (t->sched == ZG_SCHED_EARLY) {
      ZG_CHECK_CUDA(cudaEventRecord(t->ev_fork, s));
      ZG_CHECK_CUDA(cudaStreamWaitEvent(s2, t->ev_fork, 0));
    }
    // tensor cores: R1 = psi H(t)^T
    prof_begin(t, ZG_PROF_GEMM);
    ZG_TRY(tc_gemm_launch(gR1, s));
    prof_end(t, ZG_PROF_GEMM);
    if (t->sched == ZG_SCHED_LATE) {
      ZG_CHECK_CUDA(cudaEventRecord(t->ev_fork, s));
      ZG_CHECK_CUDA(cudaStreamWaitEvent(s2, t->ev_fork, 0));
    }
    prof_begin(t, ZG_PROF_GEMM2, s2);
    ZG_TRY(tc_gemm_launch(gT, s2));
    prof_end(t, ZG_PROF_GEMM2, s2);
    prof_begin(t, ZG_PROF_OMEGA, s2);
    if (impl == ZG_IMPL_TC_SPLIT) {  // its own tensor-core launch
      TcxBatch* bo = t->tcx_om;
      bo->om_out_base = out;
      bo->params = p;
      ZG_TRY(tcx_launch(*bo, t->tcx_grid_om, s2));
    } else if (impl != ZG_IMPL_TC_ALL) {  // else it runs in the tensor-core batch below
      ZG_TRY(launch_omega<float>(d, p, t->tiles, t->ntiles, t->G32, omA, omB, out + t->off_omA, out + t->off_omB,
                                 s2));
    }
    prof_end(t, ZG_PROF_OMEGA, s2);
    ZG_CHECK_CUDA(cudaEventRecord(t->ev_join, s2));
  }
  // PI partials, xi sigma^T rows, Omega xi: on the tensor cores (t->tcx), else
  // as the SIMT FP32 batch
  std::vector<GemmProb<float>> probs;
  for (int a = 0; a < L && (plan_only || impl == ZG_IMPL_SIMT); ++a) {
    int64_t r0 = t->s_start[a], r1 = t->s_start[a + 1];
    gemm_prob_f32(probs, (const float2*)(psih_f + r0 * np), (const float2*)(psil_f + r0 * np), np, 1,
                  t->IXI32 + r0 * nc, nc, 0, t->Pc32 + ((0 * L + a) * n) * nc, nc, (int)n, (int)nc, (int)(r1 - r0),
                  ml.plane);
    r0 = t->f_start[a]; r1 = t->f_start[a + 1];
    gemm_prob_f32(probs, (const float2*)(psih_f + r0 * np), (const float2*)(psil_f + r0 * np), np, 1,
                  t->IXI32 + r0 * nc, nc, 0, t->Pc32 + ((1 * L + a) * n) * nc, nc, (int)n, (int)nc, (int)(r1 - r0),
                  ml.plane);
    r0 = t->s_start[a]; r1 = t->s_start[a + 1];
    if (r1 > r0)
      gemm_prob_f32(probs, t->XI32 + r0 * nc, nullptr, nc, 0, t->sigC32 + a * n * nc, nc, 1, t->R2_32 + r0 * n, n,
                    (int)(r1 - r0), (int)n, (int)nc);
    gemm_prob_f32(probs, omA + r0, nullptr, Ns, 0, t->XIS32 + r0 * nc, nc, 0, t->ZA32 + a * N * nc, nc, (int)N,
                  (int)nc, (int)(r1 - r0));
    r0 = t->f_start[a]; r1 = t->f_start[a + 1];
    if (Ns > 0)
      gemm_prob_f32(probs, omB + (r0 - Ns), nullptr, Nf, 0, t->XIS32 + r0 * nc, nc, 0, t->ZB32 + a * Ns * nc, nc,
                    (int)Ns, (int)nc, (int)(r1 - r0));
  }
  std::vector<GemmProb<float>> probs2;
  if (t->nonorth) {
    const int64_t K = L * nc;
    gemm_prob_f32(probs2, t->Qcat32, nullptr, K, 0, t->SmR32, n, 0, t->Wn32, n, (int)n, (int)n, (int)K);
    gemm_prob_f32(probs2, t->Zcat32, nullptr, K, 0, t->SmT32, n, 0, t->R3_32, n, (int)N, (int)n, (int)K);
  }
  if (plan_only) {
    ZG_TRY(run_batches<float>(t, probs, &t->ws32, &t->ws32_cap, s, true));
    return run_batches<float>(t, probs2, &t->ws32, &t->ws32_cap, s, true);
  }
  prof_begin(t, ZG_PROF_SMALL);
  if (impl != ZG_IMPL_SIMT) {
    TcxBatch* b = impl == ZG_IMPL_TC_ALL ? t->tcx_all : t->tcx;
    b->om_out_base = out;
    b->params = p;
    ZG_TRY(tcx_launch(*b, impl == ZG_IMPL_TC_ALL ? t->tcx_grid_all : t->tcx_grid, s));
  }
  else
    ZG_TRY(run_batches<float>(t, probs, &t->ws32, &t->ws32_cap, s, false));
  if (t->nonorth) {
    ZG_TRY(launch_nonorth_gather<float>(d, t->Pc32, t->ZA32, t->ZB32, t->Qcat32, t->Zcat32, s));
    ZG_TRY(run_batches<float>(t, probs2, &t->ws32, &t->ws32_cap, s, false));
  }
  prof_end(t, ZG_PROF_SMALL);
  // join: the finalisation needs T; the next stage overwrites what Omega reads
  ZG_CHECK_CUDA(cudaStreamWaitEvent(s, t->ev_join, 0));
  prof_begin(t, ZG_PROF_FINAL);
  // the lead terms of k_sigma go with the psi finalisation into one launch when the operands allow it
  const bool merged = final_mixed_ok(d, (const float2*)psih_f, (const float2*)psil_f, np, t->R1p, 2 * np, ml.plane,
                                     hreal ? 1 : 2, (int)np);
  // without a dissipator, k_sigma (lead terms included) and the psi finalisation share one launch
  const bool all_in_one = merged && !t->dis_on;
  if (!all_in_one)
    ZG_TRY(launch_sigma_finalize<float>(d, p, t->T32, 2 * np, t->Pc32, t->dis_on ? t->dis : nullptr, out, s,
                                        hreal ? 1 : 2, (int)np, t->nonorth ? t->Wn32 : nullptr, !merged));
  if (want_J) {
    if (stage == 0)  // the stage-0 input is y itself: currents from the FP64 state
    {
      CurRows rows;
      for (int a = 0; a <= L; ++a) { rows.s[a] = t->s_start[a]; rows.f[a] = t->f_start[a]; }
      ZG_TRY(launch_currents64((int)n, (int)L, (int)nc, rows, t->lead_cols, t->Y + t->off_psi, t->IXI, t->hbar,
                               t->Jpart, t->J, s));
    }
    else
      ZG_TRY(launch_currents<float>(d, p, t->Pc32, t->J, s));
  }
  if (all_in_one)
    ZG_TRY(launch_final_all_mixed(d, p, t->T32, 2 * np, hreal ? 1 : 2, t->nonorth ? t->Wn32 : nullptr, t->Pc32, out,
                                  (const float2*)psih_f, (const float2*)psil_f, np, t->R1p, 2 * np, t->R2_32,
                                  t->ZA32, t->ZB32, out + t->off_psi, ml.plane, hreal ? 1 : 2, (int)np,
                                  t->nonorth ? t->R3_32 : nullptr, t->nonorth ? t->C0_32 : nullptr, s));
  else if (merged)
    ZG_TRY(launch_final_mixed(d, p, t->nonorth ? nullptr : t->Pc32, out, (const float2*)psih_f,
                              (const float2*)psil_f, np, t->R1p, 2 * np, t->R2_32, t->ZA32, t->ZB32,
                              out + t->off_psi, ml.plane, hreal ? 1 : 2, (int)np, t->nonorth ? t->R3_32 : nullptr,
                              t->nonorth ? t->C0_32 : nullptr, s));
  else
    ZG_TRY(launch_psi_finalize<float>(d, p, (const float2*)psih_f, (const float2*)psil_f, np, t->R1p, 2 * np,
                                      t->R2_32, t->ZA32, t->ZB32, out + t->off_psi, s, ml.plane, hreal ? 1 : 2,
                                      (int)np, t->nonorth ? t->R3_32 : nullptr, t->nonorth ? t->C0_32 : nullptr));
  prof_end(t, ZG_PROF_FINAL);
  return ZG_OK;
}

int zg_rhs(zg_traj* t, int stage, double ts, double h, const double* delta, int dH_mode, double hubbard_U,
           double* currents) {
  ZG_REQUIRE(t && delta, "null argument");
  ZG_REQUIRE(stage >= 0 && stage < t->stages, "stage %d out of range", stage);
  ZG_REQUIRE(dH_mode == ZG_DH_NONE || dH_mode == ZG_DH_HUBBARD || (dH_mode == ZG_DH_MATRIX && t->dH_set),
             "bad dH mode %d (ZG_DH_MATRIX needs zg_set_dH first)", dH_mode);
  ZG_REQUIRE(t->precision == ZG_PREC_F64 || t->cur_in == nullptr, "zg_stage_input must precede zg_rhs");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  StageParams p;
  p.h = h; p.ts = ts; p.hbar = t->hbar;
  for (int a = 0; a < ZG_MAX_LEADS; ++a) p.delta[a] = a < t->L ? delta[a] : 0.0;
  derive_params(p);
  prof_begin(t, ZG_PROF_RHS);
  ZG_TRY(launch_set_params(p, t->d_params, t->stream));
  if (t->precision == ZG_PREC_F64)
    ZG_TRY(rhs_f64(t, stage, t->d_params, dH_mode, hubbard_U, currents != nullptr));
  else
    ZG_TRY(rhs_mixed(t, stage, t->d_params, dH_mode, hubbard_U, currents != nullptr));
  prof_end(t, ZG_PROF_RHS);
  if (currents) {
    ZG_CHECK_CUDA(cudaMemcpyAsync(currents, t->J, t->L * sizeof(double), cudaMemcpyDeviceToHost, t->stream));
    ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  }
  return ZG_OK;
}

// t->err[0..2] = squared error norms of sigma, psi, Omega (no host sync)
static int enqueue_error(zg_traj* t) {
  CombineCoefs cf;
  cf.n = 0;
  for (int j = 0; j < t->stages; ++j)
    if (t->CT[j] != 0.0) { cf.idx[cf.n] = j; cf.c[cf.n] = t->CT[j]; ++cf.n; }
  const int64_t seg[4] = {0, t->off_psi, t->off_omA, t->S};
  prof_begin(t, ZG_PROF_ERROR);
  for (int k = 0; k < 3; ++k) {
    double* part = t->partial + (int64_t)k * t->nblk_err;
    if (t->precision == ZG_PREC_F64)
      ZG_TRY(launch_terr2_partials_c128(t->Y, t->S, cf, seg[k], seg[k + 1], part, t->nblk_err, t->stream));
    else
      ZG_TRY(launch_terr2_partials_mixed(t->K32, t->S, cf, seg[k], seg[k + 1], part, t->nblk_err, t->stream));
  }
  ZG_TRY(launch_reduce_partials(t->partial, t->nblk_err, 3, t->err, t->stream));
  prof_end(t, ZG_PROF_ERROR);
  return ZG_OK;
}

// y <- sum_j CH_j Y_j, skipped on the device when gate != null and *gate == 0
static int enqueue_update(zg_traj* t, const int* gate) {
  CombineCoefs cf;
  cf.n = 0;
  prof_begin(t, ZG_PROF_UPDATE);
  if (t->precision == ZG_PREC_F64) {
    for (int j = 0; j <= t->stages; ++j)
      if (t->CH[j] != 0.0) { cf.idx[cf.n] = j; cf.c[cf.n] = t->CH[j]; ++cf.n; }
    ZG_TRY(launch_step_fourth_c128(t->Y, t->S, t->stages, cf, t->S, t->stream, gate));
  } else {
    for (int j = 0; j < t->stages; ++j)
      if (t->CH[j] != 0.0) { cf.idx[cf.n] = j; cf.c[cf.n] = t->CH[j]; ++cf.n; }
    ZG_TRY(launch_update_mixed(t->Y, t->y32, t->K32, t->S, cf, t->S, t->stream, gate));
  }
  prof_end(t, ZG_PROF_UPDATE);
  return ZG_OK;
}

int zg_error_norm2(zg_traj* t, double* err2) {
  ZG_REQUIRE(t && err2, "null argument");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  ZG_TRY(enqueue_error(t));
  ZG_CHECK_CUDA(cudaMemcpyAsync(err2, t->err, 3 * sizeof(double), cudaMemcpyDeviceToHost, t->stream));
  int herr = 0;
  if (t->tc_err) ZG_CHECK_CUDA(cudaMemcpyAsync(&herr, t->tc_err, sizeof(int), cudaMemcpyDeviceToHost, t->stream));
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  prof_collect(t);
  if (herr != 0) {
    set_error("a bounded wait in the tensor-core GEMM gave up (code %d)", herr);
    return ZG_ETIMEOUT;
  }
  return ZG_OK;
}

int zg_step_fourth(zg_traj* t) {
  ZG_REQUIRE(t, "null argument");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  ZG_TRY(enqueue_update(t, nullptr));
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  return ZG_OK;
}

}  // extern "C"

static int presize_workspaces(zg_traj* t) {
  if (t->precision == ZG_PREC_F64) return rhs_f64(t, 0, t->d_params, ZG_DH_NONE, 0.0, false, true);
  return rhs_mixed(t, 0, t->d_params, ZG_DH_NONE, 0.0, false, true);
}

// out = S^-1 X (n x n, FP64, on the trajectory's stream)
static int sm1_times(zg_traj* t, const double2* X, double2* out) {
  std::vector<GemmProb<double>> pr;
  const int n = t->n;
  gemm_prob_f64(pr, t->Sm1, n, 0, X, n, 0, out, n, n, n, n);
  return run_batches<double>(t, pr, &t->ws64, &t->ws64_cap, t->stream, false);
}

extern "C" int zg_set_overlap(zg_traj* t, const double* Sm1, const double* C0) {
  ZG_REQUIRE(t, "null argument");
  ZG_REQUIRE(!Sm1 || C0, "the constant term C0 comes with S^-1");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  drop_graph(t);  // captured stages hold the old operands
  t->h_offdiag_ready = false;
  if (!Sm1) {
    t->nonorth = false;
    t->h0_real = t->h0_real_orth;
    t->dH_real = t->dH_raw_real;
    return ZG_OK;
  }
  const int64_t n = t->n, N = t->N, L = t->L, nc = t->nc, K = L * nc;
  const double2* S = (const double2*)Sm1;
  bool real = true;
  for (int64_t e = 0; e < n * n && real; ++e) real = S[e].y == 0.0;
  t->sm1_real = real;
  // S^-1 rows (SmR) and columns (SmT) at the coupling orbitals; padding rows zero
  std::vector<double2> R((size_t)(K * n), make_double2(0, 0)), Tt((size_t)(K * n), make_double2(0, 0));
  for (int64_t a = 0; a < L; ++a)
    for (int64_t k = 0; k < nc; ++k) {
      const int c = t->lead_cols_h[a * nc + k];
      if (t->colmap_h[a * n + c] != k) continue;
      for (int64_t j = 0; j < n; ++j) {
        R[(a * nc + k) * n + j] = S[c * n + j];
        Tt[(a * nc + k) * n + j] = S[j * n + c];
      }
    }
  if (!t->Sm1) {
    ZG_TRY(dalloc(t, &t->Sm1, n * n));
    ZG_TRY(dalloc(t, &t->Hn0, n * n));
    ZG_TRY(dalloc(t, &t->dHn, n * n));
    ZG_TRY(dalloc(t, &t->C0, N * n));
    if (t->precision == ZG_PREC_F64) {
      ZG_TRY(dalloc(t, &t->SmR, K * n)); ZG_TRY(dalloc(t, &t->SmT, K * n));
      ZG_TRY(dalloc(t, &t->Qcat, n * K)); ZG_TRY(dalloc(t, &t->Wn, n * n));
      ZG_TRY(dalloc(t, &t->Zcat, N * K)); ZG_TRY(dalloc(t, &t->R3, N * n));
    } else {
      ZG_TRY(dalloc(t, &t->SmR32, K * n)); ZG_TRY(dalloc(t, &t->SmT32, K * n)); ZG_TRY(dalloc(t, &t->C0_32, N * n));
      ZG_TRY(dalloc(t, &t->Qcat32, n * K)); ZG_TRY(dalloc(t, &t->Wn32, n * n));
      ZG_TRY(dalloc(t, &t->Zcat32, N * K)); ZG_TRY(dalloc(t, &t->R3_32, N * n));
    }
  }
  cudaStream_t s = t->stream;
  ZG_TRY(upload<double2>(t->Sm1, Sm1, n * n, s));
  ZG_TRY(upload<double2>(t->C0, C0, N * n, s));
  std::vector<float2> R32, T32, C32;
  if (t->precision == ZG_PREC_F64) {
    ZG_TRY(upload<double2>(t->SmR, R.data(), K * n, s));
    ZG_TRY(upload<double2>(t->SmT, Tt.data(), K * n, s));
  } else {
    R32.resize(K * n); T32.resize(K * n); C32.resize(N * n);
    to_f32(R.data(), R32.data(), K * n);
    to_f32(Tt.data(), T32.data(), K * n);
    to_f32((const double2*)C0, C32.data(), N * n);
    ZG_TRY(upload<float2>(t->SmR32, R32.data(), K * n, s));
    ZG_TRY(upload<float2>(t->SmT32, T32.data(), K * n, s));
    ZG_TRY(upload<float2>(t->C0_32, C32.data(), N * n, s));
  }
  ZG_TRY(sm1_times(t, t->H0, t->Hn0));
  if (t->dH_set) ZG_TRY(sm1_times(t, t->dH, t->dHn));
  t->nonorth = true;
  t->h0_real = t->h0_real_orth && t->sm1_real;
  t->dH_real = t->dH_raw_real && t->sm1_real;
  ZG_TRY(presize_workspaces(t));
  // the host vectors above must outlive their asynchronous copies
  ZG_CHECK_CUDA(cudaStreamSynchronize(s));
  return ZG_OK;
}

// One attempt with the controller on the device, enqueued without host syncs
// (the body of the attempt graph): stages, error norm, control, gated update,
// advance, then the controller and the tensor-core error flag to pinned memory.
static int enqueue_attempt_device(zg_traj* t) {
  cudaStream_t s = t->stream;
  // every stage's time, step size and biases at once (they depend only on the
  // controller's t and h, which change at the end of the attempt)
  StageNodes nodes;
  for (int i = 0; i < t->stages; ++i) nodes.A[i] = t->A[i];
  ZG_TRY(launch_stage_prologues(t->ctl, t->gbias, nodes, t->stages, t->hbar, t->d_params, s));
  for (int i = 0; i < t->stages; ++i) {
    ZG_TRY(zg_stage_input(t, i));
    prof_begin(t, ZG_PROF_RHS);
    if (t->precision == ZG_PREC_F64)
      ZG_TRY(rhs_f64(t, i, t->d_params + i, t->g_dH_mode, t->g_U, i == 0));
    else
      ZG_TRY(rhs_mixed(t, i, t->d_params + i, t->g_dH_mode, t->g_U, i == 0));
    prof_end(t, ZG_PROF_RHS);
  }
  ZG_TRY(enqueue_error(t));
  ZG_TRY(launch_control(t->err, t->ctl, s));
  ZG_TRY(enqueue_update(t, &t->ctl->accepted));
  ZG_TRY(launch_advance(t->ctl, t->J, t->L, t->d_recs, ZG_GRAPH_MAX_BATCH, s));
  return ZG_OK;
}

// The attempt graph rebuilds only the diagonal of the mixed path's H(t)
// operands: make sure their off-diagonal part holds H0 before it runs (a
// host-driven stage with a full dH matrix may have overwritten it).
static int ensure_h_operands(zg_traj* t) {
  if (t->precision != ZG_PREC_MIXED || t->h_offdiag_ready) return ZG_OK;
  ZG_TRY(launch_build_operands_mixed(t->n, t->np, t->nonorth ? t->Hn0 : t->H0, t->stage32,
                                     t->nonorth ? t->dHn : t->dH, t->g_dH_mode, t->g_U, 0, t->Hth, t->Htl, t->BSh,
                                     t->BSl, t->stream, t->nonorth ? t->Sm1 : nullptr));
  t->h_offdiag_ready = true;
  t->h_diag_mode = t->g_dH_mode;
  return ZG_OK;
}

static int capture_attempt_graph(zg_traj* t) {
  drop_graph(t);
  ZG_TRY(ensure_h_operands(t));
  if (t->precision == ZG_PREC_MIXED && t->h_diag_mode != t->g_dH_mode) {
    // the captured stages then skip (NONE) or rebuild (HUBBARD) the diagonal
    t->h_offdiag_ready = false;
    ZG_TRY(ensure_h_operands(t));
  }
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  const long long k0 = t_launches;
  ZG_CHECK_CUDA(cudaStreamBeginCapture(t->stream, cudaStreamCaptureModeThreadLocal));
  t->capturing = true;
  const int st = enqueue_attempt_device(t);
  t->capturing = false;
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(t->stream, &g);
  // nothing ran during capture: take the captured kernels off the launch count
  t->graph_kernels = t_launches - k0;
  g_launches.fetch_sub(t->graph_kernels);
  t_launches = k0;
  if (st != ZG_OK) {
    if (g) cudaGraphDestroy(g);
    t->graph_kernels = 0;
    return st;
  }
  if (ce != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    t->graph_kernels = 0;
    set_error("attempt graph capture failed: %s", cudaGetErrorString(ce));
    return ZG_ECUDA;
  }
  t->graph = g;
  const cudaError_t ie = cudaGraphInstantiate(&t->gexec, g, 0);
  if (ie != cudaSuccess) {
    t->gexec = nullptr;
    drop_graph(t);
    set_error("attempt graph instantiation failed: %s", cudaGetErrorString(ie));
    return ZG_ECUDA;
  }
  return ZG_OK;
}

static double bias_value(const zg_bias& b, double t, int a) {
  double V = 0.0;
  switch (b.kind) {
    case ZG_BIAS_ZERO: V = 0.0; break;
    case ZG_BIAS_EXP_RAMP: V = b.V0 * (1.0 - exp(-t / b.tau)); break;
    case ZG_BIAS_GAUSS: V = b.V0 * exp(-(t - b.tc) * (t - b.tc) / (2.0 * b.sigma * b.sigma)); break;
    case ZG_BIAS_SIN: V = b.V0 * sin(2.0 * M_PI * b.f * t); break;
    case ZG_BIAS_STEP: V = t > 0.0 ? b.V0 : 0.0; break;
    case ZG_BIAS_BOX: V = b.V0 * (tanh(t / b.tau) - tanh((t - b.tc) / b.tau)) / 2.0; break;
    default: V = 0.0;
  }
  return b.w[a] * V;
}

extern "C" {

int zg_attempt(zg_traj* t, double* time, double* h, double eps, const zg_bias* bias, int dH_mode, double hubbard_U,
               double* TE, int* accepted, double* currents) {
  ZG_REQUIRE(t && time && h && bias && TE && accepted, "null argument");
  ZG_REQUIRE(dH_mode == ZG_DH_NONE || dH_mode == ZG_DH_HUBBARD, "zg_attempt needs dH_mode NONE or HUBBARD");
  ZG_REQUIRE(!t->dis_on, "a dissipator is applied through zg_rhs only: call zg_set_dissipator(t, NULL) first");
  ZG_REQUIRE(bias->kind >= ZG_BIAS_ZERO && bias->kind <= ZG_BIAS_BOX, "unknown bias kind %d", bias->kind);
  const double t0 = *time, h0 = *h;
  double delta[ZG_MAX_LEADS];
  for (int i = 0; i < t->stages; ++i) {
    ZG_TRY(zg_stage_input(t, i));
    const double ts = t0 + t->A[i] * h0;
    for (int a = 0; a < ZG_MAX_LEADS; ++a) delta[a] = a < t->L ? bias_value(*bias, ts, a) : 0.0;
    ZG_TRY(zg_rhs(t, i, ts, h0, delta, dH_mode, hubbard_U, (i == 0 && currents) ? currents : nullptr));
  }
  double e2[3];
  ZG_TRY(zg_error_norm2(t, e2));
  const double te = sqrt(e2[0] + e2[1] + e2[2]);
  *TE = te;
  if (!std::isfinite(te)) {
    set_error("error norm is not finite (%g)", te);
    return ZG_ENONFINITE;
  }
  const int acc = te < eps;
  *accepted = acc;
  // h <- 0.9 h (eps/TE)^(1/5) (Zandpack/mpi_RK4pars_dev.py:148-149), after every attempt
  const double hn = te > 0.0 ? 0.9 * h0 * pow(eps / te, 0.2) : INFINITY;
  if (acc) {
    ZG_TRY(zg_step_fourth(t));
    *time = t0 + hn;  // the reference advances by the step size proposed next
  }
  *h = hn;
  return ZG_OK;
}

int zg_get_sigma(zg_traj* t, int slot, double* host) {
  ZG_REQUIRE(t && host, "null argument");
  ZG_REQUIRE(slot >= 0 && slot <= t->stages, "slot %d out of range", slot);
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  const int64_t nn = (int64_t)t->n * t->n;
  const double2* src;
  if (t->precision == ZG_PREC_F64) {
    src = t->slot(slot);
  } else if (slot == t->stages) {
    src = t->Y;
  } else {
    ZG_TRY(launch_f32_to_f64(t->kslot(slot), t->sig64, nn, t->stream));
    src = t->sig64;
  }
  ZG_CHECK_CUDA(cudaMemcpyAsync(host, src, nn * sizeof(double2), cudaMemcpyDeviceToHost, t->stream));
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  return ZG_OK;
}

int zg_graph_prepare(zg_traj* t, const zg_bias* bias, int dH_mode, double hubbard_U) {
  ZG_REQUIRE(t && bias, "null argument");
  ZG_REQUIRE(dH_mode == ZG_DH_NONE || dH_mode == ZG_DH_HUBBARD, "the attempt graph needs dH_mode NONE or HUBBARD");
  ZG_REQUIRE(!t->dis_on, "a dissipator is applied through zg_rhs only: call zg_set_dissipator(t, NULL) first");
  ZG_REQUIRE(bias->kind >= ZG_BIAS_ZERO && bias->kind <= ZG_BIAS_BOX, "unknown bias kind %d", bias->kind);
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  t->gbias = *bias;
  for (int a = t->L; a < ZG_MAX_LEADS; ++a) t->gbias.w[a] = 0.0;
  t->g_dH_mode = dH_mode;
  t->g_U = hubbard_U;
  t->g_prepared = false;
  ZG_TRY(capture_attempt_graph(t));
  t->g_prepared = true;
  return ZG_OK;
}

int zg_graph_set(zg_traj* t, double time, double h, double eps, double t1) {
  ZG_REQUIRE(t, "null argument");
  ZG_REQUIRE(h > 0.0 && eps > 0.0 && std::isfinite(time) && std::isfinite(h), "bad controller values");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  DevCtl c;
  memset(&c, 0, sizeof(c));
  c.t = time; c.h = h; c.eps = eps; c.t1 = t1;
  c.done = time >= t1 ? 1 : 0;
  *t->ctl_host = c;
  ZG_CHECK_CUDA(cudaMemcpyAsync(t->ctl, t->ctl_host, sizeof(DevCtl), cudaMemcpyHostToDevice, t->stream));
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  return ZG_OK;
}

int zg_graph_run(zg_traj* t, int count, zg_attempt_rec* recs, int* nrec, double* time, double* h, int* done) {
  ZG_REQUIRE(t, "null argument");
  ZG_REQUIRE(count >= 0 && count <= ZG_GRAPH_MAX_BATCH, "count %d out of range", count);
  ZG_REQUIRE(t->g_prepared, "zg_graph_prepare must precede zg_graph_run");
  ZG_REQUIRE(!t->dis_on, "a dissipator is applied through zg_rhs only: call zg_set_dissipator(t, NULL) first");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  if (!t->gexec) ZG_TRY(capture_attempt_graph(t));  // dropped by zg_set_tableau or zg_profile
  if (t->precision == ZG_PREC_MIXED && (!t->h_offdiag_ready || t->h_diag_mode != t->g_dH_mode)) {
    t->h_offdiag_ready = false;
    ZG_TRY(ensure_h_operands(t));
  }
  cudaStream_t s = t->stream;
  ZG_CHECK_CUDA(cudaMemsetAsync(&t->ctl->rec_n, 0, sizeof(int), s));
  for (int i = 0; i < count; ++i) {
    ZG_CHECK_CUDA(cudaGraphLaunch(t->gexec, s));
    g_launches.fetch_add(t->graph_kernels, std::memory_order_relaxed);
  }
  ZG_CHECK_CUDA(cudaMemcpyAsync(t->ctl_host, t->ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, s));
  ZG_CHECK_CUDA(cudaMemcpyAsync(t->recs_host, t->d_recs, (size_t)count * sizeof(zg_attempt_rec),
                                cudaMemcpyDeviceToHost, s));
  if (t->tc_err) ZG_CHECK_CUDA(cudaMemcpyAsync(t->tcerr_host, t->tc_err, sizeof(int), cudaMemcpyDeviceToHost, s));
  ZG_CHECK_CUDA(cudaStreamSynchronize(s));
  if (count > 0) graph_prof_collect(t);  // regions of the last attempt of the batch
  const DevCtl& c = *t->ctl_host;
  const int n = std::min(c.rec_n, count);
  if (recs && n > 0) memcpy(recs, t->recs_host, (size_t)n * sizeof(zg_attempt_rec));
  if (nrec) *nrec = n;
  if (time) *time = c.t;
  if (h) *h = c.h;
  if (done) *done = c.done;
  if (t->tc_err && *t->tcerr_host != 0) {
    set_error("a bounded wait in the tensor-core GEMM gave up (code %d)", *t->tcerr_host);
    return ZG_ETIMEOUT;
  }
  if (c.status != ZG_OK) {
    set_error("error norm is not finite (%g)", c.TE);
    return c.status;
  }
  return ZG_OK;
}

// ------------------------------------------------------------ steady state
int zg_stationary_setup(zg_traj* t, double ts, const double* delta, int dH_mode, double hubbard_U, const double* V,
                        const double* lam) {
  ZG_REQUIRE(t && delta && V && lam, "null argument");
  ZG_REQUIRE(t->precision == ZG_PREC_F64, "the steady state is solved on an FP64 trajectory");
  ZG_REQUIRE(!t->nonorth, "the steady state is solved in the orthogonal basis (no overlap set)");
  ZG_REQUIRE(dH_mode == ZG_DH_NONE || dH_mode == ZG_DH_HUBBARD || (dH_mode == ZG_DH_MATRIX && t->dH_set),
             "bad dH mode %d (ZG_DH_MATRIX needs zg_set_dH first)", dH_mode);
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  const size_t nn = (size_t)t->n * t->n;
  if (!t->st_V) {
    ZG_TRY(dalloc(t, &t->st_V, nn));
    ZG_TRY(dalloc(t, &t->st_Vc, nn));
    ZG_TRY(dalloc(t, &t->st_W, (size_t)t->N * t->n));
    ZG_TRY(dalloc(t, &t->st_lam, (size_t)t->n));
    ZG_TRY(dalloc(t, &t->st_delta, ZG_MAX_LEADS));
  }
  std::vector<double2> Vc(nn);
  const double2* Vh = (const double2*)V;
  for (size_t e = 0; e < nn; ++e) Vc[e] = cconj(Vh[e]);
  t->st_p.h = 1.0;
  t->st_p.ts = ts;
  t->st_p.hbar = t->hbar;
  for (int a = 0; a < ZG_MAX_LEADS; ++a) t->st_p.delta[a] = a < t->L ? delta[a] : 0.0;
  derive_params(t->st_p);
  ZG_CHECK_CUDA(cudaMemcpyAsync(t->st_V, V, nn * sizeof(double2), cudaMemcpyHostToDevice, t->stream));
  ZG_CHECK_CUDA(cudaMemcpyAsync(t->st_Vc, Vc.data(), nn * sizeof(double2), cudaMemcpyHostToDevice, t->stream));
  ZG_CHECK_CUDA(cudaMemcpyAsync(t->st_lam, lam, (size_t)t->n * sizeof(double), cudaMemcpyHostToDevice, t->stream));
  ZG_CHECK_CUDA(cudaMemcpyAsync(t->st_delta, t->st_p.delta, ZG_MAX_LEADS * sizeof(double), cudaMemcpyHostToDevice,
                                t->stream));
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  t->st_mode = dH_mode;
  t->st_U = hubbard_U;
  t->st_ready = true;
  return ZG_OK;
}

int zg_stationary_apply(zg_traj* t, const double* psi_dev, double* kpsi_dev) {
  ZG_REQUIRE(t && psi_dev && kpsi_dev, "null argument");
  ZG_REQUIRE(t->st_ready, "zg_stationary_setup must precede zg_stationary_apply");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  cudaStream_t s = t->stream;
  double2* y = t->slot(t->stages);
  const int64_t n = t->n, N = t->N;
  // y = (sigma, psi, Omega(psi)); Omega from dOmega/dt = 0 given psi
  ZG_CHECK_CUDA(cudaMemcpyAsync(y + t->off_psi, psi_dev, (size_t)N * n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  ZG_TRY(launch_set_params(t->st_p, t->d_params, s));
  const RhsDev<double> d = t->dev_view<double>();
  ZG_TRY(launch_gathers<double>(d, y, y + t->off_psi, nullptr, n, t->sigC, t->G, s));
  ZG_TRY(launch_omega<double>(d, t->d_params, t->tiles, t->ntiles, t->G, y + t->off_omA, y + t->off_omB,
                              y + t->off_omA, y + t->off_omB, s, 1));
  // k_psi of that state with h = 1: zero at the steady state
  ZG_TRY(zg_stage_input(t, 0));
  ZG_TRY(launch_set_params(t->st_p, t->d_params, s));
  ZG_TRY(rhs_f64(t, 0, t->d_params, t->st_mode, t->st_U, false));
  ZG_CHECK_CUDA(cudaMemcpyAsync(kpsi_dev, t->slot(0) + t->off_psi, (size_t)N * n * sizeof(double2),
                                cudaMemcpyDeviceToDevice, s));
  ZG_CHECK_CUDA(cudaStreamSynchronize(s));
  return ZG_OK;
}

int zg_stationary_precond(zg_traj* t, const double* r_dev, double* out_dev) {
  ZG_REQUIRE(t && r_dev && out_dev, "null argument");
  ZG_REQUIRE(t->st_ready, "zg_stationary_setup must precede zg_stationary_precond");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  cudaStream_t s = t->stream;
  const int64_t n = t->n, N = t->N;
  // out_m = i hbar r_m (H^T - x_m)^{-1} = i hbar [(r_m conj V) / (lam - x_m)] V^T
  std::vector<GemmProb<double>> p1, p2;
  gemm_prob_f64(p1, (const double2*)r_dev, n, 0, t->st_Vc, n, 0, t->st_W, n, (int)N, (int)n, (int)n);
  ZG_TRY(run_batches<double>(t, p1, &t->ws64, &t->ws64_cap, s, false));
  ZG_TRY(launch_stationary_scale((int)N, (int)n, t->Xp, t->mode_lead, t->st_delta, t->st_lam, t->hbar, t->st_W, s));
  gemm_prob_f64(p2, t->st_W, n, 0, t->st_V, n, 1, (double2*)out_dev, n, (int)N, (int)n, (int)n);
  ZG_TRY(run_batches<double>(t, p2, &t->ws64, &t->ws64_cap, s, false));
  ZG_CHECK_CUDA(cudaStreamSynchronize(s));
  return ZG_OK;
}

static int impl_mask(const zg_traj* t) {
  if (t->precision != ZG_PREC_MIXED) return 1 << ZG_IMPL_SIMT;
  return (1 << ZG_IMPL_SIMT) | (t->tcx_on ? 1 << ZG_IMPL_TC_PRODUCTS : 0) | (t->tcx_all ? 1 << ZG_IMPL_TC_ALL : 0) |
         (t->tcx_on && t->tcx_om ? 1 << ZG_IMPL_TC_SPLIT : 0);
}

int zg_set_impl(zg_traj* t, int impl) {
  ZG_REQUIRE(t, "null argument");
  ZG_REQUIRE(impl >= 0 && impl < ZG_IMPL_COUNT && (impl_mask(t) >> impl & 1),
             "implementation %d not available for this trajectory (mask %d)", impl, impl_mask(t));
  if (t->prod_impl != impl) {
    drop_graph(t);
    t->prod_impl = impl;
  }
  return ZG_OK;
}

int zg_set_schedule(zg_traj* t, int sched) {
  ZG_REQUIRE(t, "null argument");
  ZG_REQUIRE(sched == ZG_SCHED_LATE || sched == ZG_SCHED_EARLY, "schedule %d", sched);
  if (t->sched != sched) {
    drop_graph(t);
    t->sched = sched;
  }
  return ZG_OK;
}

int zg_get_schedule(const zg_traj* t, int* sched) {
  ZG_REQUIRE(t && sched, "null argument");
  *sched = t->sched;
  return ZG_OK;
}

int zg_get_impl(const zg_traj* t, int* impl, int* avail) {
  ZG_REQUIRE(t, "null argument");
  if (impl) *impl = t->prod_impl;
  if (avail) *avail = impl_mask(t);
  return ZG_OK;
}

int zg_tune(zg_traj* t, int reps, int* best, double* ms) {
  ZG_REQUIRE(t && reps >= 1 && reps <= 1000, "bad arguments");
  ZG_REQUIRE(!t->capturing, "zg_tune during graph capture");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  const int mask = impl_mask(t);
  constexpr int NV = ZG_IMPL_COUNT * ZG_SCHED_COUNT;
  double times[NV];
  for (int i = 0; i < NV; ++i) times[i] = -1.0;
  if (t->precision != ZG_PREC_MIXED) {
    if (best) *best = t->prod_impl + ZG_IMPL_COUNT * t->sched;
    if (ms) for (int i = 0; i < NV; ++i) ms[i] = times[i];
    return ZG_OK;
  }
  StageParams p;
  memset(&p, 0, sizeof(p));
  p.h = 1e-3; p.ts = 0.0; p.hbar = t->hbar;
  derive_params(p);
  cudaEvent_t e0, e1;
  ZG_CHECK_CUDA(cudaEventCreate(&e0));
  ZG_CHECK_CUDA(cudaEventCreate(&e1));
  int st = ZG_OK;
  int choice = t->prod_impl + ZG_IMPL_COUNT * t->sched;
  double tbest = 1e300;
  for (int v = 0; v < NV && st == ZG_OK; ++v) {
    const int impl = v % ZG_IMPL_COUNT, sched = v / ZG_IMPL_COUNT;
    if (!(mask >> impl & 1)) continue;
    st = zg_set_impl(t, impl);
    if (st == ZG_OK) st = zg_set_schedule(t, sched);
    if (st == ZG_OK) st = zg_stage_input(t, 0);
    if (st == ZG_OK) st = launch_set_params(p, t->d_params, t->stream);
    if (st == ZG_OK) st = rhs_mixed(t, 0, t->d_params, ZG_DH_NONE, 0.0, false);  // untimed
    if (st != ZG_OK) break;
    cudaEventRecord(e0, t->stream);
    for (int r = 0; r < reps && st == ZG_OK; ++r) st = rhs_mixed(t, 0, t->d_params, ZG_DH_NONE, 0.0, false);
    cudaEventRecord(e1, t->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      set_error("tuning run failed: %s", cudaGetErrorString(cudaGetLastError()));
      st = ZG_ECUDA;
      break;
    }
    float el = 0.f;
    cudaEventElapsedTime(&el, e0, e1);
    times[v] = el / reps;
    if (times[v] < tbest) {
      tbest = times[v];
      choice = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != ZG_OK) return st;
  ZG_TRY(zg_set_impl(t, choice % ZG_IMPL_COUNT));
  ZG_TRY(zg_set_schedule(t, choice / ZG_IMPL_COUNT));
  if (best) *best = choice;
  if (ms) for (int i = 0; i < NV; ++i) ms[i] = times[i];
  return ZG_OK;
}

int zg_profile(zg_traj* t, int enable) {
  ZG_REQUIRE(t, "null argument");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  auto& P = t->prof;
  if (enable && !P.created) {
    for (int r = 0; r < ZG_PROF_REGIONS; ++r)
      for (int i = 0; i < P.RING; ++i) {
        ZG_CHECK_CUDA(cudaEventCreate(&P.b[r][i]));
        ZG_CHECK_CUDA(cudaEventCreate(&P.e[r][i]));
      }
    P.created = true;
  }
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  prof_collect(t);
  if (P.on != (enable != 0)) drop_graph(t);  // recaptured with or without event nodes
  P.on = enable != 0;
  for (int r = 0; r < ZG_PROF_REGIONS; ++r) { P.ms[r] = 0; P.cnt[r] = 0; }
  return ZG_OK;
}

int zg_profile_read(zg_traj* t, double* ms, long long* count) {
  ZG_REQUIRE(t && ms && count, "null argument");
  ZG_CHECK_CUDA(cudaSetDevice(t->dev));
  ZG_CHECK_CUDA(cudaStreamSynchronize(t->stream));
  prof_collect(t);
  for (int r = 0; r < ZG_PROF_REGIONS; ++r) { ms[r] = t->prof.ms[r]; count[r] = t->prof.cnt[r]; }
  return ZG_OK;
}

int zg_measure_fp64_mma(int device, double* gflops) {
  ZG_REQUIRE(gflops, "null argument");
  ZG_CHECK_CUDA(cudaSetDevice(device));
  return measure_dmma(gflops);
}

int zg_measure_peaks(int device, double* out) {
  ZG_REQUIRE(out, "null argument");
  ZG_CHECK_CUDA(cudaSetDevice(device));
  return measure_peaks(out);
}

// ------------------------------------------------------------ array kernels
static int coefs_from(CombineCoefs& cf, const double* c, const int32_t* idx, int nidx, int nslots) {
  ZG_REQUIRE(nidx >= 0 && nidx <= ZG_MAX_STAGES + 1, "too many terms (%d)", nidx);
  cf.n = 0;
  for (int t = 0; t < nidx; ++t) {
    int j = idx ? idx[t] : t;
    ZG_REQUIRE(j >= 0 && j < nslots, "index %d out of range", j);
    cf.idx[cf.n] = j;
    cf.c[cf.n] = c[j];
    ++cf.n;
  }
  return ZG_OK;
}

int zg_combine_c128(const double* Y, int64_t slot_stride, int nslots, const double* b, const int32_t* idx, int nidx,
                    double* out, int64_t count, void* stream) {
  ZG_REQUIRE(b && count >= 0 && slot_stride >= count && (count == 0 || (Y && out)), "bad arguments");
  CombineCoefs cf;
  ZG_TRY(coefs_from(cf, b, idx, nidx, nslots));
  return launch_combine_c128((const double2*)Y, slot_stride, cf, (double2*)out, count, (cudaStream_t)stream);
}

int zg_terr2_c128(const double* Y, int64_t slot_stride, int nslots, const double* ct, int64_t count, double* result,
                  void* stream) {
  ZG_REQUIRE(ct && result && count >= 0 && slot_stride >= count && (count == 0 || Y), "bad arguments");
  ZG_REQUIRE(nslots >= 1 && nslots <= ZG_MAX_STAGES + 1, "nslots %d out of range", nslots);
  CombineCoefs cf;
  ZG_TRY(coefs_from(cf, ct, nullptr, nslots, nslots));
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = terr2_nblocks(count);
  double* scratch = nullptr;  // nb partial sums + 1 result
  ZG_CHECK_CUDA(cudaMallocAsync((void**)&scratch, (nb + 1) * sizeof(double), s));
  int st = launch_terr2_partials_c128((const double2*)Y, slot_stride, cf, 0, count, scratch, nb, s);
  if (st == ZG_OK) st = launch_reduce_partials(scratch, nb, 1, scratch + nb, s);
  cudaError_t e = cudaSuccess;
  if (st == ZG_OK) e = cudaMemcpyAsync(result, scratch + nb, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(scratch, s);
  if (st != ZG_OK) return st;
  if (e != cudaSuccess) { set_error("copy of the result failed: %s", cudaGetErrorString(e)); return ZG_ECUDA; }
  ZG_CHECK_CUDA(cudaStreamSynchronize(s));
  return ZG_OK;
}

int zg_step_fourth_c128(double* Y, int64_t slot_stride, int nslots, const double* ch, int64_t count, void* stream) {
  ZG_REQUIRE(ch && count >= 0 && slot_stride >= count && (count == 0 || Y), "bad arguments");
  ZG_REQUIRE(nslots >= 1 && nslots <= ZG_MAX_STAGES + 1, "nslots %d out of range", nslots);
  CombineCoefs cf;
  ZG_TRY(coefs_from(cf, ch, nullptr, nslots, nslots));
  return launch_step_fourth_c128((double2*)Y, slot_stride, nslots - 1, cf, count, (cudaStream_t)stream);
}

}  // extern "C"
