// Allocation-free entry point for the plain hafnian sieve: wg_hafnian_noalloc.
//
// Who needs it: callers that must not allocate device memory during a call -- code that runs
// inside an application's own memory arena or pool (where a cudaMalloc would bypass the pool's
// accounting or fail against its reservation), plugins in serving processes that forbid
// allocation on the request path, and latency-critical loops where cudaMalloc/cudaFree would
// synchronise the device.  They own their input and output buffers already; this entry point
// brings its own working memory instead of allocating it.
//
// How: the scratch that the sieve needs beyond its inputs and outputs -- the instance
// descriptor, the chunk queue, the per-chunk partial sums, the output scale and the work
// counter -- lives in a file-scope static __device__ array of WG_NOALLOC_SCRATCH_BYTES bytes.
// Every GPU that loads this library holds that array until the process exits.  A small setup
// kernel writes the descriptor (passed by value as a kernel argument) and the chunk table into
// the array on the device, so a call performs no allocation, no host-to-device copy and no
// host heap allocation: three kernel launches on the caller's stream.
//
// Rules for callers:
//  * inputs and outputs are DEVICE pointers on the current device;
//  * the first call on a device resolves the array's device address (cudaGetSymbolAddress)
//    and uploads the constant tables; make that first call before any stream capture;
//  * every call shares the one array, so calls whose kernels overlap on the GPU (different
//    streams, or threads without ordering) race and corrupt each other's sums: serialise them.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/walrus_gb300.h"
#include "host_common.h"
#include "sieve_kernel.cuh"

namespace wg {
void set_last_error(const char* msg);  // defined with wg_last_error()

namespace noalloc {

constexpr size_t kScratchBytes = WG_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];
static __device__ LbLane g_lane_tab[(LB_KMAX + 1) * 32];
static __device__ LbOwner g_own_tab[(LB_KMAX + 1) * (LB_KMAX + 1)];
static __device__ LbLane2 g_lane2_tab[LB2_IDS * 32];
static __device__ LbOwner2 g_own2_tab[LB2_IDS * (LB2_KMAX + 1)];

// byte offsets inside g_scratch
constexpr size_t kOffInst = 0;
constexpr size_t kOffScale = 1024;
constexpr size_t kOffCounter = 1280;
constexpr size_t kOffChunks = 1536;
constexpr int kMaxChunks = (int)((kScratchBytes - kOffChunks) / (sizeof(ChunkDev) + sizeof(double2)));
static_assert(sizeof(InstDev) <= kOffScale, "descriptor slot too small");

struct DeviceState {
  bool ready = false;
  unsigned char* scratch = nullptr;  // device address of g_scratch
  LbLane* lanes = nullptr;
  LbOwner* own = nullptr;
  LbLane2* lanes2 = nullptr;
  LbOwner2* own2 = nullptr;
  int sms = 0;
};
static DeviceState g_dev[kMaxDevices];
static std::mutex g_mu;

static int err(int code, const char* what) {
  set_last_error(what);  // reported by wg_last_error()
  return code;
}

// Once per device, with that device current: resolve the static arrays' device addresses and
// upload the constant tables of this translation unit.
static int setup(int dev, DeviceState** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceState& s = g_dev[dev];
  if (!s.ready) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess) return err(WG_ECUDA, "cudaGetSymbolAddress(scratch) failed");
    s.scratch = (unsigned char*)p;
    if (cudaGetSymbolAddress(&p, g_lane_tab) != cudaSuccess) return err(WG_ECUDA, "cudaGetSymbolAddress(lane table) failed");
    s.lanes = (LbLane*)p;
    if (cudaGetSymbolAddress(&p, g_own_tab) != cudaSuccess) return err(WG_ECUDA, "cudaGetSymbolAddress(owner table) failed");
    s.own = (LbOwner*)p;
    if (cudaGetSymbolAddress(&p, g_lane2_tab) != cudaSuccess) return err(WG_ECUDA, "cudaGetSymbolAddress(lane2 table) failed");
    s.lanes2 = (LbLane2*)p;
    if (cudaGetSymbolAddress(&p, g_own2_tab) != cudaSuccess) return err(WG_ECUDA, "cudaGetSymbolAddress(owner2 table) failed");
    s.own2 = (LbOwner2*)p;
    static double binom[BINOM_N][BINOM_N];
    for (int i = 0; i < BINOM_N; ++i)
      for (int j = 0; j < BINOM_N; ++j) {
        long double b = j > i ? 0 : 1;
        for (int q = 0; q < j && j <= i; ++q) b = b * (long double)(i - q) / (long double)(q + 1);
        binom[i][j] = (double)b;
      }
    static double inv[256];
    inv[0] = 0;
    for (int k = 1; k < 256; ++k) inv[k] = 1.0 / (double)k;
    static LbLane lanes[(LB_KMAX + 1) * 32];
    static LbOwner own[(LB_KMAX + 1) * (LB_KMAX + 1)];
    for (int k = 0; k <= LB_KMAX; ++k)
      if (!lb_schedule(k, &lanes[k * 32], &own[k * (LB_KMAX + 1)])) return err(WG_EINVAL, "no La Budde schedule");
    static LbLane2 lanes2[LB2_IDS * 32];
    static LbOwner2 own2[LB2_IDS * (LB2_KMAX + 1)];
    if (!lb_schedule2_all(lanes2, own2)) return err(WG_EINVAL, "no La Budde schedule");
    if (sieve_tables_all(&binom[0][0], inv) != cudaSuccess ||
        cudaMemcpyToSymbol(g_lane_tab, lanes, sizeof(lanes)) != cudaSuccess ||
        cudaMemcpyToSymbol(g_own_tab, own, sizeof(own)) != cudaSuccess ||
        cudaMemcpyToSymbol(g_lane2_tab, lanes2, sizeof(lanes2)) != cudaSuccess ||
        cudaMemcpyToSymbol(g_own2_tab, own2, sizeof(own2)) != cudaSuccess)
      return err(WG_ECUDA, "uploading the constant tables failed");
    if (cudaDeviceGetAttribute(&s.sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return err(WG_ECUDA, "cudaDeviceGetAttribute failed");
    s.ready = true;
  }
  *out = &s;
  return WG_OK;
}

// Writes the descriptor, the output scale, a zeroed work counter and the chunk table into the
// scratch array (whatever an earlier call left there is overwritten or not read).
static __global__ void noalloc_setup_kernel(unsigned char* scratch, const InstDev inst, double scale, int nchunks) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c == 0) {
    *reinterpret_cast<InstDev*>(scratch + kOffInst) = inst;
    *reinterpret_cast<double*>(scratch + kOffScale) = scale;
    *reinterpret_cast<unsigned int*>(scratch + kOffCounter) = 0u;
  }
  if (c < nchunks) {
    ChunkDev ch;
    ch.inst = 0;
    ch.part = c;
    // chunk c = [q c + min(c, r), q (c+1) + min(c+1, r)) with steps = q nchunks + r: no product
    // exceeds steps, so nothing overflows for any accepted term count
    const long long q = inst.steps / nchunks, r = inst.steps % nchunks;
    ch.t0 = q * c + (c < r ? c : r);
    ch.t1 = q * (c + 1) + (c + 1 < r ? c + 1 : r);
    reinterpret_cast<ChunkDev*>(scratch + kOffChunks)[c] = ch;
  }
}

}  // namespace noalloc
}  // namespace wg

using namespace wg;
using namespace wg::noalloc;

extern "C" int wg_hafnian_noalloc(const void* A_dev, int n, int dtype, const int64_t* edge_reps, int E, int glynn,
                                  double* out_dev, void* stream) {
  if (!A_dev || !out_dev || !edge_reps) return err(WG_EINVAL, "NULL argument");
  // the kernels read A in 8-byte words and write the output pair in one 16-byte access
  if (((uintptr_t)A_dev & 7u) != 0) return err(WG_EINVAL, "A must be 8-byte aligned");
  if (((uintptr_t)out_dev & 15u) != 0) return err(WG_EINVAL, "out must be 16-byte aligned");
  if (dtype != WG_FLOAT64 && dtype != WG_COMPLEX128) return err(WG_EINVAL, "dtype must be WG_FLOAT64 or WG_COMPLEX128");
  if (E < 1 || n != 2 * E) return err(WG_EINVAL, "the prepared matrix must be 2E x 2E with E >= 1");
  if (E > MAX_EDGES)
    return err(WG_EINVAL, "size beyond the maximum: at most 32 edges (a 64 x 64 matrix) per call");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return err(WG_ECUDA, "no current CUDA device");
  DeviceState* ds = nullptr;
  int rc = setup(dev, &ds);
  if (rc) return rc;

  InstDev d;
  memset(&d, 0, sizeof(d));
  long long sumr = 0, steps = 1;
  int maxr = 0, nnz = 0;
  for (int i = 0; i < E; ++i) {
    const long long r = edge_reps[i];
    if (r < 0 || r > BINOM_N - 1) return err(WG_EINVAL, "edge repetitions must lie in 0..64");
    sumr += r;
    maxr = r > maxr ? (int)r : maxr;
    nnz += r > 0;
    const int R = (i == 0 && glynn) ? (int)(r + 2) / 2 : (int)r + 1;
    d.radix[i] = R;
    d.reps[i] = (int)r;
    if (steps > (1LL << 62) / R) return err(WG_EINVAL, "too many sieve terms");
    steps *= R;
  }
  d.kind = KIND_PLAIN;
  d.n = n;
  d.E = E;
  d.glynn = glynn ? 1 : 0;
  d.N = (int)(2 * sumr);
  d.K = d.N / 2;
  d.nout = 1;
  d.half_first = d.glynn;
  d.unit_binoms = maxr <= 1;
  d.lda = n;  // the caller's n x n matrix is read in place
  d.a_off = 0;
  d.steps = steps;
  d.nchunks = 0;  // set below
  const int st = dtype == WG_COMPLEX128 ? ST_CPLX64 : ST_REAL64;
  const int m_max = 2 * nnz;
  if (sumr == 0) return err(WG_EINVAL, "no photons (every edge repetition is 0): the hafnian is 1, no sieve to run");
  if (d.K > 250) return err(WG_EINVAL, "size beyond the maximum: photon number above 250");
  if (!tile_rows_ok(st, m_max)) return err(WG_EINVAL, "size beyond the maximum: term matrix too large");
  bool all_odd = d.glynn != 0;
  for (int i = 0; i < E; ++i) all_odd = all_odd && (edge_reps[i] % 2 == 1);
  const WarpLayout L = make_layout(st, m_max, m_max, std::min(d.K, m_max), d.K + 2, 2,
                                   all_odd && d.K < m_max);
  // the same launch shape as wg_hafnian's for this workspace
  const std::pair<int, int> sh = best_shape(st, L.bytes, kDefaultWarpsPerCta);
  const int wpc = sh.first, per_sm = sh.second;
  if (wpc < 1) return err(WG_EINVAL, "size beyond the maximum: per-warp workspace does not fit");
  if (per_sm < 1) return err(WG_ECUDA, "sieve kernel cannot be resident");
  const long long resident = (long long)ds->sms * per_sm * wpc;
  long long nch = std::min<long long>(steps, 4 * resident);
  if (nch > kMaxChunks) nch = kMaxChunks;  // larger chunks: the scratch bounds the queue
  d.nchunks = (int)nch;
  d.part_base = 0;
  d.out_base = 0;
  d.scale_base = 0;
  const double scale = d.glynn ? std::ldexp(1.0, -(d.N / 2 - 1)) : 1.0;

  cudaStream_t s = (cudaStream_t)stream;
  unsigned char* scr = ds->scratch;
  const size_t off_parts = kOffChunks + sizeof(ChunkDev) * (size_t)nch;
  const size_t off_parts_al = (off_parts + 15) & ~(size_t)15;
  if (off_parts_al + sizeof(double2) * (size_t)nch > kScratchBytes)
    return err(WG_EINVAL, "size beyond the maximum: scratch array too small");
  noalloc_setup_kernel<<<(int)((nch + 255) / 256), 256, 0, s>>>(scr, d, scale, (int)nch);
  if (cudaGetLastError() != cudaSuccess) return err(WG_ECUDA, "setup kernel launch failed");

  SieveParams p;
  p.lb_lane = ds->lanes;
  p.lb_own = ds->own;
  p.lb_lane2 = ds->lanes2;
  p.lb_own2 = ds->own2;
  p.inst = reinterpret_cast<const InstDev*>(scr + kOffInst);
  p.chunks = reinterpret_cast<const ChunkDev*>(scr + kOffChunks);
  p.nchunks = (int)nch;
  p.pool = reinterpret_cast<const unsigned char*>(A_dev);
  p.partials = reinterpret_cast<double2*>(scr + off_parts_al);
  p.counter = reinterpret_cast<unsigned int*>(scr + kOffCounter);
  p.err = nullptr;
  p.L = L;
  const int ctas = (int)std::max<long long>(1, std::min<long long>((long long)ds->sms * per_sm, (nch + wpc - 1) / wpc));
  const cudaError_t e = sieve_launch(st, p, ctas, wpc, s);
  if (e != cudaSuccess) return err(WG_ECUDA, "sieve kernel launch failed");
  reduce_kernel<<<1, 32, 0, s>>>(p.inst, 1, p.partials, reinterpret_cast<const double*>(scr + kOffScale),
                                 reinterpret_cast<double2*>(out_dev), p.counter, 1, 1, 0u);
  if (cudaGetLastError() != cudaSuccess) return err(WG_ECUDA, "reduction kernel launch failed");
  return WG_OK;
}
