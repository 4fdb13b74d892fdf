// Host runtime and C ABI of the hafnian sieve (see include/walrus_gb300.h).
//
// A plan turns a list of prepared instances into
//   * one device pool holding each instance's extended matrix [[A, D], [D^T, 0], [oddV], [oddV0]]
//     converted to the kernel's scalar type,
//   * a chunk queue: every instance's term range split into chunks whose cost is balanced
//     against the number of resident warps, largest instances first,
//   * one persistent sieve launch per (scalar type, resident warps per SM) group, and one reduction
//     launch that sums chunk partials in a fixed order (bitwise reproducible results).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/walrus_gb300.h"
#include "host_common.h"
#include "sieve_kernel.cuh"
#include "state_glue.cuh"

namespace wg {

static thread_local std::string g_err;
// Per-device state: the selected device, and for every device the SM count and the La Budde
// schedule tables in its memory (the constant tables live in each device's copy of the module).
static int g_device = -1;
static int g_num_sms = 0;  // of g_device
constexpr int kMaxDev = 64;
struct DevTables {
  bool ready = false;
  int sms = 0;
  LbLane* lane = nullptr;
  LbOwner* own = nullptr;
  LbLane2* lane2 = nullptr;
  LbOwner2* own2 = nullptr;
};
static DevTables g_dev[kMaxDev];

static std::mutex g_init_mu;

// lets other translation units of the library report through wg_last_error()
void set_last_error(const char* msg) { g_err = msg; }

static int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(x)                                                                                   \
  do {                                                                                          \
    cudaError_t e_ = (x);                                                                       \
    if (e_ != cudaSuccess) return fail(WG_ECUDA, "%s: %s (%s:%d)", #x, cudaGetErrorString(e_), \
                                       __FILE__, __LINE__);                                     \
  } while (0)

static int ensure_init(int device) {
  std::lock_guard<std::mutex> lk(g_init_mu);
  if (g_device >= 0 && (device < 0 || device == g_device)) {
    CK(cudaSetDevice(g_device));
    return WG_OK;
  }
  int dev = device < 0 ? 0 : device;
  int count = 0;
  CK(cudaGetDeviceCount(&count));
  if (count <= 0) return fail(WG_ECUDA, "no CUDA device");
  if (dev >= count || dev >= kMaxDev) return fail(WG_EINVAL, "device %d not present (%d devices)", dev, count);
  CK(cudaSetDevice(dev));
  DevTables& T = g_dev[dev];
  if (T.ready) {
    g_device = dev;
    g_num_sms = T.sms;
    return WG_OK;
  }
  CK(cudaDeviceGetAttribute(&T.sms, cudaDevAttrMultiProcessorCount, dev));
  // stream-ordered plans (one-shot calls, serving batches) allocate from this process's default
  // pool of the device: keep up to 256 MiB of freed memory there instead of releasing it to the
  // CUDA driver at every synchronisation, so a repeated call reuses it
  cudaMemPool_t pool;
  CK(cudaDeviceGetDefaultMemPool(&pool, dev));
  unsigned long long keep = 256ull << 20;
  CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  // constant tables: binomials and reciprocals
  static double binom[BINOM_N][BINOM_N];
  for (int i = 0; i < BINOM_N; ++i)
    for (int j = 0; j < BINOM_N; ++j) {
      if (j > i) { binom[i][j] = 0; continue; }
      long double b = 1;
      for (int q = 0; q < j; ++q) b = b * (long double)(i - q) / (long double)(q + 1);
      binom[i][j] = (double)b;
    }
  double inv[256];
  inv[0] = 0;
  for (int k = 1; k < 256; ++k) inv[k] = 1.0 / (double)k;
  CK(sieve_tables_all(&binom[0][0], inv));
  // La Budde lane schedules for every triangle size (built once, kept for the process lifetime)
  std::vector<LbLane> lanes((LB_KMAX + 1) * 32);
  std::vector<LbOwner> own((LB_KMAX + 1) * (LB_KMAX + 1));
  for (int k = 0; k <= LB_KMAX; ++k)
    if (!lb_schedule(k, &lanes[k * 32], &own[k * (LB_KMAX + 1)]))
      return fail(WG_EINVAL, "no La Budde schedule for %d coefficients", k);
  CK(cudaMalloc(&T.lane, sizeof(LbLane) * lanes.size()));
  CK(cudaMalloc(&T.own, sizeof(LbOwner) * own.size()));
  CK(cudaMemcpy(T.lane, lanes.data(), sizeof(LbLane) * lanes.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(T.own, own.data(), sizeof(LbOwner) * own.size(), cudaMemcpyHostToDevice));
  std::vector<LbLane2> lanes2(LB2_IDS * 32);
  std::vector<LbOwner2> own2(LB2_IDS * (LB2_KMAX + 1));
  if (!lb_schedule2_all(lanes2.data(), own2.data())) return fail(WG_EINVAL, "no two-row La Budde schedule");
  CK(cudaMalloc(&T.lane2, sizeof(LbLane2) * lanes2.size()));
  CK(cudaMalloc(&T.own2, sizeof(LbOwner2) * own2.size()));
  CK(cudaMemcpy(T.lane2, lanes2.data(), sizeof(LbLane2) * lanes2.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(T.own2, own2.data(), sizeof(LbOwner2) * own2.size(), cudaMemcpyHostToDevice));
  T.ready = true;
  g_device = dev;
  g_num_sms = T.sms;
  return WG_OK;
}


struct Prepared {
  InstDev d;
  int stype;
  int rows_max, mb_max, m_max, kc_max, nser_need, narr;
  bool tile_ok;  // every term can keep its La Budde rows in dead tile columns
  double term_cost;
  std::vector<double> scales;
  std::vector<unsigned char> ext;  // extended matrix in the kernel's scalar type (empty: formed on device)
  size_t ext_bytes = 0;
  long long t_lo = 0, t_hi = 0;  // sieve terms [t_lo, t_hi) of this instance
};

struct Group {
  int stype;
  WarpLayout L;
  int wpc, ctas;
  int chunk_begin, chunk_count;
};

}  // namespace wg

struct wg_plan {
  std::vector<wg::InstDev> inst;
  std::vector<wg::ChunkDev> chunks;
  std::vector<wg::Group> groups;
  int total_out = 0;
  int nparts = 0;
  long long h2d_bytes = 0;
  int precision = 0;
  void* dmem = nullptr;
  wg::InstDev* d_inst = nullptr;
  wg::ChunkDev* d_chunks = nullptr;
  unsigned char* d_pool = nullptr;
  double2* d_partials = nullptr;
  double* d_scales = nullptr;
  double2* d_out = nullptr;
  double* d_mag = nullptr;  // per output: sum |prefactor x term| x |final scale|
  unsigned int* d_counters = nullptr;
  int* d_err = nullptr;
  bool use_graph = false;
  cudaGraphExec_t graph_exec = nullptr;
  long long device_bytes = 0;
  bool async_alloc = false;
  cudaStream_t alloc_stream = nullptr;
  // groups after the first run on side streams forked from the caller's stream, so that one
  // group's persistent launch fills the SMs that another's tail leaves idle
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> side_done;
  cudaEvent_t fork = nullptr;
  int device = 0;  // the device the plan's memory and tables live on
  bool serial_groups = false;
};

struct wg_state {
  int M = 0;
  wg::c64* d_B = nullptr;
  wg::c64* d_gamma = nullptr;
  std::vector<wg::c64> gamma;  // host copy: self-loop weights of unpaired modes
  double alpha = 1.0;          // double-float prescale (power of two, from ||B||_inf)
};

namespace wg {



static inline void put_scalar(unsigned char* dst, int st, double re, double im) {
  if (stype_mod(st)) {  // integer below 2^31 in magnitude (checked in prepare), Montgomery form
    const long long p = (long long)MOD_PRIMES[st - ST_MOD0];
    long long r = (long long)re % p;
    const uint64_t x = (uint64_t)(r < 0 ? r + p : r);
    const uint32_t v = (uint32_t)((x << 32) % (uint64_t)p);
    memcpy(dst, &v, 4);
    return;
  }
  switch (st) {
    case ST_REAL64: memcpy(dst, &re, 8); break;
    case ST_CPLX64: memcpy(dst, &re, 8); memcpy(dst + 8, &im, 8); break;
    case ST_REALDF: {
      float h = (float)re, l = (float)(re - (double)h);
      memcpy(dst, &h, 4); memcpy(dst + 4, &l, 4);
      break;
    }
    case ST_REALDD: {  // the input double is the high part exactly
      const double z = 0.0;
      memcpy(dst, &re, 8); memcpy(dst + 8, &z, 8);
      break;
    }
    case ST_CPLXDD: {
      const double z = 0.0;
      memcpy(dst, &re, 8); memcpy(dst + 8, &z, 8); memcpy(dst + 16, &im, 8); memcpy(dst + 24, &z, 8);
      break;
    }
    default: {
      float h = (float)re, l = (float)(re - (double)h);
      float hi = (float)im, li = (float)(im - (double)hi);
      memcpy(dst, &h, 4); memcpy(dst + 4, &l, 4); memcpy(dst + 8, &hi, 4); memcpy(dst + 12, &li, 4);
      break;
    }
  }
}

static inline bool prec_mod(int precision) { return precision >= WG_PREC_MOD0 && precision <= WG_PREC_MOD4; }

// 2^-e as the output scale: the FP64 value, or (modular precisions) the residue of 2^-e mod p
static inline double pow2_scale(int e, int precision) {
  if (!prec_mod(precision)) return std::ldexp(1.0, -e);
  const uint64_t p = MOD_PRIMES[precision - WG_PREC_MOD0], half = (p + 1) / 2;
  uint64_t r = 1;
  for (int i = 0; i < e; ++i) r = r * half % p;
  return (double)r;
}

static inline void get_val(const void* p, int dtype, size_t idx, double& re, double& im) {
  const double* d = (const double*)p;
  if (dtype == WG_COMPLEX128) { re = d[2 * idx]; im = d[2 * idx + 1]; }
  else { re = d[idx]; im = 0.0; }
}

static int prepare(const wg_instance& in, int precision, Prepared& P) {
  memset(&P.d, 0, sizeof(P.d));
  InstDev& d = P.d;
  if (in.dtype != WG_FLOAT64 && in.dtype != WG_COMPLEX128) return fail(WG_EINVAL, "dtype must be WG_FLOAT64 or WG_COMPLEX128");
  if (in.n < 0 || in.E < 0) return fail(WG_EINVAL, "negative size");
  if (in.n > 0 && !in.A) return fail(WG_EINVAL, "A is NULL");
  std::vector<int> reps;
  int kind = in.kind;
  int nb = 0, ne = 0;
  if (kind == WG_KIND_PLAIN || kind == WG_KIND_LOOP) {
    if (in.n != 2 * in.E) return fail(WG_EINVAL, "prepared matrix must be 2E x 2E (n=%d, E=%d)", in.n, in.E);
    for (int i = 0; i < in.E; ++i) reps.push_back((int)in.edge_reps[i]);
    if (kind == WG_KIND_LOOP) {
      nb = 1;
      if (!in.D) return fail(WG_EINVAL, "D is NULL");
      if (in.has_odd) {
        ne = 1;
        if (!in.oddV) return fail(WG_EINVAL, "oddV is NULL");
        kind = KIND_LOOP_ODD;
      }
    }
  } else if (kind == WG_KIND_BATCH_EVEN || kind == WG_KIND_BATCH_ODD) {
    const bool odd = kind == WG_KIND_BATCH_ODD;
    const int nbe = odd ? 2 : 1;
    if (in.n != 2 * (in.E + nbe)) return fail(WG_EINVAL, "batch matrix must be 2(E+%d) square", nbe);
    if (!in.D) return fail(WG_EINVAL, "D is NULL");
    if (in.batch_max < 0 || in.cutoff < 0 || in.cutoff > 1) return fail(WG_EINVAL, "bad batch_max / cutoff");
    reps.push_back(in.batch_max);
    if (odd) reps.push_back(1);
    for (int i = 0; i < in.E; ++i) reps.push_back((int)in.edge_reps[i]);
    nb = 1;
    ne = odd ? 2 : 1;
  } else {
    return fail(WG_EINVAL, "unknown kind %d", in.kind);
  }
  const int E = (int)reps.size();
  if (E > MAX_EDGES) return fail(WG_EINVAL, "at most %d edges per sieve (got %d)", MAX_EDGES, E);
  long long sumr = 0;
  int maxr = 0;
  for (int r : reps) {
    if (r < 0) return fail(WG_EINVAL, "negative edge repetition");
    if (r > BINOM_N - 1) return fail(WG_EINVAL, "edge repetition %d above the supported %d", r, BINOM_N - 1);
    sumr += r;
    maxr = std::max(maxr, r);
  }
  d.kind = kind;
  d.n = in.n;
  d.E = E;
  d.glynn = in.glynn ? 1 : 0;
  d.nb = nb;
  d.ne = ne;
  d.lda = in.n + 1;
  d.unit_binoms = maxr <= 1;
  int nout = 1;
  double alpha = 1.0;  // input prescale (double-float only): A -> alpha A, D -> sqrt(alpha) D
  if (precision == WG_PREC_DF) {
    double rs = 0;
    for (int i = 0; i < in.n; ++i) {
      double s = 0, re, im;
      for (int j = 0; j < in.n; ++j) { get_val(in.A, in.dtype, (size_t)i * in.n + j, re, im); s += std::hypot(re, im); }
      rs = std::max(rs, s);
    }
    if (rs > 0 && std::isfinite(rs)) alpha = std::exp2(-std::round(std::log2(rs)));
  }
  const double salpha = std::sqrt(alpha);
  int Nf = 0;
  if (kind == KIND_PLAIN || kind == KIND_LOOP) {
    d.N = (int)(2 * sumr);
    d.K = d.N / 2;
    d.Nodd = 0;
    d.half_first = d.glynn;
    const int e = d.glynn ? d.N / 2 - 1 : 0;
    P.scales.push_back(pow2_scale(e, precision) * std::pow(alpha, -0.5 * d.N));
  } else if (kind == KIND_LOOP_ODD) {
    d.N = (int)(2 * sumr + 1);
    d.K = d.N / 2;
    d.Nodd = d.N;
    d.half_first = 0;
    const int e = d.glynn ? d.N / 2 : 0;
    P.scales.push_back(pow2_scale(e, precision) * std::pow(alpha, -0.5 * d.N));
    d.oddloop = {in.oddloop[0] * salpha, in.oddloop[1] * salpha};
  } else {
    const bool odd = kind == KIND_BATCH_ODD;
    long long sf = 0;
    for (int i = 0; i < in.E; ++i) sf += in.edge_reps[i];
    Nf = (int)(2 * sf + (odd ? 1 : 0));
    const int Nmax = odd ? Nf + 2 * in.batch_max + in.cutoff + 1 : Nf + 2 * in.batch_max + in.cutoff;
    nout = odd ? 2 * in.batch_max + in.cutoff + 2 : 2 * in.batch_max + in.cutoff + 1;
    if (nout > 32) return fail(WG_EINVAL, "batch output length %d above 32", nout);
    d.N = Nf;
    d.K = Nmax / 2;
    d.Nodd = Nmax;
    d.batch_max = in.batch_max;
    d.half_first = 0;
    double re, im;
    get_val(in.D, in.dtype, 0, re, im);
    d.oddloop = {re * salpha, im * salpha};
    if (odd) {
      get_val(in.D, in.dtype, 1, re, im);
      d.oddloop0 = {re * salpha, im * salpha};
    }
    for (int o = 0; o < nout; ++o) {
      const int x = Nf + o;
      P.scales.push_back(pow2_scale(d.glynn ? x / 2 : 0, precision) * std::pow(alpha, -0.5 * x));
    }
  }
  d.nout = nout;
  long long steps = 1;
  for (int i = 0; i < E; ++i) {
    const int R = (i == 0 && d.half_first) ? (reps[0] + 2) / 2 : reps[i] + 1;
    d.radix[i] = R;
    d.reps[i] = reps[i];
    if (steps > (1LL << 62) / R) return fail(WG_EINVAL, "too many sieve terms");
    steps *= R;
  }
  d.steps = steps;
  if (in.term_begin == 0 && in.term_end == 0) {
    P.t_lo = 0;
    P.t_hi = steps;
  } else {
    if (in.term_begin < 0 || in.term_end < in.term_begin || in.term_end > steps)
      return fail(WG_EINVAL, "term range [%lld, %lld) outside the %lld sieve terms", (long long)in.term_begin,
                  (long long)in.term_end, steps);
    P.t_lo = in.term_begin;
    P.t_hi = in.term_end;
  }
  // term matrix size bounds
  const int m_max = 2 * (int)std::count_if(reps.begin(), reps.end(), [](int r) { return r > 0; });
  P.m_max = m_max;
  P.mb_max = m_max + nb;
  P.rows_max = m_max + nb + ne;
  P.kc_max = std::min(d.K, m_max);
  // plain kinds keep det coefficients and the series (K + 1 each); loop kinds also the odd
  // series (Nodd, Nf) and the border series and their weights (K + 1 each)
  P.nser_need = kind == KIND_PLAIN ? d.K + 2 : std::max(std::max(d.K, d.Nodd), Nf) + 2;
  P.narr = (kind == KIND_PLAIN) ? 2 : 8;
  {
    // a term with m < K+1 and no border/extra rows has columns shorter than Kc+1: only when
    // some delta can vanish (an even repetition, or inclusion/exclusion)
    bool all_odd = d.glynn != 0;
    for (int r : reps) all_odd = all_odd && (r % 2 == 1);
    P.tile_ok = (nb + ne >= 1) || (all_odd && d.K < m_max);
  }
  P.term_cost = (double)P.mb_max * P.mb_max * P.mb_max + 64.0;
  if (P.rows_max > 80) return fail(WG_EINVAL, "term matrix of %d rows above the supported 80", P.rows_max);
  if (P.kc_max > 64) return fail(WG_EINVAL, "more than 64 characteristic coefficients");
  if (d.Nodd > 250 || d.K > 250) return fail(WG_EINVAL, "photon number above the supported 250");
  const bool cplx = in.dtype == WG_COMPLEX128;
  if (prec_mod(precision)) {
    // exact sieve: integer-valued real inputs below 2^31, binomial products exact in FP64 slots
    if (cplx) return fail(WG_EINVAL, "exact precision needs float64 (real) inputs");
    auto integral = [](double v) { return std::isfinite(v) && v == std::floor(v) && std::fabs(v) < 2147483648.0; };
    for (size_t i = 0; i < (size_t)in.n * in.n; ++i)
      if (!integral(((const double*)in.A)[i])) return fail(WG_EINVAL, "exact precision needs integer matrix entries below 2^31");
    if (in.D)
      for (int i = 0; i < in.n; ++i)
        if (!integral(((const double*)in.D)[i])) return fail(WG_EINVAL, "exact precision needs integer loop weights below 2^31");
    if (in.oddV)
      for (int i = 0; i < in.n; ++i)
        if (!integral(((const double*)in.oddV)[i])) return fail(WG_EINVAL, "exact precision needs integer entries below 2^31");
    if (kind == KIND_LOOP_ODD && !integral(in.oddloop[0])) return fail(WG_EINVAL, "exact precision needs an integer self-loop weight");
    if (maxr > 50) return fail(WG_EINVAL, "exact precision supports edge repetitions up to 50");
    P.stype = ST_MOD0 + (precision - WG_PREC_MOD0);
  } else {
    P.stype = precision == WG_PREC_DF   ? (cplx ? ST_CPLXDF : ST_REALDF)
              : precision == WG_PREC_DD ? (cplx ? ST_CPLXDD : ST_REALDD)
                                        : (cplx ? ST_CPLX64 : ST_REAL64);
  }
  // extended matrix [[A, D], [D^T, 0], [oddV, 0], [oddV0, 0]]  ((n+3) x (n+1))
  const int n = in.n, lda = n + 1;
  const size_t sb = stype_bytes(P.stype);
  P.ext.assign((size_t)(n + 3) * lda * sb, 0);
  P.ext_bytes = P.ext.size();
  auto at = [&](int r, int c) { return P.ext.data() + ((size_t)r * lda + c) * sb; };
  double re, im;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      get_val(in.A, in.dtype, (size_t)r * n + c, re, im);
      put_scalar(at(r, c), P.stype, re * alpha, im * alpha);
    }
  if (nb) {
    for (int i = 0; i < n; ++i) {
      get_val(in.D, in.dtype, i, re, im);
      put_scalar(at(i, n), P.stype, re * salpha, im * salpha);
      put_scalar(at(n, i), P.stype, re * salpha, im * salpha);
    }
  }
  if (kind == KIND_LOOP_ODD) {
    for (int i = 0; i < n; ++i) {
      get_val(in.oddV, in.dtype, i, re, im);
      put_scalar(at(n + 1, i), P.stype, re * alpha, im * alpha);
    }
  }
  if (kind == KIND_BATCH_EVEN || kind == KIND_BATCH_ODD) {
    for (int i = 0; i < n; ++i) {  // oddV = A[0, :]
      get_val(in.A, in.dtype, (size_t)i, re, im);
      put_scalar(at(n + 1, i), P.stype, re * alpha, im * alpha);
    }
    if (kind == KIND_BATCH_ODD)
      for (int i = 0; i < n; ++i) {  // oddV0 = A[1, :]
        get_val(in.A, in.dtype, (size_t)n + i, re, im);
        put_scalar(at(n + 2, i), P.stype, re * alpha, im * alpha);
      }
  }
  return WG_OK;
}


// Device-side formation of instance pools from a resident Gaussian state (serving).
struct GatherDev {
  long long a_off;  // pool byte offset of the instance's extended matrix
  int x_off;        // first index of the instance's pairing in the index array
  int n;            // 2E
  int oddmode;      // -1: none
  int stype;
  double alpha, salpha;
};
struct GatherSpec {
  const c64* B = nullptr;
  const c64* gamma = nullptr;
  int M = 0;
  std::vector<GatherDev> desc;
  std::vector<int> idx;
};

static int finalize_plan(std::vector<Prepared>& P, int precision, const wg_plan_options& opt, wg_plan* pl,
                         GatherSpec* gs);

// One block per instance: writes [[B[x][:,x], gamma[x]], [gamma[x]^T, 0], [B[o, x], 0], [0]]
// (alpha / sqrt(alpha) prescaled) into the instance's pool slot in its scalar type.
static __global__ void gather_kernel(const GatherDev* __restrict__ gd, const int* __restrict__ idx,
                                     const c64* __restrict__ B, const c64* __restrict__ gamma, int M,
                                     unsigned char* __restrict__ pool) {
  const GatherDev G = gd[blockIdx.x];
  const int n = G.n, lda = n + 1;
  const int* x = idx + G.x_off;
  const int total = (n + 3) * lda;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int i = e / lda, j = e % lda;
    c64 v = {0.0, 0.0};
    double sc = 0.0;
    if (i < n && j < n) { v = B[(size_t)x[i] * M + x[j]]; sc = G.alpha; }
    else if (i < n && j == n) { v = gamma[x[i]]; sc = G.salpha; }
    else if (i == n && j < n) { v = gamma[x[j]]; sc = G.salpha; }
    else if (i == n + 1 && j < n && G.oddmode >= 0) { v = B[(size_t)G.oddmode * M + x[j]]; sc = G.alpha; }
    const double re = v.re * sc, im = v.im * sc;
    unsigned char* dst = pool + G.a_off;
    if (G.stype == ST_CPLX64) {
      reinterpret_cast<c64*>(dst)[e] = {re, im};
    } else {
      const float hr = __double2float_rn(re), hi = __double2float_rn(im);
      reinterpret_cast<cdf*>(dst)[e] = {{hr, __double2float_rn(re - (double)hr)}, {hi, __double2float_rn(im - (double)hi)}};
    }
  }
}

// Loop-hafnian instance of one serving request (the host part of prepare() for WG_KIND_LOOP,
// without a host copy of the matrix).
static int prepare_request(const wg_request& r, const wg_state& st, int precision, Prepared& P, GatherDev& g,
                           std::vector<int>& idx) {
  memset(&P.d, 0, sizeof(P.d));
  InstDev& d = P.d;
  if (r.E < 1 || r.E > MAX_EDGES || !r.x || !r.edge_reps) return fail(WG_EINVAL, "request needs 1..32 edges");
  const bool odd = r.oddmode >= 0;
  if (r.oddmode >= st.M) return fail(WG_EINVAL, "unpaired mode out of range");
  long long sumr = 0, steps = 1;
  int maxr = 0;
  for (int i = 0; i < r.E; ++i) {
    const long long rr = r.edge_reps[i];
    if (rr < 0 || rr > BINOM_N - 1) return fail(WG_EINVAL, "edge repetition out of range");
    sumr += rr;
    maxr = std::max(maxr, (int)rr);
  }
  for (int i = 0; i < 2 * r.E; ++i)
    if (r.x[i] < 0 || r.x[i] >= st.M) return fail(WG_EINVAL, "mode index out of range");
  const double alpha = precision == WG_PREC_DF ? st.alpha : 1.0, salpha = std::sqrt(alpha);
  d.kind = odd ? KIND_LOOP_ODD : KIND_LOOP;
  d.n = 2 * r.E;
  d.E = r.E;
  d.glynn = 1;
  d.nb = 1;
  d.ne = odd ? 1 : 0;
  d.lda = d.n + 1;
  d.unit_binoms = maxr <= 1;
  d.N = (int)(2 * sumr + (odd ? 1 : 0));
  d.K = d.N / 2;
  d.Nodd = odd ? d.N : 0;
  d.nout = 1;
  d.half_first = odd ? 0 : 1;
  if (odd) d.oddloop = {st.gamma[r.oddmode].re * salpha, st.gamma[r.oddmode].im * salpha};
  const int e = odd ? d.N / 2 : d.N / 2 - 1;
  P.scales.assign(1, std::ldexp(1.0, -e) * std::pow(alpha, -0.5 * d.N));
  for (int i = 0; i < r.E; ++i) {
    const int R = (i == 0 && d.half_first) ? (int)(r.edge_reps[0] + 2) / 2 : (int)r.edge_reps[i] + 1;
    d.radix[i] = R;
    d.reps[i] = (int)r.edge_reps[i];
    if (steps > (1LL << 62) / R) return fail(WG_EINVAL, "too many sieve terms");
    steps *= R;
  }
  d.steps = steps;
  P.t_lo = 0;
  P.t_hi = steps;
  int nnz = 0;
  bool all_odd = true;
  for (int i = 0; i < r.E; ++i) {
    nnz += r.edge_reps[i] > 0;
    all_odd = all_odd && (r.edge_reps[i] % 2 == 1);
  }
  P.m_max = 2 * nnz;
  P.mb_max = P.m_max + 1;
  P.rows_max = P.m_max + 1 + d.ne;
  P.kc_max = std::min(d.K, P.m_max);
  P.nser_need = std::max(d.K, d.Nodd) + 2;
  P.narr = 8;
  P.tile_ok = true;  // bordered tile
  P.term_cost = (double)P.mb_max * P.mb_max * P.mb_max + 64.0;
  if (P.rows_max > 80 || d.K > 250 || d.Nodd > 250) return fail(WG_EINVAL, "request too large");
  P.stype = precision == WG_PREC_DF ? ST_CPLXDF : ST_CPLX64;
  P.ext.clear();
  P.ext_bytes = (size_t)(d.n + 3) * (d.n + 1) * stype_bytes(P.stype);
  g.x_off = (int)idx.size();
  g.n = d.n;
  g.oddmode = r.oddmode;
  g.stype = P.stype;
  g.alpha = alpha;
  g.salpha = salpha;
  for (int i = 0; i < 2 * r.E; ++i) idx.push_back(r.x[i]);
  return WG_OK;
}

static int build_plan(const wg_instance* v, int count, int precision, const wg_plan_options& opt, wg_plan* pl) {
  if (count < 0 || (count > 0 && !v)) return fail(WG_EINVAL, "bad instance list");
  if (precision != WG_PREC_FP64 && precision != WG_PREC_DF && precision != WG_PREC_DD && !prec_mod(precision))
    return fail(WG_EINVAL, "unknown precision %d", precision);
  std::vector<Prepared> P(count);
  for (int i = 0; i < count; ++i) {
    int rc = prepare(v[i], precision, P[i]);
    if (rc) return fail(rc, "instance %d: %s", i, g_err.c_str());
  }
  return finalize_plan(P, precision, opt, pl, nullptr);
}

static int finalize_plan(std::vector<Prepared>& P, int precision, const wg_plan_options& opt, wg_plan* pl,
                         GatherSpec* gs) {
  const int count = (int)P.size();
  const double chunk_scale = opt.chunk_scale > 0 ? opt.chunk_scale : 1.0;
  const int wpc_cap = opt.max_warps_per_cta > 0 ? std::min(opt.max_warps_per_cta, 8) : kDefaultWarpsPerCta;
  pl->use_graph = opt.use_graph != 0;
  pl->serial_groups = opt.serial_groups != 0;
  pl->precision = precision;
  pl->device = g_device;
  // outputs and scales in instance order
  int out = 0;
  std::vector<double> scales;
  for (int i = 0; i < count; ++i) {
    P[i].d.out_base = out;
    P[i].d.scale_base = (int)scales.size();
    out += P[i].d.nout;
    scales.insert(scales.end(), P[i].scales.begin(), P[i].scales.end());
  }
  pl->total_out = out;
  // launch shape per (scalar class, per-warp workspace), see best_shape
  std::map<std::pair<int, int>, std::pair<int, int>> shape_memo;
  auto shape = [&](int st, int bytes) -> std::pair<int, int> {
    const auto key = std::make_pair(st, bytes);
    const auto it = shape_memo.find(key);
    if (it != shape_memo.end()) return it->second;
    return shape_memo[key] = best_shape(st, bytes, wpc_cap);
  };
  // groups by (stype, resident warps per SM of the instance's own workspace), so that a small
  // instance does not run at the occupancy of a larger one's workspace; with merge_classes one
  // group per scalar type
  struct GKey { int st, res; };
  std::vector<GKey> keys;
  std::vector<int> gid(count);
  for (int i = 0; i < count; ++i) {
    if (!tile_rows_ok(P[i].stype, P[i].rows_max)) return fail(WG_EINVAL, "instance %d: term matrix too large", i);
    int res = 0;
    if (!opt.merge_classes) {
      const WarpLayout Li = make_layout(P[i].stype, std::max(P[i].rows_max, 1), std::max(P[i].mb_max, 1),
                                        P[i].kc_max, std::max(P[i].nser_need, 2), std::max(P[i].narr, 2),
                                        P[i].tile_ok);
      const auto sh = shape(P[i].stype, Li.bytes);
      res = sh.first * sh.second;
    }
    int g = -1;
    for (size_t k = 0; k < keys.size(); ++k)
      if (keys[k].st == P[i].stype && (opt.merge_classes || keys[k].res == res)) g = (int)k;
    if (g < 0) { keys.push_back({P[i].stype, res}); g = (int)keys.size() - 1; }
    gid[i] = g;
  }
  // pool
  size_t pool_bytes = 0;
  for (int i = 0; i < count; ++i) {
    P[i].d.a_off = (long long)pool_bytes;
    pool_bytes += (P[i].ext_bytes + 255) & ~(size_t)255;
  }
  if (gs)
    for (int i = 0; i < count; ++i) gs->desc[i].a_off = P[i].d.a_off;
  int nparts = 0;
  for (size_t g = 0; g < keys.size(); ++g) {
    Group G;
    G.stype = keys[g].st;
    int rows = 1, mb = 1, kc = 0, nser = 2, narr = 2;
    bool tile = true;
    double total_cost = 0;
    std::vector<int> members;
    for (int i = 0; i < count; ++i)
      if (gid[i] == (int)g) {
        members.push_back(i);
        rows = std::max(rows, P[i].rows_max);
        mb = std::max(mb, P[i].mb_max);
        kc = std::max(kc, P[i].kc_max);
        nser = std::max(nser, P[i].nser_need);
        narr = std::max(narr, P[i].narr);
        tile = tile && P[i].tile_ok;
        total_cost += P[i].term_cost * (double)(P[i].t_hi - P[i].t_lo);
      }
    G.L = make_layout(G.stype, rows, mb, kc, nser, narr, tile);
    const auto sh = shape(G.stype, G.L.bytes);
    const int wpc = sh.first, per_sm = sh.second;
    if (wpc < 1) return fail(WG_EINVAL, "per-warp workspace of %d bytes does not fit", G.L.bytes);
    if (per_sm < 1) {
      cudaGetLastError();
      return fail(WG_ECUDA, "sieve kernel cannot be resident (workspace %d B x %d warps)", G.L.bytes, wpc);
    }
    G.wpc = wpc;
    const long long resident = (long long)g_num_sms * per_sm * wpc;
    // chunking by guided self-scheduling, largest instances first: a chunk is 1/(2 chunk_scale) of
    // a resident warp's share of the group's remaining work, capped at ~1000 term-equivalents of a
    // 40-row tile and floored at ~4 (less for small groups).  Chunk sizes fall geometrically, so
    // the last chunks -- the ones that decide when the launch ends -- are short: n = 40 takes
    // 276 ms instead of 302 ms with fixed chunks of a quarter of a warp's share.
    constexpr double kMaxChunkCost = 6.4e7, kMinChunkCost = 2.6e5;
    const double div = 2.0 * chunk_scale * (double)resident;
    const double min_cost = std::min(kMinChunkCost, total_cost / (4.0 * div));  // small groups: finer
    double remaining = total_cost;
    std::stable_sort(members.begin(), members.end(), [&](int a, int b) {
      return P[a].term_cost * (double)(P[a].t_hi - P[a].t_lo) > P[b].term_cost * (double)(P[b].t_hi - P[b].t_lo);
    });
    G.chunk_begin = (int)pl->chunks.size();
    for (int i : members) {
      InstDev& d = P[i].d;
      const double tc = P[i].term_cost;
      const long long hi = P[i].t_hi, pmin = std::max(1LL, (long long)std::ceil(min_cost / tc));
      d.part_base = nparts;
      // slots per chunk: sums; double-double kinds their compensations; floating-point kinds
      // the term magnitudes (the exact sieve's residues have none)
      const bool dd = stype_dd(P[i].stype), fl = !stype_mod(P[i].stype);
      d.comp_off = dd ? d.nout : 0;
      d.mag_off = fl ? (dd ? 2 : 1) * d.nout : 0;
      d.pstride = (1 + (dd ? 1 : 0) + (fl ? 1 : 0)) * d.nout;
      int nch = 0;
      for (long long t = P[i].t_lo; t < hi; ++nch) {
        const double want = std::min(remaining / div, kMaxChunkCost * chunk_scale);
        long long per = std::max(pmin, (long long)std::floor(want / tc));
        per = std::min(per, hi - t);
        ChunkDev ch;
        ch.inst = i;
        ch.part = nparts + nch * d.pstride;
        ch.t0 = t;
        ch.t1 = t + per;
        pl->chunks.push_back(ch);
        remaining -= (double)per * tc;
        t += per;
      }
      d.nchunks = nch;
      nparts += nch * d.pstride;
    }
    G.chunk_count = (int)pl->chunks.size() - G.chunk_begin;
    G.ctas = (int)std::min<long long>((long long)g_num_sms * per_sm, (G.chunk_count + wpc - 1) / wpc);
    G.ctas = std::max(G.ctas, 1);
    pl->groups.push_back(G);
  }
  pl->nparts = nparts;
  for (int i = 0; i < count; ++i) pl->inst.push_back(P[i].d);
  // one device allocation
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t b_inst = al(sizeof(InstDev) * std::max(count, 1));
  const size_t b_chunks = al(sizeof(ChunkDev) * std::max<size_t>(pl->chunks.size(), 1));
  const size_t b_pool = al(std::max<size_t>(pool_bytes, 16));
  const size_t b_parts = al(sizeof(double2) * std::max(nparts, 1));
  const size_t b_scales = al(sizeof(double) * std::max<size_t>(scales.size(), 1));
  const size_t b_out = al(sizeof(double2) * std::max(out, 1));
  const size_t b_mag = al(sizeof(double) * std::max(out, 1));
  const size_t b_cnt = al(sizeof(unsigned int) * std::max<size_t>(pl->groups.size(), 1));
  const size_t b_err = al(sizeof(int));
  const size_t b_gdesc = gs ? al(sizeof(GatherDev) * std::max<size_t>(gs->desc.size(), 1)) : 0;
  const size_t b_gidx = gs ? al(sizeof(int) * std::max<size_t>(gs->idx.size(), 1)) : 0;
  const size_t total =
      b_inst + b_chunks + b_pool + b_parts + b_scales + b_out + b_mag + b_cnt + b_err + b_gdesc + b_gidx;
  cudaStream_t cs = (cudaStream_t)opt.stream;
  pl->alloc_stream = cs;
  pl->async_alloc = cs != nullptr;
  const cudaError_t ae = pl->async_alloc ? cudaMallocAsync(&pl->dmem, total, cs) : cudaMalloc(&pl->dmem, total);
  if (ae != cudaSuccess) {
    cudaGetLastError();
    pl->dmem = nullptr;
    return fail(WG_ENOMEM, "device allocation of %zu bytes failed", total);
  }
  unsigned char* base = (unsigned char*)pl->dmem;
  pl->d_inst = (InstDev*)base; base += b_inst;
  pl->d_chunks = (ChunkDev*)base; base += b_chunks;
  pl->d_pool = base; base += b_pool;
  pl->d_partials = (double2*)base; base += b_parts;
  pl->d_scales = (double*)base; base += b_scales;
  pl->d_out = (double2*)base; base += b_out;
  pl->d_mag = (double*)base; base += b_mag;
  pl->d_counters = (unsigned int*)base; base += b_cnt;
  pl->d_err = (int*)base; base += b_err;
  pl->device_bytes = (long long)total;
  // staging: one host buffer with the same layout for the upload
  std::vector<unsigned char> host(b_inst + b_chunks + b_pool + b_parts + b_scales, 0);
  memcpy(host.data(), pl->inst.data(), sizeof(InstDev) * count);
  if (!pl->chunks.empty()) memcpy(host.data() + b_inst, pl->chunks.data(), sizeof(ChunkDev) * pl->chunks.size());
  for (int i = 0; i < count; ++i)
    if (!P[i].ext.empty()) memcpy(host.data() + b_inst + b_chunks + P[i].d.a_off, P[i].ext.data(), P[i].ext.size());
  if (!scales.empty()) memcpy(host.data() + b_inst + b_chunks + b_pool + b_parts, scales.data(), sizeof(double) * scales.size());
  // uploads: stream-ordered on the creation stream when one is given (pageable sources are
  // staged before cudaMemcpyAsync returns), else synchronous
  auto up = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    return cs ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, cs)
              : cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
  };
  if (gs) {
    // pools are formed on the device: only descriptors, chunks, scales and indices travel
    CK(up(pl->dmem, host.data(), b_inst + b_chunks));
    CK(up((unsigned char*)pl->dmem + b_inst + b_chunks + b_pool + b_parts,
          host.data() + b_inst + b_chunks + b_pool + b_parts, b_scales));
    GatherDev* d_desc = (GatherDev*)((unsigned char*)pl->d_err + b_err);
    int* d_idx = (int*)((unsigned char*)d_desc + b_gdesc);
    CK(up(d_desc, gs->desc.data(), sizeof(GatherDev) * gs->desc.size()));
    if (!gs->idx.empty()) CK(up(d_idx, gs->idx.data(), sizeof(int) * gs->idx.size()));
    if (count > 0) {
      gather_kernel<<<count, 256, 0, cs>>>(d_desc, d_idx, gs->B, gs->gamma, gs->M, pl->d_pool);
      CK(cudaGetLastError());
    }
    pl->h2d_bytes = (long long)(b_inst + b_chunks + b_scales + sizeof(GatherDev) * gs->desc.size() +
                                sizeof(int) * gs->idx.size());
  } else {
    CK(up(pl->dmem, host.data(), host.size()));
    pl->h2d_bytes = (long long)host.size();
  }
  if (cs) {
    CK(cudaMemsetAsync(pl->d_counters, 0, b_cnt + b_err, cs));
  } else {
    CK(cudaMemset(pl->d_counters, 0, b_cnt + b_err));
    CK(cudaStreamSynchronize(0));
  }
  return WG_OK;
}

static int launch_plan(wg_plan* pl, cudaStream_t st) {
  const size_t ng = pl->groups.size();
  const bool side = ng > 1 && !pl->serial_groups;
  if (side) {
    if (pl->side.size() < ng - 1) {
      if (!pl->fork) CK(cudaEventCreateWithFlags(&pl->fork, cudaEventDisableTiming));
      while (pl->side.size() < ng - 1) {
        cudaStream_t s2;
        cudaEvent_t e2;
        CK(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&e2, cudaEventDisableTiming));
        pl->side.push_back(s2);
        pl->side_done.push_back(e2);
      }
    }
    CK(cudaEventRecord(pl->fork, st));
    for (size_t g = 1; g < ng; ++g) CK(cudaStreamWaitEvent(pl->side[g - 1], pl->fork, 0));
  }
  for (size_t g = 0; g < ng; ++g) {
    const Group& G = pl->groups[g];
    SieveParams p;
    const DevTables& T = g_dev[pl->device];
    p.lb_lane = T.lane;
    p.lb_own = T.own;
    p.lb_lane2 = T.lane2;
    p.lb_own2 = T.own2;
    p.inst = pl->d_inst;
    p.chunks = pl->d_chunks + G.chunk_begin;
    p.nchunks = G.chunk_count;
    p.pool = pl->d_pool;
    p.partials = pl->d_partials;
    p.counter = pl->d_counters + g;
    p.err = pl->d_err;
    p.L = G.L;
    const cudaStream_t gs = (g == 0 || !side) ? st : pl->side[g - 1];
    const cudaError_t e = sieve_launch(G.stype, p, G.ctas, G.wpc, gs);
    if (e != cudaSuccess) return fail(WG_ECUDA, "sieve launch: %s", cudaGetErrorString(e));
    if (g > 0 && side) {
      CK(cudaEventRecord(pl->side_done[g - 1], gs));
      CK(cudaStreamWaitEvent(st, pl->side_done[g - 1], 0));
    }
  }
  const int ninst = (int)pl->inst.size();
  if (ninst > 0) {
    const int threads = 128;
    const int blocks = (pl->total_out * 32 + threads - 1) / threads;  // one warp per output
    const unsigned int modp = prec_mod(pl->precision) ? MOD_PRIMES[pl->precision - WG_PREC_MOD0] : 0u;
    reduce_kernel<<<std::max(blocks, 1), threads, 0, st>>>(pl->d_inst, ninst, pl->d_partials, pl->d_scales, pl->d_out,
                                                           pl->d_counters, (int)pl->groups.size(), pl->total_out, modp,
                                                           pl->d_mag);
    CK(cudaGetLastError());
  }
  return WG_OK;
}

// Direct launches, or -- with use_graph -- one CUDA graph captured on first use (the launch
// attributes are set by a direct execution first) and replayed on the caller's stream.
static int execute_plan(wg_plan* pl, cudaStream_t st) {
  if (!pl->use_graph) return launch_plan(pl, st);
  if (!pl->graph_exec) {
    int rc = launch_plan(pl, st);  // sets the kernels' shared-memory attributes, warms up
    if (rc) return rc;
    CK(cudaStreamSynchronize(st));
    cudaStream_t cap;
    CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      rc = launch_plan(pl, cap);
      e = cudaStreamEndCapture(cap, &graph);
    }
    if (e == cudaSuccess && rc == 0) e = cudaGraphInstantiate(&pl->graph_exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cap);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(WG_ECUDA, "graph capture: %s", cudaGetErrorString(e));
    return WG_OK;  // this call already executed the plan once
  }
  CK(cudaGraphLaunch(pl->graph_exec, st));
  return WG_OK;
}

static void destroy_plan(wg_plan* pl) {
  if (!pl) return;
  if (pl->graph_exec) cudaGraphExecDestroy(pl->graph_exec);
  for (cudaStream_t s2 : pl->side) cudaStreamDestroy(s2);
  for (cudaEvent_t e2 : pl->side_done) cudaEventDestroy(e2);
  if (pl->fork) cudaEventDestroy(pl->fork);
  if (pl->dmem) {
    if (pl->async_alloc) cudaFreeAsync(pl->dmem, pl->alloc_stream);
    else cudaFree(pl->dmem);
  }
  delete pl;
}

// ---------------------------------------------------------------- FP pipe microbenchmark
template <typename T>
__global__ void fma_peak_kernel(T* out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) x[c] = (T)(threadIdx.x + c);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = x[c] * a + b;
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
static int time_peak(int blocks, int threads, int iters, double* tflops) {
  T* buf = nullptr;
  CK(cudaMalloc(&buf, sizeof(T) * blocks * threads));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    CK(cudaEventRecord(e0));
    fma_peak_kernel<T><<<blocks, threads>>>(buf, iters, (T)0.999999, (T)1e-7);
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0) best = std::min(best, ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  *tflops = 2.0 * 8.0 * (double)blocks * threads * (double)iters / (best * 1e-3) / 1e12;
  return WG_OK;
}

}  // namespace wg

using namespace wg;

extern "C" {

int wg_init(int device) { return ensure_init(device); }

const char* wg_last_error(void) { return g_err.c_str(); }

int wg_instance_outputs(const wg_instance* in) {
  if (!in) return fail(WG_EINVAL, "NULL instance");
  if (in->kind == WG_KIND_BATCH_EVEN) return 2 * in->batch_max + in->cutoff + 1;
  if (in->kind == WG_KIND_BATCH_ODD) return 2 * in->batch_max + in->cutoff + 2;
  return 1;
}

long long wg_instance_terms(const wg_instance* in) {
  if (!in) return fail(WG_EINVAL, "NULL instance");
  Prepared P;
  wg_instance whole = *in;
  whole.term_begin = whole.term_end = 0;
  const int rc = prepare(whole, WG_PREC_FP64, P);
  return rc ? (long long)rc : P.d.steps;
}

int wg_plan_create_ex(const wg_instance* inst, int count, int precision, const wg_plan_options* options,
                      wg_plan** plan) {
  if (!plan) return fail(WG_EINVAL, "plan is NULL");
  *plan = nullptr;
  int rc = ensure_init(-1);
  if (rc) return rc;
  wg_plan_options opt;
  memset(&opt, 0, sizeof(opt));
  opt.chunk_scale = 1.0;
  if (options) opt = *options;
  wg_plan* pl = new wg_plan();
  rc = build_plan(inst, count, precision, opt, pl);
  if (rc) { destroy_plan(pl); return rc; }
  *plan = pl;
  return WG_OK;
}

int wg_plan_create(const wg_instance* inst, int count, int precision, double chunk_scale, wg_plan** plan) {
  wg_plan_options opt;
  memset(&opt, 0, sizeof(opt));
  opt.chunk_scale = chunk_scale;
  return wg_plan_create_ex(inst, count, precision, &opt, plan);
}

int wg_plan_execute(wg_plan* plan, void* stream) {
  if (!plan) return fail(WG_EINVAL, "plan is NULL");
  int rc = ensure_init(-1);
  if (rc) return rc;
  return execute_plan(plan, (cudaStream_t)stream);
}

int wg_plan_read(wg_plan* plan, double* out, void* stream) {
  if (!plan || (!out && plan->total_out > 0)) return fail(WG_EINVAL, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  if (plan->total_out > 0)
    CK(cudaMemcpyAsync(out, plan->d_out, sizeof(double2) * plan->total_out, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return WG_OK;
}

int wg_plan_read_magnitudes(wg_plan* plan, double* out, void* stream) {
  if (!plan || (!out && plan->total_out > 0)) return fail(WG_EINVAL, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  if (plan->total_out > 0)
    CK(cudaMemcpyAsync(out, plan->d_mag, sizeof(double) * plan->total_out, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return WG_OK;
}

int wg_plan_outputs(const wg_plan* plan) { return plan ? plan->total_out : fail(WG_EINVAL, "plan is NULL"); }

int wg_plan_kernel_launches(const wg_plan* plan) {
  return plan ? (int)plan->groups.size() + (plan->inst.empty() ? 0 : 1) : fail(WG_EINVAL, "plan is NULL");
}

int wg_plan_partials(wg_plan* plan, double* out, int capacity, void* stream) {
  if (!plan) return fail(WG_EINVAL, "plan is NULL");
  if (!out || capacity < plan->nparts) return plan->nparts;
  cudaStream_t st = (cudaStream_t)stream;
  if (plan->nparts > 0)
    CK(cudaMemcpyAsync(out, plan->d_partials, sizeof(double2) * plan->nparts, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return plan->nparts;
}

int wg_plan_chunk(const wg_plan* plan, int chunk, int* inst, int* part, long long* t0, long long* t1) {
  if (!plan || chunk < 0 || chunk >= (int)plan->chunks.size()) return fail(WG_EINVAL, "bad chunk index");
  const ChunkDev& c = plan->chunks[chunk];
  if (inst) *inst = c.inst;
  if (part) *part = c.part;
  if (t0) *t0 = c.t0;
  if (t1) *t1 = c.t1;
  return (int)plan->chunks.size();
}

int wg_state_create(const double* B, const double* gamma, int M, wg_state** state) {
  if (!state || !B || !gamma || M < 1) return fail(WG_EINVAL, "bad state arguments");
  *state = nullptr;
  int rc = ensure_init(-1);
  if (rc) return rc;
  wg_state* st = new wg_state();
  st->M = M;
  st->gamma.resize(M);
  double rs = 0;
  for (int i = 0; i < M; ++i) {
    st->gamma[i] = {gamma[2 * i], gamma[2 * i + 1]};
    double s = 0;
    for (int j = 0; j < M; ++j) s += std::hypot(B[2 * ((size_t)i * M + j)], B[2 * ((size_t)i * M + j) + 1]);
    rs = std::max(rs, s);
  }
  if (rs > 0 && std::isfinite(rs)) st->alpha = std::exp2(-std::round(std::log2(rs)));
  if (cudaMalloc(&st->d_B, sizeof(c64) * (size_t)M * M) != cudaSuccess ||
      cudaMalloc(&st->d_gamma, sizeof(c64) * M) != cudaSuccess) {
    cudaGetLastError();
    if (st->d_B) cudaFree(st->d_B);
    delete st;
    return fail(WG_ENOMEM, "state allocation failed");
  }
  CK(cudaMemcpy(st->d_B, B, sizeof(c64) * (size_t)M * M, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(st->d_gamma, gamma, sizeof(c64) * M, cudaMemcpyHostToDevice));
  *state = st;
  return WG_OK;
}

int wg_state_create_from_cov(const double* cov, const double* mu, int M, double hbar, wg_state** state,
                             double vacuum[2], double* B_out, double* gamma_out) {
  if (!state || !cov || !mu || !vacuum || M < 1 || M > 512 || !(hbar > 0))
    return fail(WG_EINVAL, "bad state arguments (1 <= M <= 512 modes, hbar > 0)");
  *state = nullptr;
  int rc = ensure_init(-1);
  if (rc) return rc;
  const int n = 2 * M;
  double *d_cov = nullptr, *d_mu = nullptr, *d_out = nullptr;
  c64 *d_Q = nullptr, *d_X = nullptr;
  wg_state* st = new wg_state();
  st->M = M;
  auto release = [&]() {
    if (d_cov) cudaFree(d_cov);
    if (d_mu) cudaFree(d_mu);
    if (d_out) cudaFree(d_out);
    if (d_Q) cudaFree(d_Q);
    if (d_X) cudaFree(d_X);
  };
  auto abandon = [&](int code, const char* what) {
    cudaGetLastError();
    release();
    if (st->d_B) cudaFree(st->d_B);
    if (st->d_gamma) cudaFree(st->d_gamma);
    delete st;
    return fail(code, "%s", what);
  };
  if (cudaMalloc(&st->d_B, sizeof(c64) * (size_t)M * M) != cudaSuccess ||
      cudaMalloc(&st->d_gamma, sizeof(c64) * M) != cudaSuccess ||
      cudaMalloc(&d_cov, sizeof(double) * (size_t)n * n) != cudaSuccess ||
      cudaMalloc(&d_mu, sizeof(double) * n) != cudaSuccess || cudaMalloc(&d_out, sizeof(double) * 8) != cudaSuccess ||
      cudaMalloc(&d_Q, sizeof(c64) * (size_t)n * n) != cudaSuccess ||
      cudaMalloc(&d_X, sizeof(c64) * (size_t)n * M) != cudaSuccess)
    return abandon(WG_ENOMEM, "state allocation failed");
  if (cudaMemcpy(d_cov, cov, sizeof(double) * (size_t)n * n, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d_mu, mu, sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess)
    return abandon(WG_ECUDA, "state upload failed");
  gaussian_state_kernel<<<1, 1024>>>(d_cov, d_mu, M, hbar, d_Q, d_X, st->d_B, st->d_gamma, d_out);
  double out[8] = {0};
  if (cudaGetLastError() != cudaSuccess || cudaMemcpy(out, d_out, sizeof(double) * 5, cudaMemcpyDeviceToHost) != cudaSuccess)
    return abandon(WG_ECUDA, "state kernel failed");
  if (out[4] != 0.0) return abandon(WG_EINVAL, "covariance is not a physical state: its Husimi matrix Q is not positive definite");
  st->gamma.resize(M);
  if (cudaMemcpy(st->gamma.data(), st->d_gamma, sizeof(c64) * M, cudaMemcpyDeviceToHost) != cudaSuccess)
    return abandon(WG_ECUDA, "state readback failed");
  if (B_out && cudaMemcpy(B_out, st->d_B, sizeof(c64) * (size_t)M * M, cudaMemcpyDeviceToHost) != cudaSuccess)
    return abandon(WG_ECUDA, "state readback failed");
  if (gamma_out) memcpy(gamma_out, st->gamma.data(), sizeof(c64) * M);
  release();
  const double rs = out[3];
  if (rs > 0 && std::isfinite(rs)) st->alpha = std::exp2(-std::round(std::log2(rs)));
  // <0|psi> = exp(-quad / 2) / det(Q)^(1/4)
  const double mag = std::exp(-0.5 * out[1] - 0.25 * out[0]);
  vacuum[0] = mag * std::cos(-0.5 * out[2]);
  vacuum[1] = mag * std::sin(-0.5 * out[2]);
  *state = st;
  return WG_OK;
}

int wg_state_destroy(wg_state* state) {
  if (!state) return WG_OK;
  if (state->d_B) cudaFree(state->d_B);
  if (state->d_gamma) cudaFree(state->d_gamma);
  delete state;
  return WG_OK;
}

int wg_plan_create_requests(const wg_state* state, const wg_request* req, int count, int precision,
                            const wg_plan_options* options, wg_plan** plan) {
  if (!plan || !state || count < 0 || (count > 0 && !req)) return fail(WG_EINVAL, "bad request list");
  *plan = nullptr;
  if (precision != WG_PREC_FP64 && precision != WG_PREC_DF) return fail(WG_EINVAL, "unknown precision %d", precision);
  int rc = ensure_init(-1);
  if (rc) return rc;
  wg_plan_options opt;
  memset(&opt, 0, sizeof(opt));
  opt.chunk_scale = 1.0;
  if (options) opt = *options;
  std::vector<Prepared> P(count);
  GatherSpec gs;
  gs.B = state->d_B;
  gs.gamma = state->d_gamma;
  gs.M = state->M;
  gs.desc.resize(count);
  for (int i = 0; i < count; ++i) {
    rc = prepare_request(req[i], *state, precision, P[i], gs.desc[i], gs.idx);
    if (rc) return fail(rc, "request %d: %s", i, g_err.c_str());
  }
  wg_plan* pl = new wg_plan();
  rc = finalize_plan(P, precision, opt, pl, &gs);
  if (rc) { destroy_plan(pl); return rc; }
  *plan = pl;
  return WG_OK;
}

long long wg_plan_device_bytes(const wg_plan* plan) { return plan ? plan->device_bytes : 0; }

int wg_plan_transfer_bytes(const wg_plan* plan, long long* h2d, long long* d2h) {
  if (!plan) return fail(WG_EINVAL, "plan is NULL");
  if (h2d) *h2d = plan->h2d_bytes;
  if (d2h) *d2h = (long long)sizeof(double2) * plan->total_out;
  return WG_OK;
}

int wg_plan_destroy(wg_plan* plan) {
  destroy_plan(plan);
  return WG_OK;
}

// One-shot plans run stream-ordered on the caller's stream, or on the calling thread's default
// stream: their memory comes from the stream-ordered pool and goes back to it without a
// device-wide synchronisation, and the uploads need none either (a small hafnian costs ~85 us
// with a cudaMalloc / cudaFree pair per call).
int wg_run(const wg_instance* inst, int count, int precision, double* out, void* stream) {
  wg_plan* pl = nullptr;
  const cudaStream_t st = stream ? (cudaStream_t)stream : cudaStreamPerThread;
  wg_plan_options opt;
  memset(&opt, 0, sizeof(opt));
  opt.chunk_scale = 1.0;
  opt.stream = st;
  int rc = wg_plan_create_ex(inst, count, precision, &opt, &pl);
  if (rc) return rc;
  rc = wg_plan_execute(pl, st);
  if (!rc) rc = wg_plan_read(pl, out, st);
  destroy_plan(pl);
  return rc;
}

int wg_hafnian(const void* A, int n, int dtype, const int64_t* edge_reps, int E, int glynn, int precision,
               double out[2], void* stream) {
  wg_instance in;
  memset(&in, 0, sizeof(in));
  in.kind = WG_KIND_PLAIN;
  in.n = n;
  in.E = E;
  in.dtype = dtype;
  in.glynn = glynn;
  in.edge_reps = edge_reps;
  in.A = A;
  return wg_run(&in, 1, precision, out, stream);
}

int wg_loop_hafnian(const void* A, const void* D, int n, int dtype, const int64_t* edge_reps, int E, int has_odd,
                    const double oddloop[2], const void* oddV, int glynn, int precision, double out[2],
                    void* stream) {
  wg_instance in;
  memset(&in, 0, sizeof(in));
  in.kind = WG_KIND_LOOP;
  in.n = n;
  in.E = E;
  in.dtype = dtype;
  in.glynn = glynn;
  in.has_odd = has_odd;
  in.edge_reps = edge_reps;
  in.A = A;
  in.D = D;
  in.oddV = oddV;
  if (has_odd && oddloop) { in.oddloop[0] = oddloop[0]; in.oddloop[1] = oddloop[1]; }
  return wg_run(&in, 1, precision, out, stream);
}

int wg_loop_hafnian_batch(const void* A, const void* D, int n, int dtype, const int64_t* fixed_edge_reps, int E,
                          int batch_max, int cutoff, int odd, int glynn, int precision, double* out, void* stream) {
  wg_instance in;
  memset(&in, 0, sizeof(in));
  in.kind = odd ? WG_KIND_BATCH_ODD : WG_KIND_BATCH_EVEN;
  in.n = n;
  in.E = E;
  in.dtype = dtype;
  in.glynn = glynn;
  in.batch_max = batch_max;
  in.cutoff = cutoff;
  in.edge_reps = fixed_edge_reps;
  in.A = A;
  in.D = D;
  return wg_run(&in, 1, precision, out, stream);
}

// Device arithmetic primitives of the kernels, evaluated elementwise for checks against IEEE and
// exact references: 0 recip_newton(x); 1 dd_recip((x, lo)) -> (hi, lo); 2 dd_div_int((x, lo), k)
// with k = (int)y -> (hi, lo); 3 dd_mul((x, lo), (y, lo2)) -> (hi, lo).  Inputs per element:
// in[4i .. 4i+3] = x, x_lo, y, y_lo; outputs out[2i], out[2i+1].
static __global__ void arith_check_kernel(int op, const double* __restrict__ in, int n, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = in[4 * i], xl = in[4 * i + 1], y = in[4 * i + 2], yl = in[4 * i + 3];
  ddr r = {0.0, 0.0};
  switch (op) {
    case 0: r.hi = recip_newton(x); break;
    case 1: r = dd_recip({x, xl}); break;
    case 2: r = dd_div_int({x, xl}, (int)y); break;
    case 3: r = dd_mul({x, xl}, {y, yl}); break;
    case 4: {  // double-float reciprocal (inputs: the float parts)
      const dfr q = Ar<dfr>::recip({(float)x, (float)xl});
      r = {(double)q.hi, (double)q.lo};
      break;
    }
    case 5: {  // complex double-float reciprocal: out = (re, im), each part's hi + lo in FP64
      const cdf q = Ar<cdf>::recip({{(float)x, (float)xl}, {(float)y, (float)yl}});
      r = {df_to_d(q.re), df_to_d(q.im)};
      break;
    }
    default: {  // double-float division by a small integer
      const dfr q = df_div_int({(float)x, (float)xl}, (int)y);
      r = {(double)q.hi, (double)q.lo};
      break;
    }
  }
  out[2 * i] = r.hi;
  out[2 * i + 1] = r.lo;
}

int wg_check_arith(int op, const double* in, int n, double* out) {
  if (op < 0 || op > 6 || n < 0 || (n > 0 && (!in || !out))) return fail(WG_EINVAL, "bad arithmetic check arguments");
  if (n == 0) return WG_OK;
  int rc = ensure_init(-1);
  if (rc) return rc;
  double *d_in = nullptr, *d_out = nullptr;
  if (cudaMalloc(&d_in, sizeof(double) * 4 * (size_t)n) != cudaSuccess ||
      cudaMalloc(&d_out, sizeof(double) * 2 * (size_t)n) != cudaSuccess) {
    cudaGetLastError();
    if (d_in) cudaFree(d_in);
    return fail(WG_ENOMEM, "arithmetic check allocation failed");
  }
  cudaError_t e = cudaMemcpy(d_in, in, sizeof(double) * 4 * (size_t)n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    arith_check_kernel<<<(n + 255) / 256, 256>>>(op, d_in, n, d_out);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, d_out, sizeof(double) * 2 * (size_t)n, cudaMemcpyDeviceToHost);
  cudaFree(d_in);
  cudaFree(d_out);
  if (e != cudaSuccess) return fail(WG_ECUDA, "arithmetic check: %s", cudaGetErrorString(e));
  return WG_OK;
}

int wg_measure_fp_peaks(double* fp64_tflops, double* fp32_tflops) {
  int rc = ensure_init(-1);
  if (rc) return rc;
  if (fp64_tflops) {
    rc = time_peak<double>(g_num_sms * 4, 256, 2000, fp64_tflops);
    if (rc) return rc;
  }
  if (fp32_tflops) {
    rc = time_peak<float>(g_num_sms * 8, 256, 20000, fp32_tflops);
    if (rc) return rc;
  }
  return WG_OK;
}

}  // extern "C"
