/*
 * walrus_gb300: C ABI of the GB300 (sm_103a) hafnian / loop-hafnian finite-difference sieve.
 *
 * The host side (input validation, special cases, edge pairing, reordering) stays in the
 * caller; these entry points replace the reference's numba sieve drivers, i.e. everything
 * below thewalrus/_hafnian.py:_haf / loop_hafnian and
 * thewalrus/loop_hafnian_batch.py:loop_hafnian_batch.  Matrices are row-major; complex data is
 * interleaved (re, im) doubles.  Host pointers unless stated otherwise.  Every entry point
 * returns 0 on success or a negative WG_E* status; wg_last_error() describes the failure.
 * There is no CPU fallback: without a usable GPU every call fails.
 */
#ifndef WALRUS_GB300_H
#define WALRUS_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define WG_OK 0
#define WG_EINVAL -1   /* bad argument, or a size beyond the kernels' limits */
#define WG_ECUDA -2    /* CUDA runtime error (no device, launch failure, ...) */
#define WG_ENOMEM -3   /* device or host allocation failed */
#define WG_EKERNEL -4  /* a kernel reported an internal inconsistency */

/* element type of matrix inputs */
#define WG_FLOAT64 0
#define WG_COMPLEX128 1

/* arithmetic of the sieve terms */
#define WG_PREC_FP64 0 /* FP64 throughout */
#define WG_PREC_DF 1   /* FP32 double-float terms; FP64 pivots, divisions and accumulation */
/* FP64 double-double terms (106-bit significand) and compensated accumulation that keeps each
 * term's low part: for sums whose terms cancel beyond what FP64 resolves (sum|term| / |sum|
 * above ~1e6).  About 15-20x the FP64 time.  Not offered for serving plans. */
#define WG_PREC_DD 7
/* Exact sieve of an integer-valued float64 instance modulo the prime WG_MOD_PRIME_k (entries and
 * loop weights integers of magnitude below 2^31): every output is a residue in [0, p), returned
 * in the real part; residues of several primes give the exact integer by the Chinese remainder
 * theorem. */
#define WG_PREC_MOD0 2
#define WG_PREC_MOD1 3
#define WG_PREC_MOD2 4
#define WG_PREC_MOD3 5
#define WG_PREC_MOD4 6
#define WG_MOD_PRIME_0 2147483647u
#define WG_MOD_PRIME_1 2147483629u
#define WG_MOD_PRIME_2 2147483587u
#define WG_MOD_PRIME_3 2147483579u
#define WG_MOD_PRIME_4 2147483563u

/* instance kinds for the batched interface */
#define WG_KIND_PLAIN 0      /* _calc_hafnian */
#define WG_KIND_LOOP 1       /* _calc_loop_hafnian (odd self-loop when has_odd) */
#define WG_KIND_BATCH_EVEN 3 /* _calc_loop_hafnian_batch_even */
#define WG_KIND_BATCH_ODD 4  /* _calc_loop_hafnian_batch_odd */

/* One sieve problem, prepared exactly as the reference prepares the arguments of its numba
 * drivers (thewalrus/_hafnian.py:415, :512; thewalrus/loop_hafnian_batch.py:51, :127). */
typedef struct wg_instance {
  int32_t kind;        /* WG_KIND_* */
  int32_t n;           /* dimension of the prepared matrix A */
  int32_t E;           /* entries of edge_reps (for batch kinds: the fixed edge reps) */
  int32_t dtype;       /* WG_FLOAT64 or WG_COMPLEX128 for A, D, oddV */
  int32_t glynn;       /* 1: finite-difference sieve; 0: inclusion/exclusion */
  int32_t has_odd;     /* WG_KIND_LOOP: an odd self-loop is present */
  int32_t batch_max;   /* batch kinds */
  int32_t cutoff;      /* batch kinds: odd_cutoff (even kind) or even_cutoff (odd kind) */
  const int64_t* edge_reps;
  const void* A;       /* n x n */
  const void* D;       /* n (loop and batch kinds) */
  const void* oddV;    /* n (WG_KIND_LOOP with has_odd) */
  double oddloop[2];   /* WG_KIND_LOOP with has_odd */
  /* Sieve terms [term_begin, term_end) of the instance's Gray-code order only (both 0: all
   * terms).  The outputs are then that shard's share of the result, scaled like the full
   * result, so the shards of a partition of [0, steps) sum to it: one GPU per shard and a
   * host-side sum is the multi-GPU form of the sieve (no collective on the data path). */
  int64_t term_begin;
  int64_t term_end;
} wg_instance;

/* Number of sieve terms of an instance (the range that term_begin/term_end index). */
long long wg_instance_terms(const wg_instance* inst);

typedef struct wg_plan wg_plan;

/* Select and initialise the CUDA device (optional: the first call initialises device 0). */
int wg_init(int device);
const char* wg_last_error(void);
/* Number of output values of one instance (1, or the batch length). */
int wg_instance_outputs(const wg_instance* inst);

/* Replaces _calc_hafnian (thewalrus/_hafnian.py:415-467) as called from _haf (:505-507).
 * A: prepared n x n matrix (n = 2E); out: {re, im}. */
int wg_hafnian(const void* A, int n, int dtype, const int64_t* edge_reps, int E, int glynn, int precision,
               double out[2], void* stream);

/* Replaces _calc_loop_hafnian (thewalrus/_hafnian.py:511-577) as called from loop_hafnian
 * (:627-630).  oddloop / oddV are read only when has_odd. */
int wg_loop_hafnian(const void* A, const void* D, int n, int dtype, const int64_t* edge_reps, int E, int has_odd,
                    const double oddloop[2], const void* oddV, int glynn, int precision, double out[2],
                    void* stream);

/* Replaces _calc_loop_hafnian_batch_even / _odd (thewalrus/loop_hafnian_batch.py:50-208) as
 * called from loop_hafnian_batch (:294-304).  odd = 0: cutoff is odd_cutoff, output length
 * 2*batch_max+cutoff+1; odd = 1: cutoff is even_cutoff, length 2*batch_max+cutoff+2.
 * out: complex interleaved. */
int wg_loop_hafnian_batch(const void* A, const void* D, int n, int dtype, const int64_t* fixed_edge_reps, int E,
                          int batch_max, int cutoff, int odd, int glynn, int precision, double* out, void* stream);

/* Batched interface: many instances of uneven size in one persistent launch per arithmetic
 * class, with a device work queue over (instance, term range) chunks.  This has no single
 * counterpart in the reference; it replaces a Python loop of _calc_* calls (the numba prange
 * pool of thewalrus/_hafnian.py:443 spread over instances).
 *   wg_plan_create : validate, prepare and upload the inputs, build the chunk queue
 *   wg_plan_execute: launch the sieve and reduction kernels on `stream` (graph-capturable)
 *   wg_plan_read   : copy all outputs (instance order, complex interleaved) to the host
 * chunk_scale (>0) multiplies the default chunks-per-warp target (1.0 = default). */
int wg_plan_create(const wg_instance* inst, int count, int precision, double chunk_scale, wg_plan** plan);

/* Tuning knobs of a plan (zero-initialised fields take the defaults):
 *   chunk_scale       chunks per resident warp relative to the default 4 (term-chunk size)
 *   max_warps_per_cta cap on warps per CTA (default 7; at most 8: as many as shared memory
 *                     allows up to the cap)
 *   merge_classes     1: one persistent launch per scalar type instead of per occupancy class
 *   use_graph         1: wg_plan_execute captures its launches into a CUDA graph on first use
 *                        and replays the graph afterwards
 *   stream            non-NULL: the plan's memory comes from the stream-ordered allocator and
 *                     its uploads run on this stream without any device-wide synchronisation
 *                     (for serving loops that build plans while others execute); the plan must
 *                     then execute on this stream, and its memory returns to the pool in stream
 *                     order at destruction */
typedef struct wg_plan_options {
  double chunk_scale;
  int32_t max_warps_per_cta;
  int32_t merge_classes;
  int32_t use_graph;
  int32_t serial_groups; /* 1: launch the groups one after another on the caller's stream (default:
                            groups after the first on side streams, overlapping their tails) */
  void* stream;
} wg_plan_options;
int wg_plan_create_ex(const wg_instance* inst, int count, int precision, const wg_plan_options* options,
                      wg_plan** plan);
int wg_plan_execute(wg_plan* plan, void* stream);
int wg_plan_read(wg_plan* plan, double* out, void* stream);
/* Per output of the last execution: the sum over sieve terms of |prefactor x term| (real plus
 * imaginary magnitude) times the output's final scale, i.e. the size of the terms the result
 * cancels from.  magnitude / |result| is the sum's condition number: the result's rounding error
 * is about (the terms' relative rounding) x magnitude.  0 for the exact precisions. */
int wg_plan_read_magnitudes(wg_plan* plan, double* out, void* stream);
int wg_plan_outputs(const wg_plan* plan);
int wg_plan_kernel_launches(const wg_plan* plan);
/* Diagnostics for chunk-level checks.  wg_plan_partials copies the unscaled per-chunk partial
 * sums (complex interleaved, nout per chunk) of the last execution when capacity (in complex
 * values) suffices and returns their count.  wg_plan_chunk describes chunk `chunk`: its
 * instance, first partial slot and Gray-code term range [t0, t1); returns the chunk count. */
int wg_plan_partials(wg_plan* plan, double* out, int capacity, void* stream);
int wg_plan_chunk(const wg_plan* plan, int chunk, int* inst, int* part, long long* t0, long long* t1);
/* Bytes moved by wg_plan_create (host to device) and by wg_plan_read (device to host). */
int wg_plan_transfer_bytes(const wg_plan* plan, long long* h2d, long long* d2h);
int wg_plan_destroy(wg_plan* plan);
/* create + execute + read + destroy, stream-ordered on `stream` (NULL: the calling thread's
 * default stream, cudaStreamPerThread): the plan's memory comes from the device's default
 * stream-ordered pool, which keeps up to 256 MiB of freed memory for the next call. */
int wg_run(const wg_instance* inst, int count, int precision, double* out, void* stream);

/* Serving: a Gaussian state resident on the device and plans whose loop-hafnian matrices are
 * formed on the device from it.  No single counterpart in the reference: it replaces the host
 * work of thewalrus/quantum/fock_tensors.py:74-92 (reduction of B and gamma by the photon
 * pattern) followed by hafnian_repeated / hafnian(loop=True).
 *   wg_state_create : upload B (M x M complex128) and gamma (M complex128) once per state
 *   wg_plan_create_requests : one loop-hafnian instance per request; request r lists its
 *     pairing (x: 2E mode indices, vertex i paired with i+E, as matched_reps returns them), its
 *     edge multiplicities and its unpaired mode (-1 if none); a gather kernel writes
 *     B[x][:, x], gamma[x] and, for an unpaired mode o, B[o, x] and gamma[o] into the pool. */
typedef struct wg_state wg_state;
typedef struct wg_request {
  const int32_t* x;          /* 2E mode indices */
  const int64_t* edge_reps;  /* E multiplicities */
  int32_t E;
  int32_t oddmode;           /* unpaired mode or -1 */
} wg_request;
int wg_state_create(const double* B, const double* gamma, int M, wg_state** state);
/* The same state formed on the device from a pure Gaussian state's xp-ordered covariance
 * (2M x 2M, row-major) and means (2M) with the conventions of thewalrus/quantum/conversions.py:
 * 69-170 and fock_tensors.py:45-98: Husimi Q, B = -(Q^-1)[M:, :M], alpha, gamma = alpha - B
 * alpha^*.  Q is factored by a Cholesky decomposition on the GPU (a covariance whose Q is not
 * positive definite is rejected with WG_EINVAL).  vacuum receives <0|psi> = exp(-(|alpha|^2 -
 * alpha^H B alpha^*)/2) / det(Q)^(1/4); B_out (M x M complex) and gamma_out (M complex), when not
 * NULL, receive copies of the resident matrices.  M <= 512. */
int wg_state_create_from_cov(const double* cov, const double* mu, int M, double hbar, wg_state** state,
                             double vacuum[2], double* B_out, double* gamma_out);
int wg_state_destroy(wg_state* state);
int wg_plan_create_requests(const wg_state* state, const wg_request* req, int count, int precision,
                            const wg_plan_options* options, wg_plan** plan);
/* Device bytes a plan holds (for admission control). */
long long wg_plan_device_bytes(const wg_plan* plan);

/* Device-time microbenchmark of the FP64 and FP32 FMA pipes (TFLOP/s, 2 flops per FMA). */
int wg_measure_fp_peaks(double* fp64_tflops, double* fp32_tflops);

/* The kernels' own arithmetic primitives evaluated elementwise on the device, for checks against
 * IEEE and exact references (no counterpart in the reference): op 0 the pivot reciprocal 1/x
 * (approximate reciprocal + one third-order step r(1 + e + e^2)), 1 the double-double reciprocal of (x, x_lo), 2 the
 * double-double quotient (x, x_lo) / k with k = (int)y, 3 the double-double product of (x, x_lo)
 * and (y, y_lo), 4 the double-float reciprocal of (x, x_lo), 5 the complex double-float
 * reciprocal of (x, x_lo) + i (y, y_lo) (out: its real and imaginary parts, each hi + lo in FP64),
 * 6 the double-float quotient (x, x_lo) / k with k = (int)y; double-float inputs are the float
 * parts, given as doubles.  in: 4 doubles per element (x, x_lo, y, y_lo); out: 2 per element
 * (hi, lo). */
int wg_check_arith(int op, const double* in, int n, double* out);

/* Allocation-free plain hafnian (FP64 terms).  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory while they call us -- code that runs inside its own
 * memory pool or arena, serving plugins that forbid allocation on the request path, and loops
 * where cudaMalloc/cudaFree would stall the device.  Same arguments and result as wg_hafnian,
 * except that A_dev (the prepared n x n matrix, n = 2E <= 64; 8-byte aligned) and
 * out_dev ({re, im}; 16-byte aligned) are DEVICE pointers on the current device, and the call
 * only enqueues work on `stream` (synchronise
 * before reading out_dev).  The working memory it needs beyond its inputs and outputs lives in
 * a static device array of WG_NOALLOC_SCRATCH_BYTES that every GPU loading this library keeps
 * until the process exits; sizes beyond what the kernels or that array hold are rejected with
 * WG_EINVAL, and so are edge repetitions that are all zero (no photons: the hafnian is 1, a
 * closed form the caller answers).  The first call on a device sets the array up (make it
 * before any stream capture).
 * All calls share the array: calls that overlap on the GPU race, so serialise them. */
#define WG_NOALLOC_SCRATCH_BYTES (512 * 1024)
int wg_hafnian_noalloc(const void* A_dev, int n, int dtype, const int64_t* edge_reps, int E, int glynn,
                       double* out_dev, void* stream);

#ifdef __cplusplus
}
#endif
#endif
