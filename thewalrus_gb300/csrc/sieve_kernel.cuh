// Device side of the hafnian / loop-hafnian finite-difference sieve.
//
// One warp owns a contiguous range ("chunk") of sieve terms of one instance and walks it in
// reflected mixed-radix Gray-code order (one edge multiplicity changes by +-1 per step).  For
// each term it
//   1. gathers the term matrix AX_S (rows/cols of nonzero delta, columns scaled by delta, halves
//      swapped) into the warp's shared-memory tile; loop variants border it with D_S / XD_S and
//      append the odd-mode rows, so that the border data of the loop terms survive the reduction;
//   2. reduces it to upper Hessenberg form by Gaussian elimination with partial pivoting (FP64
//      and residues: every subdiagonal entry normalised to exactly 1 or 0 by a diagonal
//      similarity, so that La Budde's recurrence needs no subdiagonal products; double-float:
//      classic multipliers), treating columns whose candidates are rounding residues as reduced;
//   3. runs La Budde's recurrence for the first K coefficients of det(I - eta H), two rows per
//      balanced pass (loop variants: on the anti-transposed block, whose intermediate rows are
//      the trailing submatrices' determinants that give the border series, border_prepare /
//      border_series);
//   4. forms the term's generating function: det(I - eta H)^(-1/2) (the power-trace
//      exponential of f / f_loop), times exp of the loop terms for the loop variants;
//   5. adds prefactor * coefficient into lane-resident Neumaier sums (residue sums for the exact
//      sieve).
// The reference's per-term pipeline is thewalrus/_hafnian.py:443-462 (plain), :546-569 (loop),
// thewalrus/loop_hafnian_batch.py:86-116 / :165-201 (batch), with powertrace in
// thewalrus/charpoly.py:301-327.
#pragma once
#include <cstdint>

#include "arith.cuh"

namespace wg {

constexpr int MAX_EDGES = 32;
constexpr int BINOM_N = 65;

enum Kind : int { KIND_PLAIN = 0, KIND_LOOP = 1, KIND_LOOP_ODD = 2, KIND_BATCH_EVEN = 3, KIND_BATCH_ODD = 4 };

struct InstDev {
  int kind;
  int n;          // prepared matrix dimension (2E)
  int E;          // sieve edges (lanes hold one digit each)
  int glynn;
  int N;          // photons (plain / loop); N_fixed for batch kinds
  int K;          // eta-degree of the plain / even series needed
  int Nodd;       // zeta-degree of the odd series needed (0 when unused)
  int nout;       // outputs of this instance (1, or the batch length)
  int batch_max;
  int half_first;
  int unit_binoms;  // every edge multiplicity <= 1: binomial product is 1
  int nb, ne;       // border rows/cols (0/1) and extra odd-mode rows (0..2)
  int lda;          // leading dimension of the extended matrix (n + 1)
  long long a_off;  // byte offset of the extended matrix in the pool
  long long steps;
  int radix[MAX_EDGES];
  int reps[MAX_EDGES];
  c64 oddloop, oddloop0;
  // reduction bookkeeping
  int part_base;   // first partial slot of this instance
  int nchunks;     // chunks of this instance (partials are [part_base, part_base + nchunks*pstride))
  int pstride;     // partial slots per chunk (0 reads as nout): the sums, then, when their
                   // offsets are nonzero, the compensations (double-double kinds) and the term
                   // magnitudes sum |prefactor x term| (floating-point kinds)
  int comp_off;    // slot offset of the compensations within a chunk's slots (0: none)
  int mag_off;     // slot offset of the term magnitudes (0: none)
  int out_base;    // first output slot
  int scale_base;  // first output scale
};

struct ChunkDev {
  int inst;
  int part;  // first partial slot of this chunk
  long long t0, t1;
};

// Per-warp shared-memory layout (byte offsets), identical for all warps of one launch.
struct WarpLayout {
  int ldw;       // leading dimension of the term tile (odd)
  int rows;      // tile rows allocated
  int kw;        // La Budde window size (rows and columns)
  int nser;      // series capacity (entries per array)
  int off_x, off_win, off_tb, off_part, off_ser, off_int;
  int tilewin;   // La Budde rows kept in dead tile columns (win then holds rows 0..2 only)
  int bytes;     // per warp
};

// La Budde lane schedule for one triangle size Ki (rows with Ki = min(i, Kc) coefficients):
// the r-sums of coefficients j = 2..Ki are cut into pieces, at most two pieces per lane, so that
// every lane does about Ki(Ki-1)/64 multiply-adds; piece a is (ja, r = rloa .. rloa+lena-1),
// piece b likewise.  A lane's partials go to slots 2*lane and 2*lane+1.
struct LbLane {
  signed char ja, rloa, lena, jb, rlob, lenb, pad0, pad1;
};
// the slots holding the pieces of coefficient j, summed by j's owner lane in this order
struct LbOwner {
  unsigned char n, s[7];
};
constexpr int LB_KMAX = 64;

// Two-row schedule (rows i and i+1 with K0 = min(i, Kc) and K1 = min(i+1, Kc) <= 32 coefficients,
// so K1 - K0 is 1 in the triangle and 0 in the steady state): the r-sums of both rows share one
// pass; up to three pieces per lane, piece q of lane l in slot 3*l+q, and bit q of rowmask tells
// which of the two rows it belongs to.  Tables are indexed by lb2_id(K0, K1).
struct LbLane2 {
  signed char j[3], rlo[3], len[3];
  unsigned char rowmask;
  unsigned char pad[2];
};
struct LbOwner2 {
  unsigned char n0, n1, s0[7], s1[7];
};
static_assert(sizeof(LbOwner2) == 16, "an owner record is one 16-byte load");
// byte b of an owner record held in registers (no local-memory array for the dynamic index)
__device__ __forceinline__ int owner_byte(const uint4& q, int b) {
  const unsigned w = b < 4 ? q.x : (b < 8 ? q.y : (b < 12 ? q.z : q.w));
  return (int)((w >> (8 * (b & 3))) & 0xffu);
}
constexpr int LB2_KMAX = 32;
constexpr int LB2_IDS = 2 * (LB2_KMAX + 1);
__host__ __device__ __forceinline__ int lb2_id(int K0, int K1) { return 2 * K1 + (K1 - K0); }

struct SieveParams {
  const LbLane* lb_lane;    // [(LB_KMAX+1) * 32]
  const LbOwner* lb_own;    // [(LB_KMAX+1) * (LB_KMAX+1)]
  const LbLane2* lb_lane2;  // [LB2_IDS * 32]
  const LbOwner2* lb_own2;  // [LB2_IDS * (LB2_KMAX+1)]
  const InstDev* inst;
  const ChunkDev* chunks;
  int nchunks;
  const unsigned char* pool;
  double2* partials;
  unsigned int* counter;
  int* err;
  WarpLayout L;
};

// internal linkage: every translation unit that launches the kernels owns its tables
static __constant__ double c_binom[BINOM_N][BINOM_N];
static __constant__ double c_inv[256];  // c_inv[k] = 1/k (k >= 1)

__device__ __forceinline__ double inv_int(int k) { return k < 256 ? c_inv[k] : 1.0 / (double)k; }
// 1/k modulo the prime of this translation unit's modular kernels (k < 256)
static __constant__ uint32_t c_invmod[256];

template <class S>
__device__ __forceinline__ S inv_of(int k) {  // 1/k in the scalar type (k >= 1)
  using A = Ar<S>;
  if constexpr (A::modular) return k < 256 ? S{c_invmod[k]} : A::inv_int(k);
  else return A::scale(A::one(), inv_int(k));
}

template <class S>
__device__ __forceinline__ S half_of(S x) {
  using A = Ar<S>;
  if constexpr (A::modular) return A::mul(x, A::half());
  else return A::scale_f(x, 0.5f);
}

template <class S>
__device__ __forceinline__ S scale_int(S x, int d) {
  using A = Ar<S>;
  if (d == 1) return x;
  if (d == -1) return A::neg(x);
  if constexpr (A::modular) return A::mul(x, A::of_int(d));
  else return A::scale_f(x, (float)d);  // |d| is a small repetition count: exact in float
}

template <class S>
__device__ __forceinline__ S warp_sum(S v) {
  using A = Ar<S>;
#pragma unroll
  for (int off = 16; off; off >>= 1) {
#pragma unroll
    for (int c = 0; c < A::NC; ++c) {
      typename A::Comp x = A::comp(v, c);
      A::set_comp(v, c, A::cadd(x, A::shfl_xor(x, off)));
    }
  }
  return v;
}

__device__ __forceinline__ double shfl_up_c(double v, int off) { return __shfl_up_sync(0xffffffffu, v, off); }
__device__ __forceinline__ dfr shfl_up_c(dfr v, int off) {
  return {__shfl_up_sync(0xffffffffu, v.hi, off), __shfl_up_sync(0xffffffffu, v.lo, off)};
}
__device__ __forceinline__ ddr shfl_up_c(ddr v, int off) {
  return {__shfl_up_sync(0xffffffffu, v.hi, off), __shfl_up_sync(0xffffffffu, v.lo, off)};
}
template <uint32_t P>
__device__ __forceinline__ modp<P> shfl_up_c(modp<P> v, int off) {
  return {__shfl_up_sync(0xffffffffu, v.v, off)};
}
template <class S>
__device__ __forceinline__ S shfl_up_s(S v, int off) {
  using A = Ar<S>;
#pragma unroll
  for (int c = 0; c < A::NC; ++c) A::set_comp(v, c, shfl_up_c(A::comp(v, c), off));
  return v;
}

__device__ __forceinline__ void neumaier(double& s, double& c, double x) {
  double t = s + x;
  if (fabs(s) >= fabs(x))
    c += (s - t) + x;
  else
    c += (x - t) + s;
  s = t;
}

// Column j+1 of the elimination's similarity for rows lane + 32 k, k < NF (whole 32-row blocks):
// W[a][j+1] = sum_{b=j+1}^{mb-1} W[a][b] x[b], one row per lane.
// With PARTIAL the last block holds only the rows below `rows` (relative to W).
template <class S, int NF, bool PARTIAL = false>
__device__ __forceinline__ void phase_b_rows(S* __restrict__ W, const S* __restrict__ xv, int ldw, int j, int mb,
                                             int rows = 0) {
  using A = Ar<S>;
  const int lane = threadIdx.x & 31;
  S acc[NF];
#pragma unroll
  for (int k = 0; k < NF; ++k) acc[k] = A::zero();
  const bool live = !PARTIAL || lane + 32 * (NF - 1) < rows;
  for (int b = j + 1; b < mb; ++b) {
    const S xb = xv[b];
#pragma unroll
    for (int k = 0; k < NF; ++k)
      if (k < NF - 1 || live) acc[k] = A::fma(W[(lane + 32 * k) * ldw + b], xb, acc[k]);
  }
#pragma unroll
  for (int k = 0; k < NF; ++k)
    if (k < NF - 1 || live) W[(lane + 32 * k) * ldw + j + 1] = acc[k];
}

// The same for rows base .. rows-1 (at most 24, SL = ceil((rows - base) / 8) slots of 8):
// lane = r8 + 8 c4 sums b = j+1+c4, j+5+c4, ... for rows base + r8 + 8 s, and a reduce-scatter
// over the four column lanes (lane bits 3 and 4) leaves each row's total with one lane.
template <class S, int SL>
__device__ __forceinline__ void phase_b_split(S* __restrict__ W, const S* __restrict__ xv, int ldw, int j, int mb,
                                              int rows, int base) {
  using A = Ar<S>;
  using Comp = typename A::Comp;
  const int lane = threadIdx.x & 31;
  const int r8 = lane & 7, c4 = lane >> 3;
  constexpr int NCOMP = SL * A::NC;
  constexpr int NCP = (NCOMP + 3) / 4 * 4;  // padded so the slots split over the 4 column lanes
  S acc[SL];
#pragma unroll
  for (int s = 0; s < SL; ++s) acc[s] = A::zero();
  const int iters = (mb - j - 1 + 3) >> 2;  // warp-uniform trip count
  for (int it = 0; it < iters; ++it) {
    const int b = j + 1 + c4 + 4 * it;
    const S xb = b < mb ? xv[b] : A::zero();
#pragma unroll
    for (int s = 0; s < SL; ++s) {
      const int a = base + r8 + 8 * s;
      if (b < mb && a < rows) acc[s] = A::fma(W[a * ldw + b], xb, acc[s]);
    }
  }
  Comp v[NCP];
#pragma unroll
  for (int s = 0; s < SL; ++s)
#pragma unroll
    for (int c = 0; c < A::NC; ++c) v[s * A::NC + c] = A::comp(acc[s], c);
#pragma unroll
  for (int i = NCOMP; i < NCP; ++i) v[i] = A::comp(A::zero(), 0);
  const bool h1 = (lane & 16) != 0, h2 = (lane & 8) != 0;
  if constexpr (NCOMP <= 2) {
    // one or two components: scatter them over lane bit 4 (two only), then a butterfly over bit 3
    // -- two adds where the padded reduce-scatter below takes three
    Comp z;
    if constexpr (NCOMP == 2) {
      const Comp send = h1 ? v[0] : v[1], keep = h1 ? v[1] : v[0];
      z = A::cadd(keep, A::shfl_xor(send, 16));
    } else {
      z = A::cadd(v[0], A::shfl_xor(v[0], 16));
    }
    z = A::cadd(z, A::shfl_xor(z, 8));
    __syncwarp();
    const int vi = NCOMP == 2 && h1 ? 1 : 0;
    const int s = vi / A::NC, part = vi % A::NC;
    const int a = base + r8 + 8 * s;
    if (!h2 && (NCOMP == 2 || !h1) && a < rows) reinterpret_cast<Comp*>(&W[a * ldw + j + 1])[part] = z;
  } else {
    Comp u[NCP / 2];
#pragma unroll
    for (int i = 0; i < NCP / 2; ++i) {
      Comp send = h1 ? v[i] : v[NCP / 2 + i];
      Comp keep = h1 ? v[NCP / 2 + i] : v[i];
      u[i] = A::cadd(keep, A::shfl_xor(send, 16));
    }
    Comp z[NCP / 4];
#pragma unroll
    for (int i = 0; i < NCP / 4; ++i) {
      Comp send = h2 ? u[i] : u[NCP / 4 + i];
      Comp keep = h2 ? u[NCP / 4 + i] : u[i];
      z[i] = A::cadd(keep, A::shfl_xor(send, 8));
    }
    __syncwarp();
    const int off = (h1 ? NCP / 2 : 0) + (h2 ? NCP / 4 : 0);
#pragma unroll
    for (int i = 0; i < NCP / 4; ++i) {
      const int vi = off + i;
      const int s = vi / A::NC, part = vi % A::NC;
      const int a = base + r8 + 8 * s;
      if (vi < NCOMP && a < rows) reinterpret_cast<Comp*>(&W[a * ldw + j + 1])[part] = z[i];
    }
  }
}

// ------------------------------------------------------------------------------------------
// Hessenberg reduction of the warp's tile by Gaussian elimination with partial pivoting.
// W is rows x ldw (row-major); the square part is mb x mb; rows mb..rows-1 are extra row
// vectors that receive the column operations only.
//
// FP64 scalars (normalised form): each step is the similarity X^-1 W X with X = I + (x - e)e^T,
// x = (0..0, piv, W[j+2][j], ..)^T, e = e_{j+1}: row j+1 is divided by the pivot and column
// j+1 becomes W x, so W[j+1][j] ends exactly 1 (or 0 when the column below the diagonal was
// zero) and La Budde needs no subdiagonal products.  The pivots compound geometrically under
// this scaling, which FP64's exponent range absorbs but FP32's does not, so
// double-float scalars use the classic form: multipliers l = W[a][j]/piv (|l| <= 1),
// W[j+1][j] keeps the pivot and column j+1 += sum_b W[:,b] l_b.
template <class S>
__device__ void hessenberg_elim(S* __restrict__ W, S* __restrict__ xv, int mb, int rows, int ldw, int nb) {
  using A = Ar<S>;
  const int lane = threadIdx.x & 31;

  // Normalised forms: row i of the tile is the classic elimination's row i divided by d_i, the
  // pivot row i was divided by when it was reduced (d = 1 for rows never divided), and column j
  // carries the factor d_j.  So the candidates of column j are d_j x their classic values and an
  // upper entry (i, j) is d_j / d_i x its classic value: with pivots below 1 (matrices of small
  // entries, such as Gaussian states' B) the candidates fall geometrically against the upper
  // rows -- by 1e-15 after 22 columns at |B| ~ 0.1 -- although nothing cancels.  The deflation
  // test is made in the classic frame: each upper key is raised by log2 d_i of its row, kept per
  // lane for the lane's rows nb + lane + 32 k (k < 3) as the pivot's binary exponent.
  constexpr bool kNorm = A::fp64 && !A::modular;
  int dexp[3] = {0, 0, 0};

  for (int j = 0; j + 1 < mb; ++j) {
    // --- pivot: largest max(|re|,|im|) in column j, rows j+1..mb-1, to 13 (FP64) or 16 (FP32
    // high part) significant bits, ties to the lowest row: the key's top bits and 127 - row packed
    // into one word, so one warp max-reduction picks it.  The same pass takes each lane's largest
    // key over the column's block rows nb..j (uk, never reduced): the column is deflated when
    // some lane's uk puts the best candidate at or below the deflation threshold, i.e. when max
    // uk does -- one vote, off the reduction.
    unsigned best = 0;
    unsigned long long uk = 0;
    long long ukn = 0;  // normalised forms: largest upper key in the classic frame
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int a = nb + lane + 32 * q;
      if (a < mb) {
        const unsigned long long k = A::key(W[a * ldw + j]);
        if (a > j) {
          const unsigned pk = (A::key32(k) & ~0x7fu) | (unsigned)(127 - a);
          best = pk > best ? pk : best;
        } else if constexpr (kNorm) {
          const long long k32 = (long long)A::key32(k);
          const long long adj = k32 ? k32 + ((long long)dexp[q] << 20) : 0;
          ukn = adj > ukn ? adj : ukn;
        } else {
          uk = k > uk ? k : uk;
        }
      }
    }
    best = __reduce_max_sync(0xffffffffu, best);
    bool deflate;
    if constexpr (kNorm) {
      const long long lb = (long long)(best & ~0x7fu);
      deflate = __any_sync(0xffffffffu, lb == 0 || lb <= ukn - ((long long)A::DEFLATE_BITS << 20));
    } else {
      deflate = __any_sync(0xffffffffu, (best & ~0x7fu) <= (A::key32(A::key_deflate(uk)) & ~0x7fu));
    }
    if (deflate) {
      // nothing to eliminate: the candidates are zero or rounding residues of an exact
      // cancellation; the subdiagonal becomes an exact zero and the column below it is cleared
      for (int a = j + 1 + lane; a < mb; a += 32) W[a * ldw + j] = A::zero();
      __syncwarp();
      continue;  // row j+1 is not divided: d_{j+1} = 1
    }
    const int p = 127 - (int)(best & 0x7fu);
    if (p != j + 1) {
      for (int c = j + lane; c < mb; c += 32) {
        S t = W[p * ldw + c];
        W[p * ldw + c] = W[(j + 1) * ldw + c];
        W[(j + 1) * ldw + c] = t;
      }
      __syncwarp();
      for (int r = lane; r < rows; r += 32) {
        S t = W[r * ldw + p];
        W[r * ldw + p] = W[r * ldw + j + 1];
        W[r * ldw + j + 1] = t;
      }
      __syncwarp();
    }
    const S piv = W[(j + 1) * ldw + j];
    const S rp = A::recip(piv);
    if constexpr (kNorm) {  // row j+1 is divided by piv: d_{j+1} = |piv| (as a binary exponent)
      const int e = (int)(A::key32(A::key(piv)) >> 20) - 1023;
#pragma unroll
      for (int q = 0; q < 3; ++q)
        if (nb + lane + 32 * q == j + 1) dexp[q] = e;
    }
    if constexpr (A::fp64) {
      for (int b = j + 1 + lane; b < mb; b += 32) xv[b] = (b == j + 1) ? piv : W[b * ldw + j];
      __syncwarp();
      // row j+1 /= piv  (the pivot itself becomes 1)
      for (int c = j + 1 + lane; c < mb; c += 32) W[(j + 1) * ldw + c] = A::mul(W[(j + 1) * ldw + c], rp);
      if (lane == 0) W[(j + 1) * ldw + j] = A::one();
    } else {
      for (int b = j + 1 + lane; b < mb; b += 32) xv[b] = (b == j + 1) ? A::one() : A::mul(W[b * ldw + j], rp);
    }
    __syncwarp();
    // --- phase A: rows j+2..mb-1, cols j+1..mb-1: W[a][b] -= x[a] * W[j+1][b]  (flattened)
    const int w = mb - j - 1;
    if (mb - j - 2 > 0) {
      // elements e = lane + 32 k (row-major over rows j+2.., cols j+1..) stepped without divisions;
      // full passes of 128 need no predicates, and the tail runs only the slots that hold elements
      // (a predicated FP64 instruction costs its issue slot even when no lane executes it)
      const int total = (mb - j - 2) * w;
      const int dr = 32 / w, dc = 32 % w;
      int a = j + 2 + lane / w, b = j + 1 + lane % w;
      const S* prow = W + (j + 1) * ldw;
      for (int pass = total >> 7; pass > 0; --pass) {  // four independent elements, loads before stores
        int aa[4], bb[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          aa[u] = a;
          bb[u] = b;
          b += dc;
          a += dr;
          if (b >= mb) { b -= w; a += 1; }
        }
        S vv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) vv[u] = A::fnma(xv[aa[u]], prow[bb[u]], W[aa[u] * ldw + bb[u]]);
#pragma unroll
        for (int u = 0; u < 4; ++u) W[aa[u] * ldw + bb[u]] = vv[u];
      }
      for (int rem = total & 127; rem > 0; rem -= 32) {
        if (a < mb) W[a * ldw + b] = A::fnma(xv[a], prow[b], W[a * ldw + b]);
        b += dc;
        a += dr;
        if (b >= mb) { b -= w; a += 1; }
      }
    }
    __syncwarp();
    // --- phase B: W[a][j+1] = sum_{b=j+1}^{mb-1} W[a][b] x[b] for every row a < rows.  Whole
    // 32-row blocks take one row per lane, summed in b order (every lane busy, no cross-lane
    // reduction), and so does a last block of 25..31 rows; fewer rows after the whole blocks take
    // 8 row lanes x 4 column lanes over just the 8-row slots they fill, then a reduce-scatter over
    // the column lanes (cheaper there than a mostly idle row-per-lane block).  The branches are
    // warp-uniform, so no FP64 instruction is issued for an empty slot.
    const int nfull = rows >> 5;
    for (int k0 = 0; k0 < nfull; k0 += 2) {
      if (nfull - k0 >= 2) phase_b_rows<S, 2>(W + 32 * k0 * ldw, xv, ldw, j, mb);
      else phase_b_rows<S, 1>(W + 32 * k0 * ldw, xv, ldw, j, mb);
    }
    const int rem = rows & 31;
    if (rem >= 25) {
      phase_b_rows<S, 1, true>(W + 32 * nfull * ldw, xv, ldw, j, mb, rem);
    } else if (rem > 0) {
      const int base = rows - rem;
      switch ((rem + 7) >> 3) {
        case 1: phase_b_split<S, 1>(W, xv, ldw, j, mb, rows, base); break;
        case 2: phase_b_split<S, 2>(W, xv, ldw, j, mb, rows, base); break;
        default: phase_b_split<S, 3>(W, xv, ldw, j, mb, rows, base); break;
      }
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------------------------------
// Storage of La Budde's coefficient rows c[i'][0..Kc].  Tile mode: rows 0..2 live in `win`
// (stride 3: row i' is only ever read at entries 0..i', its degree) and row i' >= 3 down block
// column i'-3 of the tile, which is dead by then (block column c is read at step c+1 for T_r and
// alpha and last at step c+2 for the subdiagonal entry); otherwise a circular window of kw rows
// (slot = i' mod kw) when the tile cannot hold Kc+1 entries per column.
template <class S>
__device__ __forceinline__ S& cw_at(S* W, int ldw, int nb, S* win, int kw, bool tile, int ip, int slot, int u) {
  if (tile) return ip >= 3 ? W[u * ldw + nb + ip - 3] : win[ip * 3 + u];
  return win[slot * kw + u];
}

// La Budde's recurrence on the Hessenberg block H (block index 1..m maps to tile index
// nb..nb+m-1).  Writes c[0..Kc] of det(I - eta H) = sum_j c_j eta^j to cpoly.
//   c[i][j] = c[i-1][j] - H(i,i) c[i-1][j-1] - sum_{r=1}^{j-1} T_r c[i-r-1][j-r-1],
//   T_r = H(i-r,i) beta_i beta_{i-1} ... beta_{i-r+1},  beta_k = H(k,k-1)
// (charpoly.py:195-282).  In the normalised FP64 form every beta is 1 or 0, so T_r is H(i-r,i)
// up to the last zero beta; otherwise the beta products come from a lane prefix-product scan.
template <class S>
__device__ void labudde(S* __restrict__ W, int ldw, int nb, int m, int Kc, S* __restrict__ win, int kw, bool tile,
                        S* __restrict__ tb, S* __restrict__ part, S* __restrict__ cpoly,
                        const LbLane* __restrict__ lbl, const LbOwner* __restrict__ lbo,
                        const LbLane2* __restrict__ lbl2, const LbOwner2* __restrict__ lbo2) {
  using A = Ar<S>;
  const int lane = threadIdx.x & 31;
  for (int jj = lane; jj <= (tile ? 0 : Kc); jj += 32)
    cw_at(W, ldw, nb, win, kw, tile, 0, 0, jj) = (jj == 0) ? A::one() : A::zero();
  __syncwarp();
  int zlast = 1;
  int prow = 0;  // circular-window slot of row i-1
  // subdiagonal products P(i, r) = beta_i ... beta_{i-r+1} for r = lane+1 and lane+33, kept in
  // registers across rows: P(i, r) = beta_i * P(i-1, r-1), P(i, 1) = beta_i
  S pr0 = A::zero(), pr1 = A::zero();
  // T_r of row i: the normalised forms read T_r = H(i-r, i) from tile column nb+i-1 (still
  // intact: La Budde rows go to columns up to nb+i-3), the others get tbr[1..R] filled; returns
  // the last usable r
  auto fill_tb = [&](int i, S* tbr) -> int {
    const int wi = nb + i - 1;
    const int R = (i - 1) < (Kc - 1) ? (i - 1) : (Kc - 1);
    int rcap = R;
    if constexpr (A::fp64) {
      if (i >= 2 && A::is_zero(W[wi * ldw + wi - 1])) zlast = i;
      rcap = (i - zlast) < R ? (i - zlast) : R;
    } else {
      const S bi = i >= 2 ? W[wi * ldw + wi - 1] : A::zero();
      const S up0 = shfl_up_s(pr0, 1);  // P(i-1, r-1) for r = lane+1
      const S prev0 = lane == 0 ? A::one() : up0;
      if (Kc > 33) {  // the second block of products (r = lane+33 <= Kc-1) only when it is read
        const S up1 = shfl_up_s(pr1, 1);
        const S last0 = A::shfl(pr0, 31);  // P(i-1, 32) feeds r = 33
        const S prev1 = lane == 0 ? last0 : up1;
        pr1 = A::mul(bi, prev1);
      }
      pr0 = A::mul(bi, prev0);
      if (lane + 1 <= R) tbr[lane + 1] = A::mul(W[(wi - lane - 1) * ldw + wi], pr0);
      if (lane + 33 <= R) tbr[lane + 33] = A::mul(W[(wi - lane - 33) * ldw + wi], pr1);
    }
    return rcap;
  };
  for (int i = 1; i <= m;) {
    if (Kc >= 2 && Kc <= LB2_KMAX && i + 1 <= m) {
      // ---- rows i and i+1 together: both r-sums need rows <= i-1 only
      const int K0 = i < Kc ? i : Kc, K1 = i + 1 < Kc ? i + 1 : Kc;
      const int sid = lb2_id(K0, K1);
      const int rc0 = fill_tb(i, tb);
      const int rc1 = fill_tb(i + 1, tb + kw);
      __syncwarp();
      const int wi = nb + i - 1;
      const S alpha0 = W[wi * ldw + wi], alpha1 = W[(wi + 1) * ldw + wi + 1];
      const int c0 = prow + 1 == kw ? 0 : prow + 1;  // circular slots of rows i and i+1
      const int c1 = c0 + 1 == kw ? 0 : c0 + 1;
      // the owner pass's inputs, taken before the pieces so that their latency overlaps them: the
      // owner record (one 16-byte load) and c[i-1][jj] - alpha0 c[i-1][jj-1] (row i-1 is final).
      // Measured at n = 40: complex FP64 -0.8 %, real FP64 -1.4 %, real double-float -10 %; complex
      // double-float +5.7 % (its piece loop wants the registers) and double-double (would spill)
      // take both after the pieces instead
      constexpr bool kEarly = !A::dd && (A::fp64 || !A::cplx);
      const int jj = lane + 1;
      auto load_owner = [&]() -> uint4 {
        return reinterpret_cast<const uint4*>(lbo2)[sid * (LB2_KMAX + 1) + (jj <= K1 ? jj : 0)];
      };
      auto row_i_start = [&]() -> S {
        const S cp = (jj <= i - 1) ? cw_at(W, ldw, nb, win, kw, tile, i - 1, prow, jj) : A::zero();
        return A::fnma(alpha0, cw_at(W, ldw, nb, win, kw, tile, i - 1, prow, jj - 1), cp);
      };
      uint4 owr = make_uint4(0u, 0u, 0u, 0u);
      S ci0 = A::zero();
      if constexpr (kEarly) {
        owr = load_owner();
        if (jj <= K0) ci0 = row_i_start();
      }
      {
        const LbLane2 sc = lbl2[sid * 32 + lane];
        const int l0 = sc.len[0], l1 = sc.len[1], l2 = sc.len[2];
        const int tot = l0 + l1 + l2;
        S acc = A::zero();
        if ((A::fp64 || A::cplx) && tile && i >= Kc + 3 && rc0 == Kc - 1 && rc1 == Kc - 1) {
          // steady state of the tile form: every c[i+row-r-1] read lives in the tile and no
          // subdiagonal zero truncates the sums, so along a piece both operands step linearly --
          // T_r = W[wi+row-r][wi+row] by -ldw (normalised forms; complex double-float reads its
          // products tb[row kw + r] by +1), c[i+row-r-1][j-r-1] = W[j-r-1][nb+i+row-r-4] by
          // -(ldw+1) -- and an iteration is two loads and one multiply-add.  (Real double-float
          // measured 3 % slower in this form than in the general loop below: it keeps that.)
          const S* __restrict__ Tsrc = A::fp64 ? W : tb;
          const int sT = A::fp64 ? -ldw : 1;
          int oT[3], oC[3];
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            const int row = (sc.rowmask >> q) & 1, jq = sc.j[q], r0 = sc.rlo[q];
            oT[q] = A::fp64 ? (wi + row - r0) * ldw + wi + row : row * kw + r0;
            oC[q] = (jq - r0 - 1) * ldw + nb + i + row - r0 - 4;
          }
          int q = 0, left = l0, pT = oT[0], pC = oC[0];
          for (int it = 0; it < tot; ++it) {
            if (left == 0) {  // next piece
              part[3 * lane + q] = acc;
              acc = A::zero();
              ++q;
              left = q == 1 ? l1 : l2;
              pT = q == 1 ? oT[1] : oT[2];
              pC = q == 1 ? oC[1] : oC[2];
            }
            acc = A::fma(Tsrc[pT], W[pC], acc);
            pT += sT;
            pC -= ldw + 1;
            --left;
          }
        } else {
        for (int it = 0; it < tot; ++it) {
          const int q = (it >= l0) + (it >= l0 + l1);
          const int start = q == 0 ? 0 : (q == 1 ? l0 : l0 + l1);
          if (it == start && it > 0) {
            part[3 * lane + q - 1] = acc;
            acc = A::zero();
          }
          const int row = (sc.rowmask >> q) & 1;
          const int j = q == 0 ? sc.j[0] : (q == 1 ? sc.j[1] : sc.j[2]);
          const int r = (q == 0 ? sc.rlo[0] : (q == 1 ? sc.rlo[1] : sc.rlo[2])) + (it - start);
          if (r <= (row ? rc1 : rc0)) {
            int slot = prow + row - r;  // circular slot of row i+row-r-1
            if (slot < 0) slot += kw;
            const S cv = cw_at(W, ldw, nb, win, kw, tile, i + row - r - 1, slot, j - r - 1);
            const S tr = A::fp64 ? W[(wi + row - r) * ldw + wi + row] : tb[row * kw + r];
            acc = A::fma(tr, cv, acc);
          }
        }
        }
        if (tot > 0) part[3 * lane + (l2 > 0 ? 2 : (l1 > 0 ? 1 : 0))] = acc;
      }
      __syncwarp();
      if constexpr (!kEarly) owr = load_owner();
      S ci = A::zero();  // c[i][jj]: zero above row i's degree (jj = i + 1 in the triangle)
      if (jj <= K0) {
        S val = ci0;
        if constexpr (!kEarly) val = row_i_start();
        const int n0 = owner_byte(owr, 0);
        for (int k = 0; k < n0; ++k) val = A::sub(val, part[owner_byte(owr, 2 + k)]);
        ci = val;
      }
      S cim1 = shfl_up_s(ci, 1);  // c[i][jj-1]
      if (lane == 0) cim1 = A::one();
      if (jj <= K1) {
        S v1 = A::fnma(alpha1, cim1, ci);
        const int n1 = owner_byte(owr, 1);
        for (int k = 0; k < n1; ++k) v1 = A::sub(v1, part[owner_byte(owr, 9 + k)]);
        if (jj <= K0) cw_at(W, ldw, nb, win, kw, tile, i, c0, jj) = ci;
        cw_at(W, ldw, nb, win, kw, tile, i + 1, c1, jj) = v1;
      }
      if (lane == 0) {
        cw_at(W, ldw, nb, win, kw, tile, i, c0, 0) = A::one();
        cw_at(W, ldw, nb, win, kw, tile, i + 1, c1, 0) = A::one();
      }
      prow = c1;
      __syncwarp();
      i += 2;
      continue;
    }
    // ---- one row
    const int wi = nb + i - 1;
    const int rcap = fill_tb(i, tb);
    __syncwarp();
    const S alpha = W[wi * ldw + wi];
    const int Ki = i < Kc ? i : Kc;
    const int crow = prow + 1 == kw ? 0 : prow + 1;
    // pieces of sum_r T_r c[i-r-1][j-r-1], balanced over the lanes (two accumulators for ILP)
    {
      const LbLane sc = lbl[Ki * 32 + lane];
      const int lena = sc.lena, tot = sc.lena + sc.lenb;
      S acc0 = A::zero(), acc1 = A::zero(), pa = A::zero();
      for (int it = 0; it < tot; ++it) {
        const bool sec = it >= lena;
        if (it == lena) { pa = A::add(acc0, acc1); acc0 = A::zero(); acc1 = A::zero(); }
        const int j = sec ? sc.jb : sc.ja;
        const int r = sec ? sc.rlob + (it - lena) : sc.rloa + it;
        if (r <= rcap) {
          int slot = prow - r;  // circular slot of row i-r-1 (row i-1 is in prow)
          if (slot < 0) slot += kw;
          const S cv = cw_at(W, ldw, nb, win, kw, tile, i - r - 1, slot, j - r - 1);
          const S tr = A::fp64 ? W[(wi - r) * ldw + wi] : tb[r];
          if (it & 1) acc1 = A::fma(tr, cv, acc1);
          else acc0 = A::fma(tr, cv, acc0);
        }
      }
      const S acc = A::add(acc0, acc1);
      if (sc.lenb) {
        part[2 * lane] = pa;
        part[2 * lane + 1] = acc;
      } else {
        part[2 * lane] = acc;
      }
    }
    __syncwarp();
    for (int jj = lane + 1; jj <= Ki; jj += 32) {
      S val = (jj <= i - 1) ? cw_at(W, ldw, nb, win, kw, tile, i - 1, prow, jj) : A::zero();
      val = A::fnma(alpha, cw_at(W, ldw, nb, win, kw, tile, i - 1, prow, jj - 1), val);
      const LbOwner* ow = &lbo[Ki * (LB_KMAX + 1) + jj];
      for (int k = 0; k < ow->n; ++k) val = A::sub(val, part[ow->s[k]]);
      cw_at(W, ldw, nb, win, kw, tile, i, crow, jj) = val;
    }
    if (lane == 0) cw_at(W, ldw, nb, win, kw, tile, i, crow, 0) = A::one();
    prow = crow;
    __syncwarp();
    ++i;
  }
  for (int jj = lane; jj <= Kc; jj += 32) cpoly[jj] = cw_at(W, ldw, nb, win, kw, tile, m, prow, jj);
  __syncwarp();
}

// g = (sum_j c_j eta^j)^(-1/2) up to degree G:  n g_n = -sum_{i=1}^{n} c_i (n - i/2) g_{n-i}.
// Right-looking: once g_k is final, every later coefficient n (n - k <= Kc) takes its term
// c_{n-k} ((n + k)/2) g_k at once, one lane per coefficient; g_{k+1} is then complete and is
// finalised by its lane.  No warp reductions: 2 DMUL + 4 DFMA per step and lane.
template <class S>
__device__ void inv_sqrt_series(const S* __restrict__ cpoly, int Kc, S* __restrict__ g, int G) {
  using A = Ar<S>;
  const int lane = threadIdx.x & 31;
  for (int n = lane; n <= G; n += 32) g[n] = n == 0 ? A::one() : A::zero();
  __syncwarp();
  for (int k = 0; k < G; ++k) {
    const S gk = g[k];
    const int hi = (k + Kc) < G ? (k + Kc) : G;
    for (int n = k + 1 + lane; n <= hi; n += 32) {
      S acc;
      if constexpr (A::modular) {
        acc = A::fma(cpoly[n - k], A::mul(gk, A::mul(A::of_int(n + k), A::half())), g[n]);
        if (n == k + 1) acc = A::neg(A::mul(acc, inv_of<S>(n)));
      } else {
        acc = A::fma(cpoly[n - k], A::scale_f(gk, 0.5f * (float)(n + k)), g[n]);
        if constexpr (A::fp64 && !A::dd) {
          if (n == k + 1) acc = A::scale(acc, -inv_int(n));
        } else {  // 1/n to the type's precision, in its own instructions
          if (n == k + 1) acc = A::neg(A::div_int(acc, n));
        }
      }
      g[n] = acc;
    }
    __syncwarp();
  }
}

// e = exp(sum_{l=1}^{Q} q_l z^l) up to degree G:  n e_n = sum_{l=1}^{n} l q_l e_{n-l}, in the same
// right-looking form (q is read as l q_l on the fly).
template <class S>
__device__ void exp_series(const S* __restrict__ q, int Q, S* __restrict__ e, int G) {
  using A = Ar<S>;
  const int lane = threadIdx.x & 31;
  for (int n = lane; n <= G; n += 32) e[n] = n == 0 ? A::one() : A::zero();
  __syncwarp();
  for (int k = 0; k < G; ++k) {
    const S ek = e[k];
    const int hi = (k + Q) < G ? (k + Q) : G;
    for (int n = k + 1 + lane; n <= hi; n += 32) {
      S acc;
      if constexpr (A::modular) {
        acc = A::fma(A::mul(q[n - k], A::of_int(n - k)), ek, e[n]);
        if (n == k + 1) acc = A::mul(acc, inv_of<S>(n));
      } else {
        acc = A::fma(A::scale_f(q[n - k], (float)(n - k)), ek, e[n]);
        if constexpr (A::fp64 && !A::dd) {
          if (n == k + 1) acc = A::scale(acc, inv_int(n));
        } else {
          if (n == k + 1) acc = A::div_int(acc, n);
        }
      }
      e[n] = acc;
    }
    __syncwarp();
  }
}

// Border data of the loop variants, without a Krylov sequence.  After the elimination the
// border column is d e_1 (block index 1..m = tile index 1..m, nb = 1) and H is upper Hessenberg
// with subdiagonal beta_i = H(i+1, i), so lam_t = d x.H^(t-1) e_1 (x = tile row 0; mu, mu0 the
// same with the extra rows y = tile rows mb, mb+1) has the generating function
//   sum_t lam_t z^t = d z x.(I - zH)^-1 e_1,
// and Cramer's rule on the Hessenberg matrix I - zH gives its first column:
//   [(I - zH)^-1]_{r,1} = z^(r-1) beta_1 .. beta_(r-1) Q_r(z) / P(z),
// Q_r(z) = det(I - z H[r+1..m, r+1..m]) (the trailing principal submatrices; Q_m = 1), P = Q_0.
// The anti-transpose H' = J H^T J is upper Hessenberg too and its leading submatrices are the
// trailing ones of H reversed and transposed -- the same determinants -- so La Budde run on H'
// yields P as usual and every Q_r as its row m - r.  Hence
//   sum_t lam_t z^t = d sum_{r=1}^{min(m,T)} x_r beta_1 .. beta_(r-1) z^r Q_r(z) / P(z):
// one sweep of T multiply-adds per series for the numerator and one for the division by P,
// where the Krylov sequence v_(t+1) = H v_t took T(T+1)/2 warp-wide steps (a third of the
// loop kinds' time at 40 photons).  (The reference forms the same quantities as matrix powers:
// loop_hafnian_batch.py f_loop / f_loop_odd, _hafnian.py f_loop.)

// Before La Budde (m >= 1): the weights w_r = x_r beta_1 .. beta_(r-1), r = 1..min(m, T), into
// xs (and the extra rows' into ys, y0s), then the Hessenberg block anti-transposed in place.
// The normalised forms have beta in {0, 1}: the weights stop at the first zero; double-float
// takes the products by a prefix scan over the lanes.
template <class S>
__device__ void border_prepare(S* __restrict__ W, int ldw, int m, int mb, int ne, int T, S* __restrict__ xs,
                               S* __restrict__ ys, S* __restrict__ y0s) {
  using A = Ar<S>;
  const int lane = threadIdx.x & 31;
  const int R = T < m ? T : m;
  S carry = A::one();  // double-float: product of the betas before this chunk
  int cut = R + 1;      // normalised forms: first r whose weight is zero
  for (int r0 = 1; r0 <= R; r0 += 32) {
    const int r = r0 + lane;
    // b = beta_(r-1) (r >= 2), the factor that joins at r
    const S b = (r >= 2 && r <= R) ? W[r * ldw + r - 1] : A::one();
    S w;
    if constexpr (A::fp64) {
      const unsigned z = __ballot_sync(0xffffffffu, r <= R && A::is_zero(b));
      if (z && cut > R) cut = r0 + __ffs(z) - 1;
      w = A::one();
    } else {  // inclusive prefix product of b over the lanes, times the carry
      w = b;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const S u = A::shfl(w, lane >= off ? lane - off : lane);
        if (lane >= off) w = A::mul(u, w);
      }
      w = A::mul(carry, w);
      carry = A::shfl(w, 31);
    }
    if (r <= R) {
      const bool live = r < cut;
      xs[r] = live ? A::mul(W[r], w) : A::zero();
      if (ne > 0) ys[r] = live ? A::mul(W[mb * ldw + r], w) : A::zero();
      if (ne > 1) y0s[r] = live ? A::mul(W[(mb + 1) * ldw + r], w) : A::zero();
    }
  }
  __syncwarp();
  // anti-transpose of the block: (a, b) <-> (m+1-b, m+1-a) over the upper Hessenberg entries
  // (b >= a-1, a set the map keeps), each pair swapped once from its member with a + b < m + 1
  const int c = m + 1;
  for (int a = 1; a + (a > 1 ? a - 1 : 1) < c; ++a) {
    const int b0 = a > 1 ? a - 1 : 1;
    for (int b = b0 + lane; a + b < c; b += 32) {
      S& p = W[a * ldw + b];
      S& q = W[(c - b) * ldw + (c - a)];
      const S t = p;
      p = q;
      q = t;
    }
  }
  __syncwarp();
}

// After La Budde on the anti-transposed block: lam_t (mu_t, mu0_t), t = 1..T, from the weights
// in lam (mu, mu0), the coefficient rows Q_r (La Budde's row m - r) and P = cpoly, overwriting
// the weights; n0..n2 are scratch series (T + 1 entries).
template <class S>
__device__ void border_series(S* __restrict__ W, int ldw, int m, int Kc, S* __restrict__ win, int kw, bool tile,
                              const S* __restrict__ cpoly, int T, int ne, S d, S* __restrict__ lam,
                              S* __restrict__ mu, S* __restrict__ mu0, S* __restrict__ n0,
                              S* __restrict__ n1, S* __restrict__ n2) {
  using A = Ar<S>;
  const int lane = threadIdx.x & 31;
  const int R = T < m ? T : m;
  // numerators: N_t = sum_{r <= min(t, R)} w_r Q_r[t - r]  (Q_r of degree min(m - r, Kc))
  for (int t = 1 + lane; t - lane <= T; t += 32) {
    S a0 = A::zero(), a1 = A::zero(), a2 = A::zero();
    for (int r = 1; r <= R; ++r) {
      const int i = m - r, k = t - r;
      if (t <= T && k >= 0 && k <= (i < Kc ? i : Kc)) {
        const S q = cw_at(W, ldw, 1, win, kw, tile, i, i % kw, k);
        a0 = A::fma(lam[r], q, a0);
        if (ne > 0) a1 = A::fma(mu[r], q, a1);
        if (ne > 1) a2 = A::fma(mu0[r], q, a2);
      }
    }
    if (t <= T) {
      n0[t] = a0;
      if (ne > 0) n1[t] = a1;
      if (ne > 1) n2[t] = a2;
    }
  }
  __syncwarp();
  // division by P (P_0 = 1, P_j = 0 above Kc), right-looking: once L_k is final every later
  // L_t takes -P_(t-k) L_k
  for (int k = 1; k < T; ++k) {
    const S l0 = n0[k];
    const S l1 = ne > 0 ? n1[k] : A::zero();
    const S l2 = ne > 1 ? n2[k] : A::zero();
    const int hi = (k + Kc) < T ? (k + Kc) : T;
    for (int t = k + 1 + lane; t <= hi; t += 32) {
      const S p = cpoly[t - k];
      n0[t] = A::fnma(p, l0, n0[t]);
      if (ne > 0) n1[t] = A::fnma(p, l1, n1[t]);
      if (ne > 1) n2[t] = A::fnma(p, l2, n2[t]);
    }
    __syncwarp();
  }
  for (int t = 1 + lane; t <= T; t += 32) {
    lam[t] = A::mul(d, n0[t]);
    if (ne > 0) mu[t] = A::mul(d, n1[t]);
    if (ne > 1) mu0[t] = A::mul(d, n2[t]);
  }
  __syncwarp();
}

// ------------------------------------------------------------------------------------------
template <class S>
static __global__ void __launch_bounds__(256) sieve_kernel(const SieveParams P) {
  using A = Ar<S>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const WarpLayout& L = P.L;
  unsigned char* ws = smem + (size_t)warp * L.bytes;
  S* W = reinterpret_cast<S*>(ws);
  S* xv = reinterpret_cast<S*>(ws + L.off_x);
  S* win = reinterpret_cast<S*>(ws + L.off_win);
  S* tb = reinterpret_cast<S*>(ws + L.off_tb);
  S* lbpart = reinterpret_cast<S*>(ws + L.off_part);
  S* ser = reinterpret_cast<S*>(ws + L.off_ser);
  short* srow = reinterpret_cast<short*>(ws + L.off_int);
  short* scol = srow + L.rows;
  short* sdel = scol + L.ldw;
  const int ldw = L.ldw;
  const int ns = L.nser;
  S* cpoly = ser;           // [0, ns)
  S* gser = ser + ns;       // [ns, 2ns)
  S* eser = ser + 2 * ns;   // even exp series (before it: a border-series numerator)
  S* oser = ser + 3 * ns;   // odd exp series (before it: a border-series numerator)
  S* lam = ser + 4 * ns;    // border series of x (before it: its weights); likewise mu, mu0
  S* mu = ser + 5 * ns;
  S* mu0 = ser + 6 * ns;
  S* qv = ser + 7 * ns;     // series exponents (before them: a border-series numerator)

  for (;;) {
    int c = 0;
    if (lane == 0) c = (int)atomicAdd(P.counter, 1u);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= P.nchunks) break;
    const ChunkDev ch = P.chunks[c];
    const InstDev& I = P.inst[ch.inst];
    const int kind = I.kind, E = I.E, n = I.n, nb = I.nb, ne = I.ne, glynn = I.glynn;
    const int lda = I.lda;
    const S* Aext = reinterpret_cast<const S*>(P.pool + I.a_off);
    const int R = lane < E ? I.radix[lane] : 1;
    const int rep = lane < E ? I.reps[lane] : 0;
    const int nout = I.nout;

    // initial reflected mixed-radix Gray digits of t0 (edge 0 most significant)
    int myd = 0;
    {
      long long tt = ch.t0;
      for (int i = E - 1; i >= 0; --i) {
        const int Ri = I.radix[i];
        const int d = (int)(tt % Ri);
        tt /= Ri;
        if (lane == i) myd = d;
      }
    }
    int g = 0, dir = 1;
    {
      int f = 0;
      for (int i = 0; i < E; ++i) {
        const int d = __shfl_sync(0xffffffffu, myd, i);
        const int Ri = I.radix[i];
        const int gi = f ? Ri - 1 - d : d;
        if (lane == i) { g = gi; dir = f ? -1 : 1; }
        f ^= (gi & 1);
      }
    }
    double s_re = 0, s_im = 0, k_re = 0, k_im = 0;  // lane o: Neumaier sum of output o
    double mag = 0;                                   // lane o: sum of |re| + |im| of its terms
    S macc = A::zero();                               // modular kinds: lane o's residue sum

    for (long long t = ch.t0; t < ch.t1; ++t) {
      if (t != ch.t0) {  // Gray step: least significant digit that can move in its direction
        const int ng = g + dir;
        const unsigned can = __ballot_sync(0xffffffffu, lane < E && ng >= 0 && ng < R);
        const int i = 31 - __clz(can);
        if (lane == i) g = ng;
        if (lane > i && lane < E) dir = -dir;
      }
      const int delta = lane < E ? (glynn ? 2 * g - rep : g) : 0;
      const unsigned nz = __ballot_sync(0xffffffffu, delta != 0);
      const bool unit_delta = __all_sync(0xffffffffu, delta >= -1 && delta <= 1);  // signs only
      const int Ep = __popc(nz);
      const int m = 2 * Ep;
      const int mb = m + nb;
      const int rows = mb + ne;
      // kept-sum and binomial product
      int ksum = lane < E ? g : 0;
#pragma unroll
      for (int off = 16; off; off >>= 1) ksum += __shfl_xor_sync(0xffffffffu, ksum, off);
      const bool batch = kind >= KIND_BATCH_EVEN;
      double bin = 1.0;
      S binm = A::one();  // modular kinds: the binomial product as a residue (exact)
      if (!I.unit_binoms) {
        bin = (lane < E && !(batch && lane == 0)) ? c_binom[rep][g] : 1.0;
        if constexpr (A::modular) {
          binm = A::of_int((long long)bin);
#pragma unroll
          for (int off = 16; off; off >>= 1) binm = A::mul(binm, A::shfl_xor(binm, off));
        } else {
#pragma unroll
          for (int off = 16; off; off >>= 1) bin *= __shfl_xor_sync(0xffffffffu, bin, off);
        }
      }
      // prefactor x term into the lane's sum: parity gives the sign, halve the Glynn halving
      // of the delta_0 = 0 term, binx an extra binomial (batch outputs)
      auto accum = [&](int parity, bool halve, S f, double binx) {
        if constexpr (A::modular) {
          S t = A::mul(binm, f);
          if (binx != 1.0) t = A::mul(t, A::of_int((long long)binx));
          if (parity) t = A::neg(t);
          if (halve) t = A::mul(t, A::half());
          macc = A::add(macc, t);
        } else {
          double pre = binx * bin;
          if (parity) pre = -pre;
          if (halve) pre *= 0.5;
          const c64 z = A::to_c64(f);
          const double xr = pre * z.re, xi = pre * z.im;
          neumaier(s_re, k_re, xr);
          neumaier(s_im, k_im, xi);
          mag += fabs(xr) + fabs(xi);
          if constexpr (A::dd) {  // the product's rounding error and the low parts join the compensation
            const c64 zl = A::lo_c64(f);
            k_re += ::fma(pre, z.re, -xr) + pre * zl.re;
            k_im += ::fma(pre, z.im, -xi) + pre * zl.im;
          }
        }
      };
      const int g0 = __shfl_sync(0xffffffffu, g, 0);
      const int g1 = __shfl_sync(0xffffffffu, g, 1);
      const int d0 = __shfl_sync(0xffffffffu, delta, 0);
      // index maps of the tile
      if (delta != 0) {
        const int pos = __popc(nz & ((1u << lane) - 1u));
        srow[nb + pos] = (short)lane;
        srow[nb + Ep + pos] = (short)(E + lane);
        scol[nb + pos] = (short)(E + lane);
        scol[nb + Ep + pos] = (short)lane;
        sdel[nb + pos] = (short)delta;
        sdel[nb + Ep + pos] = (short)delta;
      }
      if (lane == 0 && nb) { srow[0] = (short)n; scol[0] = (short)n; sdel[0] = 1; }
      if (lane < ne) srow[mb + lane] = (short)(n + 1 + lane);
      __syncwarp();
      // gather the tile
      if (mb > 0) {
        const int total = rows * mb;
        const int dr = 32 / mb, dc = 32 % mb;
        int r = lane / mb, cc = lane % mb;
        if (unit_delta) {  // sign flips on the integer pipe
          for (int e = lane; e < total; e += 32) {
            const S x = Aext[(size_t)srow[r] * lda + scol[cc]];
            W[r * ldw + cc] = sdel[cc] < 0 ? A::neg(x) : x;
            cc += dc;
            r += dr;
            if (cc >= mb) { cc -= mb; r += 1; }
          }
        } else {
          for (int e = lane; e < total; e += 32) {
            const S x = Aext[(size_t)srow[r] * lda + scol[cc]];
            W[r * ldw + cc] = scale_int(x, sdel[cc]);
            cc += dc;
            r += dr;
            if (cc >= mb) { cc -= mb; r += 1; }
          }
        }
      }
      __syncwarp();
      hessenberg_elim<S>(W, xv, mb, rows, ldw, nb);
      // loop variants: the border's weights are read off the tile and the block anti-transposed,
      // so that La Budde also yields the trailing submatrices' determinants (border_prepare)
      const int Kc = I.K < m ? I.K : m;
      const S dbord = (kind != KIND_PLAIN && m > 0) ? W[1 * ldw + 0] : A::zero();
      const bool border = kind != KIND_PLAIN && m > 0 && !A::is_zero(dbord);
      if (border) border_prepare<S>(W, ldw, m, mb, ne, I.K, lam, mu, mu0);
      // characteristic polynomial coefficients of the block (xv is free again: it may hold tb)
      labudde<S>(W, ldw, nb, m, Kc, win, L.kw, L.tilewin != 0, tb, lbpart, cpoly, P.lb_lane, P.lb_own,
                 P.lb_lane2, P.lb_own2);
      if (border) {
        border_series<S>(W, ldw, m, Kc, win, L.kw, L.tilewin != 0, cpoly, I.K, ne, dbord, lam, mu, mu0, eser,
                         oser, qv);
      } else if (kind != KIND_PLAIN) {
        for (int t = lane; t <= I.K; t += 32) {
          lam[t] = A::zero();
          if (ne > 0) mu[t] = A::zero();
          if (ne > 1) mu0[t] = A::zero();
        }
        __syncwarp();
      }
      const int Gdeg = I.K;  // degree of det^(-1/2) needed
      inv_sqrt_series<S>(cpoly, Kc, gser, Gdeg);

      if (kind == KIND_PLAIN) {
        if (lane == 0) accum((I.N / 2 - ksum) & 1, glynn && d0 == 0, gser[I.K], 1.0);
      } else {
        const int T = I.K;
        // even series: q_l = lam_l / 2, e = exp(q), f_even[h] = sum_t g_t e_{h-t}
        if (kind == KIND_LOOP || kind == KIND_BATCH_EVEN || kind == KIND_BATCH_ODD) {
          for (int l = lane; l <= T; l += 32) qv[l] = l ? half_of<S>(lam[l]) : A::zero();
          __syncwarp();
          exp_series<S>(qv, T, eser, T);
        }
        if (kind == KIND_LOOP) {
          S part = A::zero();
          for (int tq = lane; tq <= T; tq += 32) part = A::fma(gser[tq], eser[T - tq], part);
          part = warp_sum(part);
          if (lane == 0) accum((I.N / 2 - ksum) & 1, glynn && d0 == 0, part, 1.0);
        } else {
          // odd series in zeta: q'_1 = oddloop, q'_{2l} = lam_l/2, q'_{2l+1} = mu_l
          const int No = I.Nodd;
          __syncwarp();
          for (int l = lane; l <= No; l += 32) {
            S q;
            if (l == 0) q = A::zero();
            else if (l == 1) q = A::from_c64(I.oddloop);
            else if ((l & 1) == 0) q = (l / 2 <= T) ? half_of<S>(lam[l / 2]) : A::zero();
            else q = ((l - 1) / 2 <= T) ? mu[(l - 1) / 2] : A::zero();
            qv[l] = q;
          }
          __syncwarp();
          exp_series<S>(qv, No, oser, No);
          if (kind == KIND_LOOP_ODD) {
            S part = A::zero();
            for (int tq = lane; 2 * tq <= No; tq += 32) part = A::fma(gser[tq], oser[No - 2 * tq], part);
            part = warp_sum(part);
            if (lane == 0) accum((I.N / 2 - ksum) & 1, false, part, 1.0);
          } else {
            // batch: lane o handles output N_det = o
            const bool odd = kind == KIND_BATCH_ODD;
            const int Nf = I.N;
            if (odd && g0 == 0 && g1 == 0) {
              // f_loop_odd at N_fixed with the second odd mode (loop_hafnian_batch.py:181-185)
              __syncwarp();
              for (int l = lane; l <= Nf; l += 32) {
                S q;
                if (l == 0) q = A::zero();
                else if (l == 1) q = A::from_c64(I.oddloop0);
                else if ((l & 1) == 0) q = (l / 2 <= T) ? half_of<S>(lam[l / 2]) : A::zero();
                else q = ((l - 1) / 2 <= T) ? mu0[(l - 1) / 2] : A::zero();
                qv[l] = q;
              }
              __syncwarp();
              exp_series<S>(qv, Nf, mu0, Nf);  // mu0 was copied into qv above
              S part = A::zero();
              for (int tq = lane; 2 * tq <= Nf; tq += 32) part = A::fma(gser[tq], mu0[Nf - 2 * tq], part);
              part = warp_sum(part);
              if (lane == 0) accum((Nf / 2 - ksum) & 1, false, part, 1.0);
            }
            __syncwarp();
            for (int o = 0; o < nout; ++o) {
              const int start = odd ? 2 * g0 + 1 : 2 * g0;
              if (o < start) continue;
              const int Nn = Nf + o;
              S part = A::zero();
              if ((Nn & 1) == 0) {
                const int h = Nn / 2;
                for (int tq = lane; tq <= h; tq += 32) part = A::fma(gser[tq], eser[h - tq], part);
              } else {
                for (int tq = lane; 2 * tq <= Nn; tq += 32) part = A::fma(gser[tq], oser[Nn - 2 * tq], part);
              }
              part = warp_sum(part);
              if (lane == o % 32) accum((Nn / 2 - ksum) & 1, false, part, c_binom[odd ? (o - 1) / 2 : o / 2][g0]);
            }
          }
        }
      }
      __syncwarp();
    }
    if constexpr (A::modular) {
      if (lane < nout) P.partials[ch.part + lane] = make_double2((double)A::to_c64(macc).re, 0.0);
    } else if constexpr (A::dd) {  // sum and compensation kept apart
      if (lane < nout) {
        P.partials[ch.part + lane] = make_double2(s_re, s_im);
        P.partials[ch.part + I.comp_off + lane] = make_double2(k_re, k_im);
        if (I.mag_off) P.partials[ch.part + I.mag_off + lane] = make_double2(mag, 0.0);
      }
    } else {
      if (lane < nout) {
        P.partials[ch.part + lane] = make_double2(s_re + k_re, s_im + k_im);
        if (I.mag_off) P.partials[ch.part + I.mag_off + lane] = make_double2(mag, 0.0);
      }
    }
    __syncwarp();
  }
}

// sum (s1 + c1) + (s2 + c2) keeping the rounding error of the leading add
__device__ __forceinline__ void two_sum_merge(double& s, double& c, double s2, double c2) {
  const double t = s + s2;
  const double bb = t - s;
  const double e = (s - (t - bb)) + (s2 - bb);
  s = t;
  c = c + c2 + e;
}

// One warp per output: lane l Neumaier-sums the chunk partials l, l+32, ... in order, then the
// lanes merge in a fixed butterfly (bitwise reproducible), and the final scale (0.5^(N/2-1)
// etc., and the undoing of any input prescaling) is applied.  Thread 0 re-arms the work
// counters for the next execution.
static __global__ void reduce_kernel(const InstDev* __restrict__ inst, int ninst, const double2* __restrict__ partials,
                              const double* __restrict__ scales, double2* __restrict__ out, unsigned int* counters,
                              int ncounters, int total_out, unsigned int modp, double* __restrict__ mags = nullptr) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw < total_out) {
    // locate the instance (outputs are laid out instance by instance)
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (inst[mid].out_base <= gw) lo = mid; else hi = mid - 1;
    }
    const InstDev& I = inst[lo];
    const int o = gw - I.out_base;
    double sr = 0, si = 0, cr = 0, ci = 0, ms = 0;
    const int ps = I.pstride > I.nout ? I.pstride : I.nout;  // slots per chunk
    for (int c = lane; c < I.nchunks; c += 32) {
      const double2 v = partials[I.part_base + c * ps + o];
      neumaier(sr, cr, v.x);
      neumaier(si, ci, v.y);
      if (I.comp_off) {  // double-double kinds: the chunk's compensation
        const double2 w = partials[I.part_base + c * ps + I.comp_off + o];
        cr += w.x;
        ci += w.y;
      }
      if (I.mag_off) ms += partials[I.part_base + c * ps + I.mag_off + o].x;
    }
#pragma unroll
    for (int off = 16; off; off >>= 1) ms += __shfl_xor_sync(0xffffffffu, ms, off);
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const double osr = __shfl_xor_sync(0xffffffffu, sr, off), ocr = __shfl_xor_sync(0xffffffffu, cr, off);
      const double osi = __shfl_xor_sync(0xffffffffu, si, off), oci = __shfl_xor_sync(0xffffffffu, ci, off);
      if (lane & off) {  // the upper lane adds into the lower lane's sum: same order on both sides
        double a = osr, b = ocr;
        two_sum_merge(a, b, sr, cr);
        sr = a; cr = b;
        a = osi; b = oci;
        two_sum_merge(a, b, si, ci);
        si = a; ci = b;
      } else {
        two_sum_merge(sr, cr, osr, ocr);
        two_sum_merge(si, ci, osi, oci);
      }
    }
    if (lane == 0) {
      const double sc = scales[I.scale_base + o];
      if (modp) {  // residues (< 2^31) summed exactly in FP64 (fewer than 2^22 chunks), then mod p
        const unsigned long long r = (unsigned long long)(sr + cr) % modp;
        out[gw] = make_double2((double)(r * (unsigned long long)sc % modp), 0.0);
      } else {
        out[gw] = make_double2((sr + cr) * sc, (si + ci) * sc);
      }
      if (mags) mags[gw] = I.mag_off ? ms * fabs(sc) : 0.0;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0)
    for (int i = 0; i < ncounters; ++i) counters[i] = 0u;
}

}  // namespace wg
