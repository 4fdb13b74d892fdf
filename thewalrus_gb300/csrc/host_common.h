// Host-side helpers shared by the translation units that launch the sieve kernels:
// scalar classes, the tile size limit, per-warp shared-memory layout and the La Budde lane
// schedules.
#pragma once
#include <algorithm>
#include <utility>
#include <vector>

#include "kernels.h"
#include "sieve_kernel.cuh"

namespace wg {

// kernel launch and occupancy by scalar class (the kernels live in kernels_*.cu)
static inline cudaError_t sieve_launch(int stype, const SieveParams& p, int ctas, int wpc, cudaStream_t st);
static inline int sieve_occupancy(int stype, int wpc, int smem);
static inline cudaError_t sieve_tables_all(const double* binom, const double* inv);

// scalar classes
enum SType { ST_REAL64 = 0, ST_CPLX64 = 1, ST_REALDF = 2, ST_CPLXDF = 3, ST_MOD0 = 4, ST_MOD1 = 5, ST_MOD2 = 6,
             ST_MOD3 = 7, ST_MOD4 = 8, ST_REALDD = 9, ST_CPLXDD = 10 };
static inline bool stype_mod(int st) { return st >= ST_MOD0 && st <= ST_MOD4; }
static inline bool stype_dd(int st) { return st == ST_REALDD || st == ST_CPLXDD; }
static size_t stype_bytes(int st) {
  if (stype_mod(st)) return 4;
  if (stype_dd(st)) return st == ST_REALDD ? 16 : 32;
  return (st == ST_REAL64 || st == ST_REALDF) ? 8 : 16;
}
static const uint32_t MOD_PRIMES[5] = {2147483647u, 2147483629u, 2147483587u, 2147483579u, 2147483563u};

// the largest term tile a warp works on: 80 rows of complex scalars, 96 of real ones (the packed
// pivot keys hold row indices below 128)
static inline bool tile_rows_ok(int stype, int rows) {
  return rows <= ((stype == ST_CPLX64 || stype == ST_CPLXDF) ? 80 : 96);
}

static inline cudaError_t sieve_launch(int stype, const SieveParams& p, int ctas, int wpc, cudaStream_t st) {
  switch (stype) {
    case ST_CPLX64: return sieve_launch_c64(p, ctas, wpc, st);
    case ST_CPLXDF: return sieve_launch_cdf(p, ctas, wpc, st);
    case ST_REAL64: return sieve_launch_f64(p, ctas, wpc, st);
    case ST_REALDF: return sieve_launch_fdf(p, ctas, wpc, st);
    case ST_MOD0: return sieve_launch_mod0(p, ctas, wpc, st);
    case ST_MOD1: return sieve_launch_mod1(p, ctas, wpc, st);
    case ST_MOD2: return sieve_launch_mod2(p, ctas, wpc, st);
    case ST_MOD3: return sieve_launch_mod3(p, ctas, wpc, st);
    case ST_REALDD: return sieve_launch_fdd(p, ctas, wpc, st);
    case ST_CPLXDD: return sieve_launch_cdd(p, ctas, wpc, st);
    default: return sieve_launch_mod4(p, ctas, wpc, st);
  }
}

static inline int sieve_occupancy(int stype, int wpc, int smem) {
  switch (stype) {
    case ST_CPLX64: return sieve_occupancy_c64(wpc, smem);
    case ST_CPLXDF: return sieve_occupancy_cdf(wpc, smem);
    case ST_REAL64: return sieve_occupancy_f64(wpc, smem);
    case ST_REALDF: return sieve_occupancy_fdf(wpc, smem);
    case ST_MOD0: return sieve_occupancy_mod0(wpc, smem);
    case ST_MOD1: return sieve_occupancy_mod1(wpc, smem);
    case ST_MOD2: return sieve_occupancy_mod2(wpc, smem);
    case ST_MOD3: return sieve_occupancy_mod3(wpc, smem);
    case ST_REALDD: return sieve_occupancy_fdd(wpc, smem);
    case ST_CPLXDD: return sieve_occupancy_cdd(wpc, smem);
    default: return sieve_occupancy_mod4(wpc, smem);
  }
}

static inline cudaError_t sieve_tables_all(const double* binom, const double* inv) {
  cudaError_t e = sieve_tables_c64(binom, inv);
  if (e == cudaSuccess) e = sieve_tables_cdf(binom, inv);
  if (e == cudaSuccess) e = sieve_tables_f64(binom, inv);
  if (e == cudaSuccess) e = sieve_tables_fdf(binom, inv);
  if (e == cudaSuccess) e = sieve_tables_mod0(binom, inv);
  if (e == cudaSuccess) e = sieve_tables_mod1(binom, inv);
  if (e == cudaSuccess) e = sieve_tables_mod2(binom, inv);
  if (e == cudaSuccess) e = sieve_tables_mod3(binom, inv);
  if (e == cudaSuccess) e = sieve_tables_mod4(binom, inv);
  if (e == cudaSuccess) e = sieve_tables_fdd(binom, inv);
  if (e == cudaSuccess) e = sieve_tables_cdd(binom, inv);
  return e;
}

// Default cap on warps per CTA.  Below 8 the shape search below takes two CTAs of 4 warps where
// one CTA of 8 would fit (the same 8 warps per SM), and that measured faster: complex FP64
// n = 40 247.9 ms against 249.7 ms, n = 36 49.07 against 49.79 ms, double-float n = 40 135.6
// against 136.6 ms; a cap of 6 gives the same as 7, and n = 32, 42 and the real kernels (several
// CTAs per SM already) are unchanged.
constexpr int kDefaultWarpsPerCta = 7;

// Launch shape for a per-warp workspace of `bytes`: warps per CTA (at most wpc_cap) for the most
// resident warps per SM -- shared memory and registers decide how many CTAs fit -- larger CTAs
// on ties, e.g. 2 CTAs x 7 warps where 1 x 8 would leave room unused.  Returns {wpc, CTAs per
// SM}; wpc 0 when not even one warp fits.
static inline std::pair<int, int> best_shape(int stype, int bytes, int wpc_cap) {
  const int max_smem = 227 * 1024;
  const int wmax = std::min(wpc_cap, max_smem / bytes);
  if (wmax < 1) return {0, 0};
  int wpc = wmax, per_sm = sieve_occupancy(stype, wmax, wmax * bytes);
  for (int w = wmax - 1; w >= std::max(1, wmax / 2); --w) {
    const int ps = sieve_occupancy(stype, w, w * bytes);
    if (ps * w > per_sm * wpc) { wpc = w; per_sm = ps; }
  }
  return {wpc, per_sm};
}

// tilewin: La Budde's coefficient rows live in dead tile columns (only rows 0..2 need `win`)
static inline WarpLayout make_layout(int stype, int rows, int mb, int kc, int nser, int narr, bool tilewin) {
  WarpLayout L;
  const int sb = (int)stype_bytes(stype);
  // FP64 and modular scalars run the normalised elimination (unit subdiagonal), so La Budde reads
  // its T_r = H(i-r, i) straight from the tile; double-float keeps the beta products in tb
  const bool normalised = stype != ST_REALDF && stype != ST_CPLXDF;
  auto al = [](int x) { return (x + 15) & ~15; };
  L.ldw = std::max(mb, 1) | 1;
  L.rows = std::max(rows, 1);
  L.kw = kc + 1;
  L.nser = (nser + 1) & ~1;
  int off = al(L.rows * L.ldw * sb);
  L.off_x = off;
  off += al(L.ldw * sb);
  L.off_win = off;
  L.tilewin = tilewin ? 1 : 0;
  // tile mode: La Budde rows 0..2 only (row i' has entries 0..i'), stride 3; otherwise a
  // circular window of kw rows of kw entries
  off += al((tilewin ? 9 : L.kw * L.kw) * sb);
  // double-float T_r of two rows (entries r = 1..kw-2 of rows 0 and 1): in the x row, dead during
  // La Budde, when it is long enough
  L.off_tb = off;
  if (!normalised) {
    if (2 * L.kw - 1 <= L.ldw) L.off_tb = L.off_x;
    else off += al(2 * L.kw * sb);
  }
  // La Budde piece partials (3 per lane) are dead outside La Budde; with the two series arrays of
  // the plain kinds (written after La Budde) they share one region
  const int part_bytes = al(96 * sb), ser_bytes = al(narr * L.nser * sb);
  if (narr <= 2) {
    L.off_part = off;
    L.off_ser = off;
    off += std::max(part_bytes, ser_bytes);
  } else {
    L.off_part = off;
    off += part_bytes;
    L.off_ser = off;
    off += ser_bytes;
  }
  L.off_int = off;
  off += al((L.rows + 2 * L.ldw) * 2);  // 16-bit row, column and delta maps
  L.bytes = al(off);
  return L;
}

// Balanced La Budde schedule for triangle size Ki: coefficient j (2..Ki) needs j-1 products.
// Find the smallest per-lane load t for which the pieces (each j's products cut into
// ceil((j-1)/t) near-equal runs) pack into 32 lanes with at most two pieces per lane
// (largest piece first, onto the least-loaded lane that fits).
static inline bool lb_schedule(int Ki, LbLane* lanes, LbOwner* own) {
  for (int l = 0; l < 32; ++l) lanes[l] = LbLane{0, 0, 0, 0, 0, 0, 0, 0};
  for (int j = 0; j <= LB_KMAX; ++j) own[j] = LbOwner{0, {0, 0, 0, 0, 0, 0, 0}};
  const int W = Ki * (Ki - 1) / 2;
  if (W == 0) return true;
  struct Piece { int j, rlo, len; };
  for (int t = std::max(1, (W + 31) / 32); t <= 64; ++t) {
    // at most 64 pieces fit (two per lane); fixed storage, no heap allocation
    int npcs = 0;
    for (int j = 2; j <= Ki; ++j) npcs += (j - 1 + t - 1) / t;
    if (npcs > 64) continue;
    Piece pcs[64];
    npcs = 0;
    for (int j = 2; j <= Ki; ++j) {
      const int x = j - 1, p = (x + t - 1) / t;
      int r = 1;
      for (int q = 0; q < p; ++q) {
        const int len = x / p + (q < x % p ? 1 : 0);
        pcs[npcs++] = {j, r, len};
        r += len;
      }
    }
    // stable insertion sort, longest piece first
    for (int a = 1; a < npcs; ++a) {
      const Piece key = pcs[a];
      int b = a - 1;
      while (b >= 0 && pcs[b].len < key.len) { pcs[b + 1] = pcs[b]; --b; }
      pcs[b + 1] = key;
    }
    int load[32] = {0}, nseg[32] = {0};
    Piece seg[32][2];
    bool ok = true;
    for (int q = 0; q < npcs; ++q) {
      const Piece& pc = pcs[q];
      int best = -1;
      for (int l = 0; l < 32; ++l)
        if (nseg[l] < 2 && load[l] + pc.len <= t && (best < 0 || load[l] < load[best])) best = l;
      if (best < 0) { ok = false; break; }
      seg[best][nseg[best]++] = pc;
      load[best] += pc.len;
    }
    if (!ok) continue;
    bool fits = true;
    for (int l = 0; l < 32 && fits; ++l) {
      LbLane& L = lanes[l];
      if (nseg[l] > 0) { L.ja = (signed char)seg[l][0].j; L.rloa = (signed char)seg[l][0].rlo; L.lena = (signed char)seg[l][0].len; }
      if (nseg[l] > 1) { L.jb = (signed char)seg[l][1].j; L.rlob = (signed char)seg[l][1].rlo; L.lenb = (signed char)seg[l][1].len; }
      for (int k = 0; k < nseg[l]; ++k) {
        LbOwner& o = own[seg[l][k].j];
        if (o.n >= 7) { fits = false; break; }
        o.s[o.n++] = (unsigned char)(2 * l + k);
      }
    }
    if (fits) return true;
    for (int j = 0; j <= LB_KMAX; ++j) own[j] = LbOwner{0, {0, 0, 0, 0, 0, 0, 0}};
    for (int l = 0; l < 32; ++l) lanes[l] = LbLane{0, 0, 0, 0, 0, 0, 0, 0};
  }
  return false;
}

// One packing of the two-row r-sums at per-lane load t.  split_once = false: the sums longest
// first, poured into the lanes in order, a sum split where a lane fills.  split_once = true:
// each sum of t or more products gives whole lanes of t, and its remainder joins the shorter
// sums, packed first-fit longest first -- every coefficient then has at most two pieces.  At most
// three pieces per lane and seven per coefficient; false when that does not fit in 32 lanes.
static inline bool lb2_pack(int K0, int K1, int t, bool split_once, LbLane2* lanes, LbOwner2* own) {
  for (int l = 0; l < 32; ++l) lanes[l] = LbLane2{{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, 0, {0, 0}};
  for (int j = 0; j <= LB2_KMAX; ++j) own[j] = LbOwner2{0, 0, {0}, {0}};
  struct Sum { int row, j, len; };
  Sum sums[2 * (LB2_KMAX + 1)];
  int ns = 0;
  for (int row = 0; row < 2; ++row)
    for (int j = 2; j <= (row ? K1 : K0); ++j) sums[ns++] = {row, j, j - 1};
  for (int x = 1; x < ns; ++x) {  // stable insertion sort, longest first
    const Sum key = sums[x];
    int y = x - 1;
    while (y >= 0 && sums[y].len < key.len) { sums[y + 1] = sums[y]; --y; }
    sums[y + 1] = key;
  }
  int load[32] = {0}, npc[32] = {0};
  // piece (row, j, r .. r+len-1) into lane l
  auto put = [&](int l, const Sum& sm, int r, int len) -> bool {
    if (l >= 32 || npc[l] >= 3 || load[l] + len > t) return false;
    LbLane2& L = lanes[l];
    const int q = npc[l]++;
    L.j[q] = (signed char)sm.j;
    L.rlo[q] = (signed char)r;
    L.len[q] = (signed char)len;
    if (sm.row) L.rowmask |= (unsigned char)(1u << q);
    load[l] += len;
    LbOwner2& o = own[sm.j];
    unsigned char& n = sm.row ? o.n1 : o.n0;
    unsigned char* sl = sm.row ? o.s1 : o.s0;
    if (n >= 7) return false;
    sl[n++] = (unsigned char)(3 * l + q);
    return true;
  };
  if (!split_once) {
    int lane = 0;
    for (int q = 0; q < ns; ++q) {
      int r = 1, left = sums[q].len;
      while (left > 0) {
        if (lane < 32 && (load[lane] == t || npc[lane] == 3)) ++lane;
        if (lane >= 32) return false;
        const int take = std::min(left, t - load[lane]);
        if (!put(lane, sums[q], r, take)) return false;
        r += take;
        left -= take;
      }
    }
    return true;
  }
  int next = 0;  // first lane never used
  Sum rest[2 * (LB2_KMAX + 1)];
  int rlo[2 * (LB2_KMAX + 1)];
  int nr = 0;
  for (int q = 0; q < ns; ++q) {
    int r = 1, left = sums[q].len;
    while (left >= t) {
      if (!put(next++, sums[q], r, t)) return false;
      r += t;
      left -= t;
    }
    if (left > 0) { rest[nr] = {sums[q].row, sums[q].j, left}; rlo[nr++] = r; }
  }
  for (int x = 1; x < nr; ++x) {  // remainders and short sums, stable longest first
    const Sum key = rest[x];
    const int kr = rlo[x];
    int y = x - 1;
    while (y >= 0 && rest[y].len < key.len) { rest[y + 1] = rest[y]; rlo[y + 1] = rlo[y]; --y; }
    rest[y + 1] = key;
    rlo[y + 1] = kr;
  }
  for (int x = 0; x < nr; ++x) {
    int l = 0;
    while (l < 32 && !(npc[l] < 3 && load[l] + rest[x].len <= t)) ++l;
    if (l >= 32 || !put(l, rest[x], rlo[x], rest[x].len)) return false;
  }
  return true;
}

// Two-row schedule (rows i and i+1 of La Budde with K0 and K1 coefficients): of both packings
// at every per-lane load t from the smallest possible up, the one with the least kernel cost --
// 4 x the largest lane load (product iterations of four FP64 instructions, complex) plus 2 x the
// most pieces of any coefficient of each row (the owner pass's subtractions).
static inline bool lb_schedule2(int K0, int K1, LbLane2* lanes, LbOwner2* own) {
  for (int l = 0; l < 32; ++l) lanes[l] = LbLane2{{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, 0, {0, 0}};
  for (int j = 0; j <= LB2_KMAX; ++j) own[j] = LbOwner2{0, 0, {0}, {0}};
  if (K0 < 0 || K1 < K0 || K1 > LB2_KMAX) return false;
  const int W = K0 * (K0 - 1) / 2 + K1 * (K1 - 1) / 2;
  if (W == 0) return true;
  LbLane2 tl[32];
  LbOwner2 to[LB2_KMAX + 1];
  int best = -1;
  const int t0 = std::max(1, (W + 31) / 32);
  for (int t = t0; t <= 64; ++t) {
    for (int mode = 0; mode < 2; ++mode) {
      if (!lb2_pack(K0, K1, t, mode == 1, tl, to)) continue;
      int mx = 0, m0 = 0, m1 = 0;
      for (int l = 0; l < 32; ++l) mx = std::max(mx, tl[l].len[0] + tl[l].len[1] + tl[l].len[2]);
      for (int j = 0; j <= K1; ++j) { m0 = std::max(m0, (int)to[j].n0); m1 = std::max(m1, (int)to[j].n1); }
      const int cost = 4 * mx + 2 * (m0 + m1);
      if (best < 0 || cost < best) {
        best = cost;
        std::copy(tl, tl + 32, lanes);
        std::copy(to, to + LB2_KMAX + 1, own);
      }
    }
    if (best >= 0 && 4 * t >= best) break;  // loads near t cost 4t or more: stop the search
  }
  return best >= 0;
}

// every two-row table: lanes[LB2_IDS * 32], own[LB2_IDS * (LB2_KMAX + 1)], entry lb2_id(K0, K1)
static inline bool lb_schedule2_all(LbLane2* lanes, LbOwner2* own) {
  for (int K1 = 0; K1 <= LB2_KMAX; ++K1)
    for (int d = 0; d <= 1; ++d) {
      const int K0 = K1 - d, id = lb2_id(K0 < 0 ? 0 : K0, K1) + (K0 < 0 ? 1 : 0);
      if (K0 < 0) {  // unused entry (K1 = 0, K0 = -1): empty schedule
        lb_schedule2(0, 0, &lanes[id * 32], &own[id * (LB2_KMAX + 1)]);
        continue;
      }
      if (!lb_schedule2(K0, K1, &lanes[id * 32], &own[id * (LB2_KMAX + 1)])) return false;
    }
  return true;
}

}  // namespace wg
