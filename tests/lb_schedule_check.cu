// Host-only check of the La Budde lane schedules that the sieve kernel's La Budde step follows
// (host_common.h: lb_schedule for one row, lb_schedule2 for two rows): every product
// T_r c[i-r-1][j-r-1] of every coefficient j is computed by exactly one lane piece, each owner
// list names exactly the slots of its coefficient's pieces, and a lane's pieces come in slot
// order (the kernel advances through them in that order).  Built and run by
// tests/test_lb_schedules.py; prints "ok" and exits 0, or names the first violation.
#include <cstdio>
#include <set>
#include <vector>

#include "../thewalrus_gb300/csrc/host_common.h"

using namespace wg;

static int fail(const char* what, int a, int b, int c) {
  std::printf("FAIL %s (%d, %d, %d)\n", what, a, b, c);
  return 1;
}

static int check_single(int K) {
  static LbLane lanes[32];
  static LbOwner own[LB_KMAX + 1];
  if (!lb_schedule(K, lanes, own)) return fail("no single-row schedule", K, 0, 0);
  std::vector<int> seen((K + 1) * (K + 1), 0);
  std::vector<std::set<int>> slots(K + 1);
  for (int l = 0; l < 32; ++l) {
    const int js[2] = {lanes[l].ja, lanes[l].jb}, rs[2] = {lanes[l].rloa, lanes[l].rlob},
              ls[2] = {lanes[l].lena, lanes[l].lenb};
    if (ls[1] > 0 && ls[0] == 0) return fail("second piece without a first", K, l, 0);
    for (int k = 0; k < 2; ++k) {
      if (ls[k] == 0) continue;
      if (js[k] < 2 || js[k] > K) return fail("piece coefficient out of range", K, l, js[k]);
      for (int r = rs[k]; r < rs[k] + ls[k]; ++r) {
        if (r < 1 || r > js[k] - 1) return fail("piece r out of range", K, js[k], r);
        if (seen[js[k] * (K + 1) + r]++) return fail("product covered twice", K, js[k], r);
      }
      slots[js[k]].insert(2 * l + k);
    }
  }
  for (int j = 2; j <= K; ++j) {
    for (int r = 1; r < j; ++r)
      if (!seen[j * (K + 1) + r]) return fail("product not covered", K, j, r);
    std::set<int> listed(own[j].s, own[j].s + own[j].n);
    if (listed != slots[j] || (int)listed.size() != own[j].n) return fail("owner list", K, j, own[j].n);
  }
  return 0;
}

static int check_pair(int K0, int K1) {
  static LbLane2 lanes[32];
  static LbOwner2 own[LB2_KMAX + 1];
  if (!lb_schedule2(K0, K1, lanes, own)) return fail("no two-row schedule", K0, K1, 0);
  const int Kmax = K1;
  std::vector<int> seen(2 * (Kmax + 1) * (Kmax + 1), 0);
  std::vector<std::set<int>> slots0(Kmax + 1), slots1(Kmax + 1);
  for (int l = 0; l < 32; ++l) {
    const LbLane2& L = lanes[l];
    for (int q = 0; q < 3; ++q) {
      if (L.len[q] == 0) {
        for (int q2 = q + 1; q2 < 3; ++q2)
          if (L.len[q2] > 0) return fail("piece after an empty slot", K0, K1, l);
        break;
      }
      const int row = (L.rowmask >> q) & 1, j = L.j[q], Kr = row ? K1 : K0;
      if (j < 2 || j > Kr) return fail("piece coefficient out of range", K0, K1, j);
      for (int r = L.rlo[q]; r < L.rlo[q] + L.len[q]; ++r) {
        if (r < 1 || r > j - 1) return fail("piece r out of range", K0, K1, r);
        if (seen[(row * (Kmax + 1) + j) * (Kmax + 1) + r]++) return fail("product covered twice", K0, K1, j);
      }
      (row ? slots1 : slots0)[j].insert(3 * l + q);
    }
  }
  for (int row = 0; row < 2; ++row)
    for (int j = 2; j <= (row ? K1 : K0); ++j) {
      for (int r = 1; r < j; ++r)
        if (!seen[(row * (Kmax + 1) + j) * (Kmax + 1) + r]) return fail("product not covered", K0, K1, j);
      const unsigned char* s = row ? own[j].s1 : own[j].s0;
      const int n = row ? own[j].n1 : own[j].n0;
      std::set<int> listed(s, s + n);
      if (listed != (row ? slots1 : slots0)[j] || (int)listed.size() != n) return fail("owner list", K0, K1, j);
    }
  return 0;
}

int main() {
  for (int K = 0; K <= LB_KMAX; ++K)
    if (check_single(K)) return 1;
  for (int K1 = 1; K1 <= LB2_KMAX; ++K1)
    for (int K0 = K1 - 1; K0 <= K1; ++K0)
      if (check_pair(K0, K1)) return 1;
  // the tables the kernel indexes by lb2_id, built the way the plans build them
  static LbLane2 all_lanes[LB2_IDS * 32];
  static LbOwner2 all_own[LB2_IDS * (LB2_KMAX + 1)];
  if (!lb_schedule2_all(all_lanes, all_own)) return fail("lb_schedule2_all", 0, 0, 0);
  std::printf("ok\n");
  return 0;
}
