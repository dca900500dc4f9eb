// Reference-equivalent op count of the spin-orbital tiled (T), restricted and unrestricted
// (is_restricted selects the two spin filters below, as fused_common.hpp:34-130 passes it on).
//
// Restates, as host arithmetic, how ExaChem counts the work of its fused (T):
//   task list          ccsd_t_fused_driver.hpp:573-602 (p4<=p5<=p6, h1<=h2<=h3, spin sums
//                      equal, restricted: total spin <= 8)
//   restricted filter  singles.hpp:100-119 and the d1 / d2 counterparts: no variant with all six
//                      tiles beta (spin sum 12)
//   enabled equations  ccsd_t_all_fused_singles.hpp:394-553   (s1, ordering p5<=p6, h2<=h3,
//                      pair rule spin p4 == spin h1)
//                      ccsd_t_all_fused_doubles1.hpp:309-488  (d1, p4<=p5, h2<=h3, per h7
//                      tile spin p4 + spin p5 == spin h1 + spin h7)
//                      ccsd_t_all_fused_doubles2.hpp:362-544  (d2, p5<=p6, h1<=h2, per p7
//                      tile spin p4 + spin p7 == spin h1 + spin h2)
//   ops per equation   fused_common.hpp:131-261 (2 x product of the block sizes; d1/d2 also
//                      times the contracted tile)
// Duplicate permutation tuples are removed first (singles.hpp:66-72) and a surviving tuple
// contributes once per slot it matches (singles.hpp:127-177).
#include <array>
#include <cstddef>
#include <vector>

#include "../../include/ccsdt.h"

namespace {

using Tup = std::array<int, 6>; // (p4, p5, p6, h1, h2, h3)

struct Space {
  std::vector<long> range;
  std::vector<int>  spin;
  int               noab, nvab;
  bool              restricted; // is_restricted: drop the all-beta variants (spin sum 12)
};

void dedup(std::array<Tup, 9>& a) {
  for(int i = 0; i < 8; i++)
    if(a[i][0] != 0)
      for(int j = i + 1; j < 9; j++)
        if(a[i] == a[j]) a[j] = Tup{0, 0, 0, 0, 0, 0};
}

long double s1_ops(const Space& S, int h1, int h2, int h3, int p4, int p5, int p6) {
  std::array<Tup, 9> a = {Tup{p4, p5, p6, h1, h2, h3}, Tup{p4, p5, p6, h2, h1, h3},
                          Tup{p4, p5, p6, h3, h1, h2}, Tup{p5, p4, p6, h1, h2, h3},
                          Tup{p5, p4, p6, h2, h1, h3}, Tup{p5, p4, p6, h3, h1, h2},
                          Tup{p6, p4, p5, h1, h2, h3}, Tup{p6, p4, p5, h2, h1, h3},
                          Tup{p6, p4, p5, h3, h1, h2}};
  dedup(a);
  const Tup ref = {p4, p5, p6, h1, h2, h3};
  int       n   = 0;
  for(const Tup& t: a) {
    const int P4 = t[0], P5 = t[1], P6 = t[2], H1 = t[3], H2 = t[4], H3 = t[5];
    if(!(P5 <= P6 && H2 <= H3 && P4 != 0)) continue;
    const int s[6] = {S.spin[P4], S.spin[P5], S.spin[P6], S.spin[H1], S.spin[H2], S.spin[H3]};
    if(S.restricted && s[0] + s[1] + s[2] + s[3] + s[4] + s[5] == 12) continue;
    if(s[0] + s[1] + s[2] != s[3] + s[4] + s[5]) continue;
    if(s[0] != s[3]) continue;
    const Tup cands[9] = {{P4, P5, P6, H1, H2, H3}, {P4, P5, P6, H2, H1, H3}, {P4, P5, P6, H2, H3, H1},
                          {P5, P4, P6, H1, H2, H3}, {P5, P4, P6, H2, H1, H3}, {P5, P4, P6, H2, H3, H1},
                          {P5, P6, P4, H1, H2, H3}, {P5, P6, P4, H2, H1, H3}, {P5, P6, P4, H2, H3, H1}};
    for(const Tup& c: cands) n += (c == ref);
  }
  long double base = 2.0L * S.range[h1] * S.range[h2] * S.range[h3] * S.range[p4] * S.range[p5] *
                     S.range[p6];
  return n * base;
}

long double d_ops(const Space& S, int kind, int h1, int h2, int h3, int p4, int p5, int p6) {
  std::array<Tup, 9> a;
  if(kind == 1)
    a = {Tup{p4, p5, p6, h1, h2, h3}, Tup{p4, p5, p6, h2, h1, h3}, Tup{p4, p5, p6, h3, h1, h2},
         Tup{p5, p6, p4, h1, h2, h3}, Tup{p5, p6, p4, h2, h1, h3}, Tup{p5, p6, p4, h3, h1, h2},
         Tup{p4, p6, p5, h1, h2, h3}, Tup{p4, p6, p5, h2, h1, h3}, Tup{p4, p6, p5, h3, h1, h2}};
  else
    a = {Tup{p4, p5, p6, h1, h2, h3}, Tup{p4, p5, p6, h2, h3, h1}, Tup{p4, p5, p6, h1, h3, h2},
         Tup{p5, p4, p6, h1, h2, h3}, Tup{p5, p4, p6, h2, h3, h1}, Tup{p5, p4, p6, h1, h3, h2},
         Tup{p6, p4, p5, h1, h2, h3}, Tup{p6, p4, p5, h2, h3, h1}, Tup{p6, p4, p5, h1, h3, h2}};
  dedup(a);
  const Tup   ref  = {p4, p5, p6, h1, h2, h3};
  long double base = 2.0L * S.range[h1] * S.range[h2] * S.range[h3] * S.range[p4] * S.range[p5] *
                     S.range[p6];
  long double ops = 0;
  for(const Tup& t: a) {
    const int P4 = t[0], P5 = t[1], P6 = t[2], H1 = t[3], H2 = t[4], H3 = t[5];
    if(kind == 1 && !(P4 <= P5 && H2 <= H3 && P4 != 0)) continue;
    if(kind == 2 && !(P5 <= P6 && H1 <= H2 && P4 != 0)) continue;
    const int s[6] = {S.spin[P4], S.spin[P5], S.spin[P6], S.spin[H1], S.spin[H2], S.spin[H3]};
    if(S.restricted && s[0] + s[1] + s[2] + s[3] + s[4] + s[5] == 12) continue;
    if(s[0] + s[1] + s[2] != s[3] + s[4] + s[5]) continue;
    int m = 0;
    if(kind == 1) {
      const Tup cands[9] = {{P4, P5, P6, H1, H2, H3}, {P4, P5, P6, H2, H1, H3}, {P4, P5, P6, H2, H3, H1},
                            {P6, P4, P5, H1, H2, H3}, {P6, P4, P5, H2, H1, H3}, {P6, P4, P5, H2, H3, H1},
                            {P4, P6, P5, H1, H2, H3}, {P4, P6, P5, H2, H1, H3}, {P4, P6, P5, H2, H3, H1}};
      for(const Tup& c: cands) m += (c == ref);
      if(!m) continue;
      for(int x = 0; x < S.noab; x++) {
        if(S.spin[P4] + S.spin[P5] != S.spin[H1] + S.spin[x]) continue;
        ops += m * base * S.range[x];
      }
    }
    else {
      const Tup cands[9] = {{P4, P5, P6, H1, H2, H3}, {P4, P5, P6, H3, H1, H2}, {P4, P5, P6, H1, H3, H2},
                            {P5, P4, P6, H1, H2, H3}, {P5, P4, P6, H3, H1, H2}, {P5, P4, P6, H1, H3, H2},
                            {P5, P6, P4, H1, H2, H3}, {P5, P6, P4, H3, H1, H2}, {P5, P6, P4, H1, H3, H2}};
      for(const Tup& c: cands) m += (c == ref);
      if(!m) continue;
      for(int x = S.noab; x < S.noab + S.nvab; x++) {
        if(S.spin[P4] + S.spin[x] != S.spin[H1] + S.spin[H2]) continue;
        ops += m * base * S.range[x];
      }
    }
  }
  return ops;
}

// Sum over the task list of ccsd_t_fused_driver.hpp:573-602 (restricted: total spin <= 8).
void count_tasks(const Space& S, double* ops_out, long* tasks_out) {
  long double total = 0;
  long        ntask = 0;
  const int   no = S.noab, nv = S.nvab;
  for(int p4 = no; p4 < no + nv; p4++)
    for(int p5 = p4; p5 < no + nv; p5++)
      for(int p6 = p5; p6 < no + nv; p6++)
        for(int h1 = 0; h1 < no; h1++)
          for(int h2 = h1; h2 < no; h2++)
            for(int h3 = h2; h3 < no; h3++) {
              int sp = S.spin[p4] + S.spin[p5] + S.spin[p6];
              int sh = S.spin[h1] + S.spin[h2] + S.spin[h3];
              if(sp != sh || (S.restricted && sp + sh > 8)) continue;
              ntask++;
              total += s1_ops(S, h1, h2, h3, p4, p5, p6) + d_ops(S, 1, h1, h2, h3, p4, p5, p6) +
                       d_ops(S, 2, h1, h2, h3, p4, p5, p6);
            }
  *ops_out = (double) total;
  if(tasks_out) *tasks_out = ntask;
}

// MO tiles occ_a | occ_b | virt_a | virt_b with spins 1 (alpha) / 2 (beta), as k_spin holds them.
bool build_space(Space& S, const int* const (&t)[4], const int (&n)[4], bool restricted) {
  for(int r = 0; r < 4; r++)
    for(int x = 0; x < n[r]; x++) {
      if(t[r][x] <= 0) return false;
      S.range.push_back(t[r][x]);
      S.spin.push_back(r % 2 + 1);
    }
  S.noab       = n[0] + n[1];
  S.nvab       = n[2] + n[3];
  S.restricted = restricted;
  return true;
}

} // namespace

extern "C" ccsdt_status ccsdt_reference_op_count(const ccsdt_layout* L, double* ops_out,
                                                 long* tasks_out) {
  if(!L || !ops_out || L->n_occ_tiles <= 0 || L->n_vir_tiles <= 0 || !L->occ_tiles || !L->vir_tiles)
    return CCSDT_E_INVALID;
  long so = 0, sv = 0;
  for(int t = 0; t < L->n_occ_tiles; t++) so += L->occ_tiles[t];
  for(int t = 0; t < L->n_vir_tiles; t++) sv += L->vir_tiles[t];
  Space           S;
  const int* const tl[4] = {L->occ_tiles, L->occ_tiles, L->vir_tiles, L->vir_tiles};
  const int        nt[4] = {L->n_occ_tiles, L->n_occ_tiles, L->n_vir_tiles, L->n_vir_tiles};
  if(!build_space(S, tl, nt, true) || so != L->o || sv != L->v) return CCSDT_E_BAD_LAYOUT;
  count_tasks(S, ops_out, tasks_out);
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_reference_op_count_so(int n_occ_a, const int* occ_a, int n_occ_b, const int* occ_b,
                                                    int n_vir_a, const int* vir_a, int n_vir_b, const int* vir_b,
                                                    int is_restricted, double* ops_out, long* tasks_out) {
  if(!ops_out || n_occ_a < 0 || n_occ_b < 0 || n_vir_a < 0 || n_vir_b < 0 || n_occ_a + n_occ_b <= 0 ||
     n_vir_a + n_vir_b <= 0 || (n_occ_a && !occ_a) || (n_occ_b && !occ_b) || (n_vir_a && !vir_a) ||
     (n_vir_b && !vir_b))
    return CCSDT_E_INVALID;
  Space            S;
  const int* const tl[4] = {occ_a, occ_b, vir_a, vir_b};
  const int        nt[4] = {n_occ_a, n_occ_b, n_vir_a, n_vir_b};
  if(!build_space(S, tl, nt, is_restricted != 0)) return CCSDT_E_BAD_LAYOUT;
  count_tasks(S, ops_out, tasks_out);
  return CCSDT_OK;
}
