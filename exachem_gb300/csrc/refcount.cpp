// Reference-equivalent op count of the spin-orbital tiled (T) (restricted case).
//
// Restates, as host arithmetic, how ExaChem counts the work of its fused (T):
//   task list          ccsd_t_fused_driver.hpp:573-602 (p4<=p5<=p6, h1<=h2<=h3, spin sums
//                      equal, restricted: total spin <= 8)
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
    if(s[0] + s[1] + s[2] + s[3] + s[4] + s[5] == 12) continue;
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
    if(s[0] + s[1] + s[2] + s[3] + s[4] + s[5] == 12) continue;
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

} // namespace

extern "C" ccsdt_status ccsdt_reference_op_count(const ccsdt_layout* L, double* ops_out,
                                                 long* tasks_out) {
  if(!L || !ops_out || L->n_occ_tiles <= 0 || L->n_vir_tiles <= 0 || !L->occ_tiles || !L->vir_tiles)
    return CCSDT_E_INVALID;
  Space S;
  long  so = 0, sv = 0;
  for(int s = 0; s < 2; s++)
    for(int t = 0; t < L->n_occ_tiles; t++) {
      if(L->occ_tiles[t] <= 0) return CCSDT_E_BAD_LAYOUT;
      S.range.push_back(L->occ_tiles[t]);
      S.spin.push_back(s + 1);
      if(s == 0) so += L->occ_tiles[t];
    }
  for(int s = 0; s < 2; s++)
    for(int t = 0; t < L->n_vir_tiles; t++) {
      if(L->vir_tiles[t] <= 0) return CCSDT_E_BAD_LAYOUT;
      S.range.push_back(L->vir_tiles[t]);
      S.spin.push_back(s + 1);
      if(s == 0) sv += L->vir_tiles[t];
    }
  if(so != L->o || sv != L->v) return CCSDT_E_BAD_LAYOUT;
  S.noab = 2 * L->n_occ_tiles;
  S.nvab = 2 * L->n_vir_tiles;
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
              if(sp != sh || sp + sh > 8) continue;
              ntask++;
              total += s1_ops(S, h1, h2, h3, p4, p5, p6) + d_ops(S, 1, h1, h2, h3, p4, p5, p6) +
                       d_ops(S, 2, h1, h2, h3, p4, p5, p6);
            }
  *ops_out = (double) total;
  if(tasks_out) *tasks_out = ntask;
  return CCSDT_OK;
}
