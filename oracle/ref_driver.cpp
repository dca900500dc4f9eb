// Oracle "_ref": ExaChem's own CPU (T) kernel, driven on synthetic closed-shell inputs.
//
// TEST INFRASTRUCTURE ONLY (never linked into the product library).
//
// The reference headers exachem/cc/ccsd_t/ccsd_t_all_fused_cpu.hpp (which pulls in
// fused_common.hpp and the singles / doubles1 / doubles2 gather headers) are compiled
// UNMODIFIED from the reference tree, against the TAMM/HPTT stand-in in
// oracle/ref_shim/tamm/tamm.hpp.  This file supplies what ExaChem's callers would:
//
//  * the spin-orbital tiled MO space  occ_a | occ_b | virt_a | virt_b  with tile size
//    ts and a ragged last tile per range (cholesky/cholesky_2e.cpp:230-285,
//    balance_tiles = false for triples, :185-196), or explicit tile lists;
//  * k_spin (1 = alpha, 2 = beta) and k_evl_sorted in MO order (ccsd_t.cpp:209,245-249);
//  * spin-orbital T1/T2 from closed-shell amplitudes (cc/ccsd/cd_ccsd_cs_ann.cpp:26-31,
//    :949-973) and antisymmetrised V2 blocks ijab/ijka/iabc from spatial integrals
//    (cholesky/v2tensors.cpp:67-86; Cholesky vectors carry spin {1,1}, ccsd_t.cpp:68);
//  * the task loop of CCSD_T_Fused_Driver::execute restated for one rank
//    (cc/ccsd_t/ccsd_t_fused_driver.hpp:368-483, buffer sizes :176-195, CPU buffers :238-245),
//    which calls the reference's total_fused_ccsd_t_cpu for every surviving tile block.
//
// Spatial input layouts (row-major, chemist notation for integrals):
//   eps_occ[o], eps_vir[v]
//   t1[o][v]           t1[i][a]      = t_i^a
//   t2[o][o][v][v]     t2[i][j][a][b] = t_ij^ab
//   oovv[o][o][v][v]   oovv[i][j][a][b] = (ia|jb)
//   ooov[o][o][o][v]   ooov[i][j][k][a] = (ij|ka)
//   ovvv[o][v][v][v]   ovvv[i][a][b][c] = (ia|bc)

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "tamm/tamm.hpp"
using namespace tamm;

#include "exachem/cc/ccsd_t/ccsd_t_all_fused_cpu.hpp"
#include "spin_orbital.hpp"

// accounting globals the reference headers declare extern (cc/ccsd_t/ccsd_t.hpp:8-15)
double ccsdt_s1_t1_GetTime = 0, ccsdt_s1_v2_GetTime = 0, ccsdt_d1_t2_GetTime = 0,
       ccsdt_d1_v2_GetTime = 0, ccsdt_d2_t2_GetTime = 0, ccsdt_d2_v2_GetTime = 0,
       ccsd_t_data_per_rank = 0;

namespace {

std::vector<size_t> split_range(size_t n, size_t ts) {
  std::vector<size_t> t;
  for(size_t x = 0; x < n / ts; x++) t.push_back(ts);
  if(n % ts) t.push_back(n % ts);
  return t;
}

} // namespace

// The task loop of CCSD_T_Fused_Driver::execute restated for one rank
// (cc/ccsd_t/ccsd_t_fused_driver.hpp:176-195 buffer sizes, :368-483 tasks), calling the
// reference's total_fused_ccsd_t_cpu for every surviving tile block.
static int run_tasks(std::vector<size_t>& k_range, Index noab, Index nvab, Index noa, Index nva,
                     bool tilesize_opt, std::vector<int>& k_spin, std::vector<size_t>& k_offset,
                     std::vector<double>& k_evl_sorted, Tensor<double>& d_t1, Tensor<double>& d_t2,
                     exachem::cholesky_2e::V2Tensors<double>& d_v2, bool is_restricted, double* e_bracket,
                     double* e_paren, double* ops_out, long* tasks_out) {
  // buffer sizes as in ccsd_t_fused_driver.hpp:176-195
  size_t max_pdim = 0, max_hdim = 0;
  for(size_t t = noab; t < noab + nvab; t++) max_pdim = std::max(max_pdim, k_range[t]);
  for(size_t t = 0; t < noab; t++) max_hdim = std::max(max_hdim, k_range[t]);
  size_t max_d1_kernels_pertask = tilesize_opt ? 9 * noa : 9 * noab;
  size_t max_d2_kernels_pertask = tilesize_opt ? 9 * nva : 9 * nvab;
  size_t size_T_s1_t1           = 9 * max_pdim * max_hdim;
  size_t size_T_s1_v2           = 9 * (max_pdim * max_pdim) * (max_hdim * max_hdim);
  size_t size_T_d1_t2 = max_d1_kernels_pertask * (max_pdim * max_pdim) * (max_hdim * max_hdim);
  size_t size_T_d1_v2 = max_d1_kernels_pertask * max_pdim * (max_hdim * max_hdim * max_hdim);
  size_t size_T_d2_t2 = max_d2_kernels_pertask * (max_pdim * max_pdim) * (max_hdim * max_hdim);
  size_t size_T_d2_v2 = max_d2_kernels_pertask * (max_pdim * max_pdim * max_pdim) * max_hdim;

  std::vector<double> s1_t1(size_T_s1_t1), s1_v2(size_T_s1_v2), d1_t2(size_T_d1_t2),
    d1_v2(size_T_d1_v2), d2_t2(size_T_d2_t2), d2_v2(size_T_d2_v2), host_energies(2);
  std::vector<int> s1_size(6), s1_exec(9), d1_size(7 * noab), d1_exec(9 * noab), d2_size(7 * nvab),
    d2_exec(9 * nvab), h7_size(noab), p7_size(nvab);

  LRUCache<Index, std::vector<double>> c1, c2, c3, c4, c5, c6;
  std::vector<double>                  energy_l(2, 0.0);
  long                                 ntasks = 0;
  std::vector<std::tuple<size_t, size_t, size_t, size_t, size_t, size_t, double>> task_list;

  // task loop: ccsd_t_fused_driver.hpp:368-395 (single rank, every task taken)
  for(size_t t_h1b = 0; t_h1b < noab; t_h1b++)
    for(size_t t_p4b = noab; t_p4b < noab + nvab; t_p4b++)
      for(size_t t_h2b = t_h1b; t_h2b < noab; t_h2b++)
        for(size_t t_p5b = t_p4b; t_p5b < noab + nvab; t_p5b++)
          for(size_t t_p6b = t_p5b; t_p6b < noab + nvab; t_p6b++)
            for(size_t t_h3b = t_h2b; t_h3b < noab; t_h3b++) {
              int sp = k_spin[t_p4b] + k_spin[t_p5b] + k_spin[t_p6b];
              int sh = k_spin[t_h1b] + k_spin[t_h2b] + k_spin[t_h3b];
              if(sp != sh) continue;
              if(is_restricted && sp + sh > 8) continue;
              double factor = is_restricted ? 2.0 : 1.0;
              if(t_p4b == t_p5b && t_p5b == t_p6b) factor /= 6.0;
              else if(t_p4b == t_p5b || t_p5b == t_p6b) factor /= 2.0;
              if(t_h1b == t_h2b && t_h2b == t_h3b) factor /= 6.0;
              else if(t_h1b == t_h2b || t_h2b == t_h3b) factor /= 2.0;
              ntasks++;
              task_list.emplace_back(t_h1b, t_h2b, t_h3b, t_p4b, t_p5b, t_p6b, factor);
              total_fused_ccsd_t_cpu<double>(
                is_restricted, noab, nvab, 0, k_spin, k_range, k_offset, d_t1, d_t2, d_v2,
                k_evl_sorted, s1_t1.data(), s1_v2.data(), d1_t2.data(), d1_v2.data(), d2_t2.data(),
                d2_v2.data(), host_energies.data(), h7_size.data(), p7_size.data(), s1_size.data(),
                d1_size.data(), d2_size.data(), s1_exec.data(), d1_exec.data(), d2_exec.data(),
                t_h1b, t_h2b, t_h3b, t_p4b, t_p5b, t_p6b, factor, (size_t) ntasks,
                max_d1_kernels_pertask, max_d2_kernels_pertask, size_T_s1_t1, size_T_s1_v2,
                size_T_d1_t2, size_T_d1_v2, size_T_d2_t2, size_T_d2_v2, energy_l, c1, c2, c3, c4,
                c5, c6);
            }

  *e_bracket = energy_l[0];
  *e_paren   = energy_l[1];
  if(tasks_out) *tasks_out = ntasks;
  if(ops_out) {
    // the reference's own flop count (fused_common.hpp:34-128) over the same task list
    CCSD_T_Fused_Common<double> fc;
    std::vector<double>         evl = k_evl_sorted;
    long double ops = fc.ccsd_t_fully_fused_performance(is_restricted, task_list, 0, 1, noab, nvab,
                                                        k_spin, k_range, k_offset, evl);
    *ops_out = (double) ops;
  }
  return 0;
}

extern "C" int ref_ccsd_t_energy(int o, int v, int n_occ_tiles, const int* occ_tiles, int n_vir_tiles,
                                 const int* vir_tiles, const double* eps_occ, const double* eps_vir,
                                 const double* t1, const double* t2, const double* oovv,
                                 const double* ooov, const double* ovvv, double* e_bracket,
                                 double* e_paren, double* ops_out, long* tasks_out) {
  std::vector<size_t> otl(occ_tiles, occ_tiles + n_occ_tiles), vtl(vir_tiles, vir_tiles + n_vir_tiles);
  size_t so = 0, sv = 0;
  for(auto x: otl) so += x;
  for(auto x: vtl) sv += x;
  if((int) so != o || (int) sv != v) return 1;

  // MO tiles: occ_a | occ_b | virt_a | virt_b
  std::vector<size_t> k_range;
  for(auto x: otl) k_range.push_back(x);
  for(auto x: otl) k_range.push_back(x);
  for(auto x: vtl) k_range.push_back(x);
  for(auto x: vtl) k_range.push_back(x);
  const Index noa = otl.size(), nva = vtl.size();
  const Index noab = 2 * noa, nvab = 2 * nva;
  std::vector<int> k_spin;
  for(Index t = 0; t < noab; t++) k_spin.push_back(t < noa ? 1 : 2);
  for(Index t = 0; t < nvab; t++) k_spin.push_back(t < nva ? 1 : 2);
  std::vector<size_t> k_offset;
  size_t              acc = 0;
  for(auto x: k_range) {
    k_offset.push_back(acc);
    acc += x;
  }
  std::vector<double> k_evl_sorted;
  for(int s = 0; s < 2; s++)
    for(int i = 0; i < o; i++) k_evl_sorted.push_back(eps_occ[i]);
  for(int s = 0; s < 2; s++)
    for(int a = 0; a < v; a++) k_evl_sorted.push_back(eps_vir[a]);

  std::vector<size_t> OT, VT; // tile lists of the spin-orbital occ / virt spaces
  for(Index t = 0; t < noab; t++) OT.push_back(k_range[t]);
  for(Index t = 0; t < nvab; t++) VT.push_back(k_range[noab + t]);
  Tensor<double> d_t1, d_t2;
  exachem::cholesky_2e::V2Tensors<double> d_v2;
  build_spin_orbital(o, v, OT, VT, t1, t2, oovv, ooov, ovvv, d_t1, d_t2, d_v2);

  return run_tasks(k_range, noab, nvab, noa, nva, true, k_spin, k_offset, k_evl_sorted, d_t1, d_t2, d_v2, true,
                   e_bracket, e_paren, ops_out, tasks_out);
}

// the uniform tiling the reference builds from ccsdt_tilesize (cholesky_2e.cpp:230-285)
extern "C" int ref_ccsd_t_energy_ts(int o, int v, int ts, const double* eps_occ,
                                    const double* eps_vir, const double* t1, const double* t2,
                                    const double* oovv, const double* ooov, const double* ovvv,
                                    double* e_bracket, double* e_paren, double* ops_out,
                                    long* tasks_out) {
  auto            ot = split_range(o, ts), vt = split_range(v, ts);
  std::vector<int> oti(ot.begin(), ot.end()), vti(vt.begin(), vt.end());
  return ref_ccsd_t_energy(o, v, (int) oti.size(), oti.data(), (int) vti.size(), vti.data(), eps_occ,
                           eps_vir, t1, t2, oovv, ooov, ovvv, e_bracket, e_paren, ops_out, tasks_out);
}

// Any (restricted or open-shell) input given directly over spin orbitals, in the layouts of
// ExaChem's tensors: MO order occ_a | occ_b | virt_a | virt_b with the tile extents of each range;
// eps[O + V] in that order; dense t1[V][O], t2[V][V][O][O], v2ijab[O][O][V][V] = <ij||ab>,
// v2ijka[O][O][O][V] = <ij||ka>, v2iabc[O][V][V][V] = <ia||bc> over the spin-orbital occupied
// (O = occ_a + occ_b) and virtual (V = virt_a + virt_b) ranges.  is_restricted selects the
// reference's spin filter and factor (ccsd_t_fused_driver.hpp:383-392); the buffers are sized
// for every tile (tilesize_opt = false, :181-182), as alpha and beta tile counts may differ.
extern "C" int ref_ccsd_t_energy_so(int n_oa, const int* oa, int n_ob, const int* ob, int n_va, const int* va,
                                    int n_vb, const int* vb, const double* eps, const double* t1,
                                    const double* t2, const double* v2ijab, const double* v2ijka,
                                    const double* v2iabc, int is_restricted, double* e_bracket,
                                    double* e_paren, long* tasks_out) {
  std::vector<size_t> k_range;
  std::vector<int>    k_spin;
  size_t              O = 0, V = 0;
  for(int t = 0; t < n_oa; t++) k_range.push_back(oa[t]), k_spin.push_back(1), O += oa[t];
  for(int t = 0; t < n_ob; t++) k_range.push_back(ob[t]), k_spin.push_back(2), O += ob[t];
  for(int t = 0; t < n_va; t++) k_range.push_back(va[t]), k_spin.push_back(1), V += va[t];
  for(int t = 0; t < n_vb; t++) k_range.push_back(vb[t]), k_spin.push_back(2), V += vb[t];
  const Index noab = n_oa + n_ob, nvab = n_va + n_vb;
  std::vector<size_t> k_offset;
  size_t              acc = 0;
  for(auto x: k_range) {
    k_offset.push_back(acc);
    acc += x;
  }
  std::vector<double> k_evl_sorted(eps, eps + O + V);
  std::vector<size_t> OT(k_range.begin(), k_range.begin() + noab), VT(k_range.begin() + noab, k_range.end());
  Tensor<double>                          d_t1({VT, OT}), d_t2({VT, VT, OT, OT});
  exachem::cholesky_2e::V2Tensors<double> d_v2;
  d_v2.v2ijab = Tensor<double>({OT, OT, VT, VT});
  d_v2.v2ijka = Tensor<double>({OT, OT, OT, VT});
  d_v2.v2iabc = Tensor<double>({OT, VT, VT, VT});
  // the dense arrays are row-major in the tensors' own index order
  std::copy(t1, t1 + V * O, d_t1.data());
  std::copy(t2, t2 + V * V * O * O, d_t2.data());
  std::copy(v2ijab, v2ijab + O * O * V * V, d_v2.v2ijab.data());
  std::copy(v2ijka, v2ijka + O * O * O * V, d_v2.v2ijka.data());
  std::copy(v2iabc, v2iabc + O * V * V * V, d_v2.v2iabc.data());
  return run_tasks(k_range, noab, nvab, n_oa, n_va, false, k_spin, k_offset, k_evl_sorted, d_t1, d_t2, d_v2,
                   is_restricted != 0, e_bracket, e_paren, nullptr, tasks_out);
}
