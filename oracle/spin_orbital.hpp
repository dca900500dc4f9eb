// Spin-orbital tiled T1 / T2 / V2 tensors from closed-shell spatial arrays, in the form
// ExaChem's (T) driver consumes.  TEST INFRASTRUCTURE ONLY (oracle/_ref and the tests of the
// drop-in adapter).  Conventions:
//   T2 spin blocks    exachem/cc/ccsd/cd_ccsd_cs_ann.cpp:26-31 (aaaa), :949-973 (the rest)
//   T1                t1_bb = t1_aa (cd_ccsd_cs_ann.cpp:949-950)
//   V2 blocks         exachem/cholesky/v2tensors.cpp:67-86, Cholesky vectors of spin {1,1}
// Spin-orbital occupied index p < o is alpha (spatial p), p >= o beta (spatial p - o); the same
// for virtuals with v.  OT / VT: tile extents of the spin-orbital occ / virt spaces.
#pragma once

#include <cstddef>
#include <vector>

#include "tamm/tamm.hpp"

struct SpinOrb {
  size_t n;
  size_t sp(size_t p) const { return p < n ? p : p - n; }
  int    spin(size_t p) const { return p < n ? 0 : 1; }
};

inline void build_spin_orbital(int o, int v, const std::vector<size_t>& OT, const std::vector<size_t>& VT,
                               const double* t1, const double* t2, const double* oovv,
                               const double* ooov, const double* ovvv, tamm::Tensor<double>& d_t1,
                               tamm::Tensor<double>& d_t2,
                               exachem::cholesky_2e::V2Tensors<double>& d_v2) {
  const size_t O = 2 * o, V = 2 * v;
  SpinOrb      so_o{(size_t) o}, so_v{(size_t) v};
  auto T2sp = [&](size_t i, size_t j, size_t a, size_t b) {
    return t2[((i * o + j) * v + a) * v + b];
  };
  auto ovov = [&](size_t i, size_t a, size_t j, size_t b) { // (ia|jb)
    return oovv[((i * o + j) * v + a) * v + b];
  };
  auto oo_ov = [&](size_t i, size_t j, size_t k, size_t a) { // (ij|ka)
    return ooov[((i * o + j) * o + k) * v + a];
  };
  auto ov_vv = [&](size_t i, size_t a, size_t b, size_t c) { // (ia|bc)
    return ovvv[((i * v + a) * v + b) * v + c];
  };

  d_t1 = tamm::Tensor<double>({VT, OT});
  d_t2 = tamm::Tensor<double>({VT, VT, OT, OT});
  d_v2.v2ijab = tamm::Tensor<double>({OT, OT, VT, VT});
  d_v2.v2ijka = tamm::Tensor<double>({OT, OT, OT, VT});
  d_v2.v2iabc = tamm::Tensor<double>({OT, VT, VT, VT});

  for(size_t a = 0; a < V; a++)
    for(size_t i = 0; i < O; i++) {
      size_t idx[2] = {a, i};
      d_t1.at(idx) = so_v.spin(a) == so_o.spin(i) ? t1[so_o.sp(i) * v + so_v.sp(a)] : 0.0;
    }

  // T2 spin blocks (cd_ccsd_cs_ann.cpp:26-31 for aaaa, :949-973 for the rest)
  for(size_t a = 0; a < V; a++)
    for(size_t b = 0; b < V; b++)
      for(size_t i = 0; i < O; i++)
        for(size_t j = 0; j < O; j++) {
          int    sa = so_v.spin(a), sb = so_v.spin(b), si = so_o.spin(i), sj = so_o.spin(j);
          size_t A = so_v.sp(a), B = so_v.sp(b), I = so_o.sp(i), J = so_o.sp(j);
          double val = 0.0;
          if(sa == sb && si == sj && sa == si) val = T2sp(I, J, A, B) - T2sp(I, J, B, A);
          else if(sa == si && sb == sj && sa != sb) val = T2sp(I, J, A, B);  // abab / baba
          else if(sa == sj && sb == si && sa != sb) val = -T2sp(J, I, A, B); // abba / baab
          size_t idx[4] = {a, b, i, j};
          d_t2.at(idx)  = val;
        }

  // chemist integral over spin orbitals: (pq|rs) vanishes unless spin p == spin q and spin r == spin s
  for(size_t i = 0; i < O; i++)
    for(size_t j = 0; j < O; j++)
      for(size_t a = 0; a < V; a++)
        for(size_t b = 0; b < V; b++) {
          // v2ijab(h1,h2,p1,p2) = (h1 p1|h2 p2) - (h1 p2|h2 p1)
          int    si = so_o.spin(i), sj = so_o.spin(j), sa = so_v.spin(a), sb = so_v.spin(b);
          size_t I = so_o.sp(i), J = so_o.sp(j), A = so_v.sp(a), B = so_v.sp(b);
          double val = 0.0;
          if(si == sa && sj == sb) val += ovov(I, A, J, B);
          if(si == sb && sj == sa) val -= ovov(I, B, J, A);
          size_t idx[4]        = {i, j, a, b};
          d_v2.v2ijab.at(idx) = val;
        }
  for(size_t i = 0; i < O; i++)
    for(size_t j = 0; j < O; j++)
      for(size_t k = 0; k < O; k++)
        for(size_t a = 0; a < V; a++) {
          // v2ijka(h1,h2,h3,p1) = (h1 h3|h2 p1) - (h2 h3|h1 p1)
          int    si = so_o.spin(i), sj = so_o.spin(j), sk = so_o.spin(k), sa = so_v.spin(a);
          size_t I = so_o.sp(i), J = so_o.sp(j), K = so_o.sp(k), A = so_v.sp(a);
          double val = 0.0;
          if(si == sk && sj == sa) val += oo_ov(I, K, J, A);
          if(sj == sk && si == sa) val -= oo_ov(J, K, I, A);
          size_t idx[4]        = {i, j, k, a};
          d_v2.v2ijka.at(idx) = val;
        }
  for(size_t i = 0; i < O; i++)
    for(size_t a = 0; a < V; a++)
      for(size_t b = 0; b < V; b++)
        for(size_t c = 0; c < V; c++) {
          // v2iabc(h1,p1,p2,p3) = (h1 p2|p1 p3) - (h1 p3|p1 p2)
          int    si = so_o.spin(i), sa = so_v.spin(a), sb = so_v.spin(b), sc = so_v.spin(c);
          size_t I = so_o.sp(i), A = so_v.sp(a), B = so_v.sp(b), C = so_v.sp(c);
          double val = 0.0;
          if(si == sb && sa == sc) val += ov_vv(I, B, A, C);
          if(si == sc && sa == sb) val -= ov_vv(I, C, A, B);
          size_t idx[4]        = {i, a, b, c};
          d_v2.v2iabc.at(idx) = val;
        }

}
