// Exercises include/exachem_compat/ccsd_t_fused_driver.hpp the way ExaChem would feed it:
// spin-orbital tiled tensors (built with the oracle's spin_orbital.hpp on the TAMM stand-in)
// -> gather_closed_shell() -> spatial arrays, and optionally run_closed_shell() on the GPU.
// Every gather reads the tensors through SpinCheckedTensor, which throws on a spin-forbidden
// block as a block-sparse TAMM tensor would.
//
//   compat_driver <in.bin> <out.bin> [--run | --run-tiled | --cs | --chol <chol.bin> [--run]]
// in.bin : int32 o, v, noa, nva, occ tiles[noa], vir tiles[nva]; float64 eps_occ[o] eps_vir[v]
//          t1 t2 oovv ooov ovvv (C-ABI layouts)
// out.bin: the gathered float64 arrays in the same order; with --run also E[T], E(T).
// --cs   : the closed-shell CCSD's t1_aa / t2_abab tensors instead, through gather_cs_amplitudes.
// --chol : chol.bin = int32 nq, nci, ci tiles[nci]; float64 L[o+v][o+v][nq] (spatial, occupied
//          first).  The driver builds the spin-orbital Cholesky tensor cholVpr {MO, MO, CI} on the
//          TAMM stand-in, gathers it with gather_cholesky and appends L_oo, L_ov, L_vv to out.bin;
//          with --run also E[T], E(T) through run_closed_shell_cholesky.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "spin_orbital.hpp"
#include "exachem_compat/ccsd_t_fused_driver.hpp"

template<typename X>
static void rd(std::ifstream& f, X* p, size_t n) {
  f.read(reinterpret_cast<char*>(p), sizeof(X) * n);
}

// A stand-in tensor that, like a block-sparse TAMM tensor, holds no spin-forbidden blocks:
// Tensor::get of one throws.  spins[m][t] = spin of tile t of mode m; a block is allowed when the
// spins of the first half of its modes sum to those of the second half.
struct SpinCheckedTensor {
  const tamm::Tensor<double>*   t = nullptr;
  std::vector<std::vector<int>> spins;
  void get(const tamm::IndexVector& bid, std::vector<double>& buf) const {
    int lo = 0, hi = 0;
    for(size_t m = 0; m < bid.size(); m++) (m < bid.size() / 2 ? lo : hi) += spins[m][bid[m]];
    if(lo != hi) throw std::runtime_error("Tensor::get of a spin-forbidden block");
    t->get(bid, buf);
  }
};
struct SpinCheckedV2 {
  SpinCheckedTensor v2ijab, v2ijka, v2iabc;
};

// compat_driver --so <so.bin> <out.bin> [--run]: the open-shell case.
// so.bin : int32 oa, ob, va, vb, n tiles of occ_a, occ_b, virt_a, virt_b, then those tile
//          extents; float64 eps[O + V] (MO order), t1[V][O], t2[V][V][O][O], v2ijab[O][O][V][V],
//          v2ijka[O][O][O][V], v2iabc[O][V][V][V] (dense spin-orbital arrays).
// The arrays fill the TAMM stand-in tensors as they are, and each tensor is read through a
// SpinCheckedTensor, which throws on a spin-forbidden block (the gather must never ask for one);
// out.bin = gather_spin_orbital's arrays in the same order, with --run followed by E[T], E(T)
// from run_spin_orbital.
static int open_shell(int argc, char** argv) {
  std::ifstream f(argv[2], std::ios::binary);
  int           hdr[8];
  rd(f, hdr, 8);
  std::vector<int> tl(hdr[4] + hdr[5] + hdr[6] + hdr[7]);
  rd(f, tl.data(), tl.size());
  const size_t        O = (size_t) hdr[0] + hdr[1], V = (size_t) hdr[2] + hdr[3];
  std::vector<size_t> mo(tl.begin(), tl.end()), OT(tl.begin(), tl.begin() + hdr[4] + hdr[5]),
    VT(tl.begin() + hdr[4] + hdr[5], tl.end());
  std::vector<double> eps(O + V);
  rd(f, eps.data(), eps.size());
  tamm::Tensor<double>                    d_t1({VT, OT}), d_t2({VT, VT, OT, OT});
  exachem::cholesky_2e::V2Tensors<double> d_v2;
  d_v2.v2ijab = tamm::Tensor<double>({OT, OT, VT, VT});
  d_v2.v2ijka = tamm::Tensor<double>({OT, OT, OT, VT});
  d_v2.v2iabc = tamm::Tensor<double>({OT, VT, VT, VT});
  rd(f, d_t1.data(), V * O);
  rd(f, d_t2.data(), V * V * O * O);
  rd(f, d_v2.v2ijab.data(), O * O * V * V);
  rd(f, d_v2.v2ijka.data(), O * O * O * V);
  rd(f, d_v2.v2iabc.data(), O * V * V * V);
  if(!f) return 3;
  std::vector<int> so_t, sv_t; // tile spins of the occupied / virtual modes
  for(int t = 0; t < hdr[4] + hdr[5]; t++) so_t.push_back(t >= hdr[4]);
  for(int t = 0; t < hdr[6] + hdr[7]; t++) sv_t.push_back(t >= hdr[6]);
  SpinCheckedTensor c_t1{&d_t1, {sv_t, so_t}}, c_t2{&d_t2, {sv_t, sv_t, so_t, so_t}};
  SpinCheckedV2     c_v2{{&d_v2.v2ijab, {so_t, so_t, sv_t, sv_t}},
                         {&d_v2.v2ijka, {so_t, so_t, so_t, sv_t}},
                         {&d_v2.v2iabc, {so_t, sv_t, sv_t, sv_t}}};
  auto S = exachem_gb300::gather_spin_orbital<double>(mo, hdr[4], hdr[5], hdr[6], hdr[7], c_t1, c_t2, c_v2, eps);
  if((size_t) S.oa + S.ob != O || (size_t) S.va + S.vb != V) return 4;
  std::ofstream g(argv[3], std::ios::binary);
  for(auto* a: {&S.eps_occ, &S.eps_vir, &S.t1, &S.t2, &S.v2ijab, &S.v2ijka, &S.v2iabc})
    g.write(reinterpret_cast<const char*>(a->data()), sizeof(double) * a->size());
  if(argc > 4 && std::string(argv[4]) == "--run") {
    auto [e4, e5, secs] = exachem_gb300::run_spin_orbital(S);
    g.write(reinterpret_cast<const char*>(&e4), sizeof(double));
    g.write(reinterpret_cast<const char*>(&e5), sizeof(double));
    std::printf("E[T] %.17g E(T) %.17g (%.3f s)\n", e4, e5, secs);
  }
  return 0;
}

int main(int argc, char** argv) {
  if(argc > 3 && std::string(argv[1]) == "--so") return open_shell(argc, argv);
  if(argc < 3) return 2;
  std::ifstream f(argv[1], std::ios::binary);
  int           hdr[4];
  rd(f, hdr, 4);
  const int o = hdr[0], v = hdr[1], noa = hdr[2], nva = hdr[3];
  std::vector<int> ot(noa), vt(nva);
  rd(f, ot.data(), noa);
  rd(f, vt.data(), nva);
  std::vector<double> eo(o), ev(v), t1((size_t) o * v), t2((size_t) o * o * v * v), oovv(t2.size()),
    ooov((size_t) o * o * o * v), ovvv((size_t) o * v * v * v);
  for(auto* a: {&eo, &ev, &t1, &t2, &oovv, &ooov, &ovvv}) rd(f, a->data(), a->size());
  if(!f) return 3;

  // MO space occ_a | occ_b | virt_a | virt_b, as ExaChem tiles it
  std::vector<size_t> mo, OT, VT;
  for(int s = 0; s < 2; s++)
    for(int x: ot) OT.push_back(x);
  for(int s = 0; s < 2; s++)
    for(int x: vt) VT.push_back(x);
  mo.insert(mo.end(), OT.begin(), OT.end());
  mo.insert(mo.end(), VT.begin(), VT.end());
  std::vector<double> k_evl;
  for(int s = 0; s < 2; s++) k_evl.insert(k_evl.end(), eo.begin(), eo.end());
  for(int s = 0; s < 2; s++) k_evl.insert(k_evl.end(), ev.begin(), ev.end());
  tamm::Tensor<double>                    d_t1, d_t2;
  exachem::cholesky_2e::V2Tensors<double> d_v2;
  build_spin_orbital(o, v, OT, VT, t1.data(), t2.data(), oovv.data(), ooov.data(), ovvv.data(), d_t1, d_t2, d_v2);
  // every read below goes through tensors that throw on a spin-forbidden block
  std::vector<int> so_t, sv_t;
  for(size_t t = 0; t < OT.size(); t++) so_t.push_back(t >= (size_t) noa);
  for(size_t t = 0; t < VT.size(); t++) sv_t.push_back(t >= (size_t) nva);
  SpinCheckedTensor c_t1{&d_t1, {sv_t, so_t}}, c_t2{&d_t2, {sv_t, sv_t, so_t, so_t}};
  SpinCheckedV2     c_v2{{&d_v2.v2ijab, {so_t, so_t, sv_t, sv_t}},
                         {&d_v2.v2ijka, {so_t, so_t, so_t, sv_t}},
                         {&d_v2.v2iabc, {so_t, sv_t, sv_t, sv_t}}};

  if(argc > 3 && std::string(argv[3]) == "--cs") {
    // the closed-shell CCSD's own tensors: t1_aa {v_alpha, o_alpha}, t2_abab {v_alpha, v_beta,
    // o_alpha, o_beta}, tile ids from 0 in each mode; out.bin = eps_occ, eps_vir, t1, t2
    std::vector<size_t>  ota(ot.begin(), ot.end()), vta(vt.begin(), vt.end());
    tamm::Tensor<double> t1_aa({vta, ota}), t2_abab({vta, vta, ota, ota});
    for(int a = 0; a < v; a++)
      for(int i = 0; i < o; i++) t1_aa.data()[(size_t) a * o + i] = t1[(size_t) i * v + a];
    for(int a = 0; a < v; a++)
      for(int b = 0; b < v; b++)
        for(int i = 0; i < o; i++)
          for(int j = 0; j < o; j++)
            t2_abab.data()[(((size_t) a * v + b) * o + i) * o + j] = t2[(((size_t) i * o + j) * v + a) * v + b];
    auto          A = exachem_gb300::gather_cs_amplitudes<double>(mo, noa, nva, t1_aa, t2_abab, k_evl);
    std::ofstream g(argv[2], std::ios::binary);
    for(auto* x: {&A.eps_occ, &A.eps_vir, &A.t1, &A.t2})
      g.write(reinterpret_cast<const char*>(x->data()), sizeof(double) * x->size());
    return 0;
  }
  auto S = exachem_gb300::gather_closed_shell<double>(mo, noa, nva, c_t1, c_t2, c_v2, k_evl);
  std::ofstream g(argv[2], std::ios::binary);
  for(auto* a: {&S.eps_occ, &S.eps_vir, &S.t1, &S.t2, &S.oovv, &S.ooov, &S.ovvv})
    g.write(reinterpret_cast<const char*>(a->data()), sizeof(double) * a->size());
  if(argc > 4 && std::string(argv[3]) == "--chol") {
    std::ifstream c(argv[4], std::ios::binary);
    int           h2[2];
    rd(c, h2, 2);
    const int        nq = h2[0], nci = h2[1];
    std::vector<int> cit(nci);
    rd(c, cit.data(), nci);
    const size_t        n = (size_t) o + v;
    std::vector<double> L(n * n * nq);
    rd(c, L.data(), L.size());
    if(!c) return 4;
    std::vector<size_t> CT(cit.begin(), cit.end());
    // spin-orbital MO index (occ_a | occ_b | virt_a | virt_b) -> (spatial index, spin)
    auto sp = [&](size_t p, int& spin) -> size_t {
      if(p < (size_t) 2 * o) return spin = (int) (p / o), p % o;
      p -= 2 * o;
      return spin = (int) (p / v), o + p % v;
    };
    tamm::Tensor<double> chol({mo, mo, CT});
    for(size_t p = 0; p < 2 * n; p++)
      for(size_t q = 0; q < 2 * n; q++) {
        int          s1, s2;
        const size_t a = sp(p, s1), b = sp(q, s2);
        for(size_t Q = 0; Q < (size_t) nq; Q++) {
          size_t idx[3] = {p, q, Q};
          chol.at(idx)  = s1 == s2 ? L[(a * n + b) * nq + Q] : 0.0;
        }
      }
    auto C = exachem_gb300::gather_cholesky<double>(mo, noa, nva, CT, chol);
    for(auto* a: {&C.L_oo, &C.L_ov, &C.L_vv}) g.write(reinterpret_cast<const char*>(a->data()), sizeof(double) * a->size());
    if(argc > 5 && std::string(argv[5]) == "--run") {
      ccsdt_opts op{};
      op.mode = CCSDT_MODE_FP64;
      auto A = exachem_gb300::gather_amplitudes<double>(mo, noa, nva, c_t1, c_t2, k_evl);
      auto [e4, e5, secs] = exachem_gb300::run_closed_shell_cholesky(A, C, 0, op);
      g.write(reinterpret_cast<const char*>(&e4), sizeof(double));
      g.write(reinterpret_cast<const char*>(&e5), sizeof(double));
      std::printf("E[T] %.17g E(T) %.17g (%.3f s)\n", e4, e5, secs);
    }
  }
  if(argc > 3 && std::string(argv[3]) == "--run-tiled") {
    // the drop-in path: blocks through the device-side retile, then the (T) call
    ccsdt_opts op{};
    op.mode = CCSDT_MODE_FP64;
    auto [e4, e5, secs, total] = exachem_gb300::run_tiled<double>(mo, noa, nva, c_t1, c_t2, c_v2, k_evl, op,
                                                                 std::chrono::steady_clock::now(), 0);
    g.write(reinterpret_cast<const char*>(&e4), sizeof(double));
    g.write(reinterpret_cast<const char*>(&e5), sizeof(double));
    std::printf("E[T] %.17g E(T) %.17g (%.3f s device, %.3f s total)\n", e4, e5, secs, total);
  }
  if(argc > 3 && std::string(argv[3]) == "--run") {
    ccsdt_opts op{};
    op.mode = CCSDT_MODE_FP64;
    auto [e4, e5, secs] = exachem_gb300::run_closed_shell(S, 0, op);
    g.write(reinterpret_cast<const char*>(&e4), sizeof(double));
    g.write(reinterpret_cast<const char*>(&e5), sizeof(double));
    std::printf("E[T] %.17g E(T) %.17g (%.3f s)\n", e4, e5, secs);
  }
  return 0;
}
