// Drop-in replacement for ExaChem's fused (T) driver entry point
//   std::tuple<T,T,double,double> CCSD_T_Fused_Driver<T>::execute(...)
//   (exachem/cc/ccsd_t/ccsd_t_fused_driver.hpp:73-81, 91-546; called from ccsd_t.cpp:253-256)
// backed by the GB300 library (include/ccsdt.h).
//
// Entry points:
//  * gather_closed_shell(): reads the spin-orbital tiled blocks ExaChem holds - d_t1 {V,O},
//    d_t2 {V,V,O,O}, v2ijab {O,O,V,V}, v2ijka {O,O,O,V}, v2iabc {O,V,V,V}, k_evl_sorted in MO
//    order occ_a | occ_b | virt_a | virt_b - with Tensor::get(block ids, buffer), the same call
//    the reference's gathers make (ccsd_t_all_fused_singles.hpp:200,304,
//    doubles1.hpp:222,237,282, doubles2.hpp:215,230,335), and returns the closed-shell spatial
//    arrays of include/ccsdt.h.  Only alpha / alpha-beta blocks are read:
//        t_ij^ab = t2(a_alpha, b_beta, i_alpha, j_beta)         (cd_ccsd_cs_ann.cpp:949-973)
//        (ia|jb) = v2ijab(i_alpha, j_beta, a_alpha, b_beta)     (v2tensors.cpp:67-70)
//        (ij|ka) = v2ijka(i_alpha, k_beta, j_alpha, a_beta)     (v2tensors.cpp:76-78)
//        (ia|bc) = v2iabc(i_alpha, b_beta, a_alpha, c_beta)     (v2tensors.cpp:84-86)
//    (in each the exchange part of the antisymmetrised block vanishes by spin).
//    It is a template over the tensor types, so it needs only Tensor<T>::get.
//  * gather_cs_amplitudes(): the closed-shell CCSD's own t1_aa / t2_abab (no spin-orbital expansion).
//  * gather_cholesky() + run_closed_shell_cholesky(): the alternative that skips V2 - the
//    alpha-alpha blocks of the Cholesky tensor cholVpr, with the integral blocks built on the GPU.
//  * gather_spin_orbital() + run_spin_orbital(): the open-shell case (is_restricted = false) -
//    every spin-allowed block of the same tensors, alpha and beta tile lists of their own, into
//    the dense spin-orbital arrays of ccsdt_energy_spin_orbital.
//  * exachem::cc::ccsd_t::CCSD_T_Fused_Driver<T>::execute(): the reference's namespace, class and
//    signature, compiled when EXACHEM_GB300_WITH_TAMM is defined (inside an ExaChem build).  Each
//    rank of the process
//    group takes every size-th occupied triplet on its own GPU and returns its partial
//    energies; ccsd_t.cpp:262-263 already sums them with pg().reduce.
#pragma once

#include <algorithm>
#include <chrono>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "../ccsdt.h"

namespace exachem_gb300 {

struct SpatialInputs {
  int                 o = 0, v = 0;
  std::vector<int>    occ_tiles, vir_tiles; // alpha tile extents
  std::vector<double> eps_occ, eps_vir, t1, t2, oovv, ooov, ovvv;
};

namespace detail {
inline std::vector<size_t> offsets(const std::vector<size_t>& ext) {
  std::vector<size_t> off;
  size_t              s = 0;
  for(auto e: ext) {
    off.push_back(s);
    s += e;
  }
  return off;
}
} // namespace detail

namespace detail {
// t1(a_alpha, i_alpha) and t2(a_alpha, b_beta, i_alpha, j_beta) into the spatial t1 / t2; the beta
// tile ids of the tensors start at ob_base (occupied) / vb_base (virtual).
template<typename T, typename TensorT>
SpatialInputs gather_amplitudes_at(const std::vector<size_t>& mo_tiles, size_t noa, size_t nva, TensorT& d_t1,
                                   TensorT& d_t2, const std::vector<T>& k_evl_sorted, size_t ob_base,
                                   size_t vb_base);
} // namespace detail

// mo_tiles: extents of the MO tiles in the order occ_a, occ_b, virt_a, virt_b (as
// TiledIndexSpace::input_tile_sizes() returns them); noa / nva: alpha occupied / virtual tiles.
// The amplitudes and orbital energies only (the integral arrays stay empty).
template<typename T, typename TensorT>
SpatialInputs gather_amplitudes(const std::vector<size_t>& mo_tiles, size_t noa, size_t nva, TensorT& d_t1,
                                TensorT& d_t2, const std::vector<T>& k_evl_sorted) {
  return detail::gather_amplitudes_at<T>(mo_tiles, noa, nva, d_t1, d_t2, k_evl_sorted, noa, nva);
}

// The closed-shell CCSD's own amplitudes, without the spin-orbital expansion the reference runs
// before (T) (cd_ccsd_cs_ann.cpp:932-975): t1_aa {v_alpha, o_alpha} and t2_abab {v_alpha, v_beta,
// o_alpha, o_beta} as setupTensors_cs allocates them (ccsd_util.cpp:550-575), over the sub-spaces
// o_alpha = {MO("occ"), range(noa)}, o_beta = {MO("occ"), range(noa, 2 noa)} (and the virtual
// ones), whose tile ids start at 0 in each tensor.  The call then needs neither dt1_full / dt2_full
// nor the six T2-sized temporaries of the expansion.
template<typename T, typename TensorT>
SpatialInputs gather_cs_amplitudes(const std::vector<size_t>& mo_tiles, size_t noa, size_t nva, TensorT& t1_aa,
                                   TensorT& t2_abab, const std::vector<T>& k_evl_sorted) {
  return detail::gather_amplitudes_at<T>(mo_tiles, noa, nva, t1_aa, t2_abab, k_evl_sorted, 0, 0);
}

template<typename T, typename TensorT>
SpatialInputs detail::gather_amplitudes_at(const std::vector<size_t>& mo_tiles, size_t noa, size_t nva,
                                           TensorT& d_t1, TensorT& d_t2, const std::vector<T>& k_evl_sorted,
                                           size_t ob_base, size_t vb_base) {
  if(mo_tiles.size() != 2 * noa + 2 * nva) throw std::invalid_argument("MO tiles != 2 noa + 2 nva");
  std::vector<size_t> ot(mo_tiles.begin(), mo_tiles.begin() + noa);
  std::vector<size_t> vt(mo_tiles.begin() + 2 * noa, mo_tiles.begin() + 2 * noa + nva);
  for(size_t t = 0; t < noa; t++)
    if(mo_tiles[noa + t] != ot[t]) throw std::invalid_argument("closed shell needs equal alpha/beta tiles");
  for(size_t t = 0; t < nva; t++)
    if(mo_tiles[2 * noa + nva + t] != vt[t]) throw std::invalid_argument("closed shell needs equal alpha/beta tiles");
  const auto   oo = detail::offsets(ot), vo = detail::offsets(vt);
  const size_t o = oo.empty() ? 0 : oo.back() + ot.back(), v = vo.empty() ? 0 : vo.back() + vt.back();
  SpatialInputs S;
  S.o = (int) o;
  S.v = (int) v;
  for(auto x: ot) S.occ_tiles.push_back((int) x);
  for(auto x: vt) S.vir_tiles.push_back((int) x);
  if(k_evl_sorted.size() < 2 * o + 2 * v) throw std::invalid_argument("k_evl_sorted too short");
  S.eps_occ.assign(k_evl_sorted.begin(), k_evl_sorted.begin() + o);
  S.eps_vir.assign(k_evl_sorted.begin() + 2 * o, k_evl_sorted.begin() + 2 * o + v);
  S.t1.assign(o * v, 0.0);
  S.t2.assign(o * o * v * v, 0.0);
  std::vector<T> buf;
  // block ids: O tiles 0..2noa-1 (beta = alpha + noa), V tiles 0..2nva-1 (beta = alpha + nva)
  for(size_t A = 0; A < nva; A++)
    for(size_t I = 0; I < noa; I++) {
      d_t1.get({A, I}, buf); // [a][i]
      for(size_t a = 0; a < vt[A]; a++)
        for(size_t i = 0; i < ot[I]; i++) S.t1[(oo[I] + i) * v + vo[A] + a] = buf[a * ot[I] + i];
    }
  for(size_t A = 0; A < nva; A++)
    for(size_t B = 0; B < nva; B++)
      for(size_t I = 0; I < noa; I++)
        for(size_t J = 0; J < noa; J++) {
          d_t2.get({A, B + vb_base, I, J + ob_base}, buf); // [a][b][i][j], a,i alpha / b,j beta
          for(size_t a = 0; a < vt[A]; a++)
            for(size_t b = 0; b < vt[B]; b++)
              for(size_t i = 0; i < ot[I]; i++)
                for(size_t j = 0; j < ot[J]; j++)
                  S.t2[(((oo[I] + i) * o + oo[J] + j) * v + vo[A] + a) * v + vo[B] + b] =
                    buf[((a * vt[B] + b) * ot[I] + i) * ot[J] + j];
        }
  return S;
}

// gather_amplitudes plus the three integral blocks from the V2 tensors.
template<typename T, typename TensorT, typename V2T>
SpatialInputs gather_closed_shell(const std::vector<size_t>& mo_tiles, size_t noa, size_t nva,
                                  TensorT& d_t1, TensorT& d_t2, V2T& d_v2,
                                  const std::vector<T>& k_evl_sorted) {
  SpatialInputs       S = gather_amplitudes<T>(mo_tiles, noa, nva, d_t1, d_t2, k_evl_sorted);
  std::vector<size_t> ot(mo_tiles.begin(), mo_tiles.begin() + noa);
  std::vector<size_t> vt(mo_tiles.begin() + 2 * noa, mo_tiles.begin() + 2 * noa + nva);
  const auto          oo = detail::offsets(ot), vo = detail::offsets(vt);
  const size_t        o = S.o, v = S.v;
  S.oovv.assign(o * o * v * v, 0.0);
  S.ooov.assign(o * o * o * v, 0.0);
  S.ovvv.assign(o * v * v * v, 0.0);
  std::vector<T> buf;
  for(size_t A = 0; A < nva; A++)
    for(size_t B = 0; B < nva; B++)
      for(size_t I = 0; I < noa; I++)
        for(size_t J = 0; J < noa; J++) {
          d_v2.v2ijab.get({I, J + noa, A, B + nva}, buf); // [i][j][a][b]
          for(size_t i = 0; i < ot[I]; i++)
            for(size_t j = 0; j < ot[J]; j++)
              for(size_t a = 0; a < vt[A]; a++)
                for(size_t b = 0; b < vt[B]; b++)
                  S.oovv[(((oo[I] + i) * o + oo[J] + j) * v + vo[A] + a) * v + vo[B] + b] =
                    buf[((i * ot[J] + j) * vt[A] + a) * vt[B] + b];
        }
  for(size_t I = 0; I < noa; I++)
    for(size_t K = 0; K < noa; K++)
      for(size_t J = 0; J < noa; J++)
        for(size_t A = 0; A < nva; A++) {
          d_v2.v2ijka.get({I, K + noa, J, A + nva}, buf); // [i][k][j][a] = (ij|ka)
          for(size_t i = 0; i < ot[I]; i++)
            for(size_t k = 0; k < ot[K]; k++)
              for(size_t j = 0; j < ot[J]; j++)
                for(size_t a = 0; a < vt[A]; a++)
                  S.ooov[(((oo[I] + i) * o + oo[J] + j) * o + oo[K] + k) * v + vo[A] + a] =
                    buf[((i * ot[K] + k) * ot[J] + j) * vt[A] + a];
        }
  for(size_t I = 0; I < noa; I++)
    for(size_t B = 0; B < nva; B++)
      for(size_t A = 0; A < nva; A++)
        for(size_t C = 0; C < nva; C++) {
          d_v2.v2iabc.get({I, B + nva, A, C + nva}, buf); // [i][b][a][c] = (ia|bc)
          for(size_t i = 0; i < ot[I]; i++)
            for(size_t b = 0; b < vt[B]; b++)
              for(size_t a = 0; a < vt[A]; a++)
                for(size_t c = 0; c < vt[C]; c++)
                  S.ovvv[(((oo[I] + i) * v + vo[A] + a) * v + vo[B] + b) * v + vo[C] + c] =
                    buf[((i * vt[B] + b) * vt[A] + a) * vt[C] + c];
        }
  return S;
}

// The slice-count model file written by exachem_gb300.learned (JSON: {"params": [floats], ...}):
// the CCSDT_MLP_NPARAM numbers of the "params" array.
inline std::vector<float> read_slice_model(const std::string& path) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if(!f) throw std::runtime_error("cannot open the slice model " + path);
  std::string text;
  char        buf[1 << 16];
  for(size_t k; (k = std::fread(buf, 1, sizeof(buf), f)) > 0;) text.append(buf, k);
  std::fclose(f);
  const size_t key = text.find("\"params\"");
  const size_t lb  = key == std::string::npos ? key : text.find('[', key);
  if(lb == std::string::npos) throw std::runtime_error("no params array in " + path);
  std::vector<float> p;
  const char*        c = text.c_str() + lb + 1;
  while(*c && *c != ']') {
    char*        end = nullptr;
    const double x   = std::strtod(c, &end);
    if(end == c) {
      ++c; // separator
      continue;
    }
    p.push_back((float) x);
    c = end;
  }
  if((int) p.size() != CCSDT_MLP_NPARAM) throw std::runtime_error("slice model " + path + ": wrong parameter count");
  return p;
}

// Mode from the environment: EXACHEM_GB300_MODE = fp64 (default) | ozaki | learned,
// EXACHEM_GB300_SLICES = digit planes (ozaki, default 3) or the largest count (learned, default 5),
// EXACHEM_GB300_BUDGET = the learned mode's energy budget (default 1e-8),
// EXACHEM_GB300_P_STORAGE = auto (default) | ff | f32 | f64: element type of the split path's partial arrays.
inline ccsdt_opts opts_from_env() {
  ccsdt_opts  op{};
  const char* m = std::getenv("EXACHEM_GB300_MODE");
  std::string mode = m ? m : "fp64";
  if(mode == "fp64") op.mode = CCSDT_MODE_FP64;
  else if(mode == "ozaki") op.mode = CCSDT_MODE_OZAKI;
  else if(mode == "learned") op.mode = CCSDT_MODE_LEARNED;
  else throw std::invalid_argument("EXACHEM_GB300_MODE must be fp64, ozaki or learned: " + mode);
  const char* sl = std::getenv("EXACHEM_GB300_SLICES");
  op.slices      = sl ? std::atoi(sl) : (op.mode == CCSDT_MODE_LEARNED ? 5 : 3);
  const char* bu = std::getenv("EXACHEM_GB300_BUDGET");
  op.energy_budget = bu ? std::atof(bu) : 1e-8;
  // the contraction's tile configuration tuned on this system on first use (results unchanged)
  const char* at = std::getenv("EXACHEM_GB300_AUTOTUNE");
  op.autotune    = at ? std::atoi(at) != 0 : 1;
  // split and learned modes: replay the call's per-batch launch sequence from a CUDA graph
  const char* gr = std::getenv("EXACHEM_GB300_GRAPH");
  op.use_graph   = gr ? std::atoi(gr) != 0 : 0;
  const char* ps = std::getenv("EXACHEM_GB300_P_STORAGE");
  std::string pst = ps ? ps : "auto";
  if(pst == "auto") op.p_storage = 0;
  else if(pst == "ff") op.p_storage = 1;
  else if(pst == "f32") op.p_storage = 2;
  else if(pst == "f64") op.p_storage = 3;
  else throw std::invalid_argument("EXACHEM_GB300_P_STORAGE must be auto, ff, f32 or f64: " + pst);
  return op;
}

// The model the learned mode installs: EXACHEM_GB300_SLICE_MODEL (required for that mode).
inline std::vector<float> slice_model_from_env() {
  const char* p = std::getenv("EXACHEM_GB300_SLICE_MODEL");
  if(!p) throw std::invalid_argument("the learned mode needs EXACHEM_GB300_SLICE_MODEL (a slice model file)");
  return read_slice_model(p);
}

// Uploads ExaChem's tiled inputs to a handle with the device-side retile (ccsdt_upload_begin /
// blocks / end): each alpha / alpha-beta block is read with Tensor::get - the call the reference's
// gathers make - into a host staging buffer of at most `stage_doubles` and handed over as is; the
// scatter into the spatial arrays runs on the GPU.  Only t1 and the orbital energies are gathered
// on the host (o v + o + v numbers).
template<typename T, typename TensorT, typename V2T>
void upload_tiled(ccsdt_handle* h, const std::vector<size_t>& mo_tiles, size_t noa, size_t nva, TensorT& d_t1,
                  TensorT& d_t2, V2T& d_v2, const std::vector<T>& k_evl_sorted, size_t stage_doubles = 1u << 26) {
  std::vector<size_t> ot(mo_tiles.begin(), mo_tiles.begin() + noa);
  std::vector<size_t> vt(mo_tiles.begin() + 2 * noa, mo_tiles.begin() + 2 * noa + nva);
  const auto   oo = detail::offsets(ot), vo = detail::offsets(vt);
  const size_t o = oo.back() + ot.back(), v = vo.back() + vt.back();
  auto check = [&](ccsdt_status st, const char* what) {
    if(st != CCSDT_OK) throw std::runtime_error(std::string(what) + ": " + ccsdt_last_error(h));
  };
  std::vector<double> eo(k_evl_sorted.begin(), k_evl_sorted.begin() + o);
  std::vector<double> ev(k_evl_sorted.begin() + 2 * o, k_evl_sorted.begin() + 2 * o + v);
  std::vector<double> t1(o * v, 0.0);
  std::vector<T>      buf;
  for(size_t A = 0; A < nva; A++)
    for(size_t I = 0; I < noa; I++) {
      d_t1.get({A, I}, buf); // [a][i]
      for(size_t a = 0; a < vt[A]; a++)
        for(size_t i = 0; i < ot[I]; i++) t1[(oo[I] + i) * v + vo[A] + a] = buf[a * ot[I] + i];
    }
  check(ccsdt_upload_begin(h, eo.data(), ev.data(), t1.data(), 0), "ccsdt_upload_begin");
  std::vector<double>    stage;
  std::vector<int>       tiles;
  std::vector<long long> offs;
  stage.reserve(stage_doubles);
  auto flush = [&](int kind) {
    if(offs.empty()) return;
    check(ccsdt_upload_blocks(h, kind, (long) offs.size(), tiles.data(), offs.data(), stage.data(),
                              (long long) stage.size(), 0),
          "ccsdt_upload_blocks");
    stage.clear(), tiles.clear(), offs.clear();
  };
  // one block: Tensor::get (through `fetch`), appended to the staging buffer with its four tile
  // positions
  auto add = [&](int kind, auto&& fetch, std::initializer_list<size_t> pos) {
    fetch(buf);
    if(stage.size() + buf.size() > stage_doubles) flush(kind);
    offs.push_back((long long) stage.size());
    for(size_t p: pos) tiles.push_back((int) p);
    stage.insert(stage.end(), buf.begin(), buf.end());
  };
  for(size_t A = 0; A < nva; A++)
    for(size_t B = 0; B < nva; B++)
      for(size_t I = 0; I < noa; I++)
        for(size_t J = 0; J < noa; J++) add(CCSDT_BLOCKS_T2, [&](std::vector<T>& b) { d_t2.get({A, B + nva, I, J + noa}, b); }, {A, B, I, J});
  flush(CCSDT_BLOCKS_T2);
  for(size_t I = 0; I < noa; I++)
    for(size_t J = 0; J < noa; J++)
      for(size_t A = 0; A < nva; A++)
        for(size_t B = 0; B < nva; B++) add(CCSDT_BLOCKS_OOVV, [&](std::vector<T>& b) { d_v2.v2ijab.get({I, J + noa, A, B + nva}, b); }, {I, J, A, B});
  flush(CCSDT_BLOCKS_OOVV);
  for(size_t I = 0; I < noa; I++)
    for(size_t K = 0; K < noa; K++)
      for(size_t J = 0; J < noa; J++)
        for(size_t A = 0; A < nva; A++) add(CCSDT_BLOCKS_OOOV, [&](std::vector<T>& b) { d_v2.v2ijka.get({I, K + noa, J, A + nva}, b); }, {I, K, J, A});
  flush(CCSDT_BLOCKS_OOOV);
  for(size_t I = 0; I < noa; I++)
    for(size_t B = 0; B < nva; B++)
      for(size_t A = 0; A < nva; A++)
        for(size_t C = 0; C < nva; C++) add(CCSDT_BLOCKS_OVVV, [&](std::vector<T>& b) { d_v2.v2iabc.get({I, B + nva, A, C + nva}, b); }, {I, B, A, C});
  flush(CCSDT_BLOCKS_OVVV);
  check(ccsdt_upload_end(h), "ccsdt_upload_end");
}

// Runs (T) on the spatial inputs through the C ABI: returns (E[T], E(T), device seconds).
// device -1 = the calling thread's current CUDA device.
inline std::tuple<double, double, double> run_closed_shell(const SpatialInputs& S, int device,
                                                           const ccsdt_opts& opts,
                                                           const std::vector<float>* slice_model = nullptr) {
  ccsdt_layout  L{S.o, S.v, (int) S.occ_tiles.size(), S.occ_tiles.data(), (int) S.vir_tiles.size(),
                 S.vir_tiles.data()};
  ccsdt_handle* h  = nullptr;
  ccsdt_status  st = ccsdt_create(&h, &L, device);
  if(st != CCSDT_OK) throw std::runtime_error(std::string("ccsdt_create: ") + ccsdt_status_string(st));
  st = ccsdt_upload(h, S.eps_occ.data(), S.eps_vir.data(), S.t1.data(), S.t2.data(), S.oovv.data(),
                    S.ooov.data(), S.ovvv.data(), 0);
  ccsdt_result r{};
  if(st == CCSDT_OK && slice_model) st = ccsdt_set_slice_model(h, slice_model->data());
  if(st == CCSDT_OK) st = ccsdt_energy(h, &opts, &r);
  if(st != CCSDT_OK) {
    std::string msg = ccsdt_last_error(h);
    ccsdt_destroy(h);
    throw std::runtime_error("ccsdt: " + msg);
  }
  ccsdt_destroy(h);
  return {r.e_bracket_T, r.e_paren_T, r.seconds};
}

// Spatial Cholesky vectors of the closed shell, row-major with the Cholesky index fastest.
struct CholeskyInputs {
  int                 o = 0, v = 0, nq = 0;
  std::vector<double> L_oo, L_ov, L_vv; // [o][o][nq], [o][v][nq], [v][v][nq]
};

// Reads the alpha-alpha blocks (P, Q, C) of ExaChem's Cholesky tensor cholVpr {MO, MO, CI}
// (ccsd_t.cpp:46, the tensor setupV2Tensors contracts at v2tensors.cpp:66-88) with Tensor::get.
// mo_tiles / noa / nva as for gather_closed_shell; ci_tiles: the CI space's tile extents.
template<typename T, typename TensorT>
CholeskyInputs gather_cholesky(const std::vector<size_t>& mo_tiles, size_t noa, size_t nva,
                               const std::vector<size_t>& ci_tiles, TensorT& chol) {
  if(mo_tiles.size() != 2 * noa + 2 * nva) throw std::invalid_argument("MO tiles != 2 noa + 2 nva");
  std::vector<size_t> ot(mo_tiles.begin(), mo_tiles.begin() + noa);
  std::vector<size_t> vt(mo_tiles.begin() + 2 * noa, mo_tiles.begin() + 2 * noa + nva);
  const auto   oo = detail::offsets(ot), vo = detail::offsets(vt), co = detail::offsets(ci_tiles);
  const size_t o = oo.empty() ? 0 : oo.back() + ot.back(), v = vo.empty() ? 0 : vo.back() + vt.back();
  const size_t nq = co.empty() ? 0 : co.back() + ci_tiles.back();
  CholeskyInputs L;
  L.o = (int) o, L.v = (int) v, L.nq = (int) nq;
  L.L_oo.assign(o * o * nq, 0.0);
  L.L_ov.assign(o * v * nq, 0.0);
  L.L_vv.assign(v * v * nq, 0.0);
  std::vector<T> buf;
  // one alpha-alpha block family: MO tile ids (P0 + X, Q0 + Y), rows of nr / cols of nc
  auto family = [&](std::vector<double>& dst, size_t nx, size_t ny, size_t P0, size_t Q0,
                    const std::vector<size_t>& xt, const std::vector<size_t>& yt, const std::vector<size_t>& xo,
                    const std::vector<size_t>& yo, size_t ncols) {
    for(size_t X = 0; X < nx; X++)
      for(size_t Y = 0; Y < ny; Y++)
        for(size_t C = 0; C < ci_tiles.size(); C++) {
          chol.get({P0 + X, Q0 + Y, C}, buf); // [p][q][c]
          for(size_t p = 0; p < xt[X]; p++)
            for(size_t q = 0; q < yt[Y]; q++)
              for(size_t c = 0; c < ci_tiles[C]; c++)
                dst[((xo[X] + p) * ncols + yo[Y] + q) * nq + co[C] + c] = buf[(p * yt[Y] + q) * ci_tiles[C] + c];
        }
  };
  family(L.L_oo, noa, noa, 0, 0, ot, ot, oo, oo, o);
  family(L.L_ov, noa, nva, 0, 2 * noa, ot, vt, oo, vo, v);
  family(L.L_vv, nva, nva, 2 * noa, 2 * noa, vt, vt, vo, vo, v);
  return L;
}

// (T) with the integral blocks built on the device from Cholesky vectors (ccsdt_upload_cholesky);
// the amplitudes and orbital energies come from gather_amplitudes.  Returns (E[T], E(T), device s).
// max_ovvv_slabs > 0: the Cholesky-direct mode, (ia|bc) never held whole but formed slab by slab
// into a cache of that many v^3 slabs (ccsdt_upload_cholesky_direct); 0 takes
// EXACHEM_GB300_OVVV_SLABS from the environment (unset or 0: (ia|bc) built whole).
inline std::tuple<double, double, double> run_closed_shell_cholesky(const SpatialInputs& S, const CholeskyInputs& C,
                                                                    int device, const ccsdt_opts& opts,
                                                                    int max_ovvv_slabs = 0) {
  if(max_ovvv_slabs <= 0) {
    const char* e  = std::getenv("EXACHEM_GB300_OVVV_SLABS");
    max_ovvv_slabs = e ? std::atoi(e) : 0;
  }
  if(C.o != S.o || C.v != S.v) throw std::invalid_argument("Cholesky vectors and amplitudes differ in o / v");
  ccsdt_layout  L{S.o, S.v, (int) S.occ_tiles.size(), S.occ_tiles.data(), (int) S.vir_tiles.size(),
                 S.vir_tiles.data()};
  ccsdt_handle* h  = nullptr;
  ccsdt_status  st = ccsdt_create(&h, &L, device);
  if(st != CCSDT_OK) throw std::runtime_error(std::string("ccsdt_create: ") + ccsdt_status_string(st));
  st = max_ovvv_slabs > 0
         ? ccsdt_upload_cholesky_direct(h, S.eps_occ.data(), S.eps_vir.data(), S.t1.data(), S.t2.data(), C.nq,
                                        C.L_oo.data(), C.L_ov.data(), C.L_vv.data(), 0, max_ovvv_slabs)
         : ccsdt_upload_cholesky(h, S.eps_occ.data(), S.eps_vir.data(), S.t1.data(), S.t2.data(), C.nq,
                                 C.L_oo.data(), C.L_ov.data(), C.L_vv.data(), 0);
  ccsdt_result r{};
  if(st == CCSDT_OK) st = ccsdt_energy(h, &opts, &r);
  if(st != CCSDT_OK) {
    std::string msg = ccsdt_last_error(h);
    ccsdt_destroy(h);
    throw std::runtime_error("ccsdt: " + msg);
  }
  ccsdt_destroy(h);
  return {r.e_bracket_T, r.e_paren_T, r.seconds};
}

// The whole drop-in call on ExaChem's tiled tensors: handle on the current CUDA device, inputs
// through the device-side retile, (T) for this rank's shard; returns the reference driver's tuple
// (E[T], E(T), device seconds, wall seconds since t0).
template<typename T, typename TensorT, typename V2T>
std::tuple<T, T, double, double> run_tiled(const std::vector<size_t>& mo, size_t noa, size_t nva, TensorT& d_t1,
                                           TensorT& d_t2, V2T& d_v2, const std::vector<T>& k_evl_sorted,
                                           ccsdt_opts op, std::chrono::steady_clock::time_point t0,
                                           int device = -1) {
  std::vector<int> ot, vt;
  for(size_t t = 0; t < noa; t++) ot.push_back((int) mo[t]);
  for(size_t t = 0; t < nva; t++) vt.push_back((int) mo[2 * noa + t]);
  int o = 0, v = 0;
  for(int x: ot) o += x;
  for(int x: vt) v += x;
  ccsdt_layout  L{o, v, (int) ot.size(), ot.data(), (int) vt.size(), vt.data()};
  ccsdt_handle* h  = nullptr;
  ccsdt_status  st = ccsdt_create(&h, &L, device);
  if(st != CCSDT_OK) throw std::runtime_error(std::string("ccsdt_create: ") + ccsdt_status_string(st));
  try {
    upload_tiled<T>(h, mo, noa, nva, d_t1, d_t2, d_v2, k_evl_sorted);
    std::vector<float> model;
    if(op.mode == CCSDT_MODE_LEARNED) {
      model = slice_model_from_env();
      // every rank's call is one part of the whole: it is held to its share of the budget
      op.budget_triplets = o * (o + 1) * (o + 2) / 6;
      st                 = ccsdt_set_slice_model(h, model.data());
    }
    ccsdt_result r{};
    if(st == CCSDT_OK) st = ccsdt_energy(h, &op, &r);
    if(st != CCSDT_OK) throw std::runtime_error(std::string("ccsdt: ") + ccsdt_last_error(h));
    ccsdt_destroy(h);
    const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return {(T) r.e_bracket_T, (T) r.e_paren_T, r.seconds, total};
  } catch(...) {
    ccsdt_destroy(h);
    throw;
  }
}

// ---- open shell (is_restricted = false) ----------------------------------------------------

// Dense spin-orbital arrays of ccsdt_energy_spin_orbital (include/ccsdt.h): MO order occ_a | occ_b,
// virt_a | virt_b; t1[V][O], t2[V][V][O][O], v2ijab[O][O][V][V], v2ijka[O][O][O][V], v2iabc[O][V][V][V].
struct SpinOrbitalInputs {
  int                 oa = 0, ob = 0, va = 0, vb = 0;
  std::vector<double> eps_occ, eps_vir, t1, t2, v2ijab, v2ijka, v2iabc;
};

namespace detail {
// One mode of a tiled tensor: tile extents, offsets and spins (0 alpha, 1 beta).
struct ModeTiles {
  std::vector<size_t> ext, off;
  std::vector<int>    spin;
  size_t              n = 0;
};

inline ModeTiles mode_tiles(const std::vector<size_t>& ext, size_t n_alpha_tiles) {
  ModeTiles m;
  m.ext = ext;
  m.off = offsets(ext);
  for(size_t t = 0; t < ext.size(); t++) {
    m.spin.push_back(t >= n_alpha_tiles);
    m.n += ext[t];
  }
  return m;
}

// Every block of a rank-R tensor whose spins pass `allowed` (TAMM's spin check: the spins of the
// upper indices sum to those of the lower ones) is read with Tensor::get and scattered into the
// dense row-major array `dst` over the full extents; other blocks are neither read nor stored.
template<typename T, size_t R, typename TensorT, typename F>
void gather_dense(TensorT& X, const ModeTiles* const (&modes)[R], F allowed, std::vector<double>& dst) {
  size_t total = 1;
  for(size_t m = 0; m < R; m++) total *= modes[m]->n;
  dst.assign(total, 0.0);
  std::vector<T> buf;
  size_t         bid[R] = {};
  for(;;) {
    int sp[R];
    for(size_t m = 0; m < R; m++) sp[m] = modes[m]->spin[bid[m]];
    bool empty = false;
    for(size_t m = 0; m < R; m++) empty = empty || modes[m]->ext[bid[m]] == 0;
    if(!empty && allowed(sp)) {
      static_assert(R == 2 || R == 4, "T1 / T2 / V2 tensors");
      if constexpr(R == 2) X.get({bid[0], bid[1]}, buf); // tile ids as the closed-shell gathers pass them
      else X.get({bid[0], bid[1], bid[2], bid[3]}, buf);
      // the block and dst are both row-major: copy runs along the last mode
      size_t       c[R] = {}, nb = 1;
      const size_t run = modes[R - 1]->ext[bid[R - 1]];
      for(size_t m = 0; m < R; m++) nb *= modes[m]->ext[bid[m]];
      for(size_t e = 0; e < nb; e += run) {
        size_t lin = 0;
        for(size_t m = 0; m < R; m++) lin = lin * modes[m]->n + modes[m]->off[bid[m]] + c[m];
        std::copy(buf.begin() + e, buf.begin() + e + run, dst.begin() + lin);
        for(size_t m = R - 1; m-- > 0;) {
          if(++c[m] < modes[m]->ext[bid[m]]) break;
          c[m] = 0;
        }
      }
    }
    size_t m = R;
    while(m-- > 0) {
      if(++bid[m] < modes[m]->ext.size()) break;
      bid[m] = 0;
    }
    if(m == (size_t) -1) break;
  }
}
} // namespace detail

// mo_tiles: extents of the MO tiles in the order occ_a (noa tiles), occ_b (nob), virt_a (nva),
// virt_b (nvb); k_evl_sorted in the same order.  Reads the spin-allowed blocks of the tensors the
// reference driver takes (ccsd_t_fused_driver.hpp:73-81) into the dense arrays of
// ccsdt_energy_spin_orbital.
template<typename T, typename TensorT, typename V2T>
SpinOrbitalInputs gather_spin_orbital(const std::vector<size_t>& mo_tiles, size_t noa, size_t nob, size_t nva,
                                      size_t nvb, TensorT& d_t1, TensorT& d_t2, V2T& d_v2,
                                      const std::vector<T>& k_evl_sorted) {
  if(mo_tiles.size() != noa + nob + nva + nvb) throw std::invalid_argument("MO tiles != noa + nob + nva + nvb");
  const auto Om = detail::mode_tiles({mo_tiles.begin(), mo_tiles.begin() + noa + nob}, noa);
  const auto Vm = detail::mode_tiles({mo_tiles.begin() + noa + nob, mo_tiles.end()}, nva);
  SpinOrbitalInputs S;
  for(size_t t = 0; t < noa; t++) S.oa += (int) Om.ext[t];
  for(size_t t = 0; t < nva; t++) S.va += (int) Vm.ext[t];
  S.ob = (int) Om.n - S.oa;
  S.vb = (int) Vm.n - S.va;
  if(k_evl_sorted.size() < Om.n + Vm.n) throw std::invalid_argument("k_evl_sorted too short");
  S.eps_occ.assign(k_evl_sorted.begin(), k_evl_sorted.begin() + Om.n);
  S.eps_vir.assign(k_evl_sorted.begin() + Om.n, k_evl_sorted.begin() + Om.n + Vm.n);
  const detail::ModeTiles *O = &Om, *V = &Vm;
  const detail::ModeTiles* const m_t1[2]     = {V, O};
  const detail::ModeTiles* const m_t2[4]     = {V, V, O, O};
  const detail::ModeTiles* const m_ijab[4]   = {O, O, V, V};
  const detail::ModeTiles* const m_ijka[4]   = {O, O, O, V};
  const detail::ModeTiles* const m_iabc[4]   = {O, V, V, V};
  auto                           pair_rule   = [](const int* s) { return s[0] + s[1] == s[2] + s[3]; };
  detail::gather_dense<T>(d_t1, m_t1, [](const int* s) { return s[0] == s[1]; }, S.t1);
  detail::gather_dense<T>(d_t2, m_t2, pair_rule, S.t2);
  detail::gather_dense<T>(d_v2.v2ijab, m_ijab, pair_rule, S.v2ijab);
  detail::gather_dense<T>(d_v2.v2ijka, m_ijka, pair_rule, S.v2ijka);
  detail::gather_dense<T>(d_v2.v2iabc, m_iabc, pair_rule, S.v2iabc);
  return S;
}

// (T) of a gathered open-shell system on the current device: (E[T], E(T), device seconds) of the
// triplets t % shard_count == shard_index.
inline std::tuple<double, double, double> run_spin_orbital(const SpinOrbitalInputs& S, int shard_index = 0,
                                                           int shard_count = 1) {
  double             e[2] = {0.0, 0.0}, secs = 0.0;
  const ccsdt_status st =
    ccsdt_energy_spin_orbital(S.oa, S.ob, S.va, S.vb, S.eps_occ.data(), S.eps_vir.data(), S.t1.data(),
                              S.t2.data(), S.v2ijab.data(), S.v2ijka.data(), S.v2iabc.data(), 0, shard_index,
                              shard_count, e, &secs);
  if(st != CCSDT_OK) throw std::runtime_error(std::string("ccsdt_energy_spin_orbital: ") + ccsdt_status_string(st));
  return {e[0], e[1], secs};
}

} // namespace exachem_gb300

#ifdef EXACHEM_GB300_WITH_TAMM
// Inside an ExaChem build: same namespace, class name and signature as the reference driver
// (exachem/cc/ccsd_t/ccsd_t_fused_driver.hpp:19,61-81), so the call site at ccsd_t.cpp:253-256
// compiles unchanged with this header included in place of that one.
namespace exachem::cc::ccsd_t {
template<typename T>
class CCSD_T_Fused_Driver {
public:
  virtual ~CCSD_T_Fused_Driver() = default;
  virtual std::tuple<T, T, double, double>
  execute(ChemEnv& chem_env, ExecutionContext& ec, std::vector<int>& k_spin, const TiledIndexSpace& MO,
          Tensor<T>& d_t1, Tensor<T>& d_t2, exachem::cholesky_2e::V2Tensors<T>& d_v2,
          std::vector<T>& k_evl_sorted, T hf_ccsd_energy, bool is_restricted,
          LRUCache<Index, std::vector<T>>& cache_s1t, LRUCache<Index, std::vector<T>>& cache_s1v,
          LRUCache<Index, std::vector<T>>& cache_d1t, LRUCache<Index, std::vector<T>>& cache_d1v,
          LRUCache<Index, std::vector<T>>& cache_d2t, LRUCache<Index, std::vector<T>>& cache_d2v,
          bool seq_h3b = false, bool tilesize_opt = true) {
    (void) chem_env, (void) k_spin, (void) hf_ccsd_energy, (void) cache_s1t, (void) cache_s1v;
    (void) cache_d1t, (void) cache_d1v, (void) cache_d2t, (void) cache_d2v, (void) seq_h3b, (void) tilesize_opt;
    auto                t0 = std::chrono::steady_clock::now();
    std::vector<size_t> mo;
    for(auto x: MO.input_tile_sizes()) mo.push_back((size_t) x);
    const size_t noa = MO("occ_alpha").num_tiles(), nva = MO("virt_alpha").num_tiles();
    const int    rank = (int) ec.pg().rank().value(), size = (int) ec.pg().size().value();
    if(!is_restricted) { // open shell: every spin case, FP64, this rank's share of the triplets
      const size_t nob = MO("occ_beta").num_tiles(), nvb = MO("virt_beta").num_tiles();
      auto S = exachem_gb300::gather_spin_orbital<T>(mo, noa, nob, nva, nvb, d_t1, d_t2, d_v2, k_evl_sorted);
      auto [e4, e5, secs] = exachem_gb300::run_spin_orbital(S, rank, size);
      const double total  = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      return {(T) e4, (T) e5, secs, total};
    }
    ccsdt_opts op  = exachem_gb300::opts_from_env();
    op.shard_index = rank;
    op.shard_count = size;
    return exachem_gb300::run_tiled<T>(mo, noa, nva, d_t1, d_t2, d_v2, k_evl_sorted, op, t0);
  }
};
} // namespace exachem::cc::ccsd_t
#endif
