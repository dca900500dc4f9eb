// Compiles the adapter's CCSD_T_Fused_Driver<T>::execute (the EXACHEM_GB300_WITH_TAMM path, which
// only an ExaChem build defines) against minimal stand-ins for the types of its signature
// (ccsd_t_fused_driver.hpp:73-81), with the TAMM-shaped tensor of the oracle's shim.  Compile and
// link only: the stand-ins carry just what execute() calls.
#include <cstdio>
#include <string>
#include <vector>

#include "tamm/tamm.hpp"

struct ChemEnv {};
struct ProcValue {
  int v;
  int value() const { return v; }
};
struct ProcGroup {
  ProcValue rank() const { return {0}; }
  ProcValue size() const { return {1}; }
};
struct ExecutionContext {
  ProcGroup pg() const { return {}; }
};
struct TiledIndexSpace {
  std::vector<size_t> tiles;
  size_t              n = 0;
  std::vector<size_t> input_tile_sizes() const { return tiles; }
  TiledIndexSpace     operator()(const std::string&) const { return {}; }
  size_t              num_tiles() const { return n; }
};

#define EXACHEM_GB300_WITH_TAMM 1
#include "exachem_compat/ccsd_t_fused_driver.hpp"

int main(int argc, char** argv) {
  if(argc > 1 && std::string(argv[1]) == "--opts") { // the options execute() takes from the environment
    const ccsdt_opts op = exachem_gb300::opts_from_env();
    std::printf("%d %d %.3g %d %d %d\n", op.mode, op.slices, op.energy_budget, op.autotune, op.use_graph, op.p_storage);
    return 0;
  }
  if(argc > 1) { // never run: the point is that execute() compiles and links for T = double
    exachem::cc::ccsd_t::CCSD_T_Fused_Driver<double> drv; // the reference's qualified name
    ChemEnv                                  env;
    ExecutionContext                         ec;
    std::vector<int>                         k_spin;
    TiledIndexSpace                          MO;
    tamm::Tensor<double>                     d_t1, d_t2;
    exachem::cholesky_2e::V2Tensors<double>  d_v2;
    std::vector<double>                      evl;
    LRUCache<Index, std::vector<double>>     c(0);
    for(bool restricted: {true, false})
      drv.execute(env, ec, k_spin, MO, d_t1, d_t2, d_v2, evl, 0.0, restricted, c, c, c, c, c, c);
  }
  return 0;
}
