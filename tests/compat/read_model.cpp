// Reads a slice-count model file with the C++ adapter's reader and prints the parameter count
// and a checksum, for comparison with the Python loader (no GPU, no library link).
#include <cstdio>

#include "exachem_compat/ccsd_t_fused_driver.hpp"

int main(int argc, char** argv) {
  if(argc < 2) return 2;
  const std::vector<float> p = exachem_gb300::read_slice_model(argv[1]);
  double                   sum = 0, wsum = 0;
  for(size_t i = 0; i < p.size(); i++) {
    sum += p[i];
    wsum += p[i] * (double) (i % 97 + 1);
  }
  std::printf("%zu %.9e %.9e\n", p.size(), sum, wsum);
  return 0;
}
