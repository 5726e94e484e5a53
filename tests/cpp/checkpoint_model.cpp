// checkpoint_model.cpp - the fixture networks of oracle/ref_cases.inc built
// through this library's C++ model API (include/spike_gb300_model.hpp), then
// saved with the same calls the reference front end is given in
// oracle/ref_dump.cpp's save mode: connectivity and weights as binary and
// text, for every synapse and for synapse group 1, and the weights read back
// from the text file and written again in binary.  Nothing here touches a
// GPU: the files come from the front end's host arrays.
//
// Usage: checkpoint_model <va|va_mix|brunel|shapes> <dir>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "spike_gb300_model.hpp"

namespace {
#include "../../oracle/ref_cases.inc"
}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: checkpoint_model <case> <dir>\n");
    return 2;
  }
  const std::string dir = argv[2];
  RefCase r = build_case(argv[1]);
  if (!r.m) return 2;
  SpikingSynapses* s = r.syn;
  s->save_connectivity_as_binary(dir, "all_");
  s->save_connectivity_as_txt(dir, "all_");
  s->save_weights_as_binary(dir, "w_");
  s->save_weights_as_txt(dir, "w_");
  s->save_connectivity_as_binary(dir, "g1_", 1);
  s->save_connectivity_as_txt(dir, "g1_", 1);
  s->save_weights_as_binary(dir, "g1w_", 1);
  s->load_weights_from_txt(dir + "/w_SynapticWeights.txt");
  s->save_weights_as_binary(dir, "reloaded_");
  // the binary file read back reproduces the weights bit for bit
  s->load_weights_from_binary(dir + "/w_SynapticWeights.bin");
  s->save_weights_as_binary(dir, "rebin_");
  printf("synapses %d\n", s->total_number_of_synapses);
  return 0;
}
