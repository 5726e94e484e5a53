// checkpoint_model.cpp - the fixture networks of oracle/ref_cases.inc built
// through this library's C++ model API (include/spike_gb300_model.hpp), then
// saved with the same calls the reference front end is given in
// oracle/ref_dump.cpp's save mode: connectivity and weights as binary and
// text, for every synapse and for synapse group 1, and the weights read back
// from the text file and written again in binary.  Nothing here touches a
// GPU: the files come from the front end's host arrays.
//
// Usage: checkpoint_model <case> <dir>
//        checkpoint_model dump <case> <out.bin>
// The dump mode writes the synapse arrays in creation order and the label
// constants, as records (name, type, count, data) of oracle/ref_dump.cpp's
// format, for comparison with the reference front end's own arrays.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "spike_gb300_model.hpp"

namespace {
#include "../../oracle/ref_cases.inc"
}  // namespace

void put(FILE* f, const char* name, char type, const void* data, long long count) {
  const int nl = (int)strlen(name);
  fwrite(&nl, sizeof(int), 1, f);
  fwrite(name, 1, nl, f);
  fwrite(&type, 1, 1, f);
  fwrite(&count, sizeof(long long), 1, f);
  if (count > 0) fwrite(data, 4, count, f);
}

int dump(const char* c, const char* path) {
  RefCase r = build_case(c);
  if (!r.m) return 2;
  FILE* f = fopen(path, "wb");
  if (!f) return 3;
  SpikingSynapses* s = r.syn;
  const int S = s->total_number_of_synapses;
  put(f, "n_synapses", 'i', &S, 1);
  put(f, "num_syn_labels", 'i', &s->num_syn_labels, 1);
  put(f, "min_delay", 'i', &s->minimum_axonal_delay_in_timesteps, 1);
  put(f, "max_delay", 'i', &s->maximum_axonal_delay_in_timesteps, 1);
  put(f, "created_pre", 'i', s->presynaptic_neuron_indices.data(), S);
  put(f, "created_post", 'i', s->postsynaptic_neuron_indices.data(), S);
  put(f, "created_weight", 'f', s->synaptic_efficacies_or_weights.data(), S);
  put(f, "created_scale", 'f', s->weight_scaling_constants.data(), S);
  put(f, "created_delay", 'i', s->delays.data(), S);
  put(f, "created_label", 'i', s->syn_labels.data(), S);
  if (auto* cond = dynamic_cast<ConductanceSpikingSynapses*>(s)) {
    put(f, "vhat", 'f', cond->reversal_potentials_Vhat.data(), (long long)cond->reversal_potentials_Vhat.size());
    put(f, "tau_g", 'f', cond->decay_terms_tau_g.data(), (long long)cond->decay_terms_tau_g.size());
  }
  if (auto* cur = dynamic_cast<CurrentSpikingSynapses*>(s))
    put(f, "tau_syn", 'f', cur->decay_terms_tau.data(), (long long)cur->decay_terms_tau.size());
  fclose(f);
  return 0;
}

int main(int argc, char** argv) {
  if (argc == 4 && std::string(argv[1]) == "dump") return dump(argv[2], argv[3]);
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
