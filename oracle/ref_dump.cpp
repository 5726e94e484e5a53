// ref_dump.cpp - builds small networks through the REFERENCE front end
// (compiled from the reference sources by oracle/build_ref.sh, Dummy backend)
// and dumps the connectivity it produces, or the weight and connectivity files
// its save functions write, for golden fixtures.
//
// TEST INFRASTRUCTURE ONLY.  Usage: ref_dump <case> <out.bin>
//                                   ref_dump save <case> <dir>
// Cases mirror the reference examples' construction paths:
//   va      Examples/VogelsAbbottNet.cpp defaults with delay 1 step
//   va_mix  a VogelsAbbott-shaped net with rand()-drawn weights and delays
//   brunel  Examples/Brunel10K.cpp structure (connect_with_sparsity,
//           Examples/UtilityFunctions.hpp:51-82) scaled down, STDP on E->E
//   shapes  ALL_TO_ALL, ONE_TO_ONE and PAIRWISE groups (Synapses.cpp:173-307)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "Spike/Spike.hpp"

namespace {

FILE* out_file = nullptr;

void put(const char* name, char type, const void* data, long long count, int elem) {
  int nl = (int)strlen(name);
  fwrite(&nl, sizeof(int), 1, out_file);
  fwrite(name, 1, nl, out_file);
  fwrite(&type, 1, 1, out_file);
  fwrite(&count, sizeof(long long), 1, out_file);
  if (count > 0) fwrite(data, elem, count, out_file);
}
void put_i(const char* name, const int* d, long long n) { put(name, 'i', d, n, 4); }
void put_f(const char* name, const float* d, long long n) { put(name, 'f', d, n, 4); }
void put_scalar_i(const char* name, int v) { put(name, 'i', &v, 1, 4); }
void put_scalar_f(const char* name, float v) { put(name, 'f', &v, 1, 4); }

void dump_model(SpikingModel* m, SpikingSynapses* syn, SpikingNeurons* neurons,
                SpikingNeurons* inputs, STDPPlasticity* rule) {
  int S = syn->total_number_of_synapses;
  put_scalar_i("n_synapses", S);
  put_scalar_i("n_neurons", neurons->total_number_of_neurons);
  put_scalar_i("n_inputs", inputs ? inputs->total_number_of_neurons : 0);
  put_scalar_i("min_delay", syn->minimum_axonal_delay_in_timesteps);
  put_scalar_i("max_delay", syn->maximum_axonal_delay_in_timesteps);
  put_scalar_i("num_syn_labels", syn->num_syn_labels);
  put_scalar_i("timestep_grouping", m->timestep_grouping);
  put_i("sorted_pre", syn->presynaptic_neuron_indices, S);
  put_i("sorted_post", syn->postsynaptic_neuron_indices, S);
  put_f("sorted_weight", syn->synaptic_efficacies_or_weights, S);
  put_f("sorted_scale", syn->weight_scaling_constants, S);
  put_i("sorted_delay", syn->delays, S);
  put_i("sorted_label", syn->syn_labels, S);
  put_i("reversesort", syn->synapse_reversesort_indices, S);
  put_i("eff_start", neurons->per_neuron_efferent_synapse_start, neurons->total_number_of_neurons);
  put_i("eff_count", neurons->per_neuron_efferent_synapse_count, neurons->total_number_of_neurons);
  if (inputs && inputs->total_number_of_neurons > 0) {
    put_i("in_eff_start", inputs->per_neuron_efferent_synapse_start,
          inputs->total_number_of_neurons);
    put_i("in_eff_count", inputs->per_neuron_efferent_synapse_count,
          inputs->total_number_of_neurons);
  }
  auto* lifn = dynamic_cast<LIFSpikingNeurons*>(neurons);
  if (lifn) {
    put_f("tau_m", lifn->membrane_time_constants_tau_m, lifn->total_number_of_neurons);
    put_f("R", lifn->membrane_resistances_R, lifn->total_number_of_neurons);
    put_scalar_f("background_current", lifn->background_current);
    put_scalar_f("refractory", lifn->refractory_period_in_seconds);
  }
  auto* cond = dynamic_cast<ConductanceSpikingSynapses*>(syn);
  if (cond) {
    put_f("vhat", cond->reversal_potentials_Vhat.data(), cond->reversal_potentials_Vhat.size());
    put_f("tau_g", cond->decay_terms_tau_g.data(), cond->decay_terms_tau_g.size());
  }
  auto* cur = dynamic_cast<CurrentSpikingSynapses*>(syn);
  if (cur) put_f("tau_syn", cur->decay_terms_tau.data(), cur->decay_terms_tau.size());
  if (rule) put_i("plastic_sorted", rule->plastic_synapses.data(), rule->plastic_synapses.size());
}

#include "ref_cases.inc"

// Weight and connectivity files of a case as the reference's front end writes
// them (Spike/Synapses/Synapses.cpp:423-562, Spike/Synapses/SpikingSynapses.cpp:
// 136-189), for every synapse and for one synapse group, then the weights read
// back from the text file (load_weights_from_txt) and written again in binary.
int save_case(const std::string& c, const std::string& dir) {
  RefCase r = build_case(c);
  if (!r.m) return 2;
  r.m->finalise_model();
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
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc == 4 && std::string(argv[1]) == "save") return save_case(argv[2], argv[3]);
  if (argc != 3) {
    fprintf(stderr, "usage: ref_dump <va|va_mix|brunel|shapes> <out.bin> | ref_dump save <case> <dir>\n");
    return 2;
  }
  out_file = fopen(argv[2], "wb");
  if (!out_file) return 3;
  RefCase r = build_case(argv[1]);
  if (!r.m) {
    fclose(out_file);
    return 2;
  }
  r.m->finalise_model();
  dump_model(r.m, r.syn, r.neurons, r.inputs ? r.inputs : r.m->input_spiking_neurons, r.rule);
  if (std::string(argv[1]) == "brunel")
    put_f("rates", ((PoissonInputSpikingNeurons*)r.inputs)->rates, r.inputs->total_number_of_neurons);
  fclose(out_file);
  return 0;
}
