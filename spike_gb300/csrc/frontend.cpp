// frontend.cpp - model-building front end (reference-compatible API) and its
// C surface.  Host-only code; no CUDA calls except through spike_gb300.h.
//
// Built with -ffp-contract=off: the weight and delay draws below are float
// expressions of rand() and must round exactly as the reference's x86 build
// does (Spike/Synapses/Synapses.cpp:323, Spike/Synapses/SpikingSynapses.cpp:104).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <new>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/spike_gb300.h"
#include "../../include/spike_gb300_model.h"
#include "../../include/spike_gb300_model.hpp"
#include "spk_error.h"

namespace {
struct FrontError : std::runtime_error {
  int code;
  FrontError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
[[noreturn]] void fail(int code, const std::string& msg) { throw FrontError(code, msg); }
}  // namespace

// ---- neurons ---------------------------------------------------------------------
// Neurons::AddGroup + SpikingNeurons::AddGroup (Spike/Neurons/Neurons.cpp:35-78,
// Spike/Neurons/SpikingNeurons.cpp:18-34).
int SpikingNeurons::AddGroup(neuron_parameters_struct* gp) {
  auto* sp = dynamic_cast<spiking_neuron_parameters_struct*>(gp);
  if (!sp) fail(SPK_ERR_INVALID, "neuron group parameters must derive from spiking_neuron_parameters_struct");
  number_of_neurons_in_new_group = gp->group_shape[0] * gp->group_shape[1];
  if (number_of_neurons_in_new_group < 0) fail(SPK_ERR_INVALID, "Group must have at least 1 neuron.");
  total_number_of_neurons += number_of_neurons_in_new_group;
  ++total_number_of_groups;
  int new_group_id = total_number_of_groups - 1;
  start_neuron_indices_for_each_group.push_back(total_number_of_neurons - number_of_neurons_in_new_group);
  last_neuron_indices_for_each_group.push_back(total_number_of_neurons - 1);
  group_shapes.push_back({gp->group_shape[0], gp->group_shape[1]});
  for (int i = 0; i < number_of_neurons_in_new_group; ++i) {
    per_neuron_afferent_synapse_count.push_back(0);
    per_neuron_efferent_synapse_count.push_back(0);
    after_spike_reset_potentials_vreset.push_back(sp->after_spike_reset_potential_vreset);
    resting_potentials_v0.push_back(sp->resting_potential_v0);
    thresholds_for_action_potential_spikes.push_back(sp->threshold_for_action_potential_spike);
  }
  return new_group_id;
}

void SpikingNeurons::AddEfferentSynapse(int neuron_id) {
  per_neuron_efferent_synapse_count[neuron_id]++;
  if (per_neuron_efferent_synapse_count[neuron_id] > max_num_efferent_synapses)
    max_num_efferent_synapses = per_neuron_efferent_synapse_count[neuron_id];
}

// LIFSpikingNeurons::AddGroup (Spike/Neurons/LIFSpikingNeurons.cpp:18-40).
int LIFSpikingNeurons::AddGroup(neuron_parameters_struct* gp) {
  auto* lp = dynamic_cast<lif_spiking_neuron_parameters_struct*>(gp);
  if (!lp) fail(SPK_ERR_INVALID, "LIF groups need lif_spiking_neuron_parameters_struct");
  int id = SpikingNeurons::AddGroup(gp);
  refractory_period_in_seconds = lp->absolute_refractory_period;
  float tau_m = lp->somatic_capacitance_Cm / lp->somatic_leakage_conductance_g0;
  float R = 1 / lp->somatic_leakage_conductance_g0;
  for (int i = 0; i < number_of_neurons_in_new_group; ++i) {
    membrane_time_constants_tau_m.push_back(tau_m);
    membrane_resistances_R.push_back(R);
    v_init_lo.push_back(lp->v_init_lo);
    v_init_hi.push_back(lp->v_init_hi);
  }
  background_current = lp->background_current;
  return id;
}

// InputSpikingNeurons::AddGroup (Spike/Neurons/InputSpikingNeurons.cpp:6-9).
int InputSpikingNeurons::AddGroup(neuron_parameters_struct* gp) {
  int id = SpikingNeurons::AddGroup(gp);
  return -1 * id - 1;
}

void InputSpikingNeurons::select_stimulus(int stimulus_index) {
  if (stimulus_index < total_number_of_input_stimuli)
    current_stimulus_index = stimulus_index;
  else
    fail(SPK_ERR_INVALID, "Stimulus number exceeds number of stimuli loaded");
}

// PoissonInputSpikingNeurons::AddGroup / set_up_rates
// (Spike/Neurons/PoissonInputSpikingNeurons.cpp:17-31): every input takes the
// rate of the last group added.
int PoissonInputSpikingNeurons::AddGroup(neuron_parameters_struct* gp) {
  auto* pp = dynamic_cast<poisson_input_spiking_neuron_parameters_struct*>(gp);
  if (!pp) fail(SPK_ERR_INVALID, "Poisson groups need poisson_input_spiking_neuron_parameters_struct");
  int id = InputSpikingNeurons::AddGroup(gp);
  rate = pp->rate;
  set_up_rates();
  if (total_number_of_input_stimuli < 1 && !patterned()) total_number_of_input_stimuli = 1;
  return id;
}

void PoissonInputSpikingNeurons::set_up_rates() {
  rates.assign(total_number_of_neurons, rate);
}

void PoissonInputSpikingNeurons::select_stimulus(int stimulus_index) {
  InputSpikingNeurons::select_stimulus(stimulus_index);
  if (model && model->net()) {
    int rc = spk_net_select_stimulus(model->net(), stimulus_index);
    if (rc) fail(rc, spk_last_error());
  }
}

void PatternedPoissonInputSpikingNeurons::reset_stimuli() {
  total_number_of_rates = 0;
  total_number_of_input_stimuli = 0;
  stimuli_rates.clear();
}

// PatternedPoissonInputSpikingNeurons::add_stimulus
// (Spike/Neurons/PatternedPoissonInputSpikingNeurons.cpp:36-57).
int PatternedPoissonInputSpikingNeurons::add_stimulus(const float* r, int num_rates) {
  if (num_rates != total_number_of_neurons)
    fail(SPK_ERR_INVALID, "The number of neurons does not match the number of rates!");
  stimuli_rates.insert(stimuli_rates.end(), r, r + num_rates);
  total_number_of_rates += num_rates;
  ++total_number_of_input_stimuli;
  return total_number_of_input_stimuli - 1;
}
int PatternedPoissonInputSpikingNeurons::add_stimulus(std::vector<float> r) {
  return add_stimulus(r.data(), (int)r.size());
}

// ---- synapses --------------------------------------------------------------------
// Synapses constructors seed glibc rand() (Spike/Synapses/Synapses.cpp:15-25).
SpikingSynapses::SpikingSynapses() { srand(42); }
SpikingSynapses::SpikingSynapses(int seedval) { srand(seedval); }

// Synapses::AddGroup + SpikingSynapses::AddGroup
// (Spike/Synapses/Synapses.cpp:102-388, Spike/Synapses/SpikingSynapses.cpp:62-124).
int SpikingSynapses::AddGroup(int presynaptic_group_id, int postsynaptic_group_id,
                              SpikingNeurons* neurons, SpikingNeurons* input_neurons,
                              float timestep, synapse_parameters_struct* synapse_params) {
  auto* ssp = dynamic_cast<spiking_synapse_parameters_struct*>(synapse_params);
  if (!ssp) fail(SPK_ERR_INVALID, "synapse parameters must derive from spiking_synapse_parameters_struct");
  if (!neurons) fail(SPK_ERR_INVALID, "no neuron population");
  const bool pre_is_input = PRESYNAPTIC_IS_INPUT(presynaptic_group_id);
  int prestart = 0, preend = 0, poststart = 0, postend = 0;
  std::vector<int> pre_shape, post_shape;
  if (pre_is_input) {
    if (!input_neurons) fail(SPK_ERR_INVALID, "no input population");
    int g = CORRECTED_PRESYNAPTIC_ID(presynaptic_group_id, true);
    if (g < 0 || g >= input_neurons->total_number_of_groups) fail(SPK_ERR_INVALID, "bad input group id");
    pre_shape = input_neurons->group_shapes[g];
    if (presynaptic_group_id < -1) prestart = input_neurons->start_neuron_indices_for_each_group[g];
    preend = input_neurons->last_neuron_indices_for_each_group[g] + 1;
  } else {
    int g = presynaptic_group_id;
    if (g < 0 || g >= neurons->total_number_of_groups) fail(SPK_ERR_INVALID, "bad presynaptic group id");
    pre_shape = neurons->group_shapes[g];
    if (presynaptic_group_id > 0) prestart = neurons->start_neuron_indices_for_each_group[g];
    preend = neurons->last_neuron_indices_for_each_group[g] + 1;
  }
  if (postsynaptic_group_id < 0) fail(SPK_ERR_INVALID, "Input groups cannot be a postsynaptic neuron group.");
  if (postsynaptic_group_id >= neurons->total_number_of_groups) fail(SPK_ERR_INVALID, "bad postsynaptic group id");
  post_shape = neurons->group_shapes[postsynaptic_group_id];
  poststart = neurons->start_neuron_indices_for_each_group[postsynaptic_group_id];
  postend = neurons->last_neuron_indices_for_each_group[postsynaptic_group_id] + 1;

  const int original = total_number_of_synapses;
  auto add = [&](int pre_corr, int post) {
    presynaptic_neuron_indices.push_back(pre_corr);
    postsynaptic_neuron_indices.push_back(post);
  };
  switch (synapse_params->connectivity_type) {
    case CONNECTIVITY_TYPE_ALL_TO_ALL:
      for (int i = prestart; i < preend; i++)
        for (int j = poststart; j < postend; j++) add(CORRECTED_PRESYNAPTIC_ID(i, pre_is_input), j);
      break;
    case CONNECTIVITY_TYPE_ONE_TO_ONE:
      if ((preend - prestart) != (postend - poststart)) fail(SPK_ERR_INVALID, "Unequal populations for one_to_one.");
      for (int i = 0; i < (preend - prestart); i++)
        add(CORRECTED_PRESYNAPTIC_ID(prestart + i, pre_is_input), poststart + i);
      break;
    case CONNECTIVITY_TYPE_RANDOM:
      for (int i = prestart; i < preend; i++)
        for (int j = poststart; j < postend; j++) {
          float prob = ((float)rand() / (RAND_MAX));
          if (prob < synapse_params->random_connectivity_probability)
            add(CORRECTED_PRESYNAPTIC_ID(i, pre_is_input), j);
        }
      break;
    case CONNECTIVITY_TYPE_GAUSSIAN_SAMPLE: {
      // Spike/Synapses/Synapses.cpp:230-283 (a fresh default_random_engine per synapse).
      const float sigma = synapse_params->gaussian_synapses_standard_deviation;
      const int per_pair = synapse_params->max_number_of_connections_per_pair;
      const int per_post = synapse_params->gaussian_synapses_per_postsynaptic_neuron;
      const int n_post = postend - poststart;
      const int unique = per_post * n_post;
      presynaptic_neuron_indices.resize((size_t)original + (size_t)unique * per_pair);
      postsynaptic_neuron_indices.resize((size_t)original + (size_t)unique * per_pair);
      for (int i = 0; i < unique; i++) {
        int postid = i / per_post;
        float fx = ((float)(postid % post_shape[0]) / (float)post_shape[0]);
        float fy = ((float)((float)postid / (float)post_shape[1]) / (float)post_shape[1]);
        int cx = pre_shape[0] * fx;
        int cy = pre_shape[1] * fy;
        std::default_random_engine generator;
        std::normal_distribution<float> dx((float)cx, sigma);
        std::normal_distribution<float> dy((float)cy, sigma);
        int pre_x = (int)round(dx(generator));
        while ((pre_x < 0) || (pre_x >= pre_shape[0])) pre_x = (int)(dx(generator));
        int pre_y = (int)(dy(generator));
        while ((pre_y < 0) || (pre_y >= pre_shape[1])) pre_y = (int)round(dy(generator));
        for (int n = 0; n < per_pair; n++) {
          postsynaptic_neuron_indices[original + i + n * unique] = poststart + postid;
          presynaptic_neuron_indices[original + i + n * unique] =
              CORRECTED_PRESYNAPTIC_ID(prestart + pre_x + pre_shape[1] * pre_y, pre_is_input);
        }
      }
      if (unique * per_pair > largest_synapse_group_size) largest_synapse_group_size = unique * per_pair;
      break;
    }
    case CONNECTIVITY_TYPE_PAIRWISE:
      if (synapse_params->pairwise_connect_presynaptic.size() !=
          synapse_params->pairwise_connect_postsynaptic.size())
        fail(SPK_ERR_INVALID, "Synapse pre and post vectors are not the same length!");
      for (size_t i = 0; i < synapse_params->pairwise_connect_presynaptic.size(); i++)
        add(CORRECTED_PRESYNAPTIC_ID(prestart + int(synapse_params->pairwise_connect_presynaptic[i]), pre_is_input),
            poststart + int(synapse_params->pairwise_connect_postsynaptic[i]));
      break;
    default:
      fail(SPK_ERR_INVALID, "Unknown Connection Type.");
  }
  total_number_of_synapses = (int)presynaptic_neuron_indices.size();
  temp_number_of_synapses_in_last_group = total_number_of_synapses - original;
  const int n_new = temp_number_of_synapses_in_last_group;

  // Range checks the reference leaves to undefined behaviour.
  for (int i = original; i < total_number_of_synapses; ++i) {
    int p = presynaptic_neuron_indices[i], q = postsynaptic_neuron_indices[i];
    int pc = CORRECTED_PRESYNAPTIC_ID(p, pre_is_input);
    int npre = pre_is_input ? input_neurons->total_number_of_neurons : neurons->total_number_of_neurons;
    if (pc < 0 || pc >= npre || q < 0 || q >= neurons->total_number_of_neurons)
      fail(SPK_ERR_INVALID, "synapse endpoint out of range");
  }

  // Weights, afferent/efferent counts (Spike/Synapses/Synapses.cpp:314-350).
  synaptic_efficacies_or_weights.resize(total_number_of_synapses);
  weight_scaling_constants.resize(total_number_of_synapses);
  for (int i = original; i < total_number_of_synapses; i++) {
    weight_scaling_constants[i] = synapse_params->weight_scaling_constant;
    float bottom = synapse_params->weight_range[0];
    float top = synapse_params->weight_range[1];
    float weight = bottom;
    if (top != bottom) weight = bottom + (top - bottom) * ((float)rand() / (RAND_MAX));
    synaptic_efficacies_or_weights[i] = weight;
    if (synapse_params->connectivity_type == CONNECTIVITY_TYPE_PAIRWISE) {
      if ((int)synapse_params->pairwise_connect_weight.size() == n_new)
        synaptic_efficacies_or_weights[i] = synapse_params->pairwise_connect_weight[i - original];
      else if (synapse_params->pairwise_connect_weight.size() != 0)
        fail(SPK_ERR_INVALID, "PAIRWISE CONNECTION ISSUE: Weight vector length not as expected.");
    }
    int q = postsynaptic_neuron_indices[i];
    neurons->per_neuron_afferent_synapse_count[q]++;
    if (neurons->per_neuron_afferent_synapse_count[q] > maximum_number_of_afferent_synapses)
      maximum_number_of_afferent_synapses = neurons->per_neuron_afferent_synapse_count[q];
    int pc = CORRECTED_PRESYNAPTIC_ID(presynaptic_neuron_indices[i], pre_is_input);
    if (pre_is_input)
      input_neurons->AddEfferentSynapse(pc);
    else
      neurons->AddEfferentSynapse(pc);
  }
  plastic.resize(total_number_of_synapses, 0);

  // Plasticity hookup (Spike/Synapses/Synapses.cpp:352-377).
  for (Plasticity* pl : synapse_params->plasticity_vec) {
    if (pl == nullptr) continue;
    if (pl->plasticity_rule_id < 0) {
      pl->plasticity_rule_id = (int)plasticity_rule_vec.size();
      plasticity_rule_vec.push_back(pl);
    }
    pl->AddSynapseIndices(total_number_of_synapses - n_new, n_new);
  }
  postpop_start_per_group.push_back(poststart);
  prepop_is_input.push_back(pre_is_input);
  prepop_start_per_group.push_back(prestart);
  last_index_of_synapse_per_group.push_back(total_number_of_synapses);
  const int groupID = (int)last_index_of_synapse_per_group.size() - 1;

  // Delays (Spike/Synapses/SpikingSynapses.cpp:82-118).
  int dr[2] = {int(round(ssp->delay_range[0] / timestep)), int(round(ssp->delay_range[1] / timestep))};
  if ((dr[0] < 1) || (dr[1] < 1)) fail(SPK_ERR_INVALID, "Delay range must be at least one timestep.");
  delays.resize(total_number_of_synapses);
  syn_labels.resize(total_number_of_synapses);
  for (int i = total_number_of_synapses - n_new; i < total_number_of_synapses; i++) {
    float delayval = dr[0];
    if (dr[0] != dr[1]) delayval = dr[0] + (dr[1] - dr[0]) * ((float)rand() / (RAND_MAX));
    delays[i] = round(delayval);
    syn_labels[i] = 0;
    if (ssp->connectivity_type == CONNECTIVITY_TYPE_PAIRWISE) {
      if ((int)ssp->pairwise_connect_delay.size() == n_new)
        delays[i] = (int)round(ssp->pairwise_connect_delay[i + n_new - total_number_of_synapses] / timestep);
      else if (ssp->pairwise_connect_delay.size() != 0)
        fail(SPK_ERR_INVALID, "PAIRWISE CONNECTION ISSUE: Delay vector length not as expected.");
    }
    if (delays[i] < 1) fail(SPK_ERR_INVALID, "Delay must be at least one timestep.");
    if (delays[i] > maximum_axonal_delay_in_timesteps) maximum_axonal_delay_in_timesteps = delays[i];
    if (delays[i] < minimum_axonal_delay_in_timesteps) minimum_axonal_delay_in_timesteps = delays[i];
  }
  if (neurons->total_number_of_neurons > neuron_pop_size) neuron_pop_size = neurons->total_number_of_neurons;
  return groupID;
}

// Label assignment (Spike/Synapses/ConductanceSpikingSynapses.cpp:19-75).
int ConductanceSpikingSynapses::AddGroup(int pre, int post, SpikingNeurons* n, SpikingNeurons* in,
                                         float timestep, synapse_parameters_struct* p) {
  auto* cp = dynamic_cast<conductance_spiking_synapse_parameters_struct*>(p);
  if (!cp) fail(SPK_ERR_INVALID, "conductance synapses need conductance_spiking_synapse_parameters_struct");
  int gid = SpikingSynapses::AddGroup(pre, post, n, in, timestep, p);
  if (reversal_potentials_Vhat.empty()) {
    reversal_potentials_Vhat.push_back(cp->reversal_potential_Vhat);
    decay_terms_tau_g.push_back(cp->decay_term_tau_g);
  } else {
    bool found = false;
    int indextoset = 0;
    for (size_t i = 0; i < reversal_potentials_Vhat.size(); i++)
      if (reversal_potentials_Vhat[i] == cp->reversal_potential_Vhat &&
          decay_terms_tau_g[i] == cp->decay_term_tau_g) {
        found = true;
        indextoset = (int)i;
        break;
      }
    if (!found) {
      reversal_potentials_Vhat.push_back(cp->reversal_potential_Vhat);
      decay_terms_tau_g.push_back(cp->decay_term_tau_g);
      indextoset = num_syn_labels;
      num_syn_labels++;
    }
    for (int i = total_number_of_synapses - temp_number_of_synapses_in_last_group; i < total_number_of_synapses; i++)
      syn_labels[i] = indextoset;
  }
  return gid;
}

// Label assignment (Spike/Synapses/CurrentSpikingSynapses.cpp:4-48).
int CurrentSpikingSynapses::AddGroup(int pre, int post, SpikingNeurons* n, SpikingNeurons* in,
                                     float timestep, synapse_parameters_struct* p) {
  auto* cp = dynamic_cast<current_spiking_synapse_parameters_struct*>(p);
  if (!cp) fail(SPK_ERR_INVALID, "current synapses need current_spiking_synapse_parameters_struct");
  int gid = SpikingSynapses::AddGroup(pre, post, n, in, timestep, p);
  if (decay_terms_tau.empty()) {
    decay_terms_tau.push_back(cp->decay_term_tau);
  } else {
    bool found = false;
    int indextoset = 0;
    for (size_t i = 0; i < decay_terms_tau.size(); i++)
      if (decay_terms_tau[i] == cp->decay_term_tau) {
        found = true;
        indextoset = (int)i;
        break;
      }
    if (!found) {
      decay_terms_tau.push_back(cp->decay_term_tau);
      indextoset = num_syn_labels;
      num_syn_labels++;
    }
    for (int i = total_number_of_synapses - temp_number_of_synapses_in_last_group; i < total_number_of_synapses; i++)
      syn_labels[i] = indextoset;
  }
  return gid;
}

void SpikingSynapses::group_range(int synapsegroupid, int& startid, int& endid) const {
  startid = 0;
  endid = total_number_of_synapses;
  if (synapsegroupid >= 0) endid = last_index_of_synapse_per_group[synapsegroupid];
  if ((synapsegroupid > 0) && (synapsegroupid < (int)last_index_of_synapse_per_group.size()))
    startid = last_index_of_synapse_per_group[synapsegroupid - 1];
}

void SpikingSynapses::copy_weights_to_host() {
  if (!model || !model->net()) return;
  int rc = spk_net_read_weights(model->net(), synaptic_efficacies_or_weights.data(),
                                (int64_t)synaptic_efficacies_or_weights.size());
  if (rc) fail(rc, spk_last_error());
}

// save_weights_as_binary / _txt (Spike/Synapses/Synapses.cpp:525-562): creation order.
void SpikingSynapses::save_weights_as_binary(std::string path, std::string prefix, int gid) {
  copy_weights_to_host();
  int a, b;
  group_range(gid, a, b);
  std::ofstream f(path + "/" + prefix + "SynapticWeights.bin", std::ios::out | std::ios::binary);
  for (int i = a; i < b; i++) f.write((const char*)&synaptic_efficacies_or_weights[i], sizeof(float));
}
void SpikingSynapses::save_weights_as_txt(std::string path, std::string prefix, int gid) {
  copy_weights_to_host();
  int a, b;
  group_range(gid, a, b);
  std::ofstream f(path + "/" + prefix + "SynapticWeights.txt", std::ios::out | std::ios::binary);
  for (int i = a; i < b; i++) f << synaptic_efficacies_or_weights[i] << std::endl;
}
// load_weights (Spike/Synapses/Synapses.cpp:565-584).
void SpikingSynapses::load_weights(std::vector<float> weights, int gid) {
  int a, b;
  group_range(gid, a, b);
  if ((int)weights.size() != b - a) fail(SPK_ERR_INVALID, "Number of weights loading not equal to number of synapses!!");
  copy_weights_to_host();
  for (int i = a; i < b; i++) synaptic_efficacies_or_weights[i] = weights[i - a];
  if (model && model->net()) {
    int rc = spk_net_write_weights(model->net(), synaptic_efficacies_or_weights.data(),
                                   (int64_t)synaptic_efficacies_or_weights.size());
    if (rc) fail(rc, spk_last_error());
  }
}
// load_weights_from_txt / _binary (Spike/Synapses/Synapses.cpp:586-614): every
// value the stream yields (text: operator>> on float; binary: native 4-byte
// floats) in file order, then load_weights.
void SpikingSynapses::load_weights_from_txt(std::string filepath, int gid) {
  std::ifstream f(filepath, std::ios::in | std::ios::binary);
  std::vector<float> w;
  float v = 0.0f;
  while (f >> v) w.push_back(v);
  load_weights(w, gid);
}
void SpikingSynapses::load_weights_from_binary(std::string filepath, int gid) {
  std::ifstream f(filepath, std::ios::in | std::ios::binary);
  std::vector<float> w;
  float v = 0.0f;
  while (f.read(reinterpret_cast<char*>(&v), sizeof(float))) w.push_back(v);
  load_weights(w, gid);
}
// save_connectivity_as_* (Spike/Synapses/Synapses.cpp:423-519,
// Spike/Synapses/SpikingSynapses.cpp:136-189).
void SpikingSynapses::save_connectivity_as_binary(std::string path, std::string prefix, int gid) {
  copy_weights_to_host();
  int a, b;
  group_range(gid, a, b);
  int prec = 0, postc = 0;
  bool in = false;
  if (gid >= 0) {
    postc = postpop_start_per_group[gid];
    prec = prepop_start_per_group[gid];
    in = prepop_is_input[gid];
  }
  std::ofstream pf(path + "/" + prefix + "PresynapticIDs.bin", std::ios::binary);
  std::ofstream qf(path + "/" + prefix + "PostsynapticIDs.bin", std::ios::binary);
  std::ofstream wf(path + "/" + prefix + "SynapticWeights.bin", std::ios::binary);
  std::ofstream df(path + "/" + prefix + "SynapticDelays.bin", std::ios::binary);
  for (int i = a; i < b; i++) {
    int pre = gid >= 0 ? CORRECTED_PRESYNAPTIC_ID(presynaptic_neuron_indices[i], in) - prec
                       : presynaptic_neuron_indices[i];
    int post = postsynaptic_neuron_indices[i] - postc;
    pf.write((const char*)&pre, sizeof(int));
    qf.write((const char*)&post, sizeof(int));
    wf.write((const char*)&synaptic_efficacies_or_weights[i], sizeof(float));
    df.write((const char*)&delays[i], sizeof(int));
  }
}
void SpikingSynapses::save_connectivity_as_txt(std::string path, std::string prefix, int gid) {
  copy_weights_to_host();
  int a, b;
  group_range(gid, a, b);
  int prec = 0, postc = 0;
  bool in = false;
  if (gid >= 0) {
    postc = postpop_start_per_group[gid];
    prec = prepop_start_per_group[gid];
    in = prepop_is_input[gid];
  }
  std::ofstream pf(path + "/" + prefix + "PresynapticIDs.txt", std::ios::binary);
  std::ofstream qf(path + "/" + prefix + "PostsynapticIDs.txt", std::ios::binary);
  std::ofstream wf(path + "/" + prefix + "SynapticWeights.txt", std::ios::binary);
  std::ofstream df(path + "/" + prefix + "SynapticDelays.txt", std::ios::binary);
  for (int i = a; i < b; i++) {
    if (gid >= 0)
      pf << CORRECTED_PRESYNAPTIC_ID(presynaptic_neuron_indices[i], in) - prec << std::endl;
    else
      pf << presynaptic_neuron_indices[i];
    qf << postsynaptic_neuron_indices[i] - postc << std::endl;
    wf << synaptic_efficacies_or_weights[i] << std::endl;
    df << delays[i] << std::endl;
  }
}

// ---- plasticity -------------------------------------------------------------------
void Plasticity::AddSynapseIndices(int start, int n) {
  for (int id = start; id < start + n; id++) plastic_synapses.push_back(id);
}

WeightDependentSTDPPlasticity::WeightDependentSTDPPlasticity(SpikingSynapses*, SpikingNeurons*,
                                                             SpikingNeurons*,
                                                             stdp_plasticity_parameters_struct* p) {
  stdp_params = dynamic_cast<weightdependent_stdp_plasticity_parameters_struct*>(p);
  if (!stdp_params) fail(SPK_ERR_INVALID, "weight-dependent STDP needs its parameter struct");
}

EvansSTDPPlasticity::EvansSTDPPlasticity(SpikingSynapses*, SpikingNeurons*, SpikingNeurons*,
                                         stdp_plasticity_parameters_struct* p) {
  stdp_params = dynamic_cast<evans_stdp_plasticity_parameters_struct*>(p);
  if (!stdp_params) fail(SPK_ERR_INVALID, "Evans STDP needs its parameter struct");
}

InhibitorySTDPPlasticity::InhibitorySTDPPlasticity(SpikingSynapses*, SpikingNeurons*, SpikingNeurons*,
                                                   stdp_plasticity_parameters_struct* p) {
  stdp_params = dynamic_cast<inhibitory_stdp_plasticity_parameters_struct*>(p);
  if (!stdp_params) fail(SPK_ERR_INVALID, "inhibitory STDP needs its parameter struct");
}

WeightNormSTDPPlasticity::WeightNormSTDPPlasticity(SpikingSynapses*, SpikingNeurons*, SpikingNeurons*,
                                                   stdp_plasticity_parameters_struct* p) {
  plasticity_parameters = dynamic_cast<weightnorm_stdp_plasticity_parameters_struct*>(p);
  if (!plasticity_parameters) fail(SPK_ERR_INVALID, "weight normalisation needs its parameter struct");
}

CustomSTDPPlasticity::CustomSTDPPlasticity(SpikingSynapses*, SpikingNeurons*, SpikingNeurons*,
                                           stdp_plasticity_parameters_struct* p) {
  stdp_params = dynamic_cast<custom_stdp_plasticity_parameters_struct*>(p);
  if (!stdp_params) fail(SPK_ERR_INVALID, "custom STDP needs its parameter struct");
}

// ---- monitor ------------------------------------------------------------------------
void SpikingActivityMonitor::reset_state() {
  neuron_ids_of_stored_spikes_on_host.clear();
  spike_times_of_stored_spikes_on_host.clear();
  total_number_of_spikes_stored_on_host = 0;
}
// save_spikes_as_txt / _binary (Spike/ActivityMonitor/SpikingActivityMonitor.cpp:123-153).
void SpikingActivityMonitor::save_spikes_as_txt(std::string path, std::string prefix) {
  std::ofstream idf(path + "/" + prefix + "SpikeIDs.txt", std::ios::binary);
  std::ofstream tf(path + "/" + prefix + "SpikeTimes.txt", std::ios::binary);
  for (int i = 0; i < total_number_of_spikes_stored_on_host; i++) {
    idf << neuron_ids_of_stored_spikes_on_host[i] << std::endl;
    tf << spike_times_of_stored_spikes_on_host[i] << std::endl;
  }
}
void SpikingActivityMonitor::save_spikes_as_binary(std::string path, std::string prefix) {
  std::ofstream idf(path + "/" + prefix + "SpikeIDs.bin", std::ios::binary);
  std::ofstream tf(path + "/" + prefix + "SpikeTimes.bin", std::ios::binary);
  idf.write((const char*)neuron_ids_of_stored_spikes_on_host.data(),
            sizeof(int) * total_number_of_spikes_stored_on_host);
  tf.write((const char*)spike_times_of_stored_spikes_on_host.data(),
           sizeof(float) * total_number_of_spikes_stored_on_host);
}

// RateActivityMonitor::reset_state (Spike/ActivityMonitor/RateActivityMonitor.cpp:17-22
// with Spike/Backend/CUDA/ActivityMonitor/RateActivityMonitor.cu:12-16).
void RateActivityMonitor::reset_state() {
  std::fill(per_neuron_spike_counts.begin(), per_neuron_spike_counts.end(), 0);
  if (model && model->net()) spk_net_clear_rate_counts(model->net());
}

// ---- model --------------------------------------------------------------------------
SpikingModel::SpikingModel() {}
SpikingModel::~SpikingModel() {
  if (net_) spk_net_destroy(net_);
}

void SpikingModel::SetTimestep(float ts) {
  if (spiking_synapses && spiking_synapses->total_number_of_synapses > 0)
    fail(SPK_ERR_STATE, "You must set the timestep before creating any synapses.");
  timestep = ts;
}
int SpikingModel::AddNeuronGroup(neuron_parameters_struct* p) {
  if (!spiking_neurons) fail(SPK_ERR_STATE, "Please set neurons pointer before adding neuron groups.");
  return spiking_neurons->AddGroup(p);
}
int SpikingModel::AddInputNeuronGroup(neuron_parameters_struct* p) {
  if (!input_spiking_neurons) fail(SPK_ERR_STATE, "Please set input_neurons pointer before adding inputs groups.");
  return input_spiking_neurons->AddGroup(p);
}
int SpikingModel::AddSynapseGroup(int pre, int post, synapse_parameters_struct* p) {
  if (!spiking_synapses) fail(SPK_ERR_STATE, "Please set synapse pointer before adding synapses.");
  return spiking_synapses->AddGroup(pre, post, spiking_neurons, input_spiking_neurons, timestep, p);
}
void SpikingModel::AddSynapseGroupsForNeuronGroupAndEachInputGroup(int post, synapse_parameters_struct* p) {
  for (int i = 0; i < input_spiking_neurons->total_number_of_groups; i++)
    AddSynapseGroup(CORRECTED_PRESYNAPTIC_ID(i, true), post, p);
}
void SpikingModel::AddPlasticityRule(Plasticity* r) { plasticity_rule_vec.push_back(r); }
void SpikingModel::AddActivityMonitor(SpikingActivityMonitor* m) {
  m->model = this;
  monitors_vec.push_back(m);
}
void SpikingModel::AddActivityMonitor(RateActivityMonitor* m) {
  m->model = this;
  rate_monitors_vec.push_back(m);
}

int SpikingModel::build_desc(spk_net_desc* d) {
  if (!spiking_neurons || spiking_neurons->total_number_of_neurons <= 0) return SPK_ERR_INVALID;
  if (!spiking_synapses) return SPK_ERR_INVALID;
  auto* lifn = dynamic_cast<LIFSpikingNeurons*>(spiking_neurons);
  if (!lifn) return SPK_ERR_UNSUPPORTED;
  std::memset(d, 0, sizeof(*d));
  d->abi_version = SPK_ABI_VERSION;
  d->dt = timestep;
  d->synapse_kind = spiking_synapses->kind();
  d->n_neurons = lifn->total_number_of_neurons;
  groups_.clear();
  for (int g = 0; g < lifn->total_number_of_groups; ++g) {
    spk_neuron_group G{};
    G.start = lifn->start_neuron_indices_for_each_group[g];
    G.count = lifn->last_neuron_indices_for_each_group[g] - G.start + 1;
    if (G.count <= 0) continue;
    G.tau_m = lifn->membrane_time_constants_tau_m[G.start];
    G.R = lifn->membrane_resistances_R[G.start];
    G.v0 = lifn->resting_potentials_v0[G.start];
    G.vreset = lifn->after_spike_reset_potentials_vreset[G.start];
    G.theta = lifn->thresholds_for_action_potential_spikes[G.start];
    G.v_init_lo = lifn->v_init_lo[G.start];
    G.v_init_hi = lifn->v_init_hi[G.start];
    groups_.push_back(G);
  }
  d->n_groups = (int32_t)groups_.size();
  d->groups = groups_.data();
  d->refractory_period = lifn->refractory_period_in_seconds;
  d->background_current = lifn->background_current;
  auto* pin = dynamic_cast<PoissonInputSpikingNeurons*>(input_spiking_neurons);
  if (input_spiking_neurons && input_spiking_neurons->total_number_of_neurons > 0) {
    if (!pin) return SPK_ERR_UNSUPPORTED;
    d->n_inputs = pin->total_number_of_neurons;
    if (pin->patterned()) {
      auto* pp = static_cast<PatternedPoissonInputSpikingNeurons*>(pin);
      if (pp->total_number_of_input_stimuli < 1) return SPK_ERR_INVALID;
      d->n_stimuli = pp->total_number_of_input_stimuli;
      d->input_rates = pp->stimuli_rates.data();
    } else {
      rates_ = pin->rates;  // every input has the last group's rate
      d->n_stimuli = 1;
      d->input_rates = rates_.data();
    }
    d->stimulus = pin->current_stimulus_index;
  }
  SpikingSynapses* s = spiking_synapses;
  d->n_labels = s->num_syn_labels;
  label_tau_.clear();
  label_vhat_.clear();
  if (auto* c = dynamic_cast<ConductanceSpikingSynapses*>(s)) {
    label_tau_ = c->decay_terms_tau_g;
    label_vhat_ = c->reversal_potentials_Vhat;
  } else if (auto* c2 = dynamic_cast<CurrentSpikingSynapses*>(s)) {
    label_tau_ = c2->decay_terms_tau;
  }
  if (label_tau_.empty()) label_tau_.assign(d->n_labels, 1.0f);
  if (label_vhat_.empty()) label_vhat_.assign(d->n_labels, 0.0f);
  d->label_tau = label_tau_.data();
  d->label_vhat = label_vhat_.data();
  d->n_synapses = s->total_number_of_synapses;
  d->pre = s->presynaptic_neuron_indices.data();
  d->post = s->postsynaptic_neuron_indices.data();
  d->weight = s->synaptic_efficacies_or_weights.data();
  d->scale = s->weight_scaling_constants.data();
  d->delay = s->delays.data();
  d->label = s->syn_labels.data();
  // Plastic synapses: those attached to a rule that the model runs
  // (SpikingModel::perform_per_step_model_instructions iterates the model's
  // rule vector, Spike/Models/SpikingModel.cpp:202-205).
  std::fill(s->plastic.begin(), s->plastic.end(), 0);
  int n_rules = 0;
  const weightdependent_stdp_plasticity_parameters_struct* wp = nullptr;
  const WeightNormSTDPPlasticity* norm = nullptr;
  bool norm_first = false;
  d->stdp_rule = SPK_STDP_WEIGHT_DEPENDENT;
  std::memset(&d->stdp, 0, sizeof(d->stdp));
  for (Plasticity* r : plasticity_rule_vec) {
    if (auto* wn = dynamic_cast<WeightNormSTDPPlasticity*>(r)) {
      if (norm) return SPK_ERR_UNSUPPORTED;  // one normalisation per model
      norm = wn;
      norm_first = n_rules == 0;
      continue;
    }
    ++n_rules;
    if (auto* wd = dynamic_cast<WeightDependentSTDPPlasticity*>(r)) {
      wp = wd->stdp_params;
    } else if (auto* ev = dynamic_cast<EvansSTDPPlasticity*>(r)) {
      // the descriptor's field mapping for SPK_STDP_EVANS
      d->stdp_rule = SPK_STDP_EVANS;
      d->stdp.tau_minus = ev->stdp_params->decay_term_tau_D;
      d->stdp.tau_plus = ev->stdp_params->decay_term_tau_C;
      d->stdp.a_minus = ev->stdp_params->model_parameter_alpha_D;
      d->stdp.a_plus = ev->stdp_params->synaptic_neurotransmitter_concentration_alpha_C;
      d->stdp.w_max = 1.0f;
    } else if (auto* ih = dynamic_cast<InhibitorySTDPPlasticity*>(r)) {
      d->stdp_rule = SPK_STDP_INHIBITORY;
      d->stdp.tau_plus = ih->stdp_params->tau_istdp;
      d->stdp.tau_minus = ih->stdp_params->tau_istdp;
      d->stdp.lambda = ih->stdp_params->learningrate;
      d->stdp.alpha = ih->stdp_params->targetrate;
      d->stdp.w_max = 1.0f;
    } else if (auto* cu = dynamic_cast<CustomSTDPPlasticity*>(r)) {
      d->stdp_rule = SPK_STDP_CUSTOM;
      d->stdp.a_minus = cu->stdp_params->a_minus;
      d->stdp.a_plus = cu->stdp_params->a_plus;
      d->stdp.tau_minus = cu->stdp_params->tau_minus;
      d->stdp.tau_plus = cu->stdp_params->tau_plus;
      d->stdp.w_max = cu->stdp_params->w_max;
      d->stdp.lambda = cu->stdp_params->learning_rate;
      d->stdp.alpha = cu->stdp_params->a_star;
      d->stdp.clip_upper = cu->stdp_params->nearest_spike_only ? 1 : 0;
    } else {
      return SPK_ERR_UNSUPPORTED;
    }
    for (int idx : r->plastic_synapses) s->plastic[idx] = 1;
  }
  if (n_rules > 1) return SPK_ERR_UNSUPPORTED;
  d->plastic = s->plastic.data();
  d->has_stdp = n_rules == 1;
  if (wp) {
    d->stdp.a_minus = wp->a_minus;
    d->stdp.a_plus = wp->a_plus;
    d->stdp.tau_minus = wp->tau_minus;
    d->stdp.tau_plus = wp->tau_plus;
    d->stdp.lambda = wp->lambda;
    d->stdp.alpha = wp->alpha;
    d->stdp.w_max = wp->w_max;
    d->stdp.clip_upper = wp->clip_upper ? 1 : 0;
  }
  d->weight_norm = SPK_NORM_OFF;
  d->norm_initial = nullptr;
  d->norm_sum = nullptr;
  if (norm) {
    // Supported on the STDP rule's own synapses.
    if (n_rules != 1) return SPK_ERR_UNSUPPORTED;
    std::vector<uint8_t> in_norm(s->plastic.size(), 0);
    for (int idx : norm->plastic_synapses) in_norm[idx] = 1;
    if (in_norm != s->plastic) return SPK_ERR_UNSUPPORTED;
    d->weight_norm = norm_first ? SPK_NORM_BEFORE_RULE : SPK_NORM_AFTER_RULE;
    const weightnorm_stdp_plasticity_parameters_struct* np = norm->plasticity_parameters;
    if (np->settarget) {
      // WeightNormSTDPPlasticity::prepare_backend_early
      // (Spike/Plasticity/WeightNormSTDPPlasticity.cpp:31-70) with a target:
      // the host weights are rescaled to w / sqrt(S) * target and S := target,
      // after the synapses' backend has copied the unscaled weights to the
      // device (SpikingModel::init_backend prepares the synapses first,
      // Spike/Models/SpikingModel.cpp:148-153); reset_state then takes the
      // rescaled host weights as the initial weights
      // (Spike/Plasticity/WeightNormSTDPPlasticity.cpp:23-29).  So the run
      // starts from the unscaled weights, measured against the rescaled ones.
      const int N = d->n_neurons;
      std::vector<float> sum(N, 0.0f);
      for (int idx : norm->plastic_synapses) sum[s->postsynaptic_neuron_indices[idx]] += powf(s->synaptic_efficacies_or_weights[idx], 2.0f);
      norm_initial_ = s->synaptic_efficacies_or_weights;
      for (int idx : norm->plastic_synapses) {
        float w = s->synaptic_efficacies_or_weights[idx];
        w /= sqrtf(sum[s->postsynaptic_neuron_indices[idx]]);
        w *= np->target;
        norm_initial_[idx] = w;
      }
      norm_sum_.assign(N, np->target);
      d->norm_initial = norm_initial_.data();
      d->norm_sum = norm_sum_.data();
    }
  }
  d->seed = philox_seed;
  d->spike_capacity = spike_capacity;
  d->record_inputs = 0;
  for (auto* m : monitors_vec)
    if (m->neurons == input_spiking_neurons && input_spiking_neurons) d->record_inputs = 1;
  return SPK_OK;
}

void SpikingModel::finalise_model() {
  if (model_complete) return;
  if (spiking_synapses) spiking_synapses->model = this;
  if (spiking_neurons) spiking_neurons->model = this;
  if (input_spiking_neurons) input_spiking_neurons->model = this;
  for (auto* m : monitors_vec) m->model = this;
  for (auto* m : rate_monitors_vec) m->model = this;
  spk_net_desc d;
  int rc = build_desc(&d);
  if (rc) fail(rc, "model cannot be flattened into a network descriptor");
  const spk_schedule* sp = (schedule.warps_per_cta || schedule.tile_posts || schedule.ctas ||
                            schedule.steps_per_launch)
                               ? &schedule
                               : nullptr;
  rc = spk_net_create(&d, sp, &net_);
  if (rc) fail(rc, spk_last_error());
  // timestep_grouping = the minimum delay (Spike/Models/SpikingModel.cpp:98)
  int32_t G = 1;
  spk_net_timestep_grouping(net_, &G);
  timestep_grouping = G;
  model_complete = true;
}

void SpikingModel::reset_state() {
  finalise_model();
  int rc = spk_net_reset_state(net_);  // zeroes the device rate counts too
  if (rc) fail(rc, spk_last_error());
  for (auto* m : rate_monitors_vec) std::fill(m->per_neuron_spike_counts.begin(), m->per_neuron_spike_counts.end(), 0);
}
void SpikingModel::reset_time() {
  if (net_) spk_net_reset_time(net_);
}

void SpikingModel::collect_spikes() {
  for (auto* m : monitors_vec) {
    int pop = (m->neurons == input_spiking_neurons && input_spiking_neurons) ? SPK_POP_INPUTS
                                                                             : SPK_POP_NEURONS;
    int64_t n = 0;
    int rc = spk_net_spike_count(net_, pop, &n);
    if (rc) fail(rc, spk_last_error());
    size_t base = m->neuron_ids_of_stored_spikes_on_host.size();
    m->neuron_ids_of_stored_spikes_on_host.resize(base + n);
    m->spike_times_of_stored_spikes_on_host.resize(base + n);
    int64_t got = 0;
    rc = spk_net_read_spikes(net_, pop, m->neuron_ids_of_stored_spikes_on_host.data() + base,
                             m->spike_times_of_stored_spikes_on_host.data() + base, n, &got);
    if (rc) fail(rc, spk_last_error());
    m->total_number_of_spikes_stored_on_host = (int)(base + got);
  }
  spk_net_clear_spikes(net_);
}

// RateActivityMonitor::final_update (Spike/ActivityMonitor/RateActivityMonitor.cpp:28-30):
// the device counts since the last reset, copied to each rate monitor.
void SpikingModel::collect_rates() {
  for (auto* m : rate_monitors_vec) {
    const bool inputs = m->neurons == input_spiking_neurons && input_spiking_neurons;
    const int n = inputs ? input_spiking_neurons->total_number_of_neurons : spiking_neurons->total_number_of_neurons;
    m->per_neuron_spike_counts.assign(n, 0);
    int rc = spk_net_rate_counts(net_, inputs ? SPK_POP_INPUTS : SPK_POP_NEURONS, m->per_neuron_spike_counts.data(), n);
    if (rc) fail(rc, spk_last_error());
  }
}

// SpikingModel::run (Spike/Models/SpikingModel.cpp:214-236); the monitors'
// device store is drained after the run (final_update).
void SpikingModel::run(float seconds, bool plasticity_on) {
  finalise_model();
  status_ = spk_net_run(net_, seconds, plasticity_on ? 1 : 0);
  if (status_ == SPK_OK) status_ = spk_net_synchronize(net_);
  if (status_ != SPK_OK && status_ != SPK_ERR_OVERFLOW) fail(status_, spk_last_error());
  collect_spikes();
  collect_rates();
}

// ---- C surface -------------------------------------------------------------------------
struct spk_model {
  SpikingModel model;
  LIFSpikingNeurons neurons;
  PoissonInputSpikingNeurons* inputs = nullptr;
  SpikingSynapses* synapses = nullptr;
  std::vector<Plasticity*> rules;
  std::vector<stdp_plasticity_parameters_struct*> rule_params;
  SpikingActivityMonitor* neuron_monitor = nullptr;
  SpikingActivityMonitor* input_monitor = nullptr;
  RateActivityMonitor* rate_monitor[2] = {nullptr, nullptr};  // neurons, inputs
  ~spk_model() {
    for (auto* r : rules) delete r;
    for (auto* p : rule_params) delete p;
    delete neuron_monitor;
    delete input_monitor;
    delete rate_monitor[0];
    delete rate_monitor[1];
    delete synapses;
    delete inputs;
  }
};

namespace {
template <typename F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const FrontError& e) {
    spk::set_error("%s", e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    spk::set_error("host allocation failed");
    return SPK_ERR_OOM;
  } catch (const std::exception& e) {
    spk::set_error("%s", e.what());
    return SPK_ERR_INVALID;
  }
}

void fill_synapse_params(const spk_synapse_params* p, spiking_synapse_parameters_struct* s,
                         spk_model* m) {
  s->connectivity_type = p->connectivity_type;
  s->weight_range[0] = p->weight_range[0];
  s->weight_range[1] = p->weight_range[1];
  s->weight_scaling_constant = p->weight_scaling_constant;
  s->random_connectivity_probability = p->random_connectivity_probability;
  s->delay_range[0] = p->delay_range[0];
  s->delay_range[1] = p->delay_range[1];
  s->max_number_of_connections_per_pair = p->max_number_of_connections_per_pair;
  s->gaussian_synapses_per_postsynaptic_neuron = p->gaussian_synapses_per_postsynaptic_neuron;
  s->gaussian_synapses_standard_deviation = p->gaussian_synapses_standard_deviation;
  if (p->n_pairwise > 0) {
    s->pairwise_connect_presynaptic.assign(p->pairwise_connect_presynaptic,
                                           p->pairwise_connect_presynaptic + p->n_pairwise);
    s->pairwise_connect_postsynaptic.assign(p->pairwise_connect_postsynaptic,
                                            p->pairwise_connect_postsynaptic + p->n_pairwise);
    if (p->pairwise_connect_weight)
      s->pairwise_connect_weight.assign(p->pairwise_connect_weight,
                                        p->pairwise_connect_weight + p->n_pairwise);
    if (p->pairwise_connect_delay)
      s->pairwise_connect_delay.assign(p->pairwise_connect_delay,
                                       p->pairwise_connect_delay + p->n_pairwise);
  }
  for (int rid : {p->plasticity_rule, p->plasticity_rule_2}) {
    if (rid < 0) continue;
    if (rid >= (int)m->rules.size()) fail(SPK_ERR_INVALID, "unknown plasticity rule");
    s->plasticity_vec.push_back(m->rules[rid]);
  }
}

int add_group_with(spk_model* m, int32_t pre, int32_t post, const spk_synapse_params* p,
                   const std::vector<int>* pw_pre, const std::vector<int>* pw_post) {
  int kind = m->synapses->kind();
  int gid;
  if (kind == SPK_SYN_CONDUCTANCE) {
    conductance_spiking_synapse_parameters_struct s;
    fill_synapse_params(p, &s, m);
    s.reversal_potential_Vhat = p->reversal_potential_Vhat;
    s.decay_term_tau_g = p->decay_term_tau_g;
    if (pw_pre) {
      s.pairwise_connect_presynaptic = *pw_pre;
      s.pairwise_connect_postsynaptic = *pw_post;
      s.connectivity_type = CONNECTIVITY_TYPE_PAIRWISE;
    }
    gid = m->model.AddSynapseGroup(pre, post, &s);
  } else if (kind == SPK_SYN_CURRENT) {
    current_spiking_synapse_parameters_struct s;
    fill_synapse_params(p, &s, m);
    s.decay_term_tau = p->decay_term_tau;
    if (pw_pre) {
      s.pairwise_connect_presynaptic = *pw_pre;
      s.pairwise_connect_postsynaptic = *pw_post;
      s.connectivity_type = CONNECTIVITY_TYPE_PAIRWISE;
    }
    gid = m->model.AddSynapseGroup(pre, post, &s);
  } else {
    voltage_spiking_synapse_parameters_struct s;
    fill_synapse_params(p, &s, m);
    if (pw_pre) {
      s.pairwise_connect_presynaptic = *pw_pre;
      s.pairwise_connect_postsynaptic = *pw_post;
      s.connectivity_type = CONNECTIVITY_TYPE_PAIRWISE;
    }
    gid = m->model.AddSynapseGroup(pre, post, &s);
  }
  return gid;
}
}  // namespace

extern "C" {

int spk_model_create(int32_t synapse_kind, int32_t input_kind, int32_t synapse_seed, spk_model** out) {
  if (!out) return SPK_ERR_INVALID;
  return guarded([&] {
    auto* m = new spk_model();
    if (synapse_kind == SPK_SYN_CONDUCTANCE)
      m->synapses = synapse_seed < 0 ? new ConductanceSpikingSynapses() : new ConductanceSpikingSynapses(synapse_seed);
    else if (synapse_kind == SPK_SYN_CURRENT)
      m->synapses = synapse_seed < 0 ? new CurrentSpikingSynapses() : new CurrentSpikingSynapses(synapse_seed);
    else if (synapse_kind == SPK_SYN_VOLTAGE)
      m->synapses = synapse_seed < 0 ? new VoltageSpikingSynapses() : new VoltageSpikingSynapses(synapse_seed);
    else {
      delete m;
      fail(SPK_ERR_INVALID, "unknown synapse kind");
    }
    if (input_kind == SPK_INPUT_POISSON)
      m->inputs = new PoissonInputSpikingNeurons();
    else if (input_kind == SPK_INPUT_PATTERNED)
      m->inputs = new PatternedPoissonInputSpikingNeurons();
    else if (input_kind != SPK_INPUT_NONE) {
      delete m;
      fail(SPK_ERR_INVALID, "unknown input kind");
    }
    m->model.spiking_neurons = &m->neurons;
    m->model.spiking_synapses = m->synapses;
    m->model.input_spiking_neurons = m->inputs;
    m->neuron_monitor = new SpikingActivityMonitor(&m->neurons);
    m->model.AddActivityMonitor(m->neuron_monitor);
    *out = m;
    return SPK_OK;
  });
}

int spk_model_destroy(spk_model* m) {
  if (!m) return SPK_ERR_INVALID;
  delete m;
  return SPK_OK;
}

int spk_model_set_timestep(spk_model* m, float dt) {
  if (!m || !(dt > 0.0f)) return SPK_ERR_INVALID;
  return guarded([&] {
    m->model.SetTimestep(dt);
    return SPK_OK;
  });
}

int spk_model_set_seed(spk_model* m, uint64_t seed) {
  if (!m) return SPK_ERR_INVALID;
  m->model.philox_seed = seed;
  return SPK_OK;
}

int spk_model_add_neuron_group(spk_model* m, const spk_lif_params* p, int32_t* gid) {
  if (!m || !p) return SPK_ERR_INVALID;
  return guarded([&] {
    lif_spiking_neuron_parameters_struct s;
    s.group_shape[0] = p->group_shape[0];
    s.group_shape[1] = p->group_shape[1];
    s.resting_potential_v0 = p->resting_potential_v0;
    s.after_spike_reset_potential_vreset = p->after_spike_reset_potential_vreset;
    s.threshold_for_action_potential_spike = p->threshold_for_action_potential_spike;
    s.absolute_refractory_period = p->absolute_refractory_period;
    s.somatic_capacitance_Cm = p->somatic_capacitance_Cm;
    s.somatic_leakage_conductance_g0 = p->somatic_leakage_conductance_g0;
    s.background_current = p->background_current;
    s.v_init_lo = p->v_init_lo;
    s.v_init_hi = p->v_init_hi;
    int id = m->model.AddNeuronGroup(&s);
    if (gid) *gid = id;
    return SPK_OK;
  });
}

int spk_model_add_input_group(spk_model* m, int32_t s0, int32_t s1, float rate, int32_t* gid) {
  if (!m || !m->inputs) return SPK_ERR_INVALID;
  return guarded([&] {
    poisson_input_spiking_neuron_parameters_struct s;
    s.group_shape[0] = s0;
    s.group_shape[1] = s1;
    s.rate = rate;
    int id = m->model.AddInputNeuronGroup(&s);
    if (gid) *gid = id;
    return SPK_OK;
  });
}

int spk_model_add_stimulus(spk_model* m, const float* rates, int32_t n, int32_t* sid) {
  if (!m || !rates) return SPK_ERR_INVALID;
  auto* pp = dynamic_cast<PatternedPoissonInputSpikingNeurons*>(m->inputs);
  if (!pp) return SPK_ERR_INVALID;
  return guarded([&] {
    int id = pp->add_stimulus(rates, n);
    if (sid) *sid = id;
    return SPK_OK;
  });
}

int spk_model_add_plasticity_rule(spk_model* m, int32_t rule, const spk_stdp_params* p, int32_t* rid) {
  if (!m || !p) return SPK_ERR_INVALID;
  if (rule == SPK_STDP_WEIGHT_DEPENDENT) return spk_model_add_stdp_rule(m, p, rid);
  if (rule != SPK_STDP_EVANS && rule != SPK_STDP_INHIBITORY && rule != SPK_STDP_CUSTOM) return SPK_ERR_INVALID;
  return guarded([&] {
    Plasticity* r = nullptr;
    if (rule == SPK_STDP_EVANS) {
      // the descriptor's field mapping of SPK_STDP_EVANS, back into the rule's struct
      auto* ep = new evans_stdp_plasticity_parameters_struct();
      ep->decay_term_tau_D = p->tau_minus;
      ep->decay_term_tau_C = p->tau_plus;
      ep->model_parameter_alpha_D = p->a_minus;
      ep->synaptic_neurotransmitter_concentration_alpha_C = p->a_plus;
      m->rule_params.push_back(ep);
      r = new EvansSTDPPlasticity(m->synapses, &m->neurons, m->inputs, ep);
    } else if (rule == SPK_STDP_CUSTOM) {
      auto* cp = new custom_stdp_plasticity_parameters_struct();
      cp->a_minus = p->a_minus;
      cp->a_plus = p->a_plus;
      cp->tau_minus = p->tau_minus;
      cp->tau_plus = p->tau_plus;
      cp->w_max = p->w_max;
      cp->learning_rate = p->lambda;
      cp->a_star = p->alpha;
      cp->nearest_spike_only = p->clip_upper != 0;
      m->rule_params.push_back(cp);
      r = new CustomSTDPPlasticity(m->synapses, &m->neurons, m->inputs, cp);
    } else {
      auto* ip = new inhibitory_stdp_plasticity_parameters_struct();
      ip->tau_istdp = p->tau_plus;
      ip->learningrate = p->lambda;
      ip->targetrate = p->alpha;
      m->rule_params.push_back(ip);
      r = new InhibitorySTDPPlasticity(m->synapses, &m->neurons, m->inputs, ip);
    }
    m->rules.push_back(r);
    m->model.AddPlasticityRule(r);
    if (rid) *rid = (int32_t)m->rules.size() - 1;
    return SPK_OK;
  });
}

int spk_model_add_weight_norm_rule(spk_model* m, int32_t settarget, float target, int32_t* rid) {
  if (!m) return SPK_ERR_INVALID;
  return guarded([&] {
    auto* np = new weightnorm_stdp_plasticity_parameters_struct();
    np->settarget = settarget != 0;
    np->target = target;
    m->rule_params.push_back(np);
    Plasticity* r = new WeightNormSTDPPlasticity(m->synapses, &m->neurons, m->inputs, np);
    m->rules.push_back(r);
    m->model.AddPlasticityRule(r);
    if (rid) *rid = (int32_t)m->rules.size() - 1;
    return SPK_OK;
  });
}

int spk_model_add_stdp_rule(spk_model* m, const spk_stdp_params* p, int32_t* rid) {
  if (!m || !p) return SPK_ERR_INVALID;
  return guarded([&] {
    auto* wp = new weightdependent_stdp_plasticity_parameters_struct();
    wp->a_minus = p->a_minus;
    wp->a_plus = p->a_plus;
    wp->tau_minus = p->tau_minus;
    wp->tau_plus = p->tau_plus;
    wp->lambda = p->lambda;
    wp->alpha = p->alpha;
    wp->w_max = p->w_max;
    wp->clip_upper = p->clip_upper != 0;
    m->rule_params.push_back(wp);
    auto* r = new WeightDependentSTDPPlasticity(m->synapses, &m->neurons, m->inputs, wp);
    m->rules.push_back(r);
    m->model.AddPlasticityRule(r);
    if (rid) *rid = (int32_t)m->rules.size() - 1;
    return SPK_OK;
  });
}

int spk_model_add_synapse_group(spk_model* m, int32_t pre, int32_t post, const spk_synapse_params* p,
                                int32_t* gid) {
  if (!m || !p) return SPK_ERR_INVALID;
  if (p->n_pairwise > 0 && (!p->pairwise_connect_presynaptic || !p->pairwise_connect_postsynaptic))
    return SPK_ERR_INVALID;
  return guarded([&] {
    int id = add_group_with(m, pre, post, p, nullptr, nullptr);
    if (gid) *gid = id;
    return SPK_OK;
  });
}

int spk_model_connect_with_sparsity(spk_model* m, int32_t pre, int32_t post, float sparseness,
                                    const spk_synapse_params* p, int32_t* gid) {
  if (!m || !p) return SPK_ERR_INVALID;
  return guarded([&] {
    SpikingNeurons* pre_pop = pre < 0 ? (SpikingNeurons*)m->inputs : (SpikingNeurons*)&m->neurons;
    if (!pre_pop) fail(SPK_ERR_INVALID, "no input population");
    int pg = pre < 0 ? -pre - 1 : pre;
    if (pg >= pre_pop->total_number_of_groups || post < 0 || post >= m->neurons.total_number_of_groups)
      fail(SPK_ERR_INVALID, "bad group id");
    const auto& ps = pre_pop->group_shapes[pg];
    const auto& qs = m->neurons.group_shapes[post];
    int num_post = qs[0] * qs[1];
    int num_pre = ps[0] * ps[1];
    int per_post = sparseness * num_pre;
    std::vector<int> prevec, postvec;
    prevec.reserve((size_t)num_post * per_post);
    postvec.reserve((size_t)num_post * per_post);
    for (int o = 0; o < num_post; o++)
      for (int i = 0; i < per_post; i++) {
        postvec.push_back(o);
        prevec.push_back(rand() % num_pre);
      }
    int id = add_group_with(m, pre, post, p, &prevec, &postvec);
    if (gid) *gid = id;
    return SPK_OK;
  });
}

int spk_model_set_recording(spk_model* m, int32_t record_inputs, int64_t cap) {
  if (!m) return SPK_ERR_INVALID;
  m->model.spike_capacity = cap;
  if (record_inputs && m->inputs && !m->input_monitor) {
    m->input_monitor = new SpikingActivityMonitor(m->inputs);
    m->model.AddActivityMonitor(m->input_monitor);
  }
  return SPK_OK;
}

int spk_model_finalise(spk_model* m, const spk_schedule* sched) {
  if (!m) return SPK_ERR_INVALID;
  return guarded([&] {
    if (sched) m->model.schedule = *sched;
    m->model.finalise_model();
    return SPK_OK;
  });
}

int spk_model_run(spk_model* m, float seconds, int32_t plasticity_on) {
  if (!m) return SPK_ERR_INVALID;
  return guarded([&] {
    m->model.run(seconds, plasticity_on != 0);
    return m->model.last_status();
  });
}

int spk_model_reset_state(spk_model* m) {
  if (!m) return SPK_ERR_INVALID;
  return guarded([&] {
    m->model.reset_state();
    return SPK_OK;
  });
}

int spk_model_reset_time(spk_model* m) {
  if (!m) return SPK_ERR_INVALID;
  m->model.reset_time();
  return SPK_OK;
}

int spk_model_select_stimulus(spk_model* m, int32_t s) {
  if (!m || !m->inputs) return SPK_ERR_INVALID;
  return guarded([&] {
    m->inputs->select_stimulus(s);
    return SPK_OK;
  });
}

int spk_model_net(spk_model* m, spk_net** out) {
  if (!m || !out) return SPK_ERR_INVALID;
  if (!m->model.net()) return SPK_ERR_STATE;
  *out = m->model.net();
  return SPK_OK;
}

int spk_model_desc(spk_model* m, spk_net_desc* out) {
  if (!m || !out) return SPK_ERR_INVALID;
  return guarded([&] { return m->model.build_desc(out); });
}

int spk_model_counts(spk_model* m, int32_t* nn, int32_t* ni, int64_t* ns) {
  if (!m) return SPK_ERR_INVALID;
  if (nn) *nn = m->neurons.total_number_of_neurons;
  if (ni) *ni = m->inputs ? m->inputs->total_number_of_neurons : 0;
  if (ns) *ns = m->synapses->total_number_of_synapses;
  return SPK_OK;
}

int spk_model_spikes(spk_model* m, int32_t pop, const int32_t** ids, const float** times, int64_t* n) {
  if (!m || pop < 0 || pop > 1) return SPK_ERR_INVALID;
  SpikingActivityMonitor* mon = pop == SPK_POP_NEURONS ? m->neuron_monitor : m->input_monitor;
  if (!mon) {
    if (n) *n = 0;
    if (ids) *ids = nullptr;
    if (times) *times = nullptr;
    return SPK_OK;
  }
  if (ids) *ids = mon->neuron_ids_of_stored_spikes_on_host.data();
  if (times) *times = mon->spike_times_of_stored_spikes_on_host.data();
  if (n) *n = mon->total_number_of_spikes_stored_on_host;
  return SPK_OK;
}

int spk_model_clear_spikes(spk_model* m) {
  if (!m) return SPK_ERR_INVALID;
  if (m->neuron_monitor) m->neuron_monitor->reset_state();
  if (m->input_monitor) m->input_monitor->reset_state();
  return SPK_OK;
}

int spk_model_add_rate_monitor(spk_model* m, int32_t pop) {
  if (!m || pop < 0 || pop > 1) return SPK_ERR_INVALID;
  if (pop == SPK_POP_INPUTS && !m->inputs) return SPK_ERR_INVALID;
  if (m->rate_monitor[pop]) return SPK_OK;
  return guarded([&] {
    m->rate_monitor[pop] =
        new RateActivityMonitor(pop == SPK_POP_NEURONS ? (SpikingNeurons*)&m->neurons : (SpikingNeurons*)m->inputs);
    m->model.AddActivityMonitor(m->rate_monitor[pop]);
    return SPK_OK;
  });
}

int spk_model_rate_counts(spk_model* m, int32_t pop, const int32_t** counts, int64_t* n) {
  if (!m || pop < 0 || pop > 1) return SPK_ERR_INVALID;
  RateActivityMonitor* mon = m->rate_monitor[pop];
  if (counts) *counts = mon ? mon->per_neuron_spike_counts.data() : nullptr;
  if (n) *n = mon ? (int64_t)mon->per_neuron_spike_counts.size() : 0;
  return SPK_OK;
}

}  // extern "C"
