// ref_dump.cpp - builds small networks through the REFERENCE front end
// (compiled from the reference sources by oracle/build_ref.sh, Dummy backend)
// and dumps the connectivity it produces, for golden fixtures.
//
// TEST INFRASTRUCTURE ONLY.  Usage: ref_dump <case> <out.bin>
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

lif_spiking_neuron_parameters_struct* lif(int n, float v0, float vreset, float theta, float tref,
                                          float ibg) {
  auto* p = new lif_spiking_neuron_parameters_struct();
  p->group_shape[0] = 1;
  p->group_shape[1] = n;
  p->somatic_capacitance_Cm = 200.0f * pow(10.0, -12);
  p->somatic_leakage_conductance_g0 = 10.0f * pow(10.0, -9);
  p->resting_potential_v0 = v0;
  p->after_spike_reset_potential_vreset = vreset;
  p->threshold_for_action_potential_spike = theta;
  p->absolute_refractory_period = tref;
  p->background_current = ibg;
  return p;
}

// Same construction as Examples/UtilityFunctions.hpp:51-82 (fixed in-degree,
// presynaptic ids drawn with rand() % num_pre, multapses allowed).
void sparsity(int pre_group, int post_group, int n_pre, int n_post,
              voltage_spiking_synapse_parameters_struct* sp, float sparseness, SpikingModel* m) {
  int per_post = sparseness * n_pre;
  std::vector<int> prevec, postvec;
  for (int o = 0; o < n_post; o++)
    for (int i = 0; i < per_post; i++) {
      postvec.push_back(o);
      prevec.push_back(rand() % n_pre);
    }
  sp->pairwise_connect_presynaptic = prevec;
  sp->pairwise_connect_postsynaptic = postvec;
  sp->connectivity_type = CONNECTIVITY_TYPE_PAIRWISE;
  m->AddSynapseGroup(pre_group, post_group, sp);
}

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
  if (rule) put_i("plastic_sorted", rule->plastic_synapses.data(), rule->plastic_synapses.size());
}

int case_va(bool mixed) {
  SpikingModel* m = new SpikingModel();
  m->SetTimestep(0.0001f);
  auto* neurons = new LIFSpikingNeurons();
  auto* syn = new ConductanceSpikingSynapses();
  m->spiking_neurons = neurons;
  m->spiking_synapses = syn;
  int nE = mixed ? 320 : 3200, nI = mixed ? 80 : 800;
  auto* E = lif(nE, -60.0f * pow(10.0, -3), -60.0f * pow(10.0, -3), -50.0f * pow(10.0, -3),
                5.0f * pow(10, -3), 2.0f * pow(10.0, -2));
  auto* I = lif(nI, -60.0f * pow(10.0, -3), -60.0f * pow(10.0, -3), -50.0f * pow(10.0, -3),
                5.0f * pow(10, -3), 2.0f * pow(10.0, -2));
  int ge = m->AddNeuronGroup(E), gi = m->AddNeuronGroup(I);
  auto* es = new conductance_spiking_synapse_parameters_struct();
  auto* is = new conductance_spiking_synapse_parameters_struct();
  float dt = 0.0001f;
  es->delay_range[0] = 1 * dt;
  es->delay_range[1] = (mixed ? 4 : 1) * dt;
  is->delay_range[0] = 1 * dt;
  is->delay_range[1] = (mixed ? 6 : 1) * dt;
  es->reversal_potential_Vhat = 0.0f * pow(10.0, -3);
  is->reversal_potential_Vhat = -80.0f * pow(10.0, -3);
  es->weight_range[0] = mixed ? 0.2f : 0.4f;
  es->weight_range[1] = mixed ? 0.6f : 0.4f;
  is->weight_range[0] = 5.1f;
  is->weight_range[1] = mixed ? 6.1f : 5.1f;
  es->decay_term_tau_g = 5.0f * pow(10.0, -3);
  is->decay_term_tau_g = 10.0f * pow(10.0, -3);
  es->weight_scaling_constant = 10.0f * pow(10.0, -9);
  is->weight_scaling_constant = 10.0f * pow(10.0, -9);
  es->connectivity_type = CONNECTIVITY_TYPE_RANDOM;
  is->connectivity_type = CONNECTIVITY_TYPE_RANDOM;
  es->plasticity_vec.push_back(nullptr);
  is->plasticity_vec.push_back(nullptr);
  es->random_connectivity_probability = mixed ? 0.1 : 0.02;
  is->random_connectivity_probability = mixed ? 0.1 : 0.02;
  m->AddSynapseGroup(ge, ge, es);
  m->AddSynapseGroup(ge, gi, es);
  m->AddSynapseGroup(gi, ge, is);
  m->AddSynapseGroup(gi, gi, is);
  m->finalise_model();
  dump_model(m, syn, neurons, m->input_spiking_neurons, nullptr);
  return 0;
}

int case_brunel() {
  SpikingModel* m = new SpikingModel();
  float dt = 0.0001f;
  m->SetTimestep(dt);
  auto* neurons = new LIFSpikingNeurons();
  auto* inputs = new PoissonInputSpikingNeurons();
  auto* syn = new VoltageSpikingSynapses(42);
  auto* wp = new weightdependent_stdp_plasticity_parameters_struct;
  wp->a_plus = 0.005f;
  wp->a_minus = 0.00525f;
  wp->tau_plus = 0.02f;
  wp->tau_minus = 0.02f;
  wp->lambda = 1.0f;
  wp->alpha = 1.0f;
  wp->w_max = 1.0f;
  auto* rule = new WeightDependentSTDPPlasticity((SpikingSynapses*)syn, (SpikingNeurons*)neurons,
                                                 (SpikingNeurons*)inputs,
                                                 (stdp_plasticity_parameters_struct*)wp);
  m->spiking_neurons = neurons;
  m->input_spiking_neurons = inputs;
  m->spiking_synapses = syn;
  m->AddPlasticityRule(rule);
  auto* E = lif(160, 0.0f, 0.0f, 20.0f * pow(10.0, -3), 2.0f * pow(10, -3), 0.0f);
  auto* I = lif(40, 0.0f, 0.0f, 20.0f * pow(10.0, -3), 2.0f * pow(10, -3), 0.0f);
  auto* ip = new poisson_input_spiking_neuron_parameters_struct();
  ip->group_shape[0] = 1;
  ip->group_shape[1] = 150;
  ip->rate = 20.0f;
  int gin = m->AddInputNeuronGroup(ip);
  int ge = m->AddNeuronGroup(E), gi = m->AddNeuronGroup(I);
  auto* es = new voltage_spiking_synapse_parameters_struct();
  auto* is = new voltage_spiking_synapse_parameters_struct();
  auto* in = new voltage_spiking_synapse_parameters_struct();
  for (auto* p : {es, is, in}) {
    p->delay_range[0] = 1 * dt;
    p->delay_range[1] = 20 * dt;
    p->weight_scaling_constant = 1.0f;
  }
  float J = 0.1f * powf(10.0, -3.0);
  es->weight_range[0] = J;
  es->weight_range[1] = J;
  is->weight_range[0] = -5.0f * J;
  is->weight_range[1] = -5.0f * J;
  in->weight_range[0] = 0.0f;
  in->weight_range[1] = 2.0f * J;
  sparsity(gin, ge, 150, 160, in, 0.1f, m);
  sparsity(gin, gi, 150, 40, in, 0.1f, m);
  sparsity(ge, gi, 160, 40, es, 0.1f, m);
  es->plasticity_vec.push_back(rule);
  sparsity(ge, ge, 160, 160, es, 0.1f, m);
  sparsity(gi, ge, 40, 160, is, 0.1f, m);
  sparsity(gi, gi, 40, 40, is, 0.1f, m);
  m->finalise_model();
  dump_model(m, syn, neurons, inputs, rule);
  put_f("rates", inputs->rates, inputs->total_number_of_neurons);
  return 0;
}

int case_shapes() {
  SpikingModel* m = new SpikingModel();
  float dt = 0.0001f;
  m->SetTimestep(dt);
  auto* neurons = new LIFSpikingNeurons();
  auto* inputs = new PoissonInputSpikingNeurons();
  auto* syn = new VoltageSpikingSynapses(7);
  m->spiking_neurons = neurons;
  m->input_spiking_neurons = inputs;
  m->spiking_synapses = syn;
  auto* ip = new poisson_input_spiking_neuron_parameters_struct();
  ip->group_shape[0] = 4;
  ip->group_shape[1] = 5;
  ip->rate = 35.0f;
  int gin = m->AddInputNeuronGroup(ip);
  auto* A = lif(12, -0.07f, -0.075f, -0.05f, 0.003f, 0.001f);
  auto* Bg = lif(20, -0.065f, -0.07f, -0.052f, 0.002f, 0.0015f);
  int ga = m->AddNeuronGroup(A), gb = m->AddNeuronGroup(Bg);
  auto* all = new voltage_spiking_synapse_parameters_struct();
  all->connectivity_type = CONNECTIVITY_TYPE_ALL_TO_ALL;
  all->delay_range[0] = 1 * dt;
  all->delay_range[1] = 3 * dt;
  all->weight_range[0] = 0.0001f;
  all->weight_range[1] = 0.0003f;
  all->weight_scaling_constant = 2.0f;
  m->AddSynapseGroup(gin, ga, all);
  auto* one = new voltage_spiking_synapse_parameters_struct();
  one->connectivity_type = CONNECTIVITY_TYPE_ONE_TO_ONE;
  one->delay_range[0] = 2 * dt;
  one->delay_range[1] = 2 * dt;
  one->weight_range[0] = 0.0005f;
  one->weight_range[1] = 0.0005f;
  m->AddSynapseGroup(gin, gb, one);
  auto* pw = new voltage_spiking_synapse_parameters_struct();
  pw->connectivity_type = CONNECTIVITY_TYPE_PAIRWISE;
  pw->delay_range[0] = 1 * dt;
  pw->delay_range[1] = 1 * dt;
  pw->pairwise_connect_presynaptic = {0, 3, 3, 11, 5, 0};
  pw->pairwise_connect_postsynaptic = {2, 19, 19, 0, 7, 2};
  pw->pairwise_connect_weight = {0.001f, -0.002f, 0.0015f, 0.003f, -0.0005f, 0.0007f};
  pw->pairwise_connect_delay = {1 * dt, 5 * dt, 5 * dt, 2 * dt, 9 * dt, 3 * dt};
  m->AddSynapseGroup(ga, gb, pw);
  auto* rnd = new voltage_spiking_synapse_parameters_struct();
  rnd->connectivity_type = CONNECTIVITY_TYPE_RANDOM;
  rnd->random_connectivity_probability = 0.3f;
  rnd->delay_range[0] = 1 * dt;
  rnd->delay_range[1] = 7 * dt;
  rnd->weight_range[0] = -0.0002f;
  rnd->weight_range[1] = 0.0004f;
  m->AddSynapseGroup(gb, ga, rnd);
  m->finalise_model();
  dump_model(m, syn, neurons, inputs, nullptr);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: ref_dump <va|va_mix|brunel|shapes> <out.bin>\n");
    return 2;
  }
  out_file = fopen(argv[2], "wb");
  if (!out_file) return 3;
  std::string c = argv[1];
  int rc = 2;
  if (c == "va") rc = case_va(false);
  else if (c == "va_mix") rc = case_va(true);
  else if (c == "brunel") rc = case_brunel();
  else if (c == "shapes") rc = case_shapes();
  fclose(out_file);
  return rc;
}
