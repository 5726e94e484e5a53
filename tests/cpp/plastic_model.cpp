// A program written against the C++ model API the way a Spike user writes one
// (Examples/Brunel10K.cpp style): LIF neurons, Poisson inputs, voltage
// synapses, and the plasticity classes attached through plasticity_vec.
//   plastic_model desc   flatten both models and print their descriptors' rule
//                        fields (no GPU needed)
//   plastic_model run    run both models for 30 ms and print their spike counts
#include <cstdio>
#include <cstring>

#include "spike_gb300_model.hpp"

namespace {

struct Built {
  SpikingModel* model;
  SpikingActivityMonitor* monitor;
};

// 800 E + 200 I LIF neurons driven by 800 Poisson inputs; `evans` puts the
// Evans rule on the input synapses, otherwise the E->E synapses take the
// weight-dependent rule with the weight normalisation added after it.
Built build(bool evans) {
  SpikingModel* model = new SpikingModel();
  model->SetTimestep(0.0001f);
  LIFSpikingNeurons* lif = new LIFSpikingNeurons();
  PoissonInputSpikingNeurons* inputs = new PoissonInputSpikingNeurons();
  VoltageSpikingSynapses* synapses = new VoltageSpikingSynapses();
  model->spiking_neurons = lif;
  model->input_spiking_neurons = inputs;
  model->spiking_synapses = synapses;

  lif_spiking_neuron_parameters_struct exc;
  exc.group_shape[0] = 800;
  exc.group_shape[1] = 1;
  exc.somatic_capacitance_Cm = 200.0e-12f;
  exc.somatic_leakage_conductance_g0 = 10.0e-9f;
  exc.resting_potential_v0 = 0.0f;
  exc.after_spike_reset_potential_vreset = 0.0f;
  exc.threshold_for_action_potential_spike = 20.0e-3f;
  exc.absolute_refractory_period = 2.0e-3f;
  lif_spiking_neuron_parameters_struct inh = exc;
  inh.group_shape[0] = 200;
  poisson_input_spiking_neuron_parameters_struct in;
  in.group_shape[0] = 800;
  in.group_shape[1] = 1;
  in.rate = 20.0f;

  const int gin = model->AddInputNeuronGroup(&in);
  const int ge = model->AddNeuronGroup(&exc);
  const int gi = model->AddNeuronGroup(&inh);

  Plasticity* stdp = nullptr;
  Plasticity* norm = nullptr;
  if (evans) {
    auto* p = new evans_stdp_plasticity_parameters_struct();
    stdp = new EvansSTDPPlasticity(synapses, lif, inputs, p);
    model->AddPlasticityRule(stdp);
  } else {
    auto* p = new weightdependent_stdp_plasticity_parameters_struct();
    p->a_plus = 0.005f;
    p->a_minus = 0.00525f;
    stdp = new WeightDependentSTDPPlasticity(synapses, lif, inputs, p);
    auto* np = new weightnorm_stdp_plasticity_parameters_struct();
    norm = new WeightNormSTDPPlasticity(synapses, lif, inputs, np);
    model->AddPlasticityRule(stdp);
    model->AddPlasticityRule(norm);
  }

  const float J = 0.8e-3f;
  voltage_spiking_synapse_parameters_struct ext;
  ext.connectivity_type = CONNECTIVITY_TYPE_RANDOM;
  ext.random_connectivity_probability = 0.1f;
  ext.delay_range[0] = 0.0001f;
  ext.delay_range[1] = 0.002f;
  ext.weight_range[0] = evans ? 0.0f : J;
  ext.weight_range[1] = evans ? 1.0f : J;
  ext.weight_scaling_constant = evans ? 2.5f * J : 1.0f;
  if (evans) ext.plasticity_vec.push_back(stdp);
  model->AddSynapseGroup(gin, ge, &ext);
  model->AddSynapseGroup(gin, gi, &ext);

  voltage_spiking_synapse_parameters_struct ee;
  ee.connectivity_type = CONNECTIVITY_TYPE_RANDOM;
  ee.random_connectivity_probability = 0.1f;
  ee.delay_range[0] = 0.0001f;
  ee.delay_range[1] = 0.002f;
  ee.weight_range[0] = 0.5f * J;
  ee.weight_range[1] = 1.5f * J;
  if (!evans) {
    ee.plasticity_vec.push_back(stdp);
    ee.plasticity_vec.push_back(norm);
  }
  model->AddSynapseGroup(ge, ge, &ee);

  voltage_spiking_synapse_parameters_struct ie = ee;
  ie.plasticity_vec.clear();
  ie.weight_range[0] = ie.weight_range[1] = -5.0f * J;
  model->AddSynapseGroup(gi, ge, &ie);

  SpikingActivityMonitor* monitor = new SpikingActivityMonitor(lif);
  model->AddActivityMonitor(monitor);
  return Built{model, monitor};
}

}  // namespace

int main(int argc, char** argv) {
  const bool run = argc > 1 && std::strcmp(argv[1], "run") == 0;
  for (int evans = 0; evans < 2; ++evans) {
    Built b = build(evans != 0);
    if (!run) {
      spk_net_desc d;
      const int rc = b.model->build_desc(&d);
      long long plastic = 0;
      for (long long s = 0; s < d.n_synapses; ++s) plastic += d.plastic && d.plastic[s] ? 1 : 0;
      std::printf("model %d rc %d has_stdp %d stdp_rule %d weight_norm %d synapses %lld plastic %lld\n", evans, rc,
                  d.has_stdp, d.stdp_rule, d.weight_norm, (long long)d.n_synapses, plastic);
    } else {
      b.model->finalise_model();
      b.model->run(0.03f, true);
      b.model->collect_spikes();
      std::printf("model %d status %d spikes %d\n", evans, b.model->last_status(),
                  b.monitor->total_number_of_spikes_stored_on_host);
    }
  }
  return 0;
}
