// spike_gb300_model.hpp - C++ model-building front end with the reference's
// class and parameter-struct names, so programs written against Spike
// (e.g. Examples/VogelsAbbottNet.cpp, Examples/Brunel10K.cpp) build against
// this header with an include-path change.
//
// What is kept from the reference, and why (each piece has to match exactly
// for a network to be the same network):
//  - parameter structs and their defaults (Spike/Neurons/*.hpp, Spike/Synapses/*.hpp,
//    Spike/Plasticity/WeightDependentSTDPPlasticity.hpp:28-40);
//  - group ids (inputs -1-g, Spike/Neurons/InputSpikingNeurons.cpp:6-9) and the
//    presynaptic id convention (Spike/Neurons/Neurons.hpp:34-35);
//  - connectivity construction and its glibc rand() call order
//    (Spike/Synapses/Synapses.cpp:102-388, Spike/Synapses/SpikingSynapses.cpp:62-124);
//  - syn-label assignment (Spike/Synapses/ConductanceSpikingSynapses.cpp:19-75,
//    Spike/Synapses/CurrentSpikingSynapses.cpp:4-48);
//  - the quirks of global refractory period / background current and of Poisson
//    rates taken from the last group (Spike/Neurons/LIFSpikingNeurons.cpp:24,37,
//    Spike/Neurons/PoissonInputSpikingNeurons.cpp:26-31).
// What changes: there is no backend factory; finalise_model() flattens the
// model into an spk_net_desc and creates one device network (spike_gb300.h).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "spike_gb300.h"

class SpikingModel;
class Plasticity;

#define PRESYNAPTIC_IS_INPUT(id) (id < 0 ? true : false)
#define CORRECTED_PRESYNAPTIC_ID(id, is_input) (is_input ? (-1 * (id)) - 1 : id)

// ---- parameter structs --------------------------------------------------------
struct neuron_parameters_struct {
  neuron_parameters_struct() {}
  virtual ~neuron_parameters_struct() = default;
  int group_shape[2];
};
struct spiking_neuron_parameters_struct : neuron_parameters_struct {
  float resting_potential_v0 = -0.074f;
  float after_spike_reset_potential_vreset = -0.074f;
  float threshold_for_action_potential_spike = 0.03f;
  float absolute_refractory_period = 0.002f;
};
struct lif_spiking_neuron_parameters_struct : spiking_neuron_parameters_struct {
  float somatic_capacitance_Cm = 0.0f;
  float somatic_leakage_conductance_g0 = 0.0f;
  float background_current = 0.0f;
  float v_init_lo = 0.0f;  // extension: initial V ~ U(lo, hi] when lo < hi
  float v_init_hi = 0.0f;
};
struct input_spiking_neuron_parameters_struct : spiking_neuron_parameters_struct {};
struct poisson_input_spiking_neuron_parameters_struct : input_spiking_neuron_parameters_struct {
  float rate = 50.0f;
};
struct patterned_poisson_input_spiking_neuron_parameters_struct
    : poisson_input_spiking_neuron_parameters_struct {};

enum CONNECTIVITY_TYPE {
  CONNECTIVITY_TYPE_ALL_TO_ALL,
  CONNECTIVITY_TYPE_ONE_TO_ONE,
  CONNECTIVITY_TYPE_RANDOM,
  CONNECTIVITY_TYPE_GAUSSIAN_SAMPLE,
  CONNECTIVITY_TYPE_PAIRWISE
};

struct synapse_parameters_struct {
  virtual ~synapse_parameters_struct() = default;
  std::vector<int> pairwise_connect_presynaptic;
  std::vector<int> pairwise_connect_postsynaptic;
  std::vector<float> pairwise_connect_weight;
  int max_number_of_connections_per_pair = 1;
  int gaussian_synapses_per_postsynaptic_neuron = 10;
  float gaussian_synapses_standard_deviation = 10.0;
  float weight_range[2] = {0.0f, 0.0f};
  float weight_scaling_constant = 1.0;
  float random_connectivity_probability = 0.0f;
  int connectivity_type = CONNECTIVITY_TYPE_ALL_TO_ALL;
  std::vector<Plasticity*> plasticity_vec;
};
struct spiking_synapse_parameters_struct : synapse_parameters_struct {
  float delay_range[2] = {0.0f, 0.0f};
  std::vector<float> pairwise_connect_delay;
};
struct conductance_spiking_synapse_parameters_struct : spiking_synapse_parameters_struct {
  float reversal_potential_Vhat = 0.0f;
  float decay_term_tau_g = 0.001f;
};
struct current_spiking_synapse_parameters_struct : spiking_synapse_parameters_struct {
  float decay_term_tau = 0.001f;
};
struct voltage_spiking_synapse_parameters_struct : spiking_synapse_parameters_struct {};

struct plasticity_parameters_struct {
  virtual ~plasticity_parameters_struct() = default;
};
struct stdp_plasticity_parameters_struct : plasticity_parameters_struct {};
struct weightdependent_stdp_plasticity_parameters_struct : stdp_plasticity_parameters_struct {
  float a_minus = 1.0f;
  float a_plus = 1.0f;
  float tau_minus = 0.02f;
  float tau_plus = 0.02f;
  float lambda = 1.0f;
  float alpha = 1.0f;
  float w_max = 1.0f;
  bool nearest_spike_only = false;
  bool clip_upper = false;  // extension: clip at w_max as well as at 0
};

// evans_stdp_plasticity_parameters_struct (Spike/Plasticity/EvansSTDPPlasticity.hpp);
// learning_rate_rho is carried but, as in the reference's kernel, unused.
struct evans_stdp_plasticity_parameters_struct : stdp_plasticity_parameters_struct {
  float decay_term_tau_D = 0.005f;
  float model_parameter_alpha_D = 0.5f;
  float synaptic_neurotransmitter_concentration_alpha_C = 0.5f;
  float decay_term_tau_C = 0.004f;
  float learning_rate_rho = 0.1f;
};
// inhibitory_stdp_plasticity_parameters_struct
// (Spike/Plasticity/InhibitorySTDPPlasticity.hpp); momentumrate is unused there too.
struct inhibitory_stdp_plasticity_parameters_struct : stdp_plasticity_parameters_struct {
  float tau_istdp = 0.02f;
  float learningrate = 0.0004f;
  float targetrate = 10.0f;
  float momentumrate = 0.0f;
};
// weightnorm_stdp_plasticity_parameters_struct
// (Spike/Plasticity/WeightNormSTDPPlasticity.hpp:41-46).
struct weightnorm_stdp_plasticity_parameters_struct : stdp_plasticity_parameters_struct {
  bool settarget = false;
  float target = 0.0f;
};
// custom_stdp_plasticity_parameters_struct (Spike/Plasticity/CustomSTDPPlasticity.hpp);
// a_star and learning_rate start at 0 here (the reference leaves them unset).
struct custom_stdp_plasticity_parameters_struct : stdp_plasticity_parameters_struct {
  float a_minus = 1.0f;
  float a_plus = 1.0f;
  float a_star = 0.0f;
  float tau_minus = 0.02f;
  float tau_plus = 0.02f;
  float w_max = 1.0f;
  float learning_rate = 0.0f;
  bool nearest_spike_only = false;
};

// ---- neurons -------------------------------------------------------------------
class SpikingNeurons {
 public:
  virtual ~SpikingNeurons() = default;
  virtual int AddGroup(neuron_parameters_struct* group_params);
  int total_number_of_neurons = 0;
  int total_number_of_groups = 0;
  int number_of_neurons_in_new_group = 0;
  std::vector<int> start_neuron_indices_for_each_group;
  std::vector<int> last_neuron_indices_for_each_group;
  std::vector<std::vector<int>> group_shapes;
  std::vector<float> after_spike_reset_potentials_vreset, resting_potentials_v0,
      thresholds_for_action_potential_spikes;
  std::vector<int> per_neuron_afferent_synapse_count, per_neuron_efferent_synapse_count;
  int max_num_efferent_synapses = 0;
  SpikingModel* model = nullptr;
  virtual bool is_input() const { return false; }
  void AddEfferentSynapse(int neuron_id);
};

class LIFSpikingNeurons : public SpikingNeurons {
 public:
  int AddGroup(neuron_parameters_struct* group_params) override;
  std::vector<float> membrane_time_constants_tau_m, membrane_resistances_R;
  std::vector<float> v_init_lo, v_init_hi;
  float background_current = 0.0f;
  float refractory_period_in_seconds = 0.0f;
};

class InputSpikingNeurons : public SpikingNeurons {
 public:
  int AddGroup(neuron_parameters_struct* group_params) override;
  bool is_input() const override { return true; }
  virtual void select_stimulus(int stimulus_index);
  int current_stimulus_index = 0;
  int total_number_of_input_stimuli = 0;
};

class PoissonInputSpikingNeurons : public InputSpikingNeurons {
 public:
  int AddGroup(neuron_parameters_struct* group_params) override;
  void set_up_rates();
  void select_stimulus(int stimulus_index) override;
  float rate = 0;
  std::vector<float> rates;
  virtual bool patterned() const { return false; }
};

class PatternedPoissonInputSpikingNeurons : public PoissonInputSpikingNeurons {
 public:
  bool patterned() const override { return true; }
  void reset_stimuli();
  int add_stimulus(const float* rates, int num_rates);
  int add_stimulus(std::vector<float> rates);
  std::vector<float> stimuli_rates;
  int total_number_of_rates = 0;
};

// ---- synapses ------------------------------------------------------------------
class SpikingSynapses {
 public:
  SpikingSynapses();
  explicit SpikingSynapses(int seedval);
  virtual ~SpikingSynapses() = default;
  virtual int AddGroup(int presynaptic_group_id, int postsynaptic_group_id,
                       SpikingNeurons* neurons, SpikingNeurons* input_neurons, float timestep,
                       synapse_parameters_struct* synapse_params);
  virtual int kind() const = 0;

  int total_number_of_synapses = 0;
  int temp_number_of_synapses_in_last_group = 0;
  int largest_synapse_group_size = 0;
  int maximum_number_of_afferent_synapses = 0;
  std::vector<int> presynaptic_neuron_indices, postsynaptic_neuron_indices;
  std::vector<float> synaptic_efficacies_or_weights, weight_scaling_constants;
  std::vector<int> delays, syn_labels;
  std::vector<uint8_t> plastic;
  std::vector<int> last_index_of_synapse_per_group, prepop_start_per_group,
      postpop_start_per_group;
  std::vector<bool> prepop_is_input;
  int minimum_axonal_delay_in_timesteps = 1000000;
  int maximum_axonal_delay_in_timesteps = 0;
  int neuron_pop_size = 0;
  int num_syn_labels = 1;
  std::vector<Plasticity*> plasticity_rule_vec;
  SpikingModel* model = nullptr;

  // Readback in creation order (Spike/Synapses/Synapses.cpp:525-584).
  void copy_weights_to_host();
  void save_weights_as_binary(std::string path, std::string prefix = "", int synapsegroupid = -1);
  void save_weights_as_txt(std::string path, std::string prefix = "", int synapsegroupid = -1);
  void load_weights(std::vector<float> weights, int synapsegroupid = -1);
  void load_weights_from_txt(std::string filepath, int synapsegroupid = -1);
  void load_weights_from_binary(std::string filepath, int synapsegroupid = -1);
  void save_connectivity_as_binary(std::string path, std::string prefix = "",
                                   int synapsegroupid = -1);
  void save_connectivity_as_txt(std::string path, std::string prefix = "",
                                int synapsegroupid = -1);

 protected:
  void group_range(int synapsegroupid, int& startid, int& endid) const;
};

class ConductanceSpikingSynapses : public SpikingSynapses {
 public:
  using SpikingSynapses::SpikingSynapses;
  int AddGroup(int pre, int post, SpikingNeurons* n, SpikingNeurons* in, float timestep,
               synapse_parameters_struct* p) override;
  int kind() const override { return SPK_SYN_CONDUCTANCE; }
  std::vector<float> reversal_potentials_Vhat, decay_terms_tau_g;
};

class CurrentSpikingSynapses : public SpikingSynapses {
 public:
  using SpikingSynapses::SpikingSynapses;
  int AddGroup(int pre, int post, SpikingNeurons* n, SpikingNeurons* in, float timestep,
               synapse_parameters_struct* p) override;
  int kind() const override { return SPK_SYN_CURRENT; }
  std::vector<float> decay_terms_tau;
};

class VoltageSpikingSynapses : public SpikingSynapses {
 public:
  using SpikingSynapses::SpikingSynapses;
  int kind() const override { return SPK_SYN_VOLTAGE; }
};

// ---- plasticity ----------------------------------------------------------------
class Plasticity {
 public:
  virtual ~Plasticity() = default;
  int plasticity_rule_id = -1;
  std::vector<int> plastic_synapses;  // creation indices
  void AddSynapseIndices(int synapse_start_id, int num_synapses_to_add);
};

class STDPPlasticity : public Plasticity {};

class WeightDependentSTDPPlasticity : public STDPPlasticity {
 public:
  WeightDependentSTDPPlasticity(SpikingSynapses* synapses, SpikingNeurons* neurons,
                                SpikingNeurons* input_neurons,
                                stdp_plasticity_parameters_struct* stdp_parameters);
  weightdependent_stdp_plasticity_parameters_struct* stdp_params;
};

// Rules with two traces per plastic synapse, updated every timestep (the
// engine runs them in bulk mode).
class EvansSTDPPlasticity : public STDPPlasticity {
 public:
  EvansSTDPPlasticity(SpikingSynapses* synapses, SpikingNeurons* neurons, SpikingNeurons* input_neurons,
                      stdp_plasticity_parameters_struct* stdp_parameters);
  evans_stdp_plasticity_parameters_struct* stdp_params;
};

class InhibitorySTDPPlasticity : public STDPPlasticity {
 public:
  InhibitorySTDPPlasticity(SpikingSynapses* synapses, SpikingNeurons* neurons, SpikingNeurons* input_neurons,
                           stdp_plasticity_parameters_struct* stdp_parameters);
  inhibitory_stdp_plasticity_parameters_struct* stdp_params;
};

class CustomSTDPPlasticity : public STDPPlasticity {
 public:
  CustomSTDPPlasticity(SpikingSynapses* synapses, SpikingNeurons* neurons, SpikingNeurons* input_neurons,
                       stdp_plasticity_parameters_struct* stdp_parameters);
  custom_stdp_plasticity_parameters_struct* stdp_params;
};

// Per-post L2 normalisation of the plastic weights every timestep
// (Spike/Plasticity/WeightNormSTDPPlasticity.hpp).  Supported on the synapses
// of the model's STDP rule; it runs before or after that rule in the order
// the two were added.
class WeightNormSTDPPlasticity : public STDPPlasticity {
 public:
  WeightNormSTDPPlasticity(SpikingSynapses* synapses, SpikingNeurons* neurons, SpikingNeurons* input_neurons,
                           stdp_plasticity_parameters_struct* parameters);
  weightnorm_stdp_plasticity_parameters_struct* plasticity_parameters;
};

// ---- monitors ------------------------------------------------------------------
class SpikingActivityMonitor {
 public:
  explicit SpikingActivityMonitor(SpikingNeurons* neurons_parameter) : neurons(neurons_parameter) {}
  SpikingNeurons* neurons;
  SpikingModel* model = nullptr;
  std::vector<int> neuron_ids_of_stored_spikes_on_host;
  std::vector<float> spike_times_of_stored_spikes_on_host;
  int total_number_of_spikes_stored_on_host = 0;
  void reset_state();
  void save_spikes_as_txt(std::string path, std::string prefix = "");
  void save_spikes_as_binary(std::string path, std::string prefix = "");
};

// RateActivityMonitor (Spike/ActivityMonitor/RateActivityMonitor.hpp): spikes per
// neuron of its population, counted on the device as the spikes are decided,
// copied to per_neuron_spike_counts after run() (final_update) and zeroed by
// reset_state (host and device).
class RateActivityMonitor {
 public:
  explicit RateActivityMonitor(SpikingNeurons* neurons_parameter) : neurons(neurons_parameter) {}
  SpikingNeurons* neurons;
  SpikingModel* model = nullptr;
  std::vector<int> per_neuron_spike_counts;
  void reset_state();
};

// ---- model ---------------------------------------------------------------------
class SpikingModel {
 public:
  SpikingModel();
  ~SpikingModel();
  SpikingNeurons* spiking_neurons = nullptr;
  SpikingSynapses* spiking_synapses = nullptr;
  SpikingNeurons* input_spiking_neurons = nullptr;
  std::vector<Plasticity*> plasticity_rule_vec;
  std::vector<SpikingActivityMonitor*> monitors_vec;
  std::vector<RateActivityMonitor*> rate_monitors_vec;
  bool model_complete = false;
  float timestep = 0.0001f;
  int timestep_grouping = 1;
  uint64_t philox_seed = 1;  // Poisson/V-init stream key (extension)
  spk_schedule schedule{};   // zero = chosen by the library
  int64_t spike_capacity = 0;

  void SetTimestep(float timestep_parameter);
  int AddNeuronGroup(neuron_parameters_struct* group_params);
  int AddInputNeuronGroup(neuron_parameters_struct* group_params);
  int AddSynapseGroup(int presynaptic_group_id, int postsynaptic_group_id,
                      synapse_parameters_struct* synapse_params);
  void AddSynapseGroupsForNeuronGroupAndEachInputGroup(int postsynaptic_group_id,
                                                       synapse_parameters_struct* synapse_params);
  void AddPlasticityRule(Plasticity* plasticity_rule);
  void AddActivityMonitor(SpikingActivityMonitor* activityMonitor);
  void AddActivityMonitor(RateActivityMonitor* activityMonitor);
  void finalise_model();
  void reset_state();
  void reset_time();
  void run(float seconds, bool plasticity_on = true);

  // Flatten into the C-ABI descriptor (pointers into this model's arrays).
  int build_desc(spk_net_desc* out);
  spk_net* net() const { return net_; }
  int last_status() const { return status_; }
  void collect_spikes();
  void collect_rates();

 private:
  spk_net* net_ = nullptr;
  int status_ = SPK_OK;
  std::vector<spk_neuron_group> groups_;
  std::vector<float> label_tau_, label_vhat_, rates_;
  std::vector<float> empty_f_;
  std::vector<float> norm_initial_, norm_sum_;  // the weight normalisation's host arrays
};
