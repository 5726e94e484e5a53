/*
 * spike_gb300_model.h - C surface of the model-building front end.
 *
 * The front end keeps the reference's model-building API (SpikingModel,
 * Spike/Models/SpikingModel.hpp:24-67) and its connectivity construction
 * (Spike/Synapses/Synapses.cpp:102-388, Spike/Synapses/SpikingSynapses.cpp:62-124),
 * including the glibc rand() call sequence seeded by the synapse object's
 * constructor (srand(42) or srand(seed), Spike/Synapses/Synapses.cpp:15-25), so
 * a network built through it has exactly the reference's synapses, weights and
 * delays.  The C++ classes are declared in spike_gb300_model.hpp; these C
 * functions wrap them for FFI callers (Python ctypes in this repository).
 */
#ifndef SPIKE_GB300_MODEL_H
#define SPIKE_GB300_MODEL_H

#include "spike_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* CONNECTIVITY_TYPE (Spike/Synapses/Synapses.hpp:65-72) */
#define SPK_CONN_ALL_TO_ALL 0
#define SPK_CONN_ONE_TO_ONE 1
#define SPK_CONN_RANDOM 2
#define SPK_CONN_GAUSSIAN_SAMPLE 3
#define SPK_CONN_PAIRWISE 4

/* input population kinds */
#define SPK_INPUT_NONE 0
#define SPK_INPUT_POISSON 1   /* PoissonInputSpikingNeurons */
#define SPK_INPUT_PATTERNED 2 /* PatternedPoissonInputSpikingNeurons */

/* lif_spiking_neuron_parameters_struct (Spike/Neurons/LIFSpikingNeurons.hpp:7-14)
 * with the spiking_neuron_parameters_struct fields (Spike/Neurons/SpikingNeurons.hpp:13-20). */
typedef struct spk_lif_params {
  int32_t group_shape[2];
  float resting_potential_v0;
  float after_spike_reset_potential_vreset;
  float threshold_for_action_potential_spike;
  float absolute_refractory_period;
  float somatic_capacitance_Cm;
  float somatic_leakage_conductance_g0;
  float background_current;
  float v_init_lo; /* extension: initial V range; lo >= hi keeps V0 */
  float v_init_hi;
} spk_lif_params;

/* synapse_parameters_struct + spiking/conductance/current extensions
 * (Spike/Synapses/Synapses.hpp:80-92, Spike/Synapses/SpikingSynapses.hpp:20-23,
 *  Spike/Synapses/ConductanceSpikingSynapses.hpp:7-12,
 *  Spike/Synapses/CurrentSpikingSynapses.hpp:7-11). */
typedef struct spk_synapse_params {
  int32_t connectivity_type;
  float weight_range[2];
  float weight_scaling_constant;
  float random_connectivity_probability;
  float delay_range[2]; /* seconds */
  float reversal_potential_Vhat;
  float decay_term_tau_g;
  float decay_term_tau;
  int32_t max_number_of_connections_per_pair;
  int32_t gaussian_synapses_per_postsynaptic_neuron;
  float gaussian_synapses_standard_deviation;
  int32_t n_pairwise;
  const int32_t* pairwise_connect_presynaptic;
  const int32_t* pairwise_connect_postsynaptic;
  const float* pairwise_connect_weight; /* n_pairwise values or NULL */
  const float* pairwise_connect_delay;  /* n_pairwise values (s) or NULL */
  int32_t plasticity_rule;              /* rule id from spk_model_add_stdp_rule, or -1 */
  int32_t plasticity_rule_2;            /* a second rule on the same synapses (the weight
                                           normalisation), or -1 */
} spk_synapse_params;

typedef struct spk_model spk_model;

/* synapse_seed < 0 uses the reference's default constructor (srand(42)). */
int spk_model_create(int32_t synapse_kind, int32_t input_kind, int32_t synapse_seed,
                     spk_model** out);
int spk_model_destroy(spk_model* m);
int spk_model_set_timestep(spk_model* m, float dt);
int spk_model_set_seed(spk_model* m, uint64_t philox_seed);
int spk_model_add_neuron_group(spk_model* m, const spk_lif_params* p, int32_t* group_id);
int spk_model_add_input_group(spk_model* m, int32_t shape0, int32_t shape1, float rate,
                              int32_t* group_id);
int spk_model_add_stimulus(spk_model* m, const float* rates, int32_t n, int32_t* stimulus_id);
int spk_model_add_stdp_rule(spk_model* m, const spk_stdp_params* p, int32_t* rule_id);
/* Any of the SPK_STDP_* rules, its parameters in the descriptor's field
 * mapping (spike_gb300.h); one STDP rule per model (the weight normalisation,
 * spk_model_add_weight_norm_rule, may go beside it). */
int spk_model_add_plasticity_rule(spk_model* m, int32_t rule, const spk_stdp_params* p, int32_t* rule_id);
/* WeightNormSTDPPlasticity (Spike/Plasticity/WeightNormSTDPPlasticity.hpp):
 * weightnorm_stdp_plasticity_parameters_struct's settarget and target.  Its
 * synapses must be the STDP rule's; its position among the rules is the
 * order the rules were added in. */
int spk_model_add_weight_norm_rule(spk_model* m, int32_t settarget, float target, int32_t* rule_id);
int spk_model_add_synapse_group(spk_model* m, int32_t pre_group, int32_t post_group,
                                const spk_synapse_params* p, int32_t* group_id);
/* Examples/UtilityFunctions.hpp:51-82 connect_with_sparsity: fixed in-degree
 * sparseness*n_pre per post, presynaptic ids rand() % n_pre, then PAIRWISE. */
int spk_model_connect_with_sparsity(spk_model* m, int32_t pre_group, int32_t post_group,
                                    float sparseness, const spk_synapse_params* p,
                                    int32_t* group_id);
int spk_model_set_recording(spk_model* m, int32_t record_inputs, int64_t spike_capacity);
int spk_model_finalise(spk_model* m, const spk_schedule* schedule);
int spk_model_run(spk_model* m, float seconds, int32_t plasticity_on);
int spk_model_reset_state(spk_model* m);
int spk_model_reset_time(spk_model* m);
int spk_model_select_stimulus(spk_model* m, int32_t stimulus);
/* Borrowed handle of the finalised network (owned by the model). */
int spk_model_net(spk_model* m, spk_net** out);
/* Flattened descriptor over the model's host arrays (valid until the model
 * is destroyed or modified). */
int spk_model_desc(spk_model* m, spk_net_desc* out);
int spk_model_counts(spk_model* m, int32_t* n_neurons, int32_t* n_inputs, int64_t* n_synapses);
/* Spikes collected by the model's monitors after run() (SpikingActivityMonitor
 * host store): borrowed pointers, valid until the next run/clear. */
int spk_model_spikes(spk_model* m, int32_t population, const int32_t** ids, const float** times,
                     int64_t* n);
int spk_model_clear_spikes(spk_model* m);
/* A RateActivityMonitor on the model's neurons (population SPK_POP_NEURONS) or
 * inputs; its counts after run(): borrowed, valid until the next run/reset. */
int spk_model_add_rate_monitor(spk_model* m, int32_t population);
int spk_model_rate_counts(spk_model* m, int32_t population, const int32_t** counts, int64_t* n);

#ifdef __cplusplus
}
#endif

#endif
