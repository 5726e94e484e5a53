/*
 * spike_gb300.h - C ABI of the GB300-native clock-driven spiking-network step.
 *
 * This is the drop-in boundary for Spike's CUDA backend hot path.  In the
 * reference the path sits behind per-component backend plugins built by a
 * string-keyed factory (Spike/Backend/Macros.hpp:33-70) with the contract
 * prepare()/reset_state() (Spike/Backend/Backend.hpp:15-25) and one
 * state_update() virtual per component.  Here one network handle owns all of
 * the step's device state and the whole step (LIF update + threshold + spike
 * compaction, Poisson input, weight-dependent STDP, delayed propagation) runs
 * in one persistent sm_103a kernel per block of timesteps.
 *
 * Conventions
 *  - every function returns an int status: 0 (SPK_OK) or a negative SPK_ERR_*;
 *    nothing in the library exits the process (the reference calls exit(-1),
 *    Spike/Helpers/TerminalHelpers.hpp:15-20);
 *  - the caller owns every host buffer; descriptor arrays are copied at create;
 *  - a handle owns its device memory and one non-default CUDA stream;
 *  - a handle is single-threaded; distinct handles may be used from distinct
 *    host threads;
 *  - spk_last_error() returns a per-thread message for the last failure.
 *
 * Timestep grouping: the reference advances G = min delay steps per launch
 * (Spike/Models/SpikingModel.cpp:98).  A network whose minimum delay is G > 1
 * steps takes the reference's grouped times (group time start + s*G*dt,
 * substep time that + g*dt) and runs whole groups only: spk_net_run rounds
 * the step count down to whole groups as SpikingModel::run does, the
 * step-count entry points refuse other counts with SPK_ERR_INVALID.  Grouped
 * timesteps change the plasticity rules' arithmetic, which this library does
 * not restate: a network with a rule and G > 1 is rejected with
 * SPK_ERR_UNSUPPORTED.
 */
#ifndef SPIKE_GB300_H
#define SPIKE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPK_ABI_VERSION 4

/* ---- status codes ------------------------------------------------------ */
#define SPK_OK 0
#define SPK_ERR_INVALID (-1)     /* bad argument or descriptor              */
#define SPK_ERR_CUDA (-2)        /* a CUDA runtime call failed              */
#define SPK_ERR_OOM (-3)         /* device or host allocation failed        */
#define SPK_ERR_UNSUPPORTED (-4) /* valid in the reference, not implemented */
#define SPK_ERR_TIMEOUT (-5)     /* a bounded device wait gave up           */
#define SPK_ERR_OVERFLOW (-6)    /* spike store full: spikes were dropped   */
#define SPK_ERR_STATE (-7)       /* call not valid in the handle's state    */
#define SPK_ERR_BUSY (-8)        /* resource temporarily unavailable        */

/* ---- synapse kinds --------------------------------------------------------
 * Same numbering as the reference's SYNAPSE_TYPE enum
 * (Spike/Backend/CUDA/Synapses/SpikingSynapses.hpp:234-240).               */
#define SPK_SYN_CONDUCTANCE 1 /* ConductanceSpikingSynapses */
#define SPK_SYN_CURRENT 2     /* CurrentSpikingSynapses     */
#define SPK_SYN_VOLTAGE 3     /* VoltageSpikingSynapses     */

/* ---- spike populations and state fields -------------------------------- */
#define SPK_POP_NEURONS 0 /* LIF neurons (SpikingModel::spiking_neurons)     */
#define SPK_POP_INPUTS 1  /* Poisson inputs (SpikingModel::input_spiking_neurons) */

#define SPK_FIELD_V 0          /* float[n_neurons] membrane potential            */
#define SPK_FIELD_LAST_SPIKE 1 /* float[n_neurons] last spike time (s)           */
#define SPK_FIELD_SYN_TRACE 2  /* float[n_neurons*n_labels] conductance/current  */
#define SPK_FIELD_INPUT_NEXT 3 /* float[n_inputs] next Poisson spike time (s)    */
#define SPK_FIELD_RING 4       /* float[B*n_neurons*n_labels], [slot][post*L+l]  */
#define SPK_FIELD_PRE_TRACE 5  /* float[n_inputs+n_neurons] STDP pre trace, inputs first */
#define SPK_FIELD_POST_TRACE 6 /* float[n_neurons] STDP post trace               */

/* One LIF neuron group (lif_spiking_neuron_parameters_struct,
 * Spike/Neurons/LIFSpikingNeurons.hpp:7-14).  tau_m and R are the front end's
 * float values C_m/g_0 and 1/g_0 (Spike/Neurons/LIFSpikingNeurons.cpp:29-30);
 * the library derives k = dt/tau_m and k*R as the reference backend does
 * (Spike/Backend/CUDA/Neurons/LIFSpikingNeurons.cu:26-46). */
typedef struct spk_neuron_group {
  int32_t start; /* first neuron id of the group        */
  int32_t count; /* neurons in the group                */
  float tau_m;
  float R;
  float v0;     /* resting_potential_v0                */
  float vreset; /* after_spike_reset_potential_vreset  */
  float theta;  /* threshold_for_action_potential_spike */
  /* Extension (not in the reference, which resets V to v0): when
   * v_init_lo < v_init_hi, reset draws V ~ U[lo, hi) from Philox keyed by
   * (seed, neuron, SPK_DOMAIN_VINIT). */
  float v_init_lo;
  float v_init_hi;
} spk_neuron_group;

/* STDP rules (spk_net_desc.stdp_rule).  The weight-dependent rule is
 * event-driven; the Evans and inhibitory rules keep two traces per plastic
 * synapse and update every plastic synapse every timestep, seeing a
 * presynaptic spike when it arrives (its delay after it was fired), as the
 * reference's bit-buffer kernels do.  They run in bulk mode only. */
#define SPK_STDP_WEIGHT_DEPENDENT 0 /* WeightDependentSTDPPlasticity */
#define SPK_STDP_EVANS 1            /* EvansSTDPPlasticity (Spike/Plasticity/EvansSTDPPlasticity.hpp) */
#define SPK_STDP_INHIBITORY 2       /* InhibitorySTDPPlasticity (Vogels et al. 2011,
                                       Spike/Plasticity/InhibitorySTDPPlasticity.hpp) */
#define SPK_STDP_CUSTOM 3           /* CustomSTDPPlasticity (Spike/Plasticity/CustomSTDPPlasticity.hpp) */

/* Position of the weight normalisation among the model's plasticity rules
 * (SpikingModel::perform_per_step_model_instructions runs them in the order
 * added, Spike/Models/SpikingModel.cpp:202-205). */
#define SPK_NORM_OFF 0
#define SPK_NORM_AFTER_RULE 1       /* added after the STDP rule (normalises this step's updates) */
#define SPK_NORM_BEFORE_RULE 2      /* added before it */

/* weightdependent_stdp_plasticity_parameters_struct
 * (Spike/Plasticity/WeightDependentSTDPPlasticity.hpp:28-40).  The other
 * rules reuse the fields:
 *   SPK_STDP_EVANS       tau_minus = decay_term_tau_D, tau_plus = decay_term_tau_C,
 *                        a_minus = model_parameter_alpha_D,
 *                        a_plus = synaptic_neurotransmitter_concentration_alpha_C
 *                        (weights clipped to [0, 1]);
 *   SPK_STDP_INHIBITORY  tau_plus = tau_istdp, lambda = learningrate,
 *                        alpha = targetrate (weights clipped at 0);
 *   SPK_STDP_CUSTOM      a_minus, a_plus, tau_minus, tau_plus, w_max as named,
 *                        lambda = learning_rate, alpha = a_star,
 *                        clip_upper = nearest_spike_only (weights clipped at 0). */
typedef struct spk_stdp_params {
  float a_minus;
  float a_plus;
  float tau_minus;
  float tau_plus;
  float lambda;
  float alpha;
  float w_max;
  int32_t clip_upper; /* extension: also clip weights at w_max (reference clips at 0 only) */
} spk_stdp_params;

/* Flat network descriptor.  Synapse arrays are in CREATION order, with the
 * reference's presynaptic id convention: LIF neuron n -> n, input i -> -i-1
 * (Spike/Neurons/Neurons.hpp:34-35).  The library sorts them by presynaptic
 * key (inputs first in reverse order, then neurons) with a stable sort, exactly
 * as Synapses::sort_synapses does (Spike/Synapses/Synapses.cpp:33-81), and
 * keeps the reverse map for weight readback in creation order. */
typedef struct spk_net_desc {
  int32_t abi_version; /* must be SPK_ABI_VERSION */
  float dt;            /* SpikingModel::timestep (s) */
  int32_t synapse_kind;

  int32_t n_neurons;
  int32_t n_groups;
  const spk_neuron_group* groups; /* contiguous, ascending, covering [0,n_neurons) */
  float refractory_period;        /* global, from the last group added (reference quirk) */
  float background_current;       /* global, from the last group added (reference quirk) */

  int32_t n_inputs;           /* Poisson input neurons (0 allowed) */
  int32_t n_stimuli;          /* rate vectors; >= 1 when n_inputs > 0 */
  const float* input_rates;   /* [n_stimuli][n_inputs] Hz */
  int32_t stimulus;           /* selected stimulus */

  int32_t n_labels;           /* syn labels L (>= 1) */
  const float* label_tau;     /* [L] tau_g (conductance) or tau (current); unused for voltage */
  const float* label_vhat;    /* [L] reversal potentials (conductance only) */

  int64_t n_synapses;
  const int32_t* pre;
  const int32_t* post;
  const float* weight;        /* synaptic_efficacies_or_weights */
  const float* scale;         /* weight_scaling_constants */
  const int32_t* delay;       /* in timesteps, >= 1 */
  const int32_t* label;       /* syn_labels, < L */
  const uint8_t* plastic;     /* 1 = governed by the STDP rule; may be NULL */

  int32_t has_stdp;
  spk_stdp_params stdp;

  uint64_t seed;              /* Philox key (Poisson draws, V init) */
  int64_t spike_capacity;     /* device spike store entries; 0 = default */
  int32_t record_inputs;      /* also record input spikes */
  int32_t stdp_rule;          /* SPK_STDP_*; 0 = weight-dependent */
  /* Weight normalisation over the plastic synapses (WeightNormSTDPPlasticity,
   * Spike/Plasticity/WeightNormSTDPPlasticity.cpp): SPK_NORM_*.  Needs an
   * STDP rule on the same synapses; runs when plasticity is on. */
  int32_t weight_norm;
  const float* norm_initial;  /* per synapse, creation order: the rule's initial_weights
                                 (NULL: the weights) */
  const float* norm_sum;      /* per neuron: sum_squared_afferent_values (NULL: the sum of
                                 powf(w, 2) over its plastic afferents in creation order) */
} spk_net_desc;

/* Launch schedule.  Zero fields are chosen by the library (planner for a
 * single network, autotuner for a batch). */
typedef struct spk_schedule {
  int32_t warps_per_cta;    /* warps in one CTA; each warp owns one post tile   */
  int32_t tile_posts;       /* posts per tile, multiple of 32                   */
  int32_t ctas;             /* CTAs per network (1 = CTA-per-network schedule)  */
  int32_t steps_per_launch; /* timesteps advanced by one persistent launch      */
} spk_schedule;

typedef struct spk_net spk_net;
typedef struct spk_batch spk_batch;

/* ---- single network -----------------------------------------------------
 * spk_net_create replaces SpikingModel::finalise_model -> init_backend ->
 * every component's prepare() (Spike/Models/SpikingModel.cpp:82-162,
 * Spike/Backend/Macros.hpp:21-39) and ends with reset_state(). */
int spk_net_create(const spk_net_desc* desc, const spk_schedule* schedule, spk_net** out);
/* Replaces the backend destructors' cudaFree calls. */
int spk_net_destroy(spk_net* net);
/* SpikingModel::reset_state (Spike/Models/SpikingModel.cpp:181-190). */
int spk_net_reset_state(spk_net* net);
/* SpikingModel::reset_time (Spike/Models/SpikingModel.cpp:192-194). */
int spk_net_reset_time(spk_net* net);
/* InputSpikingNeurons::select_stimulus + reset of the inputs
 * (Spike/Neurons/PoissonInputSpikingNeurons.cpp:48-51). */
int spk_net_select_stimulus(spk_net* net, int32_t stimulus);
/* PatternedPoissonInputSpikingNeurons::copy_rates_to_device
 * (Spike/Backend/CUDA/Neurons/PatternedPoissonInputSpikingNeurons.cu:13-18):
 * overwrite the rates of one stimulus (n_inputs floats, Hz) with an
 * asynchronous host-to-device copy on the handle's stream (pinned host memory
 * makes it truly asynchronous).  Input state is not reset. */
int spk_net_write_rates(spk_net* net, int32_t stimulus, const float* rates, int64_t n);
/* SpikingModel::run(seconds, plasticity_on) (Spike/Models/SpikingModel.cpp:214-236):
 * ceilf(seconds/dt) steps rounded down to whole groups of G, t_s = start +
 * (s - s%G)*dt + (s%G)*dt in float, then time = start + seconds.
 * Asynchronous: returns after enqueueing; device errors surface at the next
 * synchronizing call. */
int spk_net_run(spk_net* net, float seconds, int32_t plasticity_on);
/* As spk_net_run for an explicit step count (time advances by n_steps*dt);
 * n_steps must be whole groups of the timestep grouping. */
int spk_net_run_steps(spk_net* net, int64_t n_steps, int32_t plasticity_on);
/* Start a run of n_steps steps (time advances by n_steps*dt, as in
 * spk_net_run_steps) without launching it; spk_batch_step_block then advances
 * it a block at a time (the server's continuous batching). */
int spk_net_begin_run(spk_net* net, int64_t n_steps, int32_t plasticity_on);
/* Wait for the handle's stream; returns the device status word
 * (SPK_ERR_TIMEOUT / SPK_ERR_OVERFLOW / SPK_ERR_UNSUPPORTED) or SPK_OK.
 *
 * Run boundaries follow the reference's double-buffered active lists
 * (Spike/Backend/CUDA/Synapses/SpikingSynapses.cu:156-202): list (T/G) % 2 is
 * emptied only by a group step of the other parity, so a run whose first
 * group index T/G has the parity of the last group step's (the timestep index
 * repeats at a run start when seconds/dt has a fraction below one half, as
 * for run(0.1) at dt = 1e-4; a grouped network skips one) delivers the last
 * group's spikes again in its substeps, merged with their own (a key in both
 * once).  The same happens within a run where t/dt falls within rounding of
 * a half.  Were the list to hold two or more earlier groups (two such
 * repeats in a row), SPK_ERR_UNSUPPORTED is raised and only the last group is
 * delivered again. */
int spk_net_synchronize(spk_net* net);
int spk_net_current_time(const spk_net* net, float* seconds);
/* SpikingModel::timestep_grouping (Spike/Models/SpikingModel.cpp:98): the
 * network's minimum delay in steps (1 without synapses). */
int spk_net_timestep_grouping(const spk_net* net, int32_t* G);
/* Spikes recorded since the last clear (SpikingActivityMonitor store,
 * Spike/ActivityMonitor/SpikingActivityMonitor.cpp:79-120).  Ordered by
 * step, then by presynaptic key (the canonical order).  times are the float
 * step times t_s the reference stores. */
int spk_net_spike_count(spk_net* net, int32_t population, int64_t* n);
int spk_net_read_spikes(spk_net* net, int32_t population, int32_t* ids, float* times,
                        int64_t capacity, int64_t* n_written);
int spk_net_clear_spikes(spk_net* net);
/* Rate monitor (RateActivityMonitor, Spike/ActivityMonitor/RateActivityMonitor.cpp
 * and Spike/Backend/CUDA/ActivityMonitor/RateActivityMonitor.cu:50-71): the
 * spikes of every neuron (or input) of `population` since the last clear or
 * reset, counted on the device as the spikes are decided.  count must be the
 * population's size; counts[i] is neuron (input) i's. */
int spk_net_rate_counts(spk_net* net, int32_t population, int32_t* counts, int64_t count);
int spk_net_clear_rate_counts(spk_net* net);
/* Read one state field (SPK_FIELD_*) into dst (count elements). */
int spk_net_read_state(spk_net* net, int32_t field, void* dst, int64_t count);
/* Backend::Synapses::copy_to_frontend / copy_to_backend
 * (Spike/Synapses/Synapses.hpp:54-55): weights in creation order. */
int spk_net_read_weights(spk_net* net, float* weights, int64_t n);
int spk_net_write_weights(spk_net* net, const float* weights, int64_t n);
/* Synaptic events delivered so far: sum over spikes of the spiking neuron's
 * out-degree. */
int spk_net_synaptic_events(spk_net* net, uint64_t* events);
/* STDP work done so far: plastic weights updated on a presynaptic event
 * (propagation pass) and plastic afferents updated on a postsynaptic spike
 * (afferent pass); for byte accounting. */
int spk_net_stdp_counts(spk_net* net, uint64_t* pre_updates, uint64_t* post_updates);
int spk_net_get_schedule(const spk_net* net, spk_schedule* out);
/* Snapshot of a network's dynamic state (no counterpart in the reference,
 * which saves weights and connectivity only): membrane potentials, last spike
 * times, synaptic traces, the delay ring, Poisson next-spike times, STDP
 * traces and plastic weights, the run counters and the current time.  It
 * restores into a network created from the same descriptor with the same
 * schedule (checked); the spike store is not saved (it restarts empty).  The
 * state holds no random-generator state: draws are keyed by (seed, neuron,
 * step). */
int spk_net_snapshot_bytes(spk_net* net, int64_t* bytes);
int spk_net_snapshot(spk_net* net, void* buffer, int64_t bytes);
int spk_net_restore(spk_net* net, const void* buffer, int64_t bytes);
/* Limit of every device-side wait of one CTA on another (default 4 s).  A
 * wait that runs out ends the run with SPK_ERR_TIMEOUT, returned by
 * spk_net_synchronize; the network is usable again after
 * spk_net_reset_state, which clears the failure. */
int spk_net_set_wait_limit(spk_net* net, double seconds);
/* Failure injection for testing (no counterpart in the reference, which has
 * no failure detection): the next launch of the network leaves out CTA
 * `rank`, so the other CTAs' bounded waits on it run out.  The fault is made
 * on the host (a CTA that never runs); nothing on the device faults. */
int spk_net_inject_withheld_cta(spk_net* net, int32_t rank);
int spk_net_device_bytes(const spk_net* net, int64_t* bytes);
/* Kernel launches issued so far by this handle. */
int spk_net_launch_count(const spk_net* net, int64_t* launches);
/* The handle's CUDA stream (a cudaStream_t), for callers that order their own
 * work or timing events against the engine. */
int spk_net_stream(const spk_net* net, void** stream);

/* ---- networks generated on the device -------------------------------------
 * Replaces the host connectivity builder for large networks: the reference
 * draws every (pre, post) pair of a RANDOM synapse group with rand() on the
 * host and grows its synapse arrays with one realloc per synapse
 * (Spike/Synapses/Synapses.cpp:208-228, 391-421), which takes minutes at
 * 1e8-1e9 synapses.  Here each projection connects every (pre, post) pair of
 * its rectangle with probability p, draws weight ~ U(lo, hi] and an integer
 * delay ~ U{lo..hi}, all from Philox keyed by (connectivity_seed, pre, post),
 * and the GPU writes the engine's CSR directly.
 *
 * Projections may not overlap in (pre, post), so a pair has at most one
 * synapse and its draws do not depend on how projections are listed.  The
 * synapse (creation) order of a generated network is ascending presynaptic
 * key, then post: inputs n_inputs-1 .. 0, then neurons 0 .. n_neurons-1.
 * spk_net_read_weights returns, in that order, the value each synapse
 * delivers: weight*scale for static synapses, the weight for plastic ones
 * (whose scale is applied on delivery); spk_net_write_weights is not
 * available for generated networks. */
typedef struct spk_projection {
  int32_t pre_population; /* SPK_POP_NEURONS or SPK_POP_INPUTS */
  int32_t pre_start;      /* first presynaptic index within that population */
  int32_t pre_count;
  int32_t post_start;     /* first postsynaptic neuron */
  int32_t post_count;
  float probability;      /* per pair, in [0, 1] */
  float weight_lo, weight_hi;
  float scale;            /* weight_scaling_constant */
  int32_t delay_lo, delay_hi; /* timesteps, 1 <= lo <= hi <= 255 */
  int32_t label;
  int32_t plastic;        /* governed by the STDP rule (needs has_stdp) */
} spk_projection;

typedef struct spk_gen_desc {
  int32_t abi_version;
  float dt;
  int32_t synapse_kind;
  int32_t n_neurons;
  int32_t n_groups;
  const spk_neuron_group* groups;
  float refractory_period;
  float background_current;
  int32_t n_inputs;
  int32_t n_stimuli;
  const float* input_rates; /* [n_stimuli][n_inputs] Hz */
  int32_t stimulus;
  int32_t n_labels;
  const float* label_tau;
  const float* label_vhat;
  int32_t n_projections;
  const spk_projection* projections;
  int32_t has_stdp;
  spk_stdp_params stdp;
  uint64_t seed;              /* Poisson draws and V init, as in spk_net_desc */
  uint64_t connectivity_seed; /* connection, weight and delay draws */
  int64_t spike_capacity;
  int32_t record_inputs;
  int32_t stdp_rule;          /* SPK_STDP_* of the plastic projections (the weight
                                 normalisation needs a host-built network) */
} spk_gen_desc;

int spk_net_generate(const spk_gen_desc* desc, const spk_schedule* schedule, spk_net** out);
/* Synapses of a network (created or generated). */
int spk_net_synapse_count(const spk_net* net, int64_t* n);
/* Synapses under the STDP rule (STDPPlasticity::total_number_of_plastic_synapses). */
int spk_net_plastic_synapse_count(const spk_net* net, int64_t* n);

/* ---- batch: many independent networks in one persistent launch ---------- */
/* The networks stay usable on their own between batch runs: a network may be
 * run alone, reset, snapshotted or restored, switch stimulus or change its
 * wait limit, and the next batch run starts from that state (the batch brings
 * its copies of the networks' descriptors up to date before it launches). */
int spk_batch_create(spk_net* const* nets, int32_t n_nets, const spk_schedule* schedule,
                     spk_batch** out);
int spk_batch_run_steps(spk_batch* batch, int64_t n_steps, int32_t plasticity_on);
/* Execution mode of a batch.  WAVES (default): the persistent step kernel,
 * each network's state in shared memory for a whole launch, networks packed
 * into co-resident waves.  BULK: every timestep is a few kernels over all
 * tiles of all networks (neurons, the step's key lists, propagation with
 * STDP, the afferent pass, and the per-synapse-trace rules' and weight
 * normalisation's passes where a network has them), state in HBM, kernel
 * boundaries as the only synchronization, captured in a CUDA graph per block;
 * it suits batches whose networks do not fit the GPU's shared memory at once,
 * and networks with a per-synapse-trace rule or the weight normalisation run
 * in it only.  Both modes give the same bits. */
#define SPK_BATCH_WAVES 0
#define SPK_BATCH_BULK 1
int spk_batch_set_mode(spk_batch* batch, int32_t mode);
/* One round of the batch's launches: every network advances up to
 * steps_per_launch steps of the run it was given with spk_net_begin_run
 * (networks whose run is complete do nothing).  A run split this way gives the
 * same result as the same run made in one call. */
int spk_batch_step_block(spk_batch* batch);
/* As spk_batch_run_steps with a step count and a plasticity switch per
 * network (index i = the i-th network given to spk_batch_create;
 * plasticity_on may be NULL: on for all); each network's time advances by its
 * own count. */
int spk_batch_run_steps_each(spk_batch* batch, const int64_t* n_steps, const int32_t* plasticity_on);
int spk_batch_synchronize(spk_batch* batch);
int spk_batch_launch_count(const spk_batch* batch, int64_t* launches);
/* Per-kernel timing of a batch in bulk mode (no counterpart in the
 * reference, whose examples time run() as a whole): advances the batch by
 * n_steps exactly as spk_batch_run_steps does, but launches every kernel on
 * its own, one after another on the batch stream (no graph, no programmatic
 * overlap, the afferent pass not beside propagation), between two CUDA
 * events, and adds each kind's device time in milliseconds to
 * ms[SPK_KERNEL_KINDS].  A diagnostic: the sum exceeds the graph-launched
 * time by the overlap it removes. */
#define SPK_KERNEL_NEURONS 0     /* LIF, Poisson inputs, traces, spike words */
#define SPK_KERNEL_LIST 1        /* the step's canonical key lists, spike store */
#define SPK_KERNEL_RULES 2       /* per-synapse-trace rules, weight normalisation */
#define SPK_KERNEL_POST 3        /* post-spike afferent pass (a second stream) */
#define SPK_KERNEL_PROPAGATION 4 /* delayed propagation and the STDP pre pass */
#define SPK_KERNEL_FINISH 5      /* run counters, once per block */
#define SPK_KERNEL_KINDS 6
int spk_batch_time_kernels(spk_batch* batch, int64_t n_steps, int32_t plasticity_on, double* ms);
int spk_batch_stream(const spk_batch* batch, void** stream);
/* Spikes of every network of the batch in one call: network after network,
 * each exactly as spk_net_read_spikes gives it (canonical order), gathered on
 * the device and copied with one transfer for ids and one for times (page-
 * locked ids/times buffers make it a direct DMA).  counts[n_nets] receives each
 * network's number of spikes of `population`; ids/times hold their sum.  If
 * the sum exceeds capacity nothing is copied and SPK_ERR_OVERFLOW is returned
 * (counts are still set).  clear != 0 then empties every network's store, as
 * spk_net_clear_spikes.  Replaces, for a batch, spk_net_spike_count +
 * spk_net_read_spikes + spk_net_clear_spikes per network (the monitor readback
 * of Spike/ActivityMonitor/SpikingActivityMonitor.cpp:79-153, done once for all
 * networks). */
int spk_batch_read_spikes(spk_batch* batch, int32_t population, int32_t* ids, float* times,
                          int64_t capacity, int64_t* counts, int32_t clear);
int spk_batch_destroy(spk_batch* batch);
/* Measured schedule search for a batch of generated networks (batching has
 * no counterpart in the reference).  Tries a fixed set of policies (warps per
 * CTA, largest tile), builds the networks under each, times trial_steps steps
 * of the batch in both execution modes (spk_batch_set_mode) and writes the
 * fastest policy's schedule of every network to schedules[n_nets], its trial
 * time to best_ms and its mode to best_mode (both may be NULL).  With step_us
 * (may be NULL) and the waves mode chosen it also times each network alone
 * under its schedule and writes microseconds per step, for
 * spk_net_set_step_cost (zeros for the bulk mode, which packs no waves).
 * Results never depend on the schedule or the mode.  Destroy a batch before
 * the networks it holds. */
int spk_batch_autotune(const spk_gen_desc* descs, int32_t n_nets, int32_t trial_steps,
                       spk_schedule* schedules, float* best_ms, float* step_us, int32_t* best_mode);
/* Cost of one step of the network (any unit, e.g. the step_us above).  A
 * batch orders its networks by decreasing cost into its co-resident waves, so
 * that each wave - which lasts as long as its slowest member - holds networks
 * of similar cost; without costs it orders by shared memory and CTA count. */
int spk_net_set_step_cost(spk_net* net, float cost);

/* ---- simulation server: continuous batching (no counterpart in the
 * reference) ---------------------------------------------------------------
 * A server owns one host thread that drives the GPU.  Submitted jobs (a
 * generated network and a step count) wait in a FIFO queue until the free
 * device memory, less a reserve, holds their estimated footprint; then their
 * network is generated on the device and joins the running set.  The running
 * set advances in step blocks through one batch (co-resident waves of the
 * persistent step kernel), each job by min(its remaining steps, the block);
 * jobs admitted while a block runs join at the next block, and a finished
 * job's spikes and counters are copied to the host and its device memory is
 * freed.  A job's result does not depend on what else runs with it. */
typedef struct spk_server spk_server;

typedef struct spk_server_opts {
  int32_t warps_per_cta;   /* schedule policy of admitted jobs (0 = 8)            */
  int32_t tile_posts;      /* largest tile (0 = 64)                                */
  int32_t steps_per_block; /* timesteps per batch round (0 = 1000)                 */
  int32_t max_running;     /* running jobs at most (0 = 512)                       */
  uint64_t reserve_bytes;  /* device memory kept free (0 = 8 GiB)                  */
  int32_t record_spikes;   /* keep each finished job's neuron spikes on the host   */
  int32_t mode;            /* batch execution mode, SPK_BATCH_WAVES (0) or _BULK    */
} spk_server_opts;

#define SPK_JOB_QUEUED 0
#define SPK_JOB_RUNNING 1
#define SPK_JOB_DONE 2
#define SPK_JOB_FAILED 3
#define SPK_JOB_CANCELLED 4

typedef struct spk_job_info {
  int32_t state;        /* SPK_JOB_* */
  int32_t error;        /* SPK_ERR_* of a failed job */
  int64_t steps_done;
  int64_t steps_total;
  uint64_t events;      /* synaptic events delivered */
  int64_t spikes;       /* neuron spikes */
  int64_t synapses;
  double submit_s;      /* seconds since the server started */
  double start_s;       /* admitted (network generated) */
  double finish_s;
} spk_job_info;

typedef struct spk_server_stats {
  int64_t submitted, running, queued, done, failed;
  uint64_t events;      /* all jobs, delivered so far */
  int64_t blocks;       /* batch rounds run */
  double busy_s;        /* wall time with at least one job running */
  double uptime_s;
  int64_t rebuilds;     /* batches built: at the first block and whenever jobs join */
} spk_server_stats;

int spk_server_start(const spk_server_opts* opts, spk_server** out);
/* Copies the descriptor (and every array it points to); returns the job id. */
int spk_server_submit(spk_server* server, const spk_gen_desc* desc, int64_t n_steps, int32_t plasticity_on,
                      int64_t* job);
int spk_server_poll(spk_server* server, int64_t job, spk_job_info* info);
/* Block until the job is done, failed or cancelled, or timeout_s passes
 * (SPK_ERR_BUSY). */
int spk_server_wait(spk_server* server, int64_t job, double timeout_s);
/* Neuron spikes of a finished job (needs record_spikes), ordered by step then
 * neuron. */
int spk_server_read_spikes(spk_server* server, int64_t job, int32_t* ids, float* times, int64_t capacity,
                           int64_t* n_written);
/* A queued job is dropped; a running one is stopped at the end of its block. */
int spk_server_cancel(spk_server* server, int64_t job);
/* Forget a finished job's results. */
int spk_server_release(spk_server* server, int64_t job);
int spk_server_stats_get(spk_server* server, spk_server_stats* stats);
/* Finishes nothing further: running and queued jobs are cancelled, the
 * thread joins and every device allocation of the server is freed. */
int spk_server_stop(spk_server* server);

/* Device memory a generated network will hold under a schedule (NULL = the
 * planner's), from its projections' expected synapse counts plus six
 * standard deviations, and the peak while it is generated. */
int spk_net_generate_estimate(const spk_gen_desc* desc, const spk_schedule* schedule, int64_t* device_bytes,
                              int64_t* peak_bytes);

/* ---- allocation-free stepping --------------------------------------------
 * This entry point has no counterpart in the reference.  It is for callers
 * that cannot call cudaMalloc at the point where they step a network: code
 * that runs under another framework's memory allocator (which owns every
 * device allocation of the process), real-time or embedded hosts where device
 * allocation is forbidden after start-up, and plug-ins that only receive
 * device buffers from their host application.  The caller owns every input and
 * output buffer below; the only extra device memory the step needs, the
 * per-step exchange between CTAs and the launch descriptors, is a fixed
 * SPK_NOALLOC_SCRATCH_BYTES array inside the library that every GPU loading
 * the library holds until the process exits.
 *
 * Buffer layout (the layout spk_net_create builds for the same schedule):
 *  - keys: input i has key Nin-1-i, neuron n has key KL+n, with
 *    T = warps_per_cta*ctas tiles, ITS = 32*ceil(ceil(Nin/T)/32), KL = T*ITS,
 *    n_keys = KL + T*tile_posts; a synapse's tile is post / tile_posts;
 *  - rowptr[n_keys*T + 1]: start of each (key, tile) sub-row, exclusive prefix;
 *  - entries[S] (pairs of uint32): sub-rows in (key, tile) order, synapses of
 *    one sub-row in creation order; x = post%tile_posts | delay<<16 |
 *    label<<24 | class<<28, y = float bits of weight*scale (class 0) or, for
 *    a plastic synapse (class c >= 1, scale = plastic_scales[c-1]), the index
 *    of its afferent record in csc;
 *  - csc_ptr[N+1], csc[2*P]: the plastic afferent records of each post in
 *    creation order, as (presynaptic key, float bits of the weight), needed
 *    only with plasticity;
 *  - state: V, last_spike [N]; syn_trace [N*L] (conductance/current);
 *    ring [T][max_delay+2G+1][tile_posts*L] (G = timestep_grouping, at
 *    least 1); input_next [Nin]; rates [Nin];
 *    post_trace [N] and pre_trace [n_keys] with plasticity;
 *  - spikes [2*spike_capacity] uint32 pairs (key, float time bits), in
 *    step order; spike_capacity 0 records nothing;
 *  - run_state: SPK_RUN_STATE_BYTES of device memory (8-byte aligned), zeroed
 *    by the caller before the first call; it carries the step counter and
 *    Poisson activity from call to call, and holds the spikes recorded so far
 *    (uint64 at byte 32; zero it to clear the store), the synaptic events
 *    delivered (uint64 at byte 40) and the device status (int32 at byte 48: 0,
 *    SPK_ERR_TIMEOUT, SPK_ERR_OVERFLOW or SPK_ERR_UNSUPPORTED, the last for
 *    an active list of two carried groups, see spk_net_synchronize), valid
 *    once the stream has finished.
 *    A non-zero status stays in run_state across later calls until the caller
 *    clears it.  After SPK_ERR_OVERFLOW the state is sound (only spikes beyond
 *    spike_capacity were dropped): zero the status and the spike count to go
 *    on.  After SPK_ERR_TIMEOUT the CTAs stopped at different timesteps, so
 *    the state buffers (V, last_spike, syn_trace, ring, input_next, the STDP
 *    traces and plastic weights) are inconsistent: reload them from a copy
 *    taken before the call and zero run_state before the next call.
 *
 * The first call on a device resolves the scratch array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  Every call shares the one scratch array and
 * clears the parts that must start at zero, so calls whose work overlaps on
 * the GPU (different streams, or different host threads on one device) race
 * and must be serialized by the caller.  Networks whose scratch exceeds
 * SPK_NOALLOC_SCRATCH_BYTES, and time constants that are not positive (tau_m,
 * label taus, STDP taus) or a negative refractory period, are rejected with
 * SPK_ERR_INVALID before any device work.  Plasticity
 * here is the weight-dependent rule (the persistent kernel's); the
 * per-synapse-trace rules and the weight normalisation need a network from
 * spk_net_create. */
#define SPK_NOALLOC_SCRATCH_BYTES (4u << 20)
#define SPK_RUN_STATE_BYTES 128

typedef struct spk_device_net {
  /* shape, schedule and constants (host values) */
  int32_t n_neurons, n_inputs, n_labels, synapse_kind, max_delay;
  int32_t warps_per_cta, tile_posts, ctas;
  float dt, refractory_period, background_current;
  int32_t n_groups;
  const spk_neuron_group* groups; /* host array; v_init_* ignored (state is the caller's) */
  const float* label_tau;         /* host [L] */
  const float* label_vhat;        /* host [L] */
  int32_t has_stdp;
  spk_stdp_params stdp;
  int32_t n_plastic_scales;       /* classes 1..n (<= 15) */
  const float* plastic_scales;    /* host [n_plastic_scales] */
  uint64_t seed;
  int32_t record_inputs;
  /* caller-owned device buffers */
  const int32_t* rowptr;
  uint32_t* entries;
  const int32_t* csc_ptr;
  uint32_t* csc;
  float* V;
  float* last_spike;
  float* syn_trace;
  float* ring;
  float* input_next;
  const float* rates;
  float* post_trace;
  float* pre_trace;
  uint32_t* spikes;
  int64_t spike_capacity;
  void* run_state;
  /* timestep grouping G (Spike/Models/SpikingModel.cpp:98: the minimum delay
   * in steps); 0 or 1 = none.  G > 1 needs has_stdp = 0 and n_steps a
   * multiple of G (the reference's run() advances whole groups). */
  int32_t timestep_grouping;
  /* [G * n_keys/32] spike words of each substep of the last group, zeroed by
   * the caller with run_state: a call whose first group index has the parity
   * of the last group's delivers that group's spikes again, as the
   * reference's double-buffered active lists do
   * (Spike/Backend/CUDA/Synapses/SpikingSynapses.cu:179-182). */
  uint32_t* group_bits;
} spk_device_net;

/* Advance the network n_steps timesteps from start_time (seconds) on `stream`
 * (a cudaStream_t; NULL = the legacy default stream), as spk_net_run_steps
 * does for a network created by spk_net_create.  Asynchronous; allocates no
 * device or host memory. */
int spk_step_noalloc(const spk_device_net* net, int64_t n_steps, int32_t plasticity_on, float start_time,
                     void* stream);

/* ---- misc ---------------------------------------------------------------- */
/* Backend::MemoryManager::{free_bytes,total_bytes}
 * (Spike/Backend/CUDA/Helpers/Memory.cu:7-25), returning a status instead of
 * exit(1). */
int spk_memory_info(uint64_t* free_bytes, uint64_t* total_bytes);
int spk_abi_version(void);
const char* spk_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* SPIKE_GB300_H */
