/*
 * spk_oracle.h - CPU restatement of Spike's clock-driven simulation step.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is the checker for the CUDA path: it is
 * called by the tests, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline, and never by the product library.
 *
 * It follows the reference's per-step kernels one for one, on the reference's
 * own data layout (synapse arrays sorted by presynaptic key, per-synapse STDP
 * traces, ring buffer [slot][post*L+label]), single- or multi-threaded:
 *   LIF + injection ........ Spike/Backend/CUDA/Neurons/LIFSpikingNeurons.cu:105-193,
 *                            Spike/Backend/CUDA/InlineDeviceFunctions.hpp:22-111
 *   Poisson inputs ......... Spike/Backend/CUDA/Neurons/PoissonInputSpikingNeurons.cu:96-129
 *   weight-dependent STDP .. Spike/Backend/CUDA/Plasticity/WeightDependentSTDPPlasticity.cu:85-161
 *   propagation ............ Spike/Backend/CUDA/Synapses/SpikingSynapses.cu:127,168-202
 *   step order / run ....... Spike/Models/SpikingModel.cpp:197-236
 * with two substitutions that the CUDA path shares: Philox(seed, input, step)
 * uniforms instead of per-thread XORWOW, and ring contributions applied in the
 * canonical order (step, then sorted synapse index) instead of atomic order.
 */
#ifndef SPK_ORACLE_H
#define SPK_ORACLE_H

#include "../include/spike_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_net oracle_net;

/* precision: 32 = the float path the CUDA kernels must match bit for bit,
 *            64 = the same equations integrated in double (error reports). */
int oracle_create(const spk_net_desc* desc, int precision, oracle_net** out);
int oracle_destroy(oracle_net* net);
/* Worker threads for the step (post-range ownership); 1 = sequential. */
int oracle_set_threads(oracle_net* net, int threads);
int oracle_reset_state(oracle_net* net);
int oracle_reset_time(oracle_net* net);
int oracle_select_stimulus(oracle_net* net, int stimulus);
int oracle_run(oracle_net* net, float seconds, int plasticity_on);
int oracle_run_steps(oracle_net* net, int64_t n_steps, int plasticity_on);
int oracle_current_time(const oracle_net* net, float* seconds);
int oracle_spike_count(const oracle_net* net, int population, int64_t* n);
int oracle_read_spikes(const oracle_net* net, int population, int32_t* ids, float* times,
                       int64_t capacity, int64_t* n_written);
int oracle_clear_spikes(oracle_net* net);
/* Fields as SPK_FIELD_*; values converted to float for the 64-bit twin. */
int oracle_read_state(const oracle_net* net, int field, float* dst, int64_t count);
int oracle_read_weights(const oracle_net* net, float* weights, int64_t n);
int oracle_synaptic_events(const oracle_net* net, uint64_t* events);
/* Ring depth B = D_max + 2G + 1 (SpikingSynapses.cu:48) of the network. */
int oracle_ring_depth(const oracle_net* net, int32_t* depth);
/* Timestep grouping G = the minimum delay (SpikingModel.cpp:98); 1 without synapses. */
int oracle_timestep_grouping(const oracle_net* net, int32_t* G);
/* Sorted-order connectivity as the reference backend sees it after
 * prepare_backend_early (for fixture checks): pre/post/delay in sorted order. */
int oracle_sorted_synapses(const oracle_net* net, int32_t* pre, int32_t* post, int32_t* delay,
                           int64_t n);

/* Synapses of a generated network (spk_gen_desc) in creation order; arrays
 * may be NULL to count.  Returns the synapse count, or -1. */
int64_t oracle_generate(const spk_gen_desc* desc, int32_t* pre, int32_t* post, float* weight, float* scale,
                        int32_t* delay, int32_t* label, uint8_t* plastic, int64_t capacity);

/* The shared counter-based generator and logarithm, for known-answer tests. */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float oracle_logf(float x);
/* Largest error of the shared logarithm, in units of the last place, over
 * every uniform the Poisson draw can produce (k * 2^-24, k = 1..2^24). */
double oracle_log_max_ulp(void);

#ifdef __cplusplus
}
#endif

#endif
