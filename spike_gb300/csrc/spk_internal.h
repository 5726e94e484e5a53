// spk_internal.h - host/device shared definitions of the step engine.
#pragma once

#include <math.h>
#include <stdint.h>
#include <vector_types.h>

#include "spk_error.h"
#include "spk_rng.h"

namespace spk {

constexpr int MAX_GROUPS = 16;  // LIF groups per network
constexpr int MAX_LABELS = 15;  // syn labels (4-bit field)
constexpr int MAX_CLASSES = 16; // scale classes: 0 = pre-multiplied, 1..15 plastic
constexpr int MAX_DELAY = 255;  // 8-bit delay field
constexpr int LIST_CAP = 1024;     // active presynaptic keys listed per round
constexpr int WPT_MAX = 16;        // bitmap words held per thread while listing
constexpr int STAGE_KEYS = 64;     // sub-rows staged per warp per round
constexpr int STAGE_ENTRIES = 256; // synapse entries staged per warp per round
constexpr int APPLY_TAGS = 256;    // cell-hash slots of the ordered apply

// Packed synapse entry: x = post_local[0:16) | delay[16:24) | label[24:28) |
// class[28:32), y = float bits of w*scale for class 0; for a plastic class
// (>= 1) y is the index of the synapse's afferent record in the CSC, which
// holds its weight (post-major, so a spiking post's afferents are contiguous).
SPK_HD uint32_t pack_entry(uint32_t post_local, uint32_t delay, uint32_t label, uint32_t cls) {
  return post_local | (delay << 16) | (label << 24) | (cls << 28);
}

// The times of timestep r of a run started at `start` seconds, with timestep
// grouping G: the group's current_time_in_seconds = starttime +
// s*timestep_grouping*timestep for group s = r / G
// (Spike/Models/SpikingModel.cpp:226), the timestep index roundf(t/dt) + g of
// substep g = r % G (Spike/Backend/CUDA/Neurons/LIFSpikingNeurons.cu:115,
// Spike/Backend/CUDA/Synapses/ConductanceSpikingSynapses.cu:113) and the
// substep's time t + g*timestep (LIFSpikingNeurons.cu:172,177; the spike
// monitor's time, Spike/Backend/CUDA/ActivityMonitor/SpikingActivityMonitor.cu:93).
SPK_HD void group_time(float start, int r, int G, float dt, float& t, int& T, float& tg) {
  const int s = G == 1 ? r : r / G, g = r - s * G;
  t = start + (float)(s * G) * dt;
  T = (int)roundf(t / dt) + g;
  tg = t + (float)g * dt;
}

struct GroupConst {
  int start, end;  // [start, end)
  float k, kR, v0, vreset, theta;
};

// Device-resident run control of one network.
struct RunCtl {
  float start_time;     // SpikingModel::current_time at run() entry
  int step;             // steps done in the current run
  int steps_total;      // steps in the current run
  int plastic;          // plasticity_on for this run (and the net has STDP)
  int inputs_active;    // Poisson 'active' flags (all equal, see reset)
  int record_inputs;
  long long gstep;      // steps since creation (bitmap / trace parity)
  unsigned long long spike_count;  // entries in the spike store
  unsigned long long events;       // synaptic events delivered
  int status;           // 0 or SPK_ERR_* raised on the device
  int pad;
  unsigned long long stdp_pre;     // plastic weights updated on a presynaptic event
  unsigned long long stdp_post;    // plastic afferents updated on a postsynaptic spike
  // The reference's two active-neuron lists
  // (Spike/Backend/CUDA/Synapses/SpikingSynapses.cu:156-202) are double-buffered
  // by the parity of the group index T/G: a group step appends its spikes to
  // list (T/G) % 2, delivers that whole list and empties the other one, so
  // consecutive group steps with indices of equal parity deliver the earlier
  // group's spikes again.  The index comes from the float time (roundf(t/dt)),
  // so it can repeat or skip one where a run starts and, when t/dt falls near
  // a half, within a run.  State of the lists across runs:
  int repeat;           // the current run's first group repeats the last group step's parity
  int last_group_p1;    // 1 + index of the last group step before the current run; 0: none
  int last_run_groups;  // groups of the run that ended with it
  int last_run_repeat;  // that run began by delivering a carried group again
};

// Index T/G of the group of timestep r of a run started at `start`.
SPK_HD int group_index(float start, int r, int G, float dt) {
  const int s = r / G;
  const float t = start + (float)(s * G) * dt;
  return (int)roundf(t / dt) / G;
}

// Folds the run recorded in c (if it advanced any step) into the list state.
SPK_HD void fold_finished_run(RunCtl& c, int G, float dt) {
  if (c.step <= 0) return;
  c.last_group_p1 = group_index(c.start_time, c.step - 1, G, dt) + 1;
  c.last_run_groups = c.step / G;
  c.last_run_repeat = c.repeat;
  c.step = 0;
}

// For a run of `steps` timesteps from `start`, after fold_finished_run: 1 if
// it begins by delivering the last group's spikes again (its first group
// index has the last group step's parity), 2 if the list would also hold the
// group before (a run of one group that began so, followed by another such
// start), 0 otherwise.
SPK_HD int carry_decision(const RunCtl& c, int G, float dt, float start, int steps) {
  if (steps <= 0 || c.last_group_p1 == 0) return 0;
  const int first = (int)roundf(start / dt) / G;
  if (((first ^ (c.last_group_p1 - 1)) & 1) != 0) return 0;
  return (c.last_run_groups == 1 && c.last_run_repeat) ? 2 : 1;
}

// Whether the group of timestep sr of the run in c (its index k) has the
// parity of the group step before it, so that its substeps deliver the
// earlier group's spikes again: the run's first group as decided where the
// run started, the others from the time of the group before.
SPK_HD bool group_repeats(const RunCtl& c, int sr, int k, int G, float dt) {
  if (sr < G) return c.repeat != 0;
  return ((k ^ group_index(c.start_time, sr - G, G, dt)) & 1) == 0;
}

// Everything one CTA needs to run its share of one network.
struct NetDev {
  // sizes and schedule
  int N, Nin, KL, n_keys, n_words, L, B, kind;
  int n_tiles, TS, ITS, W, nctas, n_groups;
  float dt, half_dt, t_ref, i_bg;
  // Timestep grouping G: the minimum delay in steps (Spike/Models/SpikingModel.cpp:98).
  // Timestep r of a run is substep r % G of group r / G.
  int G;
  GroupConst groups[MAX_GROUPS];
  float decay[MAX_LABELS + 1], vhat[MAX_LABELS + 1];
  float scale_tab[MAX_CLASSES];
  // STDP (G = 1 constants of WeightDependentSTDPPlasticity.cu:125-145)
  int has_stdp, clip_upper;
  float E_m, E_p, inc_m, inc_p, invE_m, invE_p, lam, lam_alpha, wmax;
  uint64_t seed;
  // connectivity
  const int* rowptr;   // [n_keys * n_tiles + 1]
  uint2* entries;      // [S]
  const int* csc_ptr;  // [N + 1] plastic afferents of each post
  uint2* csc;          // (pre key, float bits of the weight), post-major
  // home copies of the state held in shared memory during a launch
  float* V;
  float* last;
  float* gtr;          // [N*L]
  float* ring;         // [n_tiles][B][TS*L]
  float* in_next;      // [Nin]
  const float* rates;  // [Nin] of the selected stimulus
  float* post_trace;   // [N]
  float* pre_trace;    // [n_keys] own copy (home)
  float* pre_pub;      // [2][n_keys] published each step for other CTAs
  // Per-step exchange between the CTAs of a network, double-buffered by step
  // parity.  CTA r writes its active keys, inputs first then neurons, each part
  // ascending, into cta_keys[par][r][*] as (step + 1) << 32 | key | spike << 31
  // | pre-event << 30, and one stamp word (step + 1) << 32 | inputs << 16 |
  // neurons into cta_stamp[par][r].  Every word carries its step, so a
  // consumer that polls the stamps and then the keys needs no fence in
  // between: the step's only inter-CTA synchronization.
  unsigned long long* cta_keys;     // [2][nctas][key_cap]
  unsigned long long* cta_stamp;    // [2][nctas]
  int key_cap;                      // W * (TS + ITS)
  // Spike / pre-event bitmaps of the step (plastic runs only), for the
  // post-spike STDP pass to look up arbitrary presynaptic keys.
  uint32_t* bitsA;  // [2][n_words]
  uint32_t* bitsP;  // [2][n_words]
  // bulk mode: postsynaptic STDP events of the step ([n_words]); a neuron's
  // presynaptic events (bitsP) differ from these only when its last spike is
  // later than the clock (after reset_time)
  uint32_t* bitsE;
  uint2* spikes;    // spike store (key, float time bits)
  long long spike_cap;
  RunCtl* ctl;
  int* abort_flag;            // shared by a launch: set on timeout
  unsigned long long poll_ns; // limit of every wait on another CTA (globaltimer ns)
  // bulk-synchronous batches only: the step's active keys in canonical order
  uint32_t* step_list;        // [n_keys] key | spike << 31 | pre-event << 30
  int* step_count;            // keys in step_list
  // rate monitor: spikes of each key since the last clear, or null
  int* rate_counts;           // [n_keys]
  // Spike words of each substep of the last group ([G][n_words]), the list a
  // run delivers again when it starts at a group index of the same parity.
  uint32_t* gbits;
  // Rules with two traces per plastic synapse (SPK_STDP_EVANS,
  // SPK_STDP_INHIBITORY, SPK_STDP_CUSTOM; bulk mode only): the records' delays, the traces,
  // and the spike words of the last H timesteps (slot T % H), in which a
  // presynaptic spike is looked up delay steps back.
  int stdp_rule;              // SPK_STDP_*
  int H;                      // D_max + 1
  const int* csc_delay;       // [n_csc]
  float2* dense_tr;           // [n_csc]: presynaptic, postsynaptic trace
  uint32_t* hist;             // [H][n_words]
  float rule_c[8];            // the rule's constants
  // Weight normalisation of the plastic afferents (SPK_NORM_*; bulk mode
  // only): each record's initial weight and each post's sum of squares.
  int weight_norm;
  const float* norm_w0;       // [n_csc]
  const float* norm_sum;      // [N]
};

struct CtaMap {
  int net;   // index into the NetDev array
  int rank;  // CTA rank within the network
};

// Per-warp shared-memory words for a schedule (4-byte words).
struct WarpLayout {
  int stage, stw, sidx, kst, koff, kfl, kpre, tag, rowb, rowe, ring, V, last, gtr, post_tr, pre_tr, spkw, evw, pvw, fw,
      inw, inwp, in_next, in_rate, in_pre, total;
};
SPK_HD WarpLayout warp_layout(int B, int TS, int L, int ITS, int kind, int has_stdp) {
  WarpLayout w;
  int o = 0;
  w.stage = o; o += 2 * STAGE_ENTRIES;  // uint2 entries (8-byte aligned: o even)
  w.stw = o; o += has_stdp ? STAGE_ENTRIES : 0;  // weights of staged plastic entries
  w.sidx = o; o += STAGE_ENTRIES / 2;   // uint16 sub-row index per staged entry
  w.kst = o; o += STAGE_KEYS;           // sub-row start (entry index)
  w.koff = o; o += STAGE_KEYS + 4;      // exclusive prefix of sub-row lengths
  w.kfl = o; o += STAGE_KEYS;           // list word (key | spike | pre-event flags)
  w.kpre = o; o += STAGE_KEYS;          // presynaptic STDP trace of the step
  w.tag = o; o += APPLY_TAGS;           // lowest lane per cell hash (ordered apply)
  w.rowb = o; o += TS + ITS;            // synapse-row bounds of the warp's own keys
  w.rowe = o; o += TS + ITS;            //   (neurons, then inputs), for L2 prefetch
  w.ring = o; o += B * TS * L;
  w.V = o; o += TS;
  w.last = o; o += TS;
  w.gtr = o; o += (kind == 3) ? 0 : TS * L;
  w.post_tr = o; o += has_stdp ? TS : 0;
  w.pre_tr = o; o += has_stdp ? TS : 0;
  w.spkw = o; o += TS / 32;   // spike words of the tile's neurons (this step)
  w.evw = o; o += TS / 32;    // postsynaptic STDP event words of the tile's neurons
  w.pvw = o; o += TS / 32;    // presynaptic STDP event words of the tile's neurons
  w.fw = o; o += (TS + ITS) / 32;  // carried keys delivered again (neurons, then inputs)
  w.inw = o; o += ITS / 32;   // spike words of the tile's inputs
  w.inwp = o; o += ITS / 32;  // STDP pre-event words of the tile's inputs
  w.in_next = o; o += ITS;
  w.in_rate = o; o += ITS;
  w.in_pre = o; o += has_stdp ? ITS : 0;
  o = (o + 3) & ~3;
  w.total = o;
  return w;
}
// CTA-shared words: active list, per-source-segment offsets of the key gather
// (2 segments per CTA of the network), flags; a multiple of 4 words so every
// warp region starts 16-byte aligned.
constexpr int MAX_CTAS_PER_NET = 256;
constexpr int SHARED_WORDS = LIST_CAP + 2 * MAX_CTAS_PER_NET + 8;
SPK_HD int smem_bytes(int W, const WarpLayout& wl) { return 4 * (SHARED_WORDS + W * wl.total); }

}  // namespace spk
