// spk_oracle.cpp - CPU restatement of Spike's clock-driven simulation step.
//
// TEST INFRASTRUCTURE ONLY (see spk_oracle.h): the checker for the CUDA path,
// never linked into the product library.
//
// Compiled with -ffp-contract=off so every float expression below rounds
// after each operation, as the CUDA kernels do under -fmad=false.  The
// reference is cited function by function; variable names follow the
// reference where that helps the side-by-side reading.
#include "spk_oracle.h"

#include <algorithm>
#include <atomic>
#include <barrier>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iterator>
#include <new>
#include <thread>
#include <vector>

#include "../spike_gb300/csrc/spk_rng.h"

namespace {

// (int)roundf(x) as the reference's device code evaluates it: round half away
// from zero, then a saturating float->int conversion in which NaN becomes 0
// (PTX cvt.rzi.s32.f32 semantics), so the host agrees with the GPU on every
// input, including the ones C leaves undefined.
inline int round_to_int(float x) {
  if (x != x) return 0;
  float r = std::roundf(x);
  if (r >= 2147483648.0f) return 2147483647;
  if (r <= -2147483648.0f) return (-2147483647 - 1);
  return (int)r;
}
inline int round_to_int(double x) {
  if (x != x) return 0;
  double r = std::round(x);
  if (r >= 2147483648.0) return 2147483647;
  if (r <= -2147483648.0) return (-2147483647 - 1);
  return (int)r;
}

template <typename R>
struct Net {
  // ---- model constants ---------------------------------------------------
  float dt_f = 0.f;
  R dt = 0;
  int kind = 0;
  int N = 0, Nin = 0, L = 1, B = 0, Dmax = 0;
  int G = 1;  // timestep grouping: the minimum delay (Spike/Models/SpikingModel.cpp:98)
  std::vector<R> k, kR, v0, vreset, theta;  // per neuron, as the reference backend
  std::vector<float> vinit_lo, vinit_hi;    // per neuron (extension)
  R t_ref = 0, i_bg = 0;
  std::vector<float> rates;  // [n_stim][Nin]
  int n_stim = 0, stim = 0;
  std::vector<R> decay, vhat;  // per label
  uint64_t seed = 0;
  bool record_inputs = false;

  // ---- synapses in reference sorted order (Synapses::sort_synapses) -------
  int64_t S = 0;
  std::vector<int32_t> spre, spost, sdelay, slabel;
  std::vector<R> sw, sscale;
  std::vector<int64_t> revsort;          // creation index -> sorted index
  std::vector<int64_t> eff_start, eff_count;  // per key
  std::vector<int64_t> plastic_idx;       // sorted indices under the STDP rule
  bool has_stdp = false;
  int stdp_rule = SPK_STDP_WEIGHT_DEPENDENT;
  spk_stdp_params stdp{};
  R E_minus = 0, E_plus = 0, inc_minus = 0, inc_plus = 0, invE_minus = 0, invE_plus = 0;
  R vogels_decay = 0;  // expf(-timestep / tau_istdp), computed on the host
  R custom_post_decay = 0, custom_pre_decay = 0;
  // Weight normalisation (WeightNormSTDPPlasticity): per post, its plastic
  // afferents in creation order (sorted positions), their initial weights and
  // the post's sum of squares.
  int weight_norm = SPK_NORM_OFF;
  std::vector<int64_t> norm_ptr, norm_pos;
  std::vector<R> norm_w0, norm_S;
  // Spike bits of the last H timesteps per key, for rules that see a
  // presynaptic spike when it arrives (the reference's spike bit-buffers,
  // Spike/Backend/CUDA/Neurons/SpikingNeurons.cu:33-35).
  int H = 1;
  std::vector<uint8_t> hist;  // [H][keys]

  // ---- dynamic state --------------------------------------------------------
  std::vector<R> V, last, gtr, ring;  // ring [B][N*L]
  std::vector<R> in_next;              // input last_spike_time (= next spike time)
  std::vector<uint8_t> in_active;
  std::vector<R> stdp_pre, stdp_post;  // per plastic synapse (reference layout)
  float current_time = 0.f;
  uint64_t events = 0;
  std::vector<int32_t> rec_ids[2];
  std::vector<float> rec_times[2];

  // The reference's two active-neuron lists (Spike/Backend/CUDA/Synapses/SpikingSynapses.cu:156-202)
  // are double-buffered by the parity of the group index T/G: a group step
  // appends its spikes to list (T/G) % 2, delivers that whole list, and empties
  // the other one.  Consecutive group steps whose indices have equal parity
  // therefore deliver the earlier group's spikes again, to the later group's
  // slots: substep g's carried keys with substep g's own, after its STDP
  // updates, merged in key order (a key both carried and spiking once).  The
  // index comes from the float time, so this happens where a run starts at
  // the index where the last one ended (or two past it) and, where t/dt
  // falls near a half, within a run.  The state below carries it across runs.
  std::vector<std::vector<int64_t>> group_keys;  // [G]: active keys of each substep of the last group
  int64_t last_group = -1;        // index T/G of the last group step; -1: none since reset
  int64_t last_run_groups = 0;    // groups of the run that ended with it
  bool last_run_repeat = false;   // that run began by delivering its predecessor's group again

  // ---- per-step scratch -----------------------------------------------------
  std::vector<uint8_t> spiked;    // per key, this step
  std::vector<int64_t> active;    // keys delivered this step, ascending
  std::vector<int64_t> rec_keys;  // keys that spiked this step, ascending
  bool first_repeat = false;      // the run's first group repeats the last group step's parity
  int status = SPK_OK;            // SPK_ERR_UNSUPPORTED: a carried list of two groups

  // ---- threading: post-range ownership --------------------------------------
  int threads = 1;
  std::vector<int> n0, n1, i0, i1;           // owned neuron / input ranges
  std::vector<int64_t> split;                // [key][threads+1] sub-row starts
  std::vector<int64_t> p0, p1;               // plastic ranges

  int key_of_input(int i) const { return Nin - 1 - i; }  // N_in + (-i-1)
  int key_of_neuron(int n) const { return Nin + n; }
  int nkeys() const { return Nin + N; }

  int init(const spk_net_desc* d);
  void reset_state();
  void reset_inputs();
  void set_threads(int t);
  int run_steps(int64_t n_steps, float start, bool plastic);
  void lif_range(int a, int b, R t, int T);
  void poisson_range(int a, int b, R t, int T);
  void stdp_range(int64_t a, int64_t b, R t);
  void dense_stdp_range(int64_t a, int64_t b, int T);
  void normalise_weights();
  void propagate_thread(int th, int T);
};

template <typename R>
int Net<R>::init(const spk_net_desc* d) {
  dt_f = d->dt;
  dt = (R)d->dt;
  kind = d->synapse_kind;
  N = d->n_neurons;
  Nin = d->n_inputs;
  L = d->n_labels;
  seed = d->seed;
  record_inputs = d->record_inputs != 0;
  if (N <= 0 || L <= 0 || Nin < 0 || !(d->dt > 0.f)) return SPK_ERR_INVALID;
  if (kind != SPK_SYN_CONDUCTANCE && kind != SPK_SYN_CURRENT && kind != SPK_SYN_VOLTAGE)
    return SPK_ERR_INVALID;

  // LIF constants: k = timestep / tau_m and k*R, computed on the host in the
  // reference (Spike/Backend/CUDA/Neurons/LIFSpikingNeurons.cu:31-44).
  k.assign(N, 0);
  kR.assign(N, 0);
  v0.assign(N, 0);
  vreset.assign(N, 0);
  theta.assign(N, 0);
  vinit_lo.assign(N, 0.f);
  vinit_hi.assign(N, 0.f);
  for (int g = 0; g < d->n_groups; ++g) {
    const spk_neuron_group& G = d->groups[g];
    for (int n = G.start; n < G.start + G.count; ++n) {
      if (n < 0 || n >= N) return SPK_ERR_INVALID;
      if (sizeof(R) == 4) {
        float kk = d->dt / G.tau_m;
        k[n] = (R)kk;
        kR[n] = (R)(kk * G.R);
      } else {
        double kk = (double)d->dt / (double)G.tau_m;
        k[n] = (R)kk;
        kR[n] = (R)(kk * (double)G.R);
      }
      v0[n] = (R)G.v0;
      vreset[n] = (R)G.vreset;
      theta[n] = (R)G.theta;
      vinit_lo[n] = G.v_init_lo;
      vinit_hi[n] = G.v_init_hi;
    }
  }
  t_ref = (R)d->refractory_period;
  i_bg = (R)d->background_current;

  // Conductance decay expf(-dt/tau_g) on the host
  // (Spike/Backend/CUDA/Synapses/ConductanceSpikingSynapses.cu:76-78); the
  // current-synapse decay uses the same formula (written from the equations:
  // the reference's current kernel never runs, CurrentSpikingSynapses.cu:67-68).
  decay.assign(L, 0);
  vhat.assign(L, 0);
  for (int l = 0; l < L; ++l) {
    if (kind != SPK_SYN_VOLTAGE) {
      if (!d->label_tau) return SPK_ERR_INVALID;
      if (sizeof(R) == 4)
        decay[l] = (R)expf(-d->dt / d->label_tau[l]);
      else
        decay[l] = (R)std::exp(-(double)d->dt / (double)d->label_tau[l]);
    }
    if (kind == SPK_SYN_CONDUCTANCE) {
      if (!d->label_vhat) return SPK_ERR_INVALID;
      vhat[l] = (R)d->label_vhat[l];
    }
  }

  if (Nin > 0) {
    n_stim = d->n_stimuli;
    stim = d->stimulus;
    if (n_stim <= 0 || !d->input_rates || stim < 0 || stim >= n_stim) return SPK_ERR_INVALID;
    rates.assign(d->input_rates, d->input_rates + (size_t)n_stim * Nin);
  }

  // ---- sort synapses by key N_in + pre, stable (Synapses.cpp:33-81) -------
  S = d->n_synapses;
  if (S < 0) return SPK_ERR_INVALID;
  const int K = nkeys();
  std::vector<int64_t> cnt(K + 1, 0);
  Dmax = 0;
  int Dmin = 1 << 30;
  for (int64_t s = 0; s < S; ++s) {
    int p = d->pre[s], q = d->post[s], dl = d->delay[s], lb = d->label ? d->label[s] : 0;
    int key = Nin + p;
    if (key < 0 || key >= K || q < 0 || q >= N || dl < 1 || lb < 0 || lb >= L)
      return SPK_ERR_INVALID;
    cnt[key + 1]++;
    if (dl > Dmax) Dmax = dl;
    if (dl < Dmin) Dmin = dl;
  }
  // timestep_grouping = the minimum delay (Spike/Models/SpikingModel.cpp:98);
  // 1 without synapses.  The plasticity rules are restated for G = 1 only.
  G = S > 0 ? Dmin : 1;
  if (G > 1 && d->has_stdp) return SPK_ERR_UNSUPPORTED;
  for (int kk = 0; kk < K; ++kk) cnt[kk + 1] += cnt[kk];
  eff_start.assign(cnt.begin(), cnt.end() - 1);
  eff_count.assign(K, 0);
  for (int kk = 0; kk < K; ++kk) eff_count[kk] = cnt[kk + 1] - cnt[kk];
  spre.resize(S);
  spost.resize(S);
  sdelay.resize(S);
  slabel.resize(S);
  sw.resize(S);
  sscale.resize(S);
  revsort.resize(S);
  std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
  std::vector<uint8_t> splastic(S, 0);
  for (int64_t s = 0; s < S; ++s) {
    int key = Nin + d->pre[s];
    int64_t pos = fill[key]++;
    spre[pos] = d->pre[s];
    spost[pos] = d->post[s];
    sdelay[pos] = d->delay[s];
    slabel[pos] = d->label ? d->label[s] : 0;
    sw[pos] = (R)d->weight[s];
    sscale[pos] = (R)d->scale[s];
    revsort[s] = pos;
    if (d->plastic && d->plastic[s]) splastic[pos] = 1;
  }
  // Ring depth D_max + 2G + 1 (Spike/Backend/CUDA/Synapses/SpikingSynapses.cu:48).
  // Deliveries land at most D_max slots ahead, but a run of a grouped network
  // that is not whole groups skips timestep indices (the next run starts at
  // start + seconds), and a skipped slot's contents are read B steps later.
  // A network without synapses keeps a ring of delay-1 depth.
  if (S == 0) Dmax = 1;
  B = Dmax + 2 * G + 1;

  has_stdp = d->has_stdp != 0;
  stdp = d->stdp;
  stdp_rule = d->stdp_rule;
  if (stdp_rule < SPK_STDP_WEIGHT_DEPENDENT || stdp_rule > SPK_STDP_CUSTOM) return SPK_ERR_INVALID;
  if (has_stdp && stdp_rule == SPK_STDP_CUSTOM) {
    // expf(- timestep / tau_minus), expf(- timestep / tau_plus) (CustomSTDPPlasticity.cu:55-56)
    if (sizeof(R) == 4) {
      custom_post_decay = (R)expf(-d->dt / stdp.tau_minus);
      custom_pre_decay = (R)expf(-d->dt / stdp.tau_plus);
    } else {
      custom_post_decay = (R)std::exp(-(double)d->dt / (double)stdp.tau_minus);
      custom_pre_decay = (R)std::exp(-(double)d->dt / (double)stdp.tau_plus);
    }
  }
  if (has_stdp && stdp_rule == SPK_STDP_INHIBITORY) {
    // expf(- timestep / tau_istdp) (Spike/Backend/CUDA/Plasticity/InhibitorySTDPPlasticity.cu:61)
    if (sizeof(R) == 4)
      vogels_decay = (R)expf(-d->dt / stdp.tau_plus);
    else
      vogels_decay = (R)std::exp(-(double)d->dt / (double)stdp.tau_plus);
  }
  H = Dmax + 1;
  weight_norm = d->weight_norm;
  if (weight_norm < SPK_NORM_OFF || weight_norm > SPK_NORM_BEFORE_RULE) return SPK_ERR_INVALID;
  if (weight_norm != SPK_NORM_OFF && !has_stdp) return SPK_ERR_INVALID;
  norm_ptr.clear();
  norm_pos.clear();
  norm_w0.clear();
  norm_S.clear();
  if (weight_norm != SPK_NORM_OFF) {
    // WeightNormSTDPPlasticity::prepare_backend_early
    // (Spike/Plasticity/WeightNormSTDPPlasticity.cpp:31-70): the sum of
    // pow(w, 2.0f) over each post's plastic afferents in the rule's order,
    // and the initial weights.
    norm_ptr.assign((size_t)N + 1, 0);
    for (int64_t s = 0; s < S; ++s)
      if (d->plastic && d->plastic[s]) norm_ptr[(size_t)d->post[s] + 1]++;
    for (int q = 0; q < N; ++q) norm_ptr[q + 1] += norm_ptr[q];
    norm_pos.resize(norm_ptr[N]);
    norm_w0.resize(norm_ptr[N]);
    norm_S.assign(N, (R)0);
    std::vector<int64_t> fill(norm_ptr.begin(), norm_ptr.end() - 1);
    for (int64_t s = 0; s < S; ++s) {
      if (!(d->plastic && d->plastic[s])) continue;
      const int q = d->post[s];
      const int64_t j = fill[q]++;
      norm_pos[j] = revsort[s];
      norm_w0[j] = (R)(d->norm_initial ? d->norm_initial[s] : d->weight[s]);
      if (!d->norm_sum) {
        if (sizeof(R) == 4)
          norm_S[q] = (R)((float)norm_S[q] + powf(d->weight[s], 2.0f));
        else
          norm_S[q] += (R)((double)d->weight[s] * (double)d->weight[s]);
      }
    }
    if (d->norm_sum)
      for (int q = 0; q < N; ++q) norm_S[q] = (R)d->norm_sum[q];
  }
  plastic_idx.clear();
  if (has_stdp)
    for (int64_t s = 0; s < S; ++s)
      if (splastic[s]) plastic_idx.push_back(s);
  if (has_stdp) {
    // Trace constants of WeightDependentSTDPPlasticity.cu:125-145 for G = 1,
    // where the only spike sub-step is g = 0: expf(-(G*dt)/tau) for the decay,
    // a*expf(-((G-0)*dt)/tau) for the increment, 1/expf(-(G-0)*dt/tau) for
    // the on-pre / on-post rescaling.
    if (sizeof(R) == 4) {
      float em = expf(-(1.0f * d->dt) / stdp.tau_minus);
      float ep = expf(-(1.0f * d->dt) / stdp.tau_plus);
      E_minus = (R)em;
      E_plus = (R)ep;
      inc_minus = (R)(stdp.a_minus * em);
      inc_plus = (R)(stdp.a_plus * ep);
      invE_minus = (R)(1.0f / em);
      invE_plus = (R)(1.0f / ep);
    } else {
      double em = std::exp(-(double)d->dt / (double)stdp.tau_minus);
      double ep = std::exp(-(double)d->dt / (double)stdp.tau_plus);
      E_minus = (R)em;
      E_plus = (R)ep;
      inc_minus = (R)((double)stdp.a_minus * em);
      inc_plus = (R)((double)stdp.a_plus * ep);
      invE_minus = (R)(1.0 / em);
      invE_plus = (R)(1.0 / ep);
    }
  }

  V.assign(N, 0);
  last.assign(N, 0);
  gtr.assign((size_t)N * L, 0);
  ring.assign((size_t)B * N * L, 0);
  in_next.assign(Nin, 0);
  in_active.assign(Nin, 0);
  stdp_pre.assign(plastic_idx.size(), 0);
  stdp_post.assign(plastic_idx.size(), 0);
  spiked.assign(K, 0);
  hist.assign((size_t)H * K, 0);
  set_threads(1);
  reset_state();
  return SPK_OK;
}

template <typename R>
void Net<R>::reset_inputs() {
  // SpikingNeurons::reset_state: last spike time -1000
  // (Spike/Backend/CUDA/Neurons/SpikingNeurons.cu:68-94) and
  // PoissonInputSpikingNeurons::reset_state: active = false
  // (Spike/Backend/CUDA/Neurons/PoissonInputSpikingNeurons.cu:27-34).
  for (int i = 0; i < Nin; ++i) {
    in_next[i] = (R)-1000.0f;
    in_active[i] = 0;
  }
}

template <typename R>
void Net<R>::reset_state() {
  // SpikingModel::reset_state order: synapses (ring, conductance traces),
  // neurons (V := V0, last := -1000), inputs, plasticity (traces := 0)
  // (Spike/Models/SpikingModel.cpp:181-190).
  std::fill(ring.begin(), ring.end(), (R)0);
  std::fill(gtr.begin(), gtr.end(), (R)0);
  for (int n = 0; n < N; ++n) {
    if (vinit_lo[n] < vinit_hi[n]) {
      float u = spk::draw_uniform(seed, (uint32_t)n, 0u, spk::DOMAIN_VINIT);
      if (sizeof(R) == 4) {
        float span = vinit_hi[n] - vinit_lo[n];
        V[n] = (R)(vinit_lo[n] + span * u);
      } else {
        V[n] = (R)((double)vinit_lo[n] + ((double)vinit_hi[n] - (double)vinit_lo[n]) * (double)u);
      }
    } else {
      V[n] = v0[n];
    }
    last[n] = (R)-1000.0f;
  }
  reset_inputs();
  std::fill(stdp_pre.begin(), stdp_pre.end(), (R)0);
  std::fill(stdp_post.begin(), stdp_post.end(), (R)0);
  std::fill(hist.begin(), hist.end(), (uint8_t)0);
  // SpikingSynapses::reset_state empties both active lists (SpikingSynapses.cu:33)
  group_keys.assign(G, {});
  status = SPK_OK;
  last_group = -1;
  last_run_groups = 0;
  last_run_repeat = false;
}


template <typename R>
void Net<R>::set_threads(int t) {
  if (t < 1) t = 1;
  threads = t;
  n0.assign(t, 0);
  n1.assign(t, 0);
  i0.assign(t, 0);
  i1.assign(t, 0);
  for (int th = 0; th < t; ++th) {
    n0[th] = (int)((int64_t)N * th / t);
    n1[th] = (int)((int64_t)N * (th + 1) / t);
    i0[th] = (int)((int64_t)Nin * th / t);
    i1[th] = (int)((int64_t)Nin * (th + 1) / t);
  }
  // Split every efferent row by owning thread (rows keep sorted order inside
  // each part, so per-cell accumulation order is unchanged).
  const int K = nkeys();
  split.assign((size_t)K * (t + 1), 0);
  std::vector<int> owner(N, 0);
  for (int th = 0; th < t; ++th)
    for (int n = n0[th]; n < n1[th]; ++n) owner[n] = th;
  if (t > 1) {
    // Permute each row so entries are grouped by owner, stable within owner.
    std::vector<int32_t> tp(S), tq(S), td(S), tl(S);
    std::vector<R> tw(S), ts(S);
    std::vector<int64_t> perm(S);
    for (int kk = 0; kk < K; ++kk) {
      int64_t a = eff_start[kk], b = a + eff_count[kk];
      std::vector<int64_t> c(t + 1, 0);
      for (int64_t s = a; s < b; ++s) c[owner[spost[s]] + 1]++;
      for (int th = 0; th < t; ++th) c[th + 1] += c[th];
      for (int th = 0; th <= t; ++th) split[(size_t)kk * (t + 1) + th] = a + c[th];
      std::vector<int64_t> f(c.begin(), c.end() - 1);
      for (int64_t s = a; s < b; ++s) perm[s] = a + f[owner[spost[s]]]++;
    }
    for (int64_t s = 0; s < S; ++s) {
      int64_t p = perm[s];
      tp[p] = spre[s];
      tq[p] = spost[s];
      td[p] = sdelay[s];
      tl[p] = slabel[s];
      tw[p] = sw[s];
      ts[p] = sscale[s];
    }
    spre.swap(tp);
    spost.swap(tq);
    sdelay.swap(td);
    slabel.swap(tl);
    sw.swap(tw);
    sscale.swap(ts);
    for (int64_t s = 0; s < S; ++s) revsort[s] = perm[revsort[s]];
    for (auto& pi : plastic_idx) pi = perm[pi];
    for (auto& pi : norm_pos) pi = perm[pi];
    // plastic_idx order only matters for the per-synapse trace arrays, which
    // were all reset together: keep them aligned.
  } else {
    for (int kk = 0; kk < K; ++kk) {
      split[(size_t)kk * 2] = eff_start[kk];
      split[(size_t)kk * 2 + 1] = eff_start[kk] + eff_count[kk];
    }
  }
  int64_t P = (int64_t)plastic_idx.size();
  p0.assign(t, 0);
  p1.assign(t, 0);
  for (int th = 0; th < t; ++th) {
    p0[th] = P * th / t;
    p1[th] = P * (th + 1) / t;
  }
}

// lif_update_membrane_potentials with the injection kernels inlined
// (Spike/Backend/CUDA/Neurons/LIFSpikingNeurons.cu:105-193,
// Spike/Backend/CUDA/InlineDeviceFunctions.hpp:22-111) for one substep:
// tg = current_time + g*timestep, T = its timestep index (with g added).
template <typename R>
void Net<R>::lif_range(int a, int b, R tg, int T) {
  const R half_dt = (R)0.5f * dt;
  const size_t row = (size_t)N * L;
  const size_t bufferloc = (size_t)(T % B) * row;
  for (int idx = a; idx < b; ++idx) {
    R Vi = V[idx];
    R input = 0;
    if (kind == SPK_SYN_CONDUCTANCE) {
      R total = 0;
      for (int l = 0; l < L; ++l) {
        R& gl = gtr[(size_t)idx * L + l];
        R& cell = ring[bufferloc + (size_t)idx * L + l];
        R gnew = decay[l] * gl + cell;
        cell = 0;
        total += gnew * (vhat[l] - Vi);
        gl = gnew;
      }
      input = total * kR[idx];
    } else if (kind == SPK_SYN_CURRENT) {
      R total = 0;
      for (int l = 0; l < L; ++l) {
        R& il = gtr[(size_t)idx * L + l];
        R& cell = ring[bufferloc + (size_t)idx * L + l];
        R inew = il * decay[l];
        inew += cell;
        cell = 0;
        total += inew;
        il = inew;
      }
      input = total * kR[idx];
    } else {
      R total = 0;
      for (int l = 0; l < L; ++l) {
        R& cell = ring[bufferloc + (size_t)idx * L + l];
        total += cell;
        cell = 0;
      }
      input = total;
    }
    if (((tg - last[idx]) - t_ref) > half_dt) {
      const R kc = k[idx];
      Vi = kc * v0[idx] + ((R)1 - kc) * Vi + kc * i_bg + input;
      if (Vi >= theta[idx]) {
        spiked[key_of_neuron(idx)] = 1;
        last[idx] = tg;
        Vi = vreset[idx];
      }
    }
    V[idx] = Vi;
  }
}

// poisson_update_membrane_potentials_kernel
// (Spike/Backend/CUDA/Neurons/PoissonInputSpikingNeurons.cu:96-129) for one
// substep (tg, T as in lif_range),
// with the uniform drawn from Philox(seed, input, step).
template <typename R>
void Net<R>::poisson_range(int a, int b, R tg, int T) {
  const float* rt = rates.data() + (size_t)Nin * stim;
  for (int idx = a; idx < b; ++idx) {
    if ((in_next[idx] <= tg) || !in_active[idx]) {
      const R rate = (R)rt[idx];
      const float u = spk::draw_uniform(seed, (uint32_t)idx, (uint32_t)T, spk::DOMAIN_POISSON);
      R lg;
      if (sizeof(R) == 4)
        lg = (R)spk::logf_spk(u);
      else
        lg = (R)std::log((double)u);
      in_next[idx] = tg - ((R)1 / rate) * lg;
      if (in_active[idx])
        spiked[key_of_input(idx)] = 1;
      else
        in_active[idx] = 1;
    }
  }
}

// ltp_and_ltd (Spike/Backend/CUDA/Plasticity/WeightDependentSTDPPlasticity.cu:85-161),
// G = 1: pre_g, post_g are 0 for a spike at this step (or of the step before,
// when a run starts at the timestep index where the last one ended) and
// negative otherwise, so the (post_g > pre_g) / (pre_g > post_g) corrections
// never apply.
template <typename R>
void Net<R>::stdp_range(int64_t a, int64_t b, R t) {
  // G = 1 here: init refuses a rule with a larger grouping
  for (int64_t indx = a; indx < b; ++indx) {
    const int64_t idx = plastic_idx[indx];
    R pre_tr = stdp_pre[indx];
    R post_tr = stdp_post[indx];
    const int postid = spost[idx];
    const int preid = spre[idx];
    const R old_w = sw[idx];
    const bool is_input = preid < 0;
    const int corr = is_input ? (-preid - 1) : preid;
    const R pre_last = is_input ? in_next[corr] : last[corr];
    int pre_g = round_to_int((pre_last - t) / dt);
    int post_g = round_to_int((last[postid] - t) / dt);
    if (pre_g >= G) pre_g *= -1;

    post_tr *= E_minus;
    pre_tr *= E_plus;
    post_tr += (post_g >= 0) ? inc_minus : (R)0;
    pre_tr += (pre_g >= 0) ? inc_plus : (R)0;

    R syn_update = 0;
    if (pre_g >= 0) {
      R temp_post = post_tr;
      temp_post *= invE_minus;
      syn_update -= (R)stdp.lambda * (R)stdp.alpha * old_w * temp_post;
    }
    if (post_g >= 0) {
      R temp_pre = pre_tr;
      temp_pre *= invE_plus;
      syn_update += (R)stdp.lambda * ((R)stdp.w_max - old_w) * temp_pre;
    }
    R new_w = old_w + syn_update;
    if (new_w < (R)0) new_w = 0;
    if (stdp.clip_upper && new_w > (R)stdp.w_max) new_w = (R)stdp.w_max;
    sw[idx] = new_w;
    stdp_pre[indx] = pre_tr;
    stdp_post[indx] = post_tr;
  }
}

// Rules with two traces per plastic synapse, updated every timestep; a
// presynaptic spike is seen when it arrives, delay steps after it was fired
// (bit T - delay of the presynaptic bit-buffer), a postsynaptic one at T.
//   Evans: ltp_and_ltd (Spike/Backend/CUDA/Plasticity/EvansSTDPPlasticity.cu:59-141),
//     traces C (presynaptic activity) and D (postsynaptic), weights in [0, 1];
//   inhibitory: vogels_apply_stdp_to_synapse_weights_kernel
//     (Spike/Backend/CUDA/Plasticity/InhibitorySTDPPlasticity.cu:71-154),
//     weights clipped at 0; its constant term is evaluated in double, as the
//     reference's 2.0 literal makes it;
//   custom: pre and post memory traces, optionally nearest-spike, weights clipped at 0.
// WeightNormSTDPPlasticity::weight_normalization
// (Spike/Backend/CUDA/Plasticity/WeightNormSTDPPlasticity.cu:74-176): per post,
// the change of its afferents' sum of squares against their initial weights,
// (w - w0)^2 + 2 w0 (w - w0) over the afferents whose weight moved; divisor
// sqrt(S + change) / sqrt(S); the weights divided when it is not 1.  The
// reference adds the terms with atomicAdd, in no fixed order; the fixed order
// here: partial sum j takes the terms of afferents j, j + 32, j + 64, ... (in
// creation order) in turn, then the 32 partials meet in a pairwise tree
// (j with j + 16, then + 8, + 4, + 2, + 1).
template <typename R>
void Net<R>::normalise_weights() {
  for (int q = 0; q < N; ++q) {
    const int64_t a0 = norm_ptr[q], a1 = norm_ptr[q + 1];
    if (a0 == a1) continue;  // not in the rule's set
    R part[32] = {};
    for (int64_t j = a0; j < a1; ++j) {
      const R w0 = norm_w0[j];
      const R dw = sw[norm_pos[j]] - w0;
      if (dw != (R)0) part[(j - a0) % 32] += dw * dw + (R)2 * w0 * dw;
    }
    for (int o = 16; o >= 1; o >>= 1)
      for (int i = 0; i < o; ++i) part[i] = part[i] + part[i + o];
    const R upd = part[0];
    const R div = std::sqrt(norm_S[q] + upd) / std::sqrt(norm_S[q]);
    if (div != (R)1)
      for (int64_t j = a0; j < a1; ++j) sw[norm_pos[j]] = sw[norm_pos[j]] / div;
  }
}

template <typename R>
void Net<R>::dense_stdp_range(int64_t a, int64_t b, int T) {
  const int K = nkeys();
  const R dtR = dt;
  for (int64_t indx = a; indx < b; ++indx) {
    const int64_t idx = plastic_idx[indx];
    const int postid = spost[idx];
    const int preid = spre[idx];
    const int prekey = Nin + preid;  // input -i-1 -> key Nin-1-i, neuron n -> Nin+n
    int slot = (T - sdelay[idx]) % H;
    if (slot < 0) slot += H;
    const bool pre_sp = hist[(size_t)slot * K + prekey] != 0;
    const bool post_sp = spiked[Nin + postid] != 0;
    R tr_pre = stdp_pre[indx];
    R tr_post = stdp_post[indx];
    R w = sw[idx];
    if (stdp_rule == SPK_STDP_EVANS) {
      const R tau_C = (R)stdp.tau_plus, tau_D = (R)stdp.tau_minus;
      const R alpha_C = (R)stdp.a_plus, alpha_D = (R)stdp.a_minus;
      tr_pre = ((R)1 - (dtR / tau_C)) * tr_pre;
      tr_post = ((R)1 - (dtR / tau_D)) * tr_post;
      if (pre_sp) tr_pre += dtR * alpha_C * ((R)1 - tr_pre);
      if (post_sp) tr_post += dtR * alpha_D * ((R)1 - tr_post);
      R syn = 0;
      const R old_w = w;
      if (pre_sp) syn -= (old_w * tr_post);
      if (post_sp) syn += (((R)1 - old_w) * tr_pre);
      w = old_w + syn;
      if (w < (R)0) w = (R)0;
      if (w > (R)1) w = (R)1;
    } else if (stdp_rule == SPK_STDP_CUSTOM) {
      // ltp_and_ltd (Spike/Backend/CUDA/Plasticity/CustomSTDPPlasticity.cu:67-156):
      // lambda = learning_rate, alpha = a_star, clip_upper = nearest_spike_only
      const R a_plus = (R)stdp.a_plus, a_minus = (R)stdp.a_minus, lr = (R)stdp.lambda;
      const R a_star = (R)stdp.alpha, w_max = (R)stdp.w_max;
      const bool nearest = stdp.clip_upper != 0;
      tr_post *= custom_post_decay;
      tr_pre *= custom_pre_decay;
      if (pre_sp) {
        tr_pre += a_plus;
        if (nearest) tr_pre = a_plus;
      }
      if (post_sp) {
        tr_post += a_minus;
        if (nearest) tr_post = a_minus;
      }
      R syn = 0;
      const R old_w = w;
      if (pre_sp) syn -= lr * (old_w / w_max) * tr_post + lr * a_star;
      if (post_sp) syn += lr * tr_pre;
      w = old_w + syn;
      if (w < (R)0) w = (R)0;
    } else {
      const R lr = (R)stdp.lambda;
      tr_pre *= vogels_decay;
      tr_post *= vogels_decay;
      if (pre_sp) tr_pre += (R)1;
      if (post_sp) tr_post += (R)1;
      R syn = 0;
      if (pre_sp) {
        syn += lr * (tr_post);
        syn += -lr * (2.0 * (double)stdp.alpha * (double)stdp.tau_plus);
      }
      if (post_sp) syn += lr * (tr_pre);
      w += syn;
      if (w < (R)0) w = (R)0;
    }
    sw[idx] = w;
    stdp_pre[indx] = tr_pre;
    stdp_post[indx] = tr_post;
  }
}

// activate_synapses (Spike/Backend/CUDA/Synapses/SpikingSynapses.cu:168-202):
// slot (bufferloc + delay + g) % B with bufferloc = round(t/dt) % B (:127),
// contributions w*scale applied in ascending key order, then row order.
template <typename R>
void Net<R>::propagate_thread(int th, int T) {
  const size_t row = (size_t)N * L;
  const int bufferloc = T % B;
  for (int64_t key : active) {
    const int64_t a = split[(size_t)key * (threads + 1) + th];
    const int64_t b = split[(size_t)key * (threads + 1) + th + 1];
    for (int64_t s = a; s < b; ++s) {
      const int targetloc = (bufferloc + sdelay[s] + 0) % B;
      ring[(size_t)targetloc * row + (size_t)spost[s] * L + slabel[s]] += sw[s] * sscale[s];
    }
  }
}

template <typename R>
int Net<R>::run_steps(int64_t n_steps, float start, bool plastic) {
  if (n_steps == 0) return SPK_OK;  // no group step: the lists stay as they are
  {
    // The run's first group has index roundf(start/dt) / G.  If the previous
    // group step's index had the same parity, its list still holds that
    // group's spikes: they are delivered again to this group's slots, first.
    const int64_t first = round_to_int(start / dt_f) / G;
    const bool repeat = last_group >= 0 && ((first ^ last_group) & 1) == 0;
    // a run of one group that itself began this way left two groups in the list
    if (repeat && last_run_groups == 1 && last_run_repeat) status = SPK_ERR_UNSUPPORTED;
    first_repeat = repeat;
    last_run_repeat = repeat;
    last_run_groups = n_steps / G;
    // the run's last group: timestep n_steps - G
    const int64_t s_last = n_steps - G;
    const float t_last = start + (float)s_last * dt_f;
    last_group = round_to_int(t_last / dt_f) / G;
  }
  auto step_time = [&](int64_t s, R& t, int& T) {
    // Timestep s is substep g = s % G of group s / G.  The group's
    // current_time_in_seconds = starttime + s*timestep_grouping*timestep
    // (Spike/Models/SpikingModel.cpp:226), the substep's timestep index
    // (int)roundf(t/dt) + g (Spike/Backend/CUDA/Neurons/LIFSpikingNeurons.cu:84,115)
    // and its time t + g*timestep (:172,177; the spike monitor's time,
    // Spike/Backend/CUDA/ActivityMonitor/SpikingActivityMonitor.cu:93).  With
    // G = 1 that is start + s*dt.  Advancing a group substep by substep, each
    // substep's spikes delivered at its end, is the reference's group: a
    // delay of at least G steps lands every delivery past the group, so no
    // substep reads what another substep of its group delivers.
    const int64_t grp = s / G, g = s - grp * G;
    const float tf = start + (float)(grp * G) * dt_f;
    T = round_to_int(tf / dt_f) + (int)g;
    t = (sizeof(R) == 4) ? (R)(tf + (float)g * dt_f) : ((R)start + (R)(grp * G) * dt) + (R)g * dt;
  };
  // whether the group of step s has the parity of the group step before it
  auto group_repeats = [&](int64_t s) {
    if (s < G) return first_repeat;
    const int64_t g0 = s - s % G;
    const int k = round_to_int((start + (float)(g0)*dt_f) / dt_f) / G;
    const int kp = round_to_int((start + (float)(g0 - G) * dt_f) / dt_f) / G;
    return ((k ^ kp) & 1) == 0;
  };
  auto finish_step = [&](R t, int T, int64_t s) {
    active.clear();
    const int K = nkeys();
    for (int kk = 0; kk < K; ++kk)
      if (spiked[kk]) active.push_back(kk);
    rec_keys = active;
    std::vector<int64_t>& carried = group_keys[(size_t)(s % G)];
    const bool rep = group_repeats(s);
    // a carried list of two earlier groups is beyond the engine this checks
    if (rep && s % G == 0 && s >= G && group_repeats(s - G)) status = SPK_ERR_UNSUPPORTED;
    if (rep && !carried.empty()) {
      // the carried keys join the substep's list (a key in both is listed once)
      std::vector<int64_t> merged;
      std::set_union(active.begin(), active.end(), carried.begin(), carried.end(), std::back_inserter(merged));
      carried = rec_keys;
      active.swap(merged);  // counted with the step's keys below
    } else {
      carried = rec_keys;
    }
    // this step's spike bits, for the rules that look delays back
    std::copy(spiked.begin(), spiked.end(), hist.begin() + (size_t)(T % H) * K);
    for (int64_t kk : active) events += (uint64_t)eff_count[kk];
    return t;
  };
  auto record = [&](R t) {
    // SpikingActivityMonitor: (id, current_time + g*timestep), here in key order.
    const float tf = (float)t;
    for (int64_t kk : rec_keys) {
      if (kk >= Nin) {
        rec_ids[SPK_POP_NEURONS].push_back((int32_t)(kk - Nin));
        rec_times[SPK_POP_NEURONS].push_back(tf);
      } else if (record_inputs) {
        rec_ids[SPK_POP_INPUTS].push_back((int32_t)(Nin - 1 - kk));
        rec_times[SPK_POP_INPUTS].push_back(tf);
      }
    }
  };
  const bool do_stdp = plastic && has_stdp && !plastic_idx.empty() && stdp_rule == SPK_STDP_WEIGHT_DEPENDENT;
  const bool do_dense = plastic && has_stdp && !plastic_idx.empty() && stdp_rule != SPK_STDP_WEIGHT_DEPENDENT;
  // the rules in the order added (Spike/Models/SpikingModel.cpp:202-205)
  const bool norm_before = plastic && weight_norm == SPK_NORM_BEFORE_RULE;
  const bool norm_after = plastic && weight_norm == SPK_NORM_AFTER_RULE;
  if (threads <= 1) {
    for (int64_t s = 0; s < n_steps; ++s) {
      R t;
      int T;
      step_time(s, t, T);
      std::fill(spiked.begin(), spiked.end(), 0);
      lif_range(0, N, t, T);
      poisson_range(0, Nin, t, T);
      if (norm_before) normalise_weights();
      if (do_stdp) stdp_range(0, (int64_t)plastic_idx.size(), t);
      if (do_dense) dense_stdp_range(0, (int64_t)plastic_idx.size(), T);
      if (norm_after) normalise_weights();
      finish_step(t, T, s);
      propagate_thread(0, T);
      record(t);
    }
    return SPK_OK;
  }
  std::barrier<> bar(threads);
  R t_cur = 0;
  int T_cur = 0;
  auto worker = [&](int th) {
    for (int64_t s = 0; s < n_steps; ++s) {
      if (th == 0) {
        step_time(s, t_cur, T_cur);
        std::fill(spiked.begin(), spiked.end(), 0);
      }
      bar.arrive_and_wait();
      lif_range(n0[th], n1[th], t_cur, T_cur);
      poisson_range(i0[th], i1[th], t_cur, T_cur);
      bar.arrive_and_wait();
      if (norm_before) {
        if (th == 0) normalise_weights();
        bar.arrive_and_wait();
      }
      if (do_stdp) stdp_range(p0[th], p1[th], t_cur);
      if (do_dense) dense_stdp_range(p0[th], p1[th], T_cur);
      if (norm_after) {
        bar.arrive_and_wait();
        if (th == 0) normalise_weights();
      }
      // finish_step writes history slot T, which no range reads this step
      // (delays are 1..H-1)
      if (th == 0) finish_step(t_cur, T_cur, s);
      bar.arrive_and_wait();
      propagate_thread(th, T_cur);
      if (th == 0) record(t_cur);
      bar.arrive_and_wait();
    }
  };
  std::vector<std::thread> pool;
  for (int th = 1; th < threads; ++th) pool.emplace_back(worker, th);
  worker(0);
  for (auto& x : pool) x.join();
  return SPK_OK;
}

struct Handle {
  int precision = 32;
  Net<float>* f = nullptr;
  Net<double>* d = nullptr;
};

}  // namespace

struct oracle_net {
  Handle h;
};

template <typename F>
static auto dispatch(const oracle_net* n, F&& fn) {
  if (n->h.precision == 64) return fn(*n->h.d);
  return fn(*n->h.f);
}

extern "C" {

int oracle_create(const spk_net_desc* desc, int precision, oracle_net** out) {
  if (!desc || !out || desc->abi_version != SPK_ABI_VERSION) return SPK_ERR_INVALID;
  if (precision != 32 && precision != 64) return SPK_ERR_INVALID;
  oracle_net* n = new (std::nothrow) oracle_net();
  if (!n) return SPK_ERR_OOM;
  n->h.precision = precision;
  int rc;
  if (precision == 64) {
    n->h.d = new Net<double>();
    rc = n->h.d->init(desc);
  } else {
    n->h.f = new Net<float>();
    rc = n->h.f->init(desc);
  }
  if (rc != SPK_OK) {
    delete n->h.f;
    delete n->h.d;
    delete n;
    return rc;
  }
  *out = n;
  return SPK_OK;
}

int oracle_destroy(oracle_net* n) {
  if (!n) return SPK_ERR_INVALID;
  delete n->h.f;
  delete n->h.d;
  delete n;
  return SPK_OK;
}

int oracle_set_threads(oracle_net* n, int threads) {
  if (!n || threads < 1) return SPK_ERR_INVALID;
  dispatch(n, [&](auto& net) {
    net.set_threads(threads);
    return 0;
  });
  return SPK_OK;
}

int oracle_reset_state(oracle_net* n) {
  if (!n) return SPK_ERR_INVALID;
  dispatch(n, [](auto& net) {
    net.reset_state();
    return 0;
  });
  return SPK_OK;
}

int oracle_reset_time(oracle_net* n) {
  if (!n) return SPK_ERR_INVALID;
  dispatch(n, [](auto& net) {
    net.current_time = 0.0f;
    return 0;
  });
  return SPK_OK;
}

int oracle_select_stimulus(oracle_net* n, int stimulus) {
  if (!n) return SPK_ERR_INVALID;
  return dispatch(n, [&](auto& net) {
    if (stimulus < 0 || stimulus >= net.n_stim) return SPK_ERR_INVALID;
    net.stim = stimulus;
    net.reset_inputs();
    return SPK_OK;
  });
}

int oracle_run(oracle_net* n, float seconds, int plasticity_on) {
  if (!n || !(seconds >= 0.0f)) return SPK_ERR_INVALID;
  return dispatch(n, [&](auto& net) {
    // number_of_timesteps = ceil(seconds / timestep), number_of_steps =
    // number_of_timesteps / timestep_grouping in integers: whole groups
    // (Spike/Models/SpikingModel.cpp:221-222).
    const float q = seconds / net.dt_f;
    const int64_t steps = ((int64_t)std::ceil(q) / net.G) * net.G;
    const float start = net.current_time;
    const int rc = net.run_steps(steps, start, plasticity_on != 0);
    if (rc) return rc;
    net.current_time = start + seconds;
    return net.status;
  });
}

int oracle_run_steps(oracle_net* n, int64_t n_steps, int plasticity_on) {
  if (!n || n_steps < 0) return SPK_ERR_INVALID;
  return dispatch(n, [&](auto& net) {
    if (n_steps % net.G != 0) return SPK_ERR_INVALID;  // whole groups only
    const float start = net.current_time;
    const int rc = net.run_steps(n_steps, start, plasticity_on != 0);
    if (rc) return rc;
    net.current_time = start + (float)n_steps * net.dt_f;
    return net.status;
  });
}

int oracle_current_time(const oracle_net* n, float* seconds) {
  if (!n || !seconds) return SPK_ERR_INVALID;
  *seconds = dispatch(n, [](auto& net) { return net.current_time; });
  return SPK_OK;
}

int oracle_spike_count(const oracle_net* n, int population, int64_t* out) {
  if (!n || !out || population < 0 || population > 1) return SPK_ERR_INVALID;
  *out = dispatch(n, [&](auto& net) { return (int64_t)net.rec_ids[population].size(); });
  return SPK_OK;
}

int oracle_read_spikes(const oracle_net* n, int population, int32_t* ids, float* times,
                       int64_t capacity, int64_t* n_written) {
  if (!n || population < 0 || population > 1 || capacity < 0) return SPK_ERR_INVALID;
  return dispatch(n, [&](auto& net) {
    int64_t m = (int64_t)net.rec_ids[population].size();
    if (m > capacity) m = capacity;
    if (ids) std::memcpy(ids, net.rec_ids[population].data(), sizeof(int32_t) * m);
    if (times) std::memcpy(times, net.rec_times[population].data(), sizeof(float) * m);
    if (n_written) *n_written = m;
    return SPK_OK;
  });
}

int oracle_clear_spikes(oracle_net* n) {
  if (!n) return SPK_ERR_INVALID;
  dispatch(n, [](auto& net) {
    for (int p = 0; p < 2; ++p) {
      net.rec_ids[p].clear();
      net.rec_times[p].clear();
    }
    return 0;
  });
  return SPK_OK;
}

int oracle_read_state(const oracle_net* n, int field, float* dst, int64_t count) {
  if (!n || !dst) return SPK_ERR_INVALID;
  return dispatch(n, [&](auto& net) {
    auto put = [&](auto const& v) {
      if ((int64_t)v.size() != count) return SPK_ERR_INVALID;
      for (int64_t i = 0; i < count; ++i) dst[i] = (float)v[i];
      return SPK_OK;
    };
    switch (field) {
      case SPK_FIELD_V:
        return put(net.V);
      case SPK_FIELD_LAST_SPIKE:
        return put(net.last);
      case SPK_FIELD_SYN_TRACE:
        return put(net.gtr);
      case SPK_FIELD_INPUT_NEXT:
        return put(net.in_next);
      case SPK_FIELD_RING:
        return put(net.ring);
      case SPK_FIELD_PRE_TRACE:
      case SPK_FIELD_POST_TRACE: {
        // Per-neuron view of the per-synapse traces: all plastic synapses of
        // one presynaptic (postsynaptic) neuron carry the same pre (post)
        // trace, so the value is read off any of them.  Neurons with no
        // plastic synapse read 0.
        const bool pre = field == SPK_FIELD_PRE_TRACE;
        int64_t want = pre ? (int64_t)net.Nin + net.N : (int64_t)net.N;
        if (count != want) return SPK_ERR_INVALID;
        for (int64_t i = 0; i < count; ++i) dst[i] = 0.0f;
        for (size_t j = 0; j < net.plastic_idx.size(); ++j) {
          int64_t s = net.plastic_idx[j];
          if (pre) {
            int p = net.spre[s];
            int64_t slot = p < 0 ? (int64_t)(-p - 1) : (int64_t)net.Nin + p;
            dst[slot] = (float)net.stdp_pre[j];
          } else {
            dst[net.spost[s]] = (float)net.stdp_post[j];
          }
        }
        return SPK_OK;
      }
      default:
        return SPK_ERR_INVALID;
    }
  });
}

int oracle_read_weights(const oracle_net* n, float* w, int64_t count) {
  if (!n || !w) return SPK_ERR_INVALID;
  return dispatch(n, [&](auto& net) {
    if (count != net.S) return SPK_ERR_INVALID;
    for (int64_t i = 0; i < count; ++i) w[i] = (float)net.sw[net.revsort[i]];
    return SPK_OK;
  });
}

int oracle_synaptic_events(const oracle_net* n, uint64_t* events) {
  if (!n || !events) return SPK_ERR_INVALID;
  *events = dispatch(n, [](auto& net) { return net.events; });
  return SPK_OK;
}

int oracle_ring_depth(const oracle_net* n, int32_t* depth) {
  if (!n || !depth) return SPK_ERR_INVALID;
  return dispatch(n, [&](auto& net) {
    *depth = net.B;
    return SPK_OK;
  });
}

int oracle_timestep_grouping(const oracle_net* n, int32_t* G) {
  if (!n || !G) return SPK_ERR_INVALID;
  return dispatch(n, [&](auto& net) {
    *G = net.G;
    return SPK_OK;
  });
}

int oracle_sorted_synapses(const oracle_net* n, int32_t* pre, int32_t* post, int32_t* delay,
                           int64_t count) {
  if (!n) return SPK_ERR_INVALID;
  return dispatch(n, [&](auto& net) {
    if (count != net.S || net.threads != 1) return SPK_ERR_INVALID;
    for (int64_t s = 0; s < count; ++s) {
      if (pre) pre[s] = net.spre[s];
      if (post) post[s] = net.spost[s];
      if (delay) delay[s] = net.sdelay[s];
    }
    return SPK_OK;
  });
}

void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  spk::u32x4 c{ctr[0], ctr[1], ctr[2], ctr[3]};
  spk::u32x4 r = spk::philox4x32_10(c, key[0], key[1]);
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
  out[3] = r.w;
}

float oracle_logf(float x) { return spk::logf_spk(x); }

double oracle_log_max_ulp(void) {
  double worst = 0.0;
  for (uint32_t k = 1; k < (1u << 24); ++k) {
    const float u = spk::uniform_open0((k - 1u) << 8);
    const double ex = std::log((double)u);
    const double ulp = std::ldexp(1.0, std::ilogb((float)ex) - 23);
    const double e = std::fabs((double)spk::logf_spk(u) - ex) / ulp;
    if (e > worst) worst = e;
  }
  if (spk::logf_spk(1.0f) != 0.0f) worst = 1e30;
  return worst;
}

/* Connectivity of a generated network (spk_net_generate), restated on the
 * host: for each presynaptic key in order (inputs n_inputs-1 .. 0, then
 * neurons), each projection holding it (by ascending first post) and each of
 * its posts, the pair connects when the uniform of Philox(connectivity_seed,
 * (post/4, pre code, 0, CONNECT)) word post%4 is <= p; weight lo + (hi-lo)*u1
 * and delay lo + min(floor(u2*(hi-lo+1)), hi-lo) come from Philox(post, pre
 * code, 0, SYNAPSE) words 0 and 1.  Writes up to `capacity` synapses in that
 * (creation) order with the spk_net_desc id convention and returns how many
 * there are. */
// Key range [k0, k1) of the generator restatement: counts (out == nullptr)
// or writes the synapses of those keys in creation order at out offset n0.
// One Philox block of four connection uniforms serves four consecutive posts.
struct GenOut {
  int32_t *pre, *post, *delay, *label;
  float *weight, *scale;
  uint8_t* plastic;
};
static int64_t gen_keys(const spk_gen_desc* d, const std::vector<int>& order, int k0, int k1, const GenOut* out,
                        int64_t n0, int64_t capacity) {
  int64_t n = n0;
  for (int k = k0; k < k1; ++k) {
    const bool is_input = k < d->n_inputs;
    const int idx = is_input ? d->n_inputs - 1 - k : k - d->n_inputs;
    const int pop = is_input ? SPK_POP_INPUTS : SPK_POP_NEURONS;
    const uint32_t code = is_input ? (0x80000000u | (uint32_t)idx) : (uint32_t)idx;
    for (int j : order) {
      const spk_projection& P = d->projections[j];
      if (P.pre_population != pop || idx < P.pre_start || idx >= P.pre_start + P.pre_count) continue;
      uint32_t words[4] = {0, 0, 0, 0};
      for (int q = P.post_start; q < P.post_start + P.post_count; ++q) {
        if (q == P.post_start || (q & 3) == 0) {
          const spk::u32x4 c = spk::draw4(d->connectivity_seed, (uint32_t)q >> 2, code, spk::DOMAIN_CONNECT);
          words[0] = c.x;
          words[1] = c.y;
          words[2] = c.z;
          words[3] = c.w;
        }
        if (!(spk::uniform_open0(words[q & 3]) <= P.probability)) continue;
        if (out && n < capacity) {
          const spk::u32x4 r = spk::draw4(d->connectivity_seed, (uint32_t)q, code, spk::DOMAIN_SYNAPSE);
          const float span = P.weight_hi - P.weight_lo;
          const float w = P.weight_lo + span * spk::uniform_open0(r.x);
          const int nd = P.delay_hi - P.delay_lo + 1;
          int dd = (int)(spk::uniform_open0(r.y) * (float)nd);
          if (dd > nd - 1) dd = nd - 1;
          if (out->pre) out->pre[n] = is_input ? -idx - 1 : idx;
          if (out->post) out->post[n] = q;
          if (out->weight) out->weight[n] = w;
          if (out->scale) out->scale[n] = P.scale;
          if (out->delay) out->delay[n] = P.delay_lo + dd;
          if (out->label) out->label[n] = P.label;
          if (out->plastic) out->plastic[n] = P.plastic ? 1 : 0;
        }
        ++n;
      }
    }
  }
  return n - n0;
}

// The device generator (spk_gen.cuh) restated: every (pre, post) pair of a
// projection connects when its Philox(connectivity seed, post/4, pre code)
// uniform is at most the probability; a connected pair's weight and delay
// come from Philox(post, pre code).  Creation order: ascending presynaptic
// key (inputs in reverse order first, then neurons), projections by first
// post, posts ascending.  Keys are split over host threads; each range is
// counted, then written at its offset, so the order does not depend on them.
int64_t oracle_generate(const spk_gen_desc* d, int32_t* pre, int32_t* post, float* weight, float* scale,
                        int32_t* delay, int32_t* label, uint8_t* plastic, int64_t capacity) {
  if (!d || d->n_projections < 0 || (d->n_projections > 0 && !d->projections)) return -1;
  std::vector<int> order(d->n_projections);
  for (int j = 0; j < d->n_projections; ++j) order[j] = j;
  for (int a = 1; a < d->n_projections; ++a)  // stable insertion sort by first post
    for (int b = a; b > 0 && d->projections[order[b]].post_start < d->projections[order[b - 1]].post_start; --b) {
      const int t = order[b];
      order[b] = order[b - 1];
      order[b - 1] = t;
    }
  const int n_keys = d->n_inputs + d->n_neurons;
  const int T = std::max(1, std::min<int>((int)std::thread::hardware_concurrency(), 64));
  const int parts = std::max(1, std::min(n_keys, 4 * T));
  std::vector<int64_t> cnt(parts + 1, 0);
  auto key_of = [&](int p) { return (int)((int64_t)n_keys * p / parts); };
  auto run = [&](auto&& fn) {
    std::vector<std::thread> pool;
    std::atomic<int> next{0};
    for (int t = 0; t < T; ++t)
      pool.emplace_back([&]() {
        for (int p = next++; p < parts; p = next++) fn(p);
      });
    for (auto& th : pool) th.join();
  };
  run([&](int p) { cnt[p + 1] = gen_keys(d, order, key_of(p), key_of(p + 1), nullptr, 0, 0); });
  for (int p = 0; p < parts; ++p) cnt[p + 1] += cnt[p];
  const int64_t n = cnt[parts];
  const GenOut out{pre, post, delay, label, weight, scale, plastic};
  const bool any = pre || post || delay || label || weight || scale || plastic;
  if (any && capacity > 0)
    run([&](int p) {
      if (cnt[p] < capacity) gen_keys(d, order, key_of(p), key_of(p + 1), &out, cnt[p], capacity);
    });
  return n;
}

}  // extern "C"
