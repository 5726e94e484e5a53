// spk_bulk.cuh - bulk-synchronous stepping of a batch of networks.
//
// The persistent step kernel keeps each network's state in shared memory and
// synchronizes a network's CTAs every timestep through stamped words in
// global memory; a batch then runs as co-resident waves, each as slow as its
// slowest network.  In bulk mode every timestep is instead three kernels over
// all tiles of all networks of the batch, with the state in HBM and kernel
// boundaries as the only synchronization:
//
//   bulk_neurons_kernel  one warp per 32 keys: LIF + injection and Poisson
//                        inputs (the persistent kernel's phase A), STDP
//                        traces, spike / pre-event words into the network's
//                        bitmaps;
//   bulk_list_kernel     one CTA per network: the step's active keys in
//                        canonical (ascending key) order from the bitmaps, and
//                        the spike store;
//   bulk_prop_kernel     one warp per tile: the list's sub-rows of the tile
//                        staged and applied in canonical order into the tile's
//                        ring cells in HBM (the persistent kernel's rounds),
//                        with the STDP pre pass;
//   bulk_post_kernel     the post-spike afferent pass of every spiking post of
//                        every network, a warp per spiking post taken from a
//                        shared list (the list kernel builds the items);
//   bulk_dense_stdp_kernel, bulk_norm_kernel
//                        a warp per post of the networks with a
//                        per-synapse-trace STDP rule or the weight
//                        normalisation (these run in bulk mode only).
//
// Each ring cell still has one writer applying contributions in canonical
// order, and every float operation is the persistent kernel's, so a network
// gives the same bits in both modes.  A block of K timesteps is 3 to 8
// launches per timestep plus one that advances the networks' run counters,
// captured in a CUDA graph.
#pragma once

#include <cuda_runtime.h>

#include "spk_internal.h"
#include "spk_kernel.cuh"

// Tuning constants (measured on the 256-instance sweep): keys per round and
// entries per stage of the propagation kernel, words per warp of the neuron
// kernel.
#ifndef SPK_BULK_STAGE_KEYS
#define SPK_BULK_STAGE_KEYS 64
#endif
#ifndef SPK_BULK_STAGE_ENTRIES
#define SPK_BULK_STAGE_ENTRIES 256
#endif
#ifndef SPK_BULK_WPW
#define SPK_BULK_WPW 2
#endif

namespace spk {

constexpr int BULK_STAGE_KEYS = SPK_BULK_STAGE_KEYS;

// Programmatic dependent launch: a timestep's kernels are launched so that the
// next one's CTAs may start while this one drains.  Each kernel reads only
// static data (block records, descriptors, run control) before pdl_wait(),
// which returns once the previous kernel has completed and its writes are
// visible, and lets its own dependents launch only after that, so every
// earlier kernel of the stream has completed too.
__device__ __forceinline__ void pdl_wait_then_release() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
constexpr int BULK_STAGE_ENTRIES = SPK_BULK_STAGE_ENTRIES;  // entries staged per warp at a time

// Timestep s of the current block of a network's run.
struct BulkStep {
  float t, tg;
  int T, slot, g, sr;  // g: substep of the group; sr: timestep of the run
  bool live, stdp_run, inputs_active;
  // the group has the parity of the group step before it: its substeps
  // deliver that group's spikes again (bulk_rep; set by the kernels that use it)
  bool rep;
  bool dense_run;  // a per-synapse-trace rule updates this step
};

__device__ __forceinline__ BulkStep bulk_step(const NetDev& d, const RunCtl& c, int s) {
  BulkStep b;
  const int sr = c.step + s;
  b.live = sr < c.steps_total;
  const float dt = d.dt;
  group_time(c.start_time, sr, d.G, dt, b.t, b.T, b.tg);
  b.slot = b.T % d.B;
  b.g = d.G == 1 ? 0 : sr % d.G;
  // the event-driven (weight-dependent) rule's passes, or the per-synapse-trace rules' pass
  b.stdp_run = d.has_stdp && c.plastic && d.stdp_rule == SPK_STDP_WEIGHT_DEPENDENT;
  b.dense_run = d.has_stdp && c.plastic && d.stdp_rule != SPK_STDP_WEIGHT_DEPENDENT;
  b.inputs_active = c.inputs_active != 0 || s > 0;
  b.sr = sr;
  b.rep = false;
  return b;
}

// group_repeats for the step (one float division): the neuron and list kernels
__device__ __forceinline__ bool bulk_rep(const NetDev& d, const RunCtl& c, const BulkStep& st) {
  return group_repeats(c, st.sr, d.G == 1 ? st.T : (st.T - st.g) / d.G, d.G, d.dt);
}

__device__ __forceinline__ RunCtl load_ctl(const RunCtl* p) {
  RunCtl c;
  c.start_time = p->start_time;
  c.step = p->step;
  c.steps_total = p->steps_total;
  c.plastic = p->plastic;
  c.inputs_active = p->inputs_active;
  c.record_inputs = p->record_inputs;
  c.repeat = p->repeat;
  return c;
}

// ---- timestep part 1: neurons and inputs -------------------------------------------
// One CTA per block of up to BULK_BLOCK_WORDS consecutive 32-key words of one
// network (inputs: keys 0..n_inputs-1; neurons: keys KL..KL+N-1), each warp
// BULK_WPW of them.  The CTA copies the network's descriptor and run control
// into shared memory with one round of parallel loads, so each warp's only
// dependent global loads are its state loads, all issued before any update.
// Words of padding keys are never written: they stay zero from set-up.
#ifndef SPK_BULK_NEUR_MINB
#define SPK_BULK_NEUR_MINB 4
#endif
#ifndef SPK_BULK_NEUR_CTAS_PER_SM
#define SPK_BULK_NEUR_CTAS_PER_SM 8
#endif
constexpr int BULK_WPW = SPK_BULK_WPW;
#ifndef SPK_BULK_NEUR_WARPS
#define SPK_BULK_NEUR_WARPS 8
#endif
constexpr int BULK_NEUR_WARPS = SPK_BULK_NEUR_WARPS;
constexpr int BULK_BLOCK_WORDS = BULK_NEUR_WARPS * BULK_WPW;

struct BulkBlock {
  int net;            // index into the batch's NetDev array
  int word;           // first word (key / 32)
  int count;          // words in the block (<= BULK_BLOCK_WORDS), all inputs or all neurons
  int pad;
  const RunCtl* ctl;  // the network's run control, loaded beside its descriptor
  const void* pad2;
};

// LIF update of neuron n (the persistent kernel's phase A, same operations)
// with its state already loaded; returns whether it spiked.
__device__ __forceinline__ bool bulk_lif(const NetDev& d, const BulkStep& st, int n, int key, float Vi,
                                         float lastn, float* ring_cell, float input_voltage) {
  int gi = 0;
  while (gi + 1 < d.n_groups && n >= d.groups[gi].end) ++gi;
  const GroupConst G = d.groups[gi];
  const int L = d.L, kind = d.kind;
  float input;
  if (kind == SPK_SYN_CONDUCTANCE) {
    float total = 0.0f;
    for (int l = 0; l < L; ++l) {
      const float cell = ring_cell[l];
      ring_cell[l] = 0.0f;
      const float gnew = d.decay[l] * d.gtr[(size_t)n * L + l] + cell;
      total = total + gnew * (d.vhat[l] - Vi);
      d.gtr[(size_t)n * L + l] = gnew;
    }
    input = total * G.kR;
  } else if (kind == SPK_SYN_CURRENT) {
    float total = 0.0f;
    for (int l = 0; l < L; ++l) {
      const float cell = ring_cell[l];
      ring_cell[l] = 0.0f;
      float inew = d.gtr[(size_t)n * L + l] * d.decay[l];
      inew = inew + cell;
      total = total + inew;
      d.gtr[(size_t)n * L + l] = inew;
    }
    input = total * G.kR;
  } else {
    // voltage synapses: the caller summed the labels' cells in label order
    input = input_voltage;
  }
  bool spk = false;
  if (((st.tg - lastn) - d.t_ref) > 0.5f * d.dt) {
    Vi = G.k * G.v0 + (1.0f - G.k) * Vi + G.k * d.i_bg + input;
    if (Vi >= G.theta) {
      spk = true;
      d.last[n] = st.tg;
      Vi = G.vreset;
      if (d.rate_counts) d.rate_counts[key] += 1;
    }
  }
  d.V[n] = Vi;
  return spk;
}

// One block's words of one network, with the network's descriptor and the
// step's times in shared memory (no barrier inside: warps return early).
__device__ __forceinline__ void bulk_neurons_block(const NetDev& d, const BulkStep st, const BulkBlock& bb) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int w0 = w * BULK_WPW;
  if (w0 >= bb.count) return;
  struct {
    int word, count;
  } const bw = {bb.word + w0, min(BULK_WPW, bb.count - w0)};
  const int KL = d.KL;
  float* pub = d.pre_pub;
  if (bw.word * 32 >= KL) {
    const int N = d.N, L = d.L, B = d.B, TS = d.TS, kind = d.kind;
    // a word lies in one tile (TS is a multiple of 32): its tile by a shift
    // when TS is a power of two
    const bool ts_pow2 = (TS & (TS - 1)) == 0;
    const int ts_shift = __ffs(TS) - 1;
    float Vv[BULK_WPW], lv[BULK_WPW], inv[BULK_WPW], pov[BULK_WPW], prv[BULK_WPW];
    float* cellp[BULK_WPW];
    // phase 1: every word's loads in flight at once
#pragma unroll
    for (int u = 0; u < BULK_WPW; ++u) {
      Vv[u] = lv[u] = inv[u] = pov[u] = prv[u] = 0.0f;
      const int n = (bw.word + u) * 32 + lane - KL;
      const int tile = ts_pow2 ? n >> ts_shift : n / TS, li = n - tile * TS;
      cellp[u] = d.ring + ((size_t)tile * B + st.slot) * TS * L + (size_t)li * L;
      if (u < bw.count && n < N) {
        Vv[u] = d.V[n];
        lv[u] = d.last[n];
        if (kind == SPK_SYN_VOLTAGE) {
          const float* cell = cellp[u];
          float total = 0.0f;
          for (int l = 0; l < L; ++l) total = total + cell[l];
          inv[u] = total;
        }
        if (st.stdp_run) {
          pov[u] = d.post_trace[n];
          prv[u] = d.pre_trace[KL + n];
        }
      }
    }
    // phase 2: updates, traces, spike words
#pragma unroll
    for (int u = 0; u < BULK_WPW; ++u) {
      if (u >= bw.count) break;
      const int key = (bw.word + u) * 32 + lane;
      const int n = key - KL;
      bool spk = false, ev = false, pe = false;
      if (n < N) {
        float* cell = cellp[u];
        spk = bulk_lif(d, st, n, key, Vv[u], lv[u], cell, inv[u]);
        if (kind == SPK_SYN_VOLTAGE)
          for (int l = 0; l < L; ++l) cell[l] = 0.0f;
        if (st.stdp_run) {
          // g = roundf((last - t)/dt)
          // (Spike/Backend/CUDA/Plasticity/WeightDependentSTDPPlasticity.cu:113-117):
          // an event as the postsynaptic neuron for g >= 0, as the
          // presynaptic one for g == 0 (g >= G is negated), as in the
          // persistent kernel.  A spike older than a step cannot round to 0.
          const float lag = lv[u] - st.t;
          const int gq = (spk || lag < -d.dt) ? (spk ? 0 : -1) : (int)roundf(lag / d.dt);
          ev = gq >= 0;
          pe = gq == 0;
          float po = pov[u] * d.E_m;
          po = po + (ev ? d.inc_m : 0.0f);
          d.post_trace[n] = po;
          float pr = prv[u] * d.E_p;
          pr = pr + (pe ? d.inc_p : 0.0f);
          d.pre_trace[key] = pr;
          pub[key] = pr;
        }
      }
      const unsigned word = __ballot_sync(FULL, spk);
      const unsigned evword = st.stdp_run ? __ballot_sync(FULL, ev) : 0u;
      const unsigned peword = st.stdp_run ? __ballot_sync(FULL, pe) : 0u;
      if (lane == 0) {
        // delivered keys: the spikes, and in a repeating group the carried keys
        uint32_t* gb = d.gbits + (size_t)st.g * d.n_words + bw.word + u;
        d.bitsA[bw.word + u] = word | (st.rep ? *gb : 0u);
        d.bitsP[bw.word + u] = peword;
        d.bitsE[bw.word + u] = evword;
        if (d.hist) d.hist[(size_t)(st.T % d.H) * d.n_words + bw.word + u] = word;
        *gb = word;
      }
    }
  } else {
    // Poisson inputs (same operations as the persistent kernel)
    const int Nin = d.Nin;
    float nxv[BULK_WPW], rtv[BULK_WPW], prv[BULK_WPW];
#pragma unroll
    for (int u = 0; u < BULK_WPW; ++u) {
      nxv[u] = rtv[u] = prv[u] = 0.0f;
      const int key = (bw.word + u) * 32 + lane;
      if (u < bw.count && key < Nin) {
        nxv[u] = d.in_next[Nin - 1 - key];
        rtv[u] = d.rates[Nin - 1 - key];
        if (st.stdp_run) prv[u] = d.pre_trace[key];
      }
    }
#pragma unroll
    for (int u = 0; u < BULK_WPW; ++u) {
      if (u >= bw.count) break;
      const int key = (bw.word + u) * 32 + lane;
      bool spk = false, pev = false;
      if (key < Nin) {
        const int idx = Nin - 1 - key;
        float nx = nxv[u];
        if ((nx <= st.tg) || !st.inputs_active) {
          const float u01 = draw_uniform(d.seed, (uint32_t)idx, (uint32_t)st.T, DOMAIN_POISSON);
          nx = st.tg - (1.0f / rtv[u]) * logf_spk(u01);
          if (st.inputs_active) {
            spk = true;
            if (d.rate_counts) d.rate_counts[key] += 1;
          }
        }
        d.in_next[idx] = nx;
        if (st.stdp_run) {
          int pg = (int)roundf((nx - st.t) / d.dt);
          if (pg >= 1) pg *= -1;
          pev = pg >= 0;
          float pr = prv[u] * d.E_p;
          pr = pr + (pev ? d.inc_p : 0.0f);
          d.pre_trace[key] = pr;
          pub[key] = pr;
        }
      }
      const unsigned wa = __ballot_sync(FULL, spk);
      const unsigned wp = __ballot_sync(FULL, pev);
      if (lane == 0) {
        uint32_t* gb = d.gbits + (size_t)st.g * d.n_words + bw.word + u;
        d.bitsA[bw.word + u] = wa | (st.rep ? *gb : 0u);
        d.bitsP[bw.word + u] = wp;
        if (d.hist) d.hist[(size_t)(st.T % d.H) * d.n_words + bw.word + u] = wa;
        *gb = wa;
      }
    }
  }
}

// The network's descriptor and the step's times (two float divisions, thread 0)
// into shared memory.
__device__ __forceinline__ void bulk_load_net(NetDev& sd, BulkStep& sst, const NetDev* __restrict__ nets,
                                              const BulkBlock& bb, int s) {
  const uint32_t* src = (const uint32_t*)(nets + bb.net);
  uint32_t* dst = (uint32_t*)&sd;
  for (int i = threadIdx.x; i < (int)(sizeof(NetDev) / 4); i += blockDim.x) dst[i] = __ldg(src + i);
  if (threadIdx.x == 0) {
    const RunCtl c = load_ctl(bb.ctl);
    BulkStep b = bulk_step(nets[bb.net], c, s);
    if (b.live) b.rep = bulk_rep(nets[bb.net], c, b);
    sst = b;
  }
}

// CTA c takes the blocks [c*n/grid, (c+1)*n/grid) in turn.  Blocks are listed
// network by network, so consecutive blocks mostly share a network, whose
// descriptor and step the CTA loads once; with grid = n every CTA takes one
// block.
__global__ void __launch_bounds__(BULK_NEUR_WARPS * 32, SPK_BULK_NEUR_MINB)
    bulk_neurons_kernel(const NetDev* __restrict__ nets, const BulkBlock* __restrict__ blocks, int n_blocks, int s,
                        int* item_count) {
  __shared__ __align__(16) NetDev sd;
  __shared__ BulkStep sst;
  static_assert(sizeof(NetDev) % 4 == 0, "descriptor copied as words");
  const int b0 = (int)((long long)blockIdx.x * n_blocks / gridDim.x);
  const int b1 = (int)((long long)(blockIdx.x + 1) * n_blocks / gridDim.x);
  int cur = -1;
  for (int bi = b0; bi < b1; ++bi) {
    const BulkBlock bb = blocks[bi];
    if (bb.net != cur) {
      if (cur >= 0) {
        __syncthreads();  // every warp is done with the previous network's descriptor
      }
      bulk_load_net(sd, sst, nets, bb, s);
      if (cur < 0) {
        // the first descriptor (static data) is read before the wait
        pdl_wait_then_release();
        if (blockIdx.x == 0 && threadIdx.x == 0) *item_count = 0;  // the afferent-pass list of this step
      }
      __syncthreads();
      cur = bb.net;
    }
    if (sst.live) bulk_neurons_block(sd, sst, bb);
  }
  if (cur < 0) pdl_wait_then_release();
}

// ---- timestep part 2: the step's active keys and the spike store ----------------------
// One CTA of BULK_LIST_THREADS per network; each thread owns a contiguous run
// of bitmap words, so a block-wide exclusive scan of the per-thread counts
// gives every key its place in ascending key order.
constexpr int BULK_LIST_THREADS = 512;

// Work item of the afferent pass: spiking post `post` of network `net`.
struct BulkPostItem {
  int net, post;
};
// Work item of the per-synapse-trace rules' and the normalisation's passes: a
// post with plastic afferents and the range [a0, a1) of its records, fixed
// when the batch is set up.
struct BulkRuleItem {
  int net, post, a0, a1;
};
constexpr int BULK_POST_CHUNK = 128;  // afferents per warp iteration (32 lanes x 4)

__global__ void __launch_bounds__(BULK_LIST_THREADS) bulk_list_kernel(const NetDev* __restrict__ nets, int s,
                                                                      BulkPostItem* items, int* item_count,
                                                                      int item_cap) {
  __shared__ unsigned long long warp_tot[BULK_LIST_THREADS / 32];
  __shared__ unsigned long long s_base;
  __shared__ int s_item_base;
  const NetDev& d = nets[blockIdx.x];
  const RunCtl c = load_ctl(d.ctl);
  BulkStep st = bulk_step(d, c, s);
  st.rep = bulk_rep(d, c, st);
  pdl_wait_then_release();
  if (!st.live) {
    if (threadIdx.x == 0) *d.step_count = 0;
    return;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n_words = d.n_words, KL = d.KL;
  const bool rec_inputs = c.record_inputs != 0;
  // a carried list of two earlier groups is beyond this engine
  if (threadIdx.x == 0 && st.rep && st.g == 0 && st.sr >= d.G &&
      group_repeats(c, st.sr - d.G, group_index(c.start_time, st.sr - d.G, d.G, d.dt), d.G, d.dt))
    atomicCAS(&d.ctl->status, 0, SPK_ERR_UNSUPPORTED);
  const bool recording = d.spike_cap > 0;  // a network created without a spike store records nothing
  const int per = (n_words + BULK_LIST_THREADS - 1) / BULK_LIST_THREADS;
  const int w0 = min(n_words, threadIdx.x * per), w1 = min(n_words, w0 + per);
  // counts: list keys (low 32 bits) and recorded spikes (high 32 bits); the
  // step's spikes are its group words (bitsA also holds carried keys)
  const uint32_t* spw = d.gbits + (size_t)st.g * n_words;
  unsigned long long cnt = 0;
  for (int i = w0; i < w1; ++i) {
    const uint32_t a = d.bitsA[i], p = d.bitsP[i];
    const bool rec = recording && ((i << 5) >= KL || rec_inputs);
    cnt += (unsigned long long)__popc(a | p) + (rec ? ((unsigned long long)__popc(spw[i]) << 32) : 0ull);
  }
  unsigned long long incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    const unsigned long long v = lane < BULK_LIST_THREADS / 32 ? warp_tot[lane] : 0ull;
    unsigned long long wi = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(FULL, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < BULK_LIST_THREADS / 32) warp_tot[lane] = wi - v;  // exclusive per warp
    if (lane == 31) s_base = wi;                                // block total
  }
  __syncthreads();
  const unsigned long long excl = warp_tot[w] + incl - cnt;
  int pos = (int)(excl & 0xffffffffull);
  const unsigned long long sc0 = d.ctl->spike_count;
  unsigned long long sp = sc0 + (excl >> 32);
  for (int i = w0; i < w1; ++i) {
    const uint32_t a = d.bitsA[i], p = d.bitsP[i], sw = spw[i];
    const bool rec = recording && ((i << 5) >= KL || rec_inputs);
    uint32_t m = a | p;
    while (m) {
      const int b = __ffs(m) - 1;
      m &= m - 1;
      const uint32_t key = (uint32_t)(i << 5) + (uint32_t)b;
      const uint32_t fa = (a >> b) & 1u, fp = (p >> b) & 1u;
      d.step_list[pos++] = key | (fa << 31) | (fp << 30);
      if (((sw >> b) & 1u) && rec) {
        if (sp < (unsigned long long)d.spike_cap)
          d.spikes[sp] = make_uint2(key, __float_as_uint(st.tg));
        else
          atomicCAS(&d.ctl->status, 0, SPK_ERR_OVERFLOW);
        ++sp;
      }
    }
  }
  __syncthreads();  // every thread has read spike_count
  if (threadIdx.x == 0) {
    *d.step_count = (int)(s_base & 0xffffffffull);
    const unsigned long long sc = sc0 + (s_base >> 32);
    d.ctl->spike_count = sc > (unsigned long long)d.spike_cap ? (unsigned long long)d.spike_cap : sc;
  }
  if (!st.stdp_run) return;
  // afferent-pass items: one per post with an STDP event (its spike, or at a
  // repeating run start the last step's), reserved in the shared item list
  // with one atomic per network
  const int wl0 = max(w0, KL >> 5);
  int nsp = 0;
  for (int i = wl0; i < w1; ++i) nsp += __popc(d.bitsE[i]);
  int ic = nsp;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(FULL, ic, o);
    if (lane >= o) ic += y;
  }
  __syncthreads();
  if (lane == 31) warp_tot[w] = (unsigned long long)ic;
  __syncthreads();
  if (w == 0) {
    const int v = lane < BULK_LIST_THREADS / 32 ? (int)warp_tot[lane] : 0;
    int wi = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < BULK_LIST_THREADS / 32) warp_tot[lane] = (unsigned long long)(wi - v);
    if (lane == 31) s_item_base = wi > 0 ? atomicAdd(item_count, wi) : 0;
  }
  __syncthreads();
  int ipos = s_item_base + (int)warp_tot[w] + ic - nsp;
  for (int i = wl0; i < w1; ++i) {
    uint32_t a = d.bitsE[i];
    while (a) {
      const int b = __ffs(a) - 1;
      a &= a - 1;
      if (ipos < item_cap)
        items[ipos] = BulkPostItem{(int)blockIdx.x, (i << 5) + b - KL};
      else
        atomicCAS(&d.ctl->status, 0, SPK_ERR_OVERFLOW);
      ++ipos;
    }
  }
}

// ---- timestep part 3: propagation and STDP ----------------------------------------------
// One CTA per group of up to BULK_PROP_WARPS consecutive tiles of one network,
// one warp per tile.  The CTA shares what every tile of the network reads
// alike: the descriptor and run control (copied once), the step's key list
// (staged BULK_LIST_CHUNK keys at a time) and, per round of BULK_STAGE_KEYS
// keys, the keys' rowptr words of the CTA's tiles (one sector per key) and
// their presynaptic traces.  Round r + 1 is staged while the warps stage and
// apply round r's entries, so a round costs a warp two dependent loads (its
// entries, then the plastic weights they name) instead of four.
//
// Shared memory: the CTA part (list chunk, two rounds of rowptr words, key
// flags and pre traces, class scales) and per warp (entry stage, the
// tile's post traces and spike words, and `win`, the tile's ring window: the
// delay slots 1..ws after the current one, each TS * L words, read from HBM
// when the step's entries fill enough of it and written back once per dirty
// slot; contributions outside the window go to HBM directly).
#ifndef SPK_BULK_PROP_WARPS
#define SPK_BULK_PROP_WARPS 8
#endif
constexpr int BULK_PROP_WARPS = SPK_BULK_PROP_WARPS;
constexpr int BULK_RPW = BULK_PROP_WARPS + 1;  // rowptr words per key: the tiles' starts and the last end
constexpr int BULK_LIST_CHUNK = 1024;          // list keys staged at a time (a multiple of BULK_STAGE_KEYS)
#ifndef SPK_BULK_WIN_CAP
#define SPK_BULK_WIN_CAP 1024
#endif
constexpr int BULK_WIN_CAP = SPK_BULK_WIN_CAP;  // ring-window words per warp at most
static_assert(BULK_LIST_CHUNK % BULK_STAGE_KEYS == 0, "rounds never straddle a list chunk");
static_assert(BULK_STAGE_KEYS % 32 == 0, "a round is whole lanes' worth of keys");

struct BulkPropBlock {
  int net;    // index into the batch's NetDev array
  int tile0;  // first tile
  int n;      // tiles (<= BULK_PROP_WARPS)
  int pad;
  const RunCtl* ctl;     // the network's run control
  const int* n_list;     // the network's step key count
};

struct BulkPropLayout {
  // CTA part
  int list, rp, kfl, kpre, scl, cta;
  // per warp
  int stage, stw, sidx, ptr, spw, win, warp;
  int total;  // words
};
__host__ __device__ inline BulkPropLayout bulk_prop_layout(int win_words, int ts_max) {
  BulkPropLayout l;
  int o = 0;
  l.list = o; o += BULK_LIST_CHUNK;
  l.rp = o; o += 2 * BULK_STAGE_KEYS * BULK_RPW;
  l.kfl = o; o += 2 * BULK_STAGE_KEYS;
  l.kpre = o; o += 2 * BULK_STAGE_KEYS;
  l.scl = o; o += MAX_CLASSES;
  o = (o + 3) & ~3;
  l.cta = o;
  int p = 0;
  l.stage = p; p += 2 * BULK_STAGE_ENTRIES;
  l.stw = p; p += BULK_STAGE_ENTRIES;
  l.sidx = p; p += BULK_STAGE_ENTRIES / 2;
  l.ptr = p; p += ts_max;       // post traces of the tile (plastic runs)
  l.spw = p; p += ts_max / 32;  // spike words of the tile's posts (plastic runs)
  p = (p + 3) & ~3;
  l.win = p; p += win_words;    // 16-byte aligned
  p = (p + 3) & ~3;
  l.warp = p;
  l.total = l.cta + BULK_PROP_WARPS * l.warp;
  return l;
}
#ifndef SPK_BULK_PROP_MINB
#define SPK_BULK_PROP_MINB 3
#endif

// kPass: 0 the single fused pass; 1 and 2 the two passes of a batch in which
// a network normalises its weights after the event-driven rule (see below).
template <int kPass>
__global__ void __launch_bounds__(BULK_PROP_WARPS * 32, SPK_BULK_PROP_MINB)
    bulk_prop_kernel(const NetDev* __restrict__ nets, const BulkPropBlock* __restrict__ blocks, int s, int win_words,
                     int ts_max) {
  extern __shared__ __align__(16) uint32_t bsm[];
  __shared__ __align__(16) NetDev sd;
  __shared__ RunCtl sctl;
  __shared__ BulkStep sst;
  __shared__ int s_nlist;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nthr = BULK_PROP_WARPS * 32;
  const BulkPropBlock pb = blocks[blockIdx.x];
  {
    const uint32_t* src = (const uint32_t*)(nets + pb.net);
    uint32_t* dst = (uint32_t*)&sd;
    for (int i = threadIdx.x; i < (int)(sizeof(NetDev) / 4); i += nthr) dst[i] = __ldg(src + i);
    if (threadIdx.x == 0) {
      sctl = load_ctl(pb.ctl);
      sst = bulk_step(nets[pb.net], sctl, s);  // once per CTA
    }
  }
  pdl_wait_then_release();
  if (threadIdx.x == 0) s_nlist = *pb.n_list;
  __syncthreads();
  const NetDev& d = sd;
  BulkStep st = sst;
  const int n_list = s_nlist;
  if (!st.live || n_list == 0) return;  // the whole CTA
  // A network that normalises its weights after the event-driven rule's
  // updates takes two passes: the first (pass 1) only updates weights, the
  // second (pass 2, after the normalisation) only delivers.  Pass 1 does both
  // for the other networks of the batch; pass 2 skips them.
  uint32_t kmask = 0xffffffffu;
  if constexpr (kPass != 0) {
    const bool split =
        d.weight_norm == SPK_NORM_AFTER_RULE && d.has_stdp && d.stdp_rule == SPK_STDP_WEIGHT_DEPENDENT;
    if (!split) {
      if (kPass == 2) return;
    } else if (kPass == 1) {
      kmask = ~(1u << 31);
    } else {
      kmask = ~(1u << 30);
      st.stdp_run = false;
    }
  }
  const BulkPropLayout wl = bulk_prop_layout(win_words, ts_max);
  uint32_t* list_s = bsm + wl.list;
  int* rp_s = (int*)(bsm + wl.rp);
  uint32_t* kfl_s = bsm + wl.kfl;
  float* kpre_s = (float*)(bsm + wl.kpre);
  float* scl_s = (float*)(bsm + wl.scl);
  uint32_t* wreg = bsm + wl.cta + w * wl.warp;
  uint2* stage = (uint2*)(wreg + wl.stage);
  float* stage_w = (float*)(wreg + wl.stw);
  unsigned short* sidx = (unsigned short*)(wreg + wl.sidx);
  float* ptr_s = (float*)(wreg + wl.ptr);
  uint32_t* spw_s = wreg + wl.spw;
  float* win_s = (float*)(wreg + wl.win);

  const int TS = d.TS, L = d.L, B = d.B, KL = d.KL, n_tiles = d.n_tiles;
  const bool active = w < pb.n;  // warps past the network's last tile only help to stage
  const int t_idx = pb.tile0 + w, nrp = pb.n + 1;
  const int p0 = t_idx * TS;
  const int slot_words = TS * L;  // a multiple of 32
  float* ring = d.ring + (size_t)t_idx * B * slot_words;
  const float* pub = d.pre_pub;
  const uint32_t* step_list = d.step_list;
  const int* rowptr = d.rowptr + pb.tile0;
  const uint2* entries = d.entries;
  uint2* csc = d.csc;
  const bool has_stdp = d.has_stdp != 0;
  const StdpConst sc = stdp_const(d);
  if (threadIdx.x < MAX_CLASSES) scl_s[threadIdx.x] = d.scale_tab[threadIdx.x];

  // staging of one round's keys into buffer `buf` (all threads)
  auto stage_round = [&](int kb, int buf) {
    const int nk = min(BULK_STAGE_KEYS, n_list - kb);
    const int lb = kb % BULK_LIST_CHUNK;
    int* rp = rp_s + buf * BULK_STAGE_KEYS * BULK_RPW;
    for (int i = threadIdx.x; i < nk * nrp; i += nthr) {
      const int j = i / nrp, t = i - j * nrp;
      const uint32_t key = list_s[lb + j] & 0x3fffffffu;
      cp_async4(rp + j * BULK_RPW + t, rowptr + (size_t)key * n_tiles + t);
    }
    for (int j = threadIdx.x; j < nk; j += nthr) {
      const uint32_t lv = list_s[lb + j];
      kfl_s[buf * BULK_STAGE_KEYS + j] = lv & kmask;
      if (st.stdp_run) cp_async4(kpre_s + buf * BULK_STAGE_KEYS + j, pub + (lv & 0x3fffffffu));
    }
  };
  auto stage_list = [&](int kb) {
    const int n = min(BULK_LIST_CHUNK, n_list - kb);
    for (int i = threadIdx.x; i < n; i += nthr) cp_async4(list_s + i, step_list + kb + i);
  };

  if (active && st.stdp_run) {
    for (int i = lane; i < TS; i += 32) {
      if (p0 + i < d.N)
        cp_async4(ptr_s + i, d.post_trace + p0 + i);
      else
        ptr_s[i] = 0.0f;
    }
    for (int i = lane; i < TS / 32; i += 32) spw_s[i] = d.bitsE[((KL + p0) >> 5) + i];  // post events
  }
  stage_list(0);
  cp_async_wait_all();
  __syncthreads();
  stage_round(0, 0);

  unsigned long long ev = 0, n_pre = 0;
  unsigned dirty = 0u;  // window slots this lane wrote
  int ws = 0;           // the ring window's depth, chosen once the first round's entries are counted
  for (int kb = 0, r = 0; kb < n_list; kb += BULK_STAGE_KEYS, ++r) {
    const int buf = r & 1;
    const int nk = min(BULK_STAGE_KEYS, n_list - kb);
    cp_async_wait_all();
    __syncthreads();  // round r staged; every warp is done with round r - 1's buffer
    const int kn = kb + BULK_STAGE_KEYS;
    if (kn < n_list) {
      if (kn % BULK_LIST_CHUNK == 0) {
        stage_list(kn);
        cp_async_wait_all();
        __syncthreads();
      }
      stage_round(kn, buf ^ 1);
    }
    if (!active) continue;
    const int* rp = rp_s + buf * BULK_STAGE_KEYS * BULK_RPW;
    const uint32_t* kfl = kfl_s + buf * BULK_STAGE_KEYS;
    const float* kpre = kpre_s + buf * BULK_STAGE_KEYS;
    // the tile's sub-row lengths and their exclusive prefix: each lane takes
    // KPL consecutive keys, one warp scan for the round
    constexpr int KPL = BULK_STAGE_KEYS / 32;
    int lens[KPL], kstart[KPL];  // the lane's keys: sub-row lengths and first entries
    int lsum = 0;
#pragma unroll
    for (int u = 0; u < KPL; ++u) {
      const int i = lane * KPL + u;
      int len = 0;
      kstart[u] = 0;
      if (i < nk) {
        kstart[u] = rp[i * BULK_RPW + w];
        len = rp[i * BULK_RPW + w + 1] - kstart[u];
        if (kfl[i] >> 31) ev += (unsigned long long)len;
      }
      lens[u] = len;
      lsum += len;
    }
    int incl = lsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += y;
    }
    const int lane_off = incl - lsum;  // first stage slot of the lane's keys
    const int total_e = __shfl_sync(FULL, incl, 31);
    if (r == 0) {
      // A window pays when the step's entries (estimated from the first
      // round) would touch more sectors one by one than the window holds;
      // its reads overlap the first round's entry staging.
      const int ws_max = min(min(B - 2 * d.G - 1, 32), win_words / slot_words);  // D_max slots at most
      const long long est = (long long)total_e * ((n_list + BULK_STAGE_KEYS - 1) / BULK_STAGE_KEYS);
      ws = (ws_max > 0 && est * 8 > (long long)ws_max * slot_words) ? ws_max : 0;
      for (int k = 0; k < ws; ++k) {
        int sl = st.slot + 1 + k;
        if (sl >= B) sl -= B;
        const float* src = ring + (size_t)sl * slot_words;
        float* dst = win_s + k * slot_words;
        for (int i = lane * 4; i < slot_words; i += 128) cp_async16(dst + i, src + i);
      }
    }
    __syncwarp();
    for (int f0 = 0; f0 < total_e; f0 += BULK_STAGE_ENTRIES) {
      const int nf = min(BULK_STAGE_ENTRIES, total_e - f0);
      // each lane copies the part of its keys' sub-rows that falls in this
      // stage [f0, f0 + nf), all from registers: one loop over the lane's
      // consecutive slots, switching key at each sub-row end
      if constexpr (KPL == 2) {
        const int b1 = lane_off + lens[0];
        const int e1 = min(lane_off + lsum, f0 + nf);
        const int src0 = kstart[0] - lane_off, src1 = kstart[1] - b1;
        for (int f = max(lane_off, f0); f < e1; ++f) {
          const bool second = f >= b1;
          sidx[f - f0] = (unsigned short)(lane * 2 + (second ? 1 : 0));
          cp_async8(stage + (f - f0), entries + (second ? src1 : src0) + f);
        }
      } else {
        int o = lane_off;
#pragma unroll
        for (int u = 0; u < KPL; ++u) {
          const int e0 = max(o, f0), e1 = min(o + lens[u], f0 + nf);
          for (int f = e0; f < e1; ++f) {
            sidx[f - f0] = (unsigned short)(lane * KPL + u);
            cp_async8(stage + (f - f0), entries + kstart[u] - o + f);
          }
          o += lens[u];
        }
      }
      cp_async_wait_all();
      __syncwarp();
      if (has_stdp) {
        bool any = false;
        for (int f = lane; f < nf; f += 32) {
          const uint2 en = stage[f];
          if ((en.x >> 28) != 0u) {
            cp_async4(stage_w + f, &csc[en.y].y);
            any = true;
          }
        }
        if (__any_sync(FULL, any)) cp_async_wait_all();
        __syncwarp();
      }
      for (int c0 = 0; c0 < nf; c0 += 32) {
        const int f = c0 + lane;
        bool add = false, inwin = false;
        int cell = 0, wslot = 0;
        float contrib = 0.0f;
        if (f < nf) {
          const int j = sidx[f];
          const uint32_t flv = kfl[j];
          const bool A = (flv >> 31) != 0;
          const bool P = ((flv >> 30) & 1u) != 0;
          const uint2 en = stage[f];
          const int q = (int)(en.x & 0xffffu);
          const int dl = (int)((en.x >> 16) & 0xffu);
          const int lb = (int)((en.x >> 24) & 0xfu);
          const int cl = (int)(en.x >> 28);
          if (cl != 0) {
            float v = stage_w[f];
            if (st.stdp_run) {
              const bool post_ev = ((spw_s[q >> 5] >> (q & 31)) & 1u) != 0;
              if (P || post_ev) {
                v = stdp_update(sc, v, P, post_ev, ptr_s[q], kpre[j]);
                csc[en.y].y = __float_as_uint(v);
                ++n_pre;
              }
            }
            contrib = v * scl_s[cl];
          } else {
            contrib = __uint_as_float(en.y);
          }
          if (A) {
            add = true;
            if (dl >= 1 && dl <= ws) {
              inwin = true;
              wslot = dl - 1;
              cell = (wslot * TS + q) * L + lb;
            } else {
              int sl = st.slot + dl;
              if (sl >= B) sl -= B;
              cell = (sl * TS + q) * L + lb;
            }
          }
        }
        // same-cell contributions of the chunk in lane order: the lowest lane
        // of each group adds its peers' contributions one by one.  Lanes
        // without a contribution share one key: the match instruction's cost
        // grows with the number of distinct keys it sees.
        const unsigned key = add ? (inwin ? (unsigned)cell : 0x40000000u | (unsigned)cell) : 0xffffffffu;
        const unsigned peers = __match_any_sync(FULL, key);
        const bool leader = add && (__ffs(peers) - 1) == lane;
        float acc = 0.0f;
        // the leader is its group's lowest lane: its own contribution comes
        // first, then its peers' in lane order
        if (leader) acc = (inwin ? win_s[cell] : ring[cell]) + contrib;
        unsigned rest = leader ? peers & (peers - 1u) : 0u;
        while (__any_sync(FULL, rest != 0u)) {
          const int src = rest ? __ffs(rest) - 1 : lane;
          const float cv = __shfl_sync(FULL, contrib, src);
          if (rest) {
            acc = acc + cv;
            rest &= rest - 1;
          }
        }
        if (leader) {
          if (inwin) {
            win_s[cell] = acc;
            dirty |= 1u << wslot;
          } else {
            ring[cell] = acc;
          }
        }
        __syncwarp();
      }
      __syncwarp();
    }
  }
  if (!active) return;
  dirty = __reduce_or_sync(FULL, dirty);
  if (dirty) {
    for (int k = 0; k < ws; ++k) {
      if (!((dirty >> k) & 1u)) continue;
      int sl = st.slot + 1 + k;
      if (sl >= B) sl -= B;
      float4* dst = (float4*)(ring + (size_t)sl * slot_words);
      const float4* src = (const float4*)(win_s + k * slot_words);
      for (int i = lane; i < slot_words / 4; i += 32) dst[i] = src[i];
    }
  }
  // the post-spike afferent pass runs in bulk_post_kernel, over all networks'
  // spiking posts at once
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    ev += __shfl_xor_sync(FULL, ev, o);
    n_pre += __shfl_xor_sync(FULL, n_pre, o);
  }
  if (lane == 0) {
    if (ev) atomicAdd(&d.ctl->events, ev);
    if (n_pre) atomicAdd(&d.ctl->stdp_pre, n_pre);
  }
}

// ---- timestep part 4: the post-spike afferent pass of every spiking post -----------------
// Each warp takes spiking posts of the shared item list in turn and gives the
// post's plastic afferents whose presynaptic key had no event this step (those
// with an event were updated in the propagation kernel) their LTP update,
// BULK_POST_CHUNK afferents per iteration.  Each weight is updated at most once
// per step, so the order of the items does not matter.
__global__ void __launch_bounds__(256) bulk_post_kernel(const NetDev* __restrict__ nets,
                                                        const BulkPostItem* __restrict__ items,
                                                        const int* __restrict__ item_count, int item_cap) {
  const int lane = threadIdx.x & 31;
  const int n_items = min(*item_count, item_cap);
  const int n_warps = gridDim.x * (blockDim.x >> 5);
  for (int it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); it < n_items; it += n_warps) {
    const BulkPostItem item = items[it];
    const NetDev& d = nets[item.net];
    const int a0 = __ldg(d.csc_ptr + item.post), a1 = __ldg(d.csc_ptr + item.post + 1);
    const float post_tr = d.post_trace[item.post];
    const uint32_t* bA = d.bitsA;
    const uint32_t* bP = d.bitsP;
    const float* pub = d.pre_pub;
    uint2* csc = d.csc;
    const StdpConst sc = stdp_const(d);
    unsigned long long n_post = 0;
    for (int a = a0; a < a1; a += BULK_POST_CHUNK) {
      constexpr int AFF = BULK_POST_CHUNK / 32;
      uint2 cc[AFF];
#pragma unroll
      for (int u = 0; u < AFF; ++u) {
        const int ai = a + u * 32 + lane;
        cc[u] = csc[ai < a1 ? ai : a];
      }
      uint32_t vm[AFF];
      float prt[AFF];
#pragma unroll
      for (int u = 0; u < AFF; ++u) {
        const int pk = (int)cc[u].x;
        vm[u] = bA[pk >> 5] | bP[pk >> 5];
        prt[u] = pub[pk];
      }
#pragma unroll
      for (int u = 0; u < AFF; ++u) {
        const int ai = a + u * 32 + lane;
        const int pk = (int)cc[u].x;
        if (ai >= a1 || ((vm[u] >> (pk & 31)) & 1u)) continue;
        const float nw = stdp_update(sc, __uint_as_float(cc[u].y), false, true, post_tr, prt[u]);
        csc[ai].y = __float_as_uint(nw);
        ++n_post;
      }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) n_post += __shfl_xor_sync(FULL, n_post, o);
    if (lane == 0 && n_post) atomicAdd(&d.ctl->stdp_post, n_post);
  }
}

// ---- timestep part 3b: per-synapse-trace STDP rules ---------------------------------------
// Every plastic synapse of the networks whose rule keeps two traces per
// synapse, every timestep, before this timestep's propagation: the traces
// decay, a presynaptic spike is seen when it arrives (the key's spike word of
// timestep T - delay in the history), a postsynaptic one at T, and the weight
// moves.  A warp per post; the records are the post's plastic afferents.
//   Evans (EvansSTDPPlasticity.cu:95-133): traces C, D; weights in [0, 1].
//   Inhibitory (InhibitorySTDPPlasticity.cu:102-143): Vogels' memory traces;
//   weights clipped at 0; its constant term in double, as the reference's
//   2.0 literal evaluates it.
//   Custom (CustomSTDPPlasticity.cu:100-142): pre and post memory traces,
//   optionally nearest-spike, weight-scaled depression; weights clipped at 0.
// One record's update under the network's rule, in the reference's order of
// float operations.
__device__ __forceinline__ void dense_rule_update(const NetDev& d, float dt, bool pre_sp, bool post_sp, float& w,
                                                  float2& tr) {
  const float c0 = d.rule_c[0], c1 = d.rule_c[1], c2 = d.rule_c[2], c3 = d.rule_c[3];
  if (d.stdp_rule == SPK_STDP_EVANS) {
    tr.x = (1.0f - (dt / c0)) * tr.x;
    tr.y = (1.0f - (dt / c1)) * tr.y;
    if (pre_sp) tr.x += dt * c2 * (1.0f - tr.x);
    if (post_sp) tr.y += dt * c3 * (1.0f - tr.y);
    float syn = 0.0f;
    const float old_w = w;
    if (pre_sp) syn -= (old_w * tr.y);
    if (post_sp) syn += ((1.0f - old_w) * tr.x);
    w = old_w + syn;
    if (w < 0.0f) w = 0.0f;
    if (w > 1.0f) w = 1.0f;
  } else if (d.stdp_rule == SPK_STDP_INHIBITORY) {
    tr.x *= c0;
    tr.y *= c0;
    if (pre_sp) tr.x += 1.0f;
    if (post_sp) tr.y += 1.0f;
    float syn = 0.0f;
    if (pre_sp) {
      syn += c1 * (tr.y);
      syn = (float)((double)syn + (double)(-c1) * (2.0 * (double)c2 * (double)c3));
    }
    if (post_sp) syn += c1 * (tr.x);
    w += syn;
    if (w < 0.0f) w = 0.0f;
  } else {
    const float a_plus = c2, a_minus = c3, lr = d.rule_c[4], a_star = d.rule_c[5], w_max = d.rule_c[6];
    const bool nearest = d.rule_c[7] != 0.0f;
    tr.y *= c0;
    tr.x *= c1;
    if (pre_sp) {
      tr.x += a_plus;
      if (nearest) tr.x = a_plus;
    }
    if (post_sp) {
      tr.y += a_minus;
      if (nearest) tr.y = a_minus;
    }
    float syn = 0.0f;
    const float old_w = w;
    if (pre_sp) syn -= lr * (old_w / w_max) * tr.y + lr * a_star;
    if (post_sp) syn += lr * tr.x;
    w = old_w + syn;
    if (w < 0.0f) w = 0.0f;
  }
}

// Records per lane in flight: the pass is bound by HBM latency as much as
// by bandwidth (a record's history word depends on its key and delay).  With
// four blocks of 256 threads per SM (64 registers) the kernel keeps 32 warps
// per SM; at 70 registers it had 24.
constexpr int DENSE_RECS = 4;

__global__ void __launch_bounds__(256, 4) bulk_dense_stdp_kernel(const NetDev* __restrict__ nets,
                                                              const BulkRuleItem* __restrict__ items, int n_items,
                                                              int s) {
  const int lane = threadIdx.x & 31;
  const int n_warps = gridDim.x * (blockDim.x >> 5);
  int cached = -1;  // the network whose step the warp holds (items come network by network)
  BulkStep st{};
  for (int it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); it < n_items; it += n_warps) {
    const BulkRuleItem item = items[it];
    const NetDev& d = nets[item.net];
    if (item.net != cached) {
      st = bulk_step(d, load_ctl(d.ctl), s);
      cached = item.net;
    }
    if (!st.live || !st.dense_run) continue;
    const int key = d.KL + item.post;
    // the post's spike bit of this step (bitsA also holds carried keys)
    const bool post_sp = ((d.gbits[(size_t)st.g * d.n_words + (key >> 5)] >> (key & 31)) & 1u) != 0;
    const int a0 = item.a0, a1 = item.a1;
    const float dt = d.dt;
    const int H = d.H, n_words = d.n_words;
    // (T - delay) mod H from T mod H: delays are 1..H-1, so one wrap at most
    const int t_mod = st.T % H;
    uint2* const csc = d.csc;
    const int* const cdl = d.csc_delay;
    float2* const dtr = d.dense_tr;
    const uint32_t* const hist = d.hist;
    for (int a = a0 + lane; a < a1; a += 32 * DENSE_RECS) {
      uint2 rec[DENSE_RECS];
      int dl[DENSE_RECS];
      float2 tr[DENSE_RECS];
#pragma unroll
      for (int u = 0; u < DENSE_RECS; ++u) {
        const int ai = a + 32 * u;
        if (ai < a1) {
          rec[u] = csc[ai];
          dl[u] = cdl[ai];
          tr[u] = dtr[ai];
        }
      }
      uint32_t hw[DENSE_RECS];
#pragma unroll
      for (int u = 0; u < DENSE_RECS; ++u) {
        const int ai = a + 32 * u;
        hw[u] = 0u;
        if (ai < a1) {
          int slot = t_mod - dl[u];
          if (slot < 0) slot += H;
          hw[u] = hist[(size_t)slot * n_words + (rec[u].x >> 5)];
        }
      }
#pragma unroll
      for (int u = 0; u < DENSE_RECS; ++u) {
        const int ai = a + 32 * u;
        if (ai < a1) {
          const bool pre_sp = ((hw[u] >> (rec[u].x & 31)) & 1u) != 0;
          float w = __uint_as_float(rec[u].y);
          dense_rule_update(d, dt, pre_sp, post_sp, w, tr[u]);
          csc[ai].y = __float_as_uint(w);
          dtr[ai] = tr[u];
        }
      }
    }
  }
}

// ---- timestep part 3c: weight normalisation -----------------------------------------------
// WeightNormSTDPPlasticity::weight_normalization (WeightNormSTDPPlasticity.cu:
// 74-176), in one warp per post: the change of the post's sum of squared
// plastic weights against their initial weights, (w - w0)^2 + 2 w0 (w - w0)
// over the afferents whose weight moved, the divisor sqrtf(S + change) /
// sqrtf(S), and the weights divided when it is not 1.  The reference adds the
// terms with atomicAdd, in no fixed order; here the order is fixed: lane j
// adds the terms of records j, j + 32, j + 64, ... (record = creation order)
// in turn, then the 32 partial sums meet in a pairwise tree (lane i with lane
// i + 16, then + 8, + 4, + 2, + 1), which every lane evaluates alike.
// `slot` picks the networks whose normalisation runs at this point of the
// timestep (0 before the rule, 1 after the per-synapse-trace pass, 2 after the
// event-driven rule's weight-update pass).
__device__ __forceinline__ int norm_slot_of(const NetDev& d) {
  if (d.weight_norm == SPK_NORM_BEFORE_RULE) return 0;
  return d.stdp_rule == SPK_STDP_WEIGHT_DEPENDENT ? 2 : 1;
}

__global__ void __launch_bounds__(256) bulk_norm_kernel(const NetDev* __restrict__ nets,
                                                        const BulkRuleItem* __restrict__ items, int n_items, int s,
                                                        int slot) {
  const int lane = threadIdx.x & 31;
  const int n_warps = gridDim.x * (blockDim.x >> 5);
  int cached = -1;  // the network whose step the warp holds (items come network by network)
  bool run = false;
  for (int it = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); it < n_items; it += n_warps) {
    const BulkRuleItem item = items[it];
    const NetDev& d = nets[item.net];
    if (item.net != cached) {
      run = false;
      if (d.weight_norm != SPK_NORM_OFF && d.has_stdp && norm_slot_of(d) == slot) {
        const RunCtl c = load_ctl(d.ctl);
        run = bulk_step(d, c, s).live && c.plastic;
      }
      cached = item.net;
    }
    if (!run) continue;
    const int a0 = item.a0, a1 = item.a1;
    const float* const w0s = d.norm_w0;
    const uint2* const csc = d.csc;
    float upd = 0.0f;
#pragma unroll 4
    for (int a = a0 + lane; a < a1; a += 32) {
      const float w0 = w0s[a];
      const float dw = __uint_as_float(csc[a].y) - w0;
      if (dw != 0.0f) upd += dw * dw + 2.0f * w0 * dw;
    }
    // lane i + o's partial joins lane i's (and, addition being commutative,
    // lane i's joins lane i + o's): all lanes end with the tree's sum
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) upd += __shfl_xor_sync(FULL, upd, o);
    const float sum = d.norm_sum[item.post];
    const float div = sqrtf(sum + upd) / sqrtf(sum);
    if (div != 1.0f)
      for (int a = a0 + lane; a < a1; a += 32) d.csc[a].y = __float_as_uint(__uint_as_float(d.csc[a].y) / div);
  }
}

// ---- after a block: the networks' run counters -------------------------------------------
__global__ void bulk_finish_kernel(const NetDev* __restrict__ nets, int n_nets, int K) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nets) return;
  RunCtl* c = nets[i].ctl;
  const int done = max(0, min(K, c->steps_total - c->step));
  c->step += done;
  c->gstep += done;
  if (done > 0) c->inputs_active = 1;
}

}  // namespace spk
