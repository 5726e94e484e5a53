// spk_kernel.cuh - the persistent step kernel.
//
// One launch advances every network of its CTA map by up to K timesteps.
// A network is cut into n_tiles post tiles; warp w of CTA rank r owns tile
// t = r*W + w: its neurons' V / last-spike / synaptic traces, its slice of the
// delay ring buffer and a share of the Poisson inputs all live in the warp's
// shared-memory region for the whole launch.  Per timestep:
//
//   phase A  each warp updates its own neurons (LIF + injection, reference
//            Spike/Backend/CUDA/Neurons/LIFSpikingNeurons.cu:105-193 with
//            Spike/Backend/CUDA/InlineDeviceFunctions.hpp:22-111) and inputs
//            (Spike/Backend/CUDA/Neurons/PoissonInputSpikingNeurons.cu:96-129),
//            advances the per-neuron STDP traces and ballots its spike words;
//            warp 0 then publishes the CTA's active keys (inputs, then
//            neurons, each ascending), every word stamped with its step, and
//            one stamp word with their counts (replaces the atomic activation
//            list of InlineDeviceFunctions.hpp:4-18);
//   phase B  warp 0 polls the stamps of all the network's CTAs (the only
//            inter-CTA synchronization, bounded by a wall-clock limit) and
//            gathers the step's keys in ascending order into rounds of a
//            shared list; each warp stages the round's (key, tile) sub-rows of
//            the row-partitioned CSR (8 B per synapse) into shared memory with
//            cp.async and adds w*scale into its own ring cells (reference
//            activate_synapses, Spike/Backend/CUDA/Synapses/SpikingSynapses.cu:
//            168-202), after updating plastic weights of rows with a pre event
//            (WeightDependentSTDPPlasticity.cu:85-161); last, the CTA's warps
//            share the plastic afferents of its spiking posts whose
//            presynaptic key had no event (the post-spike pass).
//
// Every ring cell has exactly one writer (the tile's warp) which applies the
// contributions of a step in canonical order (ascending key, then synapse
// order), so the result is deterministic and atomic-free.  Phase A of the next
// step reads only the warp's own cells.
#pragma once

#include <cuda_runtime.h>

#include "../../include/spike_gb300.h"
#include "spk_internal.h"

namespace spk {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ int ld_volatile(const int* p) { return *(volatile const int*)p; }
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
// Bulk prefetch of a byte range into L2 (the TMA engine's L2 prefetch); the
// range is widened to 16-byte boundaries.
__device__ __forceinline__ void prefetch_l2(const void* p, size_t bytes) {
  const uintptr_t a = (uintptr_t)p & ~(uintptr_t)15;
  const uintptr_t e = ((uintptr_t)p + bytes + 15) & ~(uintptr_t)15;
  for (uintptr_t c = a; c < e; c += (1u << 20)) {
    const unsigned n = (unsigned)min((uintptr_t)(1u << 20), e - c);
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(c), "r"(n) : "memory");
  }
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
// Barrier 1 over the whole CTA: releases and retires list rounds between warp 0
// (the list builder) and the other warps, which reach it from different code.
__device__ __forceinline__ void round_barrier(int nthreads) {
  asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Re-read a stamped word until it carries `stamp`; bounded by the poll timeout
// and the launch's abort flag (ok turns false, the status records a timeout).
__device__ __forceinline__ unsigned long long repoll(const unsigned long long* p, unsigned long long v,
                                                     unsigned stamp, const NetDev& d, bool& ok) {
  unsigned long long t0 = 0ull;
  while (ok && (unsigned)(v >> 32) != stamp) {
    const unsigned long long now = globaltimer();
    if (t0 == 0ull) t0 = now;
    if (ld_volatile(d.abort_flag)) {
      ok = false;
    } else if (now - t0 > d.poll_ns) {
      atomicExch(d.abort_flag, 1);
      atomicCAS(&d.ctl->status, 0, SPK_ERR_TIMEOUT);
      ok = false;
    } else {
      v = ld_relaxed_u64(p);
    }
  }
  return v;
}

// ltp_and_ltd update of one synapse for G = 1
// (Spike/Backend/CUDA/Plasticity/WeightDependentSTDPPlasticity.cu:132-151):
// pre_ev/post_ev are "spike sub-step >= 0", the traces are this step's values.
// The STDP constants of a network, for loops that keep them in registers.
struct StdpConst {
  float invE_m, invE_p, lam, lam_alpha, wmax;
  int clip_upper;
};
__device__ __forceinline__ StdpConst stdp_const(const NetDev& d) {
  return StdpConst{d.invE_m, d.invE_p, d.lam, d.lam_alpha, d.wmax, d.clip_upper};
}
template <class C>
__device__ __forceinline__ float stdp_update(const C& d, float old_w, bool pre_ev, bool post_ev,
                                             float post_tr, float pre_tr) {
  float syn = 0.0f;
  if (pre_ev) {
    float temp_post = post_tr * d.invE_m;
    syn = syn - d.lam_alpha * old_w * temp_post;
  }
  if (post_ev) {
    float temp_pre = pre_tr * d.invE_p;
    syn = syn + d.lam * (d.wmax - old_w) * temp_pre;
  }
  float nw = old_w + syn;
  if (nw < 0.0f) nw = 0.0f;
  if (d.clip_upper && nw > d.wmax) nw = d.wmax;
  return nw;
}

__global__ void __launch_bounds__(512, 1)
    step_kernel(const NetDev* __restrict__ nets, const CtaMap* __restrict__ map, int K) {
  extern __shared__ __align__(16) uint32_t sm[];
  __shared__ float s_decay[MAX_LABELS + 1], s_vhat[MAX_LABELS + 1], s_scale[MAX_CLASSES];
  __shared__ int s_round[4];  // keys in the round, last round, poll ok
  __shared__ int s_nsp;       // spiking posts listed for the CTA's afferent pass
  __shared__ __align__(16) NetDev s_net;
  const CtaMap cm = map[blockIdx.x];
  // The network's descriptor in shared memory: the asm memory clobbers of the
  // staging copies would otherwise reload its fields from global memory in
  // every loop.
  {
    const uint32_t* src = (const uint32_t*)(nets + cm.net);
    uint32_t* dst = (uint32_t*)&s_net;
    for (int i = threadIdx.x; i < (int)(sizeof(NetDev) / 4); i += blockDim.x) dst[i] = __ldg(src + i);
  }
  __syncthreads();
  const NetDev& d = s_net;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x < MAX_LABELS + 1) {
    s_decay[threadIdx.x] = d.decay[threadIdx.x];
    s_vhat[threadIdx.x] = d.vhat[threadIdx.x];
  }
  if (threadIdx.x < MAX_CLASSES) s_scale[threadIdx.x] = d.scale_tab[threadIdx.x];
  __syncthreads();
  const int W = d.W;
  const int N = d.N, Nin = d.Nin, KL = d.KL, L = d.L, B = d.B, kind = d.kind;
  const int TS = d.TS, ITS = d.ITS, n_tiles = d.n_tiles, n_keys = d.n_keys, n_words = d.n_words;
  const float dt = d.dt;
  int* const rate_counts = d.rate_counts;  // rate monitor (one owner per key and step)

  uint32_t* list = sm;
  int* segoff = (int*)(sm + LIST_CAP);  // [2 * nctas + 1] offsets of the gather segments
  const WarpLayout wl = warp_layout(B, TS, L, ITS, kind, d.has_stdp);
  uint32_t* wreg = sm + SHARED_WORDS + w * wl.total;
  uint2* stage = (uint2*)(wreg + wl.stage);
  float* stage_w = (float*)(wreg + wl.stw);
  unsigned short* sidx = (unsigned short*)(wreg + wl.sidx);
  int* kst = (int*)(wreg + wl.kst);
  int* koff = (int*)(wreg + wl.koff);
  uint32_t* kfl = wreg + wl.kfl;
  float* kpre = (float*)(wreg + wl.kpre);
  int* tag_s = (int*)(wreg + wl.tag);
  int* rowb_s = (int*)(wreg + wl.rowb);
  int* rowe_s = (int*)(wreg + wl.rowe);
  float* ring_s = (float*)(wreg + wl.ring);
  float* V_s = (float*)(wreg + wl.V);
  float* last_s = (float*)(wreg + wl.last);
  float* gtr_s = (float*)(wreg + wl.gtr);
  float* post_s = (float*)(wreg + wl.post_tr);
  float* pre_s = (float*)(wreg + wl.pre_tr);
  uint32_t* spkw_s = wreg + wl.spkw;
  uint32_t* evw_s = wreg + wl.evw;
  uint32_t* pvw_s = wreg + wl.pvw;
  uint32_t* fw_s = wreg + wl.fw;
  uint32_t* inw_s = wreg + wl.inw;
  uint32_t* inwp_s = wreg + wl.inwp;
  float* innext_s = (float*)(wreg + wl.in_next);
  float* inrate_s = (float*)(wreg + wl.in_rate);
  float* inpre_s = (float*)(wreg + wl.in_pre);

  const RunCtl ctl0 = *d.ctl;
  const int steps_here = min(K, ctl0.steps_total - ctl0.step);
  if (steps_here <= 0) return;
  const bool stdp_run = d.has_stdp && ctl0.plastic;
  const bool recorder = cm.rank == 0 && w == W - 1 && d.spike_cap > 0;  // off warp 0's path

  const int t_idx = cm.rank * W + w;  // tile owned by this warp
  const int p0 = t_idx * TS;          // first post of the tile
  const int kin0 = t_idx * ITS;       // first input key of the tile

  // Group constants: uniform over the tile unless the tile straddles groups.
  int g_first = 0, g_last = 0;
  {
    const int n_hi = min(p0 + TS, N) - 1;
    while (g_first + 1 < d.n_groups && p0 >= d.groups[g_first].end) ++g_first;
    g_last = g_first;
    while (g_last + 1 < d.n_groups && n_hi >= d.groups[g_last].end) ++g_last;
  }
  const GroupConst G0 = d.groups[g_first];
  const float t_ref = d.t_ref, i_bg = d.i_bg;

  // ---- load the tile's state into shared memory -------------------------------
  {
    const float* rh = d.ring + (size_t)t_idx * B * TS * L;
    const int nr = B * TS * L;
    for (int i = lane; i < nr; i += 32) ring_s[i] = rh[i];
    for (int i = lane; i < TS; i += 32) {
      const int n = p0 + i;
      const bool ok = n < N;
      V_s[i] = ok ? d.V[n] : 0.0f;
      last_s[i] = ok ? d.last[n] : 0.0f;
      if (d.has_stdp) {
        post_s[i] = ok ? d.post_trace[n] : 0.0f;
        pre_s[i] = ok ? d.pre_trace[KL + n] : 0.0f;
      }
    }
    if (kind != SPK_SYN_VOLTAGE)
      for (int i = lane; i < TS * L; i += 32) {
        const int n = p0 + i / L;
        gtr_s[i] = n < N ? d.gtr[(size_t)p0 * L + i] : 0.0f;
      }
    for (int i = lane; i < ITS; i += 32) {
      const int k = kin0 + i;
      const bool ok = k < Nin;
      const int idx = Nin - 1 - k;
      innext_s[i] = ok ? d.in_next[idx] : 0.0f;
      inrate_s[i] = ok ? d.rates[idx] : 0.0f;
      if (d.has_stdp) inpre_s[i] = ok ? d.pre_trace[k] : 0.0f;
    }
  }
  for (int i = lane; i < APPLY_TAGS; i += 32) tag_s[i] = 32;
  for (int i = lane; i < TS + ITS; i += 32) {
    const int key = i < TS ? KL + p0 + i : kin0 + (i - TS);
    rowb_s[i] = __ldg(d.rowptr + (size_t)key * n_tiles);
    rowe_s[i] = __ldg(d.rowptr + (size_t)(key + 1) * n_tiles);
  }
  unsigned long long spike_count = ctl0.spike_count;
  unsigned long long ev = 0, n_pre = 0, n_post = 0;  // events, STDP pre updates, STDP post afferents
  bool inputs_active = ctl0.inputs_active != 0;
  int steps_done = 0;
  bool ok_run = true;
  __syncwarp();

  // index of the group before the one of the launch's first timestep, and of
  // the last timestep's group
  const int G = d.G;
  int k_prev = ctl0.step >= G ? group_index(ctl0.start_time, ctl0.step - G, G, dt) : 0;
  int k_last = 0;
  bool fw_dirty = true;  // the carried words in shared memory are not known to be zero
  // this lane's word of the warp's group spike words (neurons, then inputs), if any
  const int gw_n = (TS + ITS) >> 5;
  uint32_t* const gw = lane < gw_n ? d.gbits + (lane < (TS >> 5) ? ((KL + p0) >> 5) + lane
                                                                 : (kin0 >> 5) + (lane - (TS >> 5)))
                                   : nullptr;
  for (int s = 0; s < steps_here && ok_run; ++s) {
    const int sr = ctl0.step + s;
    float t, tg;
    int T;
    group_time(ctl0.start_time, sr, d.G, dt, t, T, tg);
    const int g_sub = G == 1 ? 0 : sr % G;  // substep of the group
    // A group with the parity of the group step before it (index k_prev,
    // carried from step to step) delivers that group's spikes again (carried
    // keys), in each substep's propagation after its STDP updates, as
    // activate_synapses follows the rules.  A carried list of two earlier
    // groups is beyond this engine: status.
    const int k = G == 1 ? T : (T - g_sub) / G;
    if (g_sub == 0 && s > 0) k_prev = k_last;
    const bool rep = sr < G ? ctl0.repeat != 0 : ((k ^ k_prev) & 1) == 0;
    k_last = k;
    if (rep && sr >= G && g_sub == 0 && threadIdx.x == 0 && cm.rank == 0 &&
        group_repeats(ctl0, sr - G, k_prev, G, dt))
      atomicCAS(&d.ctl->status, 0, SPK_ERR_UNSUPPORTED);
    const long long gs = ctl0.gstep + s;
    const int par = (int)(gs & 1);
    const unsigned stamp = (unsigned)(gs + 1);
    const unsigned long long stamp_hi = (unsigned long long)stamp << 32;
    uint32_t* bitsA = d.bitsA + (size_t)par * n_words;
    uint32_t* bitsP = d.bitsP + (size_t)par * n_words;
    float* pub = d.pre_pub + (size_t)par * n_keys;
    const int slot = T % B;
    const float half_dt = 0.5f * dt;

    // ---- phase A: LIF neurons of the tile ------------------------------------
    {
      float* ring_slot = ring_s + (size_t)slot * TS * L;
      for (int base = 0; base < TS; base += 32) {
        const int li = base + lane;
        const int n = p0 + li;
        bool spk = false, ev = false, pe = false;
        if (n < N) {
          GroupConst G = G0;
          if (g_last != g_first) {
            int gi = g_first;
            while (gi < g_last && n >= d.groups[gi].end) ++gi;
            G = d.groups[gi];
          }
          float Vi = V_s[li];
          float input;
          if (kind == SPK_SYN_CONDUCTANCE) {
            float total = 0.0f;
            for (int l = 0; l < L; ++l) {
              const float cell = ring_slot[li * L + l];
              ring_slot[li * L + l] = 0.0f;
              const float gnew = s_decay[l] * gtr_s[li * L + l] + cell;
              total = total + gnew * (s_vhat[l] - Vi);
              gtr_s[li * L + l] = gnew;
            }
            input = total * G.kR;
          } else if (kind == SPK_SYN_CURRENT) {
            float total = 0.0f;
            for (int l = 0; l < L; ++l) {
              const float cell = ring_slot[li * L + l];
              ring_slot[li * L + l] = 0.0f;
              float inew = gtr_s[li * L + l] * s_decay[l];
              inew = inew + cell;
              total = total + inew;
              gtr_s[li * L + l] = inew;
            }
            input = total * G.kR;
          } else {
            float total = 0.0f;
            for (int l = 0; l < L; ++l) {
              total = total + ring_slot[li * L + l];
              ring_slot[li * L + l] = 0.0f;
            }
            input = total;
          }
          if (((tg - last_s[li]) - t_ref) > half_dt) {
            Vi = G.k * G.v0 + (1.0f - G.k) * Vi + G.k * i_bg + input;
            if (Vi >= G.theta) {
              spk = true;
              last_s[li] = tg;
              Vi = G.vreset;
              if (rate_counts) rate_counts[KL + n] += 1;
            }
          }
          V_s[li] = Vi;
          if (stdp_run) {
            // g = roundf((last - t)/dt)
            // (Spike/Backend/CUDA/Plasticity/WeightDependentSTDPPlasticity.cu:113-117):
            // an event as the postsynaptic neuron for g >= 0, as the
            // presynaptic one for 0 <= g < G (g >= G is negated).  That is
            // this step's spike, or the last step's where the timestep index
            // repeats, or (post only) a spike later than the clock after
            // reset_time.  A spike older than a step cannot
            // round to 0: no division then.
            const float lag = last_s[li] - t;
            const int gq = (spk || lag < -dt) ? (spk ? 0 : -1) : (int)roundf(lag / dt);
            ev = gq >= 0;
            pe = gq == 0;
            float po = post_s[li] * d.E_m;
            po = po + (ev ? d.inc_m : 0.0f);
            post_s[li] = po;
            float pr = pre_s[li] * d.E_p;
            pr = pr + (pe ? d.inc_p : 0.0f);
            pre_s[li] = pr;
            pub[KL + n] = pr;
          }
        }
        const unsigned word = __ballot_sync(FULL, spk);
        const unsigned evword = stdp_run ? __ballot_sync(FULL, ev) : 0u;
        const unsigned peword = stdp_run ? __ballot_sync(FULL, pe) : 0u;
        if (lane == 0) {
          spkw_s[base >> 5] = word;
          if (stdp_run) {
            evw_s[base >> 5] = evword;
            pvw_s[base >> 5] = peword;
          }
        }
      }
    }
    // ---- phase A: Poisson inputs of the tile ----------------------------------
    for (int base = 0; base < ITS; base += 32) {
      const int li = base + lane;
      const int k = kin0 + li;
      bool spk = false, pev = false;
      if (k < Nin) {
        const int idx = Nin - 1 - k;
        float nx = innext_s[li];
        if ((nx <= tg) || !inputs_active) {
          const float rate = inrate_s[li];
          const float u = draw_uniform(d.seed, (uint32_t)idx, (uint32_t)T, DOMAIN_POISSON);
          nx = tg - (1.0f / rate) * logf_spk(u);
          if (inputs_active) {
            spk = true;
            if (rate_counts) rate_counts[k] += 1;
          }
        }
        innext_s[li] = nx;
        if (stdp_run) {
          int pg = (int)roundf((nx - t) / dt);
          if (pg >= 1) pg *= -1;
          pev = pg >= 0;
          float pr = inpre_s[li] * d.E_p;
          pr = pr + (pev ? d.inc_p : 0.0f);
          inpre_s[li] = pr;
          pub[k] = pr;
        }
      }
      const unsigned wa = __ballot_sync(FULL, spk);
      const unsigned wp = __ballot_sync(FULL, pev);
      if (lane == 0) {
        inw_s[base >> 5] = wa;
        inwp_s[base >> 5] = wp;
      }
    }
    inputs_active = true;

    // ---- prefetch: every CTA of the network reads the row pointers and the
    // synapse row of this warp's spiking keys this step; pull them into L2
    // now, while the keys travel (bulk prefetches, no dependent loads)
    {
      const int nl = TS >> 5, ni = ITS >> 5;
      for (int i = 0; i < nl + ni; ++i) {
        const uint32_t m = i < nl ? (spkw_s[i] | (stdp_run ? pvw_s[i] : 0u))
                                  : (inw_s[i - nl] | (stdp_run ? inwp_s[i - nl] : 0u));
        if (!((m >> lane) & 1u)) continue;
        const int li = i < nl ? 32 * i + lane : TS + 32 * (i - nl) + lane;
        const int key = i < nl ? KL + p0 + li : kin0 + (li - TS);
        prefetch_l2(d.rowptr + (size_t)key * n_tiles, sizeof(int) * (size_t)(n_tiles + 1));
        if (rowe_s[li] > rowb_s[li])
          prefetch_l2(d.entries + rowb_s[li], sizeof(uint2) * (size_t)(rowe_s[li] - rowb_s[li]));
      }
    }

    // ---- publish: the CTA's active keys, then one stamp word per CTA ---------
    __syncwarp();
    {
      // This substep's spike words are kept for a later group of the same
      // index parity; in such a repeating group (rep) the last group's words
      // are the carried keys delivered again in this substep.
      const int nl = TS >> 5, ni = ITS >> 5;
      if (gw_n <= 32) {
        // one word per lane (the common case): pointer set up once per launch;
        // the new words are stored after the CTA's stamp (below), so that the
        // stamp does not queue behind them
        if (gw && (rep || fw_dirty)) fw_s[lane] = rep ? gw[(size_t)g_sub * n_words] : 0u;
      } else {
        uint32_t* gb = d.gbits + (size_t)g_sub * n_words;
        for (int i = lane; i < nl + ni; i += 32) {
          const int wi = i < nl ? ((KL + p0) >> 5) + i : (kin0 >> 5) + (i - nl);
          if (rep || fw_dirty) fw_s[i] = rep ? gb[wi] : 0u;
          gb[wi] = i < nl ? spkw_s[i] : inw_s[i - nl];
        }
      }
      fw_dirty = rep;
    }
    // (each lane reads back only the carried words it wrote)
    if (stdp_run) {
      // bitmaps for the post-spike pass, which looks up arbitrary pre keys:
      // delivered keys (A) and STDP events (P)
      const int nl = TS >> 5, ni = ITS >> 5;
      for (int i = lane; i < nl + ni; i += 32) {
        if (i < nl) {
          const int wi = ((KL + p0) >> 5) + i;
          bitsA[wi] = spkw_s[i] | fw_s[i];
          bitsP[wi] = pvw_s[i];
        } else {
          const int wi = (kin0 >> 5) + (i - nl);
          bitsA[wi] = inw_s[i - nl] | fw_s[i];
          bitsP[wi] = inwp_s[i - nl];
        }
      }
    }
    __syncthreads();  // every warp's words are in shared memory, its traces written
    if (threadIdx.x == 0) s_nsp = 0;  // read by every thread in the previous step's afferent pass
    // The CTA's ballot words in key order: inputs of warps 0..W-1, then neurons
    // of warps 0..W-1 (x-th word: bits a = delivered keys, p = STDP pre
    // events, sp = spikes of the step, first key).  a is sp but in a group
    // that repeats the last group step's index parity, where the carried keys
    // are delivered again.
    const int nw_in = W * (ITS >> 5), nw_all = W * ((ITS >> 5) + (TS >> 5));
    // A key both carried and spiking is listed (and delivered) once.
    auto cta_word = [&](const int x, uint32_t& a, uint32_t& p, uint32_t& sp, uint32_t& wkey) {
      const int ni = ITS >> 5, nl = TS >> 5;
      a = 0u;
      p = 0u;
      sp = 0u;
      wkey = 0u;
      uint32_t f = 0u;
      if (x < nw_in) {
        const int wx = x / ni, k = x - (x / ni) * ni;
        const uint32_t* r = sm + SHARED_WORDS + wx * wl.total;
        sp = r[wl.inw + k];
        f = r[wl.fw + nl + k];
        p = stdp_run ? r[wl.inwp + k] : 0u;
        wkey = (uint32_t)((cm.rank * W + wx) * ITS + k * 32);
      } else if (x < nw_all) {
        const int y = x - nw_in;
        const int wx = y / nl, k = y - (y / nl) * nl;
        const uint32_t* r = sm + SHARED_WORDS + wx * wl.total;
        sp = r[wl.spkw + k];
        f = r[wl.fw + k];
        p = stdp_run ? r[wl.pvw + k] : 0u;
        wkey = (uint32_t)(KL + (cm.rank * W + wx) * TS + k * 32);
      }
      a = sp | f;
    };
    if (w == 0 && d.nctas > 1) {
      unsigned long long* keys_out = d.cta_keys + ((size_t)par * d.nctas + cm.rank) * d.key_cap;
      int pos = 0, n_in = 0;
      for (int x0 = 0; x0 < nw_all; x0 += 32) {
        const int x = x0 + lane;
        uint32_t a, p, sp, wkey;
        cta_word(x, a, p, sp, wkey);
        uint32_t m = a | p;
        const int c = __popc(m);
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(FULL, incl, o);
          if (lane >= o) incl += y;
        }
        int o = pos + incl - c;
        while (m) {
          const int b = __ffs(m) - 1;
          m &= m - 1;
          st_relaxed_u64(keys_out + o++, stamp_hi | (wkey + b) | (((a >> b) & 1u) << 31) | (((p >> b) & 1u) << 30) |
                                             (((sp >> b) & 1u) << 29));
        }
        n_in += __reduce_add_sync(FULL, x < nw_in ? c : 0);
        pos += __shfl_sync(FULL, incl, 31);
      }
      // The key words carry their step, so without plasticity nothing else has
      // to be ordered before the stamp.  With plasticity the other warps'
      // traces and bitmap words (through the CTA barrier) must be: one fence.
      if (stdp_run) fence_acq_rel_gpu();
      __syncwarp();
      if (lane == 0)
        st_relaxed_u64(d.cta_stamp + (size_t)par * d.nctas + cm.rank,
                       stamp_hi | ((unsigned long long)n_in << 16) | (unsigned long long)(pos - n_in));
    }
    // this substep's spike words for a later repeating group (one word per lane)
    if (gw_n <= 32 && gw) {
      const int nl = TS >> 5;
      gw[(size_t)g_sub * n_words] = lane < nl ? spkw_s[lane] : inw_s[lane - nl];
    }

    // ---- phase B: warp 0 gathers the step's active keys from every CTA ------
    // It polls the stamps of all the network's CTAs (all pending loads in
    // flight at once, bounded by a timeout), gathers their keys in ascending
    // order (inputs of CTA 0..C-1, then neurons of CTA 0..C-1) into the list
    // in rounds of at most LIST_CAP keys, records spikes (rank 0), and
    // releases each round to the CTA's other warps through a named barrier.
    // Every warp then stages and applies its tile's part of the round.
    auto process_round = [&](const int n_round) {
      if (recorder) {
            // spike store in canonical order: neurons, and inputs on request
            for (int c0 = 0; c0 < n_round; c0 += 32) {
              const int j = c0 + lane;
              bool rec = false;
              uint32_t key = 0u;
              if (j < n_round) {
                const uint32_t lv = list[j];
                key = lv & 0x1fffffffu;
                rec = ((lv >> 29) & 1u) && ((int)key >= KL || ctl0.record_inputs);
              }
              const unsigned m = __ballot_sync(FULL, rec);
              if (rec) {
                const unsigned long long sp = spike_count + (unsigned long long)__popc(m & lanemask_lt());
                if (sp < (unsigned long long)d.spike_cap)
                  d.spikes[sp] = make_uint2(key, __float_as_uint(tg));
                else
                  atomicCAS(&d.ctl->status, 0, SPK_ERR_OVERFLOW);
              }
              spike_count += (unsigned long long)__popc(m);
            }
            if (spike_count > (unsigned long long)d.spike_cap) spike_count = d.spike_cap;
          }
        for (int kb = 0; kb < n_round; kb += STAGE_KEYS) {
          const int nk = min(STAGE_KEYS, n_round - kb);
          // row pointers of the round's keys straight into shared memory
          // (cp.async: every load of the round in flight at once)
          for (int i = lane; i < nk; i += 32) {
            const uint32_t lv = list[kb + i];
            const int* rp = d.rowptr + (size_t)(lv & 0x1fffffffu) * n_tiles + t_idx;
            cp_async4(kst + i, rp);
            cp_async4(koff + i, rp + 1);
            kfl[i] = lv;
          }
          if (stdp_run) {
            // this step's presynaptic traces, written by other CTAs: L2 loads
            constexpr int KPL = STAGE_KEYS / 32;
            float prs[KPL];
#pragma unroll
            for (int u = 0; u < KPL; ++u) {
              const int i = u * 32 + lane;
              prs[u] = i < nk ? __ldcg(pub + (list[kb + i] & 0x1fffffffu)) : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < KPL; ++u) {
              const int i = u * 32 + lane;
              if (i < nk) kpre[i] = prs[u];
            }
          }
          cp_async_wait_all();
          __syncwarp();
          // the sub-row lengths and their exclusive prefix: each lane takes
          // KPL consecutive keys, one warp scan for the round
          constexpr int KPL = STAGE_KEYS / 32;
          int lens[KPL], kstart[KPL];
          int lsum = 0;
#pragma unroll
          for (int u = 0; u < KPL; ++u) {
            const int i = lane * KPL + u;
            int len = 0;
            kstart[u] = 0;
            if (i < nk) {
              kstart[u] = kst[i];
              len = koff[i] - kstart[u];
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
          __syncwarp();
          for (int f0 = 0; f0 < total_e; f0 += STAGE_ENTRIES) {
            const int nf = min(STAGE_ENTRIES, total_e - f0);
            // each lane copies the part of its keys' sub-rows that falls in
            // this stage [f0, f0 + nf), from registers (no search per entry)
            int o = lane_off;
#pragma unroll
            for (int u = 0; u < KPL; ++u) {
              const int e0 = max(o, f0), e1 = min(o + lens[u], f0 + nf);
              for (int f = e0; f < e1; ++f) {
                sidx[f - f0] = (unsigned short)(lane * KPL + u);
                cp_async8(stage + (f - f0), d.entries + kstart[u] - o + f);
              }
              o += lens[u];
            }
            cp_async_wait_all();
            __syncwarp();
            if (d.has_stdp) {
              // weights of the window's plastic entries, from their CSC records
              bool any = false;
              for (int f = lane; f < nf; f += 32) {
                const uint2 en = stage[f];
                if ((en.x >> 28) != 0u) {
                  cp_async4(stage_w + f, &d.csc[en.y].y);
                  any = true;
                }
              }
              if (__any_sync(FULL, any)) cp_async_wait_all();
              __syncwarp();
            }
            for (int c0 = 0; c0 < nf; c0 += 32) {
              const int f = c0 + lane;
              bool add = false;
              int cell = -1 - lane;
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
                const int c = (int)(en.x >> 28);
                if (c != 0) {
                  float v = stage_w[f];
                  if (stdp_run) {
                    const bool post_ev = ((evw_s[q >> 5] >> (q & 31)) & 1u) != 0;
                    if (P || post_ev) {
                      v = stdp_update(d, v, P, post_ev, post_s[q], kpre[j]);
                      d.csc[en.y].y = __float_as_uint(v);
                      ++n_pre;
                    }
                  }
                  contrib = v * s_scale[c];
                } else {
                  contrib = __uint_as_float(en.y);
                }
                if (A) {
                  add = true;
                  int sl = slot + dl;
                  if (sl >= B) sl -= B;
                  cell = (sl * TS + q) * L + lb;
                }
              }
              // Apply in lane order within a chunk, chunks in program order.
              // Each pass, the lowest pending lane of every cell hash (an
              // atomicMin on a shared tag) adds its contribution; lanes that
              // share a hash are thereby serialized in lane order, which keeps
              // same-cell additions in canonical order.
              bool pending = add;
              const int h = cell & (APPLY_TAGS - 1);
              while (__any_sync(FULL, pending)) {
                if (pending) atomicMin(tag_s + h, lane);
                __syncwarp();
                const bool win = pending && tag_s[h] == lane;
                if (win) ring_s[cell] = ring_s[cell] + contrib;
                __syncwarp();
                if (win) {
                  tag_s[h] = 32;
                  pending = false;
                }
                __syncwarp();
              }
            }
            __syncwarp();
          }
        }
    };
    const int nthreads = blockDim.x;
    if (w == 0 && d.nctas == 1) {
      // One CTA holds the whole network: the list comes straight from the
      // warps' ballot words in shared memory, with no global exchange.
      int list_n = 0;
      for (int x0 = 0; x0 < nw_all; x0 += 32) {
        uint32_t a, p, sp, wkey;
        cta_word(x0 + lane, a, p, sp, wkey);
        uint32_t m = a | p;
        const int c = __popc(m);
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(FULL, incl, o);
          if (lane >= o) incl += y;
        }
        const int tot = __shfl_sync(FULL, incl, 31);
        if (tot == 0) continue;
        if (list_n + tot > LIST_CAP) {
          if (lane == 0) {
            s_round[0] = list_n;
            s_round[1] = 0;
            s_round[2] = 1;
          }
          round_barrier(nthreads);
          process_round(list_n);
          round_barrier(nthreads);
          list_n = 0;
        }
        int o = list_n + incl - c;
        while (m) {
          const int b = __ffs(m) - 1;
          m &= m - 1;
          list[o++] = (wkey + b) | (((a >> b) & 1u) << 31) | (((p >> b) & 1u) << 30) | (((sp >> b) & 1u) << 29);
        }
        list_n += tot;
      }
      if (lane == 0) {
        s_round[0] = list_n;
        s_round[1] = 1;
        s_round[2] = 1;
      }
      round_barrier(nthreads);
      process_round(list_n);
    } else if (w == 0) {
      // Without plasticity only the key words are read from the other CTAs,
      // each carrying its step (a stale word is polled again).  They are read
      // through L1, whose lines of this buffer may be two steps old: the fence
      // drops them, here, while the other CTAs publish, rather than after the
      // last stamp arrives.
      if (!stdp_run) fence_acq_rel_gpu();
      const int C = d.nctas;
      const unsigned long long* stp = d.cta_stamp + (size_t)par * C;
      constexpr int SPL = MAX_CTAS_PER_NET / 32;
      unsigned long long sv[SPL];
      bool ok = true;
#pragma unroll
      for (int u = 0; u < SPL; ++u) {
        const int r = u * 32 + lane;
        sv[u] = r < C ? ld_relaxed_u64(stp + r) : stamp_hi;
      }
      unsigned long long t0 = 0ull;
      while (true) {
        bool pending = false;
#pragma unroll
        for (int u = 0; u < SPL; ++u) pending |= (unsigned)(sv[u] >> 32) != stamp;
        if (!__any_sync(FULL, pending)) break;
        const unsigned long long now = globaltimer();
        if (t0 == 0ull) t0 = now;
        if (now - t0 > d.poll_ns || ld_volatile(d.abort_flag)) {
          if (lane == 0 && now - t0 > d.poll_ns) {
            atomicExch(d.abort_flag, 1);
            atomicCAS(&d.ctl->status, 0, SPK_ERR_TIMEOUT);
          }
          ok = false;
          break;
        }
        __nanosleep(32);
#pragma unroll
        for (int u = 0; u < SPL; ++u) {
          const int r = u * 32 + lane;
          if (r < C && (unsigned)(sv[u] >> 32) != stamp) sv[u] = ld_relaxed_u64(stp + r);
        }
      }
      int total = 0;
      if (ok) {
        // With plasticity the traces and bitmaps published before the stamps
        // are read next: acquire them (the fence also drops stale L1 lines of
        // the key words, read next through L1).
        if (stdp_run) fence_acq_rel_gpu();
#pragma unroll
        for (int u = 0; u < SPL; ++u) {
          const int r = u * 32 + lane;
          if (r < C) {
            segoff[r] = (int)((sv[u] >> 16) & 0xffffu);
            segoff[C + r] = (int)(sv[u] & 0xffffu);
          }
        }
        __syncwarp();
        int carry = 0;
        for (int i0 = 0; i0 < 2 * C; i0 += 32) {
          const int i = i0 + lane;
          const int cnt = i < 2 * C ? segoff[i] : 0;
          int incl = cnt;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
          }
          __syncwarp();
          if (i < 2 * C) segoff[i] = carry + incl - cnt;
          carry += __shfl_sync(FULL, incl, 31);
        }
        if (lane == 0) segoff[2 * C] = carry;
        total = carry;
        __syncwarp();
      }
      for (int rbase = 0;; rbase += LIST_CAP) {
        const int n_round = ok ? min(LIST_CAP, total - rbase) : 0;
        if (ok) {
          // gather the round's keys in windows of STAGE_ENTRIES: every lane
          // issues async copies of its segments' words into warp 0's staging
          // buffer, then each word's step stamp is checked (a stale word is
          // polled again) and the key written to the list
          unsigned long long* kw = reinterpret_cast<unsigned long long*>(stage);
          for (int p0w = 0; p0w < n_round; p0w += STAGE_ENTRIES) {
            const int pw1 = min(n_round, p0w + STAGE_ENTRIES);
            for (int i = lane; i < 2 * C; i += 32) {
              const int o0 = segoff[i], o1 = segoff[i + 1];
              const int a0 = max(o0, rbase + p0w), a1 = min(o1, rbase + pw1);
              if (a0 < a1) {
                const int r = i < C ? i : i - C;
                const int skip = i < C ? 0 : segoff[r + 1] - segoff[r];  // neurons follow the CTA's inputs
                const unsigned long long* src = d.cta_keys + ((size_t)par * C + r) * d.key_cap + skip - o0;
                for (int x = a0; x < a1; ++x) cp_async8(kw + (x - rbase - p0w), src + x);
              }
            }
            cp_async_wait_all();
            __syncwarp();
            for (int x = p0w + lane; x < pw1; x += 32) {
              unsigned long long v = kw[x - p0w];
              if ((unsigned)(v >> 32) != stamp) {
                // locate the word's source to poll it again
                int i = 0;
                while (i + 1 < 2 * C && segoff[i + 1] <= rbase + x) ++i;
                const int r = i < C ? i : i - C;
                const int skip = i < C ? 0 : segoff[r + 1] - segoff[r];
                const unsigned long long* src =
                    d.cta_keys + ((size_t)par * C + r) * d.key_cap + skip + (rbase + x - segoff[i]);
                v = repoll(src, ld_relaxed_u64(src), stamp, d, ok);
              }
              list[x] = (uint32_t)v;
            }
            __syncwarp();
          }
          ok = __all_sync(FULL, ok);
        }
        const bool last = !ok || rbase + LIST_CAP >= total;
        if (lane == 0) {
          s_round[0] = n_round;
          s_round[1] = last ? 1 : 0;
          s_round[2] = ok ? 1 : 0;
        }
        round_barrier(nthreads);
        if (!ok) {
          ok_run = false;
          break;
        }
        process_round(n_round);
        if (last) break;
        round_barrier(nthreads);
      }
    } else {
      while (true) {
        round_barrier(nthreads);
        const int n = s_round[0];
        const bool last = s_round[1] != 0;
        if (s_round[2] == 0) {
          ok_run = false;
          break;
        }
        process_round(n);
        if (last) break;
        round_barrier(nthreads);
      }
    }
    if (!ok_run) break;

    // ---- phase B: plastic afferents of the CTA's spiking posts -----------------
    // Every afferent of a spiking post whose presynaptic key had no event this
    // step gets its LTP update here (those with an event were updated in the
    // pre pass).  Each weight is touched at most once, so the order is free and
    // the work is spread over all warps of the CTA: after a CTA barrier (every
    // warp has applied its rounds) the warps list their spiking posts in
    // shared memory, and the posts' afferents are cut into chunks of 32 * AFF
    // that the warps take in turn.  Posts beyond the list's capacity are done
    // by their own warp.
    if (stdp_run) {
      constexpr int AFF = 4;
      constexpr int SP_CAP = LIST_CAP / 2;
      // AFF afferents per lane: their CSC records (pre key, weight; contiguous
      // per post), then all of their bitmap words and pre traces are loaded
      // together (lanes past the end read afferent a, always valid, and skip).
      auto afferents = [&](const float post_tr, const int a, const int a1) {
        uint2 cc[AFF];
#pragma unroll
        for (int u = 0; u < AFF; ++u) {
          const int ai = a + u * 32 + lane;
          cc[u] = d.csc[ai < a1 ? ai : a];
        }
        uint32_t vm[AFF];
        float prt[AFF];
#pragma unroll
        for (int u = 0; u < AFF; ++u) {
          const int pk = (int)cc[u].x;
          vm[u] = __ldcg(bitsA + (pk >> 5)) | __ldcg(bitsP + (pk >> 5));
          prt[u] = __ldcg(pub + pk);
        }
#pragma unroll
        for (int u = 0; u < AFF; ++u) {
          const int ai = a + u * 32 + lane;
          const int pk = (int)cc[u].x;
          if (ai >= a1 || ((vm[u] >> (pk & 31)) & 1u)) continue;  // pre event: done in the pre pass
          const float nw = stdp_update(d, __uint_as_float(cc[u].y), false, true, post_tr, prt[u]);
          d.csc[ai].y = __float_as_uint(nw);
          ++n_post;
        }
      };
      __syncthreads();
      for (int wi = 0; wi < TS / 32; ++wi) {
        const uint32_t word = evw_s[wi];  // postsynaptic STDP events
        if (!word) continue;
        const int c = __popc(word);
        int base = 0;
        if (lane == 0) base = atomicAdd(&s_nsp, c);
        base = __shfl_sync(FULL, base, 0);
        const int mine = base + __popc(word & lanemask_lt());
        if (((word >> lane) & 1u) && mine < SP_CAP) {
          const int ql = wi * 32 + lane;
          list[mine] = (uint32_t)(p0 + ql);
          list[SP_CAP + mine] = __float_as_uint(post_s[ql]);
        }
        if (base + c > SP_CAP) {
          // overflow posts: this warp updates them itself
          uint32_t over = __ballot_sync(FULL, ((word >> lane) & 1u) && mine >= SP_CAP);
          while (over) {
            const int bb = __ffs(over) - 1;
            over &= over - 1;
            const int ql = wi * 32 + bb;
            const int q = p0 + ql;
            const int a0 = __ldg(d.csc_ptr + q), a1 = __ldg(d.csc_ptr + q + 1);
            for (int a = a0; a < a1; a += 32 * AFF) afferents(post_s[ql], a, a1);
          }
        }
      }
      __syncthreads();
      const int nsp = min(s_nsp, SP_CAP);
      int item0 = 0;
      for (int j = 0; j < nsp; ++j) {
        const int q = (int)list[j];
        const float post_tr = __uint_as_float(list[SP_CAP + j]);
        const int a0 = __ldg(d.csc_ptr + q), a1 = __ldg(d.csc_ptr + q + 1);
        const int nchunk = (a1 - a0 + 32 * AFF - 1) / (32 * AFF);
        for (int c = ((w - item0) % W + W) % W; c < nchunk; c += W) afferents(post_tr, a0 + c * 32 * AFF, a1);
        item0 += nchunk;
      }
    }
    ++steps_done;
  }

  // ---- write the tile's state back ---------------------------------------------
  __syncwarp();
  {
    float* rh = d.ring + (size_t)t_idx * B * TS * L;
    const int nr = B * TS * L;
    for (int i = lane; i < nr; i += 32) rh[i] = ring_s[i];
    for (int i = lane; i < TS; i += 32) {
      const int n = p0 + i;
      if (n < N) {
        d.V[n] = V_s[i];
        d.last[n] = last_s[i];
        if (d.has_stdp) {
          d.post_trace[n] = post_s[i];
          d.pre_trace[KL + n] = pre_s[i];
        }
      }
    }
    if (kind != SPK_SYN_VOLTAGE)
      for (int i = lane; i < TS * L; i += 32) {
        const int n = p0 + i / L;
        if (n < N) d.gtr[(size_t)p0 * L + i] = gtr_s[i];
      }
    for (int i = lane; i < ITS; i += 32) {
      const int k = kin0 + i;
      if (k < Nin) {
        d.in_next[Nin - 1 - k] = innext_s[i];
        if (d.has_stdp) d.pre_trace[k] = inpre_s[i];
      }
    }
  }
  // events: warp sums, one atomic per warp
  {
    unsigned long long e = ev;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) e += __shfl_xor_sync(FULL, e, o);
    if (lane == 0 && e) atomicAdd(&d.ctl->events, e);
    if (d.has_stdp) {
      unsigned long long a = n_pre, b = n_post;
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        a += __shfl_xor_sync(FULL, a, o);
        b += __shfl_xor_sync(FULL, b, o);
      }
      if (lane == 0 && a) atomicAdd(&d.ctl->stdp_pre, a);
      if (lane == 0 && b) atomicAdd(&d.ctl->stdp_post, b);
    }
  }
  if (cm.rank == 0 && w == W - 1) {
    if (lane == 0) {
      d.ctl->step = ctl0.step + steps_done;
      d.ctl->gstep = ctl0.gstep + steps_done;
      if (steps_done > 0) d.ctl->inputs_active = 1;
      if (recorder) d.ctl->spike_count = spike_count;
    }
  }
}

}  // namespace spk
