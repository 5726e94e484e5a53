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
//            advances the per-neuron STDP traces, and publishes one ballot word
//            per 32 keys into the network's spike bitmap (replaces the atomic
//            activation list of InlineDeviceFunctions.hpp:4-18);
//   barrier  CTA barrier, or a bounded arrival counter when the network spans
//            several CTAs;
//   phase B  each CTA lists the step's active presynaptic keys in ascending
//            order; each warp walks that list, reads the (key, tile) sub-row of
//            the row-partitioned CSR (8 B per synapse) and adds w*scale into
//            its own ring cells (reference activate_synapses,
//            Spike/Backend/CUDA/Synapses/SpikingSynapses.cu:168-202), after
//            updating plastic weights of rows with a pre event
//            (WeightDependentSTDPPlasticity.cu:85-161); then it updates the
//            plastic afferents of its own spiking posts whose presynaptic
//            neuron had no event.
//
// Every ring cell has exactly one writer (the tile's warp) which applies the
// contributions of a step in canonical order (ascending key, then synapse
// order), so the result is deterministic and atomic-free.  Phase A of the next
// step reads only the warp's own cells, so one barrier per step suffices.
#pragma once

#include <cuda_runtime.h>

#include "../../include/spike_gb300.h"
#include "spk_internal.h"

namespace spk {

constexpr unsigned FULL = 0xffffffffu;
constexpr unsigned long long BARRIER_TIMEOUT_NS = 4000000000ull;  // 4 s

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_volatile(const int* p) { return *(volatile const int*)p; }
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Arrival barrier over the nctas CTAs of one network.  Every wait is bounded:
// on timeout the launch's abort flag and the network status are set and all
// CTAs leave their step loops.
__device__ bool net_barrier(const NetDev& d, unsigned target, int* flag_smem) {
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    atomicAdd(d.barrier, 1u);
    const unsigned long long t0 = globaltimer();
    while (ld_acquire(d.barrier) < target) {
      if (ld_volatile(d.abort_flag)) {
        ok = 0;
        break;
      }
      if (globaltimer() - t0 > BARRIER_TIMEOUT_NS) {
        atomicExch(d.abort_flag, 1);
        atomicCAS(&d.ctl->status, 0, SPK_ERR_TIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    *flag_smem = ok;
  }
  __syncthreads();
  return *flag_smem != 0;
}

// Exclusive block-wide scan of one int per thread; returns the prefix and the
// total in *total.  scratch needs 33 ints.
__device__ int block_exclusive_scan(int v, int* scratch, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(FULL, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) scratch[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int s = lane < nw ? scratch[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(FULL, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) scratch[lane] = s;  // inclusive warp totals
    if (lane == nw - 1) scratch[32] = s;
  }
  __syncthreads();
  const int before = warp > 0 ? scratch[warp - 1] : 0;
  *total = scratch[32];
  const int r = before + x - v;
  __syncthreads();
  return r;
}

// ltp_and_ltd update of one synapse for G = 1
// (Spike/Backend/CUDA/Plasticity/WeightDependentSTDPPlasticity.cu:132-151):
// pre_ev/post_ev are "spike sub-step >= 0", the traces are this step's values.
__device__ __forceinline__ float stdp_update(const NetDev& d, float old_w, bool pre_ev, bool post_ev,
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

template <int U>
__global__ void __launch_bounds__(512, 1)
    step_kernel(const NetDev* __restrict__ nets, const CtaMap* __restrict__ map, int K) {
  extern __shared__ __align__(16) uint32_t sm[];
  const CtaMap cm = map[blockIdx.x];
  const NetDev& d = nets[cm.net];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int W = d.W;
  const int N = d.N, Nin = d.Nin, KL = d.KL, L = d.L, B = d.B, kind = d.kind;
  const int TS = d.TS, ITS = d.ITS, n_tiles = d.n_tiles, n_keys = d.n_keys, n_words = d.n_words;
  const float dt = d.dt;

  uint32_t* list = sm;
  int* scan = (int*)(sm + LIST_CAP);
  int* misc = (int*)(sm + LIST_CAP + 64);
  const WarpLayout wl = warp_layout(B, TS, L, ITS, kind, d.has_stdp);
  uint32_t* wreg = sm + SHARED_WORDS + w * wl.total;
  float* ring_s = (float*)(wreg + wl.ring);
  float* V_s = (float*)(wreg + wl.V);
  float* last_s = (float*)(wreg + wl.last);
  float* gtr_s = (float*)(wreg + wl.gtr);
  float* post_s = (float*)(wreg + wl.post_tr);
  float* pre_s = (float*)(wreg + wl.pre_tr);
  uint32_t* spkw_s = wreg + wl.spkw;
  float* innext_s = (float*)(wreg + wl.in_next);
  float* inrate_s = (float*)(wreg + wl.in_rate);
  float* inpre_s = (float*)(wreg + wl.in_pre);
  int* seg = (int*)(wreg + wl.seg);

  const RunCtl ctl0 = *d.ctl;
  const int steps_here = min(K, ctl0.steps_total - ctl0.step);
  if (steps_here <= 0) return;
  const bool stdp_run = d.has_stdp && ctl0.plastic;
  const bool rank0 = cm.rank == 0;

  const int t_idx = cm.rank * W + w;  // tile owned by this warp
  const int p0 = t_idx * TS;          // first post of the tile
  const int kin0 = t_idx * ITS;       // first input key of the tile

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
  unsigned long long spike_count = ctl0.spike_count;
  unsigned long long ev = 0;
  bool inputs_active = ctl0.inputs_active != 0;
  int steps_done = 0;
  __syncthreads();

  for (int s = 0; s < steps_here; ++s) {
    const int sr = ctl0.step + s;
    // current_time_in_seconds = starttime + s*timestep_grouping*timestep
    // (Spike/Models/SpikingModel.cpp:226), timestep_index = roundf(t/dt).
    const float t = ctl0.start_time + (float)(sr * 1) * dt;
    const int T = (int)roundf(t / dt);
    const int par = (int)((ctl0.gstep + s) & 1);
    uint32_t* bitsA = d.bitsA + (size_t)par * n_words;
    uint32_t* bitsP = d.bitsP + (size_t)par * n_words;
    float* pub = d.pre_pub + (size_t)par * n_keys;
    const int slot = T % B;
    const float tg = t + 0.0f * dt;  // t + g*timestep with g = 0
    const float half_dt = 0.5f * dt;

    // ---- phase A: LIF neurons of the tile ------------------------------------
    {
      float* ring_slot = ring_s + (size_t)slot * TS * L;
      for (int base = 0; base < TS; base += 32) {
        const int li = base + lane;
        const int n = p0 + li;
        bool spk = false;
        if (n < N) {
          int gi = 0;
          while (gi + 1 < d.n_groups && n >= d.groups[gi].end) ++gi;
          const GroupConst& G = d.groups[gi];
          float Vi = V_s[li];
          float input;
          if (kind == SPK_SYN_CONDUCTANCE) {
            float total = 0.0f;
            for (int l = 0; l < L; ++l) {
              const float cell = ring_slot[li * L + l];
              ring_slot[li * L + l] = 0.0f;
              const float gnew = d.decay[l] * gtr_s[li * L + l] + cell;
              total = total + gnew * (d.vhat[l] - Vi);
              gtr_s[li * L + l] = gnew;
            }
            input = total * G.kR;
          } else if (kind == SPK_SYN_CURRENT) {
            float total = 0.0f;
            for (int l = 0; l < L; ++l) {
              const float cell = ring_slot[li * L + l];
              ring_slot[li * L + l] = 0.0f;
              float inew = gtr_s[li * L + l] * d.decay[l];
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
          if (((tg - last_s[li]) - d.t_ref) > half_dt) {
            Vi = G.k * G.v0 + (1.0f - G.k) * Vi + G.k * d.i_bg + input;
            if (Vi >= G.theta) {
              spk = true;
              last_s[li] = tg;
              Vi = G.vreset;
            }
          }
          V_s[li] = Vi;
          if (stdp_run) {
            float po = post_s[li] * d.E_m;
            po = po + (spk ? d.inc_m : 0.0f);
            post_s[li] = po;
            float pr = pre_s[li] * d.E_p;
            pr = pr + (spk ? d.inc_p : 0.0f);
            pre_s[li] = pr;
            pub[KL + n] = pr;
          }
        }
        const unsigned word = __ballot_sync(FULL, spk);
        if (lane == 0) {
          const int wi = (KL + p0 + base) >> 5;
          bitsA[wi] = word;
          if (stdp_run) bitsP[wi] = word;
          spkw_s[base >> 5] = word;
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
          if (inputs_active) spk = true;
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
        const int wi = (kin0 + base) >> 5;
        bitsA[wi] = wa;
        if (stdp_run) bitsP[wi] = wp;
      }
    }
    inputs_active = true;

    // ---- barrier: the step's bitmap is complete --------------------------------
    if (d.nctas > 1) {
      if (!net_barrier(d, (unsigned)(d.nctas * (s + 1)), misc)) break;
    } else {
      __syncthreads();
    }

    // ---- phase B: list active keys (ascending), propagate, STDP ---------------
    const int nthreads = blockDim.x;
    for (int wbase = 0; wbase < n_words; wbase += nthreads * WPT_MAX) {
      const int wchunk = min(n_words - wbase, nthreads * WPT_MAX);
      const int wpt = (wchunk + nthreads - 1) / nthreads;
      const int my0 = wbase + threadIdx.x * wpt;
      uint32_t wA[WPT_MAX], wP[WPT_MAX];
      int cnt = 0;
#pragma unroll
      for (int i = 0; i < WPT_MAX; ++i) {
        wA[i] = 0u;
        wP[i] = 0u;
        if (i < wpt && my0 + i < wbase + wchunk) {
          wA[i] = __ldcg(bitsA + my0 + i);
          if (stdp_run) wP[i] = __ldcg(bitsP + my0 + i);
          cnt += __popc(wA[i] | wP[i]);
        }
      }
      int total;
      const int my_off = block_exclusive_scan(cnt, scan, &total);
      for (int rbase = 0; rbase < total; rbase += LIST_CAP) {
        const int n_round = min(LIST_CAP, total - rbase);
        // write this thread's keys that fall in the round
        int pos = my_off;
#pragma unroll
        for (int i = 0; i < WPT_MAX; ++i) {
          uint32_t m = wA[i] | wP[i];
          while (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1;
            if (pos >= rbase && pos < rbase + n_round) {
              const uint32_t key = (uint32_t)((my0 + i) * 32 + b);
              const uint32_t fl = (((wA[i] >> b) & 1u) << 31) | (((wP[i] >> b) & 1u) << 30);
              list[pos - rbase] = key | fl;
            }
            ++pos;
          }
        }
        __syncthreads();

        // spike store: recorded by rank 0 in list (canonical) order
        if (rank0 && d.spike_cap > 0) {
          for (int c0 = 0; c0 < n_round; c0 += nthreads) {
            const int j = c0 + threadIdx.x;
            bool rec = false;
            uint32_t key = 0;
            if (j < n_round) {
              const uint32_t lv = list[j];
              key = lv & 0x3fffffffu;
              rec = (lv >> 31) && ((int)key >= KL || ctl0.record_inputs);
            }
            int tot;
            const int off = block_exclusive_scan(rec ? 1 : 0, scan, &tot);
            if (rec) {
              const unsigned long long p = spike_count + (unsigned long long)off;
              if (p < (unsigned long long)d.spike_cap)
                d.spikes[p] = make_uint2(key, __float_as_uint(t));
              else
                atomicCAS(&d.ctl->status, 0, SPK_ERR_OVERFLOW);
            }
            spike_count += (unsigned long long)tot;
          }
          if (spike_count > (unsigned long long)d.spike_cap) spike_count = d.spike_cap;
        }

        // each warp: its tile's sub-rows of the listed keys, in list order
        for (int jb = 0; jb < n_round; jb += 32) {
          const int j = jb + lane;
          uint32_t lv = 0u;
          int rp0 = 0, len = 0;
          float prt = 0.0f;
          if (j < n_round) {
            lv = list[j];
            const int key = (int)(lv & 0x3fffffffu);
            const size_t ri = (size_t)key * n_tiles + t_idx;
            rp0 = __ldg(d.rowptr + ri);
            len = __ldg(d.rowptr + ri + 1) - rp0;
            if (stdp_run) prt = __ldcg(pub + key);
            if (lv >> 31) ev += (unsigned long long)len;
          }
          int incl = len;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
          }
          const int tot = __shfl_sync(FULL, incl, 31);
          seg[lane] = incl - len;
          seg[32 + lane] = rp0;
          seg[64 + lane] = (int)lv;
          seg[96 + lane] = __float_as_int(prt);
          __syncwarp();
          for (int f0 = 0; f0 < tot; f0 += 32 * U) {
            uint2 ent[U];
            int eid[U], jj[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
              const int f = f0 + u * 32 + lane;
              jj[u] = -1;
              eid[u] = 0;
              ent[u] = make_uint2(0u, 0u);
              if (f < tot) {
                int sj = 0;
#pragma unroll
                for (int st = 16; st >= 1; st >>= 1)
                  if (seg[sj + st] <= f) sj += st;
                const int e = seg[32 + sj] + (f - seg[sj]);
                jj[u] = sj;
                eid[u] = e;
                ent[u] = d.entries[e];
              }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
              bool add = false;
              int cell = -1 - lane;
              float contrib = 0.0f;
              if (jj[u] >= 0) {
                const uint32_t flv = (uint32_t)seg[64 + jj[u]];
                const bool A = (flv >> 31) != 0;
                const bool P = ((flv >> 30) & 1u) != 0;
                const uint32_t x = ent[u].x;
                const int q = (int)(x & 0xffffu);
                const int dl = (int)((x >> 16) & 0xffu);
                const int lb = (int)((x >> 24) & 0xfu);
                const int c = (int)(x >> 28);
                float v = __uint_as_float(ent[u].y);
                if (c != 0) {
                  if (stdp_run) {
                    const bool post_ev = ((spkw_s[q >> 5] >> (q & 31)) & 1u) != 0;
                    if (P || post_ev) {
                      v = stdp_update(d, v, P, post_ev, post_s[q], __int_as_float(seg[96 + jj[u]]));
                      d.entries[eid[u]].y = __float_as_uint(v);
                    }
                  }
                  contrib = v * d.scale_tab[c];
                } else {
                  contrib = v;
                }
                if (A) {
                  add = true;
                  int sl = slot + dl;
                  if (sl >= B) sl -= B;
                  cell = (sl * TS + q) * L + lb;
                }
              }
              // apply in lane order within a chunk (match_any groups lanes that
              // hit the same cell), chunks in program order
              const unsigned grp = __match_any_sync(FULL, cell);
              const int rank = __popc(grp & lanemask_lt());
              const int maxr = __reduce_max_sync(FULL, add ? rank : 0);
              for (int r = 0; r <= maxr; ++r) {
                if (add && rank == r) ring_s[cell] = ring_s[cell] + contrib;
                __syncwarp();
              }
            }
          }
          __syncwarp();
        }
        __syncthreads();
      }
    }

    // ---- phase B: plastic afferents of the tile's spiking posts ---------------
    if (stdp_run) {
      for (int wi = 0; wi < TS / 32; ++wi) {
        uint32_t word = spkw_s[wi];
        while (word) {
          const int b = __ffs(word) - 1;
          word &= word - 1;
          const int ql = wi * 32 + b;
          const int q = p0 + ql;
          const int a0 = __ldg(d.csc_ptr + q), a1 = __ldg(d.csc_ptr + q + 1);
          for (int a = a0 + lane; a < a1; a += 32) {
            const uint2 cc = __ldg(d.csc + a);
            const int pk = (int)cc.y;
            const uint32_t wa = __ldcg(bitsA + (pk >> 5));
            const uint32_t wp = __ldcg(bitsP + (pk >> 5));
            if (((wa | wp) >> (pk & 31)) & 1u) continue;  // row handled in the pre pass
            const float old = __uint_as_float(d.entries[cc.x].y);
            const float prt = __ldcg(pub + pk);
            const float nw = stdp_update(d, old, false, true, post_s[ql], prt);
            d.entries[cc.x].y = __float_as_uint(nw);
          }
        }
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
  }
  if (rank0 && threadIdx.x == 0) {
    d.ctl->step = ctl0.step + steps_done;
    d.ctl->gstep = ctl0.gstep + steps_done;
    if (steps_done > 0) d.ctl->inputs_active = 1;
    d.ctl->spike_count = spike_count;
  }
}

}  // namespace spk
