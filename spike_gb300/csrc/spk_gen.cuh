// spk_gen.cuh - device-side generation of a network's connectivity, written
// straight into the engine's row-partitioned CSR (spk_net_generate).
//
// One thread handles one (presynaptic key, post tile) cell at a time.  For
// every projection whose presynaptic range holds the key's neuron or input it
// draws the connection of each post of the tile with Philox keyed by
// (connectivity seed, post / 4, pre code, DOMAIN_CONNECT) - one block of four
// uniforms per four posts - and, for a connected pair, the weight and delay
// from Philox (post, pre code, DOMAIN_SYNAPSE).  The draws depend only on the
// pair, never on the schedule or on the order of the projections, so a
// network is the same for every tile size and CTA count.  A count pass sizes
// the cells, a scan turns the counts into row pointers, and a fill pass writes
// the entries of each cell in ascending post order (projections are sorted by
// first post, and those of one presynaptic neuron do not overlap).
#pragma once

#include <cuda_runtime.h>

#include "spk_internal.h"

namespace spk {

constexpr int MAX_PROJECTIONS = 64;

struct GenProj {
  int pop;              // SPK_POP_NEURONS or SPK_POP_INPUTS
  int pre_lo, pre_hi;   // presynaptic indices [lo, hi) within the population
  int post_lo, post_hi; // posts [lo, hi)
  float p;              // connection probability
  float w_lo, w_span;   // weight = w_lo + w_span * u, u in (0, 1]
  float scale;          // folded into the entry value of static synapses
  int d_lo, d_n;        // delay = d_lo + min((int)(u * d_n), d_n - 1)
  int label, cls;       // cls 0 = static, >= 1 plastic scale class
};

struct GenShape {
  int N, Nin, KL, n_tiles, TS, n_proj;
  long long n_cells;
  uint64_t seed;
};

// The synapse a pair (pre_code, q) gets from projection P: weight value as the
// entry stores it and the delay.
SPK_HD void gen_synapse(uint64_t seed, const GenProj& P, uint32_t pre_code, int q, float& value, int& delay) {
  const u32x4 r = draw4(seed, (uint32_t)q, pre_code, DOMAIN_SYNAPSE);
  const float w = P.w_lo + P.w_span * uniform_open0(r.x);
  int dn = (int)(uniform_open0(r.y) * (float)P.d_n);
  if (dn > P.d_n - 1) dn = P.d_n - 1;
  delay = P.d_lo + dn;
  value = P.cls ? w : w * P.scale;
}

// Presynaptic code of a pair draw: neurons n -> n, inputs i -> 2^31 | i.
SPK_HD uint32_t gen_pre_code(int pop, int idx) {
  return pop == SPK_POP_INPUTS ? (0x80000000u | (uint32_t)idx) : (uint32_t)idx;
}

// FILL = false: counts[c] = synapses of cell c, totals[0/1] += all / plastic,
// delay_range = [min, max] drawn delay.  FILL = true: write the cell's entries
// at rowptr[c], plus (with sort_post) each entry's sort key - its post if
// plastic, N otherwise - and presynaptic key, and per-post plastic counts.
template <bool FILL>
__global__ void __launch_bounds__(256) gen_cells_kernel(GenShape g, const GenProj* __restrict__ proj,
                                                        int* counts, unsigned long long* totals,
                                                        const int* __restrict__ rowptr, uint2* entries,
                                                        uint32_t* sort_post, uint32_t* entry_key, int* post_cnt,
                                                        int* delay_range) {
  __shared__ GenProj sp[MAX_PROJECTIONS];
  for (int j = threadIdx.x; j < g.n_proj; j += blockDim.x) sp[j] = proj[j];
  __syncthreads();
  unsigned long long n_all = 0, n_pl = 0;
  int dmin = 1 << 30, dmax = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < g.n_cells; c += stride) {
    const int key = (int)(c / g.n_tiles), tile = (int)(c - (long long)key * g.n_tiles);
    int pop, idx;
    bool real;
    if (key < g.KL) {
      pop = SPK_POP_INPUTS;
      idx = g.Nin - 1 - key;
      real = key < g.Nin;
    } else {
      pop = SPK_POP_NEURONS;
      idx = key - g.KL;
      real = idx < g.N;
    }
    int cnt = 0, pos = 0;
    if (FILL) pos = rowptr[c];
    if (real) {
      const uint32_t pre_code = gen_pre_code(pop, idx);
      const int t0 = tile * g.TS, t1 = t0 + g.TS;
      for (int j = 0; j < g.n_proj; ++j) {
        const GenProj& P = sp[j];
        if (P.pop != pop || idx < P.pre_lo || idx >= P.pre_hi) continue;
        const int q0 = max(t0, P.post_lo), q1 = min(t1, P.post_hi);
        for (int gq = q0 & ~3; gq < q1; gq += 4) {
          const u32x4 r = draw4(g.seed, (uint32_t)(gq >> 2), pre_code, DOMAIN_CONNECT);
          const uint32_t rr[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int q = gq + k;
            if (q < q0 || q >= q1 || !(uniform_open0(rr[k]) <= P.p)) continue;
            float v;
            int dl;
            gen_synapse(g.seed, P, pre_code, q, v, dl);
            if (FILL) {
              entries[pos] = make_uint2(pack_entry((uint32_t)(q - t0), (uint32_t)dl, (uint32_t)P.label,
                                                   (uint32_t)P.cls),
                                        f2u(v));
              if (sort_post) {
                sort_post[pos] = P.cls ? (uint32_t)q : (uint32_t)g.N;
                entry_key[pos] = (uint32_t)key;
                if (P.cls) atomicAdd(post_cnt + q, 1);
              }
              ++pos;
            } else {
              ++cnt;
              if (P.cls) ++n_pl;
              dmin = min(dmin, dl);
              dmax = max(dmax, dl);
            }
          }
        }
      }
    }
    if (!FILL) {
      counts[c] = cnt;
      n_all += (unsigned long long)cnt;
    }
  }
  if (!FILL) {
    for (int o = 16; o >= 1; o >>= 1) {
      n_all += __shfl_xor_sync(0xffffffffu, n_all, o);
      n_pl += __shfl_xor_sync(0xffffffffu, n_pl, o);
    }
    dmin = __reduce_min_sync(0xffffffffu, dmin);
    dmax = __reduce_max_sync(0xffffffffu, dmax);
    if ((threadIdx.x & 31) == 0) {
      if (n_all) atomicAdd(totals, n_all);
      if (n_pl) atomicAdd(totals + 1, n_pl);
      if (dmax > 0) {
        atomicMin(delay_range, dmin);
        atomicMax(delay_range + 1, dmax);
      }
    }
  }
}

__global__ void gen_iota_kernel(uint32_t* v, long long n) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) v[i] = (uint32_t)i;
}

// The i-th plastic synapse in (post, entry index) order gets afferent record
// csc[i] = (presynaptic key, weight), and for the per-synapse-trace rules its
// delay; its entry then points at the record.
__global__ void gen_csc_kernel(uint2* csc, uint2* entries, const uint32_t* sorted_entry, const uint32_t* entry_key,
                               long long P, int* csc_delay) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < P; i += stride) {
    const uint32_t e = sorted_entry[i];
    const uint2 en = entries[e];
    csc[i] = make_uint2(entry_key[e], en.y);
    if (csc_delay) csc_delay[i] = (int)((en.x >> 16) & 0xffu);
    entries[e].y = (uint32_t)i;
  }
}

}  // namespace spk
