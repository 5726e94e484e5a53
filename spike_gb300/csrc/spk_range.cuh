// spk_range.cuh - propagation over post ranges: one CTA per range of posts.
//
// The per-tile propagation of spk_bulk.cuh gives each warp a tile of up to a
// few hundred posts.  At connection probabilities of 1-5 % a presynaptic key
// then owns a sub-row of one to three entries per tile, so a warp spends most
// of its instructions on row pointers, partly used sectors and grouping lanes
// by cell.  Networks built with tiles of RANGE_MIN_TS posts or more (bulk mode
// only: such a tile's ring does not fit a warp's shared memory) propagate here
// instead, one CTA of RANGE_THREADS threads per tile ("range"):
//
//   * per chunk of up to RANGE_KEYS list keys the CTA stages the keys' sub-row
//     bounds in its range (two rowptr words per key) and scans their lengths,
//     which orders the range's entries of the step as one stream: ascending
//     key, then creation order within a sub-row, the canonical order;
//   * the stream is applied in rounds of RANGE_ROUND consecutive entries,
//     RANGE_U per thread.  A thread finds its entries' keys by a binary search
//     over the scanned lengths, loads the entries (coalesced runs of the
//     sub-rows), updates plastic weights (the STDP pre pass), and for a
//     delivering key publishes (ring cell, contribution) under its position
//     in the round and links itself into the chain of its cell's hash bucket
//     (atomicExch on the bucket's head);
//   * after a barrier the last thread to link into a bucket applies the
//     bucket's contributions: for a bucket holding one entry a single add
//     into the ring cell; otherwise, cell by cell, the contributions in
//     ascending position, which is the canonical order.
//
// So every ring cell still receives the step's contributions one by one in
// canonical order, after those of earlier rounds (a barrier separates
// rounds), and a network gives the same bits as in every other mode.  A range
// whose step is dense (about one entry per four cells of its delay slots)
// reads those slots into a shared-memory window first and writes them back
// at the end; a sparse range adds into the ring in global memory (L2).
// Either way a round preloads the ring words of its entries before its
// barrier, which is safe because only the round's bucket heads write ring
// cells, each cell by exactly one of them.
#pragma once

#include "spk_bulk.cuh"

namespace spk {

// Tuning constants (measured on the 256-instance sweep), overridable at
// compile time.
#ifndef SPK_RANGE_MIN_TS
#define SPK_RANGE_MIN_TS 512
#endif
#ifndef SPK_RANGE_WIN_CAP
#define SPK_RANGE_WIN_CAP 0
#endif
#ifndef SPK_RANGE_THREADS
#define SPK_RANGE_THREADS 256
#endif
#ifndef SPK_RANGE_U
#define SPK_RANGE_U 4
#endif
#ifndef SPK_RANGE_KEYS
#define SPK_RANGE_KEYS 1024
#endif
#ifndef SPK_RANGE_MINB
#define SPK_RANGE_MINB 3
#endif
constexpr int RANGE_MIN_TS = SPK_RANGE_MIN_TS;         // tiles propagated by bulk_range_kernel
constexpr int RANGE_WIN_CAP = SPK_RANGE_WIN_CAP;       // ring-window words of a range at most
constexpr int RANGE_HEAD_CAP = 16 * 1024;              // bucket heads of a range at most (64 KB)
constexpr int RANGE_THREADS = SPK_RANGE_THREADS;
constexpr int RANGE_U = SPK_RANGE_U;                   // stream positions per thread and round
constexpr int RANGE_ROUND = RANGE_THREADS * RANGE_U;   // entries per round
constexpr int RANGE_KEYS = SPK_RANGE_KEYS;             // list keys per chunk
constexpr int RANGE_KPT = RANGE_KEYS / RANGE_THREADS;  // keys per thread while staging
constexpr int RANGE_POS_BITS = 12;                     // position field of a head word
constexpr unsigned short RANGE_NONE = 0xffff;
static_assert(RANGE_ROUND <= (1 << RANGE_POS_BITS), "round positions fit the head word");
static_assert(RANGE_KEYS % RANGE_THREADS == 0, "whole keys per thread");

struct BulkRangeBlock {
  int net;   // index into the batch's NetDev array
  int tile;  // the range (tile) of the network
  int pad0, pad1;
  const RunCtl* ctl;  // the network's run control
  const int* n_list;  // the network's step key count
};

struct RangeShared {
  uint32_t ecell[RANGE_ROUND];      // delay cell of each position of the round
  float econ[RANGE_ROUND];          // its contribution
  unsigned short enxt[RANGE_ROUND]; // next position of its bucket's chain
  uint32_t list[RANGE_KEYS];        // list words of the chunk (key | A << 31 | P << 30)
  int kstart[RANGE_KEYS];           // first entry of each key's sub-row in the range
  int koff[RANGE_KEYS + 1];         // exclusive prefix of the sub-row lengths
  float kpre[RANGE_KEYS];           // presynaptic traces (plastic runs)
  int wsum[RANGE_THREADS / 32];
  float scl[MAX_CLASSES];
};

// Dynamic shared memory of a launch in 4-byte words: the ring window of the
// largest range followed by its bucket heads.
struct RangeSmem {
  int win_words, head_words;
};
__host__ __device__ inline size_t range_smem_bytes(const RangeSmem& z) {
  return 4 * ((size_t)z.win_words + z.head_words);
}

// A contribution's target within the range: `dc` its delay cell, the index
// (delay - 1) * TS * L + post * L + label over the delay slots after the
// current one (also its index in the ring window); where the cell lives this
// step: the window (delay <= ws) or the ring slice in global memory.
struct RangeRing {
  float* ring;   // the range's ring slice [B][TS * L]
  float* win;    // window [ws][TS * L] (shared memory)
  int ws, slot, B, slot_words;
  __device__ __forceinline__ float* global_at(uint32_t dc, int dl) const {
    int sl = slot + dl;
    if (sl >= B) sl -= B;
    return ring + (size_t)sl * slot_words + (dc - (uint32_t)(dl - 1) * slot_words);
  }
  // ring words in global memory go through L2 only: a later round's load
  // must see an earlier round's store made by another thread of the CTA
  __device__ __forceinline__ float load(uint32_t dc) const {
    const int dl = (int)(dc / (uint32_t)slot_words) + 1;
    return dl <= ws ? win[dc] : __ldcg(global_at(dc, dl));
  }
  __device__ __forceinline__ void store(uint32_t dc, float v) const {
    const int dl = (int)(dc / (uint32_t)slot_words) + 1;
    if (dl <= ws)
      win[dc] = v;
    else
      __stcg(global_at(dc, dl), v);
  }
};

// Applies a bucket chain of positions holding more than one delay cell (a
// hashed head table): cell by cell, contributions in ascending position.
// `my_cell`/`my_val` are the head's own cell and its preloaded ring word.
__device__ __noinline__ void range_apply_mixed_chain(const RangeShared& sm, const RangeRing& rr, int r,
                                                     uint32_t my_cell, float my_val) {
  unsigned long long last = 0ull;
  long long cur = -1;
  float acc = 0.0f;
  for (;;) {
    unsigned long long best = ~0ull;
    for (int it = r; it != RANGE_NONE; it = sm.enxt[it]) {
      const unsigned long long k = ((unsigned long long)sm.ecell[it] << RANGE_POS_BITS) | (unsigned)it;
      if (k >= last && k < best) best = k;
    }
    if (best == ~0ull) break;
    const uint32_t c = (uint32_t)(best >> RANGE_POS_BITS);
    const int rk = (int)(best & ((1u << RANGE_POS_BITS) - 1));
    if ((long long)c != cur) {
      if (cur >= 0) rr.store((uint32_t)cur, acc);
      cur = c;
      acc = c == my_cell ? my_val : rr.load(c);
    }
    acc = acc + sm.econ[rk];
    last = best + 1;
  }
  if (cur >= 0) rr.store((uint32_t)cur, acc);
}

// The sum, in ascending position, of a chain whose positions all hold the
// head's cell, added to `val` one contribution at a time.
__device__ __forceinline__ float range_chain_sum(const RangeShared& sm, int r, float val) {
  const int b = sm.enxt[r];
  if (sm.enxt[b] == RANGE_NONE) {  // two positions: the common case
    const int lo = min(r, b), hi = max(r, b);
    return (val + sm.econ[lo]) + sm.econ[hi];
  }
  float acc = val;
  int last = -1;
  for (;;) {
    int best = RANGE_ROUND;
    for (int it = r; it != RANGE_NONE; it = sm.enxt[it])
      if (it > last && it < best) best = it;
    if (best == RANGE_ROUND) break;
    acc = acc + sm.econ[best];
    last = best;
  }
  return acc;
}

// kPass as bulk_prop_kernel: 0 the single fused pass; 1 and 2 the two passes
// of a batch in which a network normalises its weights after the
// event-driven rule.
//
// Dynamic shared memory (`sz`, in 4-byte words): the range's ring window, the
// delay slots 1..ws after the current one, read when the step's first chunk
// says the range's entries are dense enough and written back (slots that
// received a contribution) at the end; then the bucket heads.  When the
// range's D_max delay slots fit the heads, a bucket is one delay cell, so
// every chain holds one cell; otherwise cells are hashed into the heads and a
// chain may mix cells.
template <int kPass>
__global__ void __launch_bounds__(RANGE_THREADS, SPK_RANGE_MINB)
    bulk_range_kernel(const NetDev* __restrict__ nets, const BulkRangeBlock* __restrict__ blocks, int s,
                      RangeSmem sz) {
  extern __shared__ __align__(16) float rwin[];
  __shared__ __align__(16) NetDev sd;
  __shared__ unsigned s_dirty;
  __shared__ RunCtl sctl;
  __shared__ RangeShared sm;
  __shared__ int s_nlist;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  uint32_t* head = (uint32_t*)(rwin + sz.win_words);
  const BulkRangeBlock rb = blocks[blockIdx.x];
  {
    const uint32_t* src = (const uint32_t*)(nets + rb.net);
    uint32_t* dst = (uint32_t*)&sd;
    for (int i = tid; i < (int)(sizeof(NetDev) / 4); i += RANGE_THREADS) dst[i] = __ldg(src + i);
    if (tid == 0) sctl = load_ctl(rb.ctl);
  }
  if (tid == 0) s_dirty = 0u;
  pdl_wait_then_release();
  if (tid == 0) s_nlist = *rb.n_list;
  __syncthreads();
  const NetDev& d = sd;
  BulkStep st = bulk_step(d, sctl, s);
  const int n_list = s_nlist;
  if (!st.live || n_list == 0) return;  // the whole CTA
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
  const int TS = d.TS, L = d.L, B = d.B, KL = d.KL, n_tiles = d.n_tiles;
  const int p0 = rb.tile * TS;
  const int slot_words = TS * L;  // a multiple of 32
  float* ring = d.ring + (size_t)rb.tile * B * slot_words;
  const int* rowptr = d.rowptr + rb.tile;
  const uint2* entries = d.entries;
  uint2* csc = d.csc;
  const StdpConst sc = stdp_const(d);
  if (tid < MAX_CLASSES) sm.scl[tid] = d.scale_tab[tid];
  // bucket heads: one per delay cell when they fit, else a power-of-two hash
  const int dcells = (B - 2 * d.G - 1) * slot_words;  // D_max slots
  const bool direct = dcells <= sz.head_words;
  const int hbits = 31 - __clz(max(sz.head_words, 1));
  const int hwords = direct ? dcells : (1 << hbits);
  for (int i = tid; i < hwords; i += RANGE_THREADS) head[i] = 0u;

  unsigned long long ev = 0, n_pre = 0;
  uint32_t epoch = 0;
  RangeRing rr{ring, rwin, 0, st.slot, B, slot_words};
  unsigned dirty = 0u;  // window slots this thread wrote
  for (int kb = 0; kb < n_list; kb += RANGE_KEYS) {
    const int nk = min(RANGE_KEYS, n_list - kb);
    __syncthreads();  // the previous chunk's rounds are done with the chunk arrays
    // the chunk's keys: list words, sub-row bounds in the range, traces
    int len[RANGE_KPT];
    int tsum = 0;
#pragma unroll
    for (int u = 0; u < RANGE_KPT; ++u) {
      const int j = tid * RANGE_KPT + u;
      len[u] = 0;
      if (j < nk) {
        const uint32_t lv = d.step_list[kb + j] & kmask;
        const uint32_t key = lv & 0x3fffffffu;
        const int a = rowptr[(size_t)key * n_tiles], e = rowptr[(size_t)key * n_tiles + 1];
        sm.list[j] = lv;
        sm.kstart[j] = a;
        // a key that neither delivers nor can update a plastic weight is skipped
        len[u] = ((lv >> 31) || st.stdp_run) ? e - a : 0;
        if (st.stdp_run) sm.kpre[j] = d.pre_pub[key];
      }
      tsum += len[u];
    }
    int incl = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) sm.wsum[w] = incl;
    __syncthreads();
    if (w == 0) {
      const int v = lane < RANGE_THREADS / 32 ? sm.wsum[lane] : 0;
      int wi = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, wi, o);
        if (lane >= o) wi += y;
      }
      if (lane < RANGE_THREADS / 32) sm.wsum[lane] = wi - v;
      if (lane == 31) sm.koff[RANGE_KEYS] = wi;  // the chunk's entries
    }
    __syncthreads();
    {
      int o = sm.wsum[w] + incl - tsum;
#pragma unroll
      for (int u = 0; u < RANGE_KPT; ++u) {
        sm.koff[tid * RANGE_KPT + u] = o;
        o += len[u];
      }
    }
    __syncthreads();
    const int total = sm.koff[RANGE_KEYS];
    if (kb == 0) {
      // The window pays when the step's entries (estimated from the first
      // chunk) would touch more ring sectors one by one than the window has
      // words to move: about one entry per four window words.
      const int ws_max = min(B - 2 * d.G - 1, sz.win_words / slot_words);
      const long long est = (long long)total * ((n_list + RANGE_KEYS - 1) / RANGE_KEYS);
      rr.ws = (ws_max > 0 && est * 4 > (long long)ws_max * slot_words) ? ws_max : 0;
      for (int k = 0; k < rr.ws; ++k) {
        int sl = st.slot + 1 + k;
        if (sl >= B) sl -= B;
        const float* src = ring + (size_t)sl * slot_words;
        float* dst = rwin + (size_t)k * slot_words;
        for (int i = tid * 4; i < slot_words; i += RANGE_THREADS * 4) cp_async16(dst + i, src + i);
      }
      if (rr.ws) {
        cp_async_wait_all();
        __syncthreads();
      }
    }

    // positions [base + tid*U, +U): their keys (binary search, then forward)
    // and their entries, loaded as streaming data
    auto locate = [&](int base, int (&jj)[RANGE_U], uint2 (&en)[RANGE_U]) {
      const int p = base + tid * RANGE_U;
      int j = 0;
      if (p < total) {
        int lo = 0, hi = nk - 1;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (sm.koff[mid + 1] <= p) lo = mid + 1;
          else hi = mid;
        }
        j = lo;
      }
#pragma unroll
      for (int u = 0; u < RANGE_U; ++u) {
        jj[u] = -1;
        en[u] = make_uint2(0u, 0u);
        if (p + u < total) {
          while (sm.koff[j + 1] <= p + u) ++j;
          jj[u] = j;
          en[u] = __ldcs(entries + sm.kstart[j] + (p + u - sm.koff[j]));
        }
      }
    };
    // the plastic weights of a round's entries, and with STDP their posts'
    // traces and spike words
    auto gather = [&](const int (&jj)[RANGE_U], const uint2 (&en)[RANGE_U], float (&wv)[RANGE_U],
                      float (&ptv)[RANGE_U], uint32_t (&pw)[RANGE_U]) {
#pragma unroll
      for (int u = 0; u < RANGE_U; ++u) {
        wv[u] = ptv[u] = 0.0f;
        pw[u] = 0u;
        if (jj[u] >= 0 && (en[u].x >> 28) != 0u) {
          wv[u] = __uint_as_float(csc[en[u].y].y);
          if (st.stdp_run) {
            const int q = (int)(en[u].x & 0xffffu);
            ptv[u] = d.post_trace[p0 + q];
            pw[u] = d.bitsE[(KL + p0 + q) >> 5];  // post events
          }
        }
      }
    };
    int jj[RANGE_U];
    uint2 en[RANGE_U];
    float wv[RANGE_U], ptv[RANGE_U];
    uint32_t pw[RANGE_U];
    locate(0, jj, en);
    gather(jj, en, wv, ptv, pw);
    for (int rbase = 0; rbase < total; rbase += RANGE_ROUND) {
      ++epoch;
      int jn[RANGE_U];
      uint2 enn[RANGE_U];
      const bool more = rbase + RANGE_ROUND < total;
      if (more) {
        locate(rbase + RANGE_ROUND, jn, enn);  // the next round's entries in flight
      } else {
#pragma unroll
        for (int u = 0; u < RANGE_U; ++u) {
          jn[u] = -1;
          enn[u] = make_uint2(0u, 0u);
        }
      }
      uint32_t cell[RANGE_U], tagv[RANGE_U];
      float con[RANGE_U], val[RANGE_U];
      bool add[RANGE_U];
#pragma unroll
      for (int u = 0; u < RANGE_U; ++u) {
        add[u] = false;
        cell[u] = 0u;
        tagv[u] = 0u;
        con[u] = val[u] = 0.0f;
        if (jj[u] < 0) continue;
        const uint32_t flv = sm.list[jj[u]];
        const bool A = (flv >> 31) != 0;
        const bool P = ((flv >> 30) & 1u) != 0;
        const uint32_t x = en[u].x;
        const int q = (int)(x & 0xffffu);
        const int dl = (int)((x >> 16) & 0xffu);
        const int lb = (int)((x >> 24) & 0xfu);
        const int cl = (int)(x >> 28);
        float contrib;
        if (cl != 0) {
          float v = wv[u];
          if (st.stdp_run) {
            const bool post_ev = ((pw[u] >> ((KL + p0 + q) & 31)) & 1u) != 0;
            if (P || post_ev) {
              v = stdp_update(sc, v, P, post_ev, ptv[u], sm.kpre[jj[u]]);
              csc[en[u].y].y = __float_as_uint(v);
              ++n_pre;
            }
          }
          contrib = v * sm.scl[cl];
        } else {
          contrib = __uint_as_float(en[u].y);
        }
        if (A) {
          ++ev;
          const uint32_t dc = (uint32_t)((dl - 1) * slot_words + q * L + lb);
          const int r = tid * RANGE_U + u;
          add[u] = true;
          cell[u] = dc;
          con[u] = contrib;
          val[u] = rr.load(dc);
          tagv[u] = (epoch << RANGE_POS_BITS) | (uint32_t)r;
          sm.econ[r] = contrib;
          if (!direct) sm.ecell[r] = dc;
          const uint32_t h = direct ? dc : ((dc * 0x9E3779B1u) >> (32 - hbits));
          const uint32_t prev = atomicExch(&head[h], tagv[u]);
          sm.enxt[r] = (prev >> RANGE_POS_BITS) == epoch ? (unsigned short)(prev & ((1u << RANGE_POS_BITS) - 1))
                                                           : RANGE_NONE;
        }
      }
      __syncthreads();  // the round's chains are complete
#pragma unroll
      for (int u = 0; u < RANGE_U; ++u) {
        if (!add[u]) continue;
        const uint32_t h = direct ? cell[u] : ((cell[u] * 0x9E3779B1u) >> (32 - hbits));
        if (head[h] != tagv[u]) continue;
        const int r = tid * RANGE_U + u;
        const int dl = (int)(cell[u] / (uint32_t)slot_words) + 1;
        if (sm.enxt[r] == RANGE_NONE) {
          rr.store(cell[u], val[u] + con[u]);
        } else if (direct) {
          rr.store(cell[u], range_chain_sum(sm, r, val[u]));
        } else {
          range_apply_mixed_chain(sm, rr, r, cell[u], val[u]);
          dirty |= rr.ws ? (1u << rr.ws) - 1u : 0u;
        }
        if (dl <= rr.ws) dirty |= 1u << (dl - 1);
      }
      // the next round's plastic weights in flight across the barrier
      float wn[RANGE_U], ptn[RANGE_U];
      uint32_t pwn[RANGE_U];
      gather(jn, enn, wn, ptn, pwn);
      __syncthreads();  // the round's ring words are written
#pragma unroll
      for (int u = 0; u < RANGE_U; ++u) {
        jj[u] = jn[u];
        en[u] = enn[u];
        wv[u] = wn[u];
        ptv[u] = ptn[u];
        pw[u] = pwn[u];
      }
    }
  }
  // window slots written back, each as whole 16-byte words
  if (rr.ws) {
    dirty = __reduce_or_sync(FULL, dirty);
    if (lane == 0 && dirty) atomicOr(&s_dirty, dirty);
    __syncthreads();
    const unsigned dm = s_dirty;
    for (int k = 0; k < rr.ws; ++k) {
      if (!((dm >> k) & 1u)) continue;
      int sl = st.slot + 1 + k;
      if (sl >= B) sl -= B;
      float4* dst = (float4*)(ring + (size_t)sl * slot_words);
      const float4* src = (const float4*)(rwin + (size_t)k * slot_words);
      for (int i = tid; i < slot_words / 4; i += RANGE_THREADS) dst[i] = src[i];
    }
  }
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

}  // namespace spk
