// spk_net.cu - C ABI of the step engine (spike_gb300.h): network creation
// (planner + row-partitioned CSR builder), state management, launches.
//
// Compiled with -fmad=false (device) and -Xcompiler -ffp-contract=off (host):
// the few float constants derived here on the host (k = dt/tau_m, k*R, label
// decays, STDP trace constants, initial V) must round exactly as the oracle's.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/spike_gb300.h"
#include "spk_bulk.cuh"
#include "spk_gen.cuh"
#include "spk_range.cuh"
#include "spk_internal.h"
#include "spk_kernel.cuh"

namespace spk {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

#define SPK_CUDA(call)                                                              \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      ::spk::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                       __LINE__);                                                   \
      return SPK_ERR_CUDA;                                                          \
    }                                                                               \
  } while (0)


constexpr int DEFAULT_STEPS_PER_LAUNCH = 1000;
constexpr unsigned long long DEFAULT_WAIT_LIMIT_NS = 4000000000ull;  // 4 s
constexpr int64_t DEFAULT_SPIKE_CAPACITY = 1 << 24;

// Starts a run in the run control: the run that ended is folded into the
// state of the reference's active lists first (see RunCtl), and the new run
// notes whether its first group delivers the last group's spikes again (the
// step kernels do, group_repeats).
__device__ void start_run(RunCtl* ctl, int G, float dt, float start, int steps_total, int plastic,
                          int record_inputs) {
  RunCtl c = *ctl;
  fold_finished_run(c, G, dt);
  const int carry = carry_decision(c, G, dt, start, steps_total);
  if (steps_total > 0) c.repeat = carry != 0;
  // a list holding two groups: the reference delivers both, this engine has
  // kept only the last one
  if (carry == 2 && c.status == 0) c.status = SPK_ERR_UNSUPPORTED;
  c.start_time = start;
  c.step = 0;
  c.steps_total = steps_total;
  c.plastic = plastic;
  c.record_inputs = record_inputs;
  ctl->start_time = c.start_time;
  ctl->step = c.step;
  ctl->steps_total = c.steps_total;
  ctl->plastic = c.plastic;
  ctl->record_inputs = c.record_inputs;
  ctl->status = c.status;
  ctl->repeat = c.repeat;
  ctl->last_group_p1 = c.last_group_p1;
  ctl->last_run_groups = c.last_run_groups;
  ctl->last_run_repeat = c.last_run_repeat;
}

static __global__ void set_ctl_kernel(RunCtl* ctl, int G, float dt, float start, int steps_total, int plastic,
                                      int record_inputs) {
  start_run(ctl, G, dt, start, steps_total, plastic, record_inputs);
}

static __global__ void clear_store_kernel(RunCtl* ctl) {
  ctl->spike_count = 0ull;
  if (ctl->status == SPK_ERR_OVERFLOW) ctl->status = 0;
}

static __global__ void reset_inputs_kernel(NetDev* nd, const float* rates, int Nin) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    nd->rates = rates;
    nd->ctl->inputs_active = 0;
  }
  if (i < Nin) nd->in_next[i] = -1000.0f;
}

struct DeviceInfo {
  int sms = 0;
  int max_smem = 0;
};

static int device_info(DeviceInfo* di) {
  int dev = 0;
  SPK_CUDA(cudaGetDevice(&dev));
  SPK_CUDA(cudaDeviceGetAttribute(&di->sms, cudaDevAttrMultiProcessorCount, dev));
  SPK_CUDA(cudaDeviceGetAttribute(&di->max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  // the dynamic shared-memory limit excludes the kernel's static shared memory
  cudaFuncAttributes fa;
  SPK_CUDA(cudaFuncGetAttributes(&fa, step_kernel));
  di->max_smem -= (int)fa.sharedSizeBytes;
  return SPK_OK;
}

// The maximum dynamic shared memory of a kernel function holds in the whole
// process, not for one batch: every batch sets the device's limit (less the
// kernel's static shared memory), so that none lowers another's.  *limit gets
// the smallest limit of the kernels set so far.
template <typename K>
static int allow_all_dynamic_smem(K kernel, int* limit) {
  int dev = 0, optin = 0;
  SPK_CUDA(cudaGetDevice(&dev));
  SPK_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  SPK_CUDA(cudaFuncGetAttributes(&fa, kernel));
  const int dyn = optin - (int)fa.sharedSizeBytes;
  SPK_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  *limit = *limit ? std::min(*limit, dyn) : dyn;
  return SPK_OK;
}

// A launch that may begin while the stream's previous kernel drains (the
// kernel waits for it with griddepcontrol.wait before touching its outputs).
template <typename... P, typename... A>
static cudaError_t launch_overlapped(void (*k)(P...), int grid, int block, size_t smem, cudaStream_t st,
                                     A... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

struct Plan {
  int W, TS, ITS, nctas, n_tiles, KL, n_keys, n_words, K, smem;
  // The persistent step kernel can run the plan (its shared memory fits and
  // its CTAs fit one cooperative launch).  A plan of range tiles (an explicit
  // schedule with tiles of RANGE_MIN_TS posts or more whose tile does not fit
  // a warp's shared memory) runs in bulk mode only.
  bool persistent;
};

static int plan_bytes(int B, int TS, int L, int ITS, int kind, int stdp, int W) {
  return smem_bytes(W, warp_layout(B, TS, L, ITS, kind, stdp));
}

// Choose warps per CTA, tile size and CTA count for one network.  Small
// networks run on one CTA (no inter-CTA barrier); larger ones spread tiles of
// 64-256 posts over up to one CTA per SM.  Explicit schedule fields override.
static int make_plan(int N, int Nin, int B, int L, int kind, int stdp, const spk_schedule* s,
                     const DeviceInfo& di, Plan* p) {
  auto finish = [&](int W, int TS, int nctas, bool allow_bulk = false) {
    p->W = W;
    p->TS = TS;
    p->nctas = nctas;
    p->n_tiles = W * nctas;
    p->ITS = Nin > 0 ? ((Nin + p->n_tiles - 1) / p->n_tiles + 31) / 32 * 32 : 0;
    p->KL = p->n_tiles * p->ITS;
    p->n_keys = p->KL + p->n_tiles * TS;
    p->n_words = p->n_keys / 32;
    p->smem = plan_bytes(B, TS, L, p->ITS, kind, stdp, W);
    // per-CTA key counts travel in 16-bit fields of the stamp word
    p->persistent = p->smem <= di.max_smem && nctas <= MAX_CTAS_PER_NET && W * TS <= 65535 && W * p->ITS <= 65535;
    // keys travel in 29 bits (list words carry three flags)
    const bool covers = (int64_t)p->n_tiles * TS >= N && (int64_t)p->n_keys < (1ll << 29);
    return covers && (p->persistent || (allow_bulk && TS >= RANGE_MIN_TS));
  };
  const int K = (s && s->steps_per_launch > 0) ? s->steps_per_launch : DEFAULT_STEPS_PER_LAUNCH;
  p->K = K;
  const int Wreq = (s && s->warps_per_cta > 0) ? s->warps_per_cta : 0;
  const int TSreq = (s && s->tile_posts > 0) ? s->tile_posts : 0;
  const int Creq = (s && s->ctas > 0) ? s->ctas : 0;
  if (Wreq > 16 || (TSreq && (TSreq % 32 || TSreq > 65504))) {
    set_error("schedule: warps_per_cta must be <= 16 and tile_posts a multiple of 32 below 65536");
    return SPK_ERR_INVALID;
  }
  if (Wreq || TSreq || Creq) {
    const int W = Wreq ? Wreq : 8;
    int TS = TSreq, C = Creq;
    if (!TS && C) TS = std::max(32, ((N + W * C - 1) / (W * C) + 31) / 32 * 32);
    if (!TS) TS = 64;
    if (!C) C = (N + W * TS - 1) / (W * TS);
    if (!finish(W, TS, C, true)) {
      set_error("schedule W=%d tile=%d ctas=%d does not cover %d neurons within %d B of shared memory (needs %d)",
                W, TS, C, N, di.max_smem, p->smem);
      return SPK_ERR_INVALID;
    }
    return SPK_OK;
  }
  // The step is latency-bound: the smallest tiles (most warps working in
  // parallel) win while the CTAs fit one per SM.
  if (N <= 16 * 32) {
    const int W = (N + 31) / 32;
    if (finish(W, 32, 1)) return SPK_OK;
  }
  const int W = 8;
  for (int TS : {32, 64, 96, 128, 160, 192, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096}) {
    int C = (N + W * TS - 1) / (W * TS);
    if (C > di.sms) continue;
    if (finish(W, TS, C)) return SPK_OK;
  }
  for (int Wt : {4, 2, 1})
    for (int TS = 32; TS <= 65504; TS *= 2) {
      int C = (N + Wt * TS - 1) / (Wt * TS);
      if (C > di.sms) continue;
      if (finish(Wt, TS, C)) return SPK_OK;
    }
  set_error("no schedule fits %d neurons with ring depth %d and %d labels", N, B, L);
  return SPK_ERR_UNSUPPORTED;
}

}  // namespace spk

using namespace spk;

struct spk_net {
  // model
  int N = 0, Nin = 0, L = 1, B = 0, kind = 0, n_stim = 0, stim = 0;
  int G = 1;  // timestep grouping: runs advance whole groups of G timesteps
  int64_t S = 0;
  float dt = 0.f;
  bool has_stdp = false, record_inputs = false;
  uint64_t seed = 0;
  std::vector<spk_neuron_group> groups;
  std::vector<float> weights;      // creation order (host mirror)
  std::vector<float> scales;       // creation order
  std::vector<int32_t> entry_of;   // creation index -> entry index
  std::vector<int32_t> csc_of;     // creation index -> afferent record (plastic synapses)
  std::vector<uint8_t> cls_of;     // creation index -> scale class
  std::vector<float> scale_tab;
  Plan plan{};
  // device
  void* arena = nullptr;
  size_t arena_bytes = 0;
  NetDev hd{};             // host copy of the device descriptor
  NetDev* dd = nullptr;    // device descriptor
  CtaMap* dmap = nullptr;
  float* rates_dev = nullptr;
  int* abort_dev = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  bool cooperative = false;
  int64_t launches = 0;
  float current_time = 0.0f;
  int pending_status = SPK_OK;
  bool generated = false;  // connectivity drawn on the device (no host synapse arrays)
  int withhold = -1;       // fault injection: CTA rank left out of the next launch
  int stdp_rule = SPK_STDP_WEIGHT_DEPENDENT;
  spk_batch* self_batch = nullptr;  // runs of a network with a per-synapse-trace rule (bulk mode)
  bool dense() const { return has_stdp && stdp_rule != SPK_STDP_WEIGHT_DEPENDENT; }
  int weight_norm = SPK_NORM_OFF;   // SPK_NORM_* (with an STDP rule only)
  std::vector<float> norm_w0_h;     // per plastic record: initial weight
  std::vector<float> norm_sum_h;    // per post: sum of squares
  // Runs in bulk mode only: a per-synapse-trace rule, the weight normalisation,
  // or range tiles (a plan the persistent kernel cannot run).
  bool bulk_only() const { return dense() || weight_norm != SPK_NORM_OFF || !plan.persistent; }
  // The normalisation's place in a bulk timestep: 0 before the rule, 1 after
  // the per-synapse-trace pass, 2 after the event-driven rule's updates (a
  // first propagation pass that only updates weights, and the afferent pass).
  int norm_slot() const {
    if (weight_norm == SPK_NORM_BEFORE_RULE) return 0;
    return dense() ? 1 : 2;
  }
  int64_t n_csc = 0;       // plastic afferent records
  float step_cost = 0.0f;  // measured or estimated time of one step alone (batch packing)
};

namespace spk {
struct KernelTimer;
}

struct spk_batch {
  struct Wave {
    int first;  // first CTA-map entry of the wave
    int ctas;   // CTAs of the wave (all co-resident)
    int smem;   // dynamic shared memory of the wave's launch
    bool cooperative;
  };
  std::vector<spk_net*> nets;
  NetDev* dd = nullptr;
  CtaMap* dmap = nullptr;
  int* abort_dev = nullptr;
  std::vector<Wave> waves;
  int W = 0, K = 0, total_ctas = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;  // recorded after each run; the networks' streams wait on it
  int64_t launches = 0;
  // bulk-synchronous mode (spk_bulk.cuh)
  int mode = SPK_BATCH_WAVES;
  std::vector<NetDev> hds;       // host copies of the batch's descriptors
  BulkPropBlock* dpblocks = nullptr;  // [pblocks_total] propagation tile groups
  int pblocks_total = 0;
  BulkRangeBlock* drblocks = nullptr; // [rblocks_total] propagation ranges (networks of range tiles)
  int rblocks_total = 0;
  RangeSmem range_smem{0, 0};         // ring window and bucket heads of a propagation range
  // per-kernel timing (spk_batch_time_kernels): blocks go direct, each kernel
  // between two events, and the intervals are added to timer_ms
  spk::KernelTimer* timer = nullptr;
  double* timer_ms = nullptr;
  BulkBlock* dblocks = nullptr;  // [blocks_total] blocks of 32-key words with real keys
  int blocks_total = 0;
  BulkPostItem* items = nullptr; // afferent-pass work list of a timestep
  BulkRuleItem* dense_items = nullptr;  // posts with plastic afferents of the per-synapse-trace-rule
                                        // and normalised networks
  int n_dense_items = 0;
  bool any_dense = false;       // a network with a per-synapse-trace rule
  int norm_slots = 0;           // bit k: a network normalises its weights in slot k (spk_net::norm_slot)
  int step_launches = 0;        // kernels of one bulk timestep
  int* item_count = nullptr;
  int item_cap = 0;
  bool any_plastic = false;
  int win_words = 0;            // ring-window words per propagation warp
  int ts_max = 0;               // largest post tile of the batch
  void* bulk_mem = nullptr;      // tiles, step lists and counts
  cudaGraphExec_t bulk_graph = nullptr;  // one block of K timesteps
  // The afferent pass runs beside the propagation kernel (they update
  // disjoint weights: afferents with and without a presynaptic event).
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  // spike readback of the whole batch (spk_batch_read_spikes)
  cudaEvent_t rd = nullptr;
  void* rb_mem = nullptr;       // counts, chunk list, chunk matches
  size_t rb_bytes = 0;
  int32_t* rb_ids = nullptr;    // gathered spikes
  float* rb_times = nullptr;
  int64_t rb_cap = 0;
};

namespace spk {

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

static int upload_state_defaults(spk_net* n) {
  // SpikingModel::reset_state: V := V0 (or the V-init extension), last := -1000
  // (Spike/Backend/CUDA/Neurons/SpikingNeurons.cu:68-94), ring and traces := 0
  // (SpikingSynapses.cu:28-35, ConductanceSpikingSynapses.cu:49-56),
  // inputs inactive (PoissonInputSpikingNeurons.cu:27-34), STDP traces := 0.
  const NetDev& h = n->hd;
  std::vector<float> V(n->N), last(n->N, -1000.0f);
  for (const auto& g : n->groups)
    for (int i = g.start; i < g.start + g.count; ++i) {
      if (g.v_init_lo < g.v_init_hi) {
        const float u = draw_uniform(n->seed, (uint32_t)i, 0u, DOMAIN_VINIT);
        const float span = g.v_init_hi - g.v_init_lo;
        V[i] = g.v_init_lo + span * u;
      } else {
        V[i] = g.v0;
      }
    }
  SPK_CUDA(cudaMemcpyAsync(h.V, V.data(), sizeof(float) * n->N, cudaMemcpyHostToDevice, n->stream));
  SPK_CUDA(cudaMemcpyAsync(h.last, last.data(), sizeof(float) * n->N, cudaMemcpyHostToDevice, n->stream));
  SPK_CUDA(cudaMemsetAsync(h.gtr, 0, sizeof(float) * (size_t)n->N * n->L, n->stream));
  SPK_CUDA(cudaMemsetAsync(h.ring, 0, sizeof(float) * (size_t)h.n_tiles * h.B * h.TS * h.L, n->stream));
  // RateActivityMonitor::reset_state (Spike/Backend/CUDA/ActivityMonitor/RateActivityMonitor.cu:12-16)
  if (h.rate_counts) SPK_CUDA(cudaMemsetAsync(h.rate_counts, 0, sizeof(int) * (size_t)h.n_keys, n->stream));
  // per-synapse traces := 0 (EvansSTDPPlasticity.cpp:21-26, InhibitorySTDPPlasticity.cu:13-28)
  // and the spike-bit history cleared
  if (h.dense_tr) SPK_CUDA(cudaMemsetAsync(h.dense_tr, 0, sizeof(float2) * (size_t)n->n_csc, n->stream));
  if (h.hist) SPK_CUDA(cudaMemsetAsync(h.hist, 0, sizeof(uint32_t) * (size_t)h.H * h.n_words, n->stream));
  if (n->has_stdp) {
    SPK_CUDA(cudaMemsetAsync(h.post_trace, 0, sizeof(float) * n->N, n->stream));
    SPK_CUDA(cudaMemsetAsync(h.pre_trace, 0, sizeof(float) * h.n_keys, n->stream));
    SPK_CUDA(cudaMemsetAsync(h.pre_pub, 0, sizeof(float) * 2 * (size_t)h.n_keys, n->stream));
  }
  // a run that ended on a timeout leaves the abort flag, the status and the
  // aborted step's exchange words behind: clear them
  SPK_CUDA(cudaMemsetAsync(n->abort_dev, 0, sizeof(int), n->stream));
  SPK_CUDA(cudaMemsetAsync(&h.ctl->status, 0, sizeof(int), n->stream));
  // SpikingSynapses::reset_state empties both active lists (SpikingSynapses.cu:33)
  SPK_CUDA(cudaMemsetAsync(&h.ctl->step, 0, sizeof(int), n->stream));
  SPK_CUDA(cudaMemsetAsync(&h.ctl->repeat, 0, 4 * sizeof(int), n->stream));
  SPK_CUDA(cudaMemsetAsync(h.gbits, 0, sizeof(uint32_t) * (size_t)n->G * h.n_words, n->stream));
  SPK_CUDA(cudaMemsetAsync(h.cta_stamp, 0, sizeof(unsigned long long) * 2 * (size_t)h.nctas, n->stream));
  SPK_CUDA(cudaMemsetAsync(h.cta_keys, 0, sizeof(unsigned long long) * 2 * (size_t)h.nctas * h.key_cap, n->stream));
  if (n->Nin > 0) {
    reset_inputs_kernel<<<(n->Nin + 255) / 256, 256, 0, n->stream>>>(n->dd, n->rates_dev + (size_t)n->stim * n->Nin, n->Nin);
    SPK_CUDA(cudaGetLastError());
  } else {
    int zero = 0;
    SPK_CUDA(cudaMemcpyAsync(&h.ctl->inputs_active, &zero, sizeof(int), cudaMemcpyHostToDevice, n->stream));
    SPK_CUDA(cudaStreamSynchronize(n->stream));
  }
  return SPK_OK;
}

// Starts a run of the network on `stream` (start_run in its run control).
static int begin_run_on(spk_net* n, cudaStream_t stream, float start, int64_t steps, int plastic) {
  set_ctl_kernel<<<1, 1, 0, stream>>>(n->hd.ctl, n->G, n->dt, start, (int)steps, plastic, n->record_inputs ? 1 : 0);
  SPK_CUDA(cudaGetLastError());
  return SPK_OK;
}

static int launch_block(spk_net* n) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(n->plan.nctas);
  cfg.blockDim = dim3(n->plan.W * 32);
  cfg.dynamicSmemBytes = n->plan.smem;
  cfg.stream = n->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = n->cooperative ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  SPK_CUDA(cudaLaunchKernelEx(&cfg, step_kernel, (const NetDev*)n->dd, (const CtaMap*)n->dmap,
                              n->plan.K));
  return SPK_OK;
}

static int build_graph(spk_net* n) {
  cudaGraph_t g = nullptr;
  SPK_CUDA(cudaStreamBeginCapture(n->stream, cudaStreamCaptureModeThreadLocal));
  int rc = launch_block(n);
  cudaError_t e = cudaStreamEndCapture(n->stream, &g);
  if (rc != SPK_OK || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    n->graph = nullptr;
    return SPK_OK;  // launches go direct
  }
  e = cudaGraphInstantiate(&n->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();
    n->graph = nullptr;
  }
  return SPK_OK;
}

static int run_steps_impl(spk_net* n, int64_t steps, int plastic, float start) {
  if (steps <= 0) return SPK_OK;
  if (steps > 0x7fffffff) {
    set_error("run of %lld steps exceeds the 2^31-1 step limit of one run", (long long)steps);
    return SPK_ERR_INVALID;
  }
  if (n->bulk_only()) {
    // Per-synapse-trace STDP and the weight normalisation run in bulk mode: a batch of this one network
    // (the caller sets the network's time afterwards, as for any run).
    if (!n->self_batch) {
      const spk_schedule bs{0, 0, 0, n->plan.K};
      int rc = spk_batch_create(&n, 1, &bs, &n->self_batch);
      if (rc) return rc;
    }
    n->current_time = start;
    const int64_t each = steps;
    const int32_t pl = plastic ? 1 : 0;
    return spk_batch_run_steps_each(n->self_batch, &each, &pl);
  }
  {
    const int rc = begin_run_on(n, n->stream, start, steps, (plastic && n->has_stdp) ? 1 : 0);
    if (rc) return rc;
  }
  const int64_t blocks = (steps + n->plan.K - 1) / n->plan.K;
  for (int64_t b = 0; b < blocks; ++b) {
    if (n->withhold >= 0) {
      // the launch leaves one CTA out: the others' waits on it run out
      std::vector<CtaMap> map;
      for (int r = 0; r < n->plan.nctas; ++r)
        if (r != n->withhold) map.push_back(CtaMap{0, r});
      n->withhold = -1;
      SPK_CUDA(cudaMemcpyAsync(n->dmap, map.data(), sizeof(CtaMap) * map.size(), cudaMemcpyHostToDevice, n->stream));
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)map.size());
      cfg.blockDim = dim3(n->plan.W * 32);
      cfg.dynamicSmemBytes = n->plan.smem;
      cfg.stream = n->stream;
      SPK_CUDA(cudaLaunchKernelEx(&cfg, step_kernel, (const NetDev*)n->dd, (const CtaMap*)n->dmap, n->plan.K));
      SPK_CUDA(cudaStreamSynchronize(n->stream));
      map.clear();
      for (int r = 0; r < n->plan.nctas; ++r) map.push_back(CtaMap{0, r});
      SPK_CUDA(cudaMemcpy(n->dmap, map.data(), sizeof(CtaMap) * map.size(), cudaMemcpyHostToDevice));
      ++n->launches;
      continue;
    }
    if (n->graph) {
      SPK_CUDA(cudaGraphLaunch(n->graph, n->stream));
    } else {
      int rc = launch_block(n);
      if (rc) return rc;
    }
    ++n->launches;
  }
  return SPK_OK;
}

static int read_status(spk_net* n, int* status) {
  SPK_CUDA(cudaStreamSynchronize(n->stream));
  int st = 0;
  SPK_CUDA(cudaMemcpy(&st, &n->hd.ctl->status, sizeof(int), cudaMemcpyDeviceToHost));
  *status = st;
  return SPK_OK;
}

template <typename F>
static int guarded(F&& f) {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    set_error("host allocation failed");
    return SPK_ERR_OOM;
  }
}

// Model constants shared by networks built from synapse arrays and networks
// generated on the device.
struct ModelSpec {
  float dt = 0.f;
  int kind = 0, N = 0, Nin = 0, L = 1;
  int n_groups = 0;
  const spk_neuron_group* groups = nullptr;
  float t_ref = 0.f, i_bg = 0.f;
  int n_stim = 0, stim = 0;
  const float* rates = nullptr;
  const float* label_tau = nullptr;
  const float* label_vhat = nullptr;
  int has_stdp = 0;
  spk_stdp_params stdp{};
  int stdp_rule = SPK_STDP_WEIGHT_DEPENDENT;
  int weight_norm = SPK_NORM_OFF;
  const float* norm_initial = nullptr;
  const float* norm_sum = nullptr;
  uint64_t seed = 0;
  int64_t spike_capacity = 0;
  int record_inputs = 0;
  int G = 1;  // timestep grouping: the minimum delay in steps (Spike/Models/SpikingModel.cpp:98)
};

// The time constants the step divides by (k = dt / tau_m, the label decays,
// the STDP trace decays) must be positive and the refractory period finite and
// non-negative: zero or negative values would give the run inf/NaN constants.
// Grouped timesteps change the plasticity rules' arithmetic (one update per
// group, with traces decayed over G steps:
// Spike/Backend/CUDA/Plasticity/WeightDependentSTDPPlasticity.cu:125-145),
// which this engine does not restate: a network with a rule needs G = 1.
static int check_grouping(const ModelSpec& m) {
  if (m.G > 1 && m.has_stdp) {
    set_error("minimum delay %d steps (timestep grouping %d) with a plasticity rule is not supported", m.G, m.G);
    return SPK_ERR_UNSUPPORTED;
  }
  return SPK_OK;
}

static int check_time_constants(float dt, const spk_neuron_group* groups, int n_groups, int kind, int L,
                                const float* label_tau, float refractory, bool has_stdp, const spk_stdp_params& sp) {
  for (int g = 0; g < n_groups; ++g)
    if (!(groups[g].tau_m > 0.0f) || !std::isfinite(groups[g].tau_m)) {
      set_error("group %d: tau_m %g must be positive", g, (double)groups[g].tau_m);
      return SPK_ERR_INVALID;
    }
  if (kind != SPK_SYN_VOLTAGE)
    for (int l = 0; l < L; ++l)
      if (!(label_tau[l] > 0.0f) || !std::isfinite(label_tau[l])) {
        set_error("label %d: tau %g must be positive", l, (double)label_tau[l]);
        return SPK_ERR_INVALID;
      }
  if (!(refractory >= 0.0f) || !std::isfinite(refractory)) {
    set_error("refractory period %g must be finite and non-negative", (double)refractory);
    return SPK_ERR_INVALID;
  }
  if (has_stdp && (!(sp.tau_plus > 0.0f) || !(sp.tau_minus > 0.0f) || !std::isfinite(sp.tau_plus) ||
                   !std::isfinite(sp.tau_minus))) {
    set_error("STDP tau_plus %g and tau_minus %g must be positive", (double)sp.tau_plus, (double)sp.tau_minus);
    return SPK_ERR_INVALID;
  }
  (void)dt;
  return SPK_OK;
}

static int validate_spec(const ModelSpec& m) {
  if (m.stdp_rule < SPK_STDP_WEIGHT_DEPENDENT || m.stdp_rule > SPK_STDP_CUSTOM) {
    set_error("unknown STDP rule %d", m.stdp_rule);
    return SPK_ERR_INVALID;
  }
  if (m.weight_norm < SPK_NORM_OFF || m.weight_norm > SPK_NORM_BEFORE_RULE) {
    set_error("unknown weight normalisation mode %d", m.weight_norm);
    return SPK_ERR_INVALID;
  }
  if (m.weight_norm != SPK_NORM_OFF && !m.has_stdp) {
    set_error("the weight normalisation acts on the plastic synapses of an STDP rule");
    return SPK_ERR_INVALID;
  }
  if (m.N <= 0 || m.Nin < 0 || m.L < 1 || m.L > MAX_LABELS || !(m.dt > 0.0f)) {
    set_error("sizes out of range (neurons %d, inputs %d, labels %d)", m.N, m.Nin, m.L);
    return SPK_ERR_INVALID;
  }
  if (m.kind != SPK_SYN_CONDUCTANCE && m.kind != SPK_SYN_CURRENT && m.kind != SPK_SYN_VOLTAGE) {
    set_error("unknown synapse kind %d", m.kind);
    return SPK_ERR_INVALID;
  }
  if (m.n_groups < 1 || m.n_groups > MAX_GROUPS || !m.groups) {
    set_error("between 1 and %d neuron groups are supported (got %d)", MAX_GROUPS, m.n_groups);
    return m.n_groups > MAX_GROUPS ? SPK_ERR_UNSUPPORTED : SPK_ERR_INVALID;
  }
  int expect = 0;
  for (int g = 0; g < m.n_groups; ++g) {
    if (m.groups[g].start != expect || m.groups[g].count <= 0) {
      set_error("neuron groups must be contiguous, ascending and non-empty");
      return SPK_ERR_INVALID;
    }
    expect += m.groups[g].count;
  }
  if (expect != m.N) {
    set_error("neuron groups cover %d neurons, descriptor says %d", expect, m.N);
    return SPK_ERR_INVALID;
  }
  if (m.Nin > 0 && (m.n_stim < 1 || !m.rates || m.stim < 0 || m.stim >= m.n_stim)) {
    set_error("inputs need rates and a valid stimulus");
    return SPK_ERR_INVALID;
  }
  if (m.kind != SPK_SYN_VOLTAGE && !m.label_tau) {
    set_error("conductance/current synapses need label_tau");
    return SPK_ERR_INVALID;
  }
  if (m.kind == SPK_SYN_CONDUCTANCE && !m.label_vhat) {
    set_error("conductance synapses need label_vhat");
    return SPK_ERR_INVALID;
  }
  return check_time_constants(m.dt, m.groups, m.n_groups, m.kind, m.L, m.label_tau, m.t_ref, m.has_stdp, m.stdp);
}

// A new handle with the model fields of `m` and a plan for ring depth B.
static int new_net(const ModelSpec& m, int B, int64_t S, const spk_schedule* sched, spk_net** out) {
  DeviceInfo di;
  int rc = device_info(&di);
  if (rc) return rc;
  Plan plan;
  rc = make_plan(m.N, m.Nin, B, m.L, m.kind, m.has_stdp ? 1 : 0, sched, di, &plan);
  if (rc) return rc;
  spk_net* n = new spk_net();
  n->N = m.N;
  n->Nin = m.Nin;
  n->L = m.L;
  n->B = B;
  n->G = m.G;
  n->kind = m.kind;
  n->S = S;
  n->dt = m.dt;
  n->has_stdp = m.has_stdp != 0;
  n->stdp_rule = m.stdp_rule;
  n->weight_norm = m.has_stdp ? m.weight_norm : SPK_NORM_OFF;
  n->record_inputs = m.record_inputs != 0;
  n->seed = m.seed;
  n->n_stim = m.Nin > 0 ? m.n_stim : 0;
  n->stim = m.Nin > 0 ? m.stim : 0;
  n->groups.assign(m.groups, m.groups + m.n_groups);
  n->plan = plan;
  n->scale_tab.assign(MAX_CLASSES, 0.0f);
  *out = n;
  return SPK_OK;
}

// Bytes of each part of a network's device arena, in arena order: rowptr,
// entries, csc_ptr, csc, V, last, traces, ring, input next, rates, post
// traces, pre traces, pre-trace mailbox, spike and pre-event bitmaps, CTA key
// lists and stamps, spike store, run control, abort flag, descriptor, CTA map,
// rate-monitor counts, and for per-synapse-trace STDP rules the afferent
// records' delays, their traces and the spike-word history.
static std::vector<size_t> arena_part_sizes(const Plan& plan, int N, int Nin, int L, int B, int stdp, int64_t S,
                                            int64_t n_csc, int n_stim, int64_t spike_cap, int dense = 0,
                                            int norm = 0, int G = 1) {
  const size_t n_cells = (size_t)plan.n_keys * plan.n_tiles;
  const size_t key_cap = (size_t)plan.W * (plan.TS + plan.ITS);
  return {sizeof(int32_t) * (n_cells + 1),
          sizeof(uint2) * (size_t)std::max<int64_t>(S, 1),
          sizeof(int32_t) * (stdp ? (size_t)N + 1 : 0),
          sizeof(uint2) * (size_t)n_csc,
          sizeof(float) * N,
          sizeof(float) * N,
          sizeof(float) * (size_t)N * L,
          sizeof(float) * (size_t)plan.n_tiles * B * plan.TS * L,
          sizeof(float) * std::max(Nin, 1),
          sizeof(float) * std::max<size_t>((size_t)n_stim * Nin, 1),
          sizeof(float) * (stdp ? N : 0),
          sizeof(float) * (stdp ? plan.n_keys : 0),
          sizeof(float) * (stdp ? 2 * (size_t)plan.n_keys : 0),
          sizeof(uint32_t) * 2 * (size_t)plan.n_words,
          sizeof(uint32_t) * 2 * (size_t)plan.n_words,
          sizeof(unsigned long long) * 2 * (size_t)plan.nctas * key_cap,
          sizeof(unsigned long long) * 2 * (size_t)plan.nctas,
          sizeof(uint2) * (size_t)std::max<int64_t>(spike_cap, 1),
          sizeof(RunCtl),
          sizeof(int),
          sizeof(NetDev),
          sizeof(CtaMap) * plan.nctas,
          sizeof(int) * (size_t)plan.n_keys,
          sizeof(int32_t) * (dense ? (size_t)n_csc : 0),
          sizeof(float) * (dense ? 2 * (size_t)n_csc : 0),
          sizeof(uint32_t) * (dense ? (size_t)(B - 2) * plan.n_words : 0),
          sizeof(float) * (norm ? (size_t)n_csc : 0),
          sizeof(float) * (norm ? (size_t)N : 0),
          sizeof(uint32_t) * (size_t)G * plan.n_words,
          sizeof(uint32_t) * (size_t)plan.n_words};
}

static size_t arena_total(const std::vector<size_t>& sizes) {
  size_t total = 0;
  for (size_t b : sizes) total = align_up(total, 256) + align_up(std::max<size_t>(b, 4), 256);
  return total;
}

// Allocates the device arena of `n` (CSR parts sized by S and n_csc), creates
// its stream, fills and uploads the device descriptor, uploads whichever host
// CSR arrays are given (generated networks pass none and fill them on the
// device afterwards), clears the exchange, checks co-residency and resets the
// state.  On failure `n` is destroyed.
static int setup_device(spk_net* n, const ModelSpec& m, int64_t n_csc, const int32_t* rowptr_h,
                        const uint2* entries_h, const int32_t* csc_ptr_h, const uint2* csc_h,
                        const int32_t* csc_delay_h = nullptr) {
  DeviceInfo di;
  int rc = device_info(&di);
  if (rc) {
    delete n;
    return rc;
  }
  const Plan& plan = n->plan;
  const int N = n->N, Nin = n->Nin, L = n->L, B = n->B;
  const int stdp = n->has_stdp ? 1 : 0;
  const int64_t S = n->S;
  n->n_csc = n_csc;
  const int n_tiles = plan.n_tiles, TS = plan.TS, KL = plan.KL, n_keys = plan.n_keys;
  const size_t n_cells = (size_t)n_keys * n_tiles;
  const int n_words = plan.n_words;
  const int64_t spike_cap = m.spike_capacity == 0 ? DEFAULT_SPIKE_CAPACITY : std::max<int64_t>(0, m.spike_capacity);
  struct Part {
    void** dst;
    size_t bytes;
  };
  NetDev& h = n->hd;
  std::memset(&h, 0, sizeof(h));
  void* p_rowptr = nullptr; void* p_entries = nullptr; void* p_cscptr = nullptr; void* p_csc = nullptr;
  void* p_V = nullptr; void* p_last = nullptr; void* p_gtr = nullptr; void* p_ring = nullptr;
  void* p_innext = nullptr; void* p_rates = nullptr; void* p_post = nullptr; void* p_pre = nullptr;
  void* p_pub = nullptr; void* p_bA = nullptr; void* p_bP = nullptr; void* p_spk = nullptr;
  void* p_ckeys = nullptr; void* p_cstamp = nullptr;
  const int key_cap = plan.W * (plan.TS + plan.ITS);
  void* p_ctl = nullptr; void* p_abort = nullptr; void* p_dd = nullptr; void* p_map = nullptr;
  void* p_rate = nullptr; void* p_cdelay = nullptr; void* p_dtr = nullptr; void* p_hist = nullptr;
  void* p_nw0 = nullptr; void* p_nsum = nullptr; void* p_gbits = nullptr; void* p_bE = nullptr;
  const int dense = n->dense() ? 1 : 0;
  const int norm = n->weight_norm != SPK_NORM_OFF ? 1 : 0;
  const std::vector<size_t> sizes =
      arena_part_sizes(plan, N, Nin, L, B, stdp, S, n_csc, n->n_stim, spike_cap, dense, norm, n->G);
  void** dsts[] = {&p_rowptr, &p_entries, &p_cscptr, &p_csc,   &p_V,     &p_last,   &p_gtr,  &p_ring,
                   &p_innext, &p_rates,   &p_post,   &p_pre,   &p_pub,   &p_bA,     &p_bP,   &p_ckeys,
                   &p_cstamp, &p_spk,     &p_ctl,    &p_abort, &p_dd,    &p_map,  &p_rate,
                   &p_cdelay, &p_dtr,     &p_hist,   &p_nw0,   &p_nsum,  &p_gbits, &p_bE};
  std::vector<Part> parts;
  for (size_t i = 0; i < sizes.size(); ++i) parts.push_back(Part{dsts[i], sizes[i]});
  const size_t total = arena_total(sizes);
  cudaError_t e = cudaMalloc(&n->arena, total);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("device allocation of %zu bytes failed: %s", total, cudaGetErrorString(e));
    delete n;
    return SPK_ERR_OOM;
  }
  n->arena_bytes = total;
  {
    size_t off = 0;
    for (auto& p : parts) {
      off = align_up(off, 256);
      *p.dst = (char*)n->arena + off;
      off += align_up(std::max<size_t>(p.bytes, 4), 256);
    }
  }
  auto fail_free = [&](int code) {
    if (n->stream) cudaStreamDestroy(n->stream);
    cudaFree(n->arena);
    delete n;
    return code;
  };
  if (cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("cudaStreamCreate failed");
    return fail_free(SPK_ERR_CUDA);
  }

  // ---- device descriptor ---------------------------------------------------------
  h.N = N;
  h.Nin = Nin;
  h.KL = KL;
  h.n_keys = n_keys;
  h.n_words = n_words;
  h.L = L;
  h.B = B;
  h.kind = m.kind;
  h.n_tiles = n_tiles;
  h.TS = TS;
  h.ITS = plan.ITS;
  h.W = plan.W;
  h.nctas = plan.nctas;
  h.n_groups = m.n_groups;
  h.dt = m.dt;
  h.half_dt = 0.5f * m.dt;
  h.G = n->G;
  h.t_ref = m.t_ref;
  h.i_bg = m.i_bg;
  for (int g = 0; g < m.n_groups; ++g) {
    const spk_neuron_group& G = m.groups[g];
    GroupConst& c = h.groups[g];
    c.start = G.start;
    c.end = G.start + G.count;
    // LIFSpikingNeurons.cu:31-44: k = timestep / tau_m, kR = k * R (host float).
    c.k = m.dt / G.tau_m;
    c.kR = c.k * G.R;
    c.v0 = G.v0;
    c.vreset = G.vreset;
    c.theta = G.theta;
  }
  for (int l = 0; l < L; ++l) {
    // ConductanceSpikingSynapses.cu:76-78: expf(-timestep / tau_g) on the host.
    h.decay[l] = m.kind == SPK_SYN_VOLTAGE ? 0.0f : expf(-m.dt / m.label_tau[l]);
    h.vhat[l] = m.kind == SPK_SYN_CONDUCTANCE ? m.label_vhat[l] : 0.0f;
  }
  for (int c = 0; c < MAX_CLASSES; ++c) h.scale_tab[c] = n->scale_tab[c];
  h.has_stdp = stdp;
  if (stdp) {
    const spk_stdp_params& sp = m.stdp;
    // WeightDependentSTDPPlasticity.cu:125-145 for G = 1 (see stdp_update).
    const float em = expf(-(1.0f * m.dt) / sp.tau_minus);
    const float ep = expf(-(1.0f * m.dt) / sp.tau_plus);
    h.E_m = em;
    h.E_p = ep;
    h.inc_m = sp.a_minus * em;
    h.inc_p = sp.a_plus * ep;
    h.invE_m = 1.0f / em;
    h.invE_p = 1.0f / ep;
    h.lam = sp.lambda;
    h.lam_alpha = sp.lambda * sp.alpha;
    h.wmax = sp.w_max;
    h.clip_upper = sp.clip_upper ? 1 : 0;
  }
  h.seed = m.seed;
  h.rate_counts = (int*)p_rate;
  h.gbits = (uint32_t*)p_gbits;
  h.bitsE = (uint32_t*)p_bE;
  h.stdp_rule = n->stdp_rule;
  if (dense) {
    h.H = B - 2 * n->G;  // D_max + 1
    h.csc_delay = (const int*)p_cdelay;
    h.dense_tr = (float2*)p_dtr;
    h.hist = (uint32_t*)p_hist;
    const spk_stdp_params& sp = m.stdp;
    if (n->stdp_rule == SPK_STDP_EVANS) {
      // decay_term_tau_C, decay_term_tau_D, synaptic_neurotransmitter_concentration_alpha_C,
      // model_parameter_alpha_D (Spike/Plasticity/EvansSTDPPlasticity.hpp)
      h.rule_c[0] = sp.tau_plus;
      h.rule_c[1] = sp.tau_minus;
      h.rule_c[2] = sp.a_plus;
      h.rule_c[3] = sp.a_minus;
    } else if (n->stdp_rule == SPK_STDP_INHIBITORY) {
      // trace decay expf(- timestep / tau_istdp), computed on the host as the
      // reference does (InhibitorySTDPPlasticity.cu:61), learningrate,
      // targetrate, tau_istdp
      h.rule_c[0] = expf(-m.dt / sp.tau_plus);
      h.rule_c[1] = sp.lambda;
      h.rule_c[2] = sp.alpha;
      h.rule_c[3] = sp.tau_plus;
    } else {
      // post and pre trace decays expf(- timestep / tau_minus / tau_plus),
      // computed on the host (CustomSTDPPlasticity.cu:55-56), a_plus, a_minus,
      // learning_rate, a_star, w_max, nearest_spike_only
      h.rule_c[0] = expf(-m.dt / sp.tau_minus);
      h.rule_c[1] = expf(-m.dt / sp.tau_plus);
      h.rule_c[2] = sp.a_plus;
      h.rule_c[3] = sp.a_minus;
      h.rule_c[4] = sp.lambda;
      h.rule_c[5] = sp.alpha;
      h.rule_c[6] = sp.w_max;
      h.rule_c[7] = sp.clip_upper ? 1.0f : 0.0f;
    }
  }
  h.weight_norm = n->weight_norm;
  if (norm) {
    h.norm_w0 = (const float*)p_nw0;
    h.norm_sum = (const float*)p_nsum;
  }
  h.rowptr = (const int*)p_rowptr;
  h.entries = (uint2*)p_entries;
  h.csc_ptr = (const int*)p_cscptr;
  h.csc = (uint2*)p_csc;
  h.V = (float*)p_V;
  h.last = (float*)p_last;
  h.gtr = (float*)p_gtr;
  h.ring = (float*)p_ring;
  h.in_next = (float*)p_innext;
  n->rates_dev = (float*)p_rates;
  h.rates = n->rates_dev + (size_t)n->stim * Nin;
  h.post_trace = (float*)p_post;
  h.pre_trace = (float*)p_pre;
  h.pre_pub = (float*)p_pub;
  h.bitsA = (uint32_t*)p_bA;
  h.bitsP = (uint32_t*)p_bP;
  h.cta_keys = (unsigned long long*)p_ckeys;
  h.cta_stamp = (unsigned long long*)p_cstamp;
  h.key_cap = key_cap;
  h.spikes = (uint2*)p_spk;
  h.spike_cap = spike_cap;
  h.ctl = (RunCtl*)p_ctl;
  h.abort_flag = (int*)p_abort;
  h.poll_ns = DEFAULT_WAIT_LIMIT_NS;
  n->abort_dev = (int*)p_abort;
  n->dd = (NetDev*)p_dd;
  n->dmap = (CtaMap*)p_map;

  // ---- uploads ---------------------------------------------------------------------
  auto up = [&](void* dst, const void* src, size_t bytes) -> int {
    if (bytes == 0 || !src) return SPK_OK;
    SPK_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, n->stream));
    return SPK_OK;
  };
  std::vector<CtaMap> map(plan.nctas);
  for (int r = 0; r < plan.nctas; ++r) map[r] = CtaMap{0, r};
  RunCtl ctl{};
  int urc = SPK_OK;
  urc |= up(p_rowptr, rowptr_h, sizeof(int32_t) * (n_cells + 1));
  urc |= up(p_entries, entries_h, sizeof(uint2) * S);
  urc |= up(p_cscptr, csc_ptr_h, sizeof(int32_t) * (stdp ? (size_t)N + 1 : 0));
  urc |= up(p_csc, csc_h, sizeof(uint2) * (size_t)n_csc);
  if (dense) urc |= up(p_cdelay, csc_delay_h, sizeof(int32_t) * (size_t)n_csc);
  if (norm) {
    urc |= up(p_nw0, n->norm_w0_h.data(), sizeof(float) * n->norm_w0_h.size());
    urc |= up(p_nsum, n->norm_sum_h.data(), sizeof(float) * n->norm_sum_h.size());
  }
  if (Nin > 0) urc |= up(p_rates, m.rates, sizeof(float) * (size_t)n->n_stim * Nin);
  urc |= up(p_ctl, &ctl, sizeof(ctl));
  urc |= up(p_dd, &h, sizeof(h));
  urc |= up(p_map, map.data(), sizeof(CtaMap) * map.size());
  if (urc) return fail_free(SPK_ERR_CUDA);
  if (cudaMemsetAsync(p_bA, 0, sizeof(uint32_t) * 2 * (size_t)n_words, n->stream) != cudaSuccess ||
      cudaMemsetAsync(p_bP, 0, sizeof(uint32_t) * 2 * (size_t)n_words, n->stream) != cudaSuccess ||
      cudaMemsetAsync(p_cstamp, 0, sizeof(unsigned long long) * 2 * (size_t)plan.nctas, n->stream) != cudaSuccess ||
      cudaMemsetAsync(p_ckeys, 0, sizeof(unsigned long long) * 2 * (size_t)plan.nctas * key_cap, n->stream) != cudaSuccess ||
      cudaMemsetAsync(p_abort, 0, sizeof(int), n->stream) != cudaSuccess) {
    set_error("cudaMemsetAsync failed");
    return fail_free(SPK_ERR_CUDA);
  }
  if (cudaFuncSetAttribute(step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           di.max_smem) != cudaSuccess) {
    set_error("cudaFuncSetAttribute failed: %s", cudaGetErrorString(cudaGetLastError()));
    return fail_free(SPK_ERR_CUDA);
  }
  if (plan.nctas > 1 && plan.persistent) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, step_kernel, plan.W * 32, plan.smem) !=
        cudaSuccess) {
      set_error("occupancy query failed");
      return fail_free(SPK_ERR_CUDA);
    }
    if ((int64_t)per_sm * di.sms < plan.nctas) {
      set_error("schedule needs %d co-resident CTAs, device holds %d", plan.nctas, per_sm * di.sms);
      return fail_free(SPK_ERR_UNSUPPORTED);
    }
    n->cooperative = true;
  }
  int rrc = upload_state_defaults(n);
  if (rrc) return fail_free(rrc);
  if (cudaStreamSynchronize(n->stream) != cudaSuccess) {
    set_error("initial upload failed: %s", cudaGetErrorString(cudaGetLastError()));
    return fail_free(SPK_ERR_CUDA);
  }
  if (plan.persistent) build_graph(n);
  return SPK_OK;
}

static int create_impl(const spk_net_desc* d, const spk_schedule* sched, spk_net** out) {
  if (!d || !out) {
    set_error("null argument");
    return SPK_ERR_INVALID;
  }
  if (d->abi_version != SPK_ABI_VERSION) {
    set_error("descriptor ABI version %d, library %d", d->abi_version, SPK_ABI_VERSION);
    return SPK_ERR_INVALID;
  }
  ModelSpec m;
  m.dt = d->dt;
  m.kind = d->synapse_kind;
  m.N = d->n_neurons;
  m.Nin = d->n_inputs;
  m.L = d->n_labels;
  m.n_groups = d->n_groups;
  m.groups = d->groups;
  m.t_ref = d->refractory_period;
  m.i_bg = d->background_current;
  m.n_stim = d->n_stimuli;
  m.stim = d->stimulus;
  m.rates = d->input_rates;
  m.label_tau = d->label_tau;
  m.label_vhat = d->label_vhat;
  m.has_stdp = d->has_stdp ? 1 : 0;
  m.stdp = d->stdp;
  m.stdp_rule = d->stdp_rule;
  m.weight_norm = d->weight_norm;
  m.norm_initial = d->norm_initial;
  m.norm_sum = d->norm_sum;
  m.seed = d->seed;
  m.spike_capacity = d->spike_capacity;
  m.record_inputs = d->record_inputs;
  int rc = validate_spec(m);
  if (rc) return rc;
  const int N = m.N, Nin = m.Nin, L = m.L;
  if (d->n_synapses < 0 || d->n_synapses > 0x7fffffffLL) {
    set_error("synapse count %lld out of range", (long long)d->n_synapses);
    return SPK_ERR_INVALID;
  }
  const int64_t S = d->n_synapses;
  if (S > 0 && (!d->pre || !d->post || !d->weight || !d->scale || !d->delay)) {
    set_error("synapse arrays missing");
    return SPK_ERR_INVALID;
  }
  int Dmax = 0, Dmin = 1 << 30;
  for (int64_t s = 0; s < S; ++s) {
    const int p = d->pre[s], q = d->post[s], dl = d->delay[s], lb = d->label ? d->label[s] : 0;
    if (p < -Nin || p >= N || q < 0 || q >= N || dl < 1 || lb < 0 || lb >= L) {
      set_error("synapse %lld out of range (pre %d post %d delay %d label %d)", (long long)s, p, q, dl, lb);
      return SPK_ERR_INVALID;
    }
    Dmax = std::max(Dmax, dl);
    Dmin = std::min(Dmin, dl);
  }
  // timestep_grouping = the minimum delay (Spike/Models/SpikingModel.cpp:98).
  // A network without synapses keeps G = 1: the reference's default minimum
  // (10^6 steps, Spike/Synapses/SpikingSynapses.hpp:40) would run no step.
  m.G = S > 0 ? Dmin : 1;
  rc = check_grouping(m);
  if (rc) return rc;
  if (Dmax > MAX_DELAY) {
    set_error("delay %d steps exceeds the supported maximum %d", Dmax, MAX_DELAY);
    return SPK_ERR_UNSUPPORTED;
  }
  if (S == 0) Dmax = 1;
  // Ring depth D_max + 2G + 1 (SpikingSynapses.cu:48).  The engine delivers
  // at most D_max slots ahead, but a run of a grouped network that is not
  // whole groups skips timestep indices (the next run starts at start +
  // seconds), and what was delivered to a skipped slot is read B steps later:
  // the depth decides when.
  const int B = Dmax + 2 * m.G + 1;
  const int stdp = m.has_stdp;

  spk_net* n = nullptr;
  rc = new_net(m, B, S, sched, &n);
  if (rc) return rc;
  const Plan& plan = n->plan;
  n->weights.assign(d->weight, d->weight + S);
  n->scales.assign(d->scale, d->scale + S);

  // ---- scale classes of plastic synapses ------------------------------------
  n->cls_of.assign(S, 0);
  {
    std::map<uint32_t, int> cls;
    for (int64_t s = 0; s < S; ++s) {
      if (!(stdp && d->plastic && d->plastic[s])) continue;
      const uint32_t bits = f2u(d->scale[s]);
      auto it = cls.find(bits);
      int c;
      if (it == cls.end()) {
        c = (int)cls.size() + 1;
        if (c >= MAX_CLASSES) {
          set_error("more than %d distinct weight scales among plastic synapses", MAX_CLASSES - 1);
          delete n;
          return SPK_ERR_UNSUPPORTED;
        }
        cls[bits] = c;
        n->scale_tab[c] = d->scale[s];
      } else {
        c = it->second;
      }
      n->cls_of[s] = (uint8_t)c;
    }
  }

  // ---- row-partitioned CSR: entries sorted by (key, tile), stable ------------
  const int n_tiles = plan.n_tiles, TS = plan.TS, KL = plan.KL, n_keys = plan.n_keys;
  const size_t n_cells = (size_t)n_keys * n_tiles;
  std::vector<int32_t> rowptr(n_cells + 1, 0);
  auto key_of = [&](int p) { return p < 0 ? Nin + p : KL + p; };
  for (int64_t s = 0; s < S; ++s) {
    const size_t c = (size_t)key_of(d->pre[s]) * n_tiles + d->post[s] / TS;
    rowptr[c + 1]++;
  }
  for (size_t c = 0; c < n_cells; ++c) rowptr[c + 1] += rowptr[c];
  // ---- plastic afferent records per post: (pre key, weight), creation order --
  std::vector<int32_t> csc_ptr;
  std::vector<uint2> csc;
  std::vector<int32_t> csc_delay;
  n->csc_of.assign(stdp ? S : 0, -1);
  if (stdp) {
    csc_ptr.assign((size_t)N + 1, 0);
    for (int64_t s = 0; s < S; ++s)
      if (n->cls_of[s]) csc_ptr[d->post[s] + 1]++;
    for (int q = 0; q < N; ++q) csc_ptr[q + 1] += csc_ptr[q];
    csc.resize(csc_ptr[N]);
    if (n->dense()) csc_delay.resize(csc_ptr[N]);
    std::vector<int32_t> fill(csc_ptr.begin(), csc_ptr.end() - 1);
    for (int64_t s = 0; s < S; ++s)
      if (n->cls_of[s]) {
        const int32_t pos = fill[d->post[s]]++;
        csc[pos] = make_uint2((uint32_t)key_of(d->pre[s]), f2u(d->weight[s]));
        if (n->dense()) csc_delay[pos] = d->delay[s];
        n->csc_of[s] = pos;
      }
    if (n->weight_norm != SPK_NORM_OFF) {
      // WeightNormSTDPPlasticity::prepare_backend_early
      // (Spike/Plasticity/WeightNormSTDPPlasticity.cpp:31-70): initial weights,
      // and per post the sum of pow(w, 2.0f) over its plastic afferents in
      // the rule's (creation) order, on the host
      n->norm_w0_h.assign(csc.size(), 0.0f);
      n->norm_sum_h.assign((size_t)N, 0.0f);
      for (int64_t s = 0; s < S; ++s) {
        const int32_t pos = n->csc_of[s];
        if (pos < 0) continue;
        n->norm_w0_h[pos] = m.norm_initial ? m.norm_initial[s] : d->weight[s];
        if (!m.norm_sum) n->norm_sum_h[d->post[s]] += powf(d->weight[s], 2.0f);
      }
      if (m.norm_sum) n->norm_sum_h.assign(m.norm_sum, m.norm_sum + N);
    }
  }
  // ---- entries: static synapses carry w*scale, plastic ones their record ----
  std::vector<uint2> entries(S);
  n->entry_of.resize(S);
  {
    std::vector<int32_t> fill(rowptr.begin(), rowptr.end() - 1);
    for (int64_t s = 0; s < S; ++s) {
      const int q = d->post[s];
      const size_t c = (size_t)key_of(d->pre[s]) * n_tiles + q / TS;
      const int32_t pos = fill[c]++;
      const int cl = n->cls_of[s];
      const uint32_t y = cl ? (uint32_t)n->csc_of[s] : f2u(d->weight[s] * d->scale[s]);
      entries[pos] = make_uint2(pack_entry((uint32_t)(q % TS), (uint32_t)d->delay[s],
                                           (uint32_t)(d->label ? d->label[s] : 0), (uint32_t)cl),
                                y);
      n->entry_of[s] = pos;
    }
  }
  rc = setup_device(n, m, (int64_t)csc.size(), rowptr.data(), entries.data(), stdp ? csc_ptr.data() : nullptr,
                    csc.data(), n->dense() ? csc_delay.data() : nullptr);
  if (rc) return rc;
  *out = n;
  return SPK_OK;
}

// Stream-ordered device memory released on scope exit (temporaries of network
// generation; stream-ordered so that generating a network never waits for
// kernels running on other streams, such as a batch in flight).
struct DevTemp {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  explicit DevTemp(cudaStream_t stream) : s(stream) {}
  DevTemp(const DevTemp&) = delete;
  DevTemp& operator=(const DevTemp&) = delete;
  ~DevTemp() { reset(); }
  void reset() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
  }
  bool alloc(size_t bytes) {
    reset();
    if (cudaMallocAsync(&p, std::max<size_t>(bytes, 16), s) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      set_error("device allocation of %zu bytes for network generation failed", bytes);
      return false;
    }
    return true;
  }
  template <typename T>
  T* as() const {
    return (T*)p;
  }
};

static int generate_impl(const spk_gen_desc* d, const spk_schedule* sched, spk_net** out) {
  if (!d || !out) {
    set_error("null argument");
    return SPK_ERR_INVALID;
  }
  if (d->abi_version != SPK_ABI_VERSION) {
    set_error("descriptor ABI version %d, library %d", d->abi_version, SPK_ABI_VERSION);
    return SPK_ERR_INVALID;
  }
  ModelSpec m;
  m.dt = d->dt;
  m.kind = d->synapse_kind;
  m.N = d->n_neurons;
  m.Nin = d->n_inputs;
  m.L = d->n_labels;
  m.n_groups = d->n_groups;
  m.groups = d->groups;
  m.t_ref = d->refractory_period;
  m.i_bg = d->background_current;
  m.n_stim = d->n_stimuli;
  m.stim = d->stimulus;
  m.rates = d->input_rates;
  m.label_tau = d->label_tau;
  m.label_vhat = d->label_vhat;
  m.has_stdp = d->has_stdp ? 1 : 0;
  m.stdp = d->stdp;
  m.stdp_rule = d->stdp_rule;
  m.seed = d->seed;
  m.spike_capacity = d->spike_capacity;
  m.record_inputs = d->record_inputs;
  int rc = validate_spec(m);
  if (rc) return rc;
  const int N = m.N, Nin = m.Nin, L = m.L;
  const int n_proj = d->n_projections;
  if (n_proj < 0 || n_proj > MAX_PROJECTIONS || (n_proj > 0 && !d->projections)) {
    set_error("between 0 and %d projections are supported (got %d)", MAX_PROJECTIONS, n_proj);
    return SPK_ERR_INVALID;
  }
  // ---- projections: validate, assign plastic scale classes, sort by first post
  std::vector<GenProj> proj;
  std::map<uint32_t, int> cls;
  std::vector<float> scale_tab(MAX_CLASSES, 0.0f);
  int dlo_min = 1 << 30;
  for (int j = 0; j < n_proj; ++j) {
    const spk_projection& P = d->projections[j];
    const int pop_size = P.pre_population == SPK_POP_INPUTS ? Nin : N;
    if ((P.pre_population != SPK_POP_NEURONS && P.pre_population != SPK_POP_INPUTS) || P.pre_start < 0 ||
        P.pre_count < 0 || (int64_t)P.pre_start + P.pre_count > pop_size || P.post_start < 0 || P.post_count < 0 ||
        (int64_t)P.post_start + P.post_count > N || !(P.probability >= 0.0f && P.probability <= 1.0f) ||
        P.delay_lo < 1 || P.delay_hi < P.delay_lo || P.delay_hi > MAX_DELAY || P.label < 0 || P.label >= L ||
        (P.plastic && !m.has_stdp)) {
      set_error("projection %d out of range (pre %d+%d of %d, post %d+%d, p %g, delays %d..%d, label %d, plastic %d)",
                j, P.pre_start, P.pre_count, pop_size, P.post_start, P.post_count, (double)P.probability,
                P.delay_lo, P.delay_hi, P.label, P.plastic);
      return SPK_ERR_INVALID;
    }
    for (int k = 0; k < j; ++k) {
      const spk_projection& Q = d->projections[k];
      const bool pre_overlap = Q.pre_population == P.pre_population && P.pre_start < Q.pre_start + Q.pre_count &&
                               Q.pre_start < P.pre_start + P.pre_count;
      const bool post_overlap =
          P.post_start < Q.post_start + Q.post_count && Q.post_start < P.post_start + P.post_count;
      if (pre_overlap && post_overlap && P.pre_count && P.post_count && Q.pre_count && Q.post_count) {
        set_error("projections %d and %d overlap in (pre, post)", k, j);
        return SPK_ERR_INVALID;
      }
    }
    GenProj g;
    g.pop = P.pre_population;
    g.pre_lo = P.pre_start;
    g.pre_hi = P.pre_start + P.pre_count;
    g.post_lo = P.post_start;
    g.post_hi = P.post_start + P.post_count;
    g.p = P.probability;
    g.w_lo = P.weight_lo;
    g.w_span = P.weight_hi - P.weight_lo;
    g.scale = P.scale;
    g.d_lo = P.delay_lo;
    g.d_n = P.delay_hi - P.delay_lo + 1;
    g.label = P.label;
    g.cls = 0;
    if (P.plastic) {
      const uint32_t bits = f2u(P.scale);
      auto it = cls.find(bits);
      if (it == cls.end()) {
        const int c = (int)cls.size() + 1;
        if (c >= MAX_CLASSES) {
          set_error("more than %d distinct weight scales among plastic projections", MAX_CLASSES - 1);
          return SPK_ERR_UNSUPPORTED;
        }
        cls[bits] = c;
        scale_tab[c] = P.scale;
        g.cls = c;
      } else {
        g.cls = it->second;
      }
    }
    if (P.probability > 0.0f && P.pre_count > 0 && P.post_count > 0) dlo_min = std::min(dlo_min, P.delay_lo);
    proj.push_back(g);
  }
  std::stable_sort(proj.begin(), proj.end(), [](const GenProj& a, const GenProj& b) { return a.post_lo < b.post_lo; });
  if (dlo_min != (1 << 30) && dlo_min > 1) {
    // every drawn delay is at least dlo_min, so G > 1 whatever is drawn
    m.G = dlo_min;
    rc = check_grouping(m);
    if (rc) return rc;
  }

  DeviceInfo di;
  rc = device_info(&di);
  if (rc) return rc;
  // The schedule does not change the connectivity, only the cells it is cut
  // into; the ring depth needs the largest drawn delay, so plan with the
  // largest possible one first and re-plan if fewer are drawn.
  int dmax_bound = 1;
  for (const auto& g : proj) dmax_bound = std::max(dmax_bound, g.d_lo + g.d_n - 1);
  spk_net* probe = nullptr;
  rc = new_net(m, dmax_bound + 2 * m.G + 1, 0, sched, &probe);
  if (rc) return rc;
  const Plan plan0 = probe->plan;
  delete probe;

  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("cudaStreamCreate failed");
    return SPK_ERR_CUDA;
  }
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  } sg{st};
  const int grid = std::max(1, di.sms * 8);
  auto gen_shape = [&](const Plan& pl) {
    GenShape g;
    g.N = N;
    g.Nin = Nin;
    g.KL = pl.KL;
    g.n_tiles = pl.n_tiles;
    g.TS = pl.TS;
    g.n_proj = (int)proj.size();
    g.n_cells = (long long)pl.n_keys * pl.n_tiles;
    g.seed = d->connectivity_seed;
    return g;
  };
  DevTemp proj_dev(st), small(st);
  if (!proj_dev.alloc(sizeof(GenProj) * proj.size()) || !small.alloc(64)) return SPK_ERR_OOM;
  if (!proj.empty())
    SPK_CUDA(cudaMemcpyAsync(proj_dev.p, proj.data(), sizeof(GenProj) * proj.size(), cudaMemcpyHostToDevice, st));
  unsigned long long* totals = small.as<unsigned long long>();  // [0] all, [1] plastic
  int* drange = (int*)(totals + 2);                             // [0] min, [1] max drawn delay

  // ---- count pass (with the plan for the largest possible delay) -------------------
  auto count_pass = [&](const Plan& pl, DevTemp& counts, unsigned long long host_tot[2], int host_dr[2]) -> int {
    const GenShape g = gen_shape(pl);
    if (!counts.alloc(sizeof(int) * (size_t)(g.n_cells + 1))) return SPK_ERR_OOM;
    const unsigned long long zero2[2] = {0ull, 0ull};
    const int dr0[2] = {1 << 30, 0};
    SPK_CUDA(cudaMemcpyAsync(totals, zero2, sizeof(zero2), cudaMemcpyHostToDevice, st));
    SPK_CUDA(cudaMemcpyAsync(drange, dr0, sizeof(dr0), cudaMemcpyHostToDevice, st));
    SPK_CUDA(cudaMemsetAsync(counts.as<int>() + g.n_cells, 0, sizeof(int), st));
    gen_cells_kernel<false><<<grid, 256, 0, st>>>(g, proj_dev.as<GenProj>(), counts.as<int>(), totals, nullptr,
                                                  nullptr, nullptr, nullptr, nullptr, drange);
    SPK_CUDA(cudaGetLastError());
    SPK_CUDA(cudaMemcpyAsync(host_tot, totals, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    SPK_CUDA(cudaMemcpyAsync(host_dr, drange, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    SPK_CUDA(cudaStreamSynchronize(st));
    return SPK_OK;
  };
  DevTemp counts(st);
  unsigned long long tot[2] = {0, 0};
  int dr[2] = {0, 0};
  rc = count_pass(plan0, counts, tot, dr);
  if (rc) return rc;
  if (tot[0] > 0x7fffffffull) {
    set_error("generated network has %llu synapses; at most 2^31-1 per network are supported", tot[0]);
    return SPK_ERR_UNSUPPORTED;
  }
  // timestep_grouping = the minimum drawn delay (Spike/Models/SpikingModel.cpp:98)
  m.G = tot[0] > 0 ? dr[0] : 1;
  rc = check_grouping(m);
  if (rc) return rc;
  const int Dmax = tot[0] > 0 ? dr[1] : 1;
  const int B = Dmax + 2 * m.G + 1;  // SpikingSynapses.cu:48
  spk_net* n = nullptr;
  rc = new_net(m, B, (int64_t)tot[0], sched, &n);
  if (rc) return rc;
  if (n->plan.TS != plan0.TS || n->plan.nctas != plan0.nctas || n->plan.W != plan0.W) {
    // a shallower ring let the planner pick another cut: count again
    unsigned long long tot2[2];
    int dr2[2];
    rc = count_pass(n->plan, counts, tot2, dr2);
    if (rc == SPK_OK && (tot2[0] != tot[0] || tot2[1] != tot[1])) {
      set_error("generated synapse count changed with the schedule (%llu vs %llu)", tot2[0], tot[0]);
      rc = SPK_ERR_CUDA;
    }
    if (rc) {
      delete n;
      return rc;
    }
  }
  const int64_t S = (int64_t)tot[0], P = (int64_t)tot[1];
  for (int c = 0; c < MAX_CLASSES; ++c) n->scale_tab[c] = scale_tab[c];
  n->generated = true;
  rc = setup_device(n, m, m.has_stdp ? P : 0, nullptr, nullptr, nullptr, nullptr);
  if (rc) return rc;  // n destroyed
  auto fail = [&](int code) {
    cudaStreamSynchronize(st);
    spk_net_destroy(n);
    return code;
  };
  const Plan& pl = n->plan;
  const GenShape g = gen_shape(pl);
  const long long n_cells = g.n_cells;
  // ---- row pointers, entries, plastic afferents -------------------------------------
  {
    size_t tb = 0;
    if (cub::DeviceScan::ExclusiveSum(nullptr, tb, counts.as<int>(), (int*)n->hd.rowptr, n_cells + 1, st) !=
        cudaSuccess)
      return fail(SPK_ERR_CUDA);
    DevTemp tmp(st);
    if (!tmp.alloc(tb)) return fail(SPK_ERR_OOM);
    if (cub::DeviceScan::ExclusiveSum(tmp.p, tb, counts.as<int>(), (int*)n->hd.rowptr, n_cells + 1, st) !=
        cudaSuccess) {
      set_error("row pointer scan failed: %s", cudaGetErrorString(cudaGetLastError()));
      return fail(SPK_ERR_CUDA);
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return fail(SPK_ERR_CUDA);
  }
  const bool csc = m.has_stdp && P > 0;
  DevTemp sort_a(st), sort_b(st), val_a(st), val_b(st), ekey(st), pcnt(st);
  if (m.has_stdp && !csc &&
      cudaMemsetAsync((void*)n->hd.csc_ptr, 0, sizeof(int) * ((size_t)N + 1), st) != cudaSuccess)
    return fail(SPK_ERR_CUDA);
  if (csc) {
    if (!sort_a.alloc(sizeof(uint32_t) * S) || !sort_b.alloc(sizeof(uint32_t) * S) ||
        !val_a.alloc(sizeof(uint32_t) * S) || !val_b.alloc(sizeof(uint32_t) * S) ||
        !ekey.alloc(sizeof(uint32_t) * S) || !pcnt.alloc(sizeof(int) * ((size_t)N + 1)))
      return fail(SPK_ERR_OOM);
    if (cudaMemsetAsync(pcnt.p, 0, sizeof(int) * ((size_t)N + 1), st) != cudaSuccess) return fail(SPK_ERR_CUDA);
  }
  gen_cells_kernel<true><<<grid, 256, 0, st>>>(g, proj_dev.as<GenProj>(), nullptr, nullptr, n->hd.rowptr,
                                               n->hd.entries, csc ? sort_a.as<uint32_t>() : nullptr,
                                               csc ? ekey.as<uint32_t>() : nullptr, csc ? pcnt.as<int>() : nullptr,
                                               nullptr);
  if (cudaGetLastError() != cudaSuccess) return fail(SPK_ERR_CUDA);
  if (csc) {
    size_t tb = 0;
    if (cub::DeviceScan::ExclusiveSum(nullptr, tb, pcnt.as<int>(), (int*)n->hd.csc_ptr, (long long)N + 1, st) !=
        cudaSuccess)
      return fail(SPK_ERR_CUDA);
    DevTemp tmp(st);
    if (!tmp.alloc(tb)) return fail(SPK_ERR_OOM);
    if (cub::DeviceScan::ExclusiveSum(tmp.p, tb, pcnt.as<int>(), (int*)n->hd.csc_ptr, (long long)N + 1, st) !=
        cudaSuccess)
      return fail(SPK_ERR_CUDA);
    gen_iota_kernel<<<grid, 256, 0, st>>>(val_a.as<uint32_t>(), S);
    if (cudaGetLastError() != cudaSuccess) return fail(SPK_ERR_CUDA);
    int end_bit = 1;
    while (end_bit < 32 && ((uint32_t)N >> end_bit) != 0u) ++end_bit;
    cub::DoubleBuffer<uint32_t> keys(sort_a.as<uint32_t>(), sort_b.as<uint32_t>());
    cub::DoubleBuffer<uint32_t> vals(val_a.as<uint32_t>(), val_b.as<uint32_t>());
    size_t sb = 0;
    if (cub::DeviceRadixSort::SortPairs(nullptr, sb, keys, vals, (long long)S, 0, end_bit, st) != cudaSuccess)
      return fail(SPK_ERR_CUDA);
    DevTemp stmp(st);
    if (!stmp.alloc(sb)) return fail(SPK_ERR_OOM);
    if (cub::DeviceRadixSort::SortPairs(stmp.p, sb, keys, vals, (long long)S, 0, end_bit, st) != cudaSuccess) {
      set_error("plastic afferent sort failed: %s", cudaGetErrorString(cudaGetLastError()));
      return fail(SPK_ERR_CUDA);
    }
    gen_csc_kernel<<<grid, 256, 0, st>>>(n->hd.csc, n->hd.entries, vals.Current(), ekey.as<uint32_t>(),
                                         (long long)P, const_cast<int*>(n->hd.csc_delay));
    if (cudaGetLastError() != cudaSuccess) return fail(SPK_ERR_CUDA);
    if (cudaStreamSynchronize(st) != cudaSuccess) {
      set_error("network generation failed: %s", cudaGetErrorString(cudaGetLastError()));
      return fail(SPK_ERR_CUDA);
    }
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) {
    set_error("network generation failed: %s", cudaGetErrorString(cudaGetLastError()));
    return fail(SPK_ERR_CUDA);
  }
  *out = n;
  return SPK_OK;
}

}  // namespace spk

// =====================================================================================
extern "C" {

const char* spk_last_error(void) { return spk::g_err; }
int spk_abi_version(void) { return SPK_ABI_VERSION; }

int spk_net_create(const spk_net_desc* desc, const spk_schedule* schedule, spk_net** out) {
  return guarded([&] { return create_impl(desc, schedule, out); });
}

int spk_net_generate(const spk_gen_desc* desc, const spk_schedule* schedule, spk_net** out) {
  return guarded([&] { return generate_impl(desc, schedule, out); });
}

int spk_net_set_step_cost(spk_net* n, float cost) {
  if (!n || !(cost >= 0.0f)) return SPK_ERR_INVALID;
  n->step_cost = cost;
  return SPK_OK;
}

int spk_net_generate_estimate(const spk_gen_desc* d, const spk_schedule* sched, int64_t* device_bytes,
                              int64_t* peak_bytes) {
  if (!d || d->n_neurons <= 0 || d->n_inputs < 0 || d->n_projections < 0 ||
      (d->n_projections > 0 && !d->projections))
    return SPK_ERR_INVALID;
  return guarded([&]() -> int {
    double mu = 0.0, var = 0.0, mu_p = 0.0, var_p = 0.0;
    int dmax = 1, ghi = 1 << 30;
    for (int j = 0; j < d->n_projections; ++j) {
      const spk_projection& P = d->projections[j];
      const double n = (double)P.pre_count * (double)P.post_count, p = P.probability;
      if (n * p > 0.0) ghi = std::min(ghi, P.delay_hi);  // the smallest drawn delay is at most this
      mu += n * p;
      var += n * p * (1.0 - p);
      if (P.plastic && d->has_stdp) {
        mu_p += n * p;
        var_p += n * p * (1.0 - p);
      }
      dmax = std::max(dmax, P.delay_hi);
    }
    const int64_t S = (int64_t)(mu + 6.0 * std::sqrt(var) + 16.0);
    const int64_t Pl = d->has_stdp ? (int64_t)(mu_p + 6.0 * std::sqrt(var_p) + 16.0) : 0;
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    Plan plan;
    // the deepest ring the drawn timestep grouping can need
    const int G = ghi == (1 << 30) ? 1 : std::max(1, ghi);
    const int B = dmax + 2 * G + 1;
    rc = make_plan(d->n_neurons, d->n_inputs, B, std::max(1, d->n_labels), d->synapse_kind, d->has_stdp ? 1 : 0,
                   sched, di, &plan);
    if (rc) return rc;
    const int64_t cap = d->spike_capacity == 0 ? DEFAULT_SPIKE_CAPACITY : std::max<int64_t>(0, d->spike_capacity);
    const size_t arena = arena_total(arena_part_sizes(plan, d->n_neurons, d->n_inputs, std::max(1, d->n_labels), B,
                                                      d->has_stdp ? 1 : 0, S, Pl, d->n_inputs ? d->n_stimuli : 0,
                                                      cap, 0, 0, G));
    // generation temporaries: cell counts, and for plastic synapses the sort
    // keys, values, entry keys (both buffers) and the sort's own storage
    const size_t cells = (size_t)plan.n_keys * plan.n_tiles + 1;
    const size_t temp = 4 * cells + (Pl > 0 ? (size_t)S * (5 * 4 + 8) + 4 * ((size_t)d->n_neurons + 1) : 0);
    if (device_bytes) *device_bytes = (int64_t)arena;
    if (peak_bytes) *peak_bytes = (int64_t)(arena + temp);
    return SPK_OK;
  });
}

// ---- snapshot / restore of the dynamic state ------------------------------------------
namespace {
struct SnapHeader {
  uint32_t magic, version;
  int32_t N, Nin, L, B, n_tiles, TS, ITS, KL, n_keys, nctas, has_stdp, stim;
  int64_t S, n_csc;
  float current_time;
  int32_t pad;
  RunCtl ctl;
};
constexpr uint32_t SNAP_MAGIC = 0x53504b53u;  // "SPKS"

struct SnapPart {
  void* dev;
  size_t bytes;
};

std::vector<SnapPart> snap_parts(spk_net* n) {
  const NetDev& h = n->hd;
  std::vector<SnapPart> p = {
      {h.V, sizeof(float) * n->N},
      {h.last, sizeof(float) * n->N},
      {h.gtr, sizeof(float) * (size_t)n->N * n->L},
      {h.ring, sizeof(float) * (size_t)h.n_tiles * h.B * h.TS * h.L},
      {h.in_next, sizeof(float) * (size_t)n->Nin},
  };
  if (n->has_stdp) {
    p.push_back({h.post_trace, sizeof(float) * n->N});
    p.push_back({h.pre_trace, sizeof(float) * (size_t)h.n_keys});
    p.push_back({h.csc, sizeof(uint2) * (size_t)n->n_csc});
  }
  if (n->dense()) {
    p.push_back({h.dense_tr, sizeof(float2) * (size_t)n->n_csc});
    p.push_back({h.hist, sizeof(uint32_t) * (size_t)h.H * h.n_words});
  }
  p.push_back({h.gbits, sizeof(uint32_t) * (size_t)n->G * h.n_words});  // the last group's spikes
  return p;
}
}  // namespace

int spk_net_snapshot_bytes(spk_net* n, int64_t* bytes) {
  if (!n || !bytes) return SPK_ERR_INVALID;
  return guarded([&]() -> int {
    size_t b = sizeof(SnapHeader);
    for (const auto& p : snap_parts(n)) b += p.bytes;
    *bytes = (int64_t)b;
    return SPK_OK;
  });
}

int spk_net_snapshot(spk_net* n, void* buf, int64_t bytes) {
  int64_t need = 0;
  int rc = spk_net_snapshot_bytes(n, &need);
  if (rc) return rc;
  if (!buf || bytes < need) {
    set_error("snapshot needs %lld bytes", (long long)need);
    return SPK_ERR_INVALID;
  }
  return guarded([&]() -> int {
    SPK_CUDA(cudaStreamSynchronize(n->stream));
    SnapHeader hd{};
    hd.magic = SNAP_MAGIC;
    hd.version = 2;
    hd.N = n->N;
    hd.Nin = n->Nin;
    hd.L = n->L;
    hd.B = n->B;
    hd.n_tiles = n->hd.n_tiles;
    hd.TS = n->hd.TS;
    hd.ITS = n->hd.ITS;
    hd.KL = n->hd.KL;
    hd.n_keys = n->hd.n_keys;
    hd.nctas = n->hd.nctas;
    hd.has_stdp = n->has_stdp ? 1 : 0;
    hd.stim = n->stim;
    hd.S = n->S;
    hd.n_csc = n->n_csc;
    hd.current_time = n->current_time;
    SPK_CUDA(cudaMemcpy(&hd.ctl, n->hd.ctl, sizeof(RunCtl), cudaMemcpyDeviceToHost));
    char* out = (char*)buf;
    std::memcpy(out, &hd, sizeof(hd));
    out += sizeof(hd);
    for (const auto& p : snap_parts(n)) {
      if (p.bytes) SPK_CUDA(cudaMemcpy(out, p.dev, p.bytes, cudaMemcpyDeviceToHost));
      out += p.bytes;
    }
    return SPK_OK;
  });
}

int spk_net_restore(spk_net* n, const void* buf, int64_t bytes) {
  int64_t need = 0;
  int rc = spk_net_snapshot_bytes(n, &need);
  if (rc) return rc;
  if (!buf || bytes < need) {
    set_error("snapshot of %lld bytes, the network's needs %lld", (long long)bytes, (long long)need);
    return SPK_ERR_INVALID;
  }
  SnapHeader hd;
  std::memcpy(&hd, buf, sizeof(hd));
  if (hd.magic != SNAP_MAGIC || hd.version != 2 || hd.N != n->N || hd.Nin != n->Nin || hd.L != n->L ||
      hd.B != n->B || hd.n_tiles != n->hd.n_tiles || hd.TS != n->hd.TS || hd.ITS != n->hd.ITS ||
      hd.n_keys != n->hd.n_keys || hd.nctas != n->hd.nctas || hd.has_stdp != (n->has_stdp ? 1 : 0) ||
      hd.S != n->S || hd.n_csc != n->n_csc) {
    set_error("snapshot was taken from a network of another shape or schedule");
    return SPK_ERR_INVALID;
  }
  return guarded([&]() -> int {
    SPK_CUDA(cudaStreamSynchronize(n->stream));
    const char* in = (const char*)buf + sizeof(hd);
    for (const auto& p : snap_parts(n)) {
      if (p.bytes) SPK_CUDA(cudaMemcpy(p.dev, in, p.bytes, cudaMemcpyHostToDevice));
      in += p.bytes;
    }
    RunCtl c = hd.ctl;
    fold_finished_run(c, n->G, n->dt);  // the snapshot's last run, for the active-list state
    c.step = 0;
    c.steps_total = 0;
    c.spike_count = 0;  // the spike store is not part of a snapshot
    c.status = 0;
    SPK_CUDA(cudaMemcpy(n->hd.ctl, &c, sizeof(c), cudaMemcpyHostToDevice));
    SPK_CUDA(cudaMemset(n->abort_dev, 0, sizeof(int)));
    SPK_CUDA(cudaMemset(n->hd.cta_stamp, 0, sizeof(unsigned long long) * 2 * (size_t)n->hd.nctas));
    SPK_CUDA(cudaMemset(n->hd.cta_keys, 0, sizeof(unsigned long long) * 2 * (size_t)n->hd.nctas * n->hd.key_cap));
    if (hd.stim != n->stim && n->Nin > 0 && hd.stim >= 0 && hd.stim < n->n_stim) {
      n->stim = hd.stim;
      n->hd.rates = n->rates_dev + (size_t)n->stim * n->Nin;
      SPK_CUDA(cudaMemcpy(&n->dd->rates, &n->hd.rates, sizeof(float*), cudaMemcpyHostToDevice));
    }
    n->current_time = hd.current_time;
    return SPK_OK;
  });
}

int spk_net_set_wait_limit(spk_net* n, double seconds) {
  if (!n || !(seconds >= 1e-4 && seconds <= 60.0)) {
    set_error("wait limit must be between 1e-4 and 60 seconds");
    return SPK_ERR_INVALID;
  }
  SPK_CUDA(cudaStreamSynchronize(n->stream));
  n->hd.poll_ns = (unsigned long long)(seconds * 1e9);
  SPK_CUDA(cudaMemcpy(&n->dd->poll_ns, &n->hd.poll_ns, sizeof(unsigned long long), cudaMemcpyHostToDevice));
  return SPK_OK;
}

int spk_net_inject_withheld_cta(spk_net* n, int32_t rank) {
  if (!n || n->plan.nctas < 2 || rank < 0 || rank >= n->plan.nctas) {
    set_error("withholding a CTA needs a multi-CTA network and a rank below its CTA count");
    return SPK_ERR_INVALID;
  }
  n->withhold = rank;
  return SPK_OK;
}

int spk_net_synapse_count(const spk_net* n, int64_t* count) {
  if (!n || !count) return SPK_ERR_INVALID;
  *count = n->S;
  return SPK_OK;
}

int spk_net_plastic_synapse_count(const spk_net* n, int64_t* count) {
  if (!n || !count) return SPK_ERR_INVALID;
  *count = n->has_stdp ? n->n_csc : 0;
  return SPK_OK;
}

int spk_net_destroy(spk_net* n) {
  if (!n) return SPK_ERR_INVALID;
  if (n->self_batch) spk_batch_destroy(n->self_batch);
  if (n->stream) cudaStreamSynchronize(n->stream);
  if (n->graph) cudaGraphExecDestroy(n->graph);
  if (n->stream) cudaStreamDestroy(n->stream);
  if (n->arena) cudaFree(n->arena);
  delete n;
  return SPK_OK;
}

int spk_net_reset_state(spk_net* n) {
  if (!n) return SPK_ERR_INVALID;
  int rc = upload_state_defaults(n);
  if (rc) return rc;
  SPK_CUDA(cudaStreamSynchronize(n->stream));
  return SPK_OK;
}

int spk_net_reset_time(spk_net* n) {
  if (!n) return SPK_ERR_INVALID;
  n->current_time = 0.0f;
  return SPK_OK;
}

int spk_net_select_stimulus(spk_net* n, int32_t stimulus) {
  if (!n) return SPK_ERR_INVALID;
  if (n->Nin == 0 || stimulus < 0 || stimulus >= n->n_stim) {
    set_error("stimulus %d out of range (%d loaded)", stimulus, n->n_stim);
    return SPK_ERR_INVALID;
  }
  n->stim = stimulus;
  n->hd.rates = n->rates_dev + (size_t)stimulus * n->Nin;
  reset_inputs_kernel<<<(n->Nin + 255) / 256, 256, 0, n->stream>>>(n->dd, n->hd.rates, n->Nin);
  SPK_CUDA(cudaGetLastError());
  return SPK_OK;
}

int spk_net_write_rates(spk_net* n, int32_t stimulus, const float* rates, int64_t count) {
  if (!n || !rates || stimulus < 0 || stimulus >= n->n_stim || count != n->Nin) {
    set_error("write_rates: stimulus %d of %d, %lld rates for %d inputs", stimulus, n ? n->n_stim : 0,
              (long long)count, n ? n->Nin : 0);
    return SPK_ERR_INVALID;
  }
  SPK_CUDA(cudaMemcpyAsync(n->rates_dev + (size_t)stimulus * n->Nin, rates, sizeof(float) * n->Nin,
                           cudaMemcpyHostToDevice, n->stream));
  return SPK_OK;
}

int spk_net_run(spk_net* n, float seconds, int32_t plasticity_on) {
  if (!n || !(seconds >= 0.0f)) return SPK_ERR_INVALID;
  // number_of_timesteps = ceil(seconds / timestep) in float, number_of_steps
  // = number_of_timesteps / timestep_grouping in integers (whole groups:
  // Spike/Models/SpikingModel.cpp:221-222), end time start + seconds (:235).
  const float q = seconds / n->dt;
  const int64_t steps = ((int64_t)std::ceil(q) / n->G) * n->G;
  const float start = n->current_time;
  int rc = run_steps_impl(n, steps, plasticity_on, start);
  if (rc) return rc;
  n->current_time = start + seconds;
  return SPK_OK;
}

// Runs given in timesteps advance whole groups of the network's timestep grouping.
static int check_whole_groups(const spk_net* n, int64_t n_steps) {
  if (n_steps % n->G != 0) {
    set_error("%lld timesteps are not whole groups of the network's timestep grouping %d (its minimum delay)",
              (long long)n_steps, n->G);
    return SPK_ERR_INVALID;
  }
  return SPK_OK;
}

int spk_net_begin_run(spk_net* n, int64_t n_steps, int32_t plasticity_on) {
  if (!n || n_steps < 0 || n_steps > 0x7fffffff) return SPK_ERR_INVALID;
  if (int rc = check_whole_groups(n, n_steps)) return rc;
  const float start = n->current_time;
  if (int rc = begin_run_on(n, n->stream, start, n_steps, (plasticity_on && n->has_stdp) ? 1 : 0)) return rc;
  n->current_time = start + (float)n_steps * n->dt;
  return SPK_OK;
}

int spk_net_run_steps(spk_net* n, int64_t n_steps, int32_t plasticity_on) {
  if (!n || n_steps < 0) return SPK_ERR_INVALID;
  if (int rc = check_whole_groups(n, n_steps)) return rc;
  const float start = n->current_time;
  int rc = run_steps_impl(n, n_steps, plasticity_on, start);
  if (rc) return rc;
  n->current_time = start + (float)n_steps * n->dt;
  return SPK_OK;
}

int spk_net_synchronize(spk_net* n) {
  if (!n) return SPK_ERR_INVALID;
  int st = 0;
  int rc = read_status(n, &st);
  if (rc) return rc;
  if (st == SPK_ERR_TIMEOUT) set_error("a device wait on another CTA timed out");
  if (st == SPK_ERR_OVERFLOW) set_error("the device spike store overflowed; spikes were dropped");
  if (st == SPK_ERR_UNSUPPORTED)
    set_error("a run began at the group index parity of a one-group run that itself began so: the reference "
              "then delivers two earlier groups again, this engine keeps only the last");
  return st;
}

int spk_net_timestep_grouping(const spk_net* n, int32_t* G) {
  if (!n || !G) return SPK_ERR_INVALID;
  *G = n->G;
  return SPK_OK;
}

int spk_net_current_time(const spk_net* n, float* s) {
  if (!n || !s) return SPK_ERR_INVALID;
  *s = n->current_time;
  return SPK_OK;
}

static int read_store(spk_net* n, std::vector<uint2>& out) {
  SPK_CUDA(cudaStreamSynchronize(n->stream));
  RunCtl c;
  SPK_CUDA(cudaMemcpy(&c, n->hd.ctl, sizeof(c), cudaMemcpyDeviceToHost));
  const uint64_t cnt = std::min<uint64_t>(c.spike_count, (uint64_t)n->hd.spike_cap);
  out.resize(cnt);
  if (cnt) SPK_CUDA(cudaMemcpy(out.data(), n->hd.spikes, sizeof(uint2) * cnt, cudaMemcpyDeviceToHost));
  return SPK_OK;
}

int spk_net_spike_count(spk_net* n, int32_t population, int64_t* count) {
  if (!n || !count || population < 0 || population > 1) return SPK_ERR_INVALID;
  return guarded([&] {
    std::vector<uint2> st;
    int rc = read_store(n, st);
    if (rc) return rc;
    int64_t c = 0;
    for (const auto& e : st) c += ((int)e.x >= n->hd.KL) == (population == SPK_POP_NEURONS);
    *count = c;
    return SPK_OK;
  });
}

int spk_net_read_spikes(spk_net* n, int32_t population, int32_t* ids, float* times, int64_t capacity,
                        int64_t* n_written) {
  if (!n || population < 0 || population > 1 || capacity < 0) return SPK_ERR_INVALID;
  return guarded([&] {
    std::vector<uint2> st;
    int rc = read_store(n, st);
    if (rc) return rc;
    int64_t m = 0;
    for (const auto& e : st) {
      const int key = (int)e.x;
      const bool is_neuron = key >= n->hd.KL;
      if (is_neuron != (population == SPK_POP_NEURONS)) continue;
      if (m >= capacity) break;
      if (ids) ids[m] = is_neuron ? key - n->hd.KL : n->Nin - 1 - key;
      if (times) times[m] = u2f(e.y);
      ++m;
    }
    if (n_written) *n_written = m;
    return SPK_OK;
  });
}

int spk_net_clear_spikes(spk_net* n) {
  if (!n) return SPK_ERR_INVALID;
  clear_store_kernel<<<1, 1, 0, n->stream>>>(n->hd.ctl);
  SPK_CUDA(cudaGetLastError());
  return SPK_OK;
}

int spk_net_rate_counts(spk_net* n, int32_t population, int32_t* counts, int64_t count) {
  if (!n || !counts || population < 0 || population > 1) return SPK_ERR_INVALID;
  const int64_t want = population == SPK_POP_NEURONS ? n->N : n->Nin;
  if (count != want) {
    set_error("rate_counts: %lld counts asked, the population has %lld", (long long)count, (long long)want);
    return SPK_ERR_INVALID;
  }
  return guarded([&] {
    if (count == 0) return SPK_OK;
    SPK_CUDA(cudaStreamSynchronize(n->stream));
    if (population == SPK_POP_NEURONS) {
      SPK_CUDA(cudaMemcpy(counts, n->hd.rate_counts + n->hd.KL, sizeof(int32_t) * count, cudaMemcpyDeviceToHost));
    } else {
      // input i has key Nin - 1 - i
      std::vector<int32_t> by_key(count);
      SPK_CUDA(cudaMemcpy(by_key.data(), n->hd.rate_counts, sizeof(int32_t) * count, cudaMemcpyDeviceToHost));
      for (int64_t i = 0; i < count; ++i) counts[i] = by_key[count - 1 - i];
    }
    return SPK_OK;
  });
}

int spk_net_clear_rate_counts(spk_net* n) {
  if (!n) return SPK_ERR_INVALID;
  SPK_CUDA(cudaMemsetAsync(n->hd.rate_counts, 0, sizeof(int) * (size_t)n->hd.n_keys, n->stream));
  return SPK_OK;
}

int spk_net_read_state(spk_net* n, int32_t field, void* dst, int64_t count) {
  if (!n || !dst) return SPK_ERR_INVALID;
  return guarded([&]() -> int {
    SPK_CUDA(cudaStreamSynchronize(n->stream));
    const NetDev& h = n->hd;
    float* out = (float*)dst;
    auto need = [&](int64_t c) {
      if (count != c) {
        set_error("field %d holds %lld values, %lld requested", field, (long long)c, (long long)count);
        return false;
      }
      return true;
    };
    switch (field) {
      case SPK_FIELD_V:
        if (!need(n->N)) return SPK_ERR_INVALID;
        SPK_CUDA(cudaMemcpy(out, h.V, sizeof(float) * n->N, cudaMemcpyDeviceToHost));
        return SPK_OK;
      case SPK_FIELD_LAST_SPIKE:
        if (!need(n->N)) return SPK_ERR_INVALID;
        SPK_CUDA(cudaMemcpy(out, h.last, sizeof(float) * n->N, cudaMemcpyDeviceToHost));
        return SPK_OK;
      case SPK_FIELD_SYN_TRACE:
        if (!need((int64_t)n->N * n->L)) return SPK_ERR_INVALID;
        if (n->kind == SPK_SYN_VOLTAGE) {
          std::fill(out, out + count, 0.0f);
          return SPK_OK;
        }
        SPK_CUDA(cudaMemcpy(out, h.gtr, sizeof(float) * n->N * n->L, cudaMemcpyDeviceToHost));
        return SPK_OK;
      case SPK_FIELD_INPUT_NEXT:
        if (!need(n->Nin)) return SPK_ERR_INVALID;
        if (n->Nin) SPK_CUDA(cudaMemcpy(out, h.in_next, sizeof(float) * n->Nin, cudaMemcpyDeviceToHost));
        return SPK_OK;
      case SPK_FIELD_RING: {
        if (!need((int64_t)n->B * n->N * n->L)) return SPK_ERR_INVALID;
        std::vector<float> r((size_t)h.n_tiles * h.B * h.TS * h.L);
        SPK_CUDA(cudaMemcpy(r.data(), h.ring, sizeof(float) * r.size(), cudaMemcpyDeviceToHost));
        for (int slot = 0; slot < h.B; ++slot)
          for (int q = 0; q < n->N; ++q)
            for (int l = 0; l < h.L; ++l) {
              const int t = q / h.TS, ql = q % h.TS;
              out[((size_t)slot * n->N + q) * h.L + l] = r[(((size_t)t * h.B + slot) * h.TS + ql) * h.L + l];
            }
        return SPK_OK;
      }
      case SPK_FIELD_PRE_TRACE: {
        if (!need((int64_t)n->Nin + n->N)) return SPK_ERR_INVALID;
        if (!n->has_stdp) {
          std::fill(out, out + count, 0.0f);
          return SPK_OK;
        }
        std::vector<float> p(h.n_keys);
        SPK_CUDA(cudaMemcpy(p.data(), h.pre_trace, sizeof(float) * p.size(), cudaMemcpyDeviceToHost));
        for (int i = 0; i < n->Nin; ++i) out[i] = p[n->Nin - 1 - i];
        for (int q = 0; q < n->N; ++q) out[n->Nin + q] = p[h.KL + q];
        return SPK_OK;
      }
      case SPK_FIELD_POST_TRACE:
        if (!need(n->N)) return SPK_ERR_INVALID;
        if (!n->has_stdp) {
          std::fill(out, out + count, 0.0f);
          return SPK_OK;
        }
        SPK_CUDA(cudaMemcpy(out, h.post_trace, sizeof(float) * n->N, cudaMemcpyDeviceToHost));
        return SPK_OK;
      default:
        set_error("unknown state field %d", field);
        return SPK_ERR_INVALID;
    }
  });
}

int spk_net_read_weights(spk_net* n, float* w, int64_t count) {
  if (!n || (!w && count) || count != n->S) {
    set_error("weights: %lld requested, network has %lld synapses", (long long)count, n ? (long long)n->S : 0LL);
    return SPK_ERR_INVALID;
  }
  return guarded([&]() -> int {
    std::vector<uint2> csc;
    if (n->has_stdp) {
      SPK_CUDA(cudaStreamSynchronize(n->stream));
      csc.resize(n->n_csc);
      if (n->n_csc) SPK_CUDA(cudaMemcpy(csc.data(), n->hd.csc, sizeof(uint2) * n->n_csc, cudaMemcpyDeviceToHost));
    }
    if (n->generated) {
      // creation order = entry order; the value each synapse delivers
      SPK_CUDA(cudaStreamSynchronize(n->stream));
      std::vector<uint2> e(n->S);
      if (n->S) SPK_CUDA(cudaMemcpy(e.data(), n->hd.entries, sizeof(uint2) * n->S, cudaMemcpyDeviceToHost));
      for (int64_t s = 0; s < n->S; ++s) w[s] = (e[s].x >> 28) ? u2f(csc[e[s].y].y) : u2f(e[s].y);
      return SPK_OK;
    }
    if (n->has_stdp)
      for (int64_t s = 0; s < n->S; ++s)
        if (n->cls_of[s]) n->weights[s] = u2f(csc[n->csc_of[s]].y);
    std::memcpy(w, n->weights.data(), sizeof(float) * n->S);
    return SPK_OK;
  });
}

int spk_net_write_weights(spk_net* n, const float* w, int64_t count) {
  if (!n || (!w && count) || count != n->S) return SPK_ERR_INVALID;
  if (n->generated) {
    set_error("weights of a generated network cannot be written");
    return SPK_ERR_UNSUPPORTED;
  }
  return guarded([&]() -> int {
    SPK_CUDA(cudaStreamSynchronize(n->stream));
    std::vector<uint2> e(n->S), csc(n->n_csc);
    SPK_CUDA(cudaMemcpy(e.data(), n->hd.entries, sizeof(uint2) * n->S, cudaMemcpyDeviceToHost));
    if (n->n_csc) SPK_CUDA(cudaMemcpy(csc.data(), n->hd.csc, sizeof(uint2) * n->n_csc, cudaMemcpyDeviceToHost));
    for (int64_t s = 0; s < n->S; ++s) {
      n->weights[s] = w[s];
      if (n->cls_of[s])
        csc[n->csc_of[s]].y = f2u(w[s]);
      else
        e[n->entry_of[s]].y = f2u(w[s] * n->scales[s]);
    }
    SPK_CUDA(cudaMemcpy(n->hd.entries, e.data(), sizeof(uint2) * n->S, cudaMemcpyHostToDevice));
    if (n->n_csc) SPK_CUDA(cudaMemcpy(n->hd.csc, csc.data(), sizeof(uint2) * n->n_csc, cudaMemcpyHostToDevice));
    return SPK_OK;
  });
}

int spk_net_synaptic_events(spk_net* n, uint64_t* events) {
  if (!n || !events) return SPK_ERR_INVALID;
  SPK_CUDA(cudaStreamSynchronize(n->stream));
  RunCtl c;
  SPK_CUDA(cudaMemcpy(&c, n->hd.ctl, sizeof(c), cudaMemcpyDeviceToHost));
  *events = c.events;
  return SPK_OK;
}

int spk_net_stdp_counts(spk_net* n, uint64_t* pre_updates, uint64_t* post_updates) {
  if (!n) return SPK_ERR_INVALID;
  SPK_CUDA(cudaStreamSynchronize(n->stream));
  RunCtl c;
  SPK_CUDA(cudaMemcpy(&c, n->hd.ctl, sizeof(c), cudaMemcpyDeviceToHost));
  if (pre_updates) *pre_updates = c.stdp_pre;
  if (post_updates) *post_updates = c.stdp_post;
  return SPK_OK;
}

int spk_net_get_schedule(const spk_net* n, spk_schedule* out) {
  if (!n || !out) return SPK_ERR_INVALID;
  out->warps_per_cta = n->plan.W;
  out->tile_posts = n->plan.TS;
  out->ctas = n->plan.nctas;
  out->steps_per_launch = n->plan.K;
  return SPK_OK;
}

int spk_net_device_bytes(const spk_net* n, int64_t* bytes) {
  if (!n || !bytes) return SPK_ERR_INVALID;
  *bytes = (int64_t)n->arena_bytes;
  return SPK_OK;
}

int spk_net_launch_count(const spk_net* n, int64_t* launches) {
  if (!n || !launches) return SPK_ERR_INVALID;
  // runs of a network that takes bulk mode go through its own batch
  *launches = n->launches + (n->self_batch ? n->self_batch->launches : 0);
  return SPK_OK;
}

int spk_net_stream(const spk_net* n, void** stream) {
  if (!n || !stream) return SPK_ERR_INVALID;
  *stream = (void*)n->stream;
  return SPK_OK;
}

int spk_memory_info(uint64_t* free_bytes, uint64_t* total_bytes) {
  size_t f = 0, t = 0;
  SPK_CUDA(cudaMemGetInfo(&f, &t));
  if (free_bytes) *free_bytes = f;
  if (total_bytes) *total_bytes = t;
  return SPK_OK;
}

// ---- batch -------------------------------------------------------------------------
int spk_batch_create(spk_net* const* nets, int32_t n_nets, const spk_schedule* schedule, spk_batch** out) {
  if (!nets || n_nets < 1 || !out) return SPK_ERR_INVALID;
  return guarded([&]() -> int {
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    auto* b = new spk_batch();
    b->W = nets[0] ? nets[0]->plan.W : 0;
    b->K = (schedule && schedule->steps_per_launch > 0) ? schedule->steps_per_launch
                                                        : (nets[0] ? nets[0]->plan.K : DEFAULT_STEPS_PER_LAUNCH);
    // A batch holding a network that the persistent kernel cannot run (range
    // tiles) runs in bulk mode only: it has no waves, and its networks may
    // differ in warps per CTA.
    bool all_persistent = true;
    for (int i = 0; i < n_nets; ++i) all_persistent = all_persistent && nets[i] && nets[i]->plan.persistent;
    for (int i = 0; i < n_nets; ++i) {
      spk_net* n = nets[i];
      if (!n || (all_persistent && n->plan.W != b->W)) {
        set_error("all networks of a batch need the same warps_per_cta (net %d)", i);
        delete b;
        return SPK_ERR_INVALID;
      }
      for (int j = 0; j < i; ++j)
        if (nets[j] == n) {
          set_error("network %d appears twice in the batch", i);
          delete b;
          return SPK_ERR_INVALID;
        }
      b->nets.push_back(n);
      b->total_ctas += n->plan.nctas;
    }
    // Waves: co-resident sets of CTAs, one cooperative launch each.  Networks
    // are taken in decreasing shared-memory order so that each wave's launch
    // (which gives every CTA the wave's largest footprint) wastes little.
    std::vector<int> order(n_nets);
    for (int i = 0; i < n_nets; ++i) order[i] = i;
    // With step costs (spk_net_set_step_cost) the order is by decreasing
    // cost instead, so that each wave - which lasts as long as its slowest
    // network - holds networks of similar cost.
    bool costed = false;
    for (int i = 0; i < n_nets; ++i) costed |= nets[i]->step_cost > 0.0f;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
      if (costed && nets[a]->step_cost != nets[c]->step_cost) return nets[a]->step_cost > nets[c]->step_cost;
      if (nets[a]->plan.smem != nets[c]->plan.smem) return nets[a]->plan.smem > nets[c]->plan.smem;
      return nets[a]->plan.nctas > nets[c]->plan.nctas;
    });
    std::map<int, int> per_sm_of;
    auto capacity_at = [&](int smem, int* cap) -> int {
      auto it = per_sm_of.find(smem);
      int per_sm = 0;
      if (it == per_sm_of.end()) {
        SPK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, step_kernel, b->W * 32, smem));
        per_sm_of[smem] = per_sm;
      } else {
        per_sm = it->second;
      }
      *cap = per_sm * di.sms;
      return SPK_OK;
    };
    std::vector<CtaMap> map;
    map.reserve(b->total_ctas);
    spk_batch::Wave cur{0, 0, 0, false};
    if (!all_persistent) order.clear();
    for (int i : order) {
      spk_net* n = nets[i];
      int cap = 0;
      rc = capacity_at(std::max(cur.smem, n->plan.smem), &cap);
      if (rc) {
        delete b;
        return rc;
      }
      if (cur.ctas > 0 && cur.ctas + n->plan.nctas > cap) {
        b->waves.push_back(cur);
        cur = spk_batch::Wave{(int)map.size(), 0, 0, false};
        rc = capacity_at(n->plan.smem, &cap);
        if (rc) {
          delete b;
          return rc;
        }
      }
      if (n->plan.nctas > cap) {
        set_error("network %d needs %d co-resident CTAs, device holds %d", i, n->plan.nctas, cap);
        delete b;
        return SPK_ERR_UNSUPPORTED;
      }
      for (int r = 0; r < n->plan.nctas; ++r) map.push_back(CtaMap{i, r});
      cur.ctas += n->plan.nctas;
      cur.smem = std::max(cur.smem, n->plan.smem);
      cur.cooperative |= n->plan.nctas > 1;
    }
    if (all_persistent) b->waves.push_back(cur);
    std::vector<NetDev>& hds = b->hds;
    hds.resize(n_nets);
    for (int i = 0; i < n_nets; ++i) hds[i] = nets[i]->hd;
    const size_t bytes = align_up(sizeof(NetDev) * n_nets, 256) + align_up(sizeof(CtaMap) * map.size(), 256) + 256;
    void* mem = nullptr;
    if (cudaMalloc(&mem, bytes) != cudaSuccess) {
      cudaGetLastError();
      set_error("batch: device allocation failed");
      delete b;
      return SPK_ERR_OOM;
    }
    b->dd = (NetDev*)mem;
    b->dmap = (CtaMap*)((char*)mem + align_up(sizeof(NetDev) * n_nets, 256));
    b->abort_dev = (int*)((char*)b->dmap + align_up(sizeof(CtaMap) * map.size(), 256));
    for (int i = 0; i < n_nets; ++i) hds[i].abort_flag = b->abort_dev;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) != cudaSuccess ||
        cudaMemcpy(b->dd, hds.data(), sizeof(NetDev) * n_nets, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(b->dmap, map.data(), sizeof(CtaMap) * map.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(b->abort_dev, 0, sizeof(int)) != cudaSuccess) {
      set_error("batch: setup failed: %s", cudaGetErrorString(cudaGetLastError()));
      if (b->stream) cudaStreamDestroy(b->stream);
      if (b->done) cudaEventDestroy(b->done);
      cudaFree(mem);
      delete b;
      return SPK_ERR_CUDA;
    }
    // per-synapse-trace STDP rules and the weight normalisation run in bulk mode only
    bool any_bulk_only = false;
    for (int i = 0; i < n_nets; ++i) any_bulk_only = any_bulk_only || nets[i]->bulk_only();
    if (any_bulk_only) {
      const int rc = spk_batch_set_mode(b, SPK_BATCH_BULK);
      if (rc) {
        spk_batch_destroy(b);
        return rc;
      }
    }
    *out = b;
    return SPK_OK;
  });
}

namespace spk {

// One block of K timesteps in bulk mode and the run-counter update.  A
// timestep: neurons, list, [normalisation before the rule], [per-synapse-trace
// rules], [normalisation after them], the afferent pass beside propagation,
// and where a network normalises after the event-driven rule, that
// normalisation and a second propagation pass that delivers.
//
// With `timer`, each kernel is bracketed by CUDA events on the stream it runs
// on (the per-kernel timing of spk_batch_time_kernels; launches go direct).
struct KernelTimer {
  struct Mark {
    int kind;
    cudaEvent_t a, b;
  };
  std::vector<Mark> marks;
  size_t used = 0;
  int begin(int kind, cudaStream_t st) {
    if (used == marks.size()) {
      Mark m{kind, nullptr, nullptr};
      if (cudaEventCreate(&m.a) != cudaSuccess || cudaEventCreate(&m.b) != cudaSuccess) return SPK_ERR_CUDA;
      marks.push_back(m);
    }
    marks[used].kind = kind;
    return cudaEventRecord(marks[used].a, st) == cudaSuccess ? SPK_OK : SPK_ERR_CUDA;
  }
  int end(cudaStream_t st) { return cudaEventRecord(marks[used++].b, st) == cudaSuccess ? SPK_OK : SPK_ERR_CUDA; }
  // adds the recorded intervals to ms[kind] (after the stream completed)
  int collect(double* ms) {
    for (size_t i = 0; i < used; ++i) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, marks[i].a, marks[i].b) != cudaSuccess) return SPK_ERR_CUDA;
      ms[marks[i].kind] += t;
    }
    used = 0;
    return SPK_OK;
  }
  ~KernelTimer() {
    for (auto& m : marks) {
      cudaEventDestroy(m.a);
      cudaEventDestroy(m.b);
    }
  }
};

static int bulk_launch_block(spk_batch* b, KernelTimer* timer = nullptr) {
  const int n = (int)b->nets.size();
  const int prop_smem = bulk_prop_layout(b->win_words, b->ts_max).total * 4;
  const size_t range_bytes = range_smem_bytes(b->range_smem);
  DeviceInfo di;
  const int rc0 = device_info(&di);
  if (rc0) return rc0;
  const bool split = (b->norm_slots & 4) != 0;
  const int item_grid = std::min((b->n_dense_items + 7) / 8, di.sms * 8);
  // the neurons kernel: one resident wave of CTAs, each taking a run of blocks
  const int neur_grid = std::min(b->blocks_total, di.sms * SPK_BULK_NEUR_CTAS_PER_SM);
  int per_step = 0;
#define T_BEGIN(kind, st)                         \
  do {                                            \
    if (timer) {                                  \
      const int trc = timer->begin((kind), (st)); \
      if (trc) return trc;                        \
    }                                             \
  } while (0)
#define T_END(st)                      \
  do {                                 \
    if (timer) {                       \
      const int trc = timer->end((st)); \
      if (trc) return trc;             \
    }                                  \
  } while (0)
  for (int s = 0; s < b->K; ++s) {
    per_step = 0;
    T_BEGIN(SPK_KERNEL_NEURONS, b->stream);
    SPK_CUDA(launch_overlapped(bulk_neurons_kernel, neur_grid, BULK_NEUR_WARPS * 32, 0, b->stream,
                               (const NetDev*)b->dd, (const BulkBlock*)b->dblocks, b->blocks_total, s,
                               b->item_count));
    T_END(b->stream);
    T_BEGIN(SPK_KERNEL_LIST, b->stream);
    SPK_CUDA(launch_overlapped(bulk_list_kernel, n, BULK_LIST_THREADS, 0, b->stream, (const NetDev*)b->dd, s,
                               b->items, b->item_count, b->item_cap));
    T_END(b->stream);
    per_step += 2;
    if ((b->norm_slots & 1) && b->n_dense_items) {
      T_BEGIN(SPK_KERNEL_RULES, b->stream);
      bulk_norm_kernel<<<item_grid, 256, 0, b->stream>>>(b->dd, b->dense_items, b->n_dense_items, s, 0);
      T_END(b->stream);
      ++per_step;
    }
    if (b->any_dense && b->n_dense_items) {
      T_BEGIN(SPK_KERNEL_RULES, b->stream);
      bulk_dense_stdp_kernel<<<item_grid, 256, 0, b->stream>>>(b->dd, b->dense_items, b->n_dense_items, s);
      T_END(b->stream);
      ++per_step;
    }
    if ((b->norm_slots & 2) && b->n_dense_items) {
      T_BEGIN(SPK_KERNEL_RULES, b->stream);
      bulk_norm_kernel<<<item_grid, 256, 0, b->stream>>>(b->dd, b->dense_items, b->n_dense_items, s, 1);
      T_END(b->stream);
      ++per_step;
    }
    // the afferent pass runs beside propagation on the second stream; timed
    // runs put it on the batch stream so that each kernel has the GPU alone
    cudaStream_t post_stream = timer ? b->stream : b->side;
    if (b->any_plastic) {
      SPK_CUDA(cudaEventRecord(b->fork, b->stream));
      SPK_CUDA(cudaStreamWaitEvent(post_stream, b->fork, 0));
      T_BEGIN(SPK_KERNEL_POST, post_stream);
      bulk_post_kernel<<<di.sms * 8, 256, 0, post_stream>>>(b->dd, b->items, b->item_count, b->item_cap);
      T_END(post_stream);
      SPK_CUDA(cudaEventRecord(b->join, post_stream));
      ++per_step;
    }
    T_BEGIN(SPK_KERNEL_PROPAGATION, b->stream);
    if (b->pblocks_total) {
      SPK_CUDA(launch_overlapped(split ? bulk_prop_kernel<1> : bulk_prop_kernel<0>, b->pblocks_total,
                                 BULK_PROP_WARPS * 32, (size_t)prop_smem, b->stream, (const NetDev*)b->dd,
                                 (const BulkPropBlock*)b->dpblocks, s, b->win_words, b->ts_max));
      ++per_step;
    }
    if (b->rblocks_total) {
      SPK_CUDA(launch_overlapped(split ? bulk_range_kernel<1> : bulk_range_kernel<0>, b->rblocks_total,
                                 RANGE_THREADS, range_bytes, b->stream, (const NetDev*)b->dd,
                                 (const BulkRangeBlock*)b->drblocks, s, b->range_smem));
      ++per_step;
    }
    T_END(b->stream);
    if (b->any_plastic) SPK_CUDA(cudaStreamWaitEvent(b->stream, b->join, 0));
    if (split) {
      if (b->n_dense_items) {
        T_BEGIN(SPK_KERNEL_RULES, b->stream);
        bulk_norm_kernel<<<item_grid, 256, 0, b->stream>>>(b->dd, b->dense_items, b->n_dense_items, s, 2);
        T_END(b->stream);
        ++per_step;
      }
      T_BEGIN(SPK_KERNEL_PROPAGATION, b->stream);
      if (b->pblocks_total) {
        SPK_CUDA(launch_overlapped(bulk_prop_kernel<2>, b->pblocks_total, BULK_PROP_WARPS * 32,
                                   (size_t)prop_smem, b->stream, (const NetDev*)b->dd,
                                   (const BulkPropBlock*)b->dpblocks, s, b->win_words, b->ts_max));
        ++per_step;
      }
      if (b->rblocks_total) {
        SPK_CUDA(launch_overlapped(bulk_range_kernel<2>, b->rblocks_total, RANGE_THREADS, range_bytes, b->stream,
                                   (const NetDev*)b->dd, (const BulkRangeBlock*)b->drblocks, s, b->range_smem));
        ++per_step;
      }
      T_END(b->stream);
    }
  }
  T_BEGIN(SPK_KERNEL_FINISH, b->stream);
  bulk_finish_kernel<<<(n + 255) / 256, 256, 0, b->stream>>>(b->dd, n, b->K);
  T_END(b->stream);
  SPK_CUDA(cudaGetLastError());
#undef T_BEGIN
#undef T_END
  b->step_launches = per_step;
  return SPK_OK;
}

static int bulk_run_block(spk_batch* b) {
  if (!b->bulk_graph) {
    cudaGraph_t g = nullptr;
    SPK_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = bulk_launch_block(b);
    const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc != SPK_OK || e != cudaSuccess || cudaGraphInstantiate(&b->bulk_graph, g, 0) != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      b->bulk_graph = nullptr;
      const int rc2 = bulk_launch_block(b);  // launches go direct
      b->launches += (int64_t)b->step_launches * b->K + 1;
      return rc2;
    }
    cudaGraphDestroy(g);
  }
  SPK_CUDA(cudaGraphLaunch(b->bulk_graph, b->stream));
  b->launches += (int64_t)b->step_launches * b->K + 1;
  return SPK_OK;
}

// The batch holds its own copies of the networks' descriptors.  Two fields of a
// network's descriptor change after it joins a batch: the rates of the selected
// stimulus (select_stimulus, restore) and the wait limit.  Bring the copies up to
// date before a launch, on the batch stream, behind the launches already queued.
static int refresh_descs(spk_batch* b) {
  bool changed = false;
  for (size_t i = 0; i < b->nets.size(); ++i) {
    const NetDev& src = b->nets[i]->hd;
    NetDev& dst = b->hds[i];
    if (dst.rates != src.rates || dst.poll_ns != src.poll_ns) {
      dst.rates = src.rates;
      dst.poll_ns = src.poll_ns;
      changed = true;
    }
  }
  if (changed)
    SPK_CUDA(cudaMemcpyAsync(b->dd, b->hds.data(), sizeof(NetDev) * b->hds.size(), cudaMemcpyHostToDevice,
                             b->stream));
  return SPK_OK;
}

}  // namespace spk

int spk_batch_run_steps_each(spk_batch* b, const int64_t* n_steps, const int32_t* plasticity_on) {
  if (!b || !n_steps) return SPK_ERR_INVALID;
  int64_t most = 0;
  for (size_t i = 0; i < b->nets.size(); ++i) {
    if (n_steps[i] < 0 || n_steps[i] > 0x7fffffff) return SPK_ERR_INVALID;
    if (int rc = check_whole_groups(b->nets[i], n_steps[i])) return rc;
    most = std::max(most, n_steps[i]);
  }
  if (most == 0) return SPK_OK;
  // order the batch stream after each network's pending work
  for (size_t i = 0; i < b->nets.size(); ++i) {
    spk_net* n = b->nets[i];
    SPK_CUDA(cudaStreamSynchronize(n->stream));
    const int plastic = (!plasticity_on || plasticity_on[i]) && n->has_stdp;
    if (int rc = begin_run_on(n, b->stream, n->current_time, n_steps[i], plastic ? 1 : 0)) return rc;
  }
  if (int rc = refresh_descs(b)) return rc;
  // networks that finish early leave their launches at once (no steps left)
  const int64_t blocks = (most + b->K - 1) / b->K;
  for (int64_t blk = 0; blk < blocks; ++blk) {
    if (b->mode == SPK_BATCH_BULK) {
      int rc;
      if (b->timer) {
        rc = bulk_launch_block(b, b->timer);
        b->launches += (int64_t)b->step_launches * b->K + 1;
        if (rc == SPK_OK && (cudaStreamSynchronize(b->stream) != cudaSuccess ||
                             (b->side && cudaStreamSynchronize(b->side) != cudaSuccess)))
          rc = SPK_ERR_CUDA;
        if (rc == SPK_OK) rc = b->timer->collect(b->timer_ms);
      } else {
        rc = bulk_run_block(b);
      }
      if (rc) return rc;
      continue;
    }
    for (const auto& wv : b->waves) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(wv.ctas);
      cfg.blockDim = dim3(b->W * 32);
      cfg.dynamicSmemBytes = wv.smem;
      cfg.stream = b->stream;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeCooperative;
      attr[0].val.cooperative = wv.cooperative ? 1 : 0;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      SPK_CUDA(cudaLaunchKernelEx(&cfg, step_kernel, (const NetDev*)b->dd,
                                  (const CtaMap*)(b->dmap + wv.first), b->K));
      ++b->launches;
    }
  }
  // each network's own stream (its readbacks and runs) waits for the batch
  SPK_CUDA(cudaEventRecord(b->done, b->stream));
  for (size_t i = 0; i < b->nets.size(); ++i) {
    spk_net* n = b->nets[i];
    SPK_CUDA(cudaStreamWaitEvent(n->stream, b->done, 0));
    n->current_time = n->current_time + (float)n_steps[i] * n->dt;
  }
  return SPK_OK;
}


int spk_batch_set_mode(spk_batch* b, int32_t mode) {
  if (!b || (mode != SPK_BATCH_WAVES && mode != SPK_BATCH_BULK)) return SPK_ERR_INVALID;
  if (mode == b->mode) return SPK_OK;
  if (mode == SPK_BATCH_WAVES) {
    for (const spk_net* n : b->nets)
      if (n->bulk_only()) {
        set_error("waves mode: a network with a per-synapse-trace STDP rule, the weight normalisation or "
                  "range tiles runs in bulk mode only");
        return SPK_ERR_UNSUPPORTED;
      }
    b->mode = mode;
    return SPK_OK;
  }
  return guarded([&]() -> int {
    if (!b->bulk_mem) {
      std::vector<BulkPropBlock> tiles;
      std::vector<BulkRangeBlock> ranges;
      std::vector<BulkBlock> words;
      size_t list_words = 0;
      // propagation tile groups of the networks with the most keys first: their
      // warps walk the longest key lists, so they start before the short ones
      std::vector<int> by_keys(b->nets.size());
      for (size_t i = 0; i < by_keys.size(); ++i) by_keys[i] = (int)i;
      std::stable_sort(by_keys.begin(), by_keys.end(),
                       [&](int x, int y) { return b->nets[x]->plan.n_keys > b->nets[y]->plan.n_keys; });
      for (const int i : by_keys) {
        if (b->nets[i]->plan.TS >= RANGE_MIN_TS) continue;
        for (int t = 0; t < b->nets[i]->plan.n_tiles; t += BULK_PROP_WARPS)
          tiles.push_back(BulkPropBlock{i, t, std::min(BULK_PROP_WARPS, b->nets[i]->plan.n_tiles - t), 0,
                                        b->hds[i].ctl, nullptr});
      }
      // ranges (one CTA each) of the networks with the most synapses per range first
      std::vector<int> by_load(b->nets.size());
      for (size_t i = 0; i < by_load.size(); ++i) by_load[i] = (int)i;
      auto load_of = [&](int i) { return (double)b->nets[i]->S / b->nets[i]->plan.n_tiles; };
      std::stable_sort(by_load.begin(), by_load.end(), [&](int x, int y) { return load_of(x) > load_of(y); });
      for (const int i : by_load) {
        if (b->nets[i]->plan.TS < RANGE_MIN_TS) continue;
        for (int t = 0; t < b->nets[i]->plan.n_tiles; ++t)
          ranges.push_back(BulkRangeBlock{i, t, 0, 0, b->hds[i].ctl, nullptr});
      }
      for (size_t i = 0; i < b->nets.size(); ++i) {
        const spk_net* n = b->nets[i];
        const int in_end = (n->Nin + 31) / 32, lif0 = n->plan.KL / 32, lif_end = (n->plan.KL + n->N + 31) / 32;
        for (int w = 0; w < in_end; w += BULK_BLOCK_WORDS)
          words.push_back(BulkBlock{(int)i, w, std::min(BULK_BLOCK_WORDS, in_end - w), 0, b->hds[i].ctl, nullptr});
        for (int w = lif0; w < lif_end; w += BULK_BLOCK_WORDS)
          words.push_back(BulkBlock{(int)i, w, std::min(BULK_BLOCK_WORDS, lif_end - w), 0, b->hds[i].ctl, nullptr});
        list_words += (size_t)n->plan.n_keys;
      }
      // afferent-pass items: at most one per post of every plastic network
      size_t cap = 0;
      for (const spk_net* n : b->nets)
        if (n->has_stdp) {
          cap += (size_t)n->N;
          b->any_plastic = true;
        }
      if (cap > 0x7fffffff) {
        set_error("bulk mode: the batch's afferent-pass list would exceed 2^31 items");
        return SPK_ERR_UNSUPPORTED;
      }
      b->item_cap = (int)cap;
      // posts of the networks with a per-synapse-trace rule or the weight
      // normalisation: the per-post passes
      {
        std::vector<BulkRuleItem> dense;
        b->any_dense = false;
        b->norm_slots = 0;
        for (size_t i = 0; i < b->nets.size(); ++i) {
          const spk_net* x = b->nets[i];
          if (!x->bulk_only()) continue;
          b->any_dense = b->any_dense || x->dense();
          if (x->weight_norm != SPK_NORM_OFF) b->norm_slots |= 1 << x->norm_slot();
          // the record ranges (uploaded or generated on the network's stream)
          std::vector<int32_t> cp((size_t)x->N + 1);
          SPK_CUDA(cudaStreamSynchronize(x->stream));
          SPK_CUDA(cudaMemcpy(cp.data(), x->hd.csc_ptr, sizeof(int32_t) * cp.size(), cudaMemcpyDeviceToHost));
          for (int q = 0; q < x->N; ++q)
            if (cp[q + 1] > cp[q]) dense.push_back(BulkRuleItem{(int)i, q, cp[q], cp[q + 1]});
        }
        if (!dense.empty()) {
          if (cudaMalloc(&b->dense_items, sizeof(BulkRuleItem) * dense.size()) != cudaSuccess) {
            cudaGetLastError();
            b->dense_items = nullptr;
            set_error("bulk mode: device allocation failed");
            return SPK_ERR_OOM;
          }
          SPK_CUDA(cudaMemcpy(b->dense_items, dense.data(), sizeof(BulkRuleItem) * dense.size(),
                              cudaMemcpyHostToDevice));
          b->n_dense_items = (int)dense.size();
        }
      }
      if (b->any_plastic && !b->side &&
          (cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
           cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
           cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess)) {
        cudaGetLastError();
        set_error("bulk mode: stream or event creation failed");
        return SPK_ERR_CUDA;
      }
      // ring windows: the longest delay's slots of the largest tile, capped
      b->win_words = 0;
      b->ts_max = 0;
      for (const spk_net* n : b->nets) {
        if (n->hd.TS >= RANGE_MIN_TS) continue;
        b->ts_max = std::max(b->ts_max, n->hd.TS);
        b->win_words = std::max(b->win_words, (n->hd.B - 2 * n->hd.G - 1) * n->hd.TS * n->hd.L);
      }
      b->win_words = std::min(b->win_words, BULK_WIN_CAP);
      // range windows: as many of a range's delay slots as the cap holds;
      // bucket heads: one per delay cell of the D_max slots where they fit
      b->range_smem = RangeSmem{0, 0};
      for (const spk_net* n : b->nets) {
        if (n->hd.TS < RANGE_MIN_TS) continue;
        const int slot_words = n->hd.TS * n->hd.L;
        const int ws = std::min(n->hd.B - 2 * n->hd.G - 1, RANGE_WIN_CAP / slot_words);
        b->range_smem.win_words = std::max(b->range_smem.win_words, ws * slot_words);
        b->range_smem.head_words =
            std::max(b->range_smem.head_words, std::min((n->hd.B - 2 * n->hd.G - 1) * slot_words, RANGE_HEAD_CAP));
      }
      const size_t r_bytes = align_up(sizeof(BulkRangeBlock) * ranges.size(), 256);
      const size_t t_bytes = align_up(sizeof(BulkPropBlock) * tiles.size(), 256);
      const size_t w_bytes = align_up(sizeof(BulkBlock) * words.size(), 256);
      const size_t l_bytes = align_up(sizeof(uint32_t) * list_words, 256);
      const size_t c_bytes = align_up(sizeof(int) * (b->nets.size() + 1), 256);
      const size_t i_bytes = align_up(sizeof(BulkPostItem) * std::max<size_t>(cap, 1), 256);
      if (cudaMalloc(&b->bulk_mem, t_bytes + w_bytes + l_bytes + c_bytes + i_bytes + r_bytes) != cudaSuccess) {
        cudaGetLastError();
        b->bulk_mem = nullptr;
        set_error("bulk mode: device allocation failed");
        return SPK_ERR_OOM;
      }
      b->dpblocks = (BulkPropBlock*)b->bulk_mem;
      b->pblocks_total = (int)tiles.size();
      b->dblocks = (BulkBlock*)((char*)b->bulk_mem + t_bytes);
      b->blocks_total = (int)words.size();
      uint32_t* lists = (uint32_t*)((char*)b->bulk_mem + t_bytes + w_bytes);
      int* counts = (int*)((char*)b->bulk_mem + t_bytes + w_bytes + l_bytes);
      b->item_count = counts + b->nets.size();
      b->items = (BulkPostItem*)((char*)b->bulk_mem + t_bytes + w_bytes + l_bytes + c_bytes);
      b->drblocks = (BulkRangeBlock*)((char*)b->bulk_mem + t_bytes + w_bytes + l_bytes + c_bytes + i_bytes);
      b->rblocks_total = (int)ranges.size();
      size_t off = 0;
      for (size_t i = 0; i < b->nets.size(); ++i) {
        b->hds[i].step_list = lists + off;
        b->hds[i].step_count = counts + i;
        off += (size_t)b->nets[i]->plan.n_keys;
      }
      for (BulkPropBlock& pb : tiles) pb.n_list = counts + pb.net;
      for (BulkRangeBlock& rb : ranges) rb.n_list = counts + rb.net;
      SPK_CUDA(cudaMemcpy(b->dpblocks, tiles.data(), sizeof(BulkPropBlock) * tiles.size(), cudaMemcpyHostToDevice));
      SPK_CUDA(cudaMemcpy(b->drblocks, ranges.data(), sizeof(BulkRangeBlock) * ranges.size(),
                          cudaMemcpyHostToDevice));
      SPK_CUDA(cudaMemcpy(b->dblocks, words.data(), sizeof(BulkBlock) * words.size(), cudaMemcpyHostToDevice));
      // words of padding keys are never written in bulk mode: zero them once
      SPK_CUDA(cudaStreamSynchronize(b->stream));
      for (const spk_net* n : b->nets) {
        SPK_CUDA(cudaStreamSynchronize(n->stream));
        SPK_CUDA(cudaMemset(n->hd.bitsA, 0, sizeof(uint32_t) * 2 * (size_t)n->hd.n_words));
        SPK_CUDA(cudaMemset(n->hd.bitsP, 0, sizeof(uint32_t) * 2 * (size_t)n->hd.n_words));
        SPK_CUDA(cudaMemset(n->hd.bitsE, 0, sizeof(uint32_t) * (size_t)n->hd.n_words));
      }
      SPK_CUDA(cudaMemcpy(b->dd, b->hds.data(), sizeof(NetDev) * b->hds.size(), cudaMemcpyHostToDevice));
      const int prop_smem = bulk_prop_layout(b->win_words, b->ts_max).total * 4;
      const int range_smem = (int)range_smem_bytes(b->range_smem);
      int prop_max = 0, range_max = 0;
      if (int rc = allow_all_dynamic_smem(bulk_prop_kernel<0>, &prop_max)) return rc;
      if (int rc = allow_all_dynamic_smem(bulk_prop_kernel<1>, &prop_max)) return rc;
      if (int rc = allow_all_dynamic_smem(bulk_prop_kernel<2>, &prop_max)) return rc;
      if (int rc = allow_all_dynamic_smem(bulk_range_kernel<0>, &range_max)) return rc;
      if (int rc = allow_all_dynamic_smem(bulk_range_kernel<1>, &range_max)) return rc;
      if (int rc = allow_all_dynamic_smem(bulk_range_kernel<2>, &range_max)) return rc;
      if ((b->pblocks_total && prop_smem > prop_max) || (b->rblocks_total && range_smem > range_max)) {
        set_error("bulk mode: propagation needs %d / %d B of shared memory per CTA, the device allows %d / %d",
                  prop_smem, range_smem, prop_max, range_max);
        return SPK_ERR_INVALID;
      }
    }
    b->mode = mode;
    return SPK_OK;
  });
}

int spk_batch_step_block(spk_batch* b) {
  if (!b) return SPK_ERR_INVALID;
  // order the batch stream after each network's pending work (its run set-up)
  for (spk_net* n : b->nets) SPK_CUDA(cudaStreamSynchronize(n->stream));
  if (int rc = refresh_descs(b)) return rc;
  if (b->mode == SPK_BATCH_BULK) {
    const int rc = bulk_run_block(b);
    if (rc) return rc;
    SPK_CUDA(cudaEventRecord(b->done, b->stream));
    for (spk_net* n : b->nets) SPK_CUDA(cudaStreamWaitEvent(n->stream, b->done, 0));
    return SPK_OK;
  }
  for (const auto& wv : b->waves) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(wv.ctas);
    cfg.blockDim = dim3(b->W * 32);
    cfg.dynamicSmemBytes = wv.smem;
    cfg.stream = b->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = wv.cooperative ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SPK_CUDA(cudaLaunchKernelEx(&cfg, step_kernel, (const NetDev*)b->dd, (const CtaMap*)(b->dmap + wv.first),
                                b->K));
    ++b->launches;
  }
  SPK_CUDA(cudaEventRecord(b->done, b->stream));
  for (spk_net* n : b->nets) SPK_CUDA(cudaStreamWaitEvent(n->stream, b->done, 0));
  return SPK_OK;
}

int spk_batch_run_steps(spk_batch* b, int64_t n_steps, int32_t plasticity_on) {
  if (!b || n_steps < 0 || n_steps > 0x7fffffff) return SPK_ERR_INVALID;
  if (n_steps == 0) return SPK_OK;
  return guarded([&]() -> int {
    std::vector<int64_t> each(b->nets.size(), n_steps);
    std::vector<int32_t> plastic(b->nets.size(), plasticity_on ? 1 : 0);
    return spk_batch_run_steps_each(b, each.data(), plastic.data());
  });
}

int spk_batch_time_kernels(spk_batch* b, int64_t n_steps, int32_t plasticity_on, double* ms) {
  if (!b || !ms || n_steps < 0 || n_steps > 0x7fffffff) return SPK_ERR_INVALID;
  if (b->mode != SPK_BATCH_BULK) {
    set_error("per-kernel timing needs a batch in bulk mode");
    return SPK_ERR_UNSUPPORTED;
  }
  if (n_steps == 0) return SPK_OK;
  return guarded([&]() -> int {
    KernelTimer timer;
    b->timer = &timer;
    b->timer_ms = ms;
    std::vector<int64_t> each(b->nets.size(), n_steps);
    std::vector<int32_t> plastic(b->nets.size(), plasticity_on ? 1 : 0);
    const int rc = spk_batch_run_steps_each(b, each.data(), plastic.data());
    b->timer = nullptr;
    b->timer_ms = nullptr;
    return rc;
  });
}

int spk_batch_synchronize(spk_batch* b) {
  if (!b) return SPK_ERR_INVALID;
  SPK_CUDA(cudaStreamSynchronize(b->stream));
  int worst = SPK_OK;
  for (spk_net* n : b->nets) {
    int st = 0;
    SPK_CUDA(cudaMemcpy(&st, &n->hd.ctl->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st == SPK_ERR_TIMEOUT) worst = st;
    else if (st && worst == SPK_OK) worst = st;
  }
  return worst;
}

int spk_batch_launch_count(const spk_batch* b, int64_t* launches) {
  if (!b || !launches) return SPK_ERR_INVALID;
  *launches = b->launches;
  return SPK_OK;
}

int spk_batch_stream(const spk_batch* b, void** stream) {
  if (!b || !stream) return SPK_ERR_INVALID;
  *stream = (void*)b->stream;
  return SPK_OK;
}

// ---- spike readback of a whole batch ------------------------------------------------------
namespace spk {
constexpr int SPIKE_CHUNK = 4096;  // store entries per gather CTA
struct SpikeChunk {
  int net;
  int n;             // entries in the chunk
  long long start;   // first entry of the network's store
  long long out;     // first output slot of its matching entries
};

__global__ void spike_counts_kernel(const NetDev* __restrict__ nets, int n_nets, unsigned long long* counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nets) return;
  const unsigned long long c = nets[i].ctl->spike_count;
  const unsigned long long cap = (unsigned long long)nets[i].spike_cap;
  counts[i] = c < cap ? c : cap;
}

// Entries of `population` in each chunk (networks that record their inputs
// mix both populations in one store).
__global__ void spike_match_kernel(const NetDev* __restrict__ nets, const SpikeChunk* __restrict__ chunks,
                                   int population, int* matches) {
  __shared__ int s_tot;
  const SpikeChunk ch = chunks[blockIdx.x];
  const NetDev& d = nets[ch.net];
  if (threadIdx.x == 0) s_tot = 0;
  __syncthreads();
  int m = 0;
  for (int i = threadIdx.x; i < ch.n; i += blockDim.x) {
    const bool is_neuron = (int)d.spikes[ch.start + i].x >= d.KL;
    m += is_neuron == (population == SPK_POP_NEURONS);
  }
  atomicAdd(&s_tot, m);
  __syncthreads();
  if (threadIdx.x == 0) matches[blockIdx.x] = s_tot;
}

// Matching entries of each chunk, in store order, as (id, time) at the
// chunk's output slot (ids as spk_net_read_spikes gives them).
__global__ void __launch_bounds__(256) spike_gather_kernel(const NetDev* __restrict__ nets,
                                                           const SpikeChunk* __restrict__ chunks, int population,
                                                           int32_t* ids, float* times) {
  __shared__ int warp_n[8];
  const SpikeChunk ch = chunks[blockIdx.x];
  const NetDev& d = nets[ch.net];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int KL = d.KL, Nin = d.Nin;
  long long out = ch.out;
  for (int base = 0; base < ch.n; base += 256) {
    const int i = base + (int)threadIdx.x;
    uint2 e = make_uint2(0u, 0u);
    bool m = false;
    if (i < ch.n) {
      e = d.spikes[ch.start + i];
      m = ((int)e.x >= KL) == (population == SPK_POP_NEURONS);
    }
    const unsigned bal = __ballot_sync(0xffffffffu, m);
    if (lane == 0) warp_n[w] = __popc(bal);
    __syncthreads();
    int before = 0, total = 0;
    for (int k = 0; k < 8; ++k) {
      before += k < w ? warp_n[k] : 0;
      total += warp_n[k];
    }
    if (m) {
      const long long o = out + before + __popc(bal & ((1u << lane) - 1u));
      const int key = (int)e.x;
      ids[o] = key >= KL ? key - KL : Nin - 1 - key;
      times[o] = __uint_as_float(e.y);
    }
    out += total;
    __syncthreads();
  }
}

__global__ void clear_stores_kernel(const NetDev* __restrict__ nets, int n_nets) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nets) return;
  RunCtl* ctl = nets[i].ctl;
  ctl->spike_count = 0ull;
  if (ctl->status == SPK_ERR_OVERFLOW) ctl->status = 0;
}
}  // namespace spk

int spk_batch_read_spikes(spk_batch* b, int32_t population, int32_t* ids, float* times, int64_t capacity,
                          int64_t* counts, int32_t clear) {
  if (!b || population < 0 || population > 1 || capacity < 0 || !counts) return SPK_ERR_INVALID;
  return guarded([&]() -> int {
    const int n = (int)b->nets.size();
    // after each network's own stream (per-network calls, runs alone)
    if (!b->rd) SPK_CUDA(cudaEventCreateWithFlags(&b->rd, cudaEventDisableTiming));
    for (spk_net* nt : b->nets) {
      SPK_CUDA(cudaEventRecord(b->rd, nt->stream));
      SPK_CUDA(cudaStreamWaitEvent(b->stream, b->rd, 0));
    }
    const size_t c_bytes = align_up(sizeof(unsigned long long) * n, 256);
    auto scratch = [&](size_t bytes) -> int {
      if (bytes <= b->rb_bytes) return SPK_OK;
      if (b->rb_mem) cudaFree(b->rb_mem);
      b->rb_mem = nullptr;
      b->rb_bytes = 0;
      if (cudaMalloc(&b->rb_mem, bytes) != cudaSuccess) {
        cudaGetLastError();
        set_error("spike readback: device allocation failed");
        return SPK_ERR_OOM;
      }
      b->rb_bytes = bytes;
      return SPK_OK;
    };
    int rc = scratch(c_bytes);
    if (rc) return rc;
    unsigned long long* dcounts = (unsigned long long*)b->rb_mem;
    spike_counts_kernel<<<(n + 255) / 256, 256, 0, b->stream>>>(b->dd, n, dcounts);
    std::vector<unsigned long long> stored(n);
    SPK_CUDA(cudaMemcpyAsync(stored.data(), dcounts, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost,
                             b->stream));
    SPK_CUDA(cudaStreamSynchronize(b->stream));
    std::vector<SpikeChunk> chunks;
    bool mixed = false;
    for (int i = 0; i < n; ++i) {
      mixed = mixed || b->nets[i]->record_inputs;
      for (unsigned long long st = 0; st < stored[i]; st += SPIKE_CHUNK)
        chunks.push_back(SpikeChunk{i, (int)std::min<unsigned long long>(SPIKE_CHUNK, stored[i] - st),
                                    (long long)st, 0});
    }
    const int nch = (int)chunks.size();
    const size_t ch_bytes = align_up(sizeof(SpikeChunk) * std::max(nch, 1), 256);
    const size_t m_bytes = align_up(sizeof(int) * std::max(nch, 1), 256);
    rc = scratch(c_bytes + ch_bytes + m_bytes);
    if (rc) return rc;
    SpikeChunk* dchunks = (SpikeChunk*)((char*)b->rb_mem + c_bytes);
    int* dmatch = (int*)((char*)b->rb_mem + c_bytes + ch_bytes);
    std::vector<int> match(nch);
    if (mixed && nch) {
      SPK_CUDA(cudaMemcpyAsync(dchunks, chunks.data(), sizeof(SpikeChunk) * nch, cudaMemcpyHostToDevice, b->stream));
      spike_match_kernel<<<nch, 256, 0, b->stream>>>(b->dd, dchunks, population, dmatch);
      SPK_CUDA(cudaMemcpyAsync(match.data(), dmatch, sizeof(int) * nch, cudaMemcpyDeviceToHost, b->stream));
      SPK_CUDA(cudaStreamSynchronize(b->stream));
    } else {
      // a store without inputs holds neuron spikes only
      for (int c = 0; c < nch; ++c) match[c] = population == SPK_POP_NEURONS ? chunks[c].n : 0;
    }
    long long total = 0;
    for (int i = 0; i < n; ++i) counts[i] = 0;
    for (int c = 0; c < nch; ++c) {
      chunks[c].out = total;
      total += match[c];
      counts[chunks[c].net] += match[c];
    }
    if (total > capacity) {
      set_error("spike readback: %lld spikes exceed the capacity %lld", total, (long long)capacity);
      return SPK_ERR_OVERFLOW;
    }
    if (total > 0) {
      if (total > b->rb_cap) {
        if (b->rb_ids) cudaFree(b->rb_ids);
        if (b->rb_times) cudaFree(b->rb_times);
        b->rb_ids = nullptr;
        b->rb_times = nullptr;
        b->rb_cap = 0;
        const int64_t cap = total + total / 4;
        if (cudaMalloc(&b->rb_ids, sizeof(int32_t) * cap) != cudaSuccess ||
            cudaMalloc(&b->rb_times, sizeof(float) * cap) != cudaSuccess) {
          cudaGetLastError();
          set_error("spike readback: device allocation failed");
          return SPK_ERR_OOM;
        }
        b->rb_cap = cap;
      }
      SPK_CUDA(cudaMemcpyAsync(dchunks, chunks.data(), sizeof(SpikeChunk) * nch, cudaMemcpyHostToDevice, b->stream));
      spike_gather_kernel<<<nch, 256, 0, b->stream>>>(b->dd, dchunks, population, b->rb_ids, b->rb_times);
      SPK_CUDA(cudaGetLastError());
      if (ids)
        SPK_CUDA(cudaMemcpyAsync(ids, b->rb_ids, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, b->stream));
      if (times)
        SPK_CUDA(cudaMemcpyAsync(times, b->rb_times, sizeof(float) * total, cudaMemcpyDeviceToHost, b->stream));
    }
    if (clear) clear_stores_kernel<<<(n + 255) / 256, 256, 0, b->stream>>>(b->dd, n);
    SPK_CUDA(cudaGetLastError());
    // later calls on the networks' own streams see the cleared stores
    SPK_CUDA(cudaEventRecord(b->rd, b->stream));
    for (spk_net* nt : b->nets) SPK_CUDA(cudaStreamWaitEvent(nt->stream, b->rd, 0));
    SPK_CUDA(cudaStreamSynchronize(b->stream));
    return SPK_OK;
  });
}

int spk_batch_destroy(spk_batch* b) {
  if (!b) return SPK_ERR_INVALID;
  if (b->stream) {
    cudaStreamSynchronize(b->stream);
    cudaStreamDestroy(b->stream);
  }
  if (b->done) cudaEventDestroy(b->done);
  if (b->side) {
    cudaStreamSynchronize(b->side);
    cudaStreamDestroy(b->side);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  if (b->rd) cudaEventDestroy(b->rd);
  if (b->dense_items) cudaFree(b->dense_items);
  if (b->rb_mem) cudaFree(b->rb_mem);
  if (b->rb_ids) cudaFree(b->rb_ids);
  if (b->rb_times) cudaFree(b->rb_times);
  if (b->bulk_graph) cudaGraphExecDestroy(b->bulk_graph);
  if (b->bulk_mem) cudaFree(b->bulk_mem);
  cudaFree(b->dd);
  delete b;
  return SPK_OK;
}

}  // extern "C"

// =====================================================================================
// Allocation-free stepping: the step kernel over caller-owned network buffers.
// The only device memory the library supplies is the fixed scratch array below,
// which holds what the step exchanges between CTAs plus the launch descriptors.
namespace spk {

// Scratch of spk_step_noalloc.  Every device that loads the library holds this
// array until the process exits; every call on a device shares it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[SPK_NOALLOC_SCRATCH_BYTES];

static_assert(sizeof(RunCtl) <= SPK_RUN_STATE_BYTES, "RunCtl does not fit the caller's run state");
static_assert(offsetof(RunCtl, spike_count) == 32 && offsetof(RunCtl, events) == 40 &&
                  offsetof(RunCtl, status) == 48,
              "run state offsets published in spike_gb300.h");

struct NoallocDevice {
  bool ready = false;
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
  DeviceInfo di;
};
constexpr int NOALLOC_MAX_DEVICES = 64;
static NoallocDevice g_noalloc_dev[NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mu;

// Resolves the scratch address and the step kernel's shared-memory limit of the
// current device, once per device (on the first call made with it current).
static int noalloc_device(NoallocDevice** out) {
  int dev = 0;
  SPK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
    set_error("device %d is beyond the %d devices spk_step_noalloc tracks", dev, NOALLOC_MAX_DEVICES);
    return SPK_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  NoallocDevice& nd = g_noalloc_dev[dev];
  if (!nd.ready) {
    unsigned char* ptr = nullptr;
    SPK_CUDA(cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch));
    DeviceInfo di;
    const int rc = device_info(&di);
    if (rc) return rc;
    SPK_CUDA(cudaFuncSetAttribute(step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, di.max_smem));
    nd.scratch = ptr;
    nd.di = di;
    nd.ready = true;
  }
  *out = &nd;
  return SPK_OK;
}

// Writes the network descriptor and CTA map into the scratch and clears the
// exchange stamps and keys and the abort flag.  The stamps and keys must
// start at zero: a word left by an earlier call of another network (or of
// this one after its step counter was reset) can carry a stamp this call also
// produces.  The run is then started in the caller's run state
// (set_ctl_kernel).
static __global__ void noalloc_setup_kernel(NetDev nd, NetDev* nd_out, CtaMap* map, unsigned long long* xchg,
                                            size_t xchg_words) {
  const size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = i0; i < xchg_words; i += stride) xchg[i] = 0ull;
  for (size_t r = i0; r < (size_t)nd.nctas; r += stride) map[r] = CtaMap{0, (int)r};
  if (i0 == 0) {
    *nd_out = nd;
    *nd.abort_flag = 0;
  }
}

static bool aligned(const void* p, uintptr_t a) { return ((uintptr_t)p & (a - 1)) == 0; }

static int step_noalloc_impl(const spk_device_net* a, int64_t n_steps, int plasticity_on, float start,
                             cudaStream_t stream) {
  if (!a) {
    set_error("null network");
    return SPK_ERR_INVALID;
  }
  if (n_steps < 0 || n_steps > 0x7fffffff) {
    set_error("step count %lld outside [0, 2^31-1]", (long long)n_steps);
    return SPK_ERR_INVALID;
  }
  const int N = a->n_neurons, Nin = a->n_inputs, L = a->n_labels, kind = a->synapse_kind;
  const int W = a->warps_per_cta, TS = a->tile_posts, C = a->ctas;
  const int stdp = a->has_stdp ? 1 : 0;
  if (N <= 0 || Nin < 0 || L < 1 || L > MAX_LABELS || !(a->dt > 0.0f) || a->max_delay < 1 ||
      a->max_delay > MAX_DELAY) {
    set_error("sizes out of range (neurons %d, inputs %d, labels %d, max delay %d)", N, Nin, L, a->max_delay);
    return SPK_ERR_INVALID;
  }
  if (kind != SPK_SYN_CONDUCTANCE && kind != SPK_SYN_CURRENT && kind != SPK_SYN_VOLTAGE) {
    set_error("unknown synapse kind %d", kind);
    return SPK_ERR_INVALID;
  }
  if (W < 1 || W > 16 || TS < 32 || TS % 32 || TS > 65504 || C < 1 || C > MAX_CTAS_PER_NET) {
    set_error("schedule W=%d tile=%d ctas=%d: need 1 <= W <= 16, tile a multiple of 32, 1 <= ctas <= %d", W, TS, C,
              MAX_CTAS_PER_NET);
    return SPK_ERR_INVALID;
  }
  if (a->n_groups < 1 || a->n_groups > MAX_GROUPS || !a->groups) {
    set_error("between 1 and %d neuron groups are supported (got %d)", MAX_GROUPS, a->n_groups);
    return SPK_ERR_INVALID;
  }
  {
    int expect = 0;
    for (int g = 0; g < a->n_groups; ++g) {
      if (a->groups[g].start != expect || a->groups[g].count <= 0) {
        set_error("neuron groups must be contiguous, ascending and non-empty");
        return SPK_ERR_INVALID;
      }
      expect += a->groups[g].count;
    }
    if (expect != N) {
      set_error("neuron groups cover %d neurons, the network has %d", expect, N);
      return SPK_ERR_INVALID;
    }
  }
  if ((kind != SPK_SYN_VOLTAGE && !a->label_tau) || (kind == SPK_SYN_CONDUCTANCE && !a->label_vhat)) {
    set_error("conductance/current synapses need label_tau (and label_vhat for conductance)");
    return SPK_ERR_INVALID;
  }
  const int G = a->timestep_grouping > 1 ? a->timestep_grouping : 1;
  if (G > a->max_delay || (G > 1 && stdp) || n_steps % G != 0) {
    set_error("timestep grouping %d: needs at most the maximum delay %d, no plasticity, and whole groups "
              "(%lld timesteps)", G, a->max_delay, (long long)n_steps);
    return SPK_ERR_INVALID;
  }
  if (stdp && (a->n_plastic_scales < 0 || a->n_plastic_scales >= MAX_CLASSES ||
               (a->n_plastic_scales > 0 && !a->plastic_scales))) {
    set_error("between 0 and %d plastic weight scales are supported", MAX_CLASSES - 1);
    return SPK_ERR_INVALID;
  }
  {
    const int rc = check_time_constants(a->dt, a->groups, a->n_groups, kind, L, a->label_tau, a->refractory_period,
                                        stdp != 0, a->stdp);
    if (rc) return rc;
  }
  if (!a->rowptr || !a->entries || !a->V || !a->last_spike || !a->ring || !a->run_state ||
      (kind != SPK_SYN_VOLTAGE && !a->syn_trace) || (Nin > 0 && (!a->input_next || !a->rates)) ||
      (stdp && (!a->csc_ptr || !a->csc || !a->post_trace || !a->pre_trace)) ||
      (a->spike_capacity > 0 && !a->spikes) || a->spike_capacity < 0) {
    set_error("a device buffer the network needs is missing");
    return SPK_ERR_INVALID;
  }
  if (!aligned(a->entries, 8) || !aligned(a->csc, 8) || !aligned(a->spikes, 8) || !aligned(a->run_state, 8)) {
    set_error("entries, csc, spikes and run_state must be 8-byte aligned");
    return SPK_ERR_INVALID;
  }
  const int B = a->max_delay + 2 * G + 1;  // SpikingSynapses.cu:48
  const int n_tiles = W * C;
  if ((int64_t)n_tiles * TS < N) {
    set_error("schedule W=%d tile=%d ctas=%d covers %lld of %d neurons", W, TS, C, (long long)n_tiles * TS, N);
    return SPK_ERR_INVALID;
  }
  const int ITS = Nin > 0 ? ((Nin + n_tiles - 1) / n_tiles + 31) / 32 * 32 : 0;
  if (W * TS > 65535 || W * ITS > 65535) {
    set_error("more than 65535 neurons or inputs per CTA");
    return SPK_ERR_INVALID;
  }
  const int KL = n_tiles * ITS, n_keys = KL + n_tiles * TS, n_words = n_keys / 32;
  const int key_cap = W * (TS + ITS);

  // scratch layout: descriptor, CTA map, abort flag, stamps + keys (one range to
  // clear), spike / pre-event bitmaps, published pre traces
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = align_up(off, 256);
    off = at + bytes;
    return at;
  };
  const size_t o_nd = take(sizeof(NetDev));
  const size_t o_map = take(sizeof(CtaMap) * (size_t)C);
  const size_t o_abort = take(sizeof(int));
  const size_t xchg_words = 2 * (size_t)C + 2 * (size_t)C * key_cap;
  const size_t o_xchg = take(sizeof(unsigned long long) * xchg_words);
  const size_t o_bA = take(sizeof(uint32_t) * 2 * (size_t)n_words);
  const size_t o_bP = take(sizeof(uint32_t) * 2 * (size_t)n_words);
  const size_t o_pub = take(stdp ? sizeof(float) * 2 * (size_t)n_keys : 0);
  if (off > SPK_NOALLOC_SCRATCH_BYTES) {
    set_error("network needs %zu bytes of step scratch; spk_step_noalloc holds %u", off,
              (unsigned)SPK_NOALLOC_SCRATCH_BYTES);
    return SPK_ERR_INVALID;
  }

  if (!a->group_bits) {
    set_error("group_bits missing (the last group's spike words, timestep_grouping * n_keys / 32 words)");
    return SPK_ERR_INVALID;
  }
  NoallocDevice* dev = nullptr;
  int rc = noalloc_device(&dev);
  if (rc) return rc;
  const int smem = smem_bytes(W, warp_layout(B, TS, L, ITS, kind, stdp));
  if (smem > dev->di.max_smem) {
    set_error("schedule W=%d tile=%d needs %d B of shared memory, the device offers %d", W, TS, smem,
              dev->di.max_smem);
    return SPK_ERR_INVALID;
  }
  if (C > 1) {
    int per_sm = 0;
    SPK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, step_kernel, W * 32, smem));
    if ((int64_t)per_sm * dev->di.sms < C) {
      set_error("schedule needs %d co-resident CTAs, device holds %d", C, per_sm * dev->di.sms);
      return SPK_ERR_UNSUPPORTED;
    }
  }
  if (n_steps == 0) return SPK_OK;

  unsigned char* s = dev->scratch;
  NetDev h;
  std::memset(&h, 0, sizeof(h));
  h.N = N;
  h.Nin = Nin;
  h.KL = KL;
  h.n_keys = n_keys;
  h.n_words = n_words;
  h.L = L;
  h.B = B;
  h.kind = kind;
  h.n_tiles = n_tiles;
  h.TS = TS;
  h.ITS = ITS;
  h.W = W;
  h.nctas = C;
  h.n_groups = a->n_groups;
  h.dt = a->dt;
  h.half_dt = 0.5f * a->dt;
  h.G = G;
  h.t_ref = a->refractory_period;
  h.i_bg = a->background_current;
  for (int g = 0; g < a->n_groups; ++g) {
    const spk_neuron_group& G = a->groups[g];
    GroupConst& c = h.groups[g];
    c.start = G.start;
    c.end = G.start + G.count;
    // LIFSpikingNeurons.cu:31-44: k = timestep / tau_m, kR = k * R (host float).
    c.k = a->dt / G.tau_m;
    c.kR = c.k * G.R;
    c.v0 = G.v0;
    c.vreset = G.vreset;
    c.theta = G.theta;
  }
  for (int l = 0; l < L; ++l) {
    // ConductanceSpikingSynapses.cu:76-78: expf(-timestep / tau_g) on the host.
    h.decay[l] = kind == SPK_SYN_VOLTAGE ? 0.0f : expf(-a->dt / a->label_tau[l]);
    h.vhat[l] = kind == SPK_SYN_CONDUCTANCE ? a->label_vhat[l] : 0.0f;
  }
  if (stdp)
    for (int c = 0; c < a->n_plastic_scales; ++c) h.scale_tab[c + 1] = a->plastic_scales[c];
  h.has_stdp = stdp;
  if (stdp) {
    const spk_stdp_params& sp = a->stdp;
    // WeightDependentSTDPPlasticity.cu:125-145 for G = 1.
    const float em = expf(-(1.0f * a->dt) / sp.tau_minus);
    const float ep = expf(-(1.0f * a->dt) / sp.tau_plus);
    h.E_m = em;
    h.E_p = ep;
    h.inc_m = sp.a_minus * em;
    h.inc_p = sp.a_plus * ep;
    h.invE_m = 1.0f / em;
    h.invE_p = 1.0f / ep;
    h.lam = sp.lambda;
    h.lam_alpha = sp.lambda * sp.alpha;
    h.wmax = sp.w_max;
    h.clip_upper = sp.clip_upper ? 1 : 0;
  }
  h.seed = a->seed;
  h.rowptr = a->rowptr;
  h.entries = (uint2*)a->entries;
  h.csc_ptr = a->csc_ptr;
  h.csc = (uint2*)a->csc;
  h.V = a->V;
  h.last = a->last_spike;
  h.gtr = a->syn_trace;
  h.ring = a->ring;
  h.in_next = a->input_next;
  h.rates = a->rates;
  h.post_trace = a->post_trace;
  h.pre_trace = a->pre_trace;
  h.pre_pub = stdp ? (float*)(s + o_pub) : nullptr;
  h.bitsA = (uint32_t*)(s + o_bA);
  h.bitsP = (uint32_t*)(s + o_bP);
  h.cta_stamp = (unsigned long long*)(s + o_xchg);
  h.cta_keys = h.cta_stamp + 2 * (size_t)C;
  h.key_cap = key_cap;
  h.spikes = (uint2*)a->spikes;
  h.spike_cap = a->spike_capacity;
  h.ctl = (RunCtl*)a->run_state;
  h.gbits = a->group_bits;
  h.abort_flag = (int*)(s + o_abort);
  h.poll_ns = DEFAULT_WAIT_LIMIT_NS;

  const int grid = (int)std::min<size_t>((xchg_words + 255) / 256, (size_t)dev->di.sms * 4);
  noalloc_setup_kernel<<<std::max(grid, 1), 256, 0, stream>>>(h, (NetDev*)(s + o_nd), (CtaMap*)(s + o_map),
                                                               h.cta_stamp, xchg_words);
  SPK_CUDA(cudaGetLastError());
  set_ctl_kernel<<<1, 1, 0, stream>>>(h.ctl, G, a->dt, start, (int)n_steps, (plasticity_on && stdp) ? 1 : 0,
                                      a->record_inputs ? 1 : 0);
  SPK_CUDA(cudaGetLastError());
  const int K = DEFAULT_STEPS_PER_LAUNCH;
  const int64_t blocks = (n_steps + K - 1) / K;
  for (int64_t b = 0; b < blocks; ++b) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(W * 32);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = C > 1 ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SPK_CUDA(cudaLaunchKernelEx(&cfg, step_kernel, (const NetDev*)(s + o_nd), (const CtaMap*)(s + o_map), K));
  }
  return SPK_OK;
}

}  // namespace spk

extern "C" int spk_step_noalloc(const spk_device_net* net, int64_t n_steps, int32_t plasticity_on,
                                float start_time, void* stream) {
  return spk::step_noalloc_impl(net, n_steps, plasticity_on, start_time, (cudaStream_t)stream);
}

// =====================================================================================
// Batch autotuner: a measured search over schedule policies for a set of
// generated networks.  A policy fixes warps per CTA W and a largest tile TS*;
// each network then gets the tile min(TS*, its neurons / W rounded up to 32)
// and as many CTAs as cover it, so small networks run on one CTA and large
// ones spread over CTAs of TS*-post tiles.  Every policy is built (the same
// networks, drawn again under its tiles), packed into waves and timed over a
// trial run; the fastest policy's schedules are returned.  Results do not
// depend on the schedule, only the time does.
namespace spk {

struct TunePolicy {
  int W, TS;
};

static int policy_schedules(const spk_gen_desc* descs, int n, const TunePolicy& pol, const DeviceInfo& di,
                            std::vector<spk_schedule>& out) {
  out.assign(n, spk_schedule{});
  for (int i = 0; i < n; ++i) {
    const spk_gen_desc& d = descs[i];
    int dmax = 1;
    for (int j = 0; j < d.n_projections; ++j) dmax = std::max(dmax, d.projections[j].delay_hi);
    const int B = dmax + 3;
    const int want = std::max(32, ((d.n_neurons + pol.W - 1) / pol.W + 31) / 32 * 32);
    bool ok = false;
    for (int TS = std::min(pol.TS, want); TS >= 32 && !ok; TS -= 32) {
      spk_schedule s{pol.W, TS, 0, 0};
      Plan p;
      if (make_plan(d.n_neurons, d.n_inputs, B, std::max(1, d.n_labels), d.synapse_kind, d.has_stdp ? 1 : 0, &s,
                    di, &p) == SPK_OK &&
          p.nctas <= di.sms) {
        out[i] = spk_schedule{p.W, p.TS, p.nctas, 0};
        ok = true;
      }
    }
    if (!ok) {
      set_error("autotune: no schedule with %d warps per CTA fits network %d", pol.W, i);
      return SPK_ERR_UNSUPPORTED;
    }
  }
  return SPK_OK;
}

// Times `steps` timesteps of the networks under schedules `sch` as one batch,
// in waves mode (ms[0]) and in bulk mode (ms[1]); ms[0] stays negative when a
// network runs in bulk mode only (a per-synapse-trace rule).
static int trial_policy(const spk_gen_desc* descs, int n, const std::vector<spk_schedule>& sch, int steps,
                        float* ms) {
  std::vector<spk_net*> nets(n, nullptr);
  spk_batch* b = nullptr;
  auto cleanup = [&]() {
    if (b) spk_batch_destroy(b);
    for (spk_net* x : nets)
      if (x) spk_net_destroy(x);
  };
  int rc = SPK_OK;
  for (int i = 0; i < n && rc == SPK_OK; ++i) rc = generate_impl(&descs[i], &sch[i], &nets[i]);
  const spk_schedule bs{0, 0, 0, steps};  // one launch block per trial
  if (rc == SPK_OK) rc = spk_batch_create(nets.data(), n, &bs, &b);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (rc == SPK_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) rc = SPK_ERR_CUDA;
  bool bulk_only = false;
  for (int i = 0; i < n && rc == SPK_OK; ++i) bulk_only = bulk_only || nets[i]->bulk_only();
  for (int mode = SPK_BATCH_WAVES; mode <= SPK_BATCH_BULK && rc == SPK_OK; ++mode) {
    if (mode == SPK_BATCH_WAVES && bulk_only) {
      ms[mode] = -1.0f;
      continue;
    }
    rc = spk_batch_set_mode(b, mode);
    if (rc == SPK_OK) rc = spk_batch_run_steps(b, steps, 1);  // warm-up (and graph capture)
    if (rc == SPK_OK && cudaStreamSynchronize(b->stream) != cudaSuccess) rc = SPK_ERR_CUDA;
    if (rc != SPK_OK) break;
    cudaEventRecord(e0, b->stream);
    rc = spk_batch_run_steps(b, steps, 1);
    cudaEventRecord(e1, b->stream);
    if (rc == SPK_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = SPK_ERR_CUDA;
    if (rc == SPK_OK) {
      cudaEventElapsedTime(&ms[mode], e0, e1);
      rc = spk_batch_synchronize(b);
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cleanup();
  return rc;
}

}  // namespace spk

// Time of one step of each network alone under its schedule (microseconds).
static int measure_alone(const spk_gen_desc* descs, int n, const std::vector<spk_schedule>& sch, int steps,
                         float* step_us) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    set_error("cudaEventCreate failed");
    return SPK_ERR_CUDA;
  }
  int rc = SPK_OK;
  for (int i = 0; i < n && rc == SPK_OK; ++i) {
    spk_net* x = nullptr;
    rc = generate_impl(&descs[i], &sch[i], &x);
    if (rc) break;
    rc = run_steps_impl(x, std::max(1, steps / 2), 1, x->current_time);
    x->current_time += (float)std::max(1, steps / 2) * x->dt;
    if (rc == SPK_OK) {
      cudaEventRecord(e0, x->stream);
      rc = run_steps_impl(x, steps, 1, x->current_time);
      cudaEventRecord(e1, x->stream);
    }
    float ms = 0.0f;
    if (rc == SPK_OK && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
      rc = SPK_ERR_CUDA;
    int st = SPK_OK;
    if (rc == SPK_OK && read_status(x, &st) == SPK_OK && st != SPK_OK) rc = st;
    step_us[i] = 1000.0f * ms / (float)steps;
    spk_net_destroy(x);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

extern "C" int spk_batch_autotune(const spk_gen_desc* descs, int32_t n_nets, int32_t trial_steps,
                                  spk_schedule* schedules, float* best_ms, float* step_us, int32_t* best_mode) {
  using namespace spk;
  if (!descs || n_nets < 1 || !schedules || trial_steps < 1) return SPK_ERR_INVALID;
  return guarded([&]() -> int {
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    static const TunePolicy policies[] = {{8, 32}, {8, 64}, {8, 128}, {8, 256}, {4, 128}};
    float best = -1.0f;
    int mode = SPK_BATCH_WAVES;
    std::vector<spk_schedule> sch, best_sch;
    int last_rc = SPK_ERR_UNSUPPORTED;
    for (const TunePolicy& pol : policies) {
      if (policy_schedules(descs, n_nets, pol, di, sch) != SPK_OK) continue;
      float ms[2] = {-1.0f, -1.0f};
      last_rc = trial_policy(descs, n_nets, sch, trial_steps, ms);
      if (last_rc == SPK_ERR_TIMEOUT || last_rc == SPK_ERR_CUDA) return last_rc;
      if (last_rc != SPK_OK) continue;
      for (int m = SPK_BATCH_WAVES; m <= SPK_BATCH_BULK; ++m)
        if (ms[m] >= 0.0f && (best < 0.0f || ms[m] < best)) {
          best = ms[m];
          best_sch = sch;
          mode = m;
        }
    }
    if (best < 0.0f) return last_rc;
    std::copy(best_sch.begin(), best_sch.end(), schedules);
    if (best_ms) *best_ms = best;
    if (best_mode) *best_mode = mode;
    if (step_us) {
      if (mode == SPK_BATCH_WAVES) return measure_alone(descs, n_nets, best_sch, trial_steps, step_us);
      std::fill(step_us, step_us + n_nets, 0.0f);  // bulk mode packs no waves
    }
    return SPK_OK;
  });
}
