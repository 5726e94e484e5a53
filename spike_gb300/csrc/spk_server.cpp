// spk_server.cpp - continuous-batching simulation server over the C ABI.
//
// One host thread drives the GPU.  Per step block it (1) admits queued jobs
// whose estimated device footprint fits the free memory less the reserve,
// generating their networks on the device, (2) runs every running job for
// min(remaining steps, block) steps in one batch - co-resident waves of the
// persistent step kernel, ordered by estimated step cost - and, while that
// batch runs on the GPU, admits the jobs that arrived meanwhile (they join at
// the next block), (3) collects finished jobs' counters and spikes to the
// host and frees their networks.  Only this thread calls into the engine, so
// the engine's handles stay single-threaded; submit / poll / wait touch host
// state under one mutex.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/spike_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

// A spk_gen_desc with every array it points to owned here.
struct GenCopy {
  spk_gen_desc d{};
  std::vector<spk_neuron_group> groups;
  std::vector<float> rates, tau, vhat;
  std::vector<spk_projection> projs;

  explicit GenCopy(const spk_gen_desc& src) : d(src) {
    groups.assign(src.groups, src.groups + std::max(0, src.n_groups));
    if (src.n_inputs > 0 && src.input_rates)
      rates.assign(src.input_rates, src.input_rates + (size_t)std::max(1, src.n_stimuli) * src.n_inputs);
    const int L = std::max(1, src.n_labels);
    if (src.label_tau) tau.assign(src.label_tau, src.label_tau + L);
    if (src.label_vhat) vhat.assign(src.label_vhat, src.label_vhat + L);
    if (src.n_projections > 0) projs.assign(src.projections, src.projections + src.n_projections);
    d.groups = groups.data();
    d.input_rates = rates.empty() ? nullptr : rates.data();
    d.label_tau = tau.empty() ? nullptr : tau.data();
    d.label_vhat = vhat.empty() ? nullptr : vhat.data();
    d.projections = projs.empty() ? nullptr : projs.data();
  }
};

struct Job {
  int64_t id = 0;
  std::unique_ptr<GenCopy> gen;
  int64_t steps_total = 0, steps_done = 0;
  int plastic = 1;
  int state = SPK_JOB_QUEUED, error = SPK_OK;
  bool cancel = false;
  double submit_s = 0, start_s = -1, finish_s = -1;
  int64_t bytes = 0, peak_bytes = 0;
  spk_net* net = nullptr;
  uint64_t events = 0;       // delivered so far (updated after every block)
  uint64_t events_seen = 0;  // part of `events` already counted in the server's total
  int64_t spikes = 0, synapses = 0;
  std::vector<int32_t> ids;
  std::vector<float> times;
};

}  // namespace

struct spk_server {
  spk_server_opts o{};
  int device = 0;
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv;  // submissions, cancellations, stop, job state changes
  std::deque<Job*> queue;
  std::map<int64_t, std::unique_ptr<Job>> jobs;
  bool stopping = false;
  int64_t next_id = 1;
  spk_server_stats st{};
  std::thread th;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

spk_schedule policy_schedule(const spk_server* S, const spk_gen_desc& d) {
  const int W = S->o.warps_per_cta;
  const int want = std::max(32, ((d.n_neurons + W - 1) / W + 31) / 32 * 32);
  return spk_schedule{W, std::min(S->o.tile_posts, want), 0, 0};
}

// Admit queued jobs while memory and the running limit allow; new networks go
// to `out`.  Returns after the first job that does not fit.
void admit(spk_server* S, std::vector<Job*>& out, size_t running_now) {
  while (true) {
    Job* j = nullptr;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      while (!S->queue.empty() && S->queue.front()->cancel) {
        Job* c = S->queue.front();
        S->queue.pop_front();
        c->state = SPK_JOB_CANCELLED;
        c->finish_s = S->now();
        S->cv.notify_all();
      }
      if (S->queue.empty() || S->stopping || running_now + out.size() >= (size_t)S->o.max_running) return;
      j = S->queue.front();
    }
    uint64_t free_b = 0, total_b = 0;
    if (spk_memory_info(&free_b, &total_b) != SPK_OK) return;
    if ((int64_t)free_b - (int64_t)S->o.reserve_bytes < j->peak_bytes) {
      if (running_now + out.size() > 0) return;  // wait for memory to free up
      // nothing runs and it still does not fit: it never will
      std::lock_guard<std::mutex> lk(S->mu);
      S->queue.pop_front();
      j->state = SPK_JOB_FAILED;
      j->error = SPK_ERR_OOM;
      j->finish_s = S->now();
      S->st.failed++;
      S->cv.notify_all();
      continue;
    }
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->queue.pop_front();
    }
    const spk_schedule sch = policy_schedule(S, j->gen->d);
    spk_net* net = nullptr;
    const int rc = spk_net_generate(&j->gen->d, &sch, &net);
    std::lock_guard<std::mutex> lk(S->mu);
    if (rc == SPK_ERR_OOM && running_now + out.size() > 0) {
      S->queue.push_front(j);  // retry when memory frees up
      return;
    }
    if (rc != SPK_OK) {
      j->state = SPK_JOB_FAILED;
      j->error = rc;
      j->finish_s = S->now();
      S->st.failed++;
      S->cv.notify_all();
      continue;
    }
    int64_t syn = 0;
    spk_net_synapse_count(net, &syn);
    j->synapses = syn;
    // wave packing cost: synapses, doubled for a plastic run
    spk_net_set_step_cost(net, (float)syn * ((j->plastic && j->gen->d.has_stdp) ? 2.0f : 1.0f));
    // the whole job is one run, advanced a block at a time
    const int brc = spk_net_begin_run(net, j->steps_total, j->plastic);
    if (brc != SPK_OK) {
      spk_net_destroy(net);
      j->state = SPK_JOB_FAILED;
      j->error = brc;
      j->finish_s = S->now();
      S->st.failed++;
      S->cv.notify_all();
      continue;
    }
    j->net = net;
    j->state = SPK_JOB_RUNNING;
    j->start_s = S->now();
    out.push_back(j);
  }
}

// Copy a finished job's results to the host and free its network (with
// `keep_net`, the network stays allocated: it is still held by the running
// batch, which frees it at its next rebuild; having no steps left, its
// kernels return at once meanwhile).
void finish(spk_server* S, Job* j, int status, bool keep_net = false) {
  uint64_t ev = 0;
  spk_net_synaptic_events(j->net, &ev);
  int64_t n = 0;
  std::vector<int32_t> ids;
  std::vector<float> times;
  if (spk_net_spike_count(j->net, SPK_POP_NEURONS, &n) == SPK_OK && n > 0 && S->o.record_spikes) {
    ids.resize(n);
    times.resize(n);
    int64_t got = 0;
    spk_net_read_spikes(j->net, SPK_POP_NEURONS, ids.data(), times.data(), n, &got);
    ids.resize(got);
    times.resize(got);
  }
  if (!keep_net) spk_net_destroy(j->net);
  std::lock_guard<std::mutex> lk(S->mu);
  if (!keep_net) j->net = nullptr;
  j->events_seen = j->events;
  j->events = ev;
  j->spikes = n;
  j->ids.swap(ids);
  j->times.swap(times);
  if (status != SPK_OK) {
    j->state = SPK_JOB_FAILED;
    j->error = status;
    S->st.failed++;
  } else {
    j->state = j->cancel && j->steps_done < j->steps_total ? SPK_JOB_CANCELLED : SPK_JOB_DONE;
    if (j->state == SPK_JOB_DONE) S->st.done++;
  }
  j->finish_s = S->now();
  S->st.events += ev - std::min(ev, j->events_seen);
  j->events_seen = ev;
  S->cv.notify_all();
}

// The batch is rebuilt only when its set of networks must grow: a finished
// or cancelled job leaves its network in the batch ("retired": results read,
// no steps left) until the next rebuild, which jobs joining or queued jobs
// needing its memory trigger.  A set that only shrinks keeps its batch, and
// with it the instantiated graph of the step block.
void loop(spk_server* S) {
  cudaSetDevice(S->device);
  std::vector<Job*> run, pending, retired;
  spk_batch* batch = nullptr;
  bool dirty = true;
  const int K = S->o.steps_per_block;
  auto free_retired = [&]() {
    for (Job* j : retired) {
      spk_net_destroy(j->net);
      std::lock_guard<std::mutex> lk(S->mu);
      j->net = nullptr;
    }
    retired.clear();
  };
  while (true) {
    const size_t before = run.size();
    if (batch && !retired.empty()) {
      // queued work waiting for memory gets the retired networks' share back
      bool queued = false;
      {
        std::lock_guard<std::mutex> lk(S->mu);
        queued = !S->queue.empty();
      }
      if (queued) {
        spk_batch_destroy(batch);
        batch = nullptr;
        free_retired();
        dirty = true;
      }
    }
    admit(S, run, 0);
    if (run.size() != before) dirty = true;
    if (run.empty()) {
      if (batch) {
        spk_batch_destroy(batch);
        batch = nullptr;
      }
      free_retired();
      std::unique_lock<std::mutex> lk(S->mu);
      if (S->stopping) break;
      S->cv.wait_for(lk, std::chrono::milliseconds(20));
      continue;
    }
    if (dirty) {
      if (batch) spk_batch_destroy(batch);
      batch = nullptr;
      free_retired();
      std::vector<spk_net*> nets;
      for (Job* j : run) nets.push_back(j->net);
      const spk_schedule bs{0, 0, 0, K};
      int rc = spk_batch_create(nets.data(), (int32_t)nets.size(), &bs, &batch);
      if (rc == SPK_OK && S->o.mode == SPK_BATCH_BULK) rc = spk_batch_set_mode(batch, SPK_BATCH_BULK);
      if (rc != SPK_OK) {
        if (batch) spk_batch_destroy(batch);
        batch = nullptr;
        for (Job* j : run) finish(S, j, rc);
        run.clear();
        continue;
      }
      S->st.rebuilds++;
      dirty = false;
    }
    std::vector<int64_t> steps(run.size());
    for (size_t i = 0; i < run.size(); ++i) steps[i] = std::min<int64_t>(K, run[i]->steps_total - run[i]->steps_done);
    const double tb = S->now();
    int rc = spk_batch_step_block(batch);
    // while the batch runs: admit arrivals (they join at the next block)
    if (rc == SPK_OK) admit(S, pending, run.size());
    const int st = rc == SPK_OK ? spk_batch_synchronize(batch) : rc;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->st.blocks++;
      S->st.busy_s += S->now() - tb;
      for (size_t i = 0; i < run.size(); ++i) run[i]->steps_done += steps[i];
    }
    // delivered events of every running job so far
    for (Job* j : run) {
      uint64_t ev = 0;
      if (spk_net_synaptic_events(j->net, &ev) == SPK_OK) {
        std::lock_guard<std::mutex> lk(S->mu);
        S->st.events += ev - j->events;
        j->events = ev;
      }
    }
    std::vector<Job*> keep;
    for (Job* j : run) {
      int js = SPK_OK;
      if (st != SPK_OK) js = spk_net_synchronize(j->net);
      if (js != SPK_OK) {
        // a failed block: the batch is rebuilt without this network
        if (batch) {
          spk_batch_destroy(batch);  // a batch never outlives a network it holds
          batch = nullptr;
        }
        finish(S, j, js);
        dirty = true;
      } else if (j->steps_done >= j->steps_total) {
        finish(S, j, SPK_OK, batch != nullptr);
        if (batch) retired.push_back(j);
      } else if (j->cancel) {
        // a cancelled job still has steps: the batch must drop it
        if (batch) {
          spk_batch_destroy(batch);
          batch = nullptr;
        }
        finish(S, j, SPK_OK);
        dirty = true;
      } else {
        keep.push_back(j);
      }
    }
    if (!batch) free_retired();  // the batch that held them is gone
    run.swap(keep);
    if (!pending.empty()) {
      run.insert(run.end(), pending.begin(), pending.end());
      pending.clear();
      dirty = true;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stopping) break;
  }
  if (batch) spk_batch_destroy(batch);
  free_retired();
  for (Job* j : run) {
    j->cancel = true;
    finish(S, j, SPK_OK);
  }
  for (Job* j : pending) {
    j->cancel = true;
    finish(S, j, SPK_OK);
  }
  std::lock_guard<std::mutex> lk(S->mu);
  for (Job* j : S->queue) {
    j->state = SPK_JOB_CANCELLED;
    j->finish_s = S->now();
  }
  S->queue.clear();
  S->cv.notify_all();
}

template <typename F>
int guard(F&& f) {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    return SPK_ERR_OOM;
  } catch (...) {
    return SPK_ERR_STATE;
  }
}

}  // namespace

extern "C" {

int spk_server_start(const spk_server_opts* opts, spk_server** out) {
  if (!out) return SPK_ERR_INVALID;
  return guard([&]() -> int {
    auto* S = new spk_server();
    if (opts) S->o = *opts;
    if (S->o.warps_per_cta <= 0) S->o.warps_per_cta = 8;
    if (S->o.tile_posts <= 0) S->o.tile_posts = 64;
    if (S->o.steps_per_block <= 0) S->o.steps_per_block = 1000;
    if (S->o.max_running <= 0) S->o.max_running = 512;
    if (S->o.reserve_bytes == 0) S->o.reserve_bytes = 8ull << 30;
    if (S->o.tile_posts % 32 || S->o.warps_per_cta > 16 ||
        (S->o.mode != SPK_BATCH_WAVES && S->o.mode != SPK_BATCH_BULK)) {
      delete S;
      return SPK_ERR_INVALID;
    }
    if (cudaGetDevice(&S->device) != cudaSuccess) {
      delete S;
      return SPK_ERR_CUDA;
    }
    S->t0 = Clock::now();
    S->th = std::thread(loop, S);
    *out = S;
    return SPK_OK;
  });
}

int spk_server_submit(spk_server* S, const spk_gen_desc* desc, int64_t n_steps, int32_t plasticity_on,
                      int64_t* job) {
  if (!S || !desc || !job || n_steps < 0) return SPK_ERR_INVALID;
  return guard([&]() -> int {
    auto j = std::make_unique<Job>();
    j->gen = std::make_unique<GenCopy>(*desc);
    if (!S->o.record_spikes) j->gen->d.spike_capacity = -1;
    j->steps_total = n_steps;
    j->plastic = plasticity_on ? 1 : 0;
    const spk_schedule sch = policy_schedule(S, j->gen->d);
    const int rc = spk_net_generate_estimate(&j->gen->d, &sch, &j->bytes, &j->peak_bytes);
    if (rc != SPK_OK) return rc;
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stopping) return SPK_ERR_STATE;
    j->id = S->next_id++;
    j->submit_s = S->now();
    *job = j->id;
    S->queue.push_back(j.get());
    S->jobs[j->id] = std::move(j);
    S->st.submitted++;
    S->cv.notify_all();
    return SPK_OK;
  });
}

int spk_server_poll(spk_server* S, int64_t job, spk_job_info* info) {
  if (!S || !info) return SPK_ERR_INVALID;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->jobs.find(job);
  if (it == S->jobs.end()) return SPK_ERR_INVALID;
  const Job& j = *it->second;
  info->state = j.state;
  info->error = j.error;
  info->steps_done = j.steps_done;
  info->steps_total = j.steps_total;
  info->events = j.events;
  info->spikes = j.spikes;
  info->synapses = j.synapses;
  info->submit_s = j.submit_s;
  info->start_s = j.start_s;
  info->finish_s = j.finish_s;
  return SPK_OK;
}

int spk_server_wait(spk_server* S, int64_t job, double timeout_s) {
  if (!S) return SPK_ERR_INVALID;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->jobs.find(job);
  if (it == S->jobs.end()) return SPK_ERR_INVALID;
  Job* j = it->second.get();
  const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
  while (j->state == SPK_JOB_QUEUED || j->state == SPK_JOB_RUNNING) {
    if (S->cv.wait_until(lk, until) == std::cv_status::timeout &&
        (j->state == SPK_JOB_QUEUED || j->state == SPK_JOB_RUNNING))
      return SPK_ERR_BUSY;
  }
  return SPK_OK;
}

int spk_server_read_spikes(spk_server* S, int64_t job, int32_t* ids, float* times, int64_t capacity,
                           int64_t* n_written) {
  if (!S || !n_written || capacity < 0) return SPK_ERR_INVALID;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->jobs.find(job);
  if (it == S->jobs.end()) return SPK_ERR_INVALID;
  const Job& j = *it->second;
  if (j.state != SPK_JOB_DONE && j.state != SPK_JOB_CANCELLED) return SPK_ERR_STATE;
  const int64_t n = std::min<int64_t>(capacity, (int64_t)j.ids.size());
  if (n > 0 && (!ids || !times)) return SPK_ERR_INVALID;
  if (n > 0) {
    std::memcpy(ids, j.ids.data(), sizeof(int32_t) * n);
    std::memcpy(times, j.times.data(), sizeof(float) * n);
  }
  *n_written = n;
  return SPK_OK;
}

int spk_server_cancel(spk_server* S, int64_t job) {
  if (!S) return SPK_ERR_INVALID;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->jobs.find(job);
  if (it == S->jobs.end()) return SPK_ERR_INVALID;
  it->second->cancel = true;
  S->cv.notify_all();
  return SPK_OK;
}

int spk_server_release(spk_server* S, int64_t job) {
  if (!S) return SPK_ERR_INVALID;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->jobs.find(job);
  if (it == S->jobs.end()) return SPK_ERR_INVALID;
  const int s = it->second->state;
  if (s == SPK_JOB_QUEUED || s == SPK_JOB_RUNNING) return SPK_ERR_STATE;
  S->jobs.erase(it);
  return SPK_OK;
}

int spk_server_stats_get(spk_server* S, spk_server_stats* out) {
  if (!S || !out) return SPK_ERR_INVALID;
  std::lock_guard<std::mutex> lk(S->mu);
  *out = S->st;
  int64_t running = 0, queued = 0;
  for (const auto& kv : S->jobs) {
    running += kv.second->state == SPK_JOB_RUNNING;
    queued += kv.second->state == SPK_JOB_QUEUED;
  }
  out->running = running;
  out->queued = queued;
  out->uptime_s = S->now();
  return SPK_OK;
}

int spk_server_stop(spk_server* S) {
  if (!S) return SPK_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stopping = true;
    S->cv.notify_all();
  }
  if (S->th.joinable()) S->th.join();
  delete S;
  return SPK_OK;
}

}  // extern "C"
