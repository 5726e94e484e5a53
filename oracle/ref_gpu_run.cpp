// ref_gpu_run.cpp - runs a fixture network of oracle/ref_cases.inc on the
// REFERENCE's own CUDA backend (its kernels compiled for this GPU by
// oracle/build_ref_gpu.sh) and reports what it did.
//
// TEST INFRASTRUCTURE ONLY: the GPU counterpart of ref_dump.  It pins the
// oracle's dynamics to the reference's statistically (the reference orders
// its float ring additions by atomics and draws its Poisson inputs from
// cuRAND XORWOW, so it is not bit-reproducible) and times the reference's
// kernels on the same GPU.
//
// Usage: ref_gpu_run <case> <seconds[,seconds...]> <monitor 0|1> <out_dir>
//   seconds  one run() per comma-separated value, in turn
//   case     va | va_g2 | va_g3 | brunel_cfg2 | brunel_cfg2_plastic (ref_cases.inc)
//   monitor  1: record neuron and input spikes (SpikingActivityMonitor) and
//            write them, with the final weights of the plastic synapse group,
//            to out_dir; 0: no monitor
//            (the reference examples' timing mode)
// Prints one JSON line: synapses, timesteps, wall seconds of run() (to the
// device's completion), spike counts and synaptic events (spikes times the
// out-degree of the spiking neuron or input).
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "Spike/Spike.hpp"

namespace {
#include "ref_cases.inc"
}  // namespace

int main(int argc, char** argv) {
  if (argc != 5) {
    fprintf(stderr, "usage: ref_gpu_run <case> <seconds> <monitor 0|1> <out_dir>\n");
    return 2;
  }
  const std::string name = argv[1], dir = argv[4];
  std::vector<float> runs;
  for (const char* p = argv[2]; *p;) {
    char* end = nullptr;
    runs.push_back(strtof(p, &end));
    if (end == p) return 2;
    p = (*end == ',') ? end + 1 : end;
  }
  float seconds = 0.0f;
  for (float s : runs) seconds += s;
  const bool monitor = atoi(argv[3]) != 0;
  if (name == "cdet") {
    // The reference's current-synapse backend never sets its device decay
    // constants (Spike/Backend/CUDA/Synapses/CurrentSpikingSynapses.cu:27-29);
    // its injection kernel faults on the null pointer.
    fprintf(stderr, "ref_gpu_run: the reference's current-synapse backend faults; not run\n");
    return 2;
  }
  RefCase r = build_case(name);
  if (!r.m) return 2;
  SpikingActivityMonitor* mon_n = nullptr;
  SpikingActivityMonitor* mon_i = nullptr;
  if (monitor) {
    mon_n = new SpikingActivityMonitor(r.neurons);
    r.m->AddActivityMonitor(mon_n);
    if (r.inputs) {
      mon_i = new SpikingActivityMonitor(r.inputs);
      r.m->AddActivityMonitor(mon_i);
    }
  }
  // out-degree of every presynaptic id (creation-order arrays, before the
  // model sorts them): neurons 0..N-1, inputs as -1-i
  const int N = r.neurons->total_number_of_neurons;
  const int Nin = r.inputs ? r.inputs->total_number_of_neurons : 0;
  const long long S = r.syn->total_number_of_synapses;
  std::vector<long long> deg_n(N, 0), deg_i(Nin, 0);
  for (long long s = 0; s < S; ++s) {
    const int p = r.syn->presynaptic_neuron_indices[s];
    if (p >= 0)
      ++deg_n[p];
    else
      ++deg_i[-1 - p];
  }
  r.m->finalise_model();
  cudaDeviceSynchronize();
  const auto t0 = std::chrono::steady_clock::now();
  for (float s : runs) r.m->run(s);
  cudaDeviceSynchronize();
  const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  // SpikingModel::run: ceil(seconds/dt) timesteps, whole groups of timestep_grouping
  long long steps = 0;
  for (float s : runs)
    steps += (long long)std::ceil(s / r.m->timestep) / r.m->timestep_grouping * r.m->timestep_grouping;
  long long spikes_n = -1, spikes_i = -1, events = -1;
  if (monitor) {
    mon_n->save_spikes_as_binary(dir, name + "_neurons_");
    spikes_n = mon_n->total_number_of_spikes_stored_on_host;
    events = 0;
    for (long long k = 0; k < spikes_n; ++k) events += deg_n[mon_n->neuron_ids_of_stored_spikes_on_host[k]];
    if (mon_i) {
      mon_i->save_spikes_as_binary(dir, name + "_inputs_");
      spikes_i = mon_i->total_number_of_spikes_stored_on_host;
      for (long long k = 0; k < spikes_i; ++k) events += deg_i[mon_i->neuron_ids_of_stored_spikes_on_host[k]];
    } else {
      spikes_i = 0;
    }
    // the plastic case's E->E synapses are its fourth synapse group (ref_cases.inc)
    if (r.rule) r.syn->save_weights_as_binary(dir, name + "_final_", 3);
  }
  printf("{\"case\": \"%s\", \"synapses\": %lld, \"neurons\": %d, \"inputs\": %d, \"grouping\": %d, \"seconds\": %g, \"timesteps\": %lld, "
         "\"monitor\": %d, \"wall_s\": %.6f, \"neuron_spikes\": %lld, \"input_spikes\": %lld, \"events\": %lld, "
         "\"cuda_status\": \"%s\"}\n",
         name.c_str(), S, N, Nin, r.m->timestep_grouping, (double)seconds, steps, monitor ? 1 : 0, wall, spikes_n, spikes_i, events,
         cudaGetErrorString(cudaGetLastError()));
  return 0;
}
