"""Benchmark of the clock-driven step: synaptic events/s on one GB300.

Workload (default, --workload batched): the batched sweep - 256 independent
Brunel-style LIF instances, N log-uniform in [1k, 50k] (80 % excitatory),
Bernoulli recurrent connectivity p ~ U[0.01, 0.05], g ~ U[3, 7], delays
U{1..10} steps, external drive of N/5 Poisson inputs at 20 Hz, distinct
seeds, half of them with weight-dependent STDP on the input synapses; about
4.2e9 synapses (34 GB of entries) drawn on the GPU.  The autotuner picks the
schedules, the instances run in one batch (co-resident waves of the
persistent step kernel), and the same instances run alone one after another
give the plain form (`plain`, `batched_over_plain`).

Other workloads: brunel (Examples/Brunel10K.cpp at 10,000 + 2,500 LIF with
10,000 Poisson inputs, in-degree 0.1, delays U{1..20}, 28.1 M synapses),
vogels_abbott (Examples/VogelsAbbottNet.cpp, 4,000 conductance LIF),
plastic_ff (50,000 log-normal Poisson inputs onto 200,000 LIF, 1,000
afferents each, STDP; --construction exact builds the fixed in-degree of 900
input + 100 recurrent afferents with the host front end, generated draws a
binomial in-degree of the same mean on the GPU).  Data are synthetic, built
by the reference's construction rules or drawn on the GPU.

A bench "step" is one block of --block timesteps (default 1000 = 0.1 s of
simulated time); the default step count covers the workload's simulated time
(1 s batched, 2 s brunel, 1 s vogels_abbott, 5 s plastic_ff).

Printed JSON (one line): value = synaptic events/s over the timed region
(events = sum over spikes of the spiking neuron's out-degree), device-timed
with CUDA events on the engine's stream; e2e = the same metric through the
public API with a host->device rate upload and a device->host spike readback
every step; roofline for the step kernel; cpu_baseline = the CPU oracle (a
single-thread C++ transcription of the reference step loop) on a bounded
sample.

--impl reference: the reference has no CPU implementation of the step (its
only backend is CUDA; the Dummy backend computes nothing), so the reference
arm times the oracle port of its step loop with the host's threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DT = 0.0001


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None,
                   help="timed bench steps (default: the workload's simulated time, 1000 timesteps per step)")
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="batched",
                   choices=["batched", "brunel", "vogels_abbott", "plastic_ff", "served"])
    p.add_argument("--duration", type=float, default=60.0, help="served: seconds of request arrivals")
    p.add_argument("--arrival-rate", type=float, default=20.0, help="served: mean requests per second")
    p.add_argument("--instances", type=int, default=256, help="batched: network instances")
    p.add_argument("--scale", type=float, default=1.0, help="plastic_ff: network size factor (profiling cases)")
    p.add_argument("--rule", default="weight_dependent", choices=["weight_dependent", "evans"],
                   help="plastic_ff: STDP rule of the input synapses")
    p.add_argument("--construction", default=None, choices=["exact", "generated"],
                   help="plastic_ff: exact = fixed in-degree (900 input + 100 recurrent afferents per neuron, "
                        "the host front end's connect_with_sparsity); generated = Bernoulli pairs drawn on the GPU "
                        "(binomial in-degree of the same mean; the Evans rule needs it).  Default: exact for the "
                        "weight-dependent rule, generated for the Evans rule")
    p.add_argument("--norm", default="off", choices=["off", "after", "before"],
                   help="brunel: weight-dependent STDP on the E->E synapses with the weight normalisation "
                        "added after or before it")
    p.add_argument("--tune-steps", type=int, default=100, help="batched: autotuner trial timesteps")
    p.add_argument("--mode", default="auto", choices=["auto", "waves", "bulk"],
                   help="batched: execution mode (auto: the autotuner's choice; waves without the autotuner); served: waves, else bulk")
    p.add_argument("--no-tune", action="store_true",
                   help="batched: skip the autotuner (8 warps, tiles of up to 64 posts, costs from synapse counts)")
    p.add_argument("--range", type=int, default=0,
                   help="batched: skip the autotuner and propagate over post ranges of this many posts (bulk mode)")
    p.add_argument("--plain-block", type=int, default=1000,
                   help="batched: timesteps each instance runs alone for the plain comparison")
    p.add_argument("--block", type=int, default=1000, help="timesteps per bench step")
    p.add_argument("--ctas", type=int, default=0)
    p.add_argument("--warps", type=int, default=0)
    p.add_argument("--tile", type=int, default=0)
    p.add_argument("--launch-steps", type=int, default=0)
    p.add_argument("--cpu-sample-steps", type=int, default=5000)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    a = p.parse_args()
    if a.construction is None:
        a.construction = "exact" if a.rule == "weight_dependent" else "generated"
    if a.steps is None:
        sim_s = {"batched": 1.0, "brunel": 2.0, "vogels_abbott": 1.0, "plastic_ff": 5.0, "served": 0.1}[a.workload]
        a.steps = max(1, int(round(sim_s / (a.block * DT))))
    return a


RULES = {"weight_dependent": 0, "evans": 1}


NORMS = {"off": 0, "after": 1, "before": 2}


def build_model(workload: str, scale: float = 1.0, rule: str = "weight_dependent", norm: str = "off",
                construction: str = "generated", describe_only: bool = False):
    """The workload's network and its description.  With describe_only the
    exact configuration-3 network (2e8 synapses on the host) is not built."""
    from spike_gb300 import networks
    if workload == "brunel":
        m = networks.brunel(norm=NORMS[norm])
        tag = "" if norm == "off" else f"_ee_stdp_weight_norm_{norm}"
        cfg = {"workload": f"brunel_12500_lif_10000_poisson_delays1-20{tag}", "neurons": 12500, "inputs": 10000,
               "in_degree": 2250, "delays_steps": [1, 20], "dt_ms": 0.1, "sim_s_per_config": 2.0,
               "plasticity": norm != "off"}
        L = 1
    elif workload == "vogels_abbott":
        m = networks.vogels_abbott()
        cfg = {"workload": "vogels_abbott_4000_cond_lif_p0.02_delay1", "neurons": 4000, "inputs": 0,
               "dt_ms": 0.1, "sim_s_per_config": 1.0, "plasticity": False}
        L = 2
    else:
        n_in, n_neu = int(round(50000 * scale)), int(round(200000 * scale))
        tag = "stdp" if rule == "weight_dependent" else f"{rule}_stdp"
        cfg = {"workload": f"plastic_ff_{n_neu}_lif_{n_in}_lognormal_poisson_{tag}", "neurons": n_neu,
               "inputs": n_in, "delays_steps": [1, 10], "dt_ms": 0.1, "sim_s_per_config": 5.0,
               "plasticity": True, "stdp_rule": rule}
        if construction == "exact":
            if rule != "weight_dependent":
                raise SystemExit("plastic_ff: --construction exact builds the weight-dependent rule only")
            m = None if describe_only else networks.plastic_ff(n_in=n_in, n_neurons=n_neu)
            cfg.update({"in_degree": "fixed per neuron, multapses allowed: int(sparseness x n_pre) in float as the "
                                     "reference computes it, 900 input + 99 recurrent at full size",
                        "connectivity": "host front end, connect_with_sparsity (Examples/UtilityFunctions.hpp:51-82)"})
        else:
            m = networks.plastic_ff_generated(n_in=n_in, n_neurons=n_neu, rule=RULES[rule])
            cfg.update({"in_degree": "binomial, mean 900 input + 100 recurrent", "connectivity": "drawn on the GPU"})
        L = 1
    return m, cfg, L


def algorithmic_bytes(events: int, pre_updates: int, post_updates: int, neuron_steps: int, input_steps: int,
                      L: int, trace_steps: int = 0) -> int:
    """Per-unit algorithmic HBM bytes of the step: 8 B per synaptic event
    (packed post/delay/label + fp32 weight), 8 B per plastic weight updated on
    a presynaptic event (weight read and write-back), 16 B per plastic
    afferent updated on a postsynaptic spike (afferent record + weight
    write-back + presynaptic trace), 12 + 16 L B per neuron-step, 8 B per
    input-step, 4 B per presynaptic trace published in a plastic run."""
    return (8 * events + 8 * pre_updates + 16 * post_updates + (12 + 16 * L) * neuron_steps + 8 * input_steps
            + 4 * trace_steps)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except Exception:
            return out
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except Exception:
                continue
            for i, name in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(name)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def aggregate_over_ranks(elapsed_s: float, events: int, dist, device: str):
    """Whole-job timing of replicas: the slowest rank's time and the events
    of all ranks (each rank simulates its own networks; no data-path
    exchange).  `dist` is torch.distributed or None for one process."""
    import torch
    el = torch.tensor([float(elapsed_s)], device=device, dtype=torch.float64)
    ev = torch.tensor([float(events)], device=device, dtype=torch.float64)
    if dist:
        dist.all_reduce(el, op=dist.ReduceOp.MAX)
        dist.all_reduce(ev, op=dist.ReduceOp.SUM)
    return float(el.item()), float(ev.item())


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_launch(workload: str):
    """The committed ncu summary of the timed kernel on this workload
    (profiles/step_kernel_<workload>.json): DRAM bytes of a captured launch per
    algorithmic byte (or per synaptic event) of that launch, applied to this
    run's launches."""
    path = os.path.join(ROOT, "profiles", f"step_kernel_{workload}.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


def networks_small_plastic_ff(rule: str = "weight_dependent"):
    from spike_gb300 import networks
    return networks.plastic_ff_generated(n_in=2500, n_neurons=10000, ff=900, rec=100, rule=RULES[rule])


def networks_small_plastic_ff_exact():
    """The exact (fixed in-degree) construction at 1/20 size, for the CPU samples."""
    from spike_gb300 import networks
    return networks.plastic_ff(n_in=2500, n_neurons=10000, ff=900, rec=100)


# Per plastic synapse and timestep, the weight normalisation reads the record
# (8 B) and the initial weight (4 B) and writes the weight back (8 B record).
NORM_BYTES = 20

# Per plastic synapse and timestep, a per-synapse-trace rule's pass reads the
# afferent record (8 B), its delay (4 B) and its two traces (8 B) and writes
# the weight (4 B) and the traces (8 B).
TRACE_RULE_BYTES = 32


def cpu_baseline(desc, steps: int, threads: int):
    from oracle import OracleNet
    o = OracleNet(desc, 32, threads=threads)
    t0 = time.perf_counter()
    o.run_steps(steps, True)
    el = time.perf_counter() - t0
    return o.events() / el, el


def run_reference(args, rank, world):
    """CPU reference arm: the oracle port with all host threads."""
    if rank != 0:
        return
    m, cfg, L = build_model(args.workload, args.scale, args.rule, args.norm, args.construction,
                            describe_only=True)
    threads = os.cpu_count() or 1
    from oracle import OracleNet
    from spike_gb300 import GenNetwork
    small = None
    if isinstance(m, GenNetwork):
        # too large to draw on the host: the same construction at 1/20 size
        dd = oracle_instance(networks_small_plastic_ff(args.rule))[1]
        desc = dd.desc
        cfg = {**cfg, "cpu_sample_network": "same construction at 1/20 size (2,500 inputs, 10,000 neurons)"}
    elif args.workload == "plastic_ff":
        # 2e8 synapses: the same construction at 1/20 size keeps the sample bounded
        small = networks_small_plastic_ff_exact()
        desc = small.desc()
        cfg = {**cfg, "cpu_sample_network": "same construction at 1/20 size (2,500 inputs, 10,000 neurons)"}
    else:
        desc = m.desc()
    o = OracleNet(desc, 32, threads=threads)
    sample = max(1, min(args.block, 1000))
    for _ in range(args.warmup):
        o.run_steps(sample // 4 or 1, True)
    e0 = o.events()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.run_steps(sample, True)
    el = time.perf_counter() - t0
    ev = o.events() - e0
    value = ev / el
    line = {"metric": "synaptic_events_per_s", "value": value, "unit": "events/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference", "config": {**cfg, "block_timesteps": sample},
            "sim_s_per_wall_s": args.steps * sample * DT / el,
            "cpu_baseline": {"value": value, "unit": "events/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} x {sample} timesteps of the workload"},
            "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if args.workload == "batched":
            return run_reference_batched(args, rank, world)
        return run_reference(args, rank, world)
    if args.workload == "batched":
        return run_batched(args, rank, world, local)
    if args.workload == "served":
        return run_served(args, rank, world, local)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import __graft_entry__
    __graft_entry__.build()
    from spike_gb300 import schedule

    from spike_gb300 import GenNetwork, Net
    m, cfg, L = build_model(args.workload, args.scale, args.rule, args.norm, args.construction)
    sched = schedule(args.warps, args.tile, args.ctas, args.launch_steps or args.block)
    if isinstance(m, GenNetwork):
        net = Net.generate(m, sched)
        n_neurons, n_inputs, n_syn = m.desc.n_neurons, m.desc.n_inputs, net.synapse_count()
        desc = None
    else:
        desc = m.desc()
        net = m.finalise(sched)
        n_neurons, n_inputs, n_syn = m.counts()
    trace_rule = args.workload == "plastic_ff" and args.rule != "weight_dependent"
    normalised = args.workload == "brunel" and args.norm != "off"
    # the event-driven rule's traces
    plastic_run = (args.workload == "plastic_ff" and not trace_rule) or normalised
    n_plastic = net.plastic_synapse_count()
    stream = torch.cuda.ExternalStream(net.stream())

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    # ---- device-timed throughput --------------------------------------------------
    for _ in range(args.warmup):
        net.run_steps(args.block, True)
    assert net.synchronize() == 0
    net.clear_spikes()
    barrier()
    e0, l0 = net.events(), net.launches()
    pre0, post0 = net.stdp_counts()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        start.record(stream)
        for _ in range(args.steps):
            net.run_steps(args.block, True)
        stop.record(stream)
        stop.synchronize()
        barrier()
    status = net.synchronize()
    ms = start.elapsed_time(stop)
    events = net.events() - e0
    launches = net.launches() - l0
    pre1, post1 = net.stdp_counts()
    elapsed, total_events = aggregate_over_ranks(ms / 1000.0, events, dist, "cuda")
    value = total_events / elapsed
    sim_s = args.steps * args.block * DT

    # ---- roofline of the step kernel ----------------------------------------------------
    timesteps = args.steps * args.block
    alg = algorithmic_bytes(events, pre1 - pre0, post1 - post0, n_neurons * timesteps, n_inputs * timesteps, L,
                            (n_neurons + n_inputs) * timesteps if plastic_run else 0)
    if trace_rule:
        alg += TRACE_RULE_BYTES * n_plastic * timesteps
    if normalised:
        alg += NORM_BYTES * n_plastic * timesteps
    per_launch_s = (ms / 1000.0) / max(launches, 1)
    per_launch_bytes = alg / max(launches, 1)
    peak, peak_kind = peaks()
    achieved = per_launch_bytes / per_launch_s / 1e9
    tr = traffic_per_launch(f"{args.workload}_{args.rule}" if trace_rule else
                            f"{args.workload}_norm_{args.norm}" if normalised else args.workload)
    traffic = None
    if tr and tr.get("traffic_per_alg_byte"):
        traffic = tr["traffic_per_alg_byte"] * per_launch_bytes

    # ---- end to end through the public API --------------------------------------------
    e2e = None
    if not args.no_e2e:
        rates = torch.full((max(n_inputs, 1),), 20.0, dtype=torch.float32).pin_memory()
        if n_inputs and args.workload == "plastic_ff":
            import numpy as np
            src = m.desc if isinstance(m, GenNetwork) else desc  # the stimulus the network was built with
            rates.copy_(torch.from_numpy(np.ctypeslib.as_array(src.input_rates, (n_inputs,)).copy()))
        h2d = 4 * n_inputs
        d2h = 0
        net.clear_spikes()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            if n_inputs:
                net.write_rates(0, rates.data_ptr(), n_inputs)
            net.run_steps(args.block, True)
            ids, times = net.spikes()
            d2h += 8 * len(ids) + 16
            net.clear_spikes()
        barrier()
        t_e2e = time.perf_counter() - t0
        e2e_events = net.events() - e0 - events
        e2e = {"value": e2e_events / t_e2e, "unit": "events/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": int(d2h / args.steps), "sim_s_per_wall_s": sim_s / t_e2e}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        if desc is None:
            # the generated network is too large to draw on the host: a
            # 1/20-size network of the same construction stands in
            cs = CpuSample([networks_small_plastic_ff(args.rule)])
            cv, cel = cs.run(args.cpu_sample_steps // 10, 1)
            cpu = {"value": cv, "unit": "events/s", "cores": 1, "kind": "port",
                   "sample": f"the same construction at 1/20 size (2,500 inputs, 10,000 neurons), "
                             f"{args.cpu_sample_steps // 10} timesteps from reset, {cel:.1f} s of CPU"}
        elif args.workload == "plastic_ff":
            # 2e8 synapses on one core: the exact construction at 1/20 size stands in
            small = networks_small_plastic_ff_exact()
            cv, cel = cpu_baseline(small.desc(), args.cpu_sample_steps // 10, 1)
            cpu = {"value": cv, "unit": "events/s", "cores": 1, "kind": "port",
                   "sample": f"the same construction at 1/20 size (2,500 inputs, 10,000 neurons), "
                             f"{args.cpu_sample_steps // 10} timesteps from reset, {cel:.1f} s of CPU"}
        else:
            cv, cel = cpu_baseline(desc, args.cpu_sample_steps, 1)
            cpu = {"value": cv, "unit": "events/s", "cores": 1, "kind": "port",
                   "sample": f"{args.cpu_sample_steps} timesteps ({args.cpu_sample_steps * DT:.2f} s simulated) "
                             f"from reset, {cel:.1f} s of CPU"}

    # the reference's own CUDA kernels on the same network and GPU model, once
    # (tests/golden/make_ref_gpu_stats.py): a second reference line for context
    ref_gpu = None
    ref_case = {"vogels_abbott": "va", "brunel": "brunel_cfg2"}.get(args.workload)
    if ref_case and args.rule == "weight_dependent" and args.norm == "off" and args.scale == 1.0:
        try:
            with open(os.path.join(ROOT, "tests", "golden", "ref_gpu_stats.json")) as f:
                rg = json.load(f)[ref_case]
            ref_gpu = {"value": rg["events_per_s"], "unit": "events/s", "wall_s": rg["wall_s"],
                       "sim_s": rg["seconds"], "source": "tests/golden/ref_gpu_stats.json (the reference's CUDA "
                       "backend built for sm_103a, run once on a GB300 host without a spike monitor)"}
        except Exception:
            ref_gpu = None

    if rank == 0:
        line = {
            "metric": "synaptic_events_per_s", "value": value, "unit": "events/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "ours",
            "config": {**cfg, "block_timesteps": args.block, "synapses": n_syn, "plastic_synapses": n_plastic,
                       "schedule": net.schedule(),
                       "l2": f"synapse entries {8 * n_syn / 1e6:.0f} MB > 129 MB L2 (no flush)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "sim_s_per_wall_s": sim_s * world / (elapsed * world) if world else None,
            "status": status,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "traffic_source": (f"profiles/step_kernel_*.json: DRAM bytes per algorithmic byte of "
                                            f"one ncu capture ({tr.get('capture', '')}), times this run's "
                                            f"algorithmic bytes" if tr else None),
                         "kernel": ("bulk kernels of one timestep (neurons, list, per-synapse-trace rule, "
                                    "propagation)" if trace_rule else
                                    "bulk kernels of one timestep (neurons, list, propagation passes, afferent "
                                    "pass, weight normalisation)" if normalised else "spk::step_kernel"),
                         "launches": launches,
                         "alg_bytes_per_launch": per_launch_bytes, "ms_per_launch": 1000 * per_launch_s},
            "e2e": e2e, "cpu_baseline": cpu, "reference_gpu": ref_gpu, "clocks": clk.summary(),
            "gpu_launches": launches + args.steps,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


# ---- batched sweep ------------------------------------------------------------------

PLAIN_WARMUP = 200           # timesteps each instance runs alone before the plain form is timed
BATCH_CPU_INSTANCES = 16     # instances of the sweep run by the CPU baselines, spread over its sizes
BATCH_CPU_STEPS = 100        # timesteps of each from reset


def batched_config(gens, n_syn=None):
    n = [g.desc.n_neurons for g in gens]
    cfg = {"workload": f"batched_sweep_{len(gens)}_instances_N{min(n)}-{max(n)}",
           "instances": len(gens), "neurons": int(sum(n)), "inputs": int(sum(g.desc.n_inputs for g in gens)),
           "plastic_instances": int(sum(1 for g in gens if g.desc.has_stdp)),
           "connectivity": "Bernoulli p~U[0.01,0.05], inputs n/5 at 20 Hz with p_in=4p, g~U[3,7], delays U{1..10}",
           "dt_ms": 0.1, "sim_s_per_instance_config": 1.0}
    if n_syn is not None:
        cfg["synapses"] = int(n_syn)
    return cfg


def cpu_sample_gens(gens, count=BATCH_CPU_INSTANCES):
    """`count` instances of the sweep at evenly spaced ranks of its sizes,
    smallest to largest (the CPU's events/s depends on the instance size, and
    on STDP, whose reference form updates every plastic synapse every
    timestep, so the sample spans the whole range)."""
    order = sorted(range(len(gens)), key=lambda k: gens[k].desc.n_neurons)
    n = min(count, len(order))
    pick = sorted({order[(i * (len(order) - 1)) // max(n - 1, 1)] for i in range(n)})
    return [gens[k] for k in pick], pick


def oracle_instance(gen):
    from oracle import OracleNet
    from oracle.binding import generate_synapses
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import descs
    a = generate_synapses(gen.desc)
    d = gen.desc
    groups = [dict(count=d.groups[i].count, tau_m=d.groups[i].tau_m, R=d.groups[i].R, v0=d.groups[i].v0,
                   vreset=d.groups[i].vreset, theta=d.groups[i].theta) for i in range(d.n_groups)]
    import numpy as np
    rates = np.ctypeslib.as_array(d.input_rates, (d.n_inputs,)).copy()
    dd = descs.Desc(kind=d.synapse_kind, groups=groups, refractory=d.refractory_period, n_inputs=d.n_inputs,
                    rates=rates, pre=a["pre"], post=a["post"], weight=a["weight"], scale=a["scale"],
                    delay=a["delay"], label=a["label"], plastic=a["plastic"] if d.has_stdp else None,
                    stdp=None, seed=d.seed)
    if d.has_stdp:
        dd.desc.has_stdp = 1
        dd.desc.stdp = d.stdp
        dd.desc.stdp_rule = d.stdp_rule
    return OracleNet(dd.desc, 32, threads=1), dd


class CpuSample:
    """The oracle on the CPU sample of the sweep, built once."""

    def __init__(self, gens, count=BATCH_CPU_INSTANCES):
        picked, self.index = cpu_sample_gens(gens, count)
        self.gens = picked
        self.nets = [None] * len(picked)
        import threading
        th = [threading.Thread(target=self._build, args=(i,)) for i in range(len(picked))]
        for t in th:
            t.start()
        for t in th:
            t.join()
        sizes = [g.desc.n_neurons for g in picked]
        self.label = (f"{len(self.nets)} instances of the sweep at evenly spaced size ranks (N {min(sizes)}-"
                      f"{max(sizes)}, {sum(1 for g in picked if g.desc.has_stdp)} with STDP)")

    def _build(self, i):
        self.nets[i] = oracle_instance(self.gens[i])[0]

    def run(self, steps, threads):
        """Events/s of `steps` timesteps of every sample instance, the
        instances shared out over `threads` host threads (largest first)."""
        import threading
        results = [0] * len(self.nets)
        todo = sorted(range(len(self.nets)), key=lambda i: -self.gens[i].desc.n_neurons)
        lock = threading.Lock()

        def work():
            while True:
                with lock:
                    if not todo:
                        return
                    i = todo.pop(0)
                o = self.nets[i]
                e0 = o.events()
                o.run_steps(steps, True)
                results[i] = o.events() - e0

        t0 = time.perf_counter()
        th = [threading.Thread(target=work) for _ in range(max(1, threads))]
        for t in th:
            t.start()
        for t in th:
            t.join()
        el = time.perf_counter() - t0
        return sum(results) / el, el


def run_reference_batched(args, rank, world):
    """CPU reference arm for the batched sweep: the oracle port of the
    reference's step loop on a sample of the sweep spread over its whole size
    range (cpu_sample_gens), every instance from reset, shared out over the
    host's threads."""
    if rank != 0:
        return
    from spike_gb300 import networks
    gens = networks.batched_sweep(args.instances)
    threads = os.cpu_count() or 1
    cs = CpuSample(gens)
    vals, els = [], []
    for i in range(args.warmup + args.steps):
        for o in cs.nets:
            o.reset_state()
            o.reset_time()
        v, el = cs.run(BATCH_CPU_STEPS, threads)
        if i >= args.warmup:
            vals.append(v)
            els.append(el)
    value = sum(vals) / len(vals)
    sample = f"{cs.label}, {BATCH_CPU_STEPS} timesteps each from reset per step, {threads} host threads"
    line = {"metric": "synaptic_events_per_s", "value": value, "unit": "events/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(els) / len(els),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference", "config": batched_config(gens),
            "cpu_baseline": {"value": value, "unit": "events/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batched(args, rank, world, local):
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__
    __graft_entry__.build()
    from spike_gb300 import Batch, Net, networks, schedule
    from spike_gb300 import _native as N

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    gens = networks.batched_sweep(args.instances)
    t0 = time.perf_counter()
    mode = N.SPK_BATCH_WAVES
    if args.range:
        scheds = [schedule(1, min(args.range, -(-g.desc.n_neurons // 32) * 32), 0, 0) for g in gens]
        tune_ms = None
        nets = [Net.generate(g, s) for g, s in zip(gens, scheds)]
        costs = [0.0 for _ in gens]
        mode = N.SPK_BATCH_BULK
    elif args.no_tune:
        scheds = [schedule(8, min(64, max(32, -(-(-(-g.desc.n_neurons // 8)) // 32) * 32)), 0, 0) for g in gens]
        tune_ms = None
        nets = [Net.generate(g, s) for g, s in zip(gens, scheds)]
        costs = [float(n.synapse_count()) * (2.0 if g.desc.has_stdp else 1.0) for n, g in zip(nets, gens)]
    else:
        scheds, tune_ms, costs, mode = Batch.autotune(gens, trial_steps=args.tune_steps, costs=True,
                                                      with_mode=True)
        nets = [Net.generate(g, s) for g, s in zip(gens, scheds)]
    tune_s = time.perf_counter() - t0
    for n, c in zip(nets, costs):
        if c > 0:
            n.set_step_cost(c)
    n_syn = sum(n.synapse_count() for n in nets)
    b = Batch(nets, schedule(0, 0, 0, args.block))
    if args.mode != "auto":
        mode = N.SPK_BATCH_BULK if args.mode == "bulk" else N.SPK_BATCH_WAVES
    b.set_mode(mode)
    stream = torch.cuda.ExternalStream(b.stream())
    n_neurons = sum(g.desc.n_neurons for g in gens)
    n_inputs = sum(g.desc.n_inputs for g in gens)

    for _ in range(args.warmup):
        b.run_steps(args.block, True)
    assert b.synchronize() == 0
    for n in nets:
        n.clear_spikes()
    barrier()
    e0 = sum(n.events() for n in nets)
    l0 = b.launches()
    st0 = [n.stdp_counts() for n in nets]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        start.record(stream)
        for _ in range(args.steps):
            b.run_steps(args.block, True)
        stop.record(stream)
        stop.synchronize()
        barrier()
    status = b.synchronize()
    ms = start.elapsed_time(stop)
    events = sum(n.events() for n in nets) - e0
    launches = b.launches() - l0
    elapsed, total_events = aggregate_over_ranks(ms / 1000.0, events, dist, "cuda")
    value = total_events / elapsed
    sim_s = args.steps * args.block * DT

    # roofline: algorithmic bytes of all instances over the step-kernel launches
    timesteps = args.steps * args.block
    st1 = [n.stdp_counts() for n in nets]
    pre_u = sum(b1[0] - a1[0] for a1, b1 in zip(st0, st1))
    post_u = sum(b1[1] - a1[1] for a1, b1 in zip(st0, st1))
    trace_keys = sum(g.desc.n_neurons + g.desc.n_inputs for g in gens if g.desc.has_stdp)
    alg = algorithmic_bytes(events, pre_u, post_u, n_neurons * timesteps, n_inputs * timesteps, 1,
                            trace_keys * timesteps)
    bulk = mode == N.SPK_BATCH_BULK
    # waves: one launch of the persistent kernel per wave and block; bulk: the
    # unit is one timestep of all instances (neuron, list, propagation and,
    # with plastic instances, afferent-pass kernels)
    units = timesteps if bulk else max(launches, 1)
    per_launch_s = (ms / 1000.0) / units
    per_launch_bytes = alg / units
    peak, peak_kind = peaks()
    achieved = per_launch_bytes / per_launch_s / 1e9
    tr = None if bulk else traffic_per_launch("batched")
    traffic = None
    if tr and tr.get("traffic_per_alg_byte"):
        traffic = tr["traffic_per_alg_byte"] * per_launch_bytes
    roof_kernel = ("spk::bulk_neurons_kernel + bulk_list_kernel + bulk_prop_kernel + bulk_post_kernel "
                   "(one timestep of all instances)" if bulk else "spk::step_kernel")
    roof_timestep = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind, "kernel": roof_kernel, "launches": launches,
                     "unit_timed": "timestep" if bulk else "launch", "alg_bytes_per_launch": per_launch_bytes,
                     "ms_per_launch": 1000 * per_launch_s, "events_per_timestep": events / timesteps}
    roofline, kernels = roof_timestep, None
    if bulk:
        # each kernel of one block launched alone between CUDA events on its
        # stream: the kernels' device times, and the propagation kernel's own
        # roofline (8 B per synaptic event and per plastic weight updated on a
        # presynaptic event, both done by the propagation kernel)
        ke0 = sum(n.events() for n in nets)
        ks0 = [n.stdp_counts() for n in nets]
        kms = b.time_kernels(args.block)
        kev = sum(n.events() for n in nets) - ke0
        kpre = sum(y[0] - x[0] for x, y in zip(ks0, [n.stdp_counts() for n in nets]))
        tot = sum(kms.values())
        kernels = {k: {"ms_per_timestep": v / args.block, "share": v / tot if tot else None} for k, v in kms.items()}
        prop_bytes = (8 * kev + 8 * kpre) / args.block
        prop_s = kms["propagation"] / 1000.0 / args.block
        prop_ach = prop_bytes / prop_s / 1e9 if prop_s > 0 else None
        pt = traffic_per_launch("batched_bulk_prop")
        prop_traffic = pt["dram_bytes_per_event"] * kev / args.block if pt and pt.get("dram_bytes_per_event") else None
        roofline = {"bound": "hbm", "achieved": prop_ach, "peak": peak, "unit": "GB/s",
                    "frac": prop_ach / peak if prop_ach else None, "traffic": prop_traffic,
                    "traffic_source": pt.get("source") if pt else None, "peak_kind": peak_kind,
                    "kernel": "spk::bulk_prop_kernel / bulk_range_kernel (propagation and the STDP pre pass of "
                              "all instances, one launch per timestep)",
                    "launches": args.block, "unit_timed": "timestep",
                    "alg_bytes_per_launch": prop_bytes, "ms_per_launch": 1000 * prop_s,
                    "events_per_timestep": kev / args.block,
                    "timing": "CUDA events around each launch on the batch stream, one block of timesteps"}

    # plain form: the same instances, each alone with the schedule the
    # library's planner gives it on its own (the persistent kernel), one after
    # another: PLAIN_WARMUP timesteps, then plain_block timed
    plain_ev, plain_ms, plain_sched = 0, 0.0, {}
    for g in gens:
        n = Net.generate(g, schedule(0, 0, 0, args.plain_block))
        sc = n.schedule()
        k = f"{sc['warps_per_cta']}x{sc['tile_posts']}x{sc['ctas']}"
        plain_sched[k] = plain_sched.get(k, 0) + 1
        s = torch.cuda.ExternalStream(n.stream())
        n.run_steps(PLAIN_WARMUP, True)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        pe0 = n.events()
        a0.record(s)
        n.run_steps(args.plain_block, True)
        a1.record(s)
        a1.synchronize()
        assert n.synchronize() == 0
        plain_ms += a0.elapsed_time(a1)
        plain_ev += n.events() - pe0
        n.close()
    plain = {"value": plain_ev / (plain_ms / 1000.0), "unit": "events/s",
             "sample": f"every instance alone under its own planner schedule (the persistent kernel), "
                       f"{PLAIN_WARMUP} timesteps from reset then {args.plain_block} timed, one after another",
             "schedules": plain_sched,
             "sim_s_per_wall_s": len(nets) * args.plain_block * DT / (plain_ms / 1000.0)}

    # end to end through the public API: rates up, batch step, spikes back
    e2e = None
    if not args.no_e2e:
        import numpy as np
        pinned = [torch.from_numpy(np.ctypeslib.as_array(g.desc.input_rates, (g.desc.n_inputs,)).copy()).pin_memory()
                  for g in gens]
        for n in nets:
            n.clear_spikes()
        # spike readback of all instances at once into page-locked buffers
        cap = 1 << 25
        ids_buf = torch.empty(cap, dtype=torch.int32, pin_memory=True)
        times_buf = torch.empty(cap, dtype=torch.float32, pin_memory=True)
        barrier()
        ee0 = sum(n.events() for n in nets)
        h2d = 4 * n_inputs
        d2h = 0
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for n, r in zip(nets, pinned):
                n.write_rates(0, r.data_ptr(), r.numel())
            b.run_steps(args.block, True)
            while True:
                counts = b.read_spikes_into(ids_buf.data_ptr(), times_buf.data_ptr(), cap, clear=True)
                if counts is not None:
                    break
                cap *= 2
                ids_buf = torch.empty(cap, dtype=torch.int32, pin_memory=True)
                times_buf = torch.empty(cap, dtype=torch.float32, pin_memory=True)
            d2h += 8 * int(counts.sum()) + 8 * len(nets)
        barrier()
        t_e2e = time.perf_counter() - t0
        e2e_events = sum(n.events() for n in nets) - ee0
        e2e = {"value": e2e_events / t_e2e, "unit": "events/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": int(d2h / args.steps),
               "sim_s_per_wall_s": len(nets) * sim_s / t_e2e}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the CPU sample, and the same instances over the same timesteps from
        # reset on the GPU (a batch of them alone), for a like-for-like ratio
        cs = CpuSample(gens)
        threads = os.cpu_count() or 1
        cv, cel = cs.run(BATCH_CPU_STEPS, threads)
        sub = [Net.generate(gens[k], scheds[k]) for k in cs.index]
        bs = Batch(sub, schedule(0, 0, 0, BATCH_CPU_STEPS))
        bs.set_mode(mode)
        sst = torch.cuda.ExternalStream(bs.stream())
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(sst)
        bs.run_steps(BATCH_CPU_STEPS, True)
        a1.record(sst)
        a1.synchronize()
        gpu_sample = sum(n.events() for n in sub) / (a0.elapsed_time(a1) / 1000.0)
        bs.close()
        for n in sub:
            n.close()
        cpu = {"value": cv, "unit": "events/s", "cores": threads, "kind": "port",
               "sample": f"{cs.label}, {BATCH_CPU_STEPS} timesteps each from reset, {cel:.1f} s on {threads} "
                         f"host threads",
               "gpu_on_sample": {"value": gpu_sample, "unit": "events/s",
                                 "what": "the same instances and timesteps as one batch on the GPU (device time)"}}

    if rank == 0:
        sch = {}
        for s in scheds:
            k = f"{s.warps_per_cta}x{s.tile_posts}"
            sch[k] = sch.get(k, 0) + 1
        line = {
            "metric": "synaptic_events_per_s", "value": value, "unit": "events/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "ours",
            "config": {**batched_config(gens, n_syn), "block_timesteps": args.block,
                       "schedules": sch, "autotune_s": round(tune_s, 2), "autotune_trial_ms": tune_ms,
                       "launches_per_block": launches / max(1, args.steps),
                       "autotuned": not (args.no_tune or args.range),
                       "mode": "bulk" if mode == N.SPK_BATCH_BULK else "waves",
                       "l2": f"synapse entries {8 * n_syn / 1e9:.1f} GB > 129 MB L2 (no flush)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "sim_s_per_wall_s": len(nets) * sim_s / elapsed,
            "stdp_updates": {"pre": pre_u, "post_afferents": post_u},
            "plain": plain, "batched_over_plain": value / plain["value"],
            "status": status,
            "roofline": roofline, "roofline_timestep": roof_timestep, "kernels": kernels,
            "e2e": e2e, "cpu_baseline": cpu, "clocks": clk.summary(),
            "gpu_launches": launches + args.steps * len(nets),
        }
        print(json.dumps(line), flush=True)
    b.close()
    if dist:
        dist.destroy_process_group()


# ---- served stream ------------------------------------------------------------------

def served_requests(duration, rate, seed=2024):
    """Poisson arrivals (mean `rate` per second) of jobs with N log-uniform in
    [2k, 100k], simulated time U[0.5, 5] s, 30 % with STDP, other draws as in
    the batched sweep; fixed arrival seed."""
    import numpy as np
    from spike_gb300.networks import sweep_instance
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        n = int(np.exp(rng.uniform(np.log(2000), np.log(100000))))
        p, g = float(rng.uniform(0.01, 0.05)), float(rng.uniform(3.0, 7.0))
        plastic = bool(rng.uniform() < 0.3)
        sim = float(rng.uniform(0.5, 5.0))
        out.append((t, sweep_instance(n, p, g, plastic, seed=int(rng.integers(1, 2**31))), int(round(sim / DT))))
    return out


def run_served(args, rank, world, local):
    """Requests arrive by a Poisson process for --duration seconds and are
    submitted to the continuous-batching server.  value = synaptic events the
    server delivered during the arrival window (all jobs, finished or
    running) / window; latency percentiles are over the jobs that finished
    inside the window (submit to finish).  When the window closes the server
    stops: jobs still queued or running are cancelled."""
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    import __graft_entry__
    __graft_entry__.build()
    from spike_gb300 import Server
    from spike_gb300 import _native as N
    if rank != 0:
        return
    reqs = served_requests(args.duration, args.arrival_rate)
    mode = N.SPK_BATCH_WAVES if args.mode == "waves" else N.SPK_BATCH_BULK
    srv = Server(steps_per_block=args.block, record_spikes=False, mode=mode)
    ids = []
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for (t, gen, steps) in reqs:
            wait = t - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            ids.append(srv.submit(gen, steps, True))
        rest = args.duration - (time.perf_counter() - t0)
        if rest > 0:
            time.sleep(rest)
        window = time.perf_counter() - t0
        st = srv.stats()
        infos = [srv.poll(j) for j in ids]
    srv.stop()
    lat = [i.finish_s - i.submit_s for i in infos if i.state == N.SPK_JOB_DONE]
    wait_s = [i.start_s - i.submit_s for i in infos if i.state in (N.SPK_JOB_DONE, N.SPK_JOB_RUNNING)]
    sim_done = sum(i.steps_done for i in infos) * DT
    line = {"metric": "synaptic_events_per_s", "value": float(st.events) / window, "unit": "events/s",
            "n_gpus": 1, "steps": len(ids), "warmup": 0, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "ours",
            "config": {"workload": f"served_stream_rate{args.arrival_rate:g}_N2k-100k_T0.5-5s_stdp30pct",
                       "arrival_window_s": args.duration, "block_timesteps": args.block,
                       "mode": "waves" if mode == N.SPK_BATCH_WAVES else "bulk"},
            "sim_s_per_wall_s": sim_done / window,
            "latency_s": {"p50": float(np.percentile(lat, 50)) if lat else None,
                          "p99": float(np.percentile(lat, 99)) if lat else None, "n": len(lat)},
            "admission_wait_s": {"p50": float(np.percentile(wait_s, 50)) if wait_s else None,
                                 "p99": float(np.percentile(wait_s, 99)) if wait_s else None},
            "jobs": {"submitted": len(ids),
                     "done": int(sum(1 for i in infos if i.state == N.SPK_JOB_DONE)),
                     "running_at_close": int(sum(1 for i in infos if i.state == N.SPK_JOB_RUNNING)),
                     "queued_at_close": int(sum(1 for i in infos if i.state == N.SPK_JOB_QUEUED)),
                     "failed": int(sum(1 for i in infos if i.state == N.SPK_JOB_FAILED)),
                     "blocks": int(st.blocks), "batch_rebuilds": int(st.rebuilds), "gpu_busy_s": st.busy_s},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
