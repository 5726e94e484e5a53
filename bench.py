"""Benchmark of the clock-driven step: synaptic events/s on one GB300.

Workload (default): the Brunel network of Examples/Brunel10K.cpp at the sizes
of the benchmark's second configuration - 10,000 excitatory + 2,500
inhibitory voltage-synapse LIF neurons, 10,000 Poisson inputs at 20 Hz, fixed
in-degree 0.1 (1,000 E + 250 I + 1,000 input afferents per neuron), J = 0.1 mV,
g = 5, delays U{1..20} steps, dt = 0.1 ms; 28.1 M synapses (225 MB of synapse
entries, larger than the 129 MB L2).  Data are synthetic (built by the
reference's construction rules), weights fixed as in the model.

A bench "step" is one block of --block timesteps (default 1000 = 0.1 s of
simulated time); the default 20 steps cover the configuration's 2 s.

Printed JSON (one line): value = synaptic events/s over the timed region
(events = sum over spikes of the spiking neuron's out-degree), device-timed
with CUDA events on the engine's stream; e2e = the same metric through the
public run API with a host->device rate upload and a device->host spike
readback every step; roofline for the step kernel; cpu_baseline = the CPU
oracle (a single-thread C++ transcription of the reference step loop) on a
bounded sample.

--impl reference: the reference has no CPU implementation of the step (its
only backend is CUDA; the Dummy backend computes nothing), so the reference
arm times the oracle port of its step loop with all host threads.
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
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="brunel", choices=["brunel", "vogels_abbott", "plastic_ff"])
    p.add_argument("--block", type=int, default=1000, help="timesteps per bench step")
    p.add_argument("--ctas", type=int, default=0)
    p.add_argument("--warps", type=int, default=0)
    p.add_argument("--tile", type=int, default=0)
    p.add_argument("--launch-steps", type=int, default=0)
    p.add_argument("--cpu-sample-steps", type=int, default=5000)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    return p.parse_args()


def build_model(workload: str):
    from spike_gb300 import networks
    if workload == "brunel":
        m = networks.brunel()
        cfg = {"workload": "brunel_12500_lif_10000_poisson_delays1-20", "neurons": 12500, "inputs": 10000,
               "in_degree": 2250, "delays_steps": [1, 20], "dt_ms": 0.1, "sim_s_per_config": 2.0,
               "plasticity": False}
        L = 1
    elif workload == "vogels_abbott":
        m = networks.vogels_abbott()
        cfg = {"workload": "vogels_abbott_4000_cond_lif_p0.02_delay1", "neurons": 4000, "inputs": 0,
               "dt_ms": 0.1, "sim_s_per_config": 1.0, "plasticity": False}
        L = 2
    else:
        m = networks.plastic_ff()
        cfg = {"workload": "plastic_ff_200000_lif_50000_poisson_stdp", "neurons": 200000, "inputs": 50000,
               "dt_ms": 0.1, "sim_s_per_config": 5.0, "plasticity": True}
        L = 1
    return m, cfg, L


def algorithmic_bytes(events: int, plastic_events: int, neuron_steps: int, input_steps: int, L: int) -> int:
    """Per-unit algorithmic HBM bytes of the step: 8 B per synaptic event
    (int32 post + fp32 weight), +4 B per plastic event (weight write-back),
    12 + 16 L B per neuron-step, 8 B per input-step."""
    return 8 * events + 4 * plastic_events + (12 + 16 * L) * neuron_steps + 8 * input_steps


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


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_launch(workload: str):
    """DRAM bytes per launch of the step kernel from the committed ncu summary
    (profiles/step_kernel_<workload>.json), scaled to this launch length."""
    path = os.path.join(ROOT, "profiles", f"step_kernel_{workload}.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


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
    m, cfg, L = build_model(args.workload)
    desc = m.desc()
    threads = os.cpu_count() or 1
    from oracle import OracleNet
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
        return run_reference(args, rank, world)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import __graft_entry__
    __graft_entry__.build()
    from spike_gb300 import schedule

    m, cfg, L = build_model(args.workload)
    desc = m.desc()
    sched = schedule(args.warps, args.tile, args.ctas, args.launch_steps or args.block)
    net = m.finalise(sched)
    n_neurons, n_inputs, n_syn = m.counts()
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
    el = torch.tensor([ms / 1000.0], device="cuda")
    ev = torch.tensor([float(events)], device="cuda", dtype=torch.float64)
    if dist:
        dist.all_reduce(el, op=dist.ReduceOp.MAX)
        dist.all_reduce(ev, op=dist.ReduceOp.SUM)
    elapsed = float(el.item())
    total_events = float(ev.item())
    value = total_events / elapsed
    sim_s = args.steps * args.block * DT

    # ---- roofline of the step kernel ----------------------------------------------------
    timesteps = args.steps * args.block
    alg = algorithmic_bytes(events, 0, n_neurons * timesteps, n_inputs * timesteps, L)
    per_launch_s = (ms / 1000.0) / max(launches, 1)
    per_launch_bytes = alg / max(launches, 1)
    peak, peak_kind = peaks()
    achieved = per_launch_bytes / per_launch_s / 1e9
    tr = traffic_per_launch(args.workload)
    traffic = None
    if tr and tr.get("dram_bytes_per_timestep"):
        traffic = tr["dram_bytes_per_timestep"] * (timesteps / max(launches, 1))

    # ---- end to end through the public API --------------------------------------------
    e2e = None
    if not args.no_e2e:
        rates = torch.full((max(n_inputs, 1),), 20.0, dtype=torch.float32).pin_memory()
        if n_inputs and args.workload == "plastic_ff":
            from spike_gb300 import networks
            rates.copy_(torch.from_numpy(networks.lognormal_rates(n_inputs)))
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
        cv, cel = cpu_baseline(desc, args.cpu_sample_steps, 1)
        cpu = {"value": cv, "unit": "events/s", "cores": 1, "kind": "port",
               "sample": f"{args.cpu_sample_steps} timesteps ({args.cpu_sample_steps * DT:.2f} s simulated) "
                         f"from reset, {cel:.1f} s of CPU"}

    if rank == 0:
        line = {
            "metric": "synaptic_events_per_s", "value": value, "unit": "events/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "ours",
            "config": {**cfg, "block_timesteps": args.block, "synapses": n_syn,
                       "schedule": net.schedule(), "l2": "synapse entries 225 MB > 129 MB L2 (no flush)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "sim_s_per_wall_s": sim_s * world / (elapsed * world) if world else None,
            "status": status,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": "spk::step_kernel", "launches": launches,
                         "alg_bytes_per_launch": per_launch_bytes, "ms_per_launch": 1000 * per_launch_s},
            "e2e": e2e, "cpu_baseline": cpu, "clocks": clk.summary(),
            "gpu_launches": launches + args.steps,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
