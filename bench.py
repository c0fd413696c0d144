#!/usr/bin/env python
"""Benchmark: LJ MD timesteps/s at N = 1,048,576 (64^3 FCC, density 0.84, r_cut 2.5, buffer 0.4,
dt 0.005), one JSON line on stdout.

A "step" is one MD timestep of the whole system. The state lives in HBM; the timed region is
K timesteps bracketed by a barrier and torch.cuda.synchronize(), timed with CUDA events on the
engine's own stream. Warm-up runs W Bussi (kT = 1.5) equilibration steps from a thermalised
lattice; the K timed steps are NVE (ConstantVolume without thermostat) with the Hilbert-curve
particle sort every 100 steps, as the 1M-particle configuration prescribes.

--impl reference times the CPU restatement of the reference's path (oracle/, FP64 Scalar, full
neighbour list over all host threads) on a bounded sample of the same workload.
Multi-GPU: the path is run as independent replicas, one per GPU (no collective on the data path).
"""

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

REPO = pathlib.Path(__file__).resolve().parent
for _p in (REPO, REPO / "hoomd-blue_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = "LJ MD timesteps/s at N=1M"
UNIT = "timesteps/s"
WORKLOAD = {"workload": "lj_fluid_fcc_1M", "N": 1048576, "lattice": "fcc 64^3",
            "density": 0.84, "r_cut": 2.5, "buffer": 0.4, "dt": 0.005,
            "integrator": "ConstantVolume NVE after Bussi kT=1.5 warm-up",
            "sort_period": 100, "precision": "fp32 positions/forces, fp64 reductions",
            "l2": "working set > L2 (neighbour list ~0.35 GB read per step)"}


def peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        rows = []
        for line in open(self.tmp.name):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.tmp.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        loaded = [x for x in sm if x > 0.5 * max(sm)] if sm else []
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_sim(snap, kT=1.5, seed=1, sort_period=100, thermostat=True):
    import hoomd_gb300 as hoomd
    from hoomd_gb300 import md
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=seed)
    sim.create_state_from_snapshot(snap)
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), kT)
    cell = md.nlist.Cell(buffer=WORKLOAD["buffer"])
    lj = md.pair.LJ(nlist=cell, default_r_cut=WORKLOAD["r_cut"])
    lj.params[("A", "A")] = dict(epsilon=1.0, sigma=1.0)
    method = md.methods.ConstantVolume(
        hoomd.filter.All(), md.methods.thermostats.Bussi(kT=kT) if thermostat else None)
    sim.operations.integrator = md.Integrator(dt=WORKLOAD["dt"], forces=[lj], methods=[method])
    if sort_period:
        sim.operations.tuners.append(hoomd.tune.ParticleSorter(trigger=sort_period))
    return sim, lj, cell, method


def traffic_per_launch():
    """DRAM bytes (read + write) per launch of the fused pair kernel from the committed ncu
    summary, when one exists."""
    p = REPO / "profiles" / "pair_step_lj_traffic.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("dram_bytes_per_launch_scaled_to_1M")
    return None


def cpu_baseline_sample(snap, max_seconds=20.0):
    """The oracle (single thread, FP64 Scalar, half list + third law: the reference's CPU path)
    on the same 1M-particle system: one untimed step, then as many timed steps as fit in
    ~max_seconds (at least 2)."""
    import numpy as np
    from oracle import oracle as O
    p = snap.particles
    N = p.N
    pos4 = O.make_pos4(p.position, p.typeid, 64)
    vel4 = np.zeros((N, 4))
    vel4[:, 3] = 1.0
    vel4 = O.thermalize(vel4, np.arange(N), 1.5, 0, 1, prec=64)
    sim = O.Sim(pos4, vel4, np.zeros((N, 3), np.int32), np.arange(N), snap.configuration.box,
                [[WORKLOAD["r_cut"]]], WORKLOAD["buffer"], WORKLOAD["dt"], params=[[1.0, 1.0]],
                full=False, prec=64, nthreads=1)
    t0 = time.perf_counter()
    sim.run(1)
    t1 = time.perf_counter()
    per = max(1e-3, t1 - t0)
    n = max(2, int(max_seconds / per))
    t0 = time.perf_counter()
    sim.run(n)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n} timesteps of the 1,048,576-particle LJ system after one untimed "
                      f"step; oracle FP64, half list, single thread"}


def run_gb300(args):
    import numpy as np
    import torch

    from hoomd_gb300 import workloads

    rank, world, local = dist_init()
    torch.cuda.set_device(local)
    snap = workloads.lj_fluid_fcc(m=args.fcc_m, density=WORKLOAD["density"], jitter=0.05,
                                  seed=1 + rank)
    N = snap.particles.N
    if args.fcc_m != 64:
        WORKLOAD.update(workload=f"lj_fluid_fcc_{N}", N=N, lattice=f"fcc {args.fcc_m}^3")
    sim, lj, cell, method = make_sim(snap, seed=1 + rank)
    # warm-up / equilibration (Bussi)
    sim.run(max(3, args.warmup))
    method.thermostat = None  # NVE for the timed steps
    sim._needs_prep = True
    sim.run(3)
    integ = sim._cpp_integrator
    stream = torch.cuda.ExternalStream(integ.streamHandle())
    sum_n = integ.sumNNeigh()
    phases = integ.timePhases(20)  # [step one, rebuild, fused pair step] ms
    launches0 = integ.launch_count
    builds0 = cell.num_builds

    clocks = ClockSampler(local) if rank == 0 else None
    barrier(world)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    sim.run(args.steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop() if clocks else None
    ms_max = max_over_ranks(ms, world)
    launches = integ.launch_count - launches0
    builds = cell.num_builds - builds0
    tps = args.steps / (ms_max / 1e3)

    # end to end through the public API: host snapshot in (H2D), K steps, snapshot and
    # energies out (D2H), wall clock
    snap_now = sim.state.get_snapshot()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.state.set_snapshot(snap_now)
    sim.run(args.steps)
    out = sim.state.get_snapshot()
    e_pot = lj.energy
    t_e2e = time.perf_counter() - t0
    h2d = N * (16 + 16 + 12 + 4)  # positions+type, velocities+mass, images, tags (FP32/int)
    d2h = N * (16 + 16 + 12 + 4) + N * 16  # state back + per-particle force/energy for E_pot
    e2e = {"value": args.steps / t_e2e, "unit": UNIT,
           "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
           "note": "host snapshot -> set_snapshot -> run(K) -> get_snapshot + energy, wall clock"}
    del out, e_pot

    peak, peak_kind = peaks()
    t_pair = phases[2] / 1e3
    bytes_pair = N * (16 + 4 + 16 + 16 + 16 + 12) + 4.0 * sum_n
    achieved = bytes_pair / t_pair / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic_per_launch(),
                "kernel": "k_pair<EvalLJ,1,col,single-type,fused step two + fp64 thermo>",
                "algorithmic_bytes_per_launch": bytes_pair,
                "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind ==
                "measured" else "fallback 6.8 TB/s",
                "kernel_ms": phases[2], "step_one_ms": phases[0], "rebuild_ms": phases[1]}

    line = {"metric": METRIC, "value": tps * world, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded FCC lattice, jittered, thermalised)",
            "config": dict(WORKLOAD, parallelism=f"replicas x{world}" if world > 1 else "1 GPU"),
            "pair_evals_per_s": sum_n * tps * world, "nlist_builds": builds,
            "e2e": e2e, "roofline": roofline, "gpu_launches": int(launches), "clocks": clk}
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline_sample(snap, args.cpu_seconds)
        print(json.dumps(line), flush=True)


def run_reference(args):
    """The CPU restatement of the reference's path over all host threads (FP64, full list)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np
    from hoomd_gb300 import workloads
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    snap = workloads.lj_fluid_fcc(m=64, density=WORKLOAD["density"], jitter=0.05, seed=1)
    p = snap.particles
    N = p.N
    pos4 = O.make_pos4(p.position, p.typeid, 64)
    vel4 = np.zeros((N, 4))
    vel4[:, 3] = 1.0
    vel4 = O.thermalize(vel4, np.arange(N), 1.5, 0, 1, prec=64)
    sim = O.Sim(pos4, vel4, np.zeros((N, 3), np.int32), np.arange(N), snap.configuration.box,
                [[WORKLOAD["r_cut"]]], WORKLOAD["buffer"], WORKLOAD["dt"], params=[[1.0, 1.0]],
                full=True, prec=64, nthreads=cores)
    sim.run(max(1, min(args.warmup, 3)))  # includes the first neighbour-list build
    t0 = time.perf_counter()
    sim.run(1)
    per = time.perf_counter() - t0
    n = max(2, min(args.steps, int(args.cpu_seconds * 3 / max(per, 1e-3))))
    t0 = time.perf_counter()
    sim.run(n)
    dt = time.perf_counter() - t0
    v = n / dt
    print(json.dumps({
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": n,
        "warmup": max(1, min(args.warmup, 3)), "ms_per_step": 1e3 * dt / n,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded FCC lattice, jittered, thermalised)", "config": WORKLOAD,
        "impl": "reference",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{n} of the {args.steps} requested timesteps (bounded to a "
                                   f"few minutes) of the 1,048,576-particle LJ system; oracle "
                                   f"FP64, full list, {cores} OpenMP threads"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
        flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=200)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fcc-m", type=int, default=64,
                    help="FCC cells per side (64 = the 1,048,576-particle workload; smaller "
                         "values are for profiling captures only)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
