#!/usr/bin/env python
"""Benchmark: LJ MD timesteps/s at N = 1,048,576 (64^3 FCC, density 0.84, r_cut 2.5, buffer 0.4,
dt 0.005), one JSON line on stdout.

A "step" is one MD timestep of the whole system. The state lives in HBM; the timed region is
K timesteps bracketed by a barrier and torch.cuda.synchronize(), timed with CUDA events on the
engine's own stream. Warm-up runs W Bussi (kT = 1.5) equilibration steps from a thermalised
lattice; the K timed steps are NVE (ConstantVolume without thermostat) with the Hilbert-curve
particle sort every 100 steps, as the 1M-particle configuration prescribes.

Other configurations (``--workload``): ``lj_sc_4096`` (the 4096-particle LJ fluid, Bussi
kT = 1.5), ``ka_262k`` (Kob-Andersen 80:20 mixture, N = 262,144, density 1.2, Bussi kT = 0.8,
dt 0.003, buffer 0.3, started from a jittered lattice instead of random positions plus capped
relaxation), ``table32_524k`` (32 types, 528 tabulated pair potentials, N = 524,288, density
0.8, Bussi kT = 1.5, dt 0.004, buffer 0.4). Those configurations keep their thermostat in the
timed steps. ``replicas_256``: 256 independent LJ systems (N ~ U[500, 20000], density ~
U[0.7, 0.9], Bussi kT ~ U[0.8, 2.0], dt 0.005) advanced by one persistent launch per run, with the
launch shape chosen by the ensemble's tuner during warm-up; reported in particle-timesteps/s.

With no flags (the 1M-particle workload on one GPU) the line also carries, under "workloads",
the JSON line of each other configuration (ka_262k, table32_524k, replicas_256,
table32_mlp_524k), each run as its own process of this script with the same --steps/--warmup
(``--no-secondary`` skips them).

--impl reference times the CPU restatement of the reference's path (oracle/, FP64 Scalar, full
neighbour list over all host threads) on a bounded sample of the same workload, after the same
warm-up sequence; its inputs come from the same numpy-only generators (synthetic_systems), and it
loads neither torch nor this package's compiled code.
Multi-GPU: the path is run as independent replicas, one per GPU (no collective on the data path);
``--gpus N`` without a launcher relaunches itself under torch.distributed.run with N processes.
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

UNIT = "timesteps/s"


# ------------------------------------------------------------------------------------------------
# workloads
# ------------------------------------------------------------------------------------------------
def _lj_forces(md, cell, types, pairs, r_cut):
    lj = md.pair.LJ(nlist=cell, default_r_cut=r_cut)
    for (a, b), (eps, sig, rc) in pairs.items():
        lj.params[(a, b)] = dict(epsilon=eps, sigma=sig)
        lj.r_cut[(a, b)] = rc
    return lj


class Workload:
    """One benchmark configuration: its snapshot, pair force, thermostat and oracle inputs."""

    def __init__(self, name, metric, config, make_snap, kind, pairs=None, tables=None,
                 timed_thermostat=False):
        self.name, self.metric, self.config = name, metric, config
        self.make_snap, self.kind = make_snap, kind
        self.pairs, self.tables = pairs, tables
        self.timed_thermostat = timed_thermostat

    def force(self, md, cell, snap):
        types = snap.particles.types
        if self.kind == "lj":
            return _lj_forces(md, cell, types, self.pairs, self.config["r_cut"])
        tab = md.pair.Table(nlist=cell, default_r_cut=self.config["r_cut"])
        for (i, j), v in self.tables().items():
            tab.params[(types[i], types[j])] = dict(r_min=v["r_min"], U=v["U"], F=v["F"])
        return tab

    def oracle_inputs(self, snap):
        """(kind, params, tdata, r_cut matrix) in the oracle's formats."""
        import numpy as np
        types = snap.particles.types
        nt = len(types)
        rc = np.zeros((nt, nt))
        if self.kind == "lj":
            par = np.zeros((nt * nt, 2))
            for (a, b), (eps, sig, r) in self.pairs.items():
                i, j = types.index(a), types.index(b)
                for x, y in ((i, j), (j, i)):
                    par[x * nt + y] = (sig, eps)
                    rc[x, y] = r
            return "lj", par, None, rc
        tabs = self.tables()
        par = np.zeros((nt * nt, 3))
        data, offs, off = [], {}, 0
        for (i, j), v in sorted(tabs.items()):
            offs[(i, j)] = off
            data += [v["U"], v["F"]]
            off += 2 * len(v["U"])
        for i in range(nt):
            for j in range(nt):
                a, b = min(i, j), max(i, j)
                par[i * nt + j] = (tabs[(a, b)]["r_min"], len(tabs[(a, b)]["U"]), offs[(a, b)])
                rc[i, j] = self.config["r_cut"]
        return "table", par, np.concatenate(data), rc


def workloads_registry(fcc_m=64):
    import synthetic_systems as W  # numpy only: both arms build their inputs from it
    N_fcc = 4 * fcc_m ** 3
    reg = {}
    reg["lj_fcc_1m"] = Workload(
        "lj_fcc_1m", "LJ MD timesteps/s at N=1M",
        {"workload": "lj_fluid_fcc_1M" if fcc_m == 64 else f"lj_fluid_fcc_{N_fcc}", "N": N_fcc,
         "lattice": f"fcc {fcc_m}^3", "density": 0.84, "r_cut": 2.5, "buffer": 0.4, "dt": 0.005,
         "kT": 1.5, "integrator": "ConstantVolume NVE after Bussi kT=1.5 warm-up",
         "sort_period": 100, "precision": "fp32 positions/forces, fp64 reductions",
         "l2": "working set > L2 (neighbour list ~0.35 GB read per step)"},
        lambda seed: W.lj_fluid_fcc(m=fcc_m, density=0.84, jitter=0.05, seed=seed), "lj",
        pairs={("A", "A"): (1.0, 1.0, 2.5)})
    reg["lj_sc_4096"] = Workload(
        "lj_sc_4096", "LJ MD timesteps/s at N=4096",
        {"workload": "lj_fluid_sc_4096", "N": 4096, "lattice": "sc 16^3", "density": 0.84,
         "r_cut": 2.5, "buffer": 0.4, "dt": 0.005, "kT": 1.5,
         "integrator": "ConstantVolume + Bussi kT=1.5", "sort_period": 0,
         "precision": "fp32 positions/forces, fp64 reductions", "l2": "fits in L2"},
        lambda seed: W.lj_fluid_sc(16, density=0.84, jitter=0.05, seed=seed), "lj",
        pairs={("A", "A"): (1.0, 1.0, 2.5)}, timed_thermostat=True)
    reg["ka_262k"] = Workload(
        "ka_262k", "Kob-Andersen LJ timesteps/s at N=262144",
        {"workload": "kob_andersen_262k", "N": 262144, "lattice": "jittered sc 64^3, 80:20 A:B",
         "density": 1.2, "r_cut": 2.5, "buffer": 0.3, "dt": 0.003, "kT": 0.8,
         "integrator": "ConstantVolume + Bussi kT=0.8", "sort_period": 100,
         "precision": "fp32 positions/forces, fp64 reductions", "l2": "working set > L2"},
        lambda seed: W.binary_mixture(N=262144, density=1.2, seed=seed), "lj",
        pairs={("A", "A"): (1.0, 1.0, 2.5), ("A", "B"): (1.5, 0.8, 2.0),
               ("B", "B"): (0.5, 0.88, 2.2)}, timed_thermostat=True)
    reg["table32_524k"] = Workload(
        "table32_524k", "32-type Table timesteps/s at N=524288",
        {"workload": "table_32types_524k", "N": 524288, "types": 32, "table_pairs": 528,
         "table_width": 1000, "density": 0.8, "r_min": 0.8, "r_cut": 3.0, "buffer": 0.4,
         "dt": 0.004, "kT": 1.5, "integrator": "ConstantVolume + Bussi kT=1.5",
         "sort_period": 100, "precision": "fp32 positions/forces/tables, fp64 reductions",
         "l2": "working set > L2; tables (4.2 MB) L2-resident"},
        lambda seed: W.multitype_system(N=524288, ntypes=32, density=0.8, seed=seed), "table",
        tables=lambda: W.mixture_tables(32, r_min=0.8, r_cut=3.0, width=1000, seed=2),
        timed_thermostat=True)
    return reg


# ------------------------------------------------------------------------------------------------
# harness
# ------------------------------------------------------------------------------------------------
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
    """Rank, world size and local rank from the launcher's environment; for N > 1 the process
    group (NCCL on GPUs, gloo where CUDA is absent). The ranks exchange only the barrier and the
    largest elapsed time: each runs its own independent system."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
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
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_sim(wl, snap, seed=1):
    import hoomd_gb300 as hoomd
    from hoomd_gb300 import md
    c = wl.config
    from hoomd_gb300.workloads import to_snapshot
    sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=seed)
    sim.create_state_from_snapshot(to_snapshot(snap))
    sim.state.thermalize_particle_momenta(hoomd.filter.All(), c["kT"])
    cell = md.nlist.Cell(buffer=c["buffer"])
    force = wl.force(md, cell, snap)
    method = md.methods.ConstantVolume(hoomd.filter.All(),
                                       md.methods.thermostats.Bussi(kT=c["kT"]))
    sim.operations.integrator = md.Integrator(dt=c["dt"], forces=[force], methods=[method])
    if c.get("sort_period"):
        sim.operations.tuners.append(hoomd.tune.ParticleSorter(trigger=c["sort_period"],
                                                               grid=c.get("sort_grid")))
    return sim, force, cell, method


def traffic_per_launch(wl):
    """DRAM bytes (read + write) per launch of the fused pair kernel from the committed ncu
    summary of this workload, when one exists."""
    p = REPO / "profiles" / "pair_step_lj_traffic.json"
    if wl.name == "lj_fcc_1m" and wl.config["N"] == 1048576 and p.exists():
        d = json.loads(p.read_text())
        return d.get("dram_bytes_per_launch_scaled_to_1M")
    return None


def oracle_sim(wl, snap, full, nthreads, bussi=None):
    """The oracle's whole-step runner on the workload's system, velocities thermalised at the
    workload's kT; Bussi at that kT when ``bussi`` (default: the timed steps' thermostat)."""
    import numpy as np
    from oracle import oracle as O
    p = snap.particles
    N = p.N
    kind, par, tdata, rc = wl.oracle_inputs(snap)
    pos4 = O.make_pos4(p.position, p.typeid, 64)
    vel4 = np.zeros((N, 4))
    vel4[:, 3] = 1.0
    vel4 = O.thermalize(vel4, np.arange(N), wl.config["kT"], 0, 1, prec=64)
    return O.Sim(pos4, vel4, np.zeros((N, 3), np.int32), np.arange(N), snap.configuration.box,
                 rc, wl.config["buffer"], wl.config["dt"], kind=kind, params=par, tdata=tdata,
                 full=full, prec=64, nthreads=nthreads,
                 bussi=wl.timed_thermostat if bussi is None else bussi,
                 kT=wl.config["kT"], seed=1)


def cpu_baseline_sample(wl, snap, max_seconds=20.0):
    """The oracle (single thread, FP64 Scalar, half list + third law: the reference's CPU path)
    on the same system: one untimed step, then as many timed steps as fit in ~max_seconds."""
    sim = oracle_sim(wl, snap, full=False, nthreads=1)
    t0 = time.perf_counter()
    sim.run(1)
    per = max(1e-3, time.perf_counter() - t0)
    n = max(2, int(max_seconds / per))
    t0 = time.perf_counter()
    sim.run(n)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n} timesteps of the {snap.particles.N}-particle {wl.name} system after "
                      f"one untimed step; oracle FP64, half list, single thread"}


def run_gb300(args):
    import torch

    wl = workloads_registry(args.fcc_m)[args.workload]
    if args.sort_grid:
        wl.config["sort_grid"] = args.sort_grid
    rank, world, local = dist_init()
    torch.cuda.set_device(local)
    snap = wl.make_snap(1 + rank)
    N = snap.particles.N
    # clocks sampled from before the warm-up to after the end-to-end run: at 200 ms a sample
    # the timed region alone (a few ms at K = 20) may fall between two samples
    clocks = ClockSampler(local) if rank == 0 else None
    sim, force, cell, method = make_sim(wl, snap, seed=1 + rank)
    sim.run(max(3, args.warmup))  # warm-up / equilibration (Bussi)
    if not wl.timed_thermostat:
        method.thermostat = None  # NVE for the timed steps
        sim._needs_prep = True
    # the reference tunes its kernels' launch parameters during its first steps
    # (hoomd/Autotuner.h); here the search runs once, on the warmed-up state, before the timing
    if not args.no_kernel_search:
        sim.operations.tune_kernel_parameters()
    sim.run(3)
    kernel_parameters = {**force.kernel_parameters, **cell.kernel_parameters}
    integ = sim._cpp_integrator
    stream = torch.cuda.ExternalStream(integ.streamHandle())
    sum_n = integ.sumNNeigh()
    phases = integ.timePhases(20)  # [step one, rebuild, fused pair step] ms
    launches0 = integ.launch_count
    rollbacks0 = integ.n_rollbacks

    barrier(world)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    sim.run(args.steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms = ev0.elapsed_time(ev1)
    ms_max = max_over_ranks(ms, world)
    launches = integ.launch_count - launches0
    builds = cell.num_builds  # the builds of this run (the reference's num_builds)
    rollbacks = integ.n_rollbacks - rollbacks0
    tps = args.steps / (ms_max / 1e3)

    # end to end through the public API: host snapshot in (H2D), K steps, snapshot and
    # energy out (D2H), wall clock; the median of three such round trips
    snap_now = sim.state.get_snapshot()
    trials = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.state.set_snapshot(snap_now)
        sim.run(args.steps)
        out = sim.state.get_snapshot()
        e_pot = force.energy
        trials.append(time.perf_counter() - t0)
        del out, e_pot
    t_e2e = statistics.median(trials)
    # snapshot arrays as copied: positions, velocities (FP64 x3), mass (FP64), type ids, images
    h2d = N * (24 + 24 + 8 + 4 + 12)
    d2h = N * (24 + 24 + 8 + 4 + 12) + 8  # the same arrays back, and the FP64 energy sum
    e2e = {"value": args.steps / t_e2e, "unit": UNIT,
           "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
           "trials_s": [round(t, 6) for t in trials],
           "note": "host snapshot -> set_snapshot -> run(K) -> get_snapshot + energy, wall "
                   "clock, median of 3"}
    clk = clocks.stop() if clocks else None
    if clk:
        clk["window"] = "warm-up, timed region and end-to-end run"

    peak, peak_kind = peaks()
    t_pair = phases[2] / 1e3
    bytes_pair = N * (16 + 4 + 16 + 16 + 16 + 12) + 4.0 * sum_n
    achieved = bytes_pair / t_pair / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic_per_launch(wl),
                "kernel": "k_pair_i4 (gb_md_pair_step_*: pair forces + step two + fp64 thermo)",
                "algorithmic_bytes_per_launch": bytes_pair,
                "bytes_formula": "N*(16 pos + 4 n_neigh + 16 force + 16+16 vel r/w + 12 accel) "
                                 "+ 4*sum(n_neigh)",
                "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind ==
                "measured" else "fallback 6.8 TB/s",
                "kernel_ms": phases[2], "step_one_ms": phases[0], "rebuild_ms": phases[1]}
    # the pair and neighbour-list kernels together over a step, the build amortised over the
    # steps between builds of the timed run: N*(16 pos + 16 + 16 xyzf + 4 n_neigh + 16 last_pos)
    # + 4*sum(n_neigh) bytes per build
    per_build = builds / args.steps if builds else 0.0
    bytes_nl = N * (16 + 16 + 16 + 4 + 16) + 4.0 * sum_n
    t_pn = t_pair + per_build * phases[1] / 1e3
    achieved_pn = (bytes_pair + per_build * bytes_nl) / t_pn / 1e9
    roofline["pair_nlist"] = {"achieved": achieved_pn, "frac": achieved_pn / peak,
                              "builds_per_step": per_build, "nlist_bytes_per_build": bytes_nl}
    # the build alone (cell list + neighbour list, one forced build of timePhases)
    achieved_nl = bytes_nl / (phases[1] / 1e3) / 1e9
    roofline["nlist_build"] = {"achieved": achieved_nl, "frac": achieved_nl / peak,
                               "bound": "issue (exact-rounding candidate tests)"}

    line = {"metric": wl.metric, "value": tps * world, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded lattice, jittered, thermalised)",
            "config": dict(wl.config),
            "parallelism": f"independent replicas x{world}" if world > 1 else "1 GPU",
            "pair_evals_per_s": sum_n * tps * world, "nlist_builds": builds,
            "nlist_rollbacks": rollbacks, "kernel_parameters": kernel_parameters,
            "e2e": e2e, "roofline": roofline, "gpu_launches": int(launches), "clocks": clk}
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline_sample(wl, snap, args.cpu_seconds)
        if want_secondary(args, world):
            del sim, force, cell, method
            torch.cuda.empty_cache()
            line["workloads"] = secondary_workloads(args, "gb300")
        print(json.dumps(line), flush=True)


def peak_bf16():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("bf16_tflops_sustained") or d.get("bf16_tflops")), "measured sustained"
    return 1700.0, "fallback sustained"


def run_mlp(args):
    """The 32-type Table system (N = 524,288) with the plain Table force and with the radial MLP
    surrogate trained on pairs from the plain-Table NVT run: timesteps/s of both, force RMSE."""
    import numpy as np
    import torch
    import hoomd_gb300 as hoomd
    from hoomd_gb300 import md
    from hoomd_gb300.surrogate import Surrogate
    rank, world, local = dist_init()
    torch.cuda.set_device(local)
    wl = workloads_registry()["table32_524k"]
    c = wl.config
    snap = wl.make_snap(1 + rank)
    types = snap.particles.types
    tabs = wl.tables()
    params = {(types[i], types[j]): dict(r_min=v["r_min"], U=v["U"], F=v["F"])
              for (i, j), v in tabs.items()}

    from hoomd_gb300.workloads import to_snapshot

    def make(force_fn, snapshot, thermalize):
        sim = hoomd.Simulation(device=hoomd.device.GPU(), seed=1 + rank)
        sim.create_state_from_snapshot(to_snapshot(snapshot))
        if thermalize:
            sim.state.thermalize_particle_momenta(hoomd.filter.All(), c["kT"])
        cell = md.nlist.Cell(buffer=c["buffer"])
        f = force_fn(cell)
        sim.operations.integrator = md.Integrator(dt=c["dt"], forces=[f], methods=[
            md.methods.ConstantVolume(hoomd.filter.All(),
                                      md.methods.thermostats.Bussi(kT=c["kT"]))])
        sim.operations.tuners.append(hoomd.tune.ParticleSorter(trigger=c["sort_period"]))
        return sim, f, cell

    def table_force(cell):
        t = md.pair.Table(nlist=cell, default_r_cut=c["r_cut"])
        for k, v in params.items():
            t.params[k] = v
        return t

    def timed(sim, steps):
        integ = sim._cpp_integrator
        stream = torch.cuda.ExternalStream(integ.streamHandle())
        launches0 = integ.launch_count
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        sim.run(steps)
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1), integ.launch_count - launches0

    # plain Table: equilibrate, collect training frames, time
    sim_t, tab, cell_t = make(table_force, snap, True)
    sim_t.run(max(3, args.warmup))
    box = np.array(snap.configuration.box[:3])
    frames = []
    for _ in range(args.mlp_frames):
        sim_t.run(100)
        st = sim_t.state.get_snapshot()
        frames.append((st.particles.position.copy(), st.particles.typeid.copy(), box))
    clocks = ClockSampler(local) if rank == 0 else None
    ms_t, launches_t = timed(sim_t, args.steps)
    clk = clocks.stop() if clocks else None
    phases_t = sim_t._cpp_integrator.timePhases(10)

    # surrogate: sample pairs from the frames, train with the GPU kernels
    t0 = time.perf_counter()
    sur = Surrogate.from_table(params, types, c["r_min"], c["r_cut"], seed=7)
    sur._cpp.act_split = args.mlp_act_split
    samples = sur.sample_pairs(frames, anchors=args.mlp_anchors)
    t_sample = time.perf_counter() - t0
    losses = sur.fit(samples, steps=args.mlp_train_steps, batch=8192, report=1000)
    t_train = sur._cpp.train_ms / 1e3

    # accuracy on the state the timed Table run ended in
    snap_eval = sim_t.state.get_snapshot()
    tab._cpp_obj.compute(False)
    F_table = tab.forces
    sim_m, sf, cell_m = make(lambda cell: md.pair.TableSurrogate(nlist=cell, surrogate=sur),
                             snap_eval, False)
    sim_m.run(0)
    F_mlp = sf.forces
    rmse = float(np.sqrt(np.mean((F_mlp - F_table) ** 2)))
    frms = float(np.sqrt(np.mean(F_table ** 2)))
    sim_m.run(max(3, args.warmup // 4))
    clocks = ClockSampler(local) if rank == 0 else None
    ms_m, launches_m = timed(sim_m, args.steps)
    clk_m = clocks.stop() if clocks else None
    phases_m = sim_m._cpp_integrator.timePhases(10)
    # the same run on the legacy warp-level mma.sync path, for comparison
    sur._cpp.tensor_kernel = "mma.sync"
    ms_ms, _ = timed(sim_m, args.steps)
    phases_ms = sim_m._cpp_integrator.timePhases(10)
    sur._cpp.tensor_kernel = "tcgen05"
    tps_t = args.steps / (ms_t / 1e3)
    tps_m = args.steps / (ms_m / 1e3)
    # tensor-pipe roofline of the surrogate force: FLOPs of the per-pair products
    # (2 x (32x64 + 64x64) multiply-adds for value and derivative) per evaluated pair
    sum_n = sim_m._cpp_integrator.sumNNeigh()
    N = snap.particles.N
    R = sur.r_cut
    pairs_in_cut = 0.5 * N * c["density"] * 4.0 / 3.0 * np.pi * (R ** 3 - sur.r_min ** 3)
    flops_pair = 2.0 * 2.0 * (32 * 64 + 64 * 64)
    peak, pk = peak_bf16()
    t_force = phases_m[2] / 1e3
    achieved = flops_pair * pairs_in_cut / t_force / 1e12
    line = {"metric": "MLP-surrogate vs plain Table TPS at <=1e-3 force err (32 types, N=524288)",
            "value": tps_m, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_m / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 tensor / fp32",
            "data": "synthetic (seeded 32-type tables, random types, jittered lattice)",
            "config": dict(c, workload="table32_mlp_524k", mlp="16 emb + 32 RBF -> 64 -> 64 SiLU"
                           " -> 1, force = -dU/dr", act_split=sur._cpp.act_split,
                           train_steps=args.mlp_train_steps, train_batch=8192,
                           train_samples=int(len(samples["r"])), train_frames=args.mlp_frames),
            "table_tps": tps_t, "mlp_over_table": tps_m / tps_t,
            "tensor_kernel": "tcgen05 (128-pair tiles, TMEM accumulators)",
            "mma_sync_tps": args.steps / (ms_ms / 1e3),
            "force_rmse": rmse, "force_rms": frms, "force_rmse_target": 1e-3,
            "force_rmse_ref": "GPU Table path (FP32; within 1e-5 of the FP64 oracle)",
            "train_s": t_train, "sample_s": t_sample, "train_loss": losses[-3:],
            "phases_ms": {"table": dict(zip(["step_one", "rebuild", "pair_step"], phases_t)),
                          "mlp": dict(zip(["step_one", "rebuild", "force+step_two"], phases_m)),
                          "mlp_mma_sync": dict(zip(["step_one", "rebuild", "force+step_two"],
                                                   phases_ms))},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                         "kernel": "k_mlp_forces_tc (+ pair list, step two, thermo)",
                         "flops_formula": "pairs in [r_min, r_cut) (0.5 N rho 4/3 pi (rc^3 - "
                                          "rmin^3)) x 2 x 2 x (32x64 + 64x64)",
                         "peak_kind": pk},
            "gpu_launches": int(launches_m), "clocks": clk_m, "clocks_table": clk}
    if rank == 0:
        print(json.dumps(line), flush=True)


def replica_systems(count=256):
    import synthetic_systems as W  # numpy only: both arms build their inputs from it
    return W.replica_systems(count=count, n_min=500, n_max=20000, seed=4)


REPLICA_CONFIG = {"workload": "lj_replicas_256", "replicas": 256, "N_range": [500, 20000],
                  "density_range": [0.7, 0.9], "kT_range": [0.8, 2.0], "r_cut": 2.5,
                  "buffer": 0.4, "dt": 0.005, "integrator": "ConstantVolume + Bussi per replica",
                  "launch": "one persistent kernel per run, CUDA graph",
                  "precision": "fp32 positions/forces, fp64 reductions",
                  "l2": "working set > L2 (neighbour lists ~1.4 GB)"}
REPLICA_UNIT = "particle-timesteps/s"


def run_replicas(args):
    """256 uneven LJ replicas advanced together (one persistent launch per run)."""
    import torch
    import hoomd_gb300 as hoomd
    import numpy as np
    from hoomd_gb300.workloads import to_snapshot
    rank, world, local = dist_init()
    torch.cuda.set_device(local)
    systems = [(to_snapshot(h), kT, sd) for h, kT, sd in replica_systems(args.replicas)]

    def build():
        ens = hoomd.ReplicaEnsemble(dt=0.005, r_cut=2.5, buffer=0.4)
        for snap, kT, seed in systems:
            ens.add_replica(snap, kT=kT, seed=seed + 1000 * rank)
        return ens

    clocks = ClockSampler(local) if rank == 0 else None  # warm-up to end-to-end run
    ens = build()
    Ntot = ens.total_particles
    ens.run(0)
    if args.no_tune:
        ens.set_launch(1024, 0)
        tune = [dict(block_size=1024, grid_size=0, ms_per_step=float("nan"))]
    else:
        tune = ens.autotune(steps=10, repeats=1)
    ens.run(max(3, args.warmup))
    stream = torch.cuda.ExternalStream(ens._cpp.streamHandle())
    sum_n = sum(int(np.sum(ens._cpp.neighborCounts(r))) for r in range(ens.count))
    builds0 = sum(ens.thermo(r)["n_builds"] for r in range(ens.count))
    launches0 = ens.launch_count
    cyc0 = np.asarray(ens._cpp.phaseClocks(), np.float64).reshape(-1, 4)
    barrier(world)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    ens.run(args.steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms = max_over_ranks(ev0.elapsed_time(ev1), world)
    builds = sum(ens.thermo(r)["n_builds"] for r in range(ens.count)) - builds0
    cyc = np.asarray(ens._cpp.phaseClocks(), np.float64).reshape(-1, 4) - cyc0
    big = int(np.argmax([ens.record(r)["N"] for r in range(ens.count)]))
    launches = ens.launch_count - launches0
    value = Ntot * args.steps / (ms / 1e3) * world

    # end to end through the public API: build the ensemble from host snapshots (H2D), run K
    # steps, read every replica's snapshot and energies back (D2H), wall clock
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2 = build()
    e2.run(args.steps)
    out = [e2.get_snapshot(r) for r in range(e2.count)]
    th = [e2.thermo(r) for r in range(e2.count)]
    t_e2e = time.perf_counter() - t0
    del out, th, e2
    clk = clocks.stop() if clocks else None
    if clk:
        clk["window"] = "autotune, warm-up, timed region and end-to-end run"
    mhz = (clk or {}).get("sm_mhz") or 2070.0
    phase_names = ["step_one", "nlist_build", "pair_step", "bussi_draws"]
    phase_split = {
        "all_replicas_fraction": dict(zip(phase_names, (cyc.sum(0) / cyc.sum()).round(4).tolist())),
        "largest_replica": {"N": ens.record(big)["N"], "us_per_step": dict(zip(
            phase_names, (cyc[big] / mhz / args.steps).round(2).tolist()))},
        "sm_cycles_total": float(cyc.sum()), "note": "clock64 at phase boundaries, thread 0"}
    e2e = {"value": Ntot * args.steps / t_e2e, "unit": REPLICA_UNIT,
           "h2d_bytes_per_step": Ntot * (16 + 16 + 16) / args.steps,
           "d2h_bytes_per_step": (Ntot * (16 + 16 + 16 + 16) + 256 * 240) / args.steps,
           "note": "256 host snapshots -> ReplicaEnsemble -> run(K) (prep included) -> "
                   "get_snapshot + thermo of every replica, wall clock"}

    peak, peak_kind = peaks()
    # per particle and step: step one (pos, vel, accel, last_pos read; pos, vel write) + pair
    # step (n_neigh, own pos, vel r/w, force and accel write) + 4 bytes per neighbour index
    bytes_step = Ntot * (96 + 84) + 4.0 * sum_n
    achieved = bytes_step * args.steps / (ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": None,
                "kernel": "k_replicas (gb_replicas_run: every step of every replica)",
                "algorithmic_bytes_per_step": bytes_step,
                "bytes_formula": "Ntot*(96 step one + 84 pair step) + 4*sum(n_neigh); "
                                 "neighbour-list builds not counted",
                "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"}
    best = min(tune, key=lambda t: t["ms_per_step"])
    line = {"metric": "LJ replica ensemble particle-timesteps/s (256 replicas, N 500-20000)",
            "value": value, "unit": REPLICA_UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded sizes, densities, kT; jittered lattices, MB velocities)",
            "config": dict(REPLICA_CONFIG, replicas=len(systems)),
            "total_particles": Ntot, "launch_shape": ens.launch, "tuned_from": len(tune),
            "parallelism": f"independent replicas x{world}" if world > 1 else "1 GPU",
            "timesteps_per_s": args.steps / (ms / 1e3), "pair_evals_per_s":
            sum_n * args.steps / (ms / 1e3) * world, "nlist_builds": builds,
            "autotune_best": best, "phases": phase_split, "e2e": e2e, "roofline": roofline,
            "gpu_launches": int(launches), "clocks": clk}
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = replica_cpu_sample(systems, args.cpu_seconds, 1)
        print(json.dumps(line), flush=True)


def replica_cpu_sample(systems, seconds, nthreads, warm=1):
    """The oracle on a sample of the replicas, one after another (as separate reference runs
    would be): steps until about ``seconds`` have passed, in particle-timesteps/s."""
    import numpy as np
    from oracle import oracle as O
    done, t_tot, k, names = 0, 0.0, 0, []
    for snap, kT, seed in systems[::17]:
        N = snap.particles.N
        pos4 = O.make_pos4(snap.particles.position, np.zeros(N), 64)
        vel4 = np.ones((N, 4))
        vel4[:, :3] = snap.particles.velocity
        sim = O.Sim(pos4, vel4, np.zeros((N, 3), np.int32), np.arange(N),
                    snap.configuration.box, [[2.5]], 0.4, 0.005, params=[[1.0, 1.0]],
                    full=nthreads > 1, prec=64, nthreads=nthreads, bussi=True, kT=kT, seed=seed)
        sim.run(warm)
        t0 = time.perf_counter()
        sim.run(10)
        t_tot += time.perf_counter() - t0
        done += 10 * N
        k += 1
        names.append(N)
        if t_tot > seconds:
            break
    return {"value": done / t_tot, "unit": REPLICA_UNIT, "cores": nthreads, "kind": "port",
            "sample": f"10 timesteps of each of {k} replicas (N = {names}) one after another, "
                      f"after {warm} untimed steps; oracle FP64, "
                      + ("half list, single thread" if nthreads == 1 else
                         f"full list, {nthreads} OpenMP threads")}


SECONDARY = ("ka_262k", "table32_524k", "replicas_256", "table32_mlp_524k")


def want_secondary(args, world):
    return (world == 1 and not args.no_secondary and args.workload == "lj_fcc_1m"
            and args.fcc_m == 64)


def secondary_workloads(args, impl):
    """The other benchmark configurations, each as its own process of this script (fresh device
    state) with the same --steps/--warmup; their JSON lines are kept under the headline line's
    "workloads" key. The surrogate has no counterpart in the reference's CPU path."""
    out = {}
    for w in SECONDARY:
        if impl == "reference" and w == "table32_mlp_524k":
            continue
        cmd = [sys.executable, str(REPO / "bench.py"), "--impl", impl, "--workload", w,
               "--steps", str(args.steps), "--warmup", str(args.warmup),
               "--cpu-seconds", str(args.secondary_cpu_seconds), "--no-secondary"]
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=1500)
            lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
            out[w] = json.loads(lines[-1]) if r.returncode == 0 and lines else {
                "error": f"rc={r.returncode}", "tail": (r.stdout + r.stderr)[-600:]}
        except subprocess.TimeoutExpired:
            out[w] = {"error": "timed out after 1500 s"}
    return out


def run_reference(args):
    """The CPU restatement of the reference's path over all host threads (FP64, full list)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload == "replicas_256":
        cores = os.cpu_count() or 1
        warm = max(3, args.warmup)
        cb = replica_cpu_sample(replica_systems(), args.cpu_seconds * 3, cores, warm=warm)
        v = cb["value"]
        print(json.dumps({
            "metric": "LJ replica ensemble particle-timesteps/s (256 replicas, N 500-20000)",
            "value": v, "unit": REPLICA_UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": warm, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
            "data": "synthetic (seeded sizes, densities, kT; jittered lattices, MB velocities)",
            "config": REPLICA_CONFIG, "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": REPLICA_UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}), flush=True)
        return
    wl = workloads_registry(args.fcc_m)[args.workload]
    cores = os.cpu_count() or 1
    snap = wl.make_snap(1)
    # the same sequence as the GPU arm: W Bussi warm-up steps from the thermalised lattice, then
    # (for the 1M-particle NVE workload) the thermostat removed and 3 settling steps
    sim = oracle_sim(wl, snap, full=True, nthreads=cores, bussi=True)
    warm = max(3, args.warmup)
    sim.run(warm)
    if not wl.timed_thermostat:
        sim.set_thermostat(None)
    sim.run(3)
    t0 = time.perf_counter()
    sim.run(1)
    per = time.perf_counter() - t0
    n = max(2, min(args.steps, int(args.cpu_seconds * 3 / max(per, 1e-3))))
    t0 = time.perf_counter()
    sim.run(n)
    dt = time.perf_counter() - t0
    v = n / dt
    line = {
        "metric": wl.metric, "value": v, "unit": UNIT, "n_gpus": 0, "steps": n, "warmup": warm,
        "ms_per_step": 1e3 * dt / n, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded lattice, jittered, thermalised)", "config": wl.config,
        "impl": "reference",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{n} of the {args.steps} requested timesteps (bounded to a "
                                   f"few minutes) of the {snap.particles.N}-particle {wl.name} "
                                   f"system after {warm} + 3 untimed steps; oracle FP64, full "
                                   f"list, {cores} OpenMP threads"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    del sim
    if want_secondary(args, int(os.environ.get("WORLD_SIZE", "1"))):
        line["workloads"] = secondary_workloads(args, "reference")
    print(json.dumps(line), flush=True)


def run_drift(args):
    """NVE energy drift of the 1M-particle LJ fluid: the Bussi equilibration of the workload
    (1000 steps at kT 1.5), then ``--drift-steps`` ConstantVolume steps with no thermostat, the
    total energy KE + PE (FP64 reductions) sampled every 500 steps. Prints one JSON line with the
    least-squares slope per particle per unit time and the largest excursion per particle."""
    import numpy as np
    import torch
    import hoomd_gb300 as hoomd
    from hoomd_gb300 import md

    wl = workloads_registry(args.fcc_m)["lj_fcc_1m"]
    torch.cuda.set_device(0)
    snap = wl.make_snap(1)
    N = snap.particles.N
    sim, force, cell, method = make_sim(wl, snap, seed=1)
    force.mode = args.drift_mode
    thermo = md.compute.ThermodynamicQuantities(hoomd.filter.All())
    sim.operations.computes.append(thermo)
    sim.run(1000)
    method.thermostat = None
    sim._needs_prep = True
    sim.run(0)
    every = 500
    t, e = [], []
    for k in range(args.drift_steps // every + 1):
        if k:
            sim.run(every)
        t.append(k * every * wl.config["dt"])
        e.append(thermo.kinetic_energy + thermo.potential_energy)
    t, e = np.array(t), np.array(e)
    slope = np.polyfit(t, e, 1)[0]
    print(json.dumps({
        "metric": "NVE total-energy drift", "workload": wl.config["workload"], "N": N,
        "pair_mode": args.drift_mode,
        "steps": args.drift_steps, "dt": wl.config["dt"], "sample_every": every,
        "E0_per_particle": e[0] / N, "drift_per_particle_per_tau": slope / N,
        "max_excursion_per_particle": float(np.abs(e - e[0]).max() / N),
        "relative_change": float((e[-1] - e[0]) / abs(e[0])),
        "kinetic_temperature_end": thermo.kinetic_temperature,
        "precision": "fp32 positions/forces, fp64 reductions",
        "energies": [float(x) for x in e]}), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=200)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", default="lj_fcc_1m",
                    choices=["lj_fcc_1m", "lj_sc_4096", "ka_262k", "table32_524k",
                             "replicas_256", "table32_mlp_524k"])
    ap.add_argument("--mlp-train-steps", type=int, default=20000)
    ap.add_argument("--mlp-frames", type=int, default=3)
    ap.add_argument("--mlp-anchors", type=int, default=20000)
    ap.add_argument("--replicas", type=int, default=256,
                    help="replica count of replicas_256 (256 = the benchmark; fewer for profiling)")
    ap.add_argument("--no-kernel-search", action="store_true",
                    help="keep the default kernel parameters (profiling captures: the launch "
                         "sequence then has no search launches)")
    ap.add_argument("--no-tune", action="store_true",
                    help="replicas_256: fixed 1024-thread launch instead of the tuner (profiling)")
    ap.add_argument("--mlp-act-split", type=int, default=1, choices=[0, 1],
                    help="activations as one bfloat16 (0) or the sum of two (1)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="lj_fcc_1m at one GPU: skip the other workloads' lines (by default each "
                         "runs as its own process and is reported under \"workloads\")")
    ap.add_argument("--secondary-cpu-seconds", type=float, default=5.0,
                    help="CPU-baseline sample length of each secondary workload")
    ap.add_argument("--fcc-m", type=int, default=64,
                    help="FCC cells per side of lj_fcc_1m (64 = the 1,048,576-particle workload; "
                         "smaller values are for profiling captures only)")
    ap.add_argument("--sort-grid", type=int, default=0,
                    help="ParticleSorter grid (bins per box side); 0 = the sorter's default, 256")
    ap.add_argument("--nve-drift", action="store_true",
                    help="measure the NVE energy drift of lj_fcc_1m instead of the throughput")
    ap.add_argument("--drift-steps", type=int, default=10000)
    ap.add_argument("--drift-mode", default="none", choices=["none", "shift"],
                    help="LJ energy mode of the drift run (none = the workload's)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: relaunch this command under torch.distributed.run
        import socket
        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
               f"--nproc-per-node={args.gpus}", "--master-addr", "127.0.0.1",
               "--master-port", str(port), str(pathlib.Path(__file__).resolve()), *sys.argv[1:]]
        sys.exit(subprocess.call(cmd))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world != args.gpus:
        sys.exit(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}")
    if args.nve_drift:
        run_drift(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "replicas_256":
        run_replicas(args)
    elif args.workload == "table32_mlp_524k":
        run_mlp(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
