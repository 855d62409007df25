#!/usr/bin/env python3
"""Benchmark of the explicit step: bond-updates/s on one GB300.

Workload (default): crush512_4m -- config 2 at the node count quoted for it (~4 M nodes): 512
spheres/cubes/ellipsoids of sizes U[0.6, 1.4] mm (seed 2) in a 12 mm box whose top wall moves
down at 1 m/s, lattice spacing h drawn from {0.03, 0.045, 0.06} mm (the stated {0.05, 0.075,
0.1} mm scaled by 0.6; the stated spacings give 0.89 M nodes: workload crush512) and dt =
3e-9 s (below the finest lattice's critical step). One step = predictor, contact broad phase
(rebuilt only when due), fused PD-bond/contact/wall/Verlet kernel, end-of-step kernels,
replayed as a CUDA graph. A bond-update is one live directed bond evaluated in one step.

Printed (one JSON line, rank 0):
  value       FP32-compensated form, device-timed (CUDA events, K steps, inputs resident)
  fp64        the plain FP64 form (bit-exact with the reference's CPU code) on the same setup
  e2e         pd_create_from_arrays from host arrays + K steps + pd_get_state back to host
  roofline    fused step kernel: algorithmic bytes (4.125 B/live bond + 224 B/node) per
              launch / its CUDA-event duration, against MEASURED_PEAKS.json's HBM copy rate
  cpu_baseline  the CPU oracle (restatement of the reference's serial/MPI-round-robin path)
              on a bounded sample (the first 32 particles of the same packing)
  accuracy    FP32-compensated vs FP64 after the same number of steps
--impl reference times that CPU path on the whole workload (same config; whole steps, as many
as fit in --ref-budget seconds), with its setup built on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "bond-updates/s on 1 GB300 (explicit PD step, batched FP32-comp; FP64 plain beside)"
UNIT = "bond-updates/s"
CPU_SAMPLE_PARTICLES = 32


def rank_info():
    r = int(os.environ.get("RANK", "0"))
    w = int(os.environ.get("WORLD_SIZE", "1"))
    lr = int(os.environ.get("LOCAL_RANK", str(r)))
    return r, w, lr


def dist_setup(world, backend):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def _reduce(dist, x: float, op) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(dist, x: float) -> float:
    """Slowest rank's time: the job's time (replicas run independent simulations)."""
    return _reduce(dist, x, dist.ReduceOp.MAX) if dist is not None else x


def sum_over_ranks(dist, x: float) -> float:
    """Bond-updates of all ranks: the whole job's work."""
    return _reduce(dist, x, dist.ReduceOp.SUM) if dist is not None else x


BIG_WORKLOADS = ("crush512_4m", "notched_plate")  # bonds built on the GPU (pd_query_pairs)


def load_workload(name: str, particles: int | None = None):
    """The named workload; `particles`: only its first particles (packings only, bonds on the
    CPU), for the bounded CPU sample."""
    from peridem_gb300 import gen
    fn = gen.WORKLOADS[name]
    if particles is not None and name in ("crush512", "crush512_4m"):
        return fn(count=particles)
    if name in BIG_WORKLOADS:
        gen.set_bond_builder("gpu")
        try:
            return fn()
        finally:
            gen.set_bond_builder("cpu")
    return fn()


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    def __init__(self, gpu: int):
        self.path = Path(tempfile.gettempdir()) / f"pd_clocks_{os.getpid()}.csv"
        self.p = None
        self.gpu = gpu

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            time.sleep(0.25)
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self) -> dict:
        if self.p is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, copy burst)"
        except Exception:
            pass
    return 6800.0, "fallback 6.8 TB/s"


def ncu_traffic(workload: str, precision: str, live: int, nodes: int):
    """Per-launch DRAM bytes of the fused step kernel from a committed ncu summary, scaled
    from the captured case to this launch by bonds and nodes (traffic grows with both)."""
    p = ROOT / "profiles" / "k_step_traffic.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        e = d.get(precision)
        if not e:
            return None
        per = (e["dram_bytes"]) / (4.125 * e["live_bonds"] + 224.0 * e["nodes"])
        return per * (4.125 * live + 224.0 * nodes)
    except Exception:
        return None


def time_device(sim, K: int, W: int, dist, torch):
    # a dedicated (non-default) stream: the kernels and the CUDA events share it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sim.set_stream(stream.cuda_stream)
    if W:
        sim.step(W)
    live0 = sim.live_bonds()
    sim.rebuilds_before = sim.stats()["rebuilds"]
    barrier(dist)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    sim.step(K, sync=False)
    b.record(stream)
    torch.cuda.synchronize()
    barrier(dist)
    sim.sync()
    ms = a.elapsed_time(b)
    live1 = sim.live_bonds()
    sim.rebuilds_timed = sim.stats()["rebuilds"] - sim.rebuilds_before
    return ms, live0, live1


def cpu_sample_rate(s, cfg, threads: int, steps: int, warmup: int, budget_s: float = 20.0):
    """Bond-updates/s of the CPU oracle on the first CPU_SAMPLE_PARTICLES particles."""
    from oracle import oracle as O
    sub = s.subset(list(range(min(CPU_SAMPLE_PARTICLES, s.n_particles))))
    orc = O.Oracle(sub, cfg, threads=threads)
    if warmup:
        orc.step(warmup)
    done = 0
    bonds = 0
    t0 = time.perf_counter()
    while done < steps:
        orc.step(1)
        bonds += orc.counts()["live_bonds"]
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return bonds / dt, done, sub


def compare_forms(a, b, setup, conn_a, conn_b):
    """FP32-compensated state `a` against FP64 state `b` after the same steps."""
    dref = max(np.abs(b["disp"]).max(), 1e-300)
    err = float(np.abs(a["disp"] - b["disp"]).max() / dref)
    mism = 0
    nb = 0
    for ca, cb in zip(conn_a, conn_b):
        nb += len(cb)
        if len(ca) != len(cb) or not np.array_equal(ca, cb):
            mism += len({tuple(x) for x in ca} ^ {tuple(x) for x in cb})
    rho = np.repeat(setup.rho, np.diff(setup.node_offset).astype(np.int64))
    ke_a = 0.5 * float(np.sum(rho * setup.vol * (a["vel"] ** 2).sum(1)))
    ke_b = 0.5 * float(np.sum(rho * setup.vol * (b["vel"] ** 2).sum(1)))
    return {"max_rel_disp_err": err, "broken_bond_mismatch": mism / max(1, nb), "bond_mismatches": mism,
            "live_pairs_fp64": nb, "kinetic_energy_fp64": ke_b,
            "kinetic_energy_rel_diff": abs(ke_a - ke_b) / max(abs(ke_b), 1e-300)}


def accuracy_run(name: str, nsteps: int, eps: float = 1e-7, **over):
    """Both forms of the same workload for `nsteps` steps; the FP64 form is bit-exact with the
    CPU oracle (tests/test_gpu_parity.py), so it stands for the oracle here. A third run, FP64
    from an initial displacement perturbed by eps*h per component (FP32 rounding level), gives
    the FP64 solution's own sensitivity: the floor no reduced-precision form can beat once
    fracture makes the dynamics chaotic."""
    from peridem_gb300 import gen
    from peridem_gb300.sim import Sim
    s, cfg = gen.WORKLOADS[name](**over) if over else load_workload(name)
    a = Sim(s, cfg, "fp32c")
    b = Sim(s, cfg, "fp64")
    c = Sim(s, cfg, "fp64")
    h = float(np.cbrt(np.min(s.vol)))
    rng = np.random.default_rng(12345)
    c.set_state(disp=s.disp + eps * h * rng.uniform(-1.0, 1.0, size=s.disp.shape))
    t0 = time.perf_counter()
    a.step(nsteps)
    t1 = time.perf_counter()
    b.step(nsteps)
    t2 = time.perf_counter()
    c.step(nsteps)
    n0 = s.n_bonds_directed // 2
    cb = [b.connectivity(p) for p in range(s.n_particles)]
    sb = b.state()
    out = compare_forms(a.state(), sb, s, [a.connectivity(p) for p in range(s.n_particles)], cb)
    sens = compare_forms(c.state(), sb, s, [c.connectivity(p) for p in range(s.n_particles)], cb)
    out.update(workload=name, steps=nsteps, nodes=s.n_nodes, initial_pairs=n0,
               broken_pairs_fp64=n0 - out["live_pairs_fp64"], wall_s_fp32c=t1 - t0, wall_s_fp64=t2 - t1,
               fp64_perturbed={"eps_h": eps, "max_rel_disp_err": sens["max_rel_disp_err"],
                               "broken_bond_mismatch": sens["broken_bond_mismatch"],
                               "bond_mismatches": sens["bond_mismatches"],
                               "kinetic_energy_rel_diff": sens["kinetic_energy_rel_diff"]})
    for x in (a, b, c):
        x.close()
    return out


def config_line(name: str, args, dist, torch) -> dict:
    """Bond-updates/s of one more configuration in both forms (autotuned FP32C, plain FP64),
    device-timed like the headline; bonds built on the GPU (pd_query_pairs)."""
    from peridem_gb300 import gen
    from peridem_gb300.sim import Sim
    gen.set_bond_builder("gpu")
    t0 = time.perf_counter()
    try:
        s, cfg = gen.WORKLOADS[name]()
    finally:
        gen.set_bond_builder("cpu")
    t_gen = time.perf_counter() - t0
    out = {"workload": name, "particles": s.n_particles, "nodes": s.n_nodes, "directed_bonds": s.n_bonds_directed,
           "setup_s": t_gen}
    sim = Sim(s, cfg, "fp32c")
    variant, vms = sim.autotune(4)
    out["autotune_ms_per_variant"] = [round(float(x), 4) for x in vms]
    K = args.other_steps
    ms, l0, l1 = time_device(sim, K, 3, dist, torch)
    out["fp32c"] = {"value": K * 0.5 * (l0 + l1) / (ms * 1e-3), "ms_per_step": ms / K, "variant": int(variant),
                    "graph_mode": sim.graph_mode()}
    sim.close()
    K64 = max(3, min(K, args.fp64_steps))
    sim64 = Sim(s, cfg, "fp64")
    ms64, a0, a1 = time_device(sim64, K64, 3, dist, torch)
    out["fp64"] = {"value": K64 * 0.5 * (a0 + a1) / (ms64 * 1e-3), "ms_per_step": ms64 / K64}
    sim64.close()
    out["fp32c_over_fp64"] = out["fp32c"]["value"] / out["fp64"]["value"]
    return out


def serving_run(args):
    """Config 4: the Poisson request stream served with continuous batching in the FP32-
    compensated form, beside a one-at-a-time plain FP64 queue modelled from measured service
    times of a sample of the same requests."""
    import multiprocessing as mp

    from peridem_gb300 import gen, serve
    from peridem_gb300.sim import Sim
    specs = gen.serving_stream(n=args.serve)
    t0 = time.perf_counter()
    nproc = max(1, min(16, (os.cpu_count() or 1)))
    with mp.get_context("spawn").Pool(nproc) as pool:  # setups are the client's input files
        built = pool.map(gen.build_aggregate, [sp["gen"] for sp in specs], chunksize=1)
    t_gen = time.perf_counter() - t0
    reqs = [serve.Request(sp["rid"], s, cfg, sp["gen"]["steps"], sp["arrival"])
            for sp, (s, cfg) in zip(specs, built)]
    srv = serve.Server("fp32c", chunk_steps=args.serve_chunk, max_batch=args.serve_max_batch, keep_state=False)
    t0 = time.perf_counter()
    res = srv.run(reqs)
    wall = time.perf_counter() - t0
    summ = serve.summarize(res, wall)
    cohorts = [e for e in srv.log if e[1] == "admit"]
    summ.update(cohorts=len(cohorts), max_cohort=max((len(e[2]) for e in cohorts), default=0),
                create_s_mean=float(np.mean(srv.create_s)) if srv.create_s else 0.0,
                create_s_max=float(np.max(srv.create_s)) if srv.create_s else 0.0, finish_s_total=srv.finish_s,
                peak_device_gb=srv.peak_used / 1e9, setup_gen_s=t_gen, chunk_steps=args.serve_chunk,
                nodes_mean=float(np.mean([len(r.setup.pos) for r in reqs])),
                steps_mean=float(np.mean([r.steps for r in reqs])))
    # capacity: the same requests all waiting at once (cohorts of up to max_batch share launches)
    if args.serve_burst:
        srv_b = serve.Server("fp32c", chunk_steps=args.serve_chunk, max_batch=args.serve_max_batch, keep_state=False)
        t0 = time.perf_counter()
        res_b = srv_b.run(reqs, realtime=False)
        wall_b = time.perf_counter() - t0
        sb = serve.summarize(res_b, wall_b)
        cb = [e for e in srv_b.log if e[1] == "admit"]
        summ["all_at_once"] = {k: sb[k] for k in ("completed", "wall_s", "sims_per_hour", "bond_updates_per_s",
                                                  "ttc_p50_s", "ttc_p99_s")}
        summ["all_at_once"].update(cohorts=len(cb), max_cohort=max((len(e[2]) for e in cb), default=0),
                                   peak_device_gb=srv_b.peak_used / 1e9)
    # one at a time, plain FP64: measured per-step time and creation time on a sample spread
    # over the sizes, fitted as linear in directed bonds, then a FIFO queue over the arrivals
    order = np.argsort([2 * len(r.setup.conn) for r in reqs])
    pick = sorted({int(order[int(q)]) for q in np.linspace(0, len(reqs) - 1, args.serve_fp64_sample)})
    xs, per_step, create = [], [], []
    for i in pick:
        r = reqs[i]
        tc = time.perf_counter()
        sm = Sim(r.setup, dict(r.config, timesteps=r.steps), "fp64")
        create.append(time.perf_counter() - tc)
        sm.step(5)
        tt = time.perf_counter()
        sm.step(args.serve_fp64_steps)
        per_step.append((time.perf_counter() - tt) / args.serve_fp64_steps)
        xs.append(2 * len(r.setup.conn))
        sm.close()
    A = np.vstack([np.asarray(xs, float), np.ones(len(xs))]).T
    coef, *_ = np.linalg.lstsq(A, np.asarray(per_step), rcond=None)
    cf, *_ = np.linalg.lstsq(A, np.asarray(create), rcond=None)
    svc = np.array([max(0.0, coef[0] * 2 * len(r.setup.conn) + coef[1]) * r.steps +
                    max(0.0, cf[0] * 2 * len(r.setup.conn) + cf[1]) for r in reqs])
    arr = np.array([r.arrival for r in reqs])
    ttc64 = serve.sequential_ttc(arr, svc)
    span = float(max(arr + ttc64))
    bu = sum(r.bonds * r.steps for r in res if r.error is None)
    summ["one_at_a_time_fp64"] = {
        "ttc_p50_s": float(np.percentile(ttc64, 50)), "ttc_p99_s": float(np.percentile(ttc64, 99)),
        "sims_per_hour": len(reqs) / span * 3600.0, "bond_updates_per_s": bu / span,
        "modelled_from": f"{len(pick)} requests measured ({args.serve_fp64_steps} steps each, "
                         "per-step and creation time linear in directed bonds)"}
    return summ


def workload_config(name: str, s, cfg) -> dict:
    """The workload description both arms print as `config` (the same dict)."""
    return {"workload": name, "particles": s.n_particles, "nodes": s.n_nodes,
            "directed_bonds": s.n_bonds_directed, "dt": cfg["dt"],
            "l2": f"inputs larger than L2 ({(s.n_bonds_directed * 4.125 + s.n_nodes * 224) / 1e9:.2f} GB "
                  f"touched per step vs 0.13 GB L2)"}


def reference_arm(args):
    """The reference's CPU path on the same workload: the oracle (the restatement of PeriDEM's
    step, its OpenMP threads dealt particles and particle pairs round-robin like the
    reference's MPI ranks) on all host cores. The setup is built on the host (scipy's
    query_pairs, the reference's own call), so this arm maps no engine library. Each timed step
    is one whole step of the workload; a full step of the 4 M-node packing takes tens of
    seconds, so the arm times as many of the K steps as fit in --ref-budget seconds (at least
    one) after min(W, 1) warm-up steps and reports the rate of those."""
    r, w, _ = rank_info()
    if r != 0:
        return 0
    from oracle import oracle as O
    from peridem_gb300 import gen
    gen.set_bond_builder("cpu")
    t0 = time.perf_counter()
    s, cfg = gen.WORKLOADS[args.workload]()
    t_gen = time.perf_counter() - t0
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    orc = O.Oracle(s, cfg, threads=threads)
    t_create = time.perf_counter() - t0
    warm = min(args.warmup, 1)
    if warm:
        orc.step(warm)
    done = bonds = 0
    step_s = []
    t0 = time.perf_counter()
    while done < args.steps:
        ts = time.perf_counter()
        orc.step(1)
        step_s.append(time.perf_counter() - ts)
        bonds += orc.counts()["live_bonds"]
        done += 1
        if time.perf_counter() - t0 > args.ref_budget:
            break
    dt = time.perf_counter() - t0
    orc.close()
    rate = bonds / dt
    sample = (f"the whole {args.workload} ({s.n_nodes} nodes, {s.n_bonds_directed} directed bonds): "
              f"{done} of the {args.steps} requested steps timed after {warm} warm-up step(s), "
              f"{dt / max(done, 1):.1f} s per step on {threads} threads"
              + ("" if done == args.steps else f" (stopped at the {args.ref_budget:.0f} s budget; "
                                               "the rate is per timed step)"))
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": w, "steps": done,
        "warmup": warm, "ms_per_step": 1e3 * dt / max(done, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args.workload, s, cfg),
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "setup_s": {"generate": t_gen, "create": t_create},
                         "step_s": [round(x, 3) for x in step_s]},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def ours(args):
    import torch
    r, world, lr = rank_info()
    torch.cuda.set_device(lr % max(1, torch.cuda.device_count()))
    dist = dist_setup(world, "nccl")
    from peridem_gb300.sim import Sim

    s, cfg = load_workload(args.workload)
    K, W = args.steps, args.warmup
    peak, peak_src = measured_peak()

    # ---- FP32-compensated form (the headline); the autotuner picks the bond-kernel variant on
    # a snapshot of the state and restores it
    sim = Sim(s, cfg, "fp32c")
    if args.variant >= 0:
        variant, variant_ms = args.variant, np.zeros(0)
        sim.set_variant(variant)
    else:
        variant, variant_ms = sim.autotune(8)
    with Clocks(lr) as clk:
        ms, live0, live1 = time_device(sim, K, W, dist, torch)
    clocks = clk.summary()
    graph_mode = sim.graph_mode()
    ms = max_over_ranks(dist, ms)
    bu = K * 0.5 * (live0 + live1)
    value = sum_over_ranks(dist, bu) / (ms * 1e-3)
    # phase profile for the roofline (separate launches, CUDA events per phase)
    nprof = max(3, min(20, K))
    ph = sim.profile(nprof) / nprof
    live_p = sim.live_bonds()
    bytes_alg = 4.125 * live_p + 224.0 * s.n_nodes
    achieved = bytes_alg / (ph[2] * 1e-3) / 1e9
    traffic = ncu_traffic(args.workload, "fp32c", live_p, s.n_nodes)
    steps32 = W + K + nprof

    # ---- FP64 plain form on the same setup
    fp64 = None
    acc = None
    if not args.no_fp64:
        K64 = min(K, args.fp64_steps)
        sim64 = Sim(s, cfg, "fp64")
        ms64, l0, l1 = time_device(sim64, K64, W, dist, torch)
        ms64 = max_over_ranks(dist, ms64)
        v64 = sum_over_ranks(dist, K64 * 0.5 * (l0 + l1)) / (ms64 * 1e-3)
        ph64 = sim64.profile(3) / 3
        ach64 = (4.125 * sim64.live_bonds() + 224.0 * s.n_nodes) / (ph64[2] * 1e-3) / 1e9
        # FP64 add + multiply + fused multiply-add thread instructions per directed bond of
        # k_step, counted by ncu on crush512 (sass_thread_inst_executed_op_{dadd,dmul,dfma}:
        # 3.41e9 per launch, 7.52e7 bonds)
        ops_per_bond = 45.4
        fp64 = {"value": v64, "unit": UNIT, "steps": K64, "ms_per_step": ms64 / K64,
                "kernel_ms": ph64[2], "roofline_hbm_frac": ach64 / peak,
                "fp64_ops_per_s": v64 * ops_per_bond, "fp64_ops_per_bond": ops_per_bond,
                "note": "bound by the FP64 issue rate (sqrt, reciprocal and divisions per bond), not HBM"}
        # accuracy of FP32C vs FP64 after the same number of steps on this workload
        done64 = W + K64 + 3
        if steps32 > done64:
            sim64.step(steps32 - done64)
        elif done64 > steps32:
            sim.step(done64 - steps32)
        acc = compare_forms(sim.state(), sim64.state(), s, [sim.connectivity(p) for p in range(s.n_particles)],
                            [sim64.connectivity(p) for p in range(s.n_particles)])
        acc["steps"] = max(steps32, done64)
        sim64.close()

    # ---- end to end through the C-ABI: host arrays in, K steps, state back to host
    e2e = None
    if not args.no_e2e:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim_e = Sim(s, cfg, "fp32c")
        sim_e.set_variant(variant)
        tc = time.perf_counter()
        sim_e.step(K)
        ts = time.perf_counter()
        st = sim_e.state()
        t1 = time.perf_counter()
        e2e_s = max_over_ranks(dist, t1 - t0)
        h2d = s.nbytes()
        d2h = sum(st[k].nbytes for k in ("curpos", "vel", "acc", "force", "disp"))
        e2e = {"value": sum_over_ranks(dist, K * s.n_bonds_directed) / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": h2d / K, "d2h_bytes_per_step": d2h / K,
               "what": "pd_create_from_arrays (host arrays -> HBM, bond lists built) + K steps + "
                       "pd_get_node_state to host, wall clock",
               "split_s": {"create": tc - t0, "steps": ts - tc, "readback": t1 - ts}}
        sim_e.close()

    # ---- CPU baseline (oracle port, bounded sample), rank 0 at N=1 only
    cpu = None
    if r == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rate, done, sub = cpu_sample_rate(s, cfg, threads, 1000, 1, budget_s=args.cpu_budget)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"first {sub.n_particles} particles of {args.workload} ({sub.n_nodes} nodes, "
                         f"{sub.n_bonds_directed} bonds), {done} steps, OpenMP round-robin like the MPI ranks"}

    # ---- accuracy on dynamic workloads (impact, settling), both forms on the GPU
    acc_dyn = []
    if not args.no_accuracy:
        # config 2's particle mix breaking under the top wall: the accuracy bar under fracture
        if args.acc_steps_crush > 0:
            acc_dyn.append(accuracy_run("crush_contact", args.acc_steps_crush, steps=args.acc_steps_crush))
        acc_dyn.append(accuracy_run("two_sphere", args.acc_steps_c0))
        acc_dyn.append(accuracy_run("cubes125", args.acc_steps_c1, steps=args.acc_steps_c1))
        if args.acc_steps_c2 > 0:
            acc_dyn.append(accuracy_run(args.workload, args.acc_steps_c2))
        if args.acc_steps_c3 > 0:
            from peridem_gb300 import gen as _gen
            _gen.set_bond_builder("gpu")
            try:
                acc_dyn.append(accuracy_run("notched_plate", args.acc_steps_c3))
            finally:
                _gen.set_bond_builder("cpu")

    # ---- the other configurations' throughput (both forms, same timing rules), rank 0 at N=1
    others = []
    if r == 0 and world == 1 and args.other_configs:
        for name in [x for x in args.other_configs.split(",") if x]:
            others.append(config_line(name, args, dist, torch))

    # ---- serving stream (continuous batching), rank 0 at N=1 only
    serving = None
    if r == 0 and world == 1 and args.serve > 0:
        serving = serving_run(args)

    # our kernels per step: k_bp_decide, k_extra32 (unless fused into the bond kernel: variants
    # 6-9, 14-16 and 19), the bond kernel, k_end_step; the 7 broad-phase kernels run only in
    # rebuild steps when the step graph holds them in a conditional node, else every step
    # (exiting at once unless due)
    fused = 6 <= variant <= 9 or 14 <= variant <= 16 or variant == 19 or variant >= 21
    per_step = 3 if fused else 4
    bp = 7 * (sim.rebuilds_timed if graph_mode == 2 else K)
    # the persistent step: one cooperative launch per pd_step call of up to 1024 steps
    gpu_launches = -(-K // 1024) if graph_mode == 3 else per_step * K + bp
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 bonds / f64 state", "data": "synthetic",
        "config": workload_config(args.workload, s, cfg), "precision": "fp32c",
        "parallelism": "replicas" if world > 1 else "1 GPU",
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                     "kernel": f"k_extra32 + k_bond32 (variant {variant})", "kernel_ms": ph[2],
                     "autotune_ms_per_variant": [round(float(x), 4) for x in variant_ms],
                     "phase_ms": {"predict": ph[0], "broadphase": ph[1], "step": ph[2], "end": ph[3]}},
        "cpu_baseline": cpu, "e2e": e2e, "fp64": fp64, "accuracy_vs_fp64": acc,
        "accuracy_dynamic": acc_dyn, "serving": serving, "other_configs": others,
        "gpu_launches": gpu_launches, "broadphase_rebuilds_timed": sim.rebuilds_timed, "clocks": clocks,
        "graph_mode": {0: "separate launches", 1: "step graph", 2: "step graph, conditional broad phase",
                       3: "persistent step"}.get(graph_mode),
    }
    sim.close()
    if r == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="crush512_4m")
    ap.add_argument("--fp64-steps", type=int, default=100)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--ref-budget", type=float, default=100.0,
                    help="seconds of timed steps in --impl reference (whole steps; at least one)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--variant", type=int, default=-1, help="bond-kernel variant (default: autotune)")
    ap.add_argument("--acc-steps-crush", type=int, default=2000,
                    help="steps of the fracturing crushing accuracy case (crush_contact; 0: skip)")
    ap.add_argument("--acc-steps-c0", type=int, default=2000)
    ap.add_argument("--acc-steps-c1", type=int, default=4000)
    ap.add_argument("--acc-steps-c2", type=int, default=0, help="also compare both forms on the bench workload")
    ap.add_argument("--acc-steps-c3", type=int, default=0, help="also compare both forms on the notched plate")
    ap.add_argument("--other-configs", default="two_sphere,cubes125,crush512,notched_plate",
                    help="comma-separated workloads timed beside the headline ('' to skip)")
    ap.add_argument("--other-steps", type=int, default=200)
    ap.add_argument("--serve", type=int, default=256, help="requests of the serving stream (0: skip)")
    ap.add_argument("--serve-chunk", type=int, default=500)
    ap.add_argument("--serve-burst", type=int, default=1, help="also serve the stream with every request waiting at t=0")
    ap.add_argument("--serve-max-batch", type=int, default=32)
    ap.add_argument("--serve-fp64-sample", type=int, default=12)
    ap.add_argument("--serve-fp64-steps", type=int, default=300)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return reference_arm(args)
    return ours(args)


if __name__ == "__main__":
    sys.exit(main())
