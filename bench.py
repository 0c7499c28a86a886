"""Benchmark: batched L-BFGS pose optimisation on one GB300 (and N independent replicas).

Workload (the configuration the headline metric is quoted on): one seeded synthetic
pocket (1,500 heavy atoms + polar H), a 30 A box at 0.375 A (81^3 FP32 maps), the
24-heavy-atom / 5-torsion ligand in 65,536 poses (random centre in the box, uniform
orientation, torsions U[-pi, pi)), L-BFGS with m = 8, at most 300 iterations, gradient
tolerance 1e-3 (the other constants as the reference optimiser).

A step is one batched L-BFGS pass over all 65,536 poses. Start poses are restored and
L2 is flushed (a 256 MiB write) between steps, outside the timed kernel.

With --gpus N (N > 1), one process per GPU -- launched by torchrun, or spawned here when
no launcher set WORLD_SIZE -- each optimises a cost-balanced share (pxdock_gb300.shard) of
one set of N x 65,536 starts (weak scaling); the time is the maximum over ranks.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference algorithm on the host cores (the FP64 C port of the
reference optimiser, pinned to the reference engine by the oracle tests) on all host
threads, on a bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import tempfile
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for _sub in ("protenix-dock_gb300", "oracle"):
    sys.path.insert(0, os.path.join(REPO, _sub))

import numpy as np  # noqa: E402

N_POSES = 65536
BOX_SIZE = 30.0
SPACING = 0.375
HISTORY = 8
MAX_ITER = 300
TOL_GRAD = 1e-3
SLOPE = 1e6
METRIC = "L-BFGS-optimised poses/s, batched vs plain GPU, at |dE|<=1e-3 kcal/mol"
UNIT = "poses/s"


def workload(seed_poses=2, n_poses=N_POSES):
    from pxdock_gb300 import model, synth

    rec = model.Receptor.from_json(synth.make_receptor(seed=0))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    box = model.make_box((0.0, 0.0, 0.0), (BOX_SIZE,) * 3, SPACING)
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    poses = synth.random_poses(lig, lo, hi, n_poses, seed=seed_poses)
    return rec, lig, box, poses


def config_dict(lig, box, world=1):
    return {
        "workload": "batched L-BFGS pose optimisation: 1 ligand (%d atoms, %d torsions) x %d "
                    "poses, %dx%dx%d FP32 maps (%.0f A box @ %.3f A), m=%d, max_iter=%d, "
                    "tol_grad=%g" % (lig.n_atoms, lig.n_torsions, N_POSES, box.npoints[0],
                                     box.npoints[1], box.npoints[2], BOX_SIZE, SPACING, HISTORY,
                                     MAX_ITER, TOL_GRAD),
        "poses": N_POSES,
        "ligand_atoms": lig.n_atoms,
        "grid_points": int(np.prod(list(box.npoints))),
        "l2": "flushed between steps (256 MiB write)",
        "maps": "%d maps (%d vdW types + Coulomb), %.0f MB" % (
            len(set(int(t) for t in lig.vdw_type)) + 1, len(set(int(t) for t in lig.vdw_type)),
            (len(set(int(t) for t in lig.vdw_type)) + 1) * int(np.prod(list(box.npoints))) * 16 / 1e6),
        "parallelism": "replicas" if world == 1 else
                       "replicas x%d: one process per GPU, each a cost-balanced share of one set of "
                       "%d x %d starts, no collective on the data path" % (world, world, N_POSES),
    }


def lbfgs_params(dof_mode=0):
    from pxdock_gb300 import native

    return native.lbfgs_params(max_iter=MAX_ITER, history=HISTORY, tolerance_grad=TOL_GRAD, dof_mode=dof_mode)


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), "pxdock_bench_clocks_%d.csv" % os.getpid())

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return None
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic_per_eval():
    """DRAM bytes per score+gradient evaluation from the committed ncu summary."""
    path = os.path.join(REPO, "profiles", "lbfgs_kernel_ncu.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("dram_bytes_per_eval:"):
            return float(line.split(":")[1])
    return None


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def ncu_warp_instructions_per_eval():
    """Warp instructions per score+gradient evaluation of the batched kernel, from the
    committed ncu summary (smsp__inst_executed.sum / evaluations of the captured launch)."""
    path = os.path.join(REPO, "profiles", "lbfgs_kernel_ncu.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("warp_instructions_per_eval:"):
            return float(line.split(":")[1])
    return None


def cpu_baseline(rec, lig, box, poses, target_s=15.0, use_ref=False, keep=None):
    """The reference algorithm on the host cores over a bounded sample of poses. With
    `keep` (a dict), the port's results on the sample are stored in keep["port"]."""
    import oracle
    from pxdock_gb300 import abi

    threads = cpu_threads()
    port = oracle.PortSystem(rec, lig)
    types = sorted(set(int(t) for t in lig.vdw_type))
    port.build_grid(box, types, nthreads=threads)
    port.set_slope(SLOPE)
    p = abi.lbfgs_params(max_iter=MAX_ITER, history=HISTORY, tolerance_grad=TOL_GRAD)
    n = max(threads, 16)
    while True:
        t0 = time.perf_counter()
        res = port.lbfgs_batch(p, np.zeros((n, 0)), poses[:n], threads)
        dt = time.perf_counter() - t0
        if dt >= target_s or n >= len(poses):
            break
        n = min(len(poses), int(n * max(2.0, target_s / max(dt, 1e-3) * 1.1)))
    if keep is not None:
        keep["port"] = res
    return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d of the %d poses, FP64 C port of the reference optimiser, %d threads, "
                      "%.1f s" % (n, N_POSES, threads, dt)}


def run_reference(args):
    """The reference algorithm on the host cores: the FP64 C port of the reference
    optimiser (pinned to the reference engine within 1e-10 by the oracle tests) with
    this bench's constants, on all host threads, over a bounded sample of the poses.
    The reference engine itself always builds all 99 FP64 maps per system (minutes at
    81^3 on a few cores) and hard-codes m = 100 / tol_grad = 0.5, so it is not the timed
    arm."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    rec, lig, box, poses = workload()
    threads = cpu_threads()
    t_per_step = max(5.0, 20.0 / max(1, args.steps))
    steps, samples = [], []
    for s in range(args.warmup + args.steps):
        r = cpu_baseline(rec, lig, box, poses, target_s=t_per_step)
        if s >= args.warmup:
            steps.append(r["value"])
            samples.append(r["sample"])
    value = float(np.mean(steps))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * N_POSES / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "impl": "reference", "config": config_dict(lig, box),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": samples[-1]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def screening_ligands(n, seed=3):
    """Seeded ligands of uneven size (pxdock_gb300.synth.screening_set: heavy atoms U{10..60},
    rotatable bonds U{0..15}, C 70 % / N 12 % / O 15 % / Cl 3 %), built on all host cores.
    Ligands the device path does not take (over 256 atoms, 32 torsions or 64 fragments) are
    skipped like draws the generator cannot embed."""
    import hashlib

    from pxdock_gb300 import model, synth

    # a set generated once on this host is kept in the temp directory, keyed by the
    # generator's source, so that several runs on one host build it once
    digest = hashlib.sha256(open(synth.__file__, "rb").read()).hexdigest()[:12]
    path = os.path.join(tempfile.gettempdir(), "pxdock_screening_%d_%d_%s.json" % (n, seed, digest))
    if os.path.exists(path):
        js = json.load(open(path))
    else:
        js = synth.screening_set(n, seed, cpu_threads(), _screening_accept)
        tmp = path + ".%d" % os.getpid()
        json.dump(js, open(tmp, "w"))
        os.replace(tmp, path)
    return [model.Ligand.from_json(lj) for lj in js]


def _screening_accept(lj):
    from pxdock_gb300 import model

    lig = model.Ligand.from_json(lj)
    return lig.n_atoms <= 256 and lig.n_torsions <= 32 and lig.tree.n_frags <= 64


def run_screening(args):
    """Batched L-BFGS over many ligands of uneven size and their poses in ONE persistent
    launch (the batching of the screening configuration; L-BFGS steps only)."""
    import torch

    from pxdock_gb300 import model, native, synth

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0))
    box = model.make_box((0.0, 0.0, 0.0), (BOX_SIZE,) * 3, SPACING)
    ligs = screening_ligands(args.ligands)
    ctx = native.Context(local)
    ctx.set_receptor(rec)
    types = sorted(set(int(t) for l in ligs for t in l.vdw_type))
    n_maps = 1 + len(types)
    ctx.build_grid(box, types)
    ctx.set_slope(SLOPE)
    if args.l2_residency:
        ctx.set_l2_residency(args.l2_residency)
    ids = [ctx.add_ligand(l) for l in ligs]
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    P = args.poses_per_ligand
    max_atoms = max(l.n_atoms for l in ligs)
    n = P * len(ligs)
    xyz = np.zeros((n, max_atoms, 3), np.float32)
    lig_ids = np.zeros(n, np.int32)
    for k, (l, lid) in enumerate(zip(ligs, ids)):
        xyz[k * P:(k + 1) * P, : l.n_atoms] = synth.random_poses(l, lo, hi, P, seed=10 + k)
        lig_ids[k * P:(k + 1) * P] = lid
    # interleave ligands so that every stretch of the queue mixes sizes
    order = np.random.default_rng(0).permutation(n)
    xyz, lig_ids = xyz[order], lig_ids[order]
    dev = torch.device("cuda", local)
    start = torch.from_numpy(xyz).to(dev)
    x = start.clone()
    d_ids = torch.from_numpy(lig_ids).to(dev)
    tors = torch.zeros(1, device=dev)
    energy = torch.zeros(n, dtype=torch.float64, device=dev)
    nevals = torch.zeros(n, dtype=torch.int32, device=dev)
    status = torch.zeros(n, dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    p = lbfgs_params()
    stream = torch.cuda.Stream(dev)
    # the autotuner picks each size class's kernel variant from timed probes (on copies)
    tuned = ctx.lbfgs_autotune_dev(p, n, max_atoms, d_ids.data_ptr(), start.data_ptr(), tors.data_ptr(),
                                   sample=2048, probe_iters=40, stream=stream.cuda_stream)
    events = []
    for k in range(args.warmup + args.steps):
        with torch.cuda.stream(stream):
            x.copy_(start)
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.lbfgs_dev(p, n, max_atoms, d_ids.data_ptr(), x.data_ptr(), tors.data_ptr(), energy.data_ptr(),
                          nevals.data_ptr(), status.data_ptr(), stream.cuda_stream)
            b.record(stream)
        if k >= args.warmup:
            events.append((a, b))
    torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in events]))
    ev = int(nevals.sum().item())
    sizes = [l.n_atoms for l in ligs]
    line = {"metric": "L-BFGS-optimised poses/s, uneven ligands batched in one launch", "value": n / ms * 1e3,
            "unit": "poses/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "gpu_launches": args.steps,
            "config": {"workload": "screening: %d ligands (%d-%d atoms, 0-%d torsions) x %d poses, one launch, "
                                   "81^3 maps, m=%d, max_iter=%d, tol_grad=%g"
                                   % (len(ligs), min(sizes), max(sizes), max(l.n_torsions for l in ligs), P,
                                      HISTORY, MAX_ITER, TOL_GRAD),
                       "l2": "flushed between steps (256 MiB write)",
                       "maps": "%d maps, %.0f MB" % (n_maps, n_maps * 81 ** 3 * 16 / 1e6),
                       "l2_residency": args.l2_residency},
            "evals_per_s": ev / ms * 1e3, "evals_per_pose": ev / n,
            "autotuned_variants": {str(k): v for k, v in tuned.items()},
            "status_counts": {str(k): int((status == k).sum().item()) for k in range(4)}}
    print(json.dumps(line))
    ctx.close()
    return 0


def run_docking(args):
    """Plain docking of one complex (the reference engine's search): --walkers Monte-Carlo
    walkers of the bench ligand in a 20 A box (55^3 maps), --mc-steps steps each relaxed
    by up to --relax-steps L-BFGS iterations, all walkers in one persistent launch. The CPU
    line runs the FP64 port of the same walkers (seeds, moves, relaxations) on all host
    threads over a bounded sample of walkers, scaled to the same count."""
    import concurrent.futures

    import torch

    import oracle
    from pxdock_gb300 import model, native, synth

    torch.cuda.set_device(0)
    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0))
    lig = model.Ligand.from_json(synth.make_ligand(seed=1))
    pose_sf, _ = model.load_scoring_function(os.path.join(REPO, "protenix-dock_gb300", "pxdock_gb300", "data",
                                                          "scoring_function.json"))
    box = model.make_box((0.0, 0.0, 0.0), (20.0,) * 3, SPACING)
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    types = sorted(set(int(t) for t in lig.vdw_type))
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box, types)
    ctx.set_slope(SLOPE)
    ctx.set_scoring_function(0, pose_sf)
    lid = ctx.add_ligand(lig)
    W = args.walkers
    p = native.mc_params(lo, hi, seed=0, max_nsteps=args.mc_steps, relax_nsteps=args.relax_steps)
    starts = np.repeat(lig.poses[0][None], W, axis=0)
    ids = np.arange(W)
    times = []
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = ctx.mc_search(p, lid, starts, ids)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
    gpu_s = float(np.mean(times))
    # CPU: the FP64 port walkers on the host threads, a bounded sample
    threads = cpu_threads()
    port = oracle.PortSystem(rec, lig)
    port.build_grid(box, types, nthreads=threads)
    port.set_slope(SLOPE)
    n_cpu = min(W, threads)
    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        list(ex.map(lambda w: port.mc_walker(pose_sf, lo, hi, 0, w, lig.poses[0], True, args.mc_steps,
                                             args.relax_steps), range(1, n_cpu + 1)))
    cpu_dt = time.perf_counter() - t0
    cpu_s = cpu_dt * W / n_cpu  # walkers are independent: the full search is W / n_cpu rounds
    best = float(np.min(out["pscore"][out["status"] == 0])) if np.any(out["status"] == 0) else None
    line = {"metric": "docking searches/s (one complex, %d walkers)" % W, "value": 1.0 / gpu_s,
            "unit": "searches/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * gpu_s, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded)", "gpu_launches": args.steps,
            "config": {"workload": "docking: bench ligand, %d walkers x %d MC steps, relax <= %d L-BFGS "
                                   "iterations, 55^3 maps (20 A box @ 0.375 A)" % (W, args.mc_steps, args.relax_steps)},
            "e2e": {"value": 1.0 / gpu_s, "unit": "searches/s", "h2d_bytes_per_step": int(starts.nbytes),
                    "d2h_bytes_per_step": int(out["xyz"].nbytes + 24 * W)},
            "best_pscore": best, "status_counts": {str(k): int((out["status"] == k).sum()) for k in range(3)},
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "searches/s", "cores": threads, "kind": "port",
                             "sample": "%d of %d walkers on %d threads in %.1f s, scaled to %d walkers"
                                       % (n_cpu, W, threads, cpu_dt, W)}}
    print(json.dumps(line))
    ctx.close()
    return 0


def run_screening_mc(args):
    """Screening with Monte-Carlo search: --ligands uneven ligands (screening_ligands),
    --poses-per-ligand walkers each, --mc-steps steps relaxed by up to --relax-steps L-BFGS
    iterations (the reference search's defaults), every walker of every ligand in one
    persistent launch over the 81^3 maps. The CPU line runs the FP64 port's walkers (same
    seeds, moves, relaxations) on all host threads over a bounded sample, scaled."""
    import concurrent.futures

    import torch

    import oracle
    from pxdock_gb300 import model, native, synth

    torch.cuda.set_device(0)
    native.load(auto_build=True)
    rec = model.Receptor.from_json(synth.make_receptor(seed=0))
    box = model.make_box((0.0, 0.0, 0.0), (BOX_SIZE,) * 3, SPACING)
    lo = np.array(box.init_xyz)
    hi = lo + (np.array(box.npoints) - 1) * box.spacing
    pose_sf, _ = model.load_scoring_function(os.path.join(REPO, "protenix-dock_gb300", "pxdock_gb300", "data",
                                                          "scoring_function.json"))
    ligs = screening_ligands(args.ligands)
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    types = sorted(set(int(t) for l in ligs for t in l.vdw_type))
    ctx.build_grid(box, types)
    ctx.set_slope(SLOPE)
    if args.l2_residency:
        ctx.set_l2_residency(args.l2_residency)
    ctx.set_scoring_function(0, pose_sf)
    ids = [ctx.add_ligand(l) for l in ligs]
    W = args.poses_per_ligand
    A = max(l.n_atoms for l in ligs)
    n = W * len(ligs)
    starts = np.zeros((n, A, 3))
    lig_ids = np.repeat(np.array(ids), W)
    walker = np.tile(np.arange(W), len(ligs))
    first = (walker == 0).astype(np.int32)
    for k, l in enumerate(ligs):
        starts[k * W:(k + 1) * W, : l.n_atoms] = l.poses[0]
    p = native.mc_params(lo, hi, seed=0, max_nsteps=args.mc_steps, relax_nsteps=args.relax_steps)
    times = []
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = ctx.mc_search_multi(p, lig_ids, starts, walker, first)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
    gpu_s = float(np.mean(times))
    line = {"metric": "Monte-Carlo walker-steps/s, uneven ligands batched in one launch",
            "value": n * args.mc_steps / gpu_s, "unit": "walker-steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * gpu_s, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "gpu_launches": args.steps,
            "config": {"workload": "screening with MC: %d ligands (%d-%d atoms, 0-%d torsions) x %d walkers x %d "
                                   "MC steps, relax <= %d L-BFGS iterations, 81^3 maps, one launch"
                                   % (len(ligs), min(l.n_atoms for l in ligs), max(l.n_atoms for l in ligs),
                                      max(l.n_torsions for l in ligs), W, args.mc_steps, args.relax_steps),
                       "l2_residency": args.l2_residency},
            "e2e": {"value": n * args.mc_steps / gpu_s, "unit": "walker-steps/s",
                    "h2d_bytes_per_step": int(starts.nbytes), "d2h_bytes_per_step": int(out["xyz"].nbytes + 24 * n)},
            "status_counts": {str(k): int((out["status"] == k).sum()) for k in range(3)}}
    if not args.no_cpu_baseline:
        threads = cpu_threads()
        sample = [(k, w) for k in range(0, len(ligs), max(1, len(ligs) // threads)) for w in (0,)][:threads]
        ports = {}
        for k, _ in sample:
            pt = oracle.PortSystem(rec, ligs[k])
            pt.build_grid(box, sorted(set(int(t) for t in ligs[k].vdw_type)), nthreads=threads)
            pt.set_slope(SLOPE)
            ports[k] = pt
        t0 = time.perf_counter()
        with concurrent.futures.ThreadPoolExecutor(threads) as ex:
            list(ex.map(lambda kw: ports[kw[0]].mc_walker(pose_sf, lo, hi, 0, 1, ligs[kw[0]].poses[0], False,
                                                          args.mc_steps, args.relax_steps), sample))
        cpu_dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": len(sample) * args.mc_steps / cpu_dt, "unit": "walker-steps/s",
                                "cores": threads, "kind": "port",
                                "sample": "%d walkers (one per sampled ligand) x %d MC steps on %d threads in %.1f s"
                                          % (len(sample), args.mc_steps, threads, cpu_dt)}
    print(json.dumps(line))
    ctx.close()
    return 0


DIFF_COMPLEXES = 64
DIFF_POSES = 256
DIFF_BOX = 20.0


def diff_complexes(n_complexes, seed0=100):
    """Seeded complexes of the differentiation configuration: receptor seed 100+c (1,500
    heavy atoms + polar H, 26 A cube), a ligand of U{20..40} heavy atoms and U{2..8}
    rotatable bonds, a 20 A box at 0.375 A (55^3 points)."""
    from pxdock_gb300 import model, synth

    rng = np.random.default_rng(seed0)
    out = []
    k = 0
    while len(out) < n_complexes:
        c = len(out)
        h, r = int(rng.integers(20, 41)), int(rng.integers(2, 9))
        k += 1
        try:
            lj = synth.make_ligand(seed=5000 + k, n_heavy=h, n_rot=min(r, h // 3), n_n=max(1, round(0.12 * h)),
                                   n_o=max(1, round(0.15 * h)), n_other=round(0.03 * h))
        except RuntimeError:
            continue
        rec = model.Receptor.from_json(synth.make_receptor(seed=seed0 + c))
        out.append((rec, model.Ligand.from_json(lj)))
    return out


def run_differentiate(args):
    """Differentiation through fixed poses: for every pose of every complex, the summed
    score (empirical terms with 36 weights + 32 x 256 pair tables, plus the grid-map
    docking energy) and its gradients with respect to the pose DOFs (centre, quaternion,
    torsions), the atom coordinates, the weights and the tables, through the
    torch.autograd Functions of pxdock_gb300.autograd. A step is one forward + backward
    over all poses."""
    import torch

    from pxdock_gb300 import abi, model, native
    from pxdock_gb300 import autograd as AG

    torch.cuda.set_device(0)
    native.load(auto_build=True)
    dev = torch.device("cuda", 0)
    pose_sf, _ = model.load_scoring_function(os.path.join(REPO, "protenix-dock_gb300", "pxdock_gb300", "data",
                                                          "scoring_function.json"))
    cplx = diff_complexes(args.complexes)
    P = args.poses_per_ligand
    box = model.make_box((0.0, 0.0, 0.0), (DIFF_BOX,) * 3, SPACING)
    ctxs, lids, refs, dofs = [], [], [], []
    rng = np.random.default_rng(7)
    for c, (rec, lig) in enumerate(cplx):
        ctx = native.Context(0)
        ctx.set_receptor(rec)
        ctx.build_grid(box, sorted(set(int(t) for t in lig.vdw_type)))
        ctx.set_slope(SLOPE)
        ctx.set_scoring_function(0, pose_sf)
        lid = ctx.add_ligand(lig)
        ctxs.append(ctx)
        lids.append(lid)
        x0 = lig.poses[0] - lig.poses[0].mean(axis=0)
        refs.append(torch.tensor(x0, dtype=torch.float32, device=dev))
        q = rng.normal(size=(P, 4))
        dofs.append((rng.uniform(-4.0, 4.0, size=(P, 3)), q / np.linalg.norm(q, axis=1, keepdims=True),
                     rng.uniform(-np.pi, np.pi, size=(P, lig.n_torsions))))
    A = max(l.n_atoms for _, l in cplx)
    Tmax = max(l.n_torsions for _, l in cplx)
    D = 7 + Tmax
    n = P * len(cplx)
    ctx_ids = torch.tensor(np.repeat(np.arange(len(cplx)), P).astype(np.int32), device=dev)
    lig_ids = torch.tensor(np.repeat(np.array(lids), P).astype(np.int32), device=dev)
    xyz_ref = torch.zeros((n, A, 3), dtype=torch.float32, device=dev)
    q_all = np.zeros((n, D), np.float32)
    for c, ((_, lig), (cen, qu, tq)) in enumerate(zip(cplx, dofs)):
        xyz_ref[c * P:(c + 1) * P, : lig.n_atoms] = refs[c]
        q_all[c * P:(c + 1) * P, :3] = cen
        q_all[c * P:(c + 1) * P, 3:7] = qu
        q_all[c * P:(c + 1) * P, 7:7 + lig.n_torsions] = tq
    w0 = abi.sf_weights(pose_sf)
    t0 = abi.smooth_pair_tables(1)
    # pinned host inputs (the e2e leg copies them in and the gradients out every step)
    h_q = torch.from_numpy(q_all).pin_memory()
    h_w = torch.from_numpy(w0).pin_memory()
    h_t = torch.from_numpy(t0.astype(np.float32)).pin_memory()
    d_q, d_w, d_t = h_q.to(dev), h_w.to(dev), h_t.to(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(dev)

    def step(q_dev, w_dev, t_dev):
        q = q_dev.detach().requires_grad_(True)
        w = w_dev.detach().requires_grad_(True)
        t = t_dev.detach().requires_grad_(True)
        xyz = AG.ligand_pose_multi(ctxs, ctx_ids, lig_ids, xyz_ref, q)
        s = AG.empirical_score(ctxs, lig_ids, xyz, w, t, ctx_ids=ctx_ids)
        e = AG.docking_energy(ctxs, lig_ids, xyz, ctx_ids=ctx_ids)
        total = (s + e).sum()
        total.backward()
        return total, q, w, t

    ms, e2e_ms = [], []
    launches = 5  # pose, adjoint (+ its table partial sum), docking energy; pose backward
    for k in range(args.warmup + args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            total, q, w, t = step(d_q, d_w, d_t)
            b.record(stream)
        torch.cuda.synchronize()
        if k >= args.warmup:
            ms.append(a.elapsed_time(b))
    # end to end: pinned host DOFs and parameters in, every gradient back to pinned host memory
    h_gq = torch.empty(h_q.shape, dtype=torch.float32).pin_memory()
    h_gw = torch.empty(abi.NUM_SF_WEIGHTS, dtype=torch.float64).pin_memory()
    h_gt = torch.empty(t0.shape, dtype=torch.float32).pin_memory()
    for k in range(args.warmup + args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            total, q, w, t = step(h_q.to(dev, non_blocking=True), h_w.to(dev, non_blocking=True),
                                  h_t.to(dev, non_blocking=True))
            h_gq.copy_(q.grad, non_blocking=True)
            h_gw.copy_(w.grad, non_blocking=True)
            h_gt.copy_(t.grad, non_blocking=True)
            b.record(stream)
        torch.cuda.synchronize()
        if k >= args.warmup:
            e2e_ms.append(a.elapsed_time(b))
    t_ms, e_ms = float(np.mean(ms)), float(np.mean(e2e_ms))
    cpu = None if args.no_cpu_baseline else diff_cpu_baseline(cplx, dofs, box, pose_sf, w0, t0)
    h2d = h_q.numel() * 4 + h_w.numel() * 8 + h_t.numel() * 4
    d2h = h_gq.numel() * 4 + h_gw.numel() * 8 + h_gt.numel() * 4
    sizes = [l.n_atoms for _, l in cplx]
    line = {"metric": "differentiated poses/s (score + gradients in coordinates, DOFs, 36 weights, 32x256 "
                      "pair tables)", "value": n / t_ms * 1e3, "unit": "poses/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "gpu_launches": launches * args.steps,
            "e2e": {"value": n / e_ms * 1e3, "unit": "poses/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "config": {"workload": "differentiation through fixed poses: %d complexes x %d poses, 55^3 maps each, "
                                   "ligands %d-%d atoms, forward + backward through torch.autograd, every complex in one launch per kernel"
                                   % (len(cplx), P, min(sizes), max(sizes)),
                       "l2": "flushed between steps (256 MiB write); 64 map sets exceed L2"},
            "total_score": float(total.item())}
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line))
    for c in ctxs:
        c.close()
    return 0


def diff_cpu_baseline(cplx, dofs, box, sf, weights, tables, target_s=10.0):
    """The same per-pose work on the host cores in FP64 (the port): forward kinematics,
    the empirical score with its analytic adjoint (coordinates, weights, tables) and the
    docking energy with its gradient, over the poses of the first complexes."""
    from concurrent.futures import ThreadPoolExecutor

    import oracle

    threads = cpu_threads()
    rec, lig = cplx[0]
    port = oracle.PortSystem(rec, lig)
    port.build_grid(box, sorted(set(int(t) for t in lig.vdw_type)), nthreads=threads)
    port.set_slope(SLOPE)
    centers, quats, tors = dofs[0]
    x0 = lig.poses[0] - lig.poses[0].mean(axis=0)

    def one(p):
        q = quats[p] / np.linalg.norm(quats[p])
        a, b, c, d = q
        rot = np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (a * c + b * d)],
                        [2 * (a * d + b * c), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                        [2 * (b * d - a * c), 2 * (a * b + c * d), a * a - b * b - c * c + d * d]])
        x = port.ligand_apply(x0, centers[p], rot, tors[p])
        oracle.port_score_diff(sf, rec, lig, rec.xyz, x, weights, tables)
        port.score_grad([], x)

    n = threads
    with ThreadPoolExecutor(threads) as ex:
        while True:
            t0 = time.perf_counter()
            list(ex.map(one, [k % len(centers) for k in range(n)]))
            dt = time.perf_counter() - t0
            if dt >= target_s or n >= 1 << 16:
                break
            n = int(n * max(2.0, target_s / max(dt, 1e-3) * 1.1))
    return {"value": n / dt, "unit": "poses/s", "cores": threads, "kind": "port",
            "sample": "%d pose evaluations of complex 0 (%d atoms), FP64 C port: kinematics, empirical score "
                      "with its analytic adjoint, docking energy and gradient; %d threads, %.1f s"
                      % (n, lig.n_atoms, threads, dt)}


def unroll_complexes(n_complexes, n_receptors=64, n_ligands=128, seed0=200):
    """Seeded complexes of the unrolled-optimisation configuration: n_receptors pockets
    (600 heavy atoms + polar H in a 20 A cube) and n_ligands ligands of U{15..50} heavy
    atoms and U{0..12} rotatable bonds; complex c pairs pocket c % n_receptors with ligand
    c % n_ligands (1,024 distinct pairs with the defaults)."""
    from pxdock_gb300 import model, synth

    rng = np.random.default_rng(seed0)
    recs = [model.Receptor.from_json(synth.make_receptor(seed=seed0 + r, n_heavy=600, cube=20.0, cavity=6.0))
            for r in range(min(n_receptors, n_complexes))]
    ligs, k = [], 0
    while len(ligs) < min(n_ligands, n_complexes):
        h, r = int(rng.integers(15, 51)), int(rng.integers(0, 13))
        k += 1
        try:
            lj = synth.make_ligand(seed=9000 + k, n_heavy=h, n_rot=min(r, h // 3), n_n=max(1, round(0.12 * h)),
                                   n_o=max(1, round(0.15 * h)), n_other=round(0.03 * h))
        except RuntimeError:
            continue
        ligs.append(model.Ligand.from_json(lj))
    return recs, [ligs[c % len(ligs)] for c in range(n_complexes)]


def run_unroll(args):
    """Differentiation through optimisation: 50 unrolled L-BFGS steps (checkpoints every
    10) over pose DOFs on the differentiable empirical score, for every pose of every
    complex, then the gradient of a pose-RMSD loss against seeded target poses with
    respect to the 36 weights and the 32 x 256 pair tables. A step is forward + backward."""
    import torch

    from pxdock_gb300 import abi, model, native
    from pxdock_gb300 import unroll as UN

    torch.cuda.set_device(0)
    native.load(auto_build=True)
    dev = torch.device("cuda", 0)
    sf, _ = model.load_scoring_function(os.path.join(REPO, "protenix-dock_gb300", "pxdock_gb300", "data",
                                                     "scoring_function.json"))
    n_cplx, P_each, K = args.complexes, args.poses_per_ligand, args.unroll_steps
    recs, ligs = unroll_complexes(n_cplx)
    ctxs = []
    for r in recs:
        c = native.Context(0)
        c.set_receptor(r)
        c.set_scoring_function(0, sf)
        ctxs.append(c)
    lig_of = [ctxs[c % len(ctxs)].add_ligand(ligs[c]) for c in range(n_cplx)]
    A = max(l.n_atoms for l in ligs)
    D = 7 + max(l.n_torsions for l in ligs)
    n = n_cplx * P_each
    cplx = np.repeat(np.arange(n_cplx), P_each)
    ref = np.zeros((n, A, 3), np.float32)
    for c, l in enumerate(ligs):
        ref[c * P_each:(c + 1) * P_each, : l.n_atoms] = l.poses[0] - l.poses[0].mean(axis=0)
    rng = np.random.default_rng(5)
    nt = [ligs[c].n_torsions for c in cplx]
    # seeded target poses; each start is its target perturbed (centre ~0.7 A, orientation
    # ~0.1 per quaternion component, torsions ~0.4 rad)
    qt = UN.random_dofs(rng, nt, D, centre_scale=2.0, tors_scale=np.pi)
    q0 = qt.copy()
    q0[:, :3] += rng.normal(scale=0.7, size=(n, 3))
    q0[:, 3:7] += rng.normal(scale=0.1, size=(n, 4))
    q0[:, 3:7] /= np.linalg.norm(q0[:, 3:7], axis=1, keepdims=True)
    for p in range(n):
        q0[p, 7:7 + nt[p]] += rng.normal(scale=0.4, size=nt[p])
    n_atoms = torch.tensor([ligs[c].n_atoms for c in cplx], device=dev)

    def backend(sel):
        return UN.KernelBackend(ctxs, torch.tensor((cplx[sel] % len(ctxs)).astype(np.int32), device=dev),
                                torch.tensor(np.array(lig_of)[cplx[sel]].astype(np.int32), device=dev),
                                torch.tensor(ref[sel], device=dev), D)

    def train_step(be, sel, steps=K):
        w = torch.tensor(abi.sf_weights(sf), dtype=torch.float64, device=dev, requires_grad=True)
        t = torch.tensor(abi.smooth_pair_tables(1), dtype=torch.float64, device=dev, requires_grad=True)
        # the optimiser's state (DOFs, history, two-loop dots) in FP64; the score, its
        # adjoint and the kinematics run in FP32 kernels
        q = torch.tensor(q0[sel], dtype=torch.float64, device=dev)
        target = UN.place(be, torch.tensor(qt[sel], dtype=torch.float64, device=dev)).detach()
        qK = UN.lbfgs_unroll(be, q, w, t, steps=steps, history=8, cap=0.3, every=10, truncate=args.unroll_truncate,
                             clip=args.unroll_clip)
        loss = UN.rmsd_loss(UN.place(be, qK), target, n_atoms[sel])
        loss.backward()
        return loss, w.grad, t.grad

    allsel = np.arange(n)
    be = backend(allsel)
    stream = torch.cuda.Stream(dev)
    ms = []
    torch.cuda.reset_peak_memory_stats(dev)
    free0, total_mem = torch.cuda.mem_get_info(dev)
    for k in range(args.warmup + args.steps):
        with torch.cuda.stream(stream):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            loss, gw, gt = train_step(be, allsel)
            b.record(stream)
        torch.cuda.synchronize()
        if k >= args.warmup:
            ms.append(a.elapsed_time(b))
    peak_torch = torch.cuda.max_memory_allocated(dev)
    free1, _ = torch.cuda.mem_get_info(dev)
    t_ms = float(np.mean(ms))
    line = {"metric": "unrolled-optimisation training steps/s (%d L-BFGS steps, checkpoints every 10, "
                      "RMSD loss to 36 weights + 32x256 pair tables)" % K, "value": 1e3 / t_ms, "unit": "steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "gpu_launches": int(be.launches // max(1, args.warmup + args.steps)) * args.steps,
            "config": {"workload": "differentiation through optimisation: %d complexes (%d pockets x 128 ligands, "
                                   "ligands %d-%d atoms, 0-%d torsions) x %d poses, %d unrolled L-BFGS steps "
                                   "(m=8, step cap 0.3), checkpoints every 10; objective = differentiable "
                                   "empirical score (no maps needed)"
                                   % (n_cplx, len(ctxs), min(l.n_atoms for l in ligs), max(l.n_atoms for l in ligs),
                                      max(l.n_torsions for l in ligs), P_each, K),
                       "poses": n, "gradient": "exact" if args.unroll_truncate is None and args.unroll_clip is None
                       else "truncated to the last %s steps, clipped at %s" % (args.unroll_truncate, args.unroll_clip)},
            "poses_per_s": n / t_ms * 1e3,
            "peak_hbm": {"torch_max_allocated_gb": peak_torch / 1e9,
                         "device_used_gb": (total_mem - min(free0, free1)) / 1e9},
            "loss": float(loss.item()),
            "grad_norm": {"weights": float(gw.norm().item()), "tables": float(gt.norm().item()),
                          "nonfinite": int((~torch.isfinite(gw)).sum().item() + (~torch.isfinite(gt)).sum().item())}}
    if not args.no_cpu_baseline:
        line["cpu_baseline"], line["gradient_error"] = unroll_cpu_check(args, ctxs, recs, ligs, lig_of, ref, q0, qt,
                                                                        sf, D, K, P_each, backend, train_step)
        _, line["gradient_error_5_steps"] = unroll_cpu_check(args, ctxs, recs, ligs, lig_of, ref, q0, qt, sf, D, 5,
                                                             P_each, backend, train_step)
        _, line["gradient_error_2_steps"] = unroll_cpu_check(args, ctxs, recs, ligs, lig_of, ref, q0, qt, sf, D, 2,
                                                             P_each, backend, train_step)
    print(json.dumps(line))
    for c in ctxs:
        c.close()
    return 0


def unroll_cpu_check(args, ctxs, recs, ligs, lig_of, ref, q0, qt, sf, D, K, P_each, backend, train_step,
                     n_check=8):
    """The same unroll on the first n_check complexes in FP64 on the host cores (the
    oracle's port as backend): its time, and the error of the GPU gradient.

    The score's gradient jumps at ramp ends, the LJ clamp and pair-table bin edges, so an
    unrolled trajectory is discontinuous in its start: FP32 and FP64 rounding put some
    poses on different sides of a jump and their trajectories part. The gradients are
    compared on the loss over the poses whose final DOFs agree within 1e-3 (the loss of a
    pose depends on its own trajectory only); the fraction of such poses is reported."""
    import torch

    import unroll_ref as U
    from pxdock_gb300 import abi
    from pxdock_gb300 import unroll as UN

    sel = np.arange(n_check * P_each)
    cplx = sel // P_each
    threads = cpu_threads()
    n_atoms = np.array([ligs[c].n_atoms for c in cplx])
    sides = {}
    t_cpu = 0.0
    for name in ("gpu", "cpu"):
        if name == "gpu":
            be, d, tdt = backend(sel), torch.device("cuda", 0), torch.float64
        else:
            be = U.PortBackend([U.Pose(recs[c % len(recs)], ligs[c], sf, ref[p, : ligs[c].n_atoms], D)
                                for p, c in zip(sel, cplx)], threads=threads)
            d, tdt = torch.device("cpu"), torch.float64
        w = torch.tensor(abi.sf_weights(sf), dtype=torch.float64, device=d, requires_grad=True)
        t = torch.tensor(abi.smooth_pair_tables(1), dtype=tdt, device=d, requires_grad=True)
        t0 = time.perf_counter()
        target = UN.place(be, torch.tensor(qt[sel], device=d)).detach()
        qK = UN.lbfgs_unroll(be, torch.tensor(q0[sel], device=d), w, t, steps=K, history=8, cap=0.3, every=10,
                             truncate=args.unroll_truncate, clip=args.unroll_clip)
        x = UN.place(be, qK)
        mask = (torch.arange(x.shape[1], device=d)[None, :] < torch.tensor(n_atoms, device=d)[:, None]).to(x.dtype)
        rmsd = torch.sqrt((((x - target) ** 2).sum(-1) * mask).sum(1) / torch.tensor(n_atoms, device=d).to(x.dtype))
        if name == "cpu":
            t_cpu = time.perf_counter() - t0
        sides[name] = dict(qK=qK.detach().cpu().numpy(), rmsd=rmsd, w=w, t=t)
    agree = np.abs(sides["gpu"]["qK"] - sides["cpu"]["qK"]).max(1) <= 1e-3
    out = {}
    for name, sd in sides.items():
        m = torch.tensor(agree, dtype=sd["rmsd"].dtype, device=sd["rmsd"].device)
        t0 = time.perf_counter()
        ((sd["rmsd"] * m).sum() / max(1.0, float(agree.sum()))).backward()
        if name == "cpu":
            t_cpu += time.perf_counter() - t0
        out[name] = (sd["w"].grad.cpu().numpy(), sd["t"].grad.cpu().numpy().reshape(-1))
    (wg, tg), (wc, tc) = out["gpu"], out["cpu"]
    rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))
    cpu = {"value": 1.0 / t_cpu * (n_check * P_each) / len(q0), "unit": "steps/s", "cores": threads,
           "kind": "port",
           "sample": "%d complexes x %d poses (of %d), the same unroll on the FP64 C port, %d threads, %.1f s; "
                     "value scaled to the full workload" % (n_check, P_each, len(q0) // P_each, threads, t_cpu)}
    err = {"complexes": n_check, "unrolled_steps": K, "poses_agreeing": float(agree.mean()),
           "weights_rel_l2": rel(wg, wc) if agree.any() else None,
           "tables_rel_l2": rel(tg, tc) if agree.any() else None,
           "nan": [int(np.isnan(wg).sum() + np.isnan(tg).sum()), int(np.isnan(wc).sum() + np.isnan(tc).sum())]}
    return cpu, err

def run_evaluate(args):
    """Score+gradient evaluations/s of the bench workload's poses (one evaluation per pose
    per launch, pxd_score_grad_dev), inputs resident in HBM, L2 flushed between launches."""
    import torch

    from pxdock_gb300 import native

    torch.cuda.set_device(0)
    native.load(auto_build=True)
    rec, lig, box, poses = workload(n_poses=args.poses)
    ctx = native.Context(0)
    ctx.set_receptor(rec)
    ctx.build_grid(box, sorted(set(int(t) for t in lig.vdw_type)))
    ctx.set_slope(SLOPE)
    lid = ctx.add_ligand(lig)
    n, N = args.poses, lig.n_atoms
    dev = torch.device("cuda", 0)
    x = torch.from_numpy(poses.astype(np.float32)).to(dev)
    ids = torch.full((n,), lid, dtype=torch.int32, device=dev)
    tors = torch.zeros(1, device=dev)
    e = torch.zeros(n, dtype=torch.float64, device=dev)
    g = torch.zeros_like(x)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(dev)
    ms = []
    for k in range(args.warmup + args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.score_grad_dev(n, N, ids.data_ptr(), x.data_ptr(), tors.data_ptr(), e.data_ptr(), g.data_ptr(),
                               tors.data_ptr(), stream.cuda_stream)
            b.record(stream)
        torch.cuda.synchronize()
        if k >= args.warmup:
            ms.append(a.elapsed_time(b))
    t = float(np.mean(ms))
    line = {"metric": "score+gradient evaluations/s", "value": n / t * 1e3, "unit": "evals/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "gpu_launches": args.steps,
            "config": {"workload": "one evaluation of each of %d poses of the bench ligand (%d atoms), 81^3 maps"
                                   % (n, N), "l2": "flushed between launches (256 MiB write)"}}
    print(json.dumps(line))
    ctx.close()
    return 0


def free_port():
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def spawn_ranks(n):
    """--gpus N without an outer launcher: runs N ranks of this command, one per GPU, with
    the torch.distributed environment a launcher would set (rendezvous on 127.0.0.1).
    Rank 0 prints the JSON line; the exit status is the worst rank's."""
    port = free_port()
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE=str(n), LOCAL_RANK=str(r), LOCAL_WORLD_SIZE=str(n),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.abspath(__file__)] + sys.argv[1:], env=env))
    return max(p.wait() for p in procs)


def main():
    global N_POSES, BOX_SIZE
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="optimize", choices=["optimize", "evaluate", "screening", "screening_mc", "docking", "differentiate", "unroll"],
                    help="optimize: the headline (one ligand, 65,536 poses); screening: uneven "
                         "ligands batched in one launch")
    ap.add_argument("--dof-mode", type=int, default=0, choices=[0, 1],
                    help="optimize: L-BFGS variables, 0 ligand xyz + receptor torsions (the reference's), "
                         "1 rigid body + torsions (no CPU baseline leg)")
    ap.add_argument("--ligands", type=int, default=64, help="screening: number of ligands")
    ap.add_argument("--complexes", type=int, default=None,
                    help="differentiate / unroll: number of complexes (64 / 1024)")
    ap.add_argument("--l2-residency", type=float, default=0.0,
                    help="optimize / screening / screening_mc: fraction of the persisting L2 kept for the "
                         "maps (pxd_set_l2_residency; 0: off)")
    ap.add_argument("--unroll-steps", type=int, default=50, help="unroll: L-BFGS steps")
    ap.add_argument("--unroll-truncate", type=int, default=None,
                    help="unroll: backpropagate through the last T steps only (default: all)")
    ap.add_argument("--unroll-clip", type=float, default=None,
                    help="unroll: clip each pose's state gradient row at segment boundaries")
    ap.add_argument("--walkers", type=int, default=64, help="docking: Monte-Carlo walkers (exhaustiveness)")
    ap.add_argument("--mc-steps", type=int, default=2000, help="docking: Monte-Carlo steps per walker")
    ap.add_argument("--relax-steps", type=int, default=300, help="docking: L-BFGS iterations per step")
    ap.add_argument("--poses-per-ligand", type=int, default=256, help="screening: poses per ligand")
    ap.add_argument("--poses", type=int, default=N_POSES,
                    help="poses per step (smaller only for profiling captures)")
    ap.add_argument("--box", type=float, default=BOX_SIZE,
                    help="optimize: box edge in A (30: the config's 81^3 maps; larger boxes give map sets "
                         "beyond L2, for the residency experiment)")
    args = ap.parse_args()
    N_POSES = args.poses
    BOX_SIZE = args.box
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return spawn_ranks(args.gpus)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "screening":
        return run_screening(args)
    if args.workload == "screening_mc":
        return run_screening_mc(args)
    if args.workload == "docking":
        return run_docking(args)
    if args.workload == "differentiate":
        args.complexes = args.complexes or DIFF_COMPLEXES
        return run_differentiate(args)
    if args.workload == "unroll":
        args.complexes = args.complexes or 1024
        if args.poses_per_ligand == 256:
            args.poses_per_ligand = 32
        return run_unroll(args)
    if args.workload == "evaluate":
        return run_evaluate(args)

    import torch

    from pxdock_gb300 import native

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    native.load(auto_build=True)
    if world > 1:
        # weak scaling over one workload: N x 65,536 starts (seed 2) in blocks of 65,536,
        # split by the cost-balanced partition that every rank computes alike
        from pxdock_gb300 import shard

        rec, lig, box, all_poses = workload(seed_poses=2, n_poses=N_POSES * world)
        mine = shard.rank_share([float(N_POSES)] * world, rank, world)
        poses = np.concatenate([all_poses[b * N_POSES:(b + 1) * N_POSES] for b in mine])
        del all_poses
    else:
        rec, lig, box, poses = workload(seed_poses=2)
    ctx = native.Context(local)
    ctx.set_receptor(rec)
    ctx.build_grid(box, sorted(set(int(t) for t in lig.vdw_type)))
    ctx.set_slope(SLOPE)
    if args.l2_residency:
        ctx.set_l2_residency(args.l2_residency)
    lid = ctx.add_ligand(lig)
    N = lig.n_atoms
    dev = torch.device("cuda", local)
    start = torch.from_numpy(poses.astype(np.float32)).to(dev)
    xyz = start.clone()
    ids = torch.full((N_POSES,), lid, dtype=torch.int32, device=dev)
    tors = torch.zeros(1, device=dev)
    energy = torch.zeros(N_POSES, dtype=torch.float64, device=dev)
    nevals = torch.zeros(N_POSES, dtype=torch.int32, device=dev)
    status = torch.zeros(N_POSES, dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    p = lbfgs_params(args.dof_mode)
    stream = torch.cuda.Stream(dev)
    sptr = stream.cuda_stream

    def step(ev=None):
        with torch.cuda.stream(stream):
            xyz.copy_(start)
            flush.fill_(1.0)
            if ev:
                ev[0].record(stream)
            ctx.lbfgs_dev(p, N_POSES, N, ids.data_ptr(), xyz.data_ptr(), tors.data_ptr(),
                          energy.data_ptr(), nevals.data_ptr(), status.data_ptr(), sptr)
            if ev:
                ev[1].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
    evals_total = 0
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(args.steps):
            step(events[k])
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    kernel_ms = [a.elapsed_time(b) for a, b in events]
    evals_step = int(nevals.sum().item())
    evals_total = evals_step * args.steps
    st = status.cpu().numpy()
    e_final = energy.cpu().numpy()
    gpu_out = {"xyz": xyz.cpu().numpy(), "energy": e_final, "nevals": nevals.cpu().numpy(), "status": st}
    t_dev = sum(kernel_ms) / 1000.0
    if dist:
        tt = torch.tensor([t_dev], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_dev = float(tt.item())
    value = world * N_POSES * args.steps / t_dev
    # end to end through the host-buffer C-ABI call, in place on the caller's FP64 arrays as
    # the reference's optimiser call works (host <-> device copies and conversions in the
    # timed region; restoring the starts into the work arrays is not)
    e2e_times = []
    work = np.empty_like(np.ascontiguousarray(poses, np.float64))
    w_tors = np.zeros((N_POSES, ctx.n_rotors))
    w_e, w_nev, w_st = np.zeros(N_POSES), np.zeros(N_POSES, np.int32), np.zeros(N_POSES, np.int32)
    for k in range(max(1, min(args.steps, 3))):
        np.copyto(work, poses)
        w_tors[:] = 0.0
        t1 = time.perf_counter()
        ctx.lbfgs_inplace(p, lid, work, w_tors, w_e, w_nev, w_st)
        e2e_times.append(time.perf_counter() - t1)
    out = dict(xyz=work, torsions=w_tors, energy=w_e, nevals=w_nev, status=w_st)
    t_e2e = float(np.mean(e2e_times))
    if dist:
        tt = torch.tensor([t_e2e], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_e2e = float(tt.item())
    e2e_value = world * N_POSES / t_e2e
    # plain per-pose path: one call per pose
    n_plain = 64
    t1 = time.perf_counter()
    for i in range(n_plain):
        ctx.lbfgs(p, lid, poses[i:i + 1])
    plain_value = n_plain / (time.perf_counter() - t1)
    hbm_peak, peak_kind = measured_peak()
    # the maps of the bench ligand (8 x 8.5 MB) stay L2-resident, so the bandwidth that
    # bounds the gathers is L2's: measured here, random 16-byte gathers over 64 MiB
    l2_peak = native.gather_bandwidth(local, 64 << 20, 10)
    bytes_per_eval = (256 + 24) * N
    achieved = evals_step * bytes_per_eval / (np.mean(kernel_ms) / 1000.0) / 1e9
    tpe = ncu_traffic_per_eval()
    wipe = ncu_warp_instructions_per_eval()
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": float(np.mean(kernel_ms)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": dict(config_dict(lig, box, world),
                       variables="ligand xyz + receptor torsions (the reference's)" if not args.dof_mode else
                       "rigid body + torsions: centre, quaternion, %d ligand torsions" % lig.n_torsions),
        "e2e": {"value": e2e_value, "unit": UNIT,
                # pxd_lbfgs copies the caller's FP64 coordinates both ways (narrowed to FP32
                # on the device) and returns energy (FP64), evaluations and status per pose
                "h2d_bytes_per_step": N_POSES * N * 3 * 8,
                "d2h_bytes_per_step": N_POSES * (N * 3 * 8 + 8 + 4 + 4)},
        "gpu_launches": args.steps,
        "roofline": {"bound": "l2", "achieved": achieved, "peak": l2_peak, "unit": "GB/s",
                     "frac": achieved / l2_peak,
                     "peak_kind": "measured in this run: random 16-byte gathers over 64 MiB "
                                  "(pxd_gather_bandwidth)",
                     "hbm_peak": hbm_peak, "hbm_frac": achieved / hbm_peak, "hbm_peak_kind": peak_kind,
                     "traffic": None if tpe is None else tpe * evals_step,
                     "algorithmic_bytes_per_eval": bytes_per_eval},
        "plain_gpu": {"value": plain_value, "unit": UNIT, "poses": n_plain,
                      "batched_over_plain": value / world / plain_value},
        "evals_per_s": world * evals_total / t_dev,
        "evals_per_pose": evals_step / N_POSES,
        "status_counts": {str(k): int((st == k).sum()) for k in range(4)},
        "final_energy_median": float(np.nanmedian(e_final)),
        "wall_s": wall,
    }
    clocks = clk.summary()
    if clocks:
        line["clocks"] = clocks
    if wipe is not None:
        # instruction issue: warp instructions per evaluation (ncu) x evaluations/s against
        # the SMs' four schedulers at the SM clock sampled during the timed region
        mhz = clocks["sm_mhz"] if clocks else 2070.0
        rate = wipe * evals_step / (np.mean(kernel_ms) / 1000.0)
        peak_issue = n_sm * 4 * mhz * 1e6
        line["issue"] = {"warp_instructions_per_eval": wipe, "achieved": rate, "peak": peak_issue,
                         "unit": "warp instructions/s", "frac": rate / peak_issue,
                         "sm_mhz": mhz, "sms": n_sm}
    if rank == 0 and not args.no_cpu_baseline and not args.dof_mode:
        import oracle

        keep = {}
        line["cpu_baseline"] = cpu_baseline(rec, lig, box, poses, keep=keep)
        port = keep["port"]
        k = len(port["energy"])
        # outcomes of the GPU (the last timed step) and the port on the same k starts
        gpu_k = {key: v[:k] for key, v in gpu_out.items()}
        line["parity"] = oracle.compare_outcomes(gpu_k, port)
        line["parity"]["what"] = ("GPU (run) against the FP64 port of the reference optimiser "
                                  "(ref) on the cpu_baseline sample: the first %d starts" % k)
    del out
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
