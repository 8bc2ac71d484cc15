#!/usr/bin/env python3
"""Benchmark: particles/s of the smoothing hot path (k=32 neighbour search,
smoothing length, particle density, adaptive deposit at nc = 64, 128, 256) on
the 256^3-particle NFW-clustered cube of side 512 with its 8-unit periodic
shell, seeded synthetic data.

One step = index build (Morton sort + radix tree) + neighbour search + dens +
deposit of all three meshes for one cube.  `value` times steps with inputs
resident in HBM (CUDA events on the library's stream; L2 is flushed before
every step and the inputs are larger than L2).  `e2e` times the public C-ABI
call asg_smooth on Particle records and meshes in the library's huge-page
pinned host memory (asg_host_alloc), host<->device copies included (wall
clock).  Under torchrun every rank runs an independent replica
cube (the path does not exchange data); value = total particles / max time.

--impl reference times the reference algorithm on the host cores instead.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particles/s, k=32 kNN + SPH deposit at 256^3: mixed vs plain FP32 on 1 GB300"
WORKLOAD = "cfg2"  # 256^3 particles, side 512, 5000 NFW halos, nc = 64,128,256
# --workload choices: (generator name, scale divisor, description)
WORKLOADS = {
    "cfg2": ("cfg2", 1, "cfg2: 256^3 particles, side 512, 5000 NFW halos, 8-unit periodic shell, "
                        "k=32, nc=64,128,256"),
    "cfg2_s2": ("cfg2", 2, "cfg2 model at 1/8 volume: 128^3 particles, side 256, 625 NFW halos, "
                           "8-unit periodic shell, k=32, nc=32,64,128"),
    "cfg5": ("cfg5", 1, "cfg5: 512^3 particles, side 1024, 20000 NFW halos, 8-unit periodic "
                        "shell, k=32, nc=128,256,512"),
}


def env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def max_over_ranks(x: float, dist=None, device: str = "cuda") -> float:
    """The largest of every rank's x (the job's time is its slowest replica);
    x itself when not distributed."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(n_local: int, world: int, seconds: float) -> float:
    """Whole-job particles/s of `world` independent replica cubes of n_local
    particles each, all finished within `seconds` (the max over ranks)."""
    return world * n_local / seconds


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [c.strip() for c in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def deposit_cells(x, rk, boxsize, ncs, tile=8):
    """Sum over particles and meshes of the cells each deposit touches (the
    reference's cell-range expression, coarse_mesh.cpp:72-75), and of the
    8^3-cell tiles those cells fall in."""
    x = x.astype(np.float32)
    h = rk.astype(np.float32)[:, None]
    L = np.float32(boxsize)
    cells = tiles = 0
    for nc in ncs:
        f = np.float32(nc)
        lo = np.maximum(0, np.trunc(((x - h) / L) * f).astype(np.int64))
        hi = np.minimum(nc, 1 + np.trunc(((x + h) / L) * f).astype(np.int64))
        ext = np.maximum(hi - lo, 0)
        cells += int(np.prod(ext, axis=1).sum())
        t = np.where(ext > 0, (hi - 1) // tile - lo // tile + 1, 0)
        tiles += int(np.prod(t, axis=1).sum())
    return cells, tiles


def cpu_reference_run(nthreads: int, cube, ncs):
    """One pass of the reference algorithm over `cube` on the host cores: the
    C port of the reference's kd-tree construction, neighbour search (with its
    dens scatter) and deposit of every mesh, OpenMP over nthreads cores, as the
    reference's own OpenMP build runs them.  Returns seconds."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    ig = np.zeros(cube.n, np.int32)
    O = pyoracle.Oracle()
    t0 = time.perf_counter()
    rk, dens = O.neighbor_search(cube.x, cube.left, cube.right, nthreads=nthreads)
    for nc in ncs:
        O.assign_on_mesh(cube.x, cube.v, dens, rk, ig, cube.boxsize, nc, -1, nthreads=nthreads,
                         want64=False)
    return time.perf_counter() - t0


def knn_cube_counts(x, h, sample=200000, seed=5):
    """Mean over a seeded sample of particles of C_i, the number of particles in
    the cube of half-width h_i about particle i (itself included): the
    candidates any exact 33-neighbour search must examine.  Returns (mean,
    sample size)."""
    from scipy.spatial import cKDTree

    x = np.asarray(x, np.float64)
    s = np.random.default_rng(seed).choice(len(x), min(sample, len(x)), replace=False)
    cnt = cKDTree(x).query_ball_point(x[s], r=np.asarray(h, np.float64)[s], p=np.inf,
                                      return_length=True, workers=os.cpu_count() or 1)
    return float(np.mean(cnt)), int(len(s))


def knn_sets(pos, qs, cand):
    """The 33 nearest of each query qs among its candidates cand (n_q, m): keys
    (d2, index) with d2 the reference's float32 expression, as sorted index sets."""
    p = np.asarray(pos, np.float32)
    d = p[cand] - p[qs][:, None, :]
    d2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    order = np.lexsort((cand, d2), axis=-1)
    return np.sort(np.take_along_axis(cand, order[:, :33], axis=1), axis=1)


def mesh_errors64(mesh, m64, nc):
    """Largest relative errors of n and c (cells above 1e-3 of the mean n) and
    of v against |v| + n on the same cells, against an FP64 mesh."""
    nm = nc ** 3
    n64, c64, v64 = m64[:nm], m64[2 * nm:3 * nm], m64[3 * nm:]
    sel = n64 > 1e-3 * n64.mean()
    out = {}
    for name, a, ref in (("n", 0, n64), ("c", 2 * nm, c64)):
        got = mesh[a:a + nm].astype(np.float64)
        out[name] = float(np.max(np.abs(got[sel] - ref[sel]) / ref[sel]))
    sv = np.repeat(sel, 3)
    scale = (np.abs(v64) + np.repeat(n64, 3))[sv]
    out["v"] = float(np.max(np.abs(mesh[3 * nm:].astype(np.float64)[sv] - v64[sv]) / scale))
    return out


def mixed_accuracy(cube, ncs, x_mixed, rk_plain, rk_mixed, dens_mixed, meshes_plain,
                   meshes_mixed, nthreads, sample=20000):
    """Accuracy of the mixed-precision form: neighbour-set agreement with the
    FP32 form on a seeded sample of queries (the 33 nearest among the 48
    nearest candidates of the original positions, each set by its own float32
    distances), the relative change of h, and dens and the per-cell fields of
    both forms against the FP64 oracle on the original positions (exact top-33,
    FP64 dens over those lists, FP64 deposit with the oracle's rk and dens)."""
    from scipy.spatial import cKDTree

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    x = np.asarray(cube.x, np.float32)
    rng = np.random.default_rng(11)
    qs = rng.choice(cube.n, min(sample, cube.n), replace=False)
    _, cand = cKDTree(x.astype(np.float64)).query(x[qs].astype(np.float64), k=48, workers=nthreads)
    same = np.all(knn_sets(x, qs, cand) == knn_sets(x_mixed, qs, cand), axis=1)
    rel = np.abs(rk_mixed.astype(np.float64) - rk_plain) / rk_plain
    O = pyoracle.Oracle()
    te, _, nbr = O.knn_exact(x, cube.left, cube.right, nthreads)
    rk_e, _, d64 = O.dens_from_lists(x, nbr, te)
    del nbr
    out = {"neighbour_sets_identical": {"fraction": float(same.mean()), "queries": int(len(qs))},
           "h_rel_change_vs_fp32_positions": {"max": float(rel.max()),
                                              "median": float(np.median(rel))},
           "dens_rel_err_vs_fp64_oracle": float(np.max(np.abs(dens_mixed - d64) / d64)),
           "mesh_rel_err_vs_fp64_oracle": {}}
    ig = np.zeros(cube.n, np.int32)
    for k, nc in enumerate(ncs):
        _, m64, _ = O.assign_on_mesh(x, cube.v, d64.astype(np.float32), rk_e, ig, cube.boxsize, nc,
                                     -1, nthreads=nthreads)
        out["mesh_rel_err_vs_fp64_oracle"][str(nc)] = {
            "mixed": mesh_errors64(meshes_mixed[k], m64, nc),
            "plain": mesh_errors64(meshes_plain[k], m64, nc)}
    return out


def workload_config(wl_desc: str, cube) -> dict:
    """The `config` object of both arms' lines for one workload."""
    return {"workload": wl_desc + ", plain FP32 form", "n_with_shell": int(cube.n),
            "n_local": int(cube.n_local)}


def run_reference(args):
    """The reference algorithm on the host cores (the C port; the reference's
    own build needs its sources, which the benchmark host does not have), on
    the GPU arm's workload: every timed step is one full pass over the same
    cube.  Warm-up steps run the same model at 1/8 volume (they only start the
    threads and fault in the code), so the run stays within minutes."""
    rank = env_int("RANK", 0)
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    from asmooth_gb300 import synthetic as syn

    pyoracle.build_oracle()
    gen, scale, wl_desc = WORKLOADS[args.workload]
    cube, ncs = syn.make_workload(gen, seed=2, scale=scale)
    small, sncs = syn.make_workload(gen, seed=2, scale=2 * scale)
    for _ in range(args.warmup):
        cpu_reference_run(nthreads, small, sncs)
    times = [cpu_reference_run(nthreads, cube, ncs) for _ in range(args.steps)]
    sec = statistics.mean(times)
    value = cube.n_local / sec
    sample = (f"the whole workload every timed step ({wl_desc}); C port of the reference's "
              f"kd-tree + neighbour search + deposit, OpenMP over {nthreads} host cores; warm-up "
              f"steps on the same model at 1/8 volume")
    line = {
        "metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded NFW-clustered cube in cubep3m layout)", "impl": "reference",
        "config": workload_config(wl_desc, cube),
        "threads": nthreads,
        "cpu_baseline": {"value": value, "unit": "particles/s", "cores": nthreads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "particles/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch

    rank, world, local = env_int("RANK", 0), env_int("WORLD_SIZE", 1), env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from asmooth_gb300 import api
    from asmooth_gb300 import synthetic as syn

    seed = 2 + 1000 * rank  # independent replica cube per rank
    gen, scale, wl_desc = WORKLOADS[args.workload]
    cube, ncs = syn.make_workload(gen, seed=seed, scale=scale)
    n, n_local = cube.n, cube.n_local
    x_d = torch.from_numpy(cube.x).cuda()
    v_d = torch.from_numpy(cube.v).cuda()
    ctx = api.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(512 * 2 ** 20, dtype=torch.uint8, device="cuda")

    def step():
        ctx.load_particles_device(x_d.data_ptr(), n, cube.left, cube.right, v_ptr=v_d.data_ptr())
        ctx.run_neighbor_search()
        ctx.run_deposit(cube.boxsize, ncs, sign=-1)

    step_times = []  # the last timed() call's step times, ms

    def timed(step_fn, sample_clocks):
        """W warm-up steps, then K steps each timed with CUDA events on the
        context stream, L2 flushed before each; max over ranks."""
        for _ in range(args.warmup):
            step_fn()
        torch.cuda.synchronize()
        ctx.set_timing(True)
        clocks = ClockSampler(local) if sample_clocks else None
        if clocks:
            clocks.start()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        launches0 = ctx.kernel_launches
        total_ms = 0.0
        step_times.clear()
        wall0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()  # L2 flush between timed steps (not timed)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step_fn()
            e1.record(stream)
            e1.synchronize()
            total_ms += e0.elapsed_time(e1)
            step_times.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        wall = time.perf_counter() - wall0
        launches = ctx.kernel_launches - launches0
        phases = ctx.phase_ms()
        ctx.set_timing(False)
        clk = clocks.stop() if clocks else None
        return max_over_ranks(total_ms, dist) / args.steps, phases, launches, clk, wall

    ms_step, phases, launches, clk, wall = timed(step, True)
    ms_median = statistics.median(step_times)
    value = replica_value(n_local, world, ms_step * 1e-3)

    # end to end through the public C ABI: pinned host Particle records in, out
    rec_bytes = n * api.PARTICLE_DTYPE.itemsize
    d2h = rec_bytes + sum(4 * 6 * nc ** 3 for nc in ncs) + 16 * len(ncs)
    e2e = None
    host_memory = "asg_host_alloc (huge-page pinned)"

    def host_block(shape, dtype=np.float32):
        """The library's huge-page pinned memory; torch's pinned memory if the
        host refuses it (the line then says so)."""
        nonlocal host_memory
        try:
            return api.host_array(shape, dtype)
        except MemoryError:
            host_memory = "torch pinned (asg_host_alloc refused)"
            dt = np.dtype(dtype)
            nbytes = int(np.prod(shape)) * dt.itemsize
            return torch.empty(max(nbytes, 1), dtype=torch.uint8, pin_memory=True).numpy()[
                :nbytes].view(dt).reshape(shape)

    if not args.no_e2e:
        # host arrays from the library's huge-page pinned allocator (asg_host_alloc)
        p = host_block(n, api.PARTICLE_DTYPE)
        p[:] = api.make_particles(cube.x, cube.v)
        mesh_block = host_block(sum(6 * nc ** 3 for nc in ncs))  # all meshes, one block
        mesh_host, o = [], 0
        for nc in ncs:
            mesh_host.append(mesh_block[o:o + 6 * nc ** 3])
            o += 6 * nc ** 3
        for _ in range(max(1, args.warmup)):
            ctx.smooth(p, cube.left, cube.right, cube.boxsize, ncs, -1, meshes=mesh_host)
        e2e_times = []
        for _ in range(args.steps):
            p["dens"] = 0.0
            torch.cuda.synchronize()
            w0 = time.perf_counter()
            ctx.smooth(p, cube.left, cube.right, cube.boxsize, ncs, -1, meshes=mesh_host)
            e2e_times.append(time.perf_counter() - w0)
        tt = max_over_ranks(statistics.mean(e2e_times), dist)
        e2e = {"value": replica_value(n_local, world, tt), "unit": "particles/s",
               "h2d_bytes_per_step": rec_bytes, "d2h_bytes_per_step": d2h,
               "host_memory": host_memory,
               # the spread of the calls behind the mean (host-link copy rates vary)
               "call_ms": {"min": 1e3 * min(e2e_times),
                           "median": 1e3 * statistics.median(e2e_times),
                           "max": 1e3 * max(e2e_times)}}
        rk_host = p["rk"].copy()
    else:
        rk_d = torch.empty(n, dtype=torch.float32, device="cuda")
        ctx.store_fields_device(rk_ptr=rk_d.data_ptr())
        rk_host = rk_d.cpu().numpy()
    # the plain form's meshes of the last run, for the mixed form's accuracy report
    meshes_plain = [ctx.copy_mesh(k, 6 * nc ** 3) for k, nc in enumerate(ncs)]

    # roofline of the dominant kernel (measured live above)
    fp32 = ctx.measure_fp32_peak()
    pk, pk_kind = peaks()
    cells, tile_pairs = deposit_cells(cube.x, rk_host, cube.boxsize, ncs)
    dep_stats = ctx.deposit_stats()
    c_mean, c_sample = knn_cube_counts(cube.x, rk_host)
    alg = {  # algorithmic FP32 flops per step, per phase
        "knn_t33": 8.0 * c_mean * n,  # 8 flops per distance, C_i candidates per query
        "dens": 14.0 * 32 * n,        # 14 flops per tent weight, 32 receivers per query
        "deposit": 12.0 * cells,      # 12 flops per particle-cell pair
    }
    per_step = {k: v / args.steps for k, v in phases.items()}
    dom = max(("knn_t33", "deposit", "dens"), key=lambda k: per_step.get(k, 0.0))
    achieved = alg[dom] / (per_step[dom] * 1e-3) / 1e12
    # DRAM bytes of one launch of the dominant kernel: the per-particle figure of
    # an ncu capture of a smaller cube, times this launch's particles
    traffic, pipes = None, None
    tpath = os.path.join(ROOT, "profiles", "traffic_per_launch.json")
    if os.path.exists(tpath):
        rec = json.load(open(tpath)).get(dom)
        if rec:
            traffic = rec["bytes_per_particle"] * n
            # what bounds the kernel instead of FMA throughput: ALU pipe and issue slots
            pipes = {k: rec[k] for k in ("alu_pipe_pct_of_peak", "fma_pipe_pct_of_peak",
                                         "tensor_pipe_pct_of_peak", "issue_active_pct", "kernel",
                                         "capture") if k in rec}
    # DRAM bytes per particle of each dominant kernel (the capture's figure)
    # against its algorithmic bytes: kNN reads a position (16 B) and writes
    # t33, rk and the tie flag (12 B); dens reads a position, t33, idx33 and rk
    # (28 B) and adds into one 64-bit sum (8 B); the deposit reads a particle
    # record (36 B) and writes the meshes (24 B per cell)
    alg_bpp = {"knn_t33": 28.0, "dens": 36.0, "deposit": 36.0 + sum(24 * nc ** 3 for nc in ncs) / n}
    by_kernel = {}
    if os.path.exists(tpath):
        tj = json.load(open(tpath))
        for k, a_b in alg_bpp.items():
            if k in tj:
                by_kernel[k] = {"kernel": tj[k]["kernel"],
                                "bytes_per_particle": tj[k]["bytes_per_particle"],
                                "algorithmic_bytes_per_particle": a_b,
                                "ratio": tj[k]["bytes_per_particle"] / a_b}
    hbm_alg = n * (12 + 8 + 36) + sum(24 * nc ** 3 for nc in ncs)
    roof = {"bound": "fp32", "kernel": dom, "achieved": achieved, "peak": fp32, "unit": "TFLOP/s",
            "frac": achieved / fp32, "traffic": traffic, "pipe_utilisation_ncu": pipes,
            "traffic_by_kernel": by_kernel,
            "peak_source": "measured FMA-chain kernel on this GPU (no FP32 figure in the peaks file)",
            "phase_ms_per_step": per_step,
            "alg_flops_per_step": alg,
            "knn_candidates_per_query": {"mean": c_mean, "sample": c_sample,
                                         "definition": "C_i = #{j : |x_j - x_i|_inf <= h_i}"},
            "step_alg_hbm_bytes": hbm_alg,
            "deposit_work": dict(dep_stats, exact_particle_tile_pairs=tile_pairs,
                                 particle_cell_pairs=cells),
            "step_hbm_gbs_vs_peak": {"achieved": hbm_alg / (ms_step * 1e-3) / 1e9,
                                     "peak": pk["hbm_gbs"], "peak_kind": pk_kind}}
    # the whole step against its lower bound: the larger of the algorithmic
    # HBM bytes at the measured copy rate and the algorithmic FP32 flops at the
    # measured FMA rate, over the measured step time
    t_hbm = hbm_alg / (pk["hbm_gbs"] * 1e9) * 1e3
    t_fp32 = sum(alg.values()) / (fp32 * 1e12) * 1e3
    roof["step_lower_bound"] = {"t_hbm_ms": t_hbm, "t_fp32_ms": t_fp32,
                                "t_lower_ms": max(t_hbm, t_fp32), "t_measured_ms": ms_step,
                                "achieved": max(t_hbm, t_fp32) / ms_step}

    # friends-of-friends beside the path (linking length 0.2 x mean separation 2)
    fof = None
    if not args.no_fof:
        ctx.load_particles_device(x_d.data_ptr(), n, cube.left, cube.right, v_ptr=v_d.data_ptr())
        ng = ctx.run_fof(0.4)
        ms_f = []
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ng = ctx.run_fof(0.4)
            e1.record(stream)
            e1.synchronize()
            ms_f.append(e0.elapsed_time(e1))
        fof = {"ll": 0.4, "groups": ng, "ms": statistics.median(ms_f),
               "particles_per_s": n / (statistics.median(ms_f) * 1e-3)}

    # the 512^3 cube: generated on the device (the same NFW model as the numpy
    # generator, torch's random stream), its periodic shell built on the
    # device; each step loads the cube with its shell, then kNN + dens and the
    # three meshes; then GPU FOF on the loaded set
    big = None
    if not args.no_big and world == 1 and args.workload == "cfg2":
        xb, vb = syn.nfw_cube_device(512 ** 3, 1024.0, 5, n_halos=20000)
        bncs5 = (128, 256, 512)
        ctx5 = api.Context(local)
        s5 = torch.cuda.ExternalStream(ctx5.stream)
        nb = [0, 0]

        def step5():
            nb[:] = ctx5.load_periodic_cube_device(xb.data_ptr(), 512 ** 3, 1024.0, 8.0 / 1024.0,
                                                   v_ptr=vb.data_ptr())
            ctx5.run_neighbor_search()
            ctx5.run_deposit(1024.0, bncs5, sign=-1)

        step5()
        torch.cuda.synchronize()
        ctx5.set_timing(True)
        ms5 = []
        for _ in range(3):
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s5)
            step5()
            e1.record(s5)
            e1.synchronize()
            ms5.append(e0.elapsed_time(e1))
        ph5 = {k: v / 3 for k, v in ctx5.phase_ms().items() if v}
        ctx5.set_timing(False)
        ng5 = ctx5.run_fof(0.4)
        msf5 = []
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s5)
            ng5 = ctx5.run_fof(0.4)
            e1.record(s5)
            e1.synchronize()
            msf5.append(e0.elapsed_time(e1))
        m5 = statistics.median(ms5)
        big = {"workload": "512^3 particles, side 1024, 20000 NFW halos drawn on the device, "
                           "8-unit periodic shell built on the device, k=32, nc=128,256,512, "
                           "plain FP32 form",
               "n_with_shell": nb[0], "n_local": nb[1],
               "value": nb[1] / (m5 * 1e-3), "unit": "particles/s", "ms_per_step": m5,
               "steps": 3, "step": "shell + index + kNN + dens + three meshes",
               "phase_ms_per_step": ph5,
               "fof": {"ll": 0.4, "groups": ng5, "ms": statistics.median(msf5),
                       "particles_per_s": nb[0] / (statistics.median(msf5) * 1e-3)}}
        ctx5.close()
        del xb, vb

    # the reference's own small case: 64^3 particles in 200 Plummer spheres
    # plus a uniform background, side 128, nc = 32, 64 (device time per step)
    small = None
    if not args.no_small and world == 1 and args.workload == "cfg2":
        c1, ncs1 = syn.make_workload("cfg1", seed=1)
        x1 = torch.from_numpy(c1.x).cuda()
        v1 = torch.from_numpy(c1.v).cuda()

        def step1():
            ctx.load_particles_device(x1.data_ptr(), c1.n, c1.left, c1.right, v_ptr=v1.data_ptr())
            ctx.run_neighbor_search()
            ctx.run_deposit(c1.boxsize, ncs1, sign=-1)

        for _ in range(3):
            step1()
        torch.cuda.synchronize()
        ms1 = []
        for _ in range(args.steps):
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step1()
            e1.record(stream)
            e1.synchronize()
            ms1.append(e0.elapsed_time(e1))
        m1 = statistics.median(ms1)
        small = {"workload": "64^3 particles, side 128, 50% in 200 Plummer spheres, 8-unit "
                             "periodic shell, k=32, nc=32,64, plain FP32 form",
                 "n_with_shell": int(c1.n), "n_local": int(c1.n_local),
                 "value": c1.n_local / (m1 * 1e-3), "unit": "particles/s", "ms_per_step": m1,
                 "steps": args.steps, "l2": "not flushed (the whole cube fits in L2)"}

    # mixed-precision form: positions as int32 cell index + uint16 offsets in
    # 4-unit cells, decoded on the device, then the same FP32 path
    mixed = None
    if not args.no_mixed:
        cell, off, grid = syn.quantise_positions(cube)
        cell_d = torch.from_numpy(cell).cuda()
        off_d = torch.from_numpy(off.view(np.int16)).cuda()

        def step_mixed():
            ctx.load_particles_quantised_device(cell_d.data_ptr(), off_d.data_ptr(), n, cube.left,
                                                cube.right, 4.0, grid, v_ptr=v_d.data_ptr())
            ctx.run_neighbor_search()
            ctx.run_deposit(cube.boxsize, ncs, sign=-1)

        ms_m, phases_m, launches_m, _, _ = timed(step_mixed, False)
        rkm_d = torch.empty(n, dtype=torch.float32, device="cuda")
        dm_d = torch.empty(n, dtype=torch.float32, device="cuda")
        ctx.store_fields_device(rk_ptr=rkm_d.data_ptr(), dens_ptr=dm_d.data_ptr())
        rk_m = rkm_d.cpu().numpy()
        rel = np.abs(rk_m.astype(np.float64) - rk_host) / rk_host
        mixed = {"value": replica_value(n_local, world, ms_m * 1e-3), "unit": "particles/s",
                 "ms_per_step": ms_m, "vs_plain": ms_step / ms_m, "gpu_launches": launches_m,
                 "phase_ms_per_step": {k: v / args.steps for k, v in phases_m.items()},
                 "input": "int32 cell index + 3 x uint16 offsets (4-unit cells) + float32 v",
                 "h_rel_err_vs_fp32_positions": {"max": float(rel.max()),
                                                 "median": float(np.median(rel))}}
        if rank == 0 and world == 1 and not args.no_accuracy:
            from asmooth_gb300.quantised import dequantise

            meshes_m = [ctx.copy_mesh(k, 6 * nc ** 3) for k, nc in enumerate(ncs)]
            mixed["accuracy"] = mixed_accuracy(
                cube, ncs, dequantise(cell, off, grid, cube.left, 4.0), rk_host, rk_m,
                dm_d.cpu().numpy(), meshes_plain, meshes_m, os.cpu_count() or 1)
        if not args.no_e2e:
            # inputs and outputs carved from one huge-page block
            parts = [((n,), np.int32), ((n, 3), np.uint16), ((n, 3), np.float32),
                     ((n,), np.float32), ((n,), np.float32)]
            offs, o = [], 0
            for shape, dt in parts:
                offs.append(o)
                o += -(-int(np.prod(shape)) * np.dtype(dt).itemsize // 256) * 256
            qblock = host_block(o, np.uint8)
            cell_h, off_h, v_h, rk_o, dens_o = [
                qblock[a:a + int(np.prod(shape)) * np.dtype(dt).itemsize].view(dt).reshape(shape)
                for (shape, dt), a in zip(parts, offs)]
            cell_h[:] = cell
            off_h[:] = off
            v_h[:] = cube.v
            mesh_q = [mesh_block[o - 6 * nc ** 3:o] for nc, o in
                      zip(ncs, np.cumsum([6 * nc ** 3 for nc in ncs]))]

            def call():
                ctx.smooth_quantised(cell_h, off_h, v_h, cube.left, cube.right, 4.0, grid,
                                     cube.boxsize, ncs, -1, meshes=mesh_q, rk=rk_o, dens=dens_o)

            for _ in range(max(1, args.warmup)):
                call()
            times = []
            for _ in range(args.steps):
                torch.cuda.synchronize()
                w0 = time.perf_counter()
                call()
                times.append(time.perf_counter() - w0)
            tt = max_over_ranks(statistics.mean(times), dist)
            mixed["e2e"] = {"value": replica_value(n_local, world, tt), "unit": "particles/s",
                            "h2d_bytes_per_step": 22 * n,
                            "d2h_bytes_per_step": 8 * n + sum(4 * 6 * nc ** 3 for nc in ncs)
                            + 16 * len(ncs),
                            "call_ms": {"min": 1e3 * min(times), "median": 1e3 * statistics.median(times),
                                        "max": 1e3 * max(times)}}

    # batched form: the 27-cube x 3-redshift workload through one CUDA graph
    batch = None
    if not args.no_batch:
        items, bncs = syn.make_batch(scale=args.batch_scale, workers=os.cpu_count() or 1)
        with api.Batch(ctx, items, bncs) as bt:
            if not args.no_tune:
                bt.tune()
            tuned = bt.config()
            bt.set_streams(args.batch_streams)
            bt.run()  # plan, capture, first replay
            gms = []
            for _ in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                bt.run()
                gms.append(bt.stats()["graph_ms"])
            st = bt.stats()
            # the mixed-precision batched form: every item as int32 cell index +
            # uint16 offsets in 4-unit cells, decoded on the device in the graph
            from asmooth_gb300.quantised import quantise

            for i, c in enumerate(items):
                cq, oq, gq = quantise(c.x, c.left, c.right, 4.0)
                bt.set_item_quantised(i, cq, oq, c.v, 4.0, gq)
            bt.run()
            gmq = []
            for _ in range(args.steps):
                flush.zero_()
                torch.cuda.synchronize()
                bt.run()
                gmq.append(bt.stats()["graph_ms"])
        g = max_over_ranks(statistics.median(gms), dist)
        gq_ms = max_over_ranks(statistics.median(gmq), dist)
        batch = {"items": len(items), "nc": list(bncs), "particles_local": st["particles_local"],
                 "particles_with_shell": int(sum(c.n for c in items)),
                 "graph_ms": g, "value": replica_value(st["particles_local"], world, g * 1e-3),
                 "unit": "particles/s", "kernels_per_graph": st["kernels"],
                 "config": tuned, "tuned": not args.no_tune, "streams": args.batch_streams,
                 "mixed": {"graph_ms": gq_ms,
                           "value": replica_value(st["particles_local"], world, gq_ms * 1e-3),
                           "unit": "particles/s",
                           "vs_plain_batch": g / gq_ms,
                           "vs_plain_single_cube":
                               replica_value(st["particles_local"], world, gq_ms * 1e-3) / value,
                           "input": "int32 cell index + 3 x uint16 offsets (4-unit cells) + "
                                    "float32 v per particle"},
                 "workload": "27 cubes of side 256 (128^3 +- clustering-dependent count, halo "
                             "fraction U[0.2,0.8]) x 3 redshifts (halos contracted 1, 0.7, 0.5)"
                             + (f", scale 1/{args.batch_scale}" if args.batch_scale > 1 else "")}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle

        pyoracle.build_oracle()
        nthreads = os.cpu_count() or 1
        dt = cpu_reference_run(nthreads, cube, ncs)
        cpu = {"value": n_local / dt, "unit": "particles/s", "cores": nthreads, "kind": "port",
               "sample": f"one pass over the whole workload ({wl_desc}): C port of the "
                         f"reference's kd-tree + neighbour search + deposit, OpenMP over "
                         f"{nthreads} host cores"}
    line = {
        "metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "ms_per_step_median": ms_median,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded NFW-clustered cube in cubep3m layout)",
        "config": dict(workload_config(wl_desc, cube), parallelism=f"replicas x{world}",
                       l2="flushed before every timed step; inputs larger than L2"),
        "e2e": e2e,
        "gpu_launches": launches,
        "roofline": roof,
        "clocks": clk,
        "wall_s_timed": wall,
    }
    if mixed:
        line["mixed"] = mixed
    if fof:
        line["fof"] = fof
    if big:
        line["cube_512"] = big
    if small:
        line["cube_64"] = small
    if batch:
        line["batch"] = batch
    if cpu:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision leg")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the mixed form's accuracy report against the FP64 oracle")
    ap.add_argument("--workload", default="cfg2", choices=sorted(WORKLOADS),
                    help="cfg2_s2: the cfg2 model at 1/8 volume, for profiling captures; "
                         "cfg5: the 512^3 cube")
    ap.add_argument("--no-fof", action="store_true",
                    help="skip timing GPU FOF (linking length 0.4) on the loaded cube")
    ap.add_argument("--no-small", action="store_true",
                    help="skip the 64^3 Plummer cube (the reference's own small case)")
    ap.add_argument("--no-big", action="store_true",
                    help="skip the 512^3 cube (device-generated) and its FOF")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the batched form (27 cubes x 3 redshifts, one CUDA graph)")
    ap.add_argument("--batch-scale", type=int, default=1,
                    help="divide the batched cubes' side by this (quick runs)")
    ap.add_argument("--no-tune", action="store_true", help="skip autotuning the batched form")
    ap.add_argument("--batch-streams", type=int, default=4,
                    help="concurrent streams inside the batched form's graph")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
