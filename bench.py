"""Benchmark: LJ + Coulomb velocity-Verlet throughput (atom-steps/s) on GB300.

Workload (the at-scale configuration): 262,144 atoms uniform in a cube of side
68 (no two closer than 0.8 sigma), charges +/-1 (half each), sigma = eps = 1,
Coulomb k = 1, cutoff 2.5, skin 0.3, dt = 1e-3, FP32 forces with FP64
positions and velocities, neighbour list rebuilt every 10 steps.  One bench
step = 100 MD steps (10 rebuild windows), so the default --steps 10 times the
configuration's 1000 MD steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints ONE JSON line on rank 0.  Multi-GPU runs are independent replicas (the
path has no exchange step): value = all ranks' atom-steps / max rank time.
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

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "naivedynamics.jl_gb300")
for _p in (REPO, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

N_ATOMS = 262144
SIDE = 68.0
MD_PER_STEP = 100
REBUILD = 10
UNION_NAMES = {0: "blocks", 1: "tree"}
SEED = 0x4E440002
METRIC = "LJ+Coulomb atom-steps/s @262k (FP32 forces, FP64 x/v, rebuild every 10)"
UNIT = "atom-steps/s"
WORKLOAD = ("lj_coulomb_262144: N=262144, cube side 68, min separation 0.8, q=+/-1, "
            "sigma=eps=1, k=1, r_c=2.5, dt=1e-3, rebuild every 10")
# the workload as both arms report it (the arms' own settings are reported
# beside it: "engine" for the GPU arm, "reference_path" for the CPU arm)
CONFIG = {"workload": WORKLOAD, "n_atoms": N_ATOMS, "side": SIDE, "cutoff": 2.5, "dt": 1e-3,
          "rebuild_every": REBUILD,
          "l2": "GPU arm: 512 MB buffer written before every timed step (outside the events); "
                "CPU arm: not applicable"}
REF_SKIN = 0.3


def _plain(o):
    """JSON-ready copy: numpy scalars and arrays as Python numbers and lists."""
    if isinstance(o, dict):
        return {k: _plain(v) for k, v in o.items()}
    if isinstance(o, (list, tuple)):
        return [_plain(v) for v in o]
    if hasattr(o, "tolist"):
        return o.tolist()
    return o


def _plain(o):
    """JSON-ready copy: numpy scalars and arrays as Python numbers and lists."""
    if isinstance(o, dict):
        return {k: _plain(v) for k, v in o.items()}
    if isinstance(o, (list, tuple)):
        return [_plain(v) for v in o]
    if hasattr(o, "tolist"):
        return o.tolist()
    return o


def _md_params(nd, order=None):
    return nd.md_params(sigma=1.0, epsilon=1.0, coulomb_k=1.0, cutoff=2.5, skin=0.3, dt=1e-3,
                        box_lo=(0, 0, 0), box_hi=(SIDE, SIDE, SIDE), atomsperleaf=4,
                        rebuild_every=REBUILD,
                        order=nd.ND_ORDER_SPATIAL if order is None else order)


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for (_, _, r) in rows for k in range(4) if r[k] == "Active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


def _peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def _ncu_traffic():
    """Per-launch DRAM bytes of the step kernel from the committed ncu summary."""
    try:
        with open(os.path.join(REPO, "profiles", "md_step_262k.json")) as f:
            return json.load(f).get("dram_bytes_per_launch")
    except (OSError, ValueError):
        return None


def _ref_session(R):
    """The reference path on the host cores, from the oracle library alone:
    inputs from its own generators (the GPU arm's inputs bit for bit), then the
    oracle restatement of leafbuild_traverse_bvh (reference Morton order) at
    r_c + skin, FP64 LJ + Coulomb over that list and KDK velocity Verlet, as a
    session whose first list and forces are built at creation."""
    x, v, q = R.synth_lj_system(SEED, N_ATOMS, SIDE, 0.8, charges=True)
    p = R.md_params(coulomb_k=1.0, cutoff=2.5, box_hi=(SIDE,) * 3, dt=1e-3)
    return R.MDSession(p, x, v, q, rebuild=REBUILD, skin=REF_SKIN, apl=4,
                       order=R.REF_ORDER_REFERENCE)


def cpu_baseline_sample(windows=2):
    """Steady-state windows of the CPU reference path: each window is REBUILD
    MD steps with one leaf-BVH build and REBUILD force evaluations."""
    from oracle import naiveref as R
    sess = _ref_session(R)
    sess.steps(REBUILD)  # one untimed window
    t0 = time.perf_counter()
    sess.steps(REBUILD * windows)
    dt = time.perf_counter() - t0
    sess.close()
    return {"value": N_ATOMS * REBUILD * windows / dt, "unit": UNIT, "cores": R.num_threads(),
            "kind": "port",
            "sample": f"{N_ATOMS} atoms x {windows} steady-state windows of {REBUILD} MD steps "
                      f"(one leaf-BVH build in reference Morton order per window, FP64 forces, "
                      f"OpenMP over {R.num_threads()} threads), {dt:.2f} s"}


def run_reference(args):
    """The CPU reference arm: the oracle port of the reference path (Julia is
    not installed here or on the GPU machine) on all host threads, one
    steady-state window of REBUILD MD steps per bench step.  Loads the oracle
    library only."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    from oracle import naiveref as R
    sess = _ref_session(R)
    times = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        sess.steps(REBUILD)
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
    sess.close()
    total_t = sum(times)
    value = N_ATOMS * REBUILD * len(times) / total_t
    sample = (f"{N_ATOMS} atoms, {len(times)} steady-state windows of {REBUILD} MD steps, each "
              f"one leaf-BVH build (reference Morton order, r_c + skin {REF_SKIN}) and "
              f"{REBUILD} FP64 force evaluations, OpenMP over {R.num_threads()} threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total_t / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": CONFIG,
            "reference_path": ("oracle port of leafbuild_traverse_bvh + FP64 forces + KDK; "
                               f"{REBUILD} MD steps per bench step (reference Julia not "
                               "installable: no julia)"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": R.num_threads(),
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(_plain(line)), flush=True)


ENSEMBLE_STEPS = 200


def batched_leg(nd, ctx, ext, flush):
    """Batched ensemble (512 LJ systems, sizes log-uniform in [256, 16384],
    density U[0.6, 0.9], sigma U[0.9, 1.1], eps U[0.8, 1.2], r_c 2.5, dt 1e-3,
    rebuild every 10, 200 steps) through one autotuned engine, against the same
    systems run one by one through the plain engine.  Both timed with CUDA
    events on the library's stream, inputs resident, L2 flushed before each.
    On N GPUs every rank runs its share of the systems (greedy balance of the
    atom counts; no exchange): atom-steps summed over ranks over the slowest
    rank's time."""
    import numpy as np
    import torch
    from naivedynamics import replicas

    ws, rank = replicas.world()
    e_all = nd.synth.ensemble(nd.synth.SEED_ENSEMBLE)
    e = replicas.take_systems(e_all, replicas.shard_systems(e_all["n_atoms"], ws)[rank])
    table = nd.systems_table(e["n_atoms"], e["sigma"], e["epsilon"], e["box_lo"], e["box_hi"])
    base = nd.md_params(cutoff=2.5, skin=0.3, dt=1e-3, atomsperleaf=4, rebuild_every=REBUILD)
    t0 = time.perf_counter()
    tuned, _ = nd.autotune(base, e["x"], e["v"], systems=table, trial_steps=50, ctx=ctx)
    tune_s = time.perf_counter() - t0
    n_tot = int(e["n_atoms"].sum())
    off = np.concatenate([[0], np.cumsum(e["n_atoms"])])

    def timed(run):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(ext):
            a.record(ext)
            run()
            b.record(ext)
        ctx.synchronize()
        return a.elapsed_time(b) * 1e-3

    bat = nd.Ensemble(tuned, table, e["x"], e["v"], ctx=ctx)
    _, _, f_bat = bat.get()
    pe_bat0, _ = bat.energies()
    bat.run(REBUILD)  # the opening window (its own captured graph)
    bat.sync()
    l0 = ctx.launch_count()
    d0 = bat.diagnostics()
    t_bat = timed(lambda: bat.run(ENSEMBLE_STEPS))
    bat_diag = bat.diagnostics()
    bat_launches = ctx.launch_count() - l0 + bat_diag["body_kernels"] - d0["body_kernels"]
    x_end, _, f_end = bat.get()
    pe_end, _ = bat.energies()
    bat.close()
    # every system's forces and potential energy against the FP64 oracle run
    # on that system alone, at the input and after the timed steps
    from oracle import naiveref as R
    pa = l2 = er = 0.0
    for k in range(len(e["n_atoms"])):
        sl = slice(int(off[k]), int(off[k + 1]))
        pk = R.md_params(sigma=float(e["sigma"][k]), epsilon=float(e["epsilon"][k]), cutoff=2.5,
                         box_lo=tuple(e["box_lo"][k]), box_hi=tuple(e["box_hi"][k]), dt=1e-3)
        for xx, ff, pe in ((e["x"][sl], f_bat[sl], pe_bat0[k]), (x_end[sl], f_end[sl], pe_end[k])):
            g, u, _ = R.forces(pk, xx)
            a_, b_ = _force_errors(ff, g)
            pa, l2, er = max(pa, a_), max(l2, b_), max(er, abs(pe - u) / abs(u))
    errors = {"force_err_per_atom": pa, "force_err_l2": l2, "energy_rel": er,
              "over": f"{len(e['n_atoms'])} systems, input and after {ENSEMBLE_STEPS + REBUILD} "
                      "steps", "bar": 1e-5}

    plain = []
    f_err = 0.0
    for k in range(len(e["n_atoms"])):
        sl = slice(int(off[k]), int(off[k + 1]))
        side = float(e["box_hi"][k][0])
        p = nd.md_params(sigma=float(e["sigma"][k]), epsilon=float(e["epsilon"][k]), cutoff=2.5,
                         skin=tuned.skin, dt=1e-3, box_lo=(0, 0, 0), box_hi=(side, side, side),
                         atomsperleaf=tuned.atomsperleaf, rebuild_every=REBUILD,
                         resort_every=tuned.resort_every, stage_policy=tuned.stage_policy,
                         union_search=tuned.union_search,
                         refit_check_every=tuned.refit_check_every)
        eng = nd.MDEngine(p, e["x"][sl], e["v"][sl], ctx=ctx)
        _, _, fp = eng.get()
        f_err = max(f_err, float(np.linalg.norm(f_bat[sl] - fp) / np.linalg.norm(fp)))
        eng.run(REBUILD)
        plain.append(eng)
    ctx.synchronize()
    t_plain = timed(lambda: [eng.run(ENSEMBLE_STEPS) for eng in plain])
    for eng in plain:
        eng.close()
    work = replicas.sum_over_ranks(n_tot * ENSEMBLE_STEPS)
    t_bat = replicas.max_over_ranks(t_bat)
    t_plain = replicas.max_over_ranks(t_plain)
    v_bat = work / t_bat
    v_plain = work / t_plain
    n_all = int(e_all["n_atoms"].sum())
    return {"metric": "ensemble atom-steps/s, batched vs plain", "unit": UNIT, "errors": errors,
            "workload": (f"ensemble_512: {len(e_all['n_atoms'])} LJ systems, {n_all} atoms "
                         f"(N_s {int(e_all['n_atoms'].min())}..{int(e_all['n_atoms'].max())}), "
                         "rho U[0.6,0.9], sigma U[0.9,1.1], eps U[0.8,1.2], r_c 2.5, "
                         f"skin {tuned.skin:.1f} (autotuned), "
                         f"dt 1e-3, rebuild every 10, {ENSEMBLE_STEPS} steps"),
            "value": v_bat, "plain_value": v_plain, "batched_over_plain": v_bat / v_plain,
            "batched_s": t_bat, "plain_s": t_plain, "batched_gpu_launches": bat_launches,
            "force_rel_l2_batched_vs_plain_max": f_err,
            "skin_violations": bat_diag["skin_violations"],
            "early_refits": bat_diag["early_refits"],
            "tuned": {"skin": tuned.skin, "atomsperleaf": tuned.atomsperleaf,
                      "resort_every": tuned.resort_every,
                      "stage_policy": tuned.stage_policy,
                      "union_search": UNION_NAMES[tuned.union_search],
                      "refit_check_every": max(tuned.refit_check_every, 1),
                      "autotune_s": round(tune_s, 2)},
            "plain_path": "512 nd_md engines run one after another on one stream (graphs)",
            "sharding": f"{ws} rank(s), greedy balance of the systems' atom counts"}


COMPAT_N, COMPAT_STEPS = 4096, 20


def compat_leg(nd, ctx, ext, flush, cpu=True):
    """simulate! as written (nd_compat_simulate): 4,096 atoms from a collector
    shaped like the reference scripts' (unit box, temperature 0.01, masses in
    [1, 5), charges in +-1e-9), 20 steps of stepwidth 1 over the all-pairs
    list, timed as one call with host buffers in and out (the reference's
    poslog included); the oracle's literal restatement of the same loop on
    the host cores is the CPU comparison."""
    import numpy as np

    import torch

    rng = np.random.default_rng(SEED)
    n = COMPAT_N
    m = rng.uniform(1.0, 5.0, n).astype(np.float32)
    q = rng.uniform(-1e-9, 1e-9, n).astype(np.float32)
    x = rng.uniform(0.0, 1.0, (n, 3)).astype(np.float32)
    v = np.repeat((np.float32(0.01) / np.float32(n) * np.float32(3 * n) / m)[:, None], 3, axis=1)
    spec = nd.SimSpec(duration=COMPAT_STEPS, stepwidth=1, vDamp=1.0)
    clct = nd.GenericRandomCollector(objectnumber=n, minDim=(0.0, 0.0, 0.0),
                                     maxDim=(1.0, 1.0, 1.0), temperature=0.01)
    walls, dev = [], []
    for k in range(4):
        sys_ = nd.GenericObjectCollection(x, v, mass=m, charge=q)
        flush.fill_(float(k))
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        a.record(ext)
        log = nd.simulate_compat_(sys_, spec, clct, ctx=ctx)
        b.record(ext)
        b.synchronize()
        if k > 0:
            walls.append(time.perf_counter() - t0)
            dev.append(a.elapsed_time(b) * 1e-3)
    wall = float(np.median(walls))
    out = {"workload": f"simulate! as written, {n} atoms, {COMPAT_STEPS} steps (all-pairs list)",
           "metric": "atom-steps/s", "value": n * COMPAT_STEPS / wall,
           "ms_per_md_step": wall * 1e3 / COMPAT_STEPS,
           "device_span_ms_per_md_step": float(np.median(dev)) * 1e3 / COMPAT_STEPS,
           "api": "nd_compat_simulate, host arrays and the poslog copied in the timed call",
           "finite_fraction_final": float(np.isfinite(log[0]).mean())}
    if cpu:
        from oracle import naiveref as R
        steps = 2
        t0 = time.perf_counter()
        R.compat_simulate(x, v, np.zeros((n, 3)), m, q, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 0.01, n,
                          1, steps, 1.0, log=False)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n * steps / dt, "unit": "atom-steps/s", "cores": 1,
                               "kind": "port",
                               "sample": f"{n} atoms x {steps} steps of the oracle's sequential "
                                         f"restatement, {dt:.2f} s"}
    return out


def plain_leg(nd, ctx, ext, flush):
    """Plain LJ velocity Verlet at 4,096 atoms (cube side 17, min separation
    0.8, v ~ N(0,1), sigma = eps = 1, r_c 2.5, dt 1e-3, rebuild every 10):
    100 steps through the captured graphs of an autotuned engine, CUDA events
    on the library's stream, 3 untimed repetitions first; the oracle's FP64
    KDK loop with its leaf BVH on the host cores beside it."""
    import numpy as np
    import torch

    n, side, steps = 4096, 17.0, 100
    x, v, _ = nd.synth.lj_system(nd.synth.SEED_PLAIN_LJ, n, side, 0.8)
    p0 = nd.md_params(cutoff=2.5, skin=0.3, dt=1e-3, box_hi=(side,) * 3, atomsperleaf=4,
                      rebuild_every=REBUILD)
    t0 = time.perf_counter()
    p, _ = nd.autotune(p0, x, v, trial_steps=50, ctx=ctx)
    tune_s, tune_cached = time.perf_counter() - t0, nd.autotune.last_cached
    # the same call again: served from the tuned-settings cache
    t0 = time.perf_counter()
    p_again, _ = nd.autotune(p0, x, v, trial_steps=50, ctx=ctx)
    again_s, again_cached = time.perf_counter() - t0, nd.autotune.last_cached
    assert all(getattr(p_again, k) == getattr(p, k) for k in nd.TUNED_FIELDS)
    eng = nd.MDEngine(p, x, v, ctx=ctx)
    times = []
    for k in range(6):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(ext):
            a.record(ext)
            eng.run(steps)
            b.record(ext)
        eng.sync()
        if k >= 3:
            times.append(a.elapsed_time(b))
    d = eng.diagnostics()
    eng.close()
    # errors against FP64: forces at the input and after 100 steps, the
    # 100-step energy drift of both (truncated LJ: energy jumps where pairs
    # cross r_c, in both)
    from oracle import naiveref as R
    pr = R.md_params(cutoff=2.5, box_hi=(side,) * 3, dt=1e-3)
    e = nd.MDEngine(p, x, v, ctx=ctx)
    _, _, f0 = e.get()
    pe0, ke0 = e.energy()
    e.run(steps)
    x1, v1, f1 = e.get()
    pe1, ke1 = e.energy()
    e.close()
    g0, u0, _ = R.forces(pr, x)
    xr, vr, _ = R.md_run(pr, x, v, steps=steps)
    g1, u1, _ = R.forces(pr, x1)
    _, ur, _ = R.forces(pr, xr)
    kr = 0.5 * float((vr ** 2).sum())
    ke_0 = 0.5 * float((v ** 2).sum())
    pa = max(_force_errors(f0, g0)[0], _force_errors(f1, g1)[0])
    l2 = max(_force_errors(f0, g0)[1], _force_errors(f1, g1)[1])
    drift = abs((pe1 + ke1) - (pe0 + ke0)) / abs(pe0 + ke0)
    drift64 = abs((ur + kr) - (u0 + ke_0)) / abs(u0 + ke_0)
    errors = {"force_err_per_atom": pa, "force_err_l2": l2,
              "energy_rel": max(abs(pe0 - u0) / abs(u0), abs(pe1 - u1) / abs(u1)),
              "energy_drift_100_steps": drift, "energy_drift_100_steps_fp64": drift64,
              "max_dx_vs_fp64_100_steps": float(np.abs(x1 - xr).max()), "bar": 1e-5}
    ms = float(np.median(times))
    out = {"metric": "plain LJ atom-steps/s @4096", "unit": UNIT, "errors": errors,
           "workload": "plain_lj_4096: N=4096 uniform cube side 17 (min separation 0.8), "
                       "sigma=eps=1, r_c 2.5, skin 0.1-0.5 (autotuned), dt 1e-3, rebuild every "
                       "10, 100 steps",
           "value": n * steps / (ms * 1e-3), "ms_per_100_steps": ms,
           "tuned": {"skin": p.skin, "atomsperleaf": p.atomsperleaf,
                     "resort_every": p.resort_every, "stage_policy": p.stage_policy,
                     "union_search": UNION_NAMES[p.union_search],
                     "refit_check_every": max(p.refit_check_every, 1),
                     "threads_per_atom": p.threads_per_atom, "cta_split": p.cta_split,
                     "autotune_s": round(tune_s, 3), "autotune_from_cache": tune_cached,
                     "second_call_s": round(again_s, 4),
                     "second_call_from_cache": again_cached},
           "early_refits": d["early_refits"], "skin_violations": d["skin_violations"]}
    t0 = time.perf_counter()
    R.md_run_bvh(pr, x, v, steps=steps, rebuild=REBUILD, skin=0.3, apl=4,
                 order=R.REF_ORDER_REFERENCE)
    cs = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": n * steps / cs, "unit": UNIT, "cores": R.num_threads(),
                           "kind": "port",
                           "sample": f"the same 100 steps (leaf BVH in reference order every 10 "
                                     f"steps, FP64 forces, OpenMP), {cs:.2f} s"}
    return out


STRESS_N = 4194304


def stress_leg(nd, ctx, ext, flush, steps=3, cpu=True, points=STRESS_N):
    """Neighbour-search stress: 4,194,304 Float32 points in 64 isotropic
    Gaussian clusters (centres uniform in a cube of side 400, sigma U[2, 10]),
    r = 2.5, LBVH build + traversal + emission of the half pair list (i, j, d)
    into device memory (nd_leaf_pairs_dev, spatial order, two-phase emission),
    inputs resident, L2 flushed before each call.  cpu: the oracle's leaf-BVH
    build + order-free hash traversal of the same points on all host cores."""
    import numpy as np
    import torch

    x = nd.synth.cluster_positions(nd.synth.SEED_NS_STRESS, points, 64, 400.0, 2.0, 10.0)
    spec = nd.SpheresBVHSpecs(2.5, points, 4)
    xt = torch.from_numpy(x).cuda()
    st, cnt = nd.neighbor_pairs_dev(xt, spec, None, None, None, 0, ctx=ctx)
    pi = torch.empty(cnt, dtype=torch.int32, device="cuda")
    pj = torch.empty(cnt, dtype=torch.int32, device="cuda")
    pd = torch.empty(cnt, dtype=torch.float32, device="cuda")
    times = []
    for k in range(steps + 1):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(ext):
            a.record(ext)
            st, c2 = nd.neighbor_pairs_dev(xt, spec, pi, pj, pd, cnt, ctx=ctx)
            b.record(ext)
        torch.cuda.synchronize()
        assert st == 0 and c2 == cnt
        if k > 0:
            times.append(a.elapsed_time(b))
    h = nd.pair_hash_dev(pi, pj, pd, cnt, ctx=ctx)
    del pi, pj, pd
    torch.cuda.empty_cache()
    ms = float(np.median(times))
    out = {"metric": "neighbour-search pairs/s (LBVH build + traversal + emission)",
           "unit": "pairs/s",
           "workload": (f"ns_stress_{points}: 64 Gaussian clusters x {points // 64} Float32 points, "
                        "centres U[0,400)^3, sigma U[2,10], r 2.5, atomsperleaf 4, spatial order, "
                        "half list (i, j, d) written to device memory"),
           "value": cnt / (ms * 1e-3), "pairs": cnt, "ms_per_call": ms,
           "bytes_written_per_pair": 12, "pair_hash": [str(h[0]), str(h[1])]}
    if cpu:
        from oracle import naiveref as R
        t0 = time.perf_counter()
        t = R.tree(x, 2.5, 4, order=1)
        cnt_ref, h_ref = R.leaf_traverse_hash(t, 2.5, 4)
        cs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": cnt_ref / cs, "unit": "pairs/s", "cores": R.num_threads(),
                               "kind": "port",
                               "sample": (f"oracle leafTreeData + leafneighbor_traverse of the same "
                                          f"{points} points (pairs hashed, not stored), {cs:.2f} s")}
        out["pairs_and_hash_equal_cpu"] = bool(cnt_ref == cnt and tuple(h_ref) == tuple(h))
    return out


ADJ_N = 32768
ADJ_STEPS = 1000


def adjoint_leg(nd, ctx, ext, flush, steps=ADJ_STEPS, check_every=1):
    """Differentiable trajectory: 32,768 LJ atoms at density 0.83 (cube side
    (N/0.83)^(1/3), min separation 0.8), 1000 steps dt 1e-3, loss = squared
    deviation of the Gaussian-smoothed pair-distance histogram (64 bins on
    [0, 2.5]) from the histogram of the same seed run at sigma 1.05, eps 0.9;
    gradient wrt sigma, eps, x0, v0 with checkpoints every 50 steps.  Forward
    and backward passes timed with CUDA events on the library's stream (one
    captured graph each); the plain engine's 1000 steps on the same state are
    timed beside them.  check_every: early-refit check interval of the
    forward pass."""
    import numpy as np
    import torch

    side = (ADJ_N / 0.83) ** (1.0 / 3.0)
    x, v, _ = nd.synth.lj_system(nd.synth.SEED_ADJOINT, ADJ_N, side, 0.8)
    mp = nd.md_params(sigma=1.05, epsilon=0.9, cutoff=2.5, skin=0.3, dt=1e-3,
                      box_hi=(side,) * 3, atomsperleaf=4, rebuild_every=REBUILD, resort_every=5,
                      refit_check_every=check_every)
    adj = nd.Adjoint(mp, nd.adj_spec(steps, checkpoint_every=50), x, v, ctx=ctx)
    _, target = adj.forward()
    adj.set_params(1.0, 1.0)
    adj.set_target(target)
    adj.forward()
    adj.backward()  # captures both graphs
    fwd, bwd = [], []
    for _ in range(3):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        loss, _ = adj.forward()
        g = adj.backward()
        f_ms, b_ms = adj.times()
        fwd.append(f_ms)
        bwd.append(b_ms)
    adj.close()
    mp.sigma, mp.epsilon = 1.0, 1.0
    eng = nd.MDEngine(mp, x, v, ctx=ctx)
    eng.run(REBUILD)
    eng.sync()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush.fill_(1.0)
    torch.cuda.synchronize()
    with torch.cuda.stream(ext):
        a.record(ext)
        eng.run(steps)
        b.record(ext)
    eng.sync()
    plain_ms = a.elapsed_time(b)
    eng.close()
    f_ms, b_ms = float(np.median(fwd)), float(np.median(bwd))
    return {"metric": "adjoint step time / forward step time", "unit": "ratio",
            "workload": (f"adjoint_32768: N={ADJ_N} LJ, cube side {side:.2f} (density 0.83), "
                         f"{steps} steps dt 1e-3, histogram loss (64 bins on [0, 2.5], "
                         "Gaussian width = bin width) vs the sigma 1.05 / eps 0.9 run, "
                         "checkpoints every 50 steps, skin 0.3, rebuild every 10"),
            "refit_check_every": check_every,
            "value": b_ms / f_ms, "forward_ms_per_step": f_ms / steps,
            "adjoint_ms_per_step": b_ms / steps,
            "plain_engine_ms_per_step": plain_ms / steps,
            "adjoint_over_plain_forward": (b_ms / steps) / (plain_ms / steps),
            "loss": loss, "dL_dsigma": g["sigma"], "dL_depsilon": g["epsilon"],
            "dL_dx0_norm": float(np.linalg.norm(g["x0"])),
            "target": "<= 3 (adjoint step vs forward step)"}


def run_gb300(args):
    import numpy as np
    import torch
    import naivedynamics as nd

    from naivedynamics import replicas

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    ctx = nd.Context(local)
    ext = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))

    x, v, q = nd.synth.lj_system(SEED + rank, N_ATOMS, SIDE, 0.8, charges=True)
    xd = torch.from_numpy(x).cuda()
    vd = torch.from_numpy(v).cuda()
    qd = torch.from_numpy(q).cuda()
    # engine settings (skin, leaf width, re-sort interval, staging) from the
    # library's autotuner on this state, outside the timed region
    t0 = time.perf_counter()
    params, _ = nd.autotune(_md_params(nd), x, v, q, trial_steps=50, ctx=ctx)
    tune_s, tune_cached = time.perf_counter() - t0, nd.autotune.last_cached
    eng = nd.MDEngine(params, xd, vd, qd, device=True, ctx=ctx)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        ctx.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        eng.run(MD_PER_STEP)
    eng.sync()

    # ---- timed region: K bench steps, L2 flushed before each (outside the events)
    events = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
    launches0 = ctx.launch_count()
    diag0 = eng.diagnostics()
    barrier()
    wall0 = time.perf_counter()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.fill_(float(k))
            torch.cuda.synchronize()
            with torch.cuda.stream(ext):
                events[k][0].record(ext)
                eng.run(MD_PER_STEP)
                events[k][1].record(ext)
        eng.sync()
        barrier()
    wall = time.perf_counter() - wall0
    diag = eng.diagnostics()
    early = diag["early_refits"] - diag0["early_refits"]
    # kernel nodes of the launched graphs plus the kernels of the conditional
    # rebuild bodies that ran
    launches = (ctx.launch_count() - launches0 + diag["body_kernels"] - diag0["body_kernels"])
    t_ms = sum(s.elapsed_time(e) for (s, e) in events)
    t_max = replicas.max_over_ranks(t_ms)  # the job's time: its slowest replica's
    stats = eng.stats()

    # ---- roofline of the dominant kernel: k_md_step launches each bracketed
    # by a pair of CUDA events on the library's stream (nd_md_step_times: ten
    # windows run eagerly, the same kernels and rebuild decisions as the
    # captured graphs -- and the launches an ncu launch list can see, since
    # ncu does not profile kernel nodes of graphs with conditional nodes)
    k_ms = float(statistics.mean(eng.step_times(10 * REBUILD)))
    nbr = stats["list_pairs"] / N_ATOMS  # full-list neighbours per atom
    # algorithmic bytes per atom of one fused step: x, v read+write (FP64, 96),
    # own fixed-point record read (16) + next record write (16), force write
    # (16), build-position read (16), list count (4), 2 B per listed neighbour
    # (uint16 index into the block's staged union)
    bytes_per_atom = 96 + 16 + 16 + 16 + 16 + 4 + 2 * nbr
    traffic_alg = bytes_per_atom * N_ATOMS
    peaks, peak_kind = _peaks()
    achieved = traffic_alg / (k_ms * 1e-3) / 1e9
    traffic = _ncu_traffic()

    # ---- e2e: simulate!(sys, spec, clct) through the public API with pinned
    # host buffers: H2D of x, v, q and D2H of x, v, f inside every step
    xh = torch.from_numpy(x.copy()).pin_memory()
    vh = torch.from_numpy(v.copy()).pin_memory()
    qh = torch.from_numpy(q.copy()).pin_memory()
    fh = torch.empty((N_ATOMS, 3), dtype=torch.float32).pin_memory()
    import ctypes
    from naivedynamics import _lib
    L = _lib.lib()

    def e2e_call():
        st = L.nd_simulate(ctx.handle, ctypes.byref(params), N_ATOMS, xh.data_ptr(),
                           vh.data_ptr(), fh.data_ptr(), qh.data_ptr(), None, MD_PER_STEP)
        ctx.check(st, "nd_simulate")

    for _ in range(max(1, args.warmup)):
        e2e_call()
    barrier()
    e2e_t = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_call()
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = replicas.max_over_ranks(sum(e2e_t))

    total_atom_steps = ws * N_ATOMS * MD_PER_STEP * args.steps
    value = total_atom_steps / (t_max * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair math, f64 state",
        "data": "synthetic (seeded splitmix64 generators)",
        "config": CONFIG,
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                     "traffic": traffic, "kernel": "k_md_step (fused force + KDK step)",
                     "kernel_ms": k_ms, "algorithmic_bytes_per_launch": traffic_alg,
                     "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"},
        "e2e": {"value": total_atom_steps / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": int(x.nbytes + v.nbytes + q.nbytes),
                "d2h_bytes_per_step": int(x.nbytes + v.nbytes + fh.numel() * 4),
                "api": "nd_simulate (simulate!) with pinned host buffers"},
        "engine": {"md_steps_per_step": MD_PER_STEP,
                   "atom_order": f"3-D Hilbert, re-sorted every {params.resort_every}th rebuild, "
                                 "refit between",
                   "tuned": {"skin": params.skin, "atomsperleaf": params.atomsperleaf,
                             "resort_every": params.resort_every,
                             "stage_policy": params.stage_policy,
                             "union_search": UNION_NAMES[params.union_search],
                             "refit_check_every": max(params.refit_check_every, 1),
                             "threads_per_atom": params.threads_per_atom,
                             "autotune_s": round(tune_s, 2),
                             "autotune_from_cache": tune_cached},
                   "parallelism": f"replicas x{ws}" if ws > 1 else "1 GPU",
                   "neighbours_per_atom": round(nbr, 2),
                   "skin_violations": diag["skin_violations"],
                   "early_refits_timed": early,
                   "resorts_timed": diag["resorts"] - diag0["resorts"],
                   "refits_timed": diag["refits"] - diag0["refits"],
                   "wall_s_timed_region": round(wall, 4)},
    }
    clocks = clk.summary()
    if clocks:
        line["clocks"] = clocks
    if diag["skin_violations"] > 0:
        print(f"warning: {diag['skin_violations']} atom-steps ran on lists an atom had left by "
              "more than skin/2", file=sys.stderr)
    errors = {}
    if rank == 0:
        errors["lj_coulomb_262144"] = headline_errors(nd, eng, x, q)
    eng.close()
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample()
    b = None
    if not args.no_batched:
        b = batched_leg(nd, ctx, ext, flush)  # every rank runs its share of the systems
    if rank == 0 and not args.no_plain:
        line["plain_lj_4096"] = plain_leg(nd, ctx, ext, flush)
        errors["plain_lj_4096"] = line["plain_lj_4096"].pop("errors")
    if rank == 0 and not args.no_adjoint:
        line["adjoint"] = adjoint_leg(nd, ctx, ext, flush, steps=args.adjoint_steps,
                                      check_every=args.adjoint_check_every)
    if rank == 0 and not args.no_stress:
        line["ns_stress"] = stress_leg(nd, ctx, ext, flush, cpu=not args.no_cpu_baseline)
    if rank == 0 and not args.no_compat:
        line["compat_simulate"] = compat_leg(nd, ctx, ext, flush, cpu=not args.no_cpu_baseline)
    if rank == 0:
        # the per-result errors and the batched result last, compact, so that
        # the end of the line carries them
        if b is not None:
            errors["ensemble_512"] = b.pop("errors")
        line["errors_vs_fp64"] = errors
        if b is not None:
            # the ensemble's own FP64 force errors beside its speed-up
            b["force_err_vs_fp64"] = {k: errors["ensemble_512"][k]
                                      for k in ("force_err_per_atom", "force_err_l2")}
            line["batched"] = b
        print(json.dumps(_plain(line)), flush=True)
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def _force_errors(f32, f64):
    """(max_i |dF_i| / max(|F64_i|, 1e-3 rms|F64|), |dF|_2 / |F64|_2)."""
    import numpy as np
    df = np.linalg.norm(np.asarray(f32, np.float64) - f64, axis=1)
    nf = np.linalg.norm(f64, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(nf ** 2))
    return (float(np.max(df / np.maximum(nf, floor))),
            float(np.linalg.norm(df) / np.linalg.norm(f64)))


def headline_errors(nd, eng, x0, q):
    """Force and energy errors of the headline engine against the FP64 oracle:
    at the bench's input (a fresh engine with the same settings) and at the
    state the timed steps left."""
    from oracle import naiveref as R
    p = R.md_params(coulomb_k=1.0, cutoff=2.5, box_hi=(SIDE,) * 3, dt=1e-3)
    x1, _, f1 = eng.get()
    pe1, _ = eng.energy()
    f64, u64, _ = R.forces(p, x1, q)
    pa1, l21 = _force_errors(f1, f64)
    import numpy as np
    e = nd.MDEngine(eng.params, x0, np.zeros_like(x0), q, ctx=eng.ctx)
    _, _, f0 = e.get()
    pe0, _ = e.energy()
    e.close()
    g64, v64, _ = R.forces(p, x0, q)
    pa0, l20 = _force_errors(f0, g64)
    return {"force_err_per_atom": max(pa0, pa1), "force_err_l2": max(l20, l21),
            "energy_rel": max(abs(pe0 - v64) / abs(v64), abs(pe1 - u64) / abs(u64)),
            "at": "input and end of the timed steps", "bar": 1e-5}


def md_eager_leg(nd, ctx, union_search="blocks", check_every=3, skin=0.4, apl=4,
                 stage_policy=0):
    """The headline workload with the settings the autotuner picks for it
    (by default skin 0.4, 4 atoms per leaf, re-sort every 10th window; the
    given union search and early-refit check interval), created and run for
    ten windows eagerly (nd_md_step_times), so that every kernel is a plain
    launch in a known order for profiling: engine creation (three builds),
    then per window a rebuild and ten steps."""
    import numpy as np

    import torch

    x, v, q = nd.synth.lj_system(SEED, N_ATOMS, SIDE, 0.8, charges=True)
    p = _md_params(nd)
    p.skin, p.atomsperleaf, p.resort_every = skin, apl, 10
    p.stage_policy = stage_policy
    p.union_search = {v_: k for k, v_ in UNION_NAMES.items()}[union_search]
    p.refit_check_every = check_every
    eng = nd.MDEngine(p, x, v, q, ctx=ctx)
    ms = eng.step_times(10 * REBUILD)
    # then the same settings through the captured graphs, CUDA events
    ext = torch.cuda.ExternalStream(ctx.stream)
    graph_ms = []
    for k in range(4):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(ext):
            a.record(ext)
            eng.run(MD_PER_STEP)
            b.record(ext)
        eng.sync()
        if k > 0:
            graph_ms.append(a.elapsed_time(b))
    d = eng.diagnostics()
    nbr = eng.stats()["list_pairs"] / N_ATOMS
    eng.close()
    return {"workload": WORKLOAD + f" (fixed settings: skin {skin}, {apl} atoms per leaf, "
                                   f"union search {union_search}, early-refit checks every "
                                   f"{check_every} steps)",
            "neighbours_per_atom": round(nbr, 2),
            "early_refits": d["early_refits"], "skin_violations": d["skin_violations"],
            "step_kernel_ms_mean": float(np.mean(ms)),
            "graph_ms_per_100_steps": float(np.median(graph_ms)),
            "atom_steps_per_s": N_ATOMS * MD_PER_STEP / (float(np.median(graph_ms)) * 1e-3)}


def run_only(args):
    import torch
    import naivedynamics as nd

    torch.cuda.set_device(0)
    ctx = nd.Context(0)
    ext = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", 0))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    if args.only == "md":
        out = md_eager_leg(nd, ctx, union_search=args.union_search,
                           check_every=args.check_every, skin=args.skin, apl=args.apl,
                           stage_policy=args.stage_policy)
    elif args.only == "plain":
        out = plain_leg(nd, ctx, ext, flush)
    elif args.only == "batched":
        out = batched_leg(nd, ctx, ext, flush)
    elif args.only == "adjoint":
        out = adjoint_leg(nd, ctx, ext, flush, steps=args.adjoint_steps,
                          check_every=args.adjoint_check_every)
    elif args.only == "compat":
        out = compat_leg(nd, ctx, ext, flush, cpu=not args.no_cpu_baseline)
    else:
        out = stress_leg(nd, ctx, ext, flush, cpu=not args.no_cpu_baseline,
                         points=args.stress_points)
    print(json.dumps(_plain(out)), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30,
                    help="timed bench steps (100 MD steps each: 30 span about a quarter of a "
                         "second, several clock samples; the reference arm times one 10-step "
                         "CPU sample per bench step)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched-ensemble measurement")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the adjoint (differentiable trajectory) measurement")
    ap.add_argument("--adjoint-steps", type=int, default=ADJ_STEPS,
                    help="MD steps of the adjoint measurement (a multiple of 50)")
    ap.add_argument("--adjoint-check-every", type=int, default=1,
                    help="early-refit check interval of the adjoint's forward pass")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the 4,096-atom plain LJ measurement")
    ap.add_argument("--no-stress", action="store_true",
                    help="skip the neighbour-search stress measurement")
    ap.add_argument("--stress-points", type=int, default=STRESS_N,
                    help="points of the stress measurement with --only stress (64 clusters)")
    ap.add_argument("--union-search", choices=["blocks", "tree"], default="blocks",
                    help="union search of the fixed-settings engine of --only md")
    ap.add_argument("--check-every", type=int, default=3,
                    help="early-refit check interval of the fixed-settings engine of --only md")
    ap.add_argument("--skin", type=float, default=0.4,
                    help="skin of the fixed-settings engine of --only md")
    ap.add_argument("--apl", type=int, default=4,
                    help="atoms per leaf of the fixed-settings engine of --only md")
    ap.add_argument("--stage-policy", type=int, default=0, choices=[0, 1],
                    help="union staging of the fixed-settings engine of --only md "
                         "(0: near the mean union, 1: every union record)")
    ap.add_argument("--no-compat", action="store_true",
                    help="skip the simulate!-as-written measurement")
    ap.add_argument("--only", choices=["md", "plain", "batched", "adjoint", "stress", "compat"],
                    help="run one secondary measurement alone and print its JSON object "
                         "(for profiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.only:
        run_only(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
