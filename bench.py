"""Benchmark: body-steps/s of the full rigid-body step on GB300.

Workloads (--config), seeded synthetic scenes of the stated sizes:
  batched  (default) 1024 independent joint + contact scenes (body counts
           log-uniform in [16, 2048]; rope / ball-socket / spring chains and
           0-200 loose boxes on the ground), dt 1/60, 10 AVBD iterations,
           packed into one device world
  pyramid  10-level pyramid of 55 unit cubes, dt 1/60, 10 iterations, up to
           8 contacts per pair
  field    32 x 32 x 8 cube field dropped on the ground, dt 1/60, 10 iterations
  pile     50,000 mixed convex bodies (boxes, 42-vertex hulls, tetrahedra),
           dt 1/120, 12 iterations
  wall     400 x 500-brick wall at x = 1e5 m and 1000 spheres, dt 1/120,
           15 iterations, FP32/FP64 split precision
Each step is dio_step: broad -> narrow -> rows + warm start -> solve.

One JSON line on rank 0:
  value      body-steps/s with the world resident in HBM (CUDA events on the
             library's stream, K steps, max over ranks)
  e2e        the same metric through the public API with pinned host buffers:
             every step re-uploads poses + state (dio_world_set_state) and
             reads poses + state back (dio_world_download); timed with the
             batch as one world and as several worlds on several streams
             (dio_worlds_step_host), the faster reported
  per_phase  the same K steps with the solve launched per phase (init,
             primal / dual per iteration, recover) instead of one scene-chunk
             launch, and the primal kernel's roofline
  plain      the one-scene-per-launch path (one context per scene) on a
             sample of scenes, for the batched-vs-plain ratio
  roofline   the dominant solve kernel: algorithmic bytes per launch / event
             time
  fp64_error position / angle error of the FP32 and split worlds against an
             all-FP64 world after --error-steps steps, per content class,
             beside the chaos floor (FP64 from positions nudged by one FP32
             ulp against FP64)
  cpu_baseline  the CPU oracle (OpenMP over bodies / rows) on the same
             workload
--impl reference times the CPU restatement of the reference path on the
same workload (the reference is Rust + Vulkan; neither toolchain nor a
Vulkan device exists here).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "body-steps/s at 10 iters, batched vs plain on 1 GB300; max pos err vs FP64 (m)"

# workload -> (description, precision, contacts per pair, pairs / rows per body of the capacity)
CONFIGS = {
    "batched": ("batched {scenes} scenes (rope / ball-socket / spring chains + loose boxes), dt 1/60, "
                "10 iterations", "f32", 4, (2, 4)),
    "pyramid": ("10-level pyramid of 55 unit cubes on the ground, dt 1/60, 10 iterations, up to 8 contacts "
                "per pair", "f32", 8, (64, 200)),
    "field": ("32 x 32 x 8 cube field (side 0.5 m, random orientations) dropped on the ground, dt 1/60, "
              "10 iterations", "f32", 4, (24, 24)),
    "pile": ("mixed convex pile of 50,000 bodies (40% boxes, 40% 42-vertex hulls, 20% tetrahedra), dt 1/120, "
             "12 iterations", "f32", 4, (16, 32)),
    "wall": ("wall throw: 400 x 500 bricks at x = 1e5 m + 1000 spheres at 30 m/s, dt 1/120, 15 iterations, "
             "FP32 Hessian / FP64 poses", "split", 4, (8, 16)),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="batched", choices=sorted(CONFIGS))
    ap.add_argument("--scenes", type=int, default=1024)
    ap.add_argument("--strong", action="store_true",
                    help="N > 1: shard one batch across the ranks (strong scaling) instead of a batch per rank")
    ap.add_argument("--plain-scenes", type=int, default=128)
    ap.add_argument("--error-steps", type=int, default=600,
                    help="steps of the FP32 / split / FP64 error study (capped by the workload's own step count)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-worlds", type=int, default=8,
                    help="e2e: the batch as this many worlds on as many streams (dio_worlds_step_host)")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-f64", action="store_true")
    ap.add_argument("--no-per-phase", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default configuration (profiling runs)")
    ap.add_argument("--block-size", type=int, default=None, choices=[0, 640],
                    help="threads per CTA of the scene-chunk solve (0: 512); default: the autotuner's choice")
    ap.add_argument("--primal-variant", type=int, default=None,
                    help="primal kernel variant of the per-phase solve; default: the autotuner's choice")
    ap.add_argument("--colored", action="store_true",
                    help="coloured Gauss-Seidel solver mode instead of the reference's Jacobi schedule")
    ap.add_argument("--per-phase", action="store_true",
                    help="time the per-phase solve launches as the headline (profiling the primal kernel)")
    ap.add_argument("--save-state", default=None, metavar="PATH",
                    help="after the timed region, write the world as a checkpoint image")
    ap.add_argument("--load-state", default=None, metavar="PATH",
                    help="resume the world from a checkpoint image before the warm-up (profiling a late step)")
    ap.add_argument("--precision", default=None, choices=["f32", "split"],
                    help="arithmetic of the timed world (split: FP64 poses / lambda, FP32 Hessian); "
                         "default: the workload's own")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.samples = []
        self.idx = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, nm in enumerate(names):
                if len(s) > 5 + k and s[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def measured_hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_workload(args, rank, world):
    """The rank's scenes and the scaling mode.  batched: a batch of
    args.scenes scenes per rank (weak scaling: rank r steps sub-batch r of
    the N-batch workload), or with --strong one batch sharded across the
    ranks by cost (dio_dist.shard_scenes).  Single-scene workloads run one
    replica per rank."""
    from diomedes_gb300 import dist as dio_dist
    from diomedes_gb300 import scenes

    if args.config == "batched":
        if args.strong and world > 1:
            full = scenes.batched(n_scenes=args.scenes)
            mine = dio_dist.shard_scenes(dio_dist.scene_costs(full.scene_offsets, full.constraints), world)[rank]
            return full.select(mine), "strong"
        return scenes.batched(n_scenes=args.scenes, seed=4 + 1000 * rank), "weak"
    make = {"pyramid": lambda: scenes.pyramid(levels=10), "field": lambda: scenes.cube_field(nx=32, nz=32, ny=8),
            "pile": lambda: scenes.mixed_pile(n=50000), "wall": lambda: scenes.wall_throw(cols=400, rows=500)}
    return make[args.config](), "weak"


def world_capacity(sc, per_body=(2, 4)):
    from diomedes_gb300 import compute

    # overflow is reported (DIO_ERR_CAPACITY), never dropped; the batched
    # scenes carry ~0.6 rows and ~0.01 pairs per body
    n = sc.n
    return compute.capacity(n, max_pairs=max(1024, per_body[0] * n), max_contacts=max(4096, per_body[1] * n),
                            max_joints=max(1, len(sc.constraints)), max_scenes=sc.n_scenes,
                            max_hull_vertices=max(1, 0 if sc.hull_vertices is None else len(sc.hull_vertices)))


def primal_bytes(n_dyn, m, j_inc):
    """Compulsory bytes of one primal launch (SoA FP32 model): per dynamic body
    132 B (snapshot, initial, inertial, inverse mass/moment, CSR offset, new
    pose), per contact row 108 B + two 4-byte CSR entries, per joint
    incidence 44 B + 4 B."""
    return 132 * n_dyn + (108 + 8) * m + 48 * j_inc


def chunk_solve_bytes(n, m, j_inc):
    """Compulsory bytes of one scene-chunk solve launch (the whole step's
    init, iterations and recover; every array element read or written once):
    per body 152 B (pose, velocities, inverse mass / moment and the two CSR
    offsets read; pose and velocities written), per contact row 148 B (row
    payload, friction and bodies read, lambda / penalty written, two CSR
    entries of 8 B), per joint incidence 48 B."""
    return 152 * n + 148 * m + 48 * j_inc


def iteration_bytes(n_dyn, m, j_inc):
    """The per-iteration compulsory model of a per-phase solve, which re-reads
    every pose and row each iteration: 188 N + 248 M + 52 J (J joints, two
    incidences each)."""
    return 188 * n_dyn + 248 * m + 26 * j_inc


# DRAM traffic of one k_primal launch over its algorithmic bytes, from one ncu
# capture at the timed state (the world saved after 310 steps and resumed:
# dram__bytes_read.sum + dram__bytes_write.sum of one launch, 117.95 MB,
# against 110.81 MB for its 219,619 contact rows).  The timed launches are
# reported at this ratio of their own algorithmic bytes.
PRIMAL_TRAFFIC_RATIO = 117.95 / 110.81


def primal_gather_bytes(n_dyn, pair_rows, cont_rows, j_inc):
    """Gather-inclusive upper bound of one primal launch: the compulsory bytes
    plus, per row incidence, the row payload and CSR entries again and the
    other body's snapshot and step-start pose (64 B, SoA float4) for pair
    rows; per joint incidence the 48 B joint view and the other body's
    snapshot pose (32 B)."""
    incid = 2 * pair_rows + cont_rows
    return 132 * n_dyn + incid * (108 + 8) + 2 * pair_rows * 64 + j_inc * (48 + 32)


def run_cpu(sc, steps, warmup, threads, budget_s=20.0, contacts_per_pair=4):
    """CPU oracle (f32) on a scene: body-steps/s over the steps after
    `warmup` untimed ones (stops early at the time budget)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as O

    w = O.World(sc, threads=threads, contacts_per_pair=contacts_per_pair)
    w.step(sc.options, warmup)
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        w.step(sc.options, 1)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return sc.n * done / dt, done, dt


def workload_config(args, sc, scaling, world):
    desc = CONFIGS[args.config][0].format(scenes=sc.n_scenes)
    return {"workload": desc, "bodies_per_gpu": sc.n, "scenes_per_gpu": sc.n_scenes, "joints": len(sc.constraints),
            "l2": "working set > L2 (129 MB)" if sc.n > 100_000 else "working set within L2 (129 MB)",
            "parallelism": f"scene-sharded x{world} ({scaling})" if args.config == "batched"
            else f"replicas x{world}"}


def reference_arm(args, rank, world):
    """The reference's path on the host cores: the CPU restatement (the
    reference itself is Rust + Vulkan), on this arm's workload, W untimed
    steps then up to K timed steps within a time budget."""
    if rank != 0:
        return
    sc, scaling = make_workload(args, 0, 1)
    threads = os.cpu_count() or 1
    v, done, dt = run_cpu(sc, max(1, args.steps), max(0, args.warmup), threads, budget_s=90.0,
                          contacts_per_pair=CONFIGS[args.config][2])
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "body-steps/s", "n_gpus": args.gpus,
        "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(1, done), "higher_is_better": True,
        "scaling": scaling, "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, sc, scaling, world),
        "cpu_baseline": {"value": v, "unit": "body-steps/s", "cores": threads, "kind": "port",
                         "sample": f"the whole workload ({sc.n} bodies), {done} steps after {args.warmup} "
                                   "untimed ones"},
        "e2e": {"value": v, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def body_classes(sc):
    """Dynamic bodies grouped by content: for joint scenes by the kind of
    joint they hang on (rope, ball-socket, spring, rod) or loose; otherwise
    by shape."""
    from diomedes_gb300 import abi

    dyn = sc.state["inv_mass"] != 0
    cls = {}
    if len(sc.constraints):
        kinds = {0: "spring", 1: "rod", 2: "ball_socket", 3: "rope"}
        tag = np.full(sc.n, -1, np.int64)
        for k in kinds:
            c = sc.constraints[sc.constraints["kind"] == k]
            tag[c["a"]] = k
            tag[c["b"]] = k
        for k, name in kinds.items():
            idx = np.flatnonzero(dyn & (tag == k))
            if len(idx):
                cls[name] = idx
        loose = np.flatnonzero(dyn & (tag < 0))
        if len(loose):
            cls["loose_box"] = loose
    else:
        shapes = {abi.SPHERE: "sphere", abi.CUBE: "cube", abi.TETRAHEDRON: "tetrahedron", abi.BOX: "box",
                  abi.HULL: "hull"}
        for t, name in shapes.items():
            idx = np.flatnonzero(dyn & (sc.bodies["shape"]["tag"] == t))
            if len(idx):
                cls[name] = idx
    cls["all"] = np.flatnonzero(dyn)
    return cls


def error_study(sc, o, steps, cap, cpp, tuned):
    """FP32, split and all-FP64 worlds stepped `steps` from the same initial
    state, plus the chaos floor: an FP64 world whose dynamic bodies' initial
    positions are nudged by one FP32 ulp.  Max / median position error (m)
    and max angle error (rad) per content class against the FP64 world."""
    from diomedes_gb300 import compute

    pos0 = sc.positions_f64 if sc.positions_f64 is not None else sc.bodies["position"][:, :3].astype(np.float64)
    dyn = sc.state["inv_mass"] != 0
    nudged = pos0.copy()
    nudged[dyn] = pos0[dyn] + np.spacing(pos0[dyn].astype(np.float32)).astype(np.float64)

    from diomedes_gb300 import abi

    def run(precision, positions_f64=None, horizon=None):
        """Step to `horizon` (or as far as the capacity lets the world go, in
        blocks of 25 steps, when horizon is None); returns the poses and the
        steps done."""
        kw = sc.upload_kwargs()
        if positions_f64 is not None:
            kw["positions_f64"] = positions_f64
        w = compute.World(cap, precision=precision, contacts_per_pair=cpp, **tuned)
        w.upload(sc.bodies, sc.state, **kw)
        done, last = 0, None
        target = steps if horizon is None else horizon
        while done < target:
            k = min(25, target - done)
            try:
                w.step(o, k)
            except abi.DioError as e:
                if e.status not in (abi.DIO_ERR_CAPACITY, abi.DIO_ERR_NONFINITE) or horizon is not None:
                    raise
                break
            done += k
            last = w.download_f64()
        w.close()
        return last, done

    worlds = {"fp64": (2, None), "fp32": (0, None), "split": (1, None), "chaos_floor": (2, nudged)}
    got = {name: run(prec, pos) for name, (prec, pos) in worlds.items()}
    horizon = min(done for _, done in got.values())
    if horizon == 0:
        return {"steps": 0, "horizon_note": "a world outgrew its capacity or went non-finite within 25 steps"}
    for name, (prec, pos) in worlds.items():  # worlds that went further: again, to the common horizon
        if got[name][1] != horizon:
            got[name] = run(prec, pos, horizon)
    p64, q64 = got["fp64"][0]
    runs = {k: got[k][0] for k in ("fp32", "split", "chaos_floor")}

    def ang(q):
        c = np.abs((q * q64).sum(axis=1))
        return 2.0 * np.arccos(np.clip(c, 0.0, 1.0))

    out = {"steps": horizon, "classes": {}}
    if horizon < steps:
        out["horizon_note"] = (f"a world outgrew its pair / row capacity or went non-finite after {horizon} of "
                               f"{steps} steps (the stack compresses, candidate pairs multiply); errors at that step")
    for name, idx in body_classes(sc).items():
        row = {"bodies": int(len(idx))}
        for k, (p, q) in runs.items():
            e = np.abs(p[idx] - p64[idx]).max(axis=1)
            row[k] = {"max_pos_err_m": float(e.max()), "median_pos_err_m": float(np.median(e)),
                      "max_angle_err_rad": float(ang(q)[idx].max())}
        out["classes"][name] = row
    allc = out["classes"]["all"]
    out["max_pos_err_m"] = allc["split"]["max_pos_err_m"]
    out["median_pos_err_m"] = allc["split"]["median_pos_err_m"]
    out["fp32_max_pos_err_m"] = allc["fp32"]["max_pos_err_m"]
    out["chaos_floor_max_pos_err_m"] = allc["chaos_floor"]["max_pos_err_m"]
    return out


def tuned_config(w):
    c = w.configure()
    return {"primal_variant": c.primal_variant, "bvh_rebuild_period": c.bvh_rebuild_period,
            "batched_solver": c.batched_solver, "block_size": c.block_size}


def main():
    args = parse()
    if args.load_state:
        args.no_f64 = True  # the FP64 comparison steps from the initial state
    rank, world, local = dist_info()
    if args.impl == "reference":
        return reference_arm(args, rank, world)

    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    from diomedes_gb300 import abi, compute
    from diomedes_gb300 import dist as dio_dist

    sc, scaling = make_workload(args, rank, world)
    _, default_prec, cpp, per_body = CONFIGS[args.config]
    prec = 1 if (args.precision or default_prec) == "split" else 0
    cap = world_capacity(sc, per_body)
    stream = torch.cuda.current_stream()
    w = compute.World(cap, profile=0, precision=prec, contacts_per_pair=cpp)
    w.set_stream(stream.cuda_stream)
    w.upload(sc.bodies, sc.state, **sc.upload_kwargs())
    if args.load_state:
        with open(args.load_state, "rb") as f:
            w.resume(f.read())
    o = sc.options
    # the warm-up in two parts: the tuner times its candidates from the state
    # the first part reaches (and restores it), the last three steps capture
    # the chosen configuration's step graphs
    w_pre = max(0, args.warmup - 3)
    if w_pre:
        w.step(o, w_pre)
    if not args.no_tune:
        # solve launch, CTA size / launch shape, LBVH rebuild period; state restored
        w.autotune(o, trial_steps=16)
    if args.per_phase:
        w.configure(batched_solver=abi.SOLVE_PER_PHASE)
    if args.block_size is not None:
        w.configure(block_size=args.block_size)
    if args.primal_variant is not None:
        w.configure(primal_variant=args.primal_variant)
    if args.colored:
        w.configure(solver_mode=abi.SOLVER_COLORED)
    tuned = tuned_config(w)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # the clock sampler starts with the warm-up so that its 50 ms samples
    # cover the (sub-second) timed region
    with Clocks(local) as clk:
        w.step(o, args.warmup - w_pre)
        torch.cuda.synchronize()
        w.reset_timers()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        w.step(o, args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    st = w.stats()
    if args.save_state:
        with open(args.save_state, "wb") as f:
            f.write(w.checkpoint())
    state_after = w.checkpoint()  # the passes below start from the state the timed steps reached

    # a second pass of the same K steps with the per-phase / per-launch event
    # timers on (they add an event pair per span, so the headline pass above
    # runs without them): phase split and the solve kernel's launch duration
    w.configure(profile=1)
    w.step(o, 3)
    torch.cuda.synchronize()
    w.reset_timers()
    q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    q0.record(stream)
    w.step(o, args.steps)
    q1.record(stream)
    torch.cuda.synchronize()
    stp = w.stats()
    ms_profiled = q0.elapsed_time(q1)
    w.configure(profile=0)

    # max time over ranks, body-steps summed over ranks (each rank owns its scenes)
    ms_max, body_steps = dio_dist.frame(dist, ms, sc.n * args.steps, device="cuda")
    n_dyn = int((sc.state["inv_mass"] != 0).sum())
    value = body_steps / (ms_max / 1e3)
    peak, peak_kind = measured_hbm_peak()
    j_inc = 2 * len(sc.constraints)
    rows_now = w.contacts()
    cont_rows = int((rows_now["b"] == 0xFFFFFFFF).sum())
    m_now = int(stp["contacts"])

    def primal_roofline(s):
        prim_ms = s["primal_ms"] / max(1, s["primal_launches"])
        pb = primal_bytes(n_dyn, s["contacts"], j_inc)
        pg = primal_gather_bytes(n_dyn, len(rows_now) - cont_rows, cont_rows, j_inc)
        ach = pb / (prim_ms / 1e3) / 1e9 if prim_ms > 0 else None
        return {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak if ach else None,
                "traffic": PRIMAL_TRAFFIC_RATIO * pb,
                "traffic_source": "ncu DRAM bytes of one launch at the timed state (step 310), scaled by "
                                  "algorithmic bytes",
                "kernel": "k_primal", "bytes_per_launch": pb, "avg_launch_ms": prim_ms, "peak_kind": peak_kind,
                "gather_bytes_per_launch": pg,
                "achieved_gather": pg / (prim_ms / 1e3) / 1e9 if prim_ms > 0 else None}

    if stp["chunk_launches"]:
        chunk_ms = stp["chunk_ms"] / stp["chunk_launches"]
        cb = chunk_solve_bytes(sc.n, m_now, j_inc)
        ach = cb / (chunk_ms / 1e3) / 1e9
        it_b = iteration_bytes(n_dyn, m_now, j_inc) * int(o.iterations)
        roofline = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                    "traffic": None, "kernel": "k_solve_chunks", "bytes_per_launch": cb, "avg_launch_ms": chunk_ms,
                    "peak_kind": peak_kind,
                    "limiter": "SM issue, not HBM: poses stay in shared memory across the iterations, rows and "
                               "joint views are re-read from L1 / L2",
                    "per_phase_equivalent_bytes": it_b,
                    "per_phase_equivalent_GBs": it_b / (chunk_ms / 1e3) / 1e9}
    else:
        roofline = primal_roofline(stp)

    # the same K steps from the same state with the solve launched per
    # phase (init, primal / dual per iteration, recover): the primal
    # kernel's roofline and the gain of the one-launch solve
    per_phase = None
    if stp["chunk_launches"] and not args.no_per_phase:
        w.resume(state_after)
        w.configure(batched_solver=abi.SOLVE_PER_PHASE)
        w.step(o, 3)
        torch.cuda.synchronize()
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r0.record(stream)
        w.step(o, args.steps)
        r1.record(stream)
        torch.cuda.synchronize()
        pp_ms = r0.elapsed_time(r1)
        w.configure(profile=1)
        w.step(o, 3)
        torch.cuda.synchronize()
        w.reset_timers()
        w.step(o, args.steps)
        torch.cuda.synchronize()
        spp = w.stats()
        w.configure(profile=0, batched_solver=tuned["batched_solver"])
        per_phase = {"value": sc.n * args.steps / (pp_ms / 1e3), "ms_per_step": pp_ms / args.steps,
                     "roofline": primal_roofline(spp),
                     "phase_ms_per_step": {k: spp[f"{k}_ms"] / args.steps
                                           for k in ("broad", "narrow", "rows", "solve", "primal", "dual")}}

    # end to end through the public API with host buffers: the demos'
    # per-frame loop (upload poses + velocities, step, read them back), with
    # the 64-byte motion records (shapes, masses and joints stay on the
    # device); the same loop with the full body + state records beside it
    e2e = None
    if not args.no_e2e:
        w.resume(state_after)

        def pinned(dtype, count):  # the caller's page-locked host array (cudaHostAlloc through torch)
            return torch.empty(count * dtype.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(dtype)

        hm = pinned(abi.MOTION, sc.n)
        w.download_motion_into(hm)
        k2 = max(3, args.steps // 2)
        # (1) the batch as one world: set_motion, dio_step, download_motion in series
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(k2):
            w.set_motion(hm)
            w.step(o, 1)
            w.download_motion_into(hm)
        t1 = time.perf_counter()
        single = sc.n * k2 / (t1 - t0)
        # (2) the same batch as G worlds (contiguous runs of whole scenes) on
        # G streams: one world's host copies overlap the other worlds' steps
        piped, piped_full, parts = 0.0, 0.0, [sc]
        if sc.n_scenes > 1:
            parts, starts = sc.split(args.e2e_worlds)
            worlds, streams = [], []
            for p, lo in zip(parts, starts):
                wg = compute.World(world_capacity(p, per_body), profile=0, precision=prec, contacts_per_pair=cpp)
                streams.append(torch.cuda.Stream())
                wg.set_stream(streams[-1].cuda_stream)
                wg.upload(p.bodies, p.state, **p.upload_kwargs())
                wg.configure(**tuned)
                worlds.append(wg)
            vm = [hm[lo:lo + p.n] for p, lo in zip(parts, starts)]
            compute.step_motion_host(worlds, vm, o, args.warmup)  # from the state reached above
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            compute.step_motion_host(worlds, vm, o, k2)
            t1 = time.perf_counter()
            piped = sc.n * k2 / (t1 - t0)
            # (3) the full GpuBody + GpuAvbdBodyState records (192 B per body each way)
            hb, hs = pinned(sc.bodies.dtype, sc.n), pinned(sc.state.dtype, sc.n)
            worlds[0].download_into(hb[:parts[0].n], hs[:parts[0].n])
            for wg, p, lo in zip(worlds[1:], parts[1:], starts[1:]):
                wg.download_into(hb[lo:lo + p.n], hs[lo:lo + p.n])
            vb = [hb[lo:lo + p.n] for p, lo in zip(parts, starts)]
            vs = [hs[lo:lo + p.n] for p, lo in zip(parts, starts)]
            compute.step_host(worlds, vb, vs, o, 2)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            compute.step_host(worlds, vb, vs, o, k2)
            t1 = time.perf_counter()
            piped_full = sc.n * k2 / (t1 - t0)
            for wg in worlds:
                wg.close()
        t_ms = 1e3 * sc.n * k2 / max(piped, single)  # this rank's time for its share
        t_max, units = dio_dist.frame(dist, t_ms, sc.n * k2, device="cuda")
        e2e = {"value": units / (t_max / 1e3), "unit": "body-steps/s",
               "h2d_bytes_per_step": int(hm.nbytes), "d2h_bytes_per_step": int(hm.nbytes),
               "records": "DioBodyMotion, 64 B per body each way", "steps": k2,
               "worlds": len(parts) if piped >= single else 1, "one_world": single,
               "worlds_on_streams": {"worlds": len(parts), "value": piped},
               "full_records_worlds_on_streams": {"value": piped_full, "bytes_per_step_each_way": 192 * sc.n}}

    # plain path: one context per scene, stepped one scene at a time
    plain = None
    if not args.no_plain and rank == 0 and sc.n_scenes > 1:
        idx = np.linspace(0, sc.n_scenes - 1, min(args.plain_scenes, sc.n_scenes)).astype(int)
        worlds, nb = [], 0
        for s in idx:
            one = sc.select([s])
            pw = compute.World(world_capacity(one, per_body), contacts_per_pair=cpp)
            pw.set_stream(stream.cuda_stream)
            pw.upload(one.bodies, one.state, **one.upload_kwargs())
            worlds.append(pw)
            nb += one.n
        for pw in worlds:
            pw.step(o, 2)
        torch.cuda.synchronize()
        kp = 3
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(kp):
            for pw in worlds:
                pw.step(o, 1)
        p1.record(stream)
        torch.cuda.synchronize()
        pv = nb * kp / (p0.elapsed_time(p1) / 1e3)
        plain = {"value": pv, "unit": "body-steps/s", "sample": f"{len(idx)} of {sc.n_scenes} scenes ({nb} bodies)",
                 "batched_over_plain": value / world / pv}
        for pw in worlds:
            pw.close()

    # errors against the all-FP64 world at the workload's horizon, with the
    # split path's throughput on the same batch beside the FP32 one
    f64 = None
    if not args.no_f64 and rank == 0:
        steps_err = max(1, min(args.error_steps, int(sc.steps)))
        f64 = error_study(sc, o, steps_err, cap, cpp, tuned)
        if not prec:
            ws = compute.World(cap, precision=1, contacts_per_pair=cpp, **tuned)
            ws.set_stream(stream.cuda_stream)
            ws.upload(sc.bodies, sc.state, **sc.upload_kwargs())
            ws.step(o, args.warmup)
            torch.cuda.synchronize()
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            ws.step(o, args.steps)
            s1.record(stream)
            torch.cuda.synchronize()
            ws.close()
            sv = sc.n * args.steps / (s0.elapsed_time(s1) / 1e3)
            f64["split_throughput"] = {"value": sv, "unit": "body-steps/s",
                                       "batched_over_plain": sv / plain["value"] if plain else None}

    cpu = None
    if not args.no_cpu and rank == 0:
        threads = os.cpu_count() or 1
        ks = max(1, min(args.steps, 20))
        wu = min(args.warmup, 5)
        v, done, dt = run_cpu(sc, ks, wu, threads, budget_s=25.0, contacts_per_pair=cpp)
        v1, done1, _ = run_cpu(sc, 2, 0, 1, budget_s=10.0, contacts_per_pair=cpp)
        cpu = {"value": v, "unit": "body-steps/s", "cores": threads, "kind": "port",
               "sample": f"the whole workload ({sc.n} bodies): {done} steps after {wu} untimed ones, from the "
                         "initial state",
               "single_thread": {"value": v1, "cores": 1, "steps": done1}}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": scaling, "vs_baseline": None, "dtype": "f64/f32 split" if prec else "f32",
            "data": "synthetic", "config": workload_config(args, sc, scaling, world),
            "run": {"contacts_last_step": st["contacts"], "pairs_last_step": st["pairs"], "tuned": tuned,
                    "contacts_per_pair": cpp},
            "e2e": e2e, "per_phase": per_phase, "plain": plain, "fp64_error": f64,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": st["kernel_launches"],
            "phase_ms_per_step": {k: stp[f"{k}_ms"] / args.steps
                                  for k in ("broad", "narrow", "rows", "solve", "primal", "dual", "chunk")},
            "profiled_ms_per_step": ms_profiled / args.steps,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
