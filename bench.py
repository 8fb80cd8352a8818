"""Throughput of the GB300 contact pipeline on the 100k-body mixed pile.

Workload: 100,000 bodies drawn uniformly from box / sphere / capsule / cylinder / cone /
32-point hull, uniform in a 120 x 200 x 120 volume over a static ground box and a
64 x 64-cell heightfield (amplitude 2); dt = 1/100, 4 substeps, 8 + 4 iterations,
float32.  Seeded synthetic scene (numpy PCG64), no dataset.  The scene is first stepped
until the pile has formed (untimed), then K steps are timed.

A "step" is one full World.Step: broadphase, narrowphase + manifold, contact cache,
colouring, substepped solve + integration, contact and body update.

  value   contacts/s = active contact points summed over the timed steps / device time
          (CUDA events on the library's stream; state resident in HBM; L2 flushed
          between steps by a 256 MiB write)
  e2e     the same metric through jg_step_host: bodies copied from pinned host memory to
          the device and back every step, copies inside the timed region
  roofline  the substepped solve kernel against HBM bandwidth, bytes per step =
          S * ((I + R) * 276 * C + 320 * C + 116 * N) + 52 * N
  cpu_baseline  the oracle's multithreaded Regular-mode restatement of the reference
          (C++ restatement of Jitter2, all host threads) on 2 steps of the same state
  fp64_error  one step from the timed state replayed by the FP64 oracle in the GPU's order:
          errors in contact normal, depth, point, impulse, velocity and position
  fp64_drift  a 4000-body pile stepped 1000 times on the GPU and in the FP64 oracle: the
          gaps of kinetic and potential energy and the final momenta
  learned_warm_start  the learned against the plain warm start on 50 towers + 49k rubble,
          trained on 10M pairs: iterations to 1e-4 (cap 64) and 1e-2, the iterations the
          learned start needs to match the plain 8-iteration residual, contacts/s at equal
          iterations and at equal accuracy

--config c1 | c2 | c4 | c5 runs the workload's other configurations (1000-box grid, 20k
pile, 4096 batched worlds, towers + rubble) and prints their line; the default (c3, the
100k pile) is the headline.  --impl reference times the CPU restatement alone (the
reference is C# and no .NET runtime exists on either machine) and prints the same line
with "impl": "reference".
Multi-GPU: the single world does not shard ("replicas only"); with N ranks each rank
steps its own replica and value sums contacts over ranks / max time.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

N_BODIES = 100000
SETTLE_STEPS = 800
SEED = 12347
# Both arms time the same formed pile: whichever arm forms it first stores the body state
# here, and the other loads it (the driver runs the reference arm first on the same box).
STATE_CACHE = os.environ.get("JG_BENCH_CACHE", "/tmp/jitter_gb300_bench")

# Figures from ncu captures (profiles/), labelled with the commit they were taken at:
# they do not follow later code changes.
CAPTURE = {"k_solve_tasks_dram_bytes": 0.067e9, "k_mpr_fma_pipe_pct": 33.2,
           "source": "ncu captures of the formed 100k pile: k_solve_tasks at commit 0e4443c "
                     "(profiles/k_solve_tasks_pile100k.md; later commits keep its partition of this pile), "
                     "k_mpr at commit 20319af (profiles/k_mpr_k_epa_pile100k.md); narrowphase unchanged since"}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed loop runs."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", os.environ.get("LOCAL_RANK", "0"),
                                          "--query-gpu=" + q, "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_scene(n=N_BODIES):
    from jitterphysics2_gb300 import scenes
    return scenes.mixed_pile(n=n, box=(120.0, 200.0, 120.0), seed=SEED)


# The workload's configurations; c3 (the 100k pile) is the headline line, the others
# are run with --config for the results table.  Settle steps before timing:
CONFIG_SETTLE = {"c3": SETTLE_STEPS, "c1": 300, "c2": 600, "c4": 200, "c5": 100}


def c3_config(n_bodies, settle):
    """The workload object both arms print for the 100k pile."""
    return {"name": "c3", "workload": "mixed pile, %d bodies, 120x200x120 over ground + heightfield, formed in %d "
                                      "steps; dt 0.01, 4 substeps, (8,4) iterations" % (n_bodies, settle),
            "bodies": n_bodies, "settle_steps": settle, "parallelism": "replicas only",
            "l2": "working set above L2 (bodies, contact cache and schedule, several hundred MB); "
                  "the GPU arm also writes 256 MiB between timed steps"}


def state_path(n, settle):
    return os.path.join(STATE_CACHE, "c3_seed%d_n%d_settle%d.npy" % (SEED, n, settle))


def load_state(n, settle):
    """The formed pile's bodies stored by an earlier arm on this machine, or None."""
    from jitterphysics2_gb300 import abi
    p = state_path(n, settle)
    if not os.path.exists(p):
        return None
    b = np.load(p)
    return b if b.dtype == abi.BODY_DTYPE and len(b) == n + 2 else None


def store_state(bodies, n, settle):
    try:
        os.makedirs(STATE_CACHE, exist_ok=True)
        tmp = state_path(n, settle) + ".%d.tmp" % os.getpid()
        np.save(tmp, bodies)
        os.replace(tmp + ".npy" if not tmp.endswith(".npy") else tmp, state_path(n, settle))
    except OSError:
        pass


def config_scene(name, n):
    from jitterphysics2_gb300 import scenes
    if name == "c3":
        return make_scene(n), None, "mixed pile, %d bodies, 120x200x120 over ground + heightfield"
    if name == "c1":
        return scenes.box_grid(n_side=10), None, "1000 unit boxes in a 10x10x10 grid on a ground box"
    if name == "c2":
        return (scenes.mixed_pile(n=20000, box=(60.0, 120.0, 60.0), seed=12346), None,
                "mixed pile, 20k bodies, 60x120x60 over ground + heightfield")
    if name == "c4":
        return (scenes.batched_worlds(), None,
                "4096 batched worlds, 8-512 bodies each, capsule chains (BallSocket + HingeAngle)")
    if name == "c5":
        return scenes.towers_rubble(), None, "50 towers x 20 unit boxes + 49k mixed rubble"
    raise SystemExit("unknown config " + name)


def solver_bytes(counters, n_bodies, substeps=4, iters=8, relax=4):
    c = counters["contacts"]
    return substeps * ((iters + relax) * 276 * c + 320 * c + 116 * n_bodies) + 52 * n_bodies


def cpu_baseline(scene, bodies, contacts, steps=2):
    """The oracle's multithreaded Regular-mode step on the GPU's settled state."""
    import oracle_lib as O
    threads = os.cpu_count() or 1
    sc = dict(scene)
    sc["bodies"] = bodies
    o = O.OracleWorld(sc)
    o.set_contacts(contacts)
    total_t, total_c = 0.0, 0
    for _ in range(steps):
        t = o.step_mt(scene["dt"], threads)
        total_t += t
        total_c += o.counters()["contacts"]
    return {"value": total_c / total_t, "unit": "contacts/s", "cores": threads, "kind": "port",
            "sample": "%d steps of the GPU-settled %d-body state (C++ restatement of Jitter2, Regular mode)"
                      % (steps, len(bodies)),
            "seconds": total_t}


def learned_section(eval_steps=10, target_pairs=10_000_000, cap=64, workload_iterations=8):
    """Learned against plain warm start on the towers-and-rubble workload (50 towers of
    20 unit boxes + 49k mixed rubble).  Training: (features, converged impulse) pairs of the
    contacts created in scenes of successive seeds, up to target_pairs, on the device's own
    kernels.  Evaluation, from identical states at eval_steps steps: the first substep's
    residual curve up to `cap` iterations; iterations to 1e-4 (capped, as defined for the
    workload) and to 1e-2; the iterations the learned start needs to reach the residual the
    plain start has after the workload's 8 iterations; contacts/s of both at 8 iterations
    and of the learned start at that matching iteration count (equal accuracy)."""
    from jitterphysics2_gb300 import abi, learned, scenes
    from jitterphysics2_gb300.world import World, world_for_scene
    t0 = time.perf_counter()
    X, T = learned.collect_many(lambda seed: scenes.towers_rubble(seed=seed), range(101, 141), steps=200, start=10,
                                target_pairs=target_pairs)
    t_collect = time.perf_counter() - t0
    params = learned.init_params(X, T, seed=0)
    trainer = World(max_bodies=16)
    trainer.mlp_load(params)
    losses = learned.train(trainer, X, T, epochs=8, batch=8192, lr=2e-3)
    params = trainer.mlp_export()
    trainer.close()
    t_train = time.perf_counter() - t0 - t_collect
    sc = scenes.towers_rubble(seed=12349)
    ip, il, rp, rl = learned.paired_residuals(sc, params, steps=eval_steps, settle=60, iterations=cap)
    to = lambda r, tol: float(np.mean([learned.iterations_to(x, tol) for x in r]))
    k_match = learned.iterations_to_match(rl, rp, workload_iterations)
    k_eq = int(np.ceil(k_match.mean()))
    settler = world_for_scene(sc)
    for _ in range(60):
        settler.step(sc["dt"])
    state = settler.export_state()
    settler.close()
    rate_plain = learned.throughput(sc, state, params, workload_iterations, eval_steps, False)
    rate_learned = learned.throughput(sc, state, params, workload_iterations, eval_steps, True)
    rate_learned_eq = learned.throughput(sc, state, params, k_eq, eval_steps, True)
    gm = lambda a: float(np.exp(np.mean(np.log(np.maximum(a, 1e-30)))))
    return {"workload": "50 towers x 20 unit boxes + 49k mixed rubble, dt 1/100, 4 substeps",
            "training_pairs": int(len(X)), "collect_seconds": t_collect, "train_seconds": t_train,
            "loss_first_epoch": losses[0], "loss_last_epoch": losses[-1], "iteration_cap": cap,
            "iters_to_1e-4_plain": to(rp, 1e-4), "iters_to_1e-4_learned": to(rl, 1e-4),
            "iters_to_1e-2_plain": to(rp, 1e-2), "iters_to_1e-2_learned": to(rl, 1e-2),
            "residual_after_8_plain": gm(rp[:, 7]), "residual_after_8_learned": gm(rl[:, 7]),
            "residual_after_cap_plain": gm(rp[:, -1]), "residual_after_cap_learned": gm(rl[:, -1]),
            "iters_learned_to_match_plain_8": float(k_match.mean()),
            "contacts_per_s_plain": rate_plain, "contacts_per_s_learned_same_iterations": rate_learned,
            "contacts_per_s_learned_same_accuracy": rate_learned_eq, "learned_iterations_same_accuracy": k_eq,
            "steps_compared": eval_steps, "seconds": time.perf_counter() - t0}


def fp64_section(scene, bodies, contacts_before, contacts_after, gpu_after):
    """One step from the GPU's state replayed by the FP64 oracle in the GPU's solve order:
    errors of the FP32 path in contact normal, depth, point, impulse, velocity and position."""
    import precision_lib
    t0 = time.perf_counter()
    r = precision_lib.one_step_errors(scene, bodies, contacts_before, contacts_after, gpu_after)
    r["seconds"] = time.perf_counter() - t0
    r["sample"] = "one step of the formed pile from identical state, FP64 oracle in the GPU's order"
    return r


def drift_section(n=4000, steps=1000):
    """Momentum and energy of a pile (the 20k pile's recipe at n bodies, gravity, ground and
    heightfield) over `steps` steps from the seeded start, FP32 on the GPU against the FP64
    oracle (multithreaded): the relative gaps of kinetic and potential energy."""
    import precision_lib
    from jitterphysics2_gb300 import scenes
    from jitterphysics2_gb300.world import world_for_scene
    t0 = time.perf_counter()
    sc = scenes.mixed_pile(n=n, box=(30.0, 60.0, 30.0), seed=12350)
    w = world_for_scene(sc)
    d = precision_lib.drift(sc, w, steps, threads=os.cpu_count() or 1)
    w.close()
    u0 = abs(d["u_fp64"][0])
    k_scale = max(float(np.max(d["k_fp64"])), 1e-9)
    return {"workload": "mixed pile, %d bodies, 30x60x30 over ground + heightfield, %d steps from the seeded start"
                        % (n, steps),
            "potential_gap_final": float(abs(d["u_gpu"][-1] - d["u_fp64"][-1]) / u0),
            "potential_gap_max": float(np.max(np.abs(d["u_gpu"] - d["u_fp64"])) / u0),
            "kinetic_gap_max_of_peak": float(np.max(np.abs(d["k_gpu"] - d["k_fp64"])) / k_scale),
            "kinetic_final_gpu": float(d["k_gpu"][-1]), "kinetic_final_fp64": float(d["k_fp64"][-1]),
            "momentum_final_gpu": float(np.linalg.norm(d["p_gpu"][-1])),
            "momentum_final_fp64": float(np.linalg.norm(d["p_fp64"][-1])),
            "seconds": time.perf_counter() - t0}


def dist_setup(n_gpus):
    if n_gpus <= 1 or "RANK" not in os.environ:
        return 0, 1, None
    import torch.distributed as dist
    dist.init_process_group("nccl" if os.environ.get("JG_DIST_BACKEND", "nccl") == "nccl" else "gloo")
    return dist.get_rank(), dist.get_world_size(), dist


def reduce_over_ranks(total_ms, contacts, dist, device="cuda"):
    """Replicas only (the world does not shard): the job's time is the slowest rank's, its
    contact count the sum over ranks.  No collective when running alone."""
    if dist is None:
        return float(total_ms), float(contacts)
    import torch
    tt = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    cc = torch.tensor([float(contacts)], dtype=torch.float64, device=device)
    dist.all_reduce(cc, op=dist.ReduceOp.SUM)
    return float(tt.item()), float(cc.item())


def run_reference(args):
    """The CPU arm: the oracle's multithreaded Regular-mode restatement of World.Step on
    all host threads, on the same formed pile as the GPU arm.  It loads only the oracle
    library (scene construction and parameters are pure Python)."""
    rank, ws, dist = dist_setup(args.gpus)
    if rank != 0:
        return
    import oracle_lib as O
    sc = make_scene(args.bodies)
    threads = os.cpu_count() or 1
    bodies = load_state(args.bodies, args.settle)
    state = "loaded (formed by the other arm on this machine)"
    if bodies is None:
        t0 = time.perf_counter()
        o = O.OracleWorld(sc)
        for _ in range(args.settle):
            o.step_mt(sc["dt"], threads)
        bodies = o.bodies()
        store_state(bodies, args.bodies, args.settle)
        state = "formed here by the CPU restatement in %.0f s" % (time.perf_counter() - t0)
    else:
        sc = dict(sc)
        sc["bodies"] = bodies
        o = O.OracleWorld(sc)
    for _ in range(args.warmup):
        o.step_mt(sc["dt"], threads)
    total_t, total_c = 0.0, 0
    for _ in range(args.steps):
        total_t += o.step_mt(sc["dt"], threads)
        total_c += o.counters()["contacts"]
    v = total_c / total_t if total_t > 0 else 0.0
    line = {"metric": "contacts/s @100k bodies", "value": v, "unit": "contacts/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference", "config": c3_config(len(bodies) - 2, args.settle),
            "contacts_per_step": total_c / max(args.steps, 1), "state": state,
            "note": "C++ restatement of Jitter2 World.Step (Regular mode, grid broadphase); the C# reference needs "
                    "a .NET runtime, absent on both machines",
            "cpu_baseline": {"value": v, "unit": "contacts/s", "cores": threads, "kind": "port",
                             "sample": "%d warm-up + %d timed multithreaded steps of the formed pile at the "
                                       "workload's settings" % (args.warmup, args.steps)},
            "e2e": {"value": v, "unit": "contacts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--settle", type=int, default=None, help="settle steps (default: the config's)")
    ap.add_argument("--bodies", type=int, default=N_BODIES, help="smaller piles for profiling captures")
    ap.add_argument("--config", default="c3", help="c3 (headline, default), c1, c2, c4, c5")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-extras", action="store_true", help="skip the FP64 and learned warm start sections")
    args = ap.parse_args()
    if args.settle is None:
        args.settle = CONFIG_SETTLE.get(args.config, SETTLE_STEPS)
    if args.impl == "reference":
        return run_reference(args)

    rank, ws, dist = dist_setup(args.gpus)
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from jitterphysics2_gb300 import abi
    from jitterphysics2_gb300.world import world_for_scene

    sc, _, workload = config_scene(args.config, args.bodies)
    prm = sc["params"]
    S, I, R = prm.get("substeps", 1), prm.get("solver_iterations", 6), prm.get("relax_iterations", 4)
    state = None
    if args.config == "c3":
        # the formed pile: from the other arm when it formed it on this machine, else
        # formed here with the same settings and stored for the other arm
        bodies = load_state(args.bodies, args.settle) if rank == 0 or ws == 1 else None
        if bodies is not None:
            sc = dict(sc)
            sc["bodies"] = bodies
            w = world_for_scene(sc)
            state = "loaded (formed by the other arm on this machine)"
        else:
            w = world_for_scene(sc)
            for _ in range(args.settle):
                w.step(sc["dt"])
            if rank == 0:
                store_state(w.bodies(), args.bodies, args.settle)
            state = "formed here on the device"
    else:
        w = world_for_scene(sc)
        for _ in range(args.settle):
            w.step(sc["dt"])
    for _ in range(max(3, args.warmup)):
        w.step(sc["dt"])
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    # device-timed steps (inputs resident), bracketed by a barrier when several ranks run
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler()
    clocks.start()
    step_ms, solve_ms, contacts, sbytes, launches, stages = [], [], 0, [], 0, []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        w.step(sc["dt"])
        t = w.timings()
        c = w.counters()
        step_ms.append(t["total"])
        solve_ms.append(t["solve"])
        stages.append(t)
        contacts += c["contacts"]
        sbytes.append(solver_bytes(c, len(sc["bodies"]), S, I, R))
        launches += c["kernel_launches"]
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    stage_ms = {k: float(np.mean([s[k] for s in stages])) for k in stages[0]}
    clk = clocks.stop()
    total_ms, contacts_all = reduce_over_ranks(float(np.sum(step_ms)), contacts, dist)
    value = contacts_all / (total_ms / 1e3)

    # end to end through the host-buffer call
    host = np.ascontiguousarray(w.bodies())
    pinned = torch.from_numpy(host.view(np.uint8)).pin_memory()
    hb = pinned.numpy().view(abi.BODY_DTYPE)
    e2e_c, t0 = 0, time.perf_counter()
    for _ in range(args.steps):
        w.step_host(sc["dt"], hb)
        e2e_c += w.counters()["contacts"]
    e2e_s = time.perf_counter() - t0
    nbytes = hb.nbytes

    peak, peak_kind = peaks()
    # a graph replay (batched worlds) is timed as a whole: the solver's bytes over the whole
    # step's time is then a lower bound of its rate
    solve_timed = all(t > 0 for t in solve_ms)
    if not solve_timed:
        solve_ms = step_ms
    achieved = float(np.mean([b / (s / 1e3) for b, s in zip(sbytes, solve_ms)])) / 1e9
    nb = len(sc["bodies"])
    cnt = w.counters()
    metric = "contacts/s @100k bodies" if args.config == "c3" else "contacts/s"
    line = {"metric": metric, "value": value, "unit": "contacts/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scene)",
            "config": c3_config(nb - 2, args.settle) if args.config == "c3" else
                      {"name": args.config,
                       "workload": "%s; dt %.5g, %d substeps, (%d,%d) iterations" % (workload % nb if "%d" in workload
                                                                                    else workload, sc["dt"], S, I, R),
                       "bodies": nb, "settle_steps": args.settle, "parallelism": "replicas only",
                       "l2": "flushed between steps (256 MiB write)"},
            "state": state,
            "contacts_per_step": contacts / args.steps, "arbiters": cnt["arbiters"],
            "solver_tasks": cnt["solver_tasks"], "task_colors": cnt["task_colors"],
            "task_arbiters": cnt["task_arbiters"], "remainder_colors": cnt["colors"],
            "body_steps_per_s": nb * args.steps * ws / (total_ms / 1e3),
            "e2e": {"value": e2e_c / e2e_s, "unit": "contacts/s", "h2d_bytes_per_step": nbytes,
                    "d2h_bytes_per_step": nbytes},
            "roofline": {"bound": "hbm", "kernel": "k_solve_tasks", "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         # DRAM bytes read + written by one k_solve_tasks launch of the formed
                         # 100k pile, from an ncu capture (rows stay in L2 across passes, so
                         # DRAM traffic is below the algorithmic bytes)
                         "traffic": CAPTURE["k_solve_tasks_dram_bytes"] if args.config == "c3" and nb == N_BODIES + 2
                         else None, "traffic_source": CAPTURE["source"],
                         "solve_ms_per_step": float(np.mean(solve_ms)),
                         "timed_span": "solve kernel" if solve_timed else "whole step (graph replay)",
                         "bytes_model": "S*((I+R)*276*C + 320*C + 116*N) + 52*N"},
            # the narrowphase is bound by the FP32 pipe, not HBM: FMA-pipe cycles active of the
            # MPR kernel from an ncu capture of this workload
            "narrowphase": {"bound": "fp32 pipe", "kernel": "k_mpr", "fma_pipe_active_pct": CAPTURE["k_mpr_fma_pipe_pct"],
                            "fma_source": CAPTURE["source"], "ms_per_step": stage_ms["narrowphase"]}
            if args.config == "c3" and nb == N_BODIES + 2 else None,
            "clocks": clk, "gpu_launches": launches,
            "step_launch": "one CUDA-graph launch per step (jg_batch_step), %d kernels in the graph"
                           % (launches // max(args.steps, 1)) if sc.get("n_worlds", 1) > 1 else
                           "%d kernel launches per step" % (launches // max(args.steps, 1)),
            "stage_ms": stage_ms}
    extras = rank == 0 and not args.no_extras and args.config == "c3"
    if extras:
        b0, c0 = w.bodies(), w.contacts()
        w.step(sc["dt"])
        line["fp64_error"] = fp64_section(sc, b0, c0, w.contacts(), w.bodies())
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(sc, w.bodies(), w.contacts())
    w.close()
    if extras:
        line["fp64_drift"] = drift_section()
        line["learned_warm_start"] = learned_section()
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
