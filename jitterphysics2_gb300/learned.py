"""Learned warm start for new contacts: parameter initialisation, training-data
collection from seeded scenes, training on the GPU, and the residual comparison
(iterations to reach a residual, learned against plain warm start).

No counterpart in the reference: Jitter2 starts every new contact from zero impulse
(Contact.cs:727) and only cached contacts are warm-started.
"""
import numpy as np

from . import abi
from .world import world_for_scene


def init_params(X, T, seed=0):
    """He-initialised weights; feature standardisation and output scale from the data."""
    rng = np.random.default_rng(seed)
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.float64)
    mean = X.mean(0)
    scale = 1.0 / np.maximum(X.std(0), 1e-6)
    oscale = np.maximum(np.sqrt((T ** 2).mean(0)), 1e-6)
    H, I, O = abi.MLP_HID, abi.MLP_IN, abi.MLP_OUT
    parts = [rng.normal(0, np.sqrt(2.0 / I), (H, I)), np.zeros(H),
             rng.normal(0, np.sqrt(2.0 / H), (H, H)), np.zeros(H),
             rng.normal(0, np.sqrt(1.0 / H), (O, H)), np.zeros(O),
             mean, scale, oscale]
    return np.concatenate([np.ravel(p) for p in parts]).astype(np.float32)


def collect(scene, steps, start=0):
    """Steps a world of `scene` and returns the (features, converged impulse) pairs of
    every contact created during steps start..steps-1."""
    w = world_for_scene(scene)
    w.collect_training(capacity=1 << 17)  # arm
    xs, ts = [], []
    for s in range(steps):
        w.step(scene["dt"])
        x, t = w.collect_training(capacity=1 << 17)
        if s >= start and len(x):
            xs.append(x)
            ts.append(t)
    w.close()
    if not xs:
        return np.zeros((0, abi.MLP_IN), np.float32), np.zeros((0, abi.MLP_OUT), np.float32)
    return np.concatenate(xs), np.concatenate(ts)


def collect_many(make_scene, seeds, steps, start, target_pairs):
    """collect() over scenes of successive seeds until target_pairs pairs are gathered."""
    xs, ts, n = [], [], 0
    for seed in seeds:
        x, t = collect(make_scene(seed), steps=steps, start=start)
        xs.append(x)
        ts.append(t)
        n += len(x)
        if n >= target_pairs:
            break
    return np.concatenate(xs)[:target_pairs], np.concatenate(ts)[:target_pairs]


def train(world, X, T, epochs=20, batch=4096, lr=2e-3, seed=0):
    """Adam on the GPU (jg_mlp_train_step) over shuffled minibatches; returns the mean
    loss of every epoch."""
    rng = np.random.default_rng(seed)
    n = len(X)
    losses = []
    for e in range(epochs):
        order = rng.permutation(n)
        tot, cnt = 0.0, 0
        step_lr = lr * (0.5 ** (e // max(1, epochs // 3)))
        for i in range(0, n, batch):
            idx = order[i:i + batch]
            tot += world.mlp_train_step(X[idx], T[idx], step_lr) * len(idx)
            cnt += len(idx)
        losses.append(tot / max(cnt, 1))
    return losses


def iterations_to(resid, tol=1e-4):
    """First iteration (1-based) whose residual is at most tol; len(resid) + 1 if none."""
    for k, r in enumerate(resid):
        if r <= tol:
            return k + 1
    return len(resid) + 1


def iterations_to_match(resid_learned, resid_plain, k):
    """Per step, the iterations the learned warm start needs to reach the residual the plain
    one has after k iterations (len + 1 when it never does)."""
    return np.array([iterations_to(rl, rp[k - 1]) for rl, rp in zip(resid_learned, resid_plain)])


def throughput(scene, state, params, iterations, steps, learned_start):
    """Contacts per second over `steps` steps from `state` at `iterations` solver
    iterations, plain or learned warm start."""
    mode = abi.WARMSTART_MLP if learned_start else abi.WARMSTART_CACHED
    w = world_for_scene(scene, warm_start_mode=mode, solver_iterations=iterations)
    if learned_start:
        w.mlp_load(params)
    w.import_state(state)
    ms, cnt = 0.0, 0
    for _ in range(steps):
        w.step(scene["dt"])
        ms += w.timings()["total"]
        cnt += w.counters()["contacts"]
    w.close()
    return cnt / (ms / 1e3)


def paired_residuals(scene, params, steps, settle, iterations=32, tol=1e-4):
    """From the same state at each of `steps` steps (after `settle` steps of the plain
    solver at the scene's own iteration count), one step with the plain (cached) warm
    start and one with the learned warm start, both with `iterations` iterations; returns
    the iterations to `tol` and the residual curves of both."""
    kw = dict(record_residual=1, solver_iterations=iterations)
    settler = world_for_scene(scene, warm_start_mode=abi.WARMSTART_CACHED)
    for _ in range(settle):
        settler.step(scene["dt"])
    plain = world_for_scene(scene, warm_start_mode=abi.WARMSTART_CACHED, **kw)
    plain.import_state(settler.export_state())
    settler.close()
    learned = world_for_scene(scene, warm_start_mode=abi.WARMSTART_MLP, **kw)
    learned.mlp_load(params)
    it_plain, it_learned, r_plain, r_learned = [], [], [], []
    for _ in range(steps):
        state = plain.export_state()
        learned.import_state(state)
        learned.step(scene["dt"])
        rl = learned.residuals()
        plain.step(scene["dt"])
        rp = plain.residuals()
        it_plain.append(iterations_to(rp, tol))
        it_learned.append(iterations_to(rl, tol))
        r_plain.append(rp)
        r_learned.append(rl)
    plain.close()
    learned.close()
    return np.array(it_plain), np.array(it_learned), np.array(r_plain), np.array(r_learned)
