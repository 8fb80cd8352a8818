"""Batched independent worlds (one launch sequence for all worlds; each world's arbiters
form one task of the partitioned solve) and the autotuner."""
import numpy as np
import pytest

from jitterphysics2_gb300 import abi, scenes
from jitterphysics2_gb300.world import world_for_scene

pytestmark = pytest.mark.gpu


def quat_mat(q):
    x, y, z, w = [np.asarray(q[..., i], np.float64) for i in range(4)]
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
                     np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
                     np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], -2)


def anchor_errors(b0, b1, joints):
    """World-space distance between the two bodies' copies of each BallSocket anchor."""
    err = []
    for kind, i, j, init in joints:
        if kind != abi.CONSTRAINT_BALLSOCKET:
            continue
        a = np.asarray(init, np.float64)
        la1 = quat_mat(b0["orientation"][i]).T @ (a - b0["position"][i])
        la2 = quat_mat(b0["orientation"][j]).T @ (a - b0["position"][j])
        p1 = b1["position"][i] + quat_mat(b1["orientation"][i]) @ la1
        p2 = b1["position"][j] + quat_mat(b1["orientation"][j]) @ la2
        err.append(np.linalg.norm(p1 - p2))
    return np.array(err)


def test_batched_worlds_step_independently():
    sc = scenes.batched_worlds(n_worlds=96, lo=8, hi=160, seed=3)
    w = world_for_scene(sc)
    b0 = w.bodies()
    for _ in range(150):
        w.step(sc["dt"])
    c = w.counters()
    assert c["status"] == 0
    b = w.bodies()
    world = sc["bodies"]["world"]
    con = w.contacts()
    assert len(con) > 500
    # contacts only ever join bodies of one world
    assert np.array_equal(world[con["body1"]], world[con["body2"]])
    # every world is one task of the partitioned solve: no arbiter left to global colours
    assert c["task_arbiters"] == c["arbiters"], c
    assert c["solver_tasks"] >= len(np.unique(world[con["body1"]])), c
    dyn = b["motion_type"] == abi.MOTION_DYNAMIC
    assert np.isfinite(b["position"]).all() and b["position"][dyn, 1].min() > -0.5
    assert np.abs(b["velocity"][dyn]).max() < 20.0
    # the capsule chains hold together
    err = anchor_errors(b0, b, sc["joints"])
    assert len(err) > 50 and np.median(err) < 0.01 and err.max() < 0.1, (np.median(err), err.max())


def test_autotune_picks_a_working_launch_shape():
    sc = scenes.batched_worlds(n_worlds=32, lo=8, hi=96, seed=4)
    w = world_for_scene(sc)
    for _ in range(40):
        w.step(sc["dt"])
    before = w.bodies()
    chosen = w.autotune(sc["dt"], steps=2)
    if chosen["partitioned_solve"]:
        assert chosen["solver_block"] in (64, 96, 128) and chosen["solver_ctas_per_sm"] in (1, 2)
    else:
        assert chosen["solver_block"] in (128, 256, 512) and chosen["solver_ctas_per_sm"] in (1, 2, 4)
    assert chosen["sched_cells_per_sm"] == 0.0   # batched worlds: one cell per world, not tuned
    # the tuner restores the state it timed from
    after = w.bodies()
    assert np.array_equal(before["position"], after["position"])
    for _ in range(5):
        w.step(sc["dt"])
    assert w.counters()["status"] == 0


def test_batched_worlds_without_joints_hand_off_and_match_the_oracle():
    # without joints there is no remainder, so the task solve runs without grid barriers
    # between its phases (each world is one task and waits only on its own previous pass);
    # one step from identical state must match the oracle replaying the GPU's order
    from test_gpu_parity import _one_step_velocity_errors
    sc = dict(scenes.batched_worlds(n_worlds=48, lo=8, hi=96, seed=5))
    sc["joints"] = []
    w = world_for_scene(sc)
    for _ in range(120):
        w.step(sc["dt"])
    c = w.counters()
    assert c["status"] == 0 and c["colors"] == 0 and c["task_arbiters"] == c["arbiters"], c
    err = _one_step_velocity_errors(sc, w)
    assert np.mean(err < 1e-3) >= 0.999, (np.mean(err < 1e-3), np.sort(err)[-5:])


def test_batched_graph_step_equals_stream_steps():
    """jg_batch_step (one CUDA-graph launch per step) gives the bits of the same step issued
    launch by launch (jg_step without a graph)."""
    import ctypes
    sc = scenes.batched_worlds(n_worlds=64, lo=8, hi=64, seed=8)
    a = world_for_scene(sc)
    b = world_for_scene(sc)
    for _ in range(40):
        a.step(sc["dt"])
        abi.check(b._lib.jg_step(b.handle, ctypes.c_float(sc["dt"])), "jg_step")
    ba, bb = a.bodies(), b.bodies()
    assert a.counters()["status"] == 0 and a.counters()["contacts"] > 0
    assert np.array_equal(ba["position"], bb["position"]) and np.array_equal(ba["velocity"], bb["velocity"])
    assert a.timings()["total"] > 0


def test_autotune_on_a_single_world_picks_a_cell_density():
    sc = scenes.mixed_pile(n=2000, box=(30.0, 10.0, 30.0), y0=0.0, cells=16, seed=23, lattice=2.0)
    w = world_for_scene(sc)
    for _ in range(30):
        w.step(sc["dt"])
    before = w.bodies()
    chosen = w.autotune(sc["dt"], steps=1)
    if chosen["partitioned_solve"]:
        assert chosen["sched_cells_per_sm"] in (0.0, 1.0, 2.0, 3.0, 4.5, 6.0, 9.0), chosen
    after = w.bodies()
    assert np.array_equal(before["position"], after["position"])
    for _ in range(3):
        w.step(sc["dt"])
    assert w.counters()["status"] == 0
