"""GPU parity against the oracle, through the C ABI.

Thresholds (from the workload definition): contact normal, depth and point within 1e-4
relative; post-solve velocities within 1e-3 after one step from identical states.
The solver comparison replays the GPU's colour order in the oracle: rows inside one
colour share no dynamic body, so that order is a valid Gauss-Seidel order of the
reference solver, and the two runs must agree up to float rounding.
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi, scenes
from jitterphysics2_gb300.world import world_for_scene

pytestmark = pytest.mark.gpu


def quat_rotate(q, v):
    x, y, z, w = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    return R @ v


def test_free_fall_matches_oracle_bitwise():
    sc = scenes.box_grid(n_side=4)
    w = world_for_scene(sc)
    o = O.OracleWorld(sc)
    for _ in range(5):
        w.step(sc["dt"])
        o.step(sc["dt"])
    gb, ob = w.bodies(), o.bodies()
    # no contacts yet: integration and the body update only, identical float rounding
    assert np.array_equal(gb["position"], ob["position"])
    assert np.array_equal(gb["velocity"], ob["velocity"])
    assert np.array_equal(gb["orientation"], ob["orientation"])


def _settled_pile(n=400, steps=250, seed=7):
    sc = scenes.mixed_pile(n=n, box=(20.0, 3.0, 20.0), y0=0.0, cells=8, seed=seed, lattice=3.0)
    w = world_for_scene(sc)
    for _ in range(steps):
        w.step(sc["dt"])
    return sc, w


def test_narrowphase_matches_oracle_on_a_pile():
    """Contacts registered by one step from a settled state (empty caches on both sides):
    the GPU's contact cache against the oracle's after its narrowphase and AddContact."""
    sc, w = _settled_pile()
    state = w.bodies()
    sc2 = dict(sc)
    sc2["bodies"] = state
    g = world_for_scene(sc2)
    g.step(sc["dt"])
    gc = g.contacts()
    o = O.OracleWorld(sc2)
    o.narrowphase()
    oc = o.contacts()
    assert len(gc) > 100 and len(oc) > 100
    stats = compare_contact_caches(gc, oc)
    # the same colliding pairs and slots, contact normal and point within 1e-4 (relative)
    # for at least 99.9 % of contacts
    assert stats["common_keys"] >= 0.999 * stats["keys"], stats
    assert stats["slot_mismatch"] <= 0.001 * stats["common_keys"], stats
    assert stats["normal_ok"] >= 0.999 and stats["point_ok"] >= 0.999, stats


def compare_contact_caches(gc, oc):
    """Contact caches of the GPU and the oracle, matched by (shape1, shape2, slot): pair
    and slot agreement, and per matched contact the normal error and the local point
    error relative to max(1, |point|)."""
    def index(rows):
        d = {}
        for r in rows:
            d.setdefault((int(r["shape1"]), int(r["shape2"])), {})[int(r["slot"])] = r
        return d

    G, Oo = index(gc), index(oc)
    keys = set(G) | set(Oo)
    common = set(G) & set(Oo)
    nrm_err, pt_err, mismatch = [], [], []
    for k in common:
        if set(G[k]) != set(Oo[k]):
            mismatch.append((k, sorted(G[k]), sorted(Oo[k])))
            continue
        for slot, r in G[k].items():
            q = Oo[k][slot]
            nrm_err.append(np.abs(np.asarray(r["normal"], np.float64) - q["normal"]).max())
            scale = max(1.0, np.abs(q["pos1_local"]).max())
            pt_err.append(np.abs(np.asarray(r["pos1_local"], np.float64) - q["pos1_local"]).max() / scale)
    nrm_err, pt_err = np.array(nrm_err), np.array(pt_err)
    return {"keys": len(keys), "common_keys": len(common), "slot_mismatch": len(mismatch),
            "mismatch_examples": mismatch[:5], "contacts": len(nrm_err),
            "normal_ok": float(np.mean(nrm_err < 1e-4)) if len(nrm_err) else 1.0,
            "point_ok": float(np.mean(pt_err < 1e-4)) if len(pt_err) else 1.0,
            "normal_err_max": float(nrm_err.max()) if len(nrm_err) else 0.0,
            "point_err_max": float(pt_err.max()) if len(pt_err) else 0.0}


def _one_step_velocity_errors(sc, w):
    b0 = w.bodies()
    c0 = w.contacts()
    w.step(sc["dt"])
    b1 = w.bodies()
    c1 = w.contacts()
    assert len(c1) > 100
    o = O.OracleWorld(sc, external_order=True)
    o.set_bodies(b0)
    o.set_contacts(c0)
    o.narrowphase()
    for c in c1:
        o.set_arbiter_color(c["shape1"], c["shape2"], c["color"])
    o.step(sc["dt"], narrow=False)
    ob = o.bodies()
    dyn = b1["motion_type"] == abi.MOTION_DYNAMIC
    dv = np.abs(b1["velocity"][dyn] - ob["velocity"][dyn]).max(axis=1)
    dw = np.abs(b1["angular_velocity"][dyn] - ob["angular_velocity"][dyn]).max(axis=1)
    return np.maximum(dv, dw)


@pytest.mark.parametrize("partitioned", [1, 0])
def test_one_step_solve_matches_oracle_on_resting_boxes(partitioned):
    # resting boxes: shallow contacts, MPR only, so both sides hold identical contacts and
    # the solve in the GPU's order must agree to float rounding; partitioned=1 solves in
    # spatial tasks, 0 in global colours only
    sc = scenes.box_grid(n_side=6)
    w = world_for_scene(sc, partitioned_solve=partitioned)
    for _ in range(350):
        w.step(sc["dt"])
    c = w.counters()
    if partitioned:
        assert c["solver_tasks"] >= 1 and c["task_arbiters"] == c["arbiters"]
    else:
        assert c["solver_tasks"] == 0
    err = _one_step_velocity_errors(sc, w)
    assert err.max() < 1e-3, err.max()


def test_partitioned_schedule_covers_a_wide_pile():
    # a pile wider than a cell: several tasks per grid, nearly every arbiter in a task
    sc = scenes.mixed_pile(n=3000, box=(60.0, 4.0, 60.0), y0=0.0, cells=8, seed=9, lattice=2.0)
    w = world_for_scene(sc)
    for _ in range(60):
        w.step(sc["dt"])
    c = w.counters()
    assert c["status"] == 0
    assert c["solver_tasks"] > 10, c
    assert c["task_arbiters"] >= 0.95 * c["arbiters"], c
    b = w.bodies()
    dyn = b["motion_type"] == abi.MOTION_DYNAMIC
    assert np.isfinite(b["velocity"]).all() and np.abs(b["velocity"][dyn]).max() < 20.0


def test_one_step_solve_matches_oracle_on_a_pile():
    # mixed pile with deep contacts (EPA with FP64 face data on both sides): post-solve
    # velocities within 1e-3 for at least 99.9 % of bodies
    sc, w = _settled_pile(seed=11)
    err = _one_step_velocity_errors(sc, w)
    assert np.mean(err < 1e-3) >= 0.999, (np.mean(err < 1e-3), np.sort(err)[-5:])


def test_one_step_solve_with_joints_matches_oracle():
    # capsule chains linked by BallSocket + HingeAngle over a small pile: joints are solved
    # in global colours after the contact tasks; the oracle replays contacts and joints
    # in the GPU's order keys, warm-started with the GPU's joint impulses
    sc = scenes.batched_worlds(n_worlds=1, lo=24, hi=48, seed=5)
    assert len(sc["joints"]) >= 8
    w = world_for_scene(sc)
    for _ in range(80):
        w.step(sc["dt"])
    b0, c0 = w.bodies(), w.contacts()
    _, j0 = w.constraints()
    w.step(sc["dt"])
    b1, c1 = w.bodies(), w.contacts()
    k1, j1 = w.constraints()
    assert (k1 >= 768).all() and np.abs(j1).max() > 0
    o = O.OracleWorld(sc, external_order=True)
    o.set_bodies(b0)
    o.set_contacts(c0)
    o.set_joint_impulses(j0)
    o.narrowphase()
    for c in c1:
        o.set_arbiter_color(c["shape1"], c["shape2"], c["color"])
    o.set_joint_colors(k1)
    o.step(sc["dt"], narrow=False)
    ob = o.bodies()
    dyn = b1["motion_type"] == abi.MOTION_DYNAMIC
    err = np.maximum(np.abs(b1["velocity"][dyn] - ob["velocity"][dyn]).max(axis=1),
                     np.abs(b1["angular_velocity"][dyn] - ob["angular_velocity"][dyn]).max(axis=1))
    jerr = np.abs(j1 - o.joint_impulses(len(j1))).max(axis=1) / np.maximum(1.0, np.abs(j1).max(axis=1))
    assert np.mean(err < 1e-3) >= 0.999, (np.mean(err < 1e-3), np.sort(err)[-5:])
    assert np.mean(jerr < 1e-3) >= 0.999, np.sort(jerr)[-5:]


def test_colours_are_conflict_free():
    sc, w = _settled_pile(n=300, steps=30, seed=5)
    c = w.contacts()
    b = w.bodies()
    dyn = b["motion_type"] == abi.MOTION_DYNAMIC
    seen = {}
    arbs = {}
    for r in c:
        arbs[(int(r["shape1"]), int(r["shape2"]))] = (int(r["body1"]), int(r["body2"]), int(r["color"]))
    for (b1, b2, col) in arbs.values():
        for body in (b1, b2):
            if not dyn[body]:
                continue
            key = (body, col)
            assert key not in seen, "two rows of colour %d share body %d" % (col, body)
            seen[key] = True


def test_box_grid_settles_without_explosion():
    sc = scenes.box_grid()
    w = world_for_scene(sc)
    for _ in range(300):
        w.step(sc["dt"])
    b = w.bodies()
    dyn = b["motion_type"] == abi.MOTION_DYNAMIC
    # ten-high columns sway and may shed a top box, which then falls freely from about 10 m
    # (under 15 m/s); nothing tunnels through the ground and nothing blows up
    assert np.abs(b["velocity"][dyn]).max() < 15.0
    assert np.sum(np.abs(b["velocity"][dyn]).max(axis=1) > 3.0) <= 5
    assert b["position"][dyn, 1].min() > 0.3
    c = w.counters()
    assert c["status"] == 0 and c["contacts"] > 1000


def test_cuda_graph_step_equals_stream_step():
    # the step captured once per arbiter-buffer parity and replayed gives the same bits
    sc = scenes.mixed_pile(n=300, box=(15.0, 6.0, 15.0), y0=0.0, cells=8, seed=13, lattice=2.5)
    a = world_for_scene(sc)
    b = world_for_scene(sc, use_graph=1)
    for _ in range(60):
        a.step(sc["dt"])
        b.step(sc["dt"])
    ba, bb = a.bodies(), b.bodies()
    assert np.array_equal(ba["position"], bb["position"])
    assert np.array_equal(ba["velocity"], bb["velocity"])
    assert b.counters()["status"] == 0 and b.counters()["contacts"] == a.counters()["contacts"]


def test_invalid_dt_raises_argument_exception():
    from jitterphysics2_gb300.world import ArgumentException
    sc = scenes.box_grid(n_side=2)
    w = world_for_scene(sc)
    with pytest.raises(ArgumentException):
        w.step(-0.01)
    with pytest.raises(ArgumentException):
        w.step(float("nan"))
    w.step(0.0)  # a zero step does nothing (World.Step.cs:163)


def test_state_export_import_round_trip():
    sc, w = _settled_pile(n=200, steps=20, seed=3)
    s = w.export_state()
    w.step(sc["dt"])
    a = w.bodies()
    w.import_state(s)
    w.step(sc["dt"])
    b = w.bodies()
    assert np.array_equal(a["position"], b["position"])


def test_stabilize_matches_the_oracle():
    """World.Stabilize on a formed pile: the present contacts re-solved with 10 iterations and
    2 relaxation passes, no integration; the oracle replays it in the GPU's order."""
    sc, w = _settled_pile(n=300, steps=120, seed=43)
    b0, c0 = w.bodies(), w.contacts()
    w.stabilize(sc["dt"], 10, 2)
    b1, c1 = w.bodies(), w.contacts()
    assert np.array_equal(b0["position"], b1["position"]) and np.array_equal(b0["orientation"], b1["orientation"])
    assert w.counters()["status"] == 0 and len(c1) > 100
    o = O.OracleWorld(sc, external_order=True)
    o.set_bodies(b0)
    o.set_contacts(c0)
    for c in c1:
        o.set_arbiter_color(c["shape1"], c["shape2"], c["color"])
    o.stabilize(sc["dt"], 10, 2)
    ob = o.bodies()
    dyn = b1["motion_type"] == abi.MOTION_DYNAMIC
    err = np.maximum(np.abs(b1["velocity"][dyn] - ob["velocity"][dyn]).max(axis=1),
                     np.abs(b1["angular_velocity"][dyn] - ob["angular_velocity"][dyn]).max(axis=1))
    assert np.mean(err < 1e-3) >= 0.999, np.sort(err)[-5:]
    from jitterphysics2_gb300.world import ArgumentException
    for args in ((-0.01, 4, 0), (0.01, 0, 0), (0.01, 4, -1), (float("nan"), 4, 0)):
        with pytest.raises(ArgumentException):
            w.stabilize(*args)
