"""Islands and sleeping on the device (World.AllowDeactivation, World.cs:333; CheckDeactivation,
World.Step.cs:1289-1371; IslandHelper.cs), through the C ABI, against the oracle's restatement.

- Lockstep: a box grid stepped on the GPU and, from the same start, in the oracle replaying
  the GPU's solve order every step: positions, velocities and every body's active flag agree
  bit for bit through the fall, the rest and the sleep.
- The reference's SleepTests (Behavior/SleepTests.cs), on the device: a body's deactivation
  time, the static body going inactive, a stack sleeping and waking together, kinematic bodies
  kept awake by motion and sleeping once stopped; a dropped box waking only the island it
  strikes; no sleep without deactivation.
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi, scenes
from jitterphysics2_gb300.world import world_for_scene

pytestmark = pytest.mark.gpu


def awake(bodies):
    return (bodies["flags"] & abi.BODY_ACTIVE) != 0


def with_sleep(sc):
    sc = dict(sc)
    sc["params"] = dict(sc.get("params", {}), allow_deactivation=1)
    return sc


def test_box_grid_sleeps_in_lockstep_with_the_oracle():
    sc = with_sleep(scenes.box_grid(n_side=3))
    g = world_for_scene(sc)
    o = O.OracleWorld(sc, external_order=True)
    dyn = sc["bodies"]["motion_type"] == abi.MOTION_DYNAMIC
    asleep_at = None
    for s in range(1, 361):
        g.step(sc["dt"])
        o.narrowphase()
        for c in g.contacts():
            o.set_arbiter_color(c["shape1"], c["shape2"], c["color"])
        o.step(sc["dt"], narrow=False)
        gb, ob = g.bodies(), o.bodies()
        assert np.array_equal(awake(gb), awake(ob)), s
        assert np.array_equal(gb["position"], ob["position"]), s
        assert np.array_equal(gb["velocity"], ob["velocity"]), s
        if asleep_at is None and not awake(gb)[dyn].any():
            asleep_at = s
            frozen = gb["position"].copy()
    assert asleep_at is not None and 100 < asleep_at < 300, asleep_at
    assert np.array_equal(g.bodies()["position"], frozen)
    assert g.counters()["arbiters"] > 0 and g.counters()["status"] == 0  # sleeping contacts are kept


def test_without_deactivation_nothing_sleeps():
    sc = scenes.box_grid(n_side=3)
    g = world_for_scene(sc)
    for _ in range(360):
        g.step(sc["dt"])
    assert awake(g.bodies()).all()


def _pile_and_a_dropped_box(height=30.0):
    sc = scenes.box_grid(n_side=2)
    b, s = sc["bodies"], sc["shapes"]
    nb = np.concatenate([b, b[1:2]])
    ns = np.concatenate([s, s[1:2]])
    k = len(b)
    nb["position"][k] = (b["position"][1][0], height, b["position"][1][2])
    ns["body"][k] = k
    return with_sleep(dict(sc, bodies=nb, shapes=ns)), k


def test_a_new_contact_wakes_only_the_island_it_touches():
    sc, dropped = _pile_and_a_dropped_box()
    g = world_for_scene(sc)
    b0 = sc["bodies"]
    pile = np.arange(1, dropped)
    same_column = pile[np.linalg.norm(b0["position"][pile][:, [0, 2]] - b0["position"][dropped, [0, 2]], axis=1) < 0.5]
    other = np.setdiff1d(pile, same_column)
    slept = woke = False
    for _ in range(500):
        g.step(sc["dt"])
        aw = awake(g.bodies())
        if not aw[pile].any():
            slept = True
        if slept and aw[same_column].all():
            woke = True
            assert not aw[other].any()
            break
    assert slept and woke and awake(g.bodies())[dropped]


def _lone_bodies(n, motion=abi.MOTION_DYNAMIC, boxes=None):
    b = np.zeros(n, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY | abi.BODY_GYROSCOPIC
    b["linear_damping"] = 0.998
    b["angular_damping"] = 0.995
    b["friction"] = 0.2
    b["motion_type"] = motion
    b["inv_mass"] = 0.0 if motion != abi.MOTION_DYNAMIC else 1.0
    b["inv_inertia"] = 0.0 if motion != abi.MOTION_DYNAMIC else (1, 0, 0, 1, 0, 1)
    s = np.zeros(0, abi.SHAPE_DTYPE) if boxes is None else boxes
    return dict(bodies=b, shapes=s, hull=np.zeros((0, 3), np.float32), triangles=np.zeros(0, abi.TRIANGLE_DTYPE),
                params=dict(gravity=(0.0, 0.0, 0.0), allow_deactivation=1), dt=0.01)


def _advance(w, seconds, dt=0.01):
    for _ in range(int(round(seconds / dt))):
        w.step(dt)


def _unit_box():
    s = np.zeros(1, abi.SHAPE_DTYPE)
    s["kind"] = abi.SHAPE_BOX
    s["dims"][0, :3] = 0.5
    return s


def test_deactivation_time_of_a_body():
    # SleepTests.DeactivationTime (SleepTests.cs:38-84)
    w = world_for_scene(_lone_bodies(1, boxes=_unit_box()))
    w.set_body_sleep(0, 3.0)
    assert awake(w.bodies())[0]
    _advance(w, 1)
    assert awake(w.bodies())[0]
    _advance(w, 3)
    assert not awake(w.bodies())[0]
    w.set_body_sleep(0, 5.0)
    w.activate_body(0)
    assert not awake(w.bodies())[0]            # the request takes effect at the next step
    _advance(w, 1)
    assert awake(w.bodies())[0]
    _advance(w, 3)
    assert awake(w.bodies())[0]
    _advance(w, 2)
    assert not awake(w.bodies())[0]


def test_a_static_body_goes_inactive():
    # SleepTests.StaticBodySleepingAndWake (SleepTests.cs:5-36), its first step
    w = world_for_scene(_lone_bodies(1, abi.MOTION_STATIC, _unit_box()))
    _advance(w, 1)
    assert not awake(w.bodies())[0]


def test_a_stack_sleeps_and_wakes_together():
    # SleepTests.StackedSleeping (SleepTests.cs:125-168)
    s = np.zeros(3, abi.SHAPE_DTYPE)
    s["kind"] = abi.SHAPE_BOX
    s["body"] = (0, 1, 2)
    s["dims"][:, :3] = 0.5
    sc = _lone_bodies(3, boxes=s)
    b = sc["bodies"]
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_GYROSCOPIC
    b["position"][:, 1] = (0.0, 1.0, 2.0)
    b["motion_type"][0] = abi.MOTION_STATIC
    b["inv_mass"][0] = 0.0
    b["inv_inertia"][0] = 0.0
    sc["params"] = dict(allow_deactivation=1)
    w = world_for_scene(sc)
    _advance(w, 3)
    assert not awake(w.bodies()).any()
    w.activate_body(1)
    _advance(w, 0.01)
    assert awake(w.bodies())[1] and awake(w.bodies())[2]
    _advance(w, 2)
    assert not awake(w.bodies())[1] and not awake(w.bodies())[2]


@pytest.mark.parametrize("speed", [0.2, 1e-25])
@pytest.mark.parametrize("angular", [False, True])
def test_a_moving_kinematic_body_stays_awake(angular, speed):
    # SleepTests.MovingKinematicBodyStaysAwake (SleepTests.cs:290-322)
    sc = _lone_bodies(1, abi.MOTION_KINEMATIC, _unit_box())
    v = np.array([0.0, speed, 0.0]) if angular else np.array([speed, 0.0, 0.0])
    sc["bodies"]["angular_velocity" if angular else "velocity"][0] = v
    w = world_for_scene(sc)
    w.set_body_sleep(0, 0.5)
    _advance(w, 3)
    b = w.bodies()
    assert awake(b)[0]
    np.testing.assert_array_equal(b["angular_velocity" if angular else "velocity"][0], v.astype(np.float32))


@pytest.mark.parametrize("angular", [False, True])
def test_a_kinematic_body_sleeps_once_it_stops(angular):
    # SleepTests.KinematicBodySleepsAfterMotionStops (SleepTests.cs:348-366)
    sc = _lone_bodies(1, abi.MOTION_KINEMATIC, _unit_box())
    sc["bodies"]["angular_velocity" if angular else "velocity"][0] = (0, 0.2, 0) if angular else (0.2, 0, 0)
    w = world_for_scene(sc)
    w.set_body_sleep(0, 0.1)
    _advance(w, 1)
    assert awake(w.bodies())[0]
    b = w.bodies()
    b["angular_velocity"][0] = 0.0
    b["velocity"][0] = 0.0
    w.set_bodies(b)
    _advance(w, 1)
    assert not awake(w.bodies())[0]


def test_sleep_settings_reject_invalid_values():
    w = world_for_scene(_lone_bodies(1, boxes=_unit_box()))
    for args in ((-1.0, 0.1, 0.1), (1.0, float("nan"), 0.1)):
        with pytest.raises(abi.JitterError):
            w.set_body_sleep(0, *args)
    with pytest.raises(abi.JitterError):
        w.activate_body(5)
