"""Islands and sleeping in the oracle (CPU): World.AllowDeactivation (World.cs:333).

The oracle restates the reference's deactivation: islands are the connected components of
non-static bodies joined by arbiters and constraints (IslandHelper.cs); a body at rest
(|v|^2 and |w|^2 below 0.1) for the deactivation time (1 s) stops marking its island
(RigidBody.cs:723-743); an island nobody marked goes to sleep at the next step's
CheckDeactivation (World.Step.cs:1289-1371), and a new arbiter wakes the islands of both its
bodies (HandleDeferredArbiters / AddToActiveList, World.Step.cs:880-914, World.cs:903-910).
Sleeping bodies are not integrated and their contacts are neither solved nor updated.
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi, scenes


def _awake(o):
    return (o.bodies()["flags"] & abi.BODY_ACTIVE) != 0


def test_a_resting_pile_falls_asleep_and_stays_still():
    sc = scenes.box_grid(n_side=3)
    o = O.OracleWorld(sc)
    o.allow_deactivation(True)
    dyn = sc["bodies"]["motion_type"] == abi.MOTION_DYNAMIC
    asleep_at = None
    for s in range(1, 401):
        o.step(sc["dt"])
        if asleep_at is None and not _awake(o)[dyn].any():
            asleep_at = s
            frozen = o.bodies()["position"].copy()
    # the pile settles within about a second and then rests for the deactivation time
    assert asleep_at is not None and 100 < asleep_at < 300, asleep_at
    assert not _awake(o)[~dyn].any()          # the static ground's island sleeps as well
    np.testing.assert_array_equal(o.bodies()["position"], frozen)
    assert o.counters()["arbiters"] > 0       # sleeping contacts are kept


def test_without_deactivation_nothing_sleeps():
    sc = scenes.box_grid(n_side=3)
    o = O.OracleWorld(sc)
    for _ in range(400):
        o.step(sc["dt"])
    assert _awake(o).all()


def _pile_and_a_dropped_box(height=30.0):
    sc = scenes.box_grid(n_side=2)
    b, s = sc["bodies"], sc["shapes"]
    nb = np.concatenate([b, b[1:2]])
    ns = np.concatenate([s, s[1:2]])
    k = len(b)
    nb["position"][k] = (b["position"][1][0], height, b["position"][1][2])
    ns["body"][k] = k
    sc = dict(sc, bodies=nb, shapes=ns)
    return sc, k


def test_a_new_contact_wakes_only_the_island_it_touches():
    sc, dropped = _pile_and_a_dropped_box()
    o = O.OracleWorld(sc)
    o.allow_deactivation(True)
    b0 = sc["bodies"]
    pile = np.arange(1, dropped)
    same_column = pile[np.linalg.norm(b0["position"][pile][:, [0, 2]] - b0["position"][dropped, [0, 2]], axis=1) < 0.5]
    other = np.setdiff1d(pile, same_column)
    slept = woke = False
    for _ in range(500):
        o.step(sc["dt"])
        aw = _awake(o)
        if not aw[pile].any():
            slept = True
        if slept and aw[same_column].all():
            woke = True
            assert not aw[other].any()
            break
    assert slept and woke
    # the struck column moves again, then settles
    assert _awake(o)[dropped]


def test_deactivation_keeps_the_default_path_unchanged_until_sleep():
    # before any island sleeps, the step with deactivation is the step without it
    sc = scenes.box_grid(n_side=2)
    a, b = O.OracleWorld(sc), O.OracleWorld(sc)
    b.allow_deactivation(True)
    for _ in range(60):
        a.step(sc["dt"])
        b.step(sc["dt"])
    np.testing.assert_array_equal(a.bodies()["position"], b.bodies()["position"])


# ---- the reference's SleepTests (Behavior/SleepTests.cs), restated --------------------------
def _lone_bodies(n, motion=abi.MOTION_DYNAMIC, boxes=None):
    """n bodies of the reference's defaults (mass 1, identity inertia) without gravity."""
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
                params=dict(gravity=(0.0, 0.0, 0.0)))


def _advance(o, seconds, dt=0.01):
    for _ in range(int(seconds / dt)):
        o.step(dt)


def test_deactivation_time_of_a_body():
    # SleepTests.DeactivationTime (SleepTests.cs:38-84)
    o = O.OracleWorld(_lone_bodies(1))
    o.allow_deactivation(True)
    o.deactivation_time(0, 3.0)
    assert _awake(o)[0]
    _advance(o, 1)
    assert _awake(o)[0]
    _advance(o, 3)
    assert not _awake(o)[0]
    o.deactivation_time(0, 5.0)
    o.activate(0)
    assert not _awake(o)[0]           # the request takes effect at the next step
    _advance(o, 1)
    assert _awake(o)[0]
    _advance(o, 3)
    assert _awake(o)[0]
    _advance(o, 2)
    assert not _awake(o)[0]


def test_a_static_body_goes_inactive():
    # SleepTests.StaticBodySleepingAndWake (SleepTests.cs:5-36), its first step
    s = np.zeros(1, abi.SHAPE_DTYPE)
    s["kind"] = abi.SHAPE_BOX
    s["dims"][0, :3] = 0.5
    o = O.OracleWorld(_lone_bodies(1, abi.MOTION_STATIC, s))
    o.allow_deactivation(True)
    _advance(o, 1)
    assert not _awake(o)[0]


def test_a_stack_sleeps_and_wakes_together():
    # SleepTests.StackedSleeping (SleepTests.cs:125-168): a static base and two unit boxes
    # stacked on it; waking the middle box wakes the top one through their contact
    s = np.zeros(3, abi.SHAPE_DTYPE)
    s["kind"] = abi.SHAPE_BOX
    s["body"] = (0, 1, 2)
    s["dims"][:, :3] = 0.5
    sc = _lone_bodies(3, boxes=s)
    b = sc["bodies"]
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_GYROSCOPIC          # gravity on, as the reference's world
    b["position"][:, 1] = (0.0, 1.0, 2.0)
    b["motion_type"][0] = abi.MOTION_STATIC
    b["inv_mass"][0] = 0.0
    b["inv_inertia"][0] = 0.0
    sc["params"] = {}
    o = O.OracleWorld(sc)
    o.allow_deactivation(True)
    _advance(o, 3)
    assert not _awake(o).any()
    o.activate(1)
    _advance(o, 0.01)
    assert _awake(o)[1] and _awake(o)[2]
    _advance(o, 2)
    assert not _awake(o)[1] and not _awake(o)[2]


@pytest.mark.parametrize("deactivation", [0.0, 0.5])
@pytest.mark.parametrize("speed", [0.2, 1e-7, 1e-25])
@pytest.mark.parametrize("angular", [False, True])
def test_a_moving_kinematic_body_stays_awake(angular, speed, deactivation):
    # SleepTests.MovingKinematicBodyStaysAwake (SleepTests.cs:290-322)
    s = np.zeros(1, abi.SHAPE_DTYPE)
    s["kind"] = abi.SHAPE_BOX
    s["dims"][0, :3] = 0.5
    sc = _lone_bodies(1, abi.MOTION_KINEMATIC, s)
    v = np.array([0.0, speed, 0.0]) if angular else np.array([speed, 0.0, 0.0])
    if angular:
        sc["bodies"]["angular_velocity"][0] = v
    else:
        sc["bodies"]["velocity"][0] = v
    o = O.OracleWorld(sc)
    o.allow_deactivation(True)
    o.deactivation_time(0, deactivation)
    _advance(o, 3)
    b = o.bodies()
    assert _awake(o)[0]
    np.testing.assert_array_equal(b["angular_velocity" if angular else "velocity"][0], v.astype(np.float32))
    if angular:
        x, y, z, w = b["orientation"][0].astype(np.float64)
        fwd = np.array([1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w)])
        disp = np.arctan2(-fwd[2], fwd[0])
    else:
        disp = float(b["position"][0][0])
    assert disp == pytest.approx(3 * speed, rel=0.05)


@pytest.mark.parametrize("angular", [False, True])
def test_a_kinematic_body_sleeps_once_it_stops(angular):
    # SleepTests.KinematicBodySleepsAfterMotionStops (SleepTests.cs:348-366)
    s = np.zeros(1, abi.SHAPE_DTYPE)
    s["kind"] = abi.SHAPE_BOX
    s["dims"][0, :3] = 0.5
    sc = _lone_bodies(1, abi.MOTION_KINEMATIC, s)
    sc["bodies"]["angular_velocity" if angular else "velocity"][0] = (0, 0.2, 0) if angular else (0.2, 0, 0)
    o = O.OracleWorld(sc)
    o.allow_deactivation(True)
    o.deactivation_time(0, 0.1)
    _advance(o, 1)
    assert _awake(o)[0]
    b = o.bodies()
    b["angular_velocity"][0] = 0.0
    b["velocity"][0] = 0.0
    o.set_bodies(b)
    _advance(o, 1)
    assert not _awake(o)[0]
