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
