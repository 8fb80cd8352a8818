"""DistanceLimit, ConeLimit and TwistAngle on the GPU against the oracle, through the C ABI.

The limb-chain scene joins boxes the way a ragdoll limb is joined (BallSocket + ConeLimit +
TwistAngle per joint, a DistanceLimit per chain).  One step from the GPU's state is
replayed in the oracle in the GPU's order keys, warm-started with the GPU's impulses:
velocities within 1e-3, impulses within 1e-3 relative.  Over 240 steps the GPU holds the
limits.  Run side by side from the start, the GPU (colour order) and the oracle (creation
order) solve the shared-body rows of a chain in different, equally valid Gauss-Seidel
orders, so their trajectories separate slowly: 2.7e-3 after 30 steps was measured, and the
side-by-side check allows 1e-2.  The limits are soft (softness 0.001, bias 0.2, 8
iterations on 6-link chains): the oracle itself, in its creation order and in reversed and
random valid orders, lets a cone angle overshoot its 0.5 rad limit by up to 0.11 rad over
240 steps and a twist its 0.3 rad limit by up to 0.006, so the GPU is held to the same
bands (0.15 and 0.05).
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi, scenes
from jitterphysics2_gb300.world import world_for_scene
from test_oracle_constraints import chain_limits

pytestmark = pytest.mark.gpu


def test_one_step_of_limb_chains_matches_the_oracle():
    sc = scenes.limb_chains(n_chains=16)
    w = world_for_scene(sc)
    for _ in range(60):
        w.step(sc["dt"])
    b0 = w.bodies()
    _, j0 = w.constraints()
    w.step(sc["dt"])
    b1 = w.bodies()
    k1, j1 = w.constraints()
    assert np.abs(j1).max() > 0
    o = O.OracleWorld(sc, external_order=True)
    o.set_bodies(b0)
    o.set_joint_impulses(j0)
    o.narrowphase()
    o.set_joint_colors(k1)
    o.step(sc["dt"], narrow=False)
    ob = o.bodies()
    dyn = b1["motion_type"] == abi.MOTION_DYNAMIC
    err = np.maximum(np.abs(b1["velocity"][dyn] - ob["velocity"][dyn]).max(axis=1),
                     np.abs(b1["angular_velocity"][dyn] - ob["angular_velocity"][dyn]).max(axis=1))
    jerr = np.abs(j1 - o.joint_impulses(len(j1))).max(axis=1) / np.maximum(1e-3, np.abs(j1).max(axis=1))
    assert err.max() < 1e-3, np.sort(err)[-5:]
    assert np.mean(jerr < 1e-3) > 0.95, np.sort(jerr)[-5:]


def test_limb_chains_hold_their_limits_and_follow_the_oracle():
    sc = scenes.limb_chains(n_chains=16)
    w = world_for_scene(sc)
    o = O.OracleWorld(sc)
    for _ in range(30):
        w.step(sc["dt"])
        o.step(sc["dt"])
    np.testing.assert_allclose(w.bodies()["position"], o.bodies()["position"], atol=1e-2)
    for _ in range(210):
        w.step(sc["dt"])
    cones, twists, dists = chain_limits(sc, w.bodies())
    assert cones.max() < 0.5 + 0.15
    assert np.abs(twists).max() < 0.3 + 0.05
    assert dists.max() < 6.0 + 0.05 and dists.min() > 3.0 - 0.05


@pytest.mark.parametrize("kind, init", [
    (abi.CONSTRAINT_CONELIMIT, (1, 0, 0, 1, 0, 0, 0.0, 0.0)),          # fixed tilt of zero
    (abi.CONSTRAINT_CONELIMIT, (1, 0, 0, 1, 0, 0, np.pi, np.pi)),      # fixed tilt of pi
    (abi.CONSTRAINT_CONELIMIT, (1, 0, 0, 1, 0, 0, 0.6, 0.5)),          # min above max
    (abi.CONSTRAINT_CONELIMIT, (1, 0, 0, 1, 0, 0, -0.1, 0.5)),         # below zero
    (abi.CONSTRAINT_CONELIMIT, (0, 0, 0, 1, 0, 0, 0.0, 0.5)),          # zero axis
    (abi.CONSTRAINT_TWISTANGLE, (1, 0, 0, 1, 0, 0, -np.inf, 0.5)),     # infinite limit
    (abi.CONSTRAINT_DISTANCELIMIT, (0, 0, 0, 1, 0, 0, np.nan, 0.0)),   # NaN limit
    (abi.CONSTRAINT_DISTANCELIMIT, (0, np.inf, 0, 1, 0, 0, 0.0, 0.0)),  # infinite anchor
])
def test_invalid_constraint_arguments_raise(kind, init):
    sc = scenes.limb_chains(n_chains=1, links=2)
    w = world_for_scene(sc)
    with pytest.raises(abi.JitterError) as e:
        w.add_constraint(kind, 1, 2, init)
    assert e.value.code == abi.JG_ERR_INVALID_ARG


# ---- FixedAngle, PointOnPlane, AngularMotor, LinearMotor ----------------------------------
def _quat_rotate(q, v):
    q = np.asarray(q, np.float64)
    u, w = q[..., :3], q[..., 3:]
    t = 2 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def test_one_step_of_mechanism_chains_matches_the_oracle():
    """Motor, weld, plane and slider rows (scenes.mechanism_chains): one step from the GPU's
    state replayed in the oracle in the GPU's order keys, warm-started with the GPU's
    impulses."""
    sc = scenes.mechanism_chains(n_chains=16)
    w = world_for_scene(sc)
    for _ in range(40):
        w.step(sc["dt"])
    b0 = w.bodies()
    _, j0 = w.constraints()
    w.step(sc["dt"])
    b1 = w.bodies()
    k1, j1 = w.constraints()
    o = O.OracleWorld(sc, external_order=True)
    o.set_bodies(b0)
    o.set_joint_impulses(j0)
    o.narrowphase()
    o.set_joint_colors(k1)
    o.step(sc["dt"], narrow=False)
    ob = o.bodies()
    dyn = b1["motion_type"] == abi.MOTION_DYNAMIC
    err = np.maximum(np.abs(b1["velocity"][dyn] - ob["velocity"][dyn]).max(axis=1),
                     np.abs(b1["angular_velocity"][dyn] - ob["angular_velocity"][dyn]).max(axis=1))
    jo = o.joint_impulses(len(j1))
    jerr = np.abs(j1 - jo).max(axis=1) / np.maximum(1e-3, np.abs(j1).max(axis=1))
    kinds = np.array([j[0] for j in sc["joints"]])
    for kind in (abi.CONSTRAINT_FIXEDANGLE, abi.CONSTRAINT_POINTONPLANE, abi.CONSTRAINT_ANGULARMOTOR,
                 abi.CONSTRAINT_LINEARMOTOR):
        assert np.abs(j1[kinds == kind]).max() > 0, kind     # every kind carries an impulse
    assert err.max() < 1e-3, np.sort(err)[-5:]
    assert np.mean(jerr < 1e-3) >= 0.999, np.sort(jerr)[-5:]


def test_mechanism_chains_keep_their_welds_planes_and_drives():
    sc = scenes.mechanism_chains(n_chains=8)
    w = world_for_scene(sc)
    q0 = sc["bodies"]["orientation"].astype(np.float64)
    for _ in range(200):
        w.step(sc["dt"])
    b = w.bodies()
    assert w.counters()["status"] == 0
    q = b["orientation"].astype(np.float64)
    per = 5
    for c in range(8):
        a = c * per
        # welded links keep their relative rotation: conj(q1) q2 unchanged
        for l1, l2 in ((a + 1, a + 2), (a + 3, a + 4)):
            def rel(qq):
                x1 = np.array([-qq[l1][0], -qq[l1][1], -qq[l1][2], qq[l1][3]])
                x2 = qq[l2]
                return np.array([x1[3] * x2[0] + x1[0] * x2[3] + x1[1] * x2[2] - x1[2] * x2[1],
                                 x1[3] * x2[1] - x1[0] * x2[2] + x1[1] * x2[3] + x1[2] * x2[0],
                                 x1[3] * x2[2] + x1[0] * x2[1] - x1[1] * x2[0] + x1[2] * x2[3],
                                 x1[3] * x2[3] - x1[0] * x2[0] - x1[1] * x2[1] - x1[2] * x2[2]])
            r0, r1 = rel(q0), rel(q)
            assert min(np.abs(r1 - r0).max(), np.abs(r1 + r0).max()) < 0.02
        # the plane of link 2 holds link 3's anchor (its centre) at zero height in link 2's frame
        n = _quat_rotate(q[a + 2], np.array([0.0, 1.0, 0.0]))
        assert abs((b["position"][a + 3] - b["position"][a + 2]) @ n) < 0.02
        # the angular motor spins link 1 about the chain axis at its target (2 rad/s)
        axis0 = _quat_rotate(q[a], np.array([1.0, 0.0, 0.0]))
        axis1 = _quat_rotate(q[a + 1], np.array([1.0, 0.0, 0.0]))
        assert abs(b["angular_velocity"][a + 1] @ axis1 - b["angular_velocity"][a] @ axis0 - 2.0) < 0.2


@pytest.mark.parametrize("kind, init", [
    (abi.CONSTRAINT_POINTONPLANE, (0, 0, 0) + (0, 0, 0) + (1, 0, 0) + (0.0, 0.0)),    # zero axis
    (abi.CONSTRAINT_POINTONPLANE, (0, 1, 0) + (0, 0, 0) + (1, 0, 0) + (np.nan, 0.0)), # NaN limit
    (abi.CONSTRAINT_ANGULARMOTOR, (1, 0, 0, 0, 0, 0, 1.0, 1.0)),                      # zero axis
    (abi.CONSTRAINT_LINEARMOTOR, (1, 0, 0, 1, 0, 0, 1.0, -1.0)),                      # negative force
])
def test_invalid_mechanism_arguments_raise(kind, init):
    sc = scenes.mechanism_chains(n_chains=1)
    w = world_for_scene(sc)
    with pytest.raises(abi.JitterError) as e:
        w.add_constraint(kind, 1, 2, init)
    assert e.value.code == abi.JG_ERR_INVALID_ARG
