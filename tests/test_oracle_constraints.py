"""DistanceLimit, ConeLimit and TwistAngle in the oracle (CPU).

The reference's own constraint-level cases (DistanceLimitRegressionTests.cs: a fixed
distance limit on a unit mass stops it in one iteration with impulse -1 at any separation;
coincident anchors leave the body alone and clear the cached impulse) are restated with
one Prepare + Iterate of the joint alone, bias and softness zero.  The cone and twist rows
are checked the same way against the rates they must cancel, and the limb-chain scene
(BallSocket + ConeLimit + TwistAngle per joint, a DistanceLimit per chain) against the
limits it must hold.
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi, scenes

PI = np.pi


def _pair(q1=(0, 0, 0, 1), inv_inertia=(0, 0, 0, 0, 0, 0), velocity=(0, 0, 0), angular=(0, 0, 0)):
    """Body 0: static at the origin (the reference's NullBody).  Body 1: unit inverse mass."""
    b = np.zeros(2, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
    b["linear_damping"] = b["angular_damping"] = 1.0
    b["motion_type"][0] = abi.MOTION_STATIC
    b["orientation"][1] = q1
    b["inv_mass"][1] = 1.0
    b["inv_inertia"][1] = inv_inertia
    b["velocity"][1] = velocity
    b["angular_velocity"][1] = angular
    sc = dict(bodies=b, shapes=np.zeros(0, abi.SHAPE_DTYPE), hull=np.zeros((0, 3), np.float32),
              triangles=np.zeros(0, abi.TRIANGLE_DTYPE))
    return O.OracleWorld(sc)


FIXED = (1e-6, -1e-6)   # LinearLimit.Fixed / AngularLimit.Fixed


@pytest.mark.parametrize("separation", [1e-3, 1e-7, 1e-10])
def test_fixed_distance_stops_a_unit_mass_at_any_separation(separation):
    o = _pair(velocity=(0, 1, 0))
    j = o.add_joint(abi.CONSTRAINT_DISTANCELIMIT, 0, 1, (0, 0, 0, 0, separation, 0) + FIXED)
    o.joint_solve(j, 0.01, 0.0, 0.0)
    assert o.joint_impulses(1)[0, 0] == pytest.approx(-1.0, abs=1e-5)
    assert np.linalg.norm(o.bodies()["velocity"][1]) < 1e-5


def test_coincident_anchors_leave_the_body_and_clear_the_cached_impulse():
    o = _pair(velocity=(0, 1, 0))
    j = o.add_joint(abi.CONSTRAINT_DISTANCELIMIT, 0, 1, (0, 0, 0, 0, 0, 0) + FIXED)
    o.set_joint_impulses([[-1.0, 0.0, 0.0]])
    o.joint_solve(j, 0.01, 0.0, 0.0)
    assert o.joint_impulses(1)[0, 0] == 0.0
    np.testing.assert_array_equal(o.bodies()["velocity"][1], (0, 1, 0))


def _qz(angle):
    return (0.0, 0.0, np.sin(angle / 2), np.cos(angle / 2))


def _qx(angle):
    return (np.sin(angle / 2), 0.0, 0.0, np.cos(angle / 2))


@pytest.mark.parametrize("spin, stopped", [(1.0, True), (-1.0, False)])
def test_cone_beyond_its_limit_stops_only_the_opening_rate(spin, stopped):
    # body 1's axis is turned 0.6 rad about z from body 0's, past the 0.5 rad cone: a spin
    # opening the cone further is cancelled, one closing it is left alone
    o = _pair(q1=_qz(0.6), inv_inertia=(1, 0, 0, 1, 0, 1), angular=(0, 0, spin))
    a2 = (np.cos(0.6), np.sin(0.6), 0.0)
    j = o.add_joint(abi.CONSTRAINT_CONELIMIT, 0, 1, (1, 0, 0) + a2 + (0.0, 0.5))
    o.joint_solve(j, 0.01, 0.0, 0.0)
    w = o.bodies()["angular_velocity"][1]
    if stopped:
        assert np.abs(w).max() < 1e-6 and o.joint_impulses(1)[0, 0] < 0
    else:
        np.testing.assert_allclose(w, (0, 0, spin), atol=1e-7)
        assert o.joint_impulses(1)[0, 0] == 0.0


@pytest.mark.parametrize("spin, stopped", [(1.0, True), (-1.0, False)])
def test_twist_beyond_its_limit_stops_only_the_outward_rate(spin, stopped):
    # both axes along x, the joint created at rest; body 1 is then turned 0.4 rad about x,
    # past the 0.3 rad twist limit
    o = _pair(inv_inertia=(1, 0, 0, 1, 0, 1))
    j = o.add_joint(abi.CONSTRAINT_TWISTANGLE, 0, 1, (1, 0, 0, 1, 0, 0, -0.3, 0.3))
    b = o.bodies()
    b["orientation"][1] = _qx(0.4)
    b["angular_velocity"][1] = (spin, 0, 0)
    o.set_bodies(b)
    o.joint_solve(j, 0.01, 0.0, 0.0)
    w = o.bodies()["angular_velocity"][1]
    if stopped:
        assert np.abs(w).max() < 1e-6
    else:
        np.testing.assert_allclose(w, (spin, 0, 0), atol=1e-7)


def _quat_mul(a, b):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    return np.array([aw * bx + bw * ax + ay * bz - az * by, aw * by + bw * ay + az * bx - ax * bz,
                     aw * bz + bw * az + ax * by - ay * bx, aw * bw - (ax * bx + ay * by + az * bz)])


def _rot(q, v):
    x, y, z, w = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    return R @ np.asarray(v, np.float64)


def chain_limits(sc, b):
    """Cone angles, twist angles (TwistAngle.Angle, TwistAngle.cs:240-258, with Q0 = 1 and
    B = x for the limb chains) and anchor-to-last-link distances of a limb-chain state."""
    cones, twists, dists = [], [], []
    q = b["orientation"].astype(np.float64)
    for kind, i, k, init in sc["joints"]:
        if kind == abi.CONSTRAINT_CONELIMIT:
            a1, a2 = _rot(q[i], (1, 0, 0)), _rot(q[k], (1, 0, 0))
            cones.append(np.arctan2(np.linalg.norm(np.cross(a1, a2)), np.dot(a1, a2)))
        elif kind == abi.CONSTRAINT_TWISTANGLE:
            c = q[i] * (-1, -1, -1, 1)
            r = _quat_mul(c, q[k])
            if r[3] < 0:
                r = -r
            proj = r[0]
            perp = r[:3] - np.array([proj, 0, 0])
            twists.append(2 * np.arctan2(proj, np.sqrt(r[3] ** 2 + perp @ perp)))
        elif kind == abi.CONSTRAINT_DISTANCELIMIT:
            dists.append(np.linalg.norm(b["position"][k].astype(np.float64) - b["position"][i]))
    return np.array(cones), np.array(twists), np.array(dists)


def test_limb_chains_hold_their_limits():
    sc = scenes.limb_chains(n_chains=4)
    o = O.OracleWorld(sc)
    for _ in range(120):
        o.step(sc["dt"])
    cones, twists, dists = chain_limits(sc, o.bodies())
    assert cones.max() < 0.5 + 0.03 and cones.max() > 0.3
    assert np.abs(twists).max() < 0.3 + 0.03
    assert dists.max() < 6.0 + 0.01 and dists.min() > 3.0 - 0.01


def test_limb_chains_in_float_follow_double():
    sc = scenes.limb_chains(n_chains=4)
    f, d = O.OracleWorld(sc, real="f"), O.OracleWorld(sc, real="d")
    for _ in range(30):
        f.step(sc["dt"])
        d.step(sc["dt"])
    np.testing.assert_allclose(f.bodies()["position"], d.bodies()["position"], atol=2e-3)
