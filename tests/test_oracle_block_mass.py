"""BallSocket and FixedAngle rows against the reference's block-mass cases
(Constraints/ConstraintBlockMassTests.cs), restated on the oracle: one Prepare + Iterate of
the joint alone (bias and softness zero) on a body whose inverse mass and inverse inertia
are set directly (SetMassInertia(..., setAsInverse: true)), body 0 static.  Singular,
weak, uniformly extreme and mixed extreme responses must stop exactly the responsive
motion and leave the rest, and an unrepresentable response must change nothing.
Tolerance 1e-4 (FP32) as the reference's.  FixedAngle is restated in the oracle ahead of
its device row (kind 6 here).
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi

FIXEDANGLE = 6
TOL = 1e-4
LINEAR_AXES, ANGULAR_AXES = 7, 56          # MotionAxes bits: linear x y z, angular x y z


def _world(inv_inertia, inv_mass, allowed=63, w=(0, 0, 0), v=(0, 0, 0), q=(0, 0, 0, 1)):
    b = np.zeros(2, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["orientation"][1] = q
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
    b["flags"][1] |= (63 ^ allowed) << abi.BODY_LOCKS_SHIFT
    b["linear_damping"] = b["angular_damping"] = 1.0
    b["motion_type"][0] = abi.MOTION_STATIC
    b["inv_mass"][1] = inv_mass
    b["inv_inertia"][1] = inv_inertia
    b["angular_velocity"][1] = w
    b["velocity"][1] = v
    return O.OracleWorld(dict(bodies=b, shapes=np.zeros(0, abi.SHAPE_DTYPE), hull=np.zeros((0, 3), np.float32),
                              triangles=np.zeros(0, abi.TRIANGLE_DTYPE)))


def _solve(o, kind, init=(0, 0, 0)):
    j = o.add_joint(kind, 0, 1, init)
    o.joint_solve(j, 0.01, 0.0, 0.0)
    b = o.bodies()
    return b["velocity"][1].astype(np.float64), b["angular_velocity"][1].astype(np.float64), o.joint_impulses(1)[0]


IDENT = (1, 0, 0, 1, 0, 1)


@pytest.mark.parametrize("oblique", [False, True])
@pytest.mark.parametrize("locks", [False, True])
def test_ballsocket_singular_response_keeps_the_free_rotation(locks, oblique):
    anchor = np.array([1.0, 2.0, 3.0]) / np.sqrt(14.0) if oblique else np.array([1.0, 0.0, 0.0])
    w0 = np.array([3.0, 2.0, 1.0])
    o = _world(IDENT, 0.0, ANGULAR_AXES if locks else 63, w=w0)
    v, w, _ = _solve(o, abi.CONSTRAINT_BALLSOCKET, anchor)
    anchor32 = anchor.astype(np.float32).astype(np.float64)
    assert np.abs(w - anchor32 * anchor32.dot(w0)).max() < TOL
    assert np.linalg.norm(np.cross(w, anchor32)) < TOL
    assert w @ w <= w0 @ w0 + 1e-6
    np.testing.assert_array_equal(v, 0.0)


@pytest.mark.parametrize("locks", [False, True])
def test_ballsocket_singular_response_keeps_an_independent_weak_row(locks):
    o = _world((0, 0, 0, 1e-9, 0, 1), 0.0, ANGULAR_AXES if locks else 63, w=(0, 2, 3))
    _, w, imp = _solve(o, abi.CONSTRAINT_BALLSOCKET, (1, 0, 0))
    assert np.abs(w).max() < TOL and np.isfinite(imp).all()


@pytest.mark.parametrize("locks", [False, True])
@pytest.mark.parametrize("large", [False, True])
def test_ballsocket_uniform_mass_scale_keeps_translation(large, locks):
    inv_mass = 1e20 if large else 1e-13
    o = _world((0, 0, 0, 0, 0, 0), inv_mass, LINEAR_AXES if locks else 63, v=(1, -2, 3))
    v, _, imp = _solve(o, abi.CONSTRAINT_BALLSOCKET, (0, 0, 0))
    assert np.abs(v).max() < TOL
    assert np.isfinite(imp).all()
    assert np.abs(imp.astype(np.float64) * np.float32(inv_mass) + (1, -2, 3)).max() < TOL


@pytest.mark.parametrize("allowed", [63, ANGULAR_AXES, LINEAR_AXES | 16 | 32])
def test_fixed_angle_half_turn_stops_the_responsive_rotation(allowed):
    o = _world(IDENT, 1.0, allowed, w=(0, 1, 0), q=(0, 0, 0, 1))
    j = o.add_joint(FIXEDANGLE, 0, 1, (0, 0, 0))
    b = o.bodies()
    b["orientation"][1] = (1, 0, 0, 0)
    o.set_bodies(b)
    o.joint_solve(j, 0.01, 0.0, 0.0)
    assert np.abs(o.bodies()["angular_velocity"][1]).max() < TOL
    assert np.isfinite(o.joint_impulses(1)).all()


@pytest.mark.parametrize("locks", [False, True])
def test_fixed_angle_singular_inertia_keeps_the_responsive_axes(locks):
    o = _world((0, 0, 0, 1, 0, 1), 0.0, ANGULAR_AXES if locks else 63, w=(3, 2, 1))
    _, w, imp = _solve(o, FIXEDANGLE)
    assert np.abs(w - (3, 0, 0)).max() < TOL and np.isfinite(imp).all()


@pytest.mark.parametrize("lock", [False, True])
@pytest.mark.parametrize("large", [False, True])
def test_fixed_angle_uniform_inertia_scale_keeps_the_response(large, lock):
    s = 1e20 if large else 1e-13
    o = _world((s, 0, 0, s, 0, s), 0.0, (16 | 32) if lock else 63, w=(0, -2, 3))
    _, w, imp = _solve(o, FIXEDANGLE)
    assert np.abs(w).max() < TOL and np.isfinite(imp).all()


def test_fixed_angle_mixed_extreme_inertia_keeps_every_row():
    o = _world((1e20, 0, 0, 1e20, 0, 1e-20), 0.0, w=(1, -2, 3))
    _, w, imp = _solve(o, FIXEDANGLE)
    assert np.isfinite(w).all() and np.abs(w).max() < TOL and np.isfinite(imp).all()


@pytest.mark.parametrize("angular", [False, True])
def test_unrepresentable_response_changes_nothing(angular):
    eps = float(np.finfo(np.float32).smallest_subnormal)
    w0 = np.array([1.0, -2.0, 3.0])
    if angular:
        o = _world((eps, 0, 0, eps, 0, eps), 0.0, w=w0)
        _, w, imp = _solve(o, FIXEDANGLE)
        np.testing.assert_array_equal(w, w0)
    else:
        o = _world((0, 0, 0, 0, 0, 0), eps, v=w0)
        v, _, imp = _solve(o, abi.CONSTRAINT_BALLSOCKET, (0, 0, 0))
        np.testing.assert_array_equal(v, w0)
    np.testing.assert_array_equal(imp, 0.0)
