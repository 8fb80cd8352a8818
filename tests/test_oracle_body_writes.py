"""No constraint row writes a non-dynamic body (ConstraintBodyWriteTests.cs:8-44), restated
on the oracle for every kind it has: after a Prepare + Iterate that caches an impulse, the
static or kinematic support's velocities are set to -0.0 and must come out of the next
Prepare (warm start) or Iterate bitwise unchanged, with the support first or second.
"""
import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi

FIXEDANGLE, POINTONPLANE, ANGULARMOTOR, LINEARMOTOR = 6, 7, 8, 9
KINDS = {
    "BallSocket": (abi.CONSTRAINT_BALLSOCKET, (1, 0.5, 2)),
    "DistanceLimit": (abi.CONSTRAINT_DISTANCELIMIT, (0, 0, 0, 2, 1, 3, 0.5, 1.0)),
    "PointOnPlane": (POINTONPLANE, (0, 1, 0, 0, 0, 0, 2, 1, 3, -0.5, -0.2)),
    "ConeLimit": (abi.CONSTRAINT_CONELIMIT, (1, 0, 0, 0.6, 0.8, 0, 0.0, 0.3)),
    "FixedAngle": (FIXEDANGLE, (0, 0, 0)),
    "HingeAngle": (abi.CONSTRAINT_HINGEANGLE, (0, 1, 0, -0.2, 0.2)),
    "TwistAngle": (abi.CONSTRAINT_TWISTANGLE, (1, 0, 0, 1, 0, 0, -0.1, 0.1)),
    "AngularMotor": (ANGULARMOTOR, (1, 0, 0, 1, 0, 0, 5.0, 100.0)),
    "LinearMotor": (LINEARMOTOR, (1, 0, 0, 1, 0, 0, 5.0, 100.0)),
}


@pytest.mark.parametrize("warm_start", [False, True])
@pytest.mark.parametrize("reverse", [False, True])
@pytest.mark.parametrize("support", ["static", "kinematic"])
@pytest.mark.parametrize("kind", sorted(KINDS))
def test_a_non_dynamic_body_stays_bitwise_unchanged(kind, support, reverse, warm_start):
    b = np.zeros(2, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
    b["linear_damping"] = b["angular_damping"] = 1.0
    sup, dyn = (1, 0) if reverse else (0, 1)
    b["motion_type"][sup] = abi.MOTION_STATIC if support == "static" else abi.MOTION_KINEMATIC
    b["inv_mass"][dyn] = 1.0
    b["inv_inertia"][dyn] = (1, 0, 0, 1, 0, 1)
    b["position"][dyn] = (2, 1, 3)
    b["velocity"][dyn] = (1, 2, 3)
    b["angular_velocity"][dyn] = (2, -3, 1)
    # a twisted, tilted body so that the angular limits are active
    b["orientation"][dyn] = (0.3, 0.2, 0.1, 0.927361)
    o = O.OracleWorld(dict(bodies=b, shapes=np.zeros(0, abi.SHAPE_DTYPE), hull=np.zeros((0, 3), np.float32),
                           triangles=np.zeros(0, abi.TRIANGLE_DTYPE)))
    k, init = KINDS[kind]
    j = o.add_joint(k, 0, 1, init)
    o.joint_solve(j, 0.01, 0.2, 0.001)            # caches an impulse
    s = o.bodies()
    s["velocity"][sup] = -0.0
    s["angular_velocity"][sup] = -0.0
    o.set_bodies(s)
    before = o.bodies()[sup].tobytes()
    if warm_start:
        o.joint_solve(j, 0.01, 0.2, 0.001, iterate=False)
    else:
        o.joint_iterate(j, 0.01)
    assert o.bodies()[sup].tobytes() == before
