"""ctypes access to the CPU oracle (oracle/_build/liboracle.so), the tests' checker.

The oracle restates the reference's hot path in C++; it is built by oracle/Makefile
(also run by __graft_entry__.build()).  Only tests, smoke() and bench.py's CPU-baseline
leg use it.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_build", "liboracle.so")

import sys  # noqa: E402
sys.path.insert(0, ROOT)
from jitterphysics2_gb300 import abi  # noqa: E402

_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle")], check=True, capture_output=True)
    lib = ctypes.CDLL(LIB)
    P, I, F, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_double
    for suf in ("f", "d"):
        sig = {
            "jor_world_create": (P, []), "jor_world_destroy": (None, [P]), "jor_world_config": (None, [P, P]),
            "jor_world_set_bodies": (None, [P, P, I]), "jor_world_get_bodies": (None, [P, P, I]),
            "jor_world_get_bodies_d": (None, [P, P, I]),
            "jor_world_set_shapes": (None, [P, P, I, P, I, P, I]), "jor_world_add_joint": (I, [P, I, I, I, P]),
            "jor_world_set_joint_colors": (None, [P, P, I]), "jor_world_get_joint_impulses": (None, [P, P, I]),
            "jor_world_set_joint_impulses": (None, [P, P, I]),
            "jor_world_external_order": (None, [P, I]), "jor_world_set_contacts": (None, [P, P, I]),
            "jor_world_get_contacts": (I, [P, P, I]), "jor_world_set_arbiter_color": (None, [P, I, I, I]),
            "jor_world_register_contact": (None, [P, I, I, P, P, P]), "jor_world_narrowphase": (None, [P]),
            "jor_world_set_step_dt": (None, [P, F]), "jor_world_register_linear_contact": (None, [P, I, I, P, P, P]),
            "jor_world_register_manifold": (None, [P, I, I, P, P, I, P]), "jor_world_set_deactivation": (None, [P, I]),
            "jor_world_body_deactivation_time": (None, [P, I, D]), "jor_world_activate_body": (None, [P, I]),
            "jor_world_body_sleep_thresholds": (None, [P, I, D, D]),
            "jor_world_shape_box": (None, [P, I, F, P]), "jor_world_joint_solve": (None, [P, I, F, F, F, I]), "jor_world_joint_iterate": (None, [P, I, F]),
            "jor_world_joint_run": (None, [P, I, F, I, I, I]), "jor_world_joint_impulse": (None, [P, I, P]),
            "jor_world_set_servo": (None, [P, I, P, F]), "jor_world_line_distance": (D, [P, I]), "jor_world_elliptical_swing": (None, [P, I, P]),
            "jor_world_joint_data": (None, [P, I, P]), "jor_world_joint_angle": (D, [P, I]),
            "jor_world_joint_set_limit": (None, [P, I, D, D]), "jor_world_joint_params": (None, [P, I, D, D]),
            "jor_world_joint_limit_params": (None, [P, I, D, D]), "jor_world_joint_matrix": (None, [P, I, P]), "jor_world_set_orientation_d": (None, [P, I, P]),
            "jor_world_prepare": (None, [P, F, I]), "jor_world_iterate": (None, [P, I]),
            "jor_world_set_penalty": (None, [P, I, I, D]), "jor_world_set_arbiter_mode": (None, [P, I, I]),
            "jor_world_set_orientation": (None, [P, I, P]), "jor_world_inertia_world": (None, [P, I, P]),
            "jor_world_step": (None, [P, F, I]), "jor_world_step_mt": (D, [P, F, I]),
            "jor_world_stabilize": (None, [P, F, I, I]),
            "jor_world_counters": (None, [P, P]), "jor_world_pairs": (I, [P, P, I]),
            "jor_world_pairs_sweep": (I, [P, P, I]),
            "jor_world_residuals": (I, [P, P, I]), "jor_world_detect": (I, [P, I, I, P]),
            "jor_world_collide": (I, [P, I, I, P]),
            "jor_support": (None, [P, P, P, P]), "jor_aabb": (None, [P, P, P, P, P]),
            "jor_collide": (I, [P, P, P, P, P, P, P, P, D, I, P]),
            "jor_manifold": (I, [P, P, P, P, P, P, P, P, P, P, P, P]),
            "jor_sweep": (I, [P, P, P, P, P, P, P, P, P, P, P]), "jor_simplex": (I, [P, I, P]),
            "jor_exact_side": (I, [P, P, P, P]), "jor_filter_side": (I, [P, P, P, P, P]),
            "jor_stable_sincos": (None, [D, P, P]), "jor_stable_atan2": (D, [D, D]),
            "jor_shortest_angle": (D, [D, D]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name + "_" + suf)
            fn.restype = res
            fn.argtypes = args
    _lib = lib
    return lib


def p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None and a.size else None


def shape(kind, dims=(0, 0, 0, 0), center=(0, 0, 0), count=0):
    s = np.zeros(1, abi.SHAPE_DTYPE)
    s["kind"] = kind
    d = list(dims) + [0] * (4 - len(dims))
    s["dims"][0] = d[:4]
    s["center"][0] = center
    s["data_count"] = count
    return s


def box(hx, hy, hz):
    return shape(abi.SHAPE_BOX, (hx, hy, hz))


def sphere(r):
    return shape(abi.SHAPE_SPHERE, (r,))


def capsule(r, half_length):
    return shape(abi.SHAPE_CAPSULE, (r, half_length))


def cylinder(r, height):
    return shape(abi.SHAPE_CYLINDER, (r, height))


def cone(r, height):
    return shape(abi.SHAPE_CONE, (r, height))


def hull(points, center=None):
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    c = pts.mean(0) if center is None else center
    s = shape(abi.SHAPE_POINTCLOUD, (0, 0, 0), c, len(pts))
    return s, pts


def _shape_args(s):
    if isinstance(s, tuple):
        return s[0], s[1]
    return s, None


def collide(a, b, qa, qb, pa, pb, threshold=0.02, mode=0, real="f"):
    """mode 0: NarrowPhase.MprEpa; mode 1: NarrowPhase.Collision.  Returns (hit, pA, pB, n, pen, epa_calls)."""
    lib = load()
    sa, va = _shape_args(a)
    sb, vb = _shape_args(b)
    out = np.zeros(12, np.float64)
    args = [np.ascontiguousarray(x, np.float64) for x in (qa, qb, pa, pb)]
    fn = getattr(lib, "jor_collide_" + real)
    hit = fn(p(sa), p(va), p(sb), p(vb), p(args[0]), p(args[1]), p(args[2]), p(args[3]), threshold, mode, p(out))
    return bool(hit), out[0:3], out[3:6], out[6:9], out[9], int(out[10])


def manifold(a, b, qa, qb, pa, pb, pA, pB, n, real="f"):
    lib = load()
    sa, va = _shape_args(a)
    sb, vb = _shape_args(b)
    out = np.zeros(24, np.float64)
    args = [np.ascontiguousarray(x, np.float64) for x in (qa, qb, pa, pb, pA, pB, n)]
    k = getattr(lib, "jor_manifold_" + real)(p(sa), p(va), p(sb), p(vb), *[p(x) for x in args], p(out))
    m = out[:6 * k].reshape(k, 6)
    return m[:, :3], m[:, 3:]


def aabb(s, q, pos, real="f"):
    """World bounding box (min, max) of a shape at an orientation and position."""
    lib = load()
    sa, va = _shape_args(s)
    out = np.zeros(6, np.float64)
    args = [np.ascontiguousarray(x, np.float64) for x in (q, pos)]
    getattr(lib, "jor_aabb_" + real)(p(sa), p(va), p(args[0]), p(args[1]), p(out))
    return out[:3], out[3:]


def sweep(a, b, qa, qb, pa, pb, va, vb, real="f"):
    """NarrowPhase.Sweep: (hit, pA, pB, n, toi), points at the bodies' current poses."""
    lib = load()
    sa, ra = _shape_args(a)
    sb, rb = _shape_args(b)
    out = np.zeros(10, np.float64)
    args = [np.ascontiguousarray(x, np.float64) for x in (qa, qb, pa, pb, va, vb)]
    hit = getattr(lib, "jor_sweep_" + real)(p(sa), p(ra), p(sb), p(rb), *[p(x) for x in args], p(out))
    return bool(hit), out[0:3], out[3:6], out[6:9], out[9]


def simplex(vertices, real="f"):
    """SimplexSolverAB.AddVertex over the vertices in order: (last result, closest point)."""
    v = np.ascontiguousarray(vertices, np.float64).reshape(-1, 3)
    out = np.zeros(3, np.float64)
    r = getattr(load(), "jor_simplex_" + real)(p(v), len(v), p(out))
    return bool(r), out


def support(s, d, real="f"):
    lib = load()
    sa, va = _shape_args(s)
    out = np.zeros(3, np.float64)
    getattr(lib, "jor_support_" + real)(p(sa), p(va), p(np.ascontiguousarray(d, np.float64)), p(out))
    return out


class OracleWorld:
    """A CPU world loaded with the same scene dict the GPU world takes."""

    def __init__(self, scene, real="f", external_order=False, **params):
        self.lib = load()
        self.s = real
        self.h = getattr(self.lib, "jor_world_create_" + real)()
        prm = dict(scene.get("params", {}))
        prm.update(params)
        wp = abi.params_struct(**prm)
        getattr(self.lib, "jor_world_config_" + real)(self.h, ctypes.byref(wp))
        self.n = len(scene["bodies"])
        b = np.ascontiguousarray(scene["bodies"], abi.BODY_DTYPE)
        getattr(self.lib, "jor_world_set_bodies_" + real)(self.h, p(b), len(b))
        sh = np.ascontiguousarray(scene["shapes"], abi.SHAPE_DTYPE)
        hl = np.ascontiguousarray(scene["hull"], np.float32).reshape(-1, 3)
        tr = np.ascontiguousarray(scene["triangles"], abi.TRIANGLE_DTYPE)
        getattr(self.lib, "jor_world_set_shapes_" + real)(self.h, p(sh), len(sh), p(hl), len(hl), p(tr), len(tr))
        for kind, b1, b2, init in scene.get("joints", []):
            v = np.ascontiguousarray(init, np.float32)
            getattr(self.lib, "jor_world_add_joint_" + real)(self.h, kind, b1, b2, p(v))
        getattr(self.lib, "jor_world_external_order_" + real)(self.h, 1 if external_order else 0)
        # World.AllowDeactivation: off unless the scene asks for it, as world_for_scene does
        self.allow_deactivation(bool(prm.get("allow_deactivation", 0)))

    def fn(self, name):
        return getattr(self.lib, name + "_" + self.s)

    def __del__(self):
        try:
            self.fn("jor_world_destroy")(self.h)
        except Exception:
            pass

    def step(self, dt, narrow=True):
        self.fn("jor_world_step")(self.h, dt, 1 if narrow else 0)

    def stabilize(self, dt, iterations, relax=0):
        """World.Stabilize: the present contacts and constraints re-solved, no integration."""
        self.fn("jor_world_stabilize")(self.h, dt, iterations, relax)

    def step_mt(self, dt, threads):
        return self.fn("jor_world_step_mt")(self.h, dt, threads)

    def bodies(self):
        out = np.zeros(self.n, abi.BODY_DTYPE)
        self.fn("jor_world_get_bodies")(self.h, p(out), self.n)
        return out

    def bodies_d(self):
        """Body state at full precision: position, orientation, velocity, angular velocity
        as float64 fields, the other fields as bodies() gives them."""
        raw = np.zeros((self.n, 13), np.float64)
        self.fn("jor_world_get_bodies_d")(self.h, p(raw), self.n)
        base = self.bodies()
        fields = [(name, base.dtype.fields[name][0]) for name in base.dtype.names]
        dt = np.dtype([(name, np.float64, (k,)) if name in ("position", "orientation", "velocity", "angular_velocity")
                       else (name, t) for name, t in fields
                       for k in [{"position": 3, "orientation": 4, "velocity": 3, "angular_velocity": 3}.get(name, 0)]])
        out = np.zeros(self.n, dt)
        for name in base.dtype.names:
            if name not in ("position", "orientation", "velocity", "angular_velocity"):
                out[name] = base[name]
        out["position"] = raw[:, 0:3]
        out["orientation"] = raw[:, 3:7]
        out["velocity"] = raw[:, 7:10]
        out["angular_velocity"] = raw[:, 10:13]
        return out

    def set_bodies(self, b):
        b = np.ascontiguousarray(b, abi.BODY_DTYPE)
        self.fn("jor_world_set_bodies")(self.h, p(b), len(b))

    def contacts(self):
        n = self.fn("jor_world_get_contacts")(self.h, None, 0)
        out = np.zeros(max(n, 1), abi.CONTACT_DTYPE)
        self.fn("jor_world_get_contacts")(self.h, p(out), n)
        return out[:n]

    def set_contacts(self, c):
        c = np.ascontiguousarray(c, abi.CONTACT_DTYPE)
        self.fn("jor_world_set_contacts")(self.h, p(c), len(c))

    def set_arbiter_color(self, s1, s2, color):
        self.fn("jor_world_set_arbiter_color")(self.h, int(s1), int(s2), int(color))

    def set_joint_colors(self, colors):
        c = np.ascontiguousarray(colors, np.int32)
        self.fn("jor_world_set_joint_colors")(self.h, p(c), len(c))

    def joint_solve(self, j, dt, bias, softness, iterate=True):
        """Prepare (and Iterate) one joint alone, bias factor and softness overridden."""
        self.fn("jor_world_joint_solve")(self.h, j, dt, bias, softness, 1 if iterate else 0)

    def joint_run(self, j, dt, substeps=1, iterations=12, prepare=True):
        """One Prepare (unless prepare is False) and `iterations` Iterates of joint j alone under
        TimeStep(dt, substeps), with the joint's own bias and softness (ServoTests.cs:51-56)."""
        self.fn("jor_world_joint_run")(self.h, j, dt, substeps, 1 if prepare else 0, iterations)

    def line_distance(self, j):
        """PointOnLine.Distance: anchor 2's position along the line."""
        return self.fn("jor_world_line_distance")(self.h, j)

    def elliptical_swing(self, j):
        """EllipticalConeLimit.GetSwing: (along the reference, across it), radians."""
        out = np.zeros(2, np.float64)
        self.fn("jor_world_elliptical_swing")(self.h, j, out.ctypes.data)
        return out

    def joint_impulse(self, j):
        out = np.zeros(3, np.float64)
        self.fn("jor_world_joint_impulse")(self.h, j, out.ctypes.data)
        return out

    def set_servo(self, j, target, maximum):
        v = np.ascontiguousarray(np.atleast_1d(target), np.float32)
        self.fn("jor_world_set_servo")(self.h, j, v.ctypes.data, maximum)

    def joint_iterate(self, j, dt):
        """One Iterate of joint j alone."""
        self.fn("jor_world_joint_iterate")(self.h, j, dt)

    def joint_data(self, j):
        """(jr0, jr1, effective mass, clamp, impulse) of a one-row joint after its Prepare."""
        out = np.zeros(12, np.float64)
        self.fn("jor_world_joint_data")(self.h, j, p(out))
        return out[0:3], out[3:6], out[6], int(out[7]), out[8]

    def joint_bias(self, j):
        """The joint's bias vector after its last Prepare (one-row kinds: the first entry)."""
        out = np.zeros(12, np.float64)
        self.fn("jor_world_joint_data")(self.h, j, p(out))
        return out[9:12]

    def deactivation_time(self, body, seconds):
        """RigidBody.DeactivationTime of one body."""
        self.fn("jor_world_body_deactivation_time")(self.h, body, float(seconds))

    def activate(self, body):
        """RigidBody.SetActivationState(true): the body wakes at the next step."""
        self.fn("jor_world_activate_body")(self.h, body)

    def shape_box(self, s, dt):
        """World bounding box (min, max) of shape s for a step of length dt."""
        out = np.zeros(6, np.float64)
        self.fn("jor_world_shape_box")(self.h, s, float(dt), p(out))
        return out[:3], out[3:]

    def allow_deactivation(self, on=True):
        """World.AllowDeactivation: islands at rest for the deactivation time go to sleep."""
        self.fn("jor_world_set_deactivation")(self.h, 1 if on else 0)

    def set_orientation_d(self, body, q):
        """Set one body's orientation at the oracle's own precision (not through float32)."""
        v = np.ascontiguousarray(q, np.float64)
        self.fn("jor_world_set_orientation_d")(self.h, body, p(v))

    def joint_angle(self, j):
        return self.fn("jor_world_joint_angle")(self.h, j)

    def joint_params(self, j, bias, softness):
        self.fn("jor_world_joint_params")(self.h, j, float(bias), float(softness))

    def joint_limit_params(self, j, bias, softness):
        self.fn("jor_world_joint_limit_params")(self.h, j, float(bias), float(softness))

    def joint_matrix(self, j):
        """(Jacobian 3x3 as stored, Q0, local axis) of a three-row joint after its Prepare."""
        out = np.zeros(16, np.float64)
        self.fn("jor_world_joint_matrix")(self.h, j, p(out))
        return out[:9].reshape(3, 3), out[9:13], out[13:16]

    def joint_set_limit(self, j, lo, hi):
        self.fn("jor_world_joint_set_limit")(self.h, j, float(lo), float(hi))

    def add_joint(self, kind, b1, b2, init):
        v = np.ascontiguousarray(init, np.float32)
        return self.fn("jor_world_add_joint")(self.h, kind, b1, b2, p(v))

    def joint_impulses(self, n):
        out = np.zeros((n, 3), np.float32)
        self.fn("jor_world_get_joint_impulses")(self.h, p(out), n)
        return out

    def set_joint_impulses(self, imp):
        v = np.ascontiguousarray(imp, np.float32).reshape(-1, 3)
        self.fn("jor_world_set_joint_impulses")(self.h, p(v), len(v))

    def external_order(self, on):
        self.fn("jor_world_external_order")(self.h, 1 if on else 0)

    def register_contact(self, s1, s2, p1, p2, n, linear_only=False):
        """World.RegisterContact of one point; linear_only removes SolveMode.Angular."""
        a = [np.ascontiguousarray(x, np.float32) for x in (p1, p2, n)]
        name = "jor_world_register_linear_contact" if linear_only else "jor_world_register_contact"
        self.fn(name)(self.h, s1, s2, p(a[0]), p(a[1]), p(a[2]))

    def register_manifold(self, s1, s2, pa, pb, n):
        """World.RegisterContact of a CollisionManifold (up to four points)."""
        a = np.ascontiguousarray(pa, np.float32).reshape(-1, 3)
        b = np.ascontiguousarray(pb, np.float32).reshape(-1, 3)
        v = np.ascontiguousarray(n, np.float32)
        self.fn("jor_world_register_manifold")(self.h, s1, s2, p(a), p(b), len(a), p(v))

    def narrowphase(self, dt=None):
        """Detection alone; dt is the step length the speculative branch tests against."""
        if dt is not None:
            self.fn("jor_world_set_step_dt")(self.h, float(dt))
        self.fn("jor_world_narrowphase")(self.h)

    def counters(self):
        out = np.zeros(8, np.int64)
        self.fn("jor_world_counters")(self.h, p(out))
        return dict(zip(["pairs", "colliding", "points", "arbiters", "contacts", "epa_calls", "epa_failures",
                         "speculative"], out.tolist()))

    def pairs(self, sweep=False):
        name = "jor_world_pairs_sweep" if sweep else "jor_world_pairs"
        n = self.fn(name)(self.h, None, 0)
        out = np.zeros((max(n, 1), 2), np.int32)
        self.fn(name)(self.h, p(out), n)
        return out[:n]

    def residuals(self):
        out = np.zeros(64, np.float32)
        n = self.fn("jor_world_residuals")(self.h, p(out), 64)
        return out[:n].copy()

    def collide(self, s1, s2):
        """NarrowPhase.MprEpa on two of the world's shapes: (hit, pA, pB, n, pen)."""
        out = np.zeros(10, np.float64)
        hit = self.fn("jor_world_collide")(self.h, s1, s2, p(out))
        return bool(hit), out[0:3], out[3:6], out[6:9], out[9]

    def detect(self, s1, s2):
        out = np.zeros(40, np.float64)
        hit = self.fn("jor_world_detect")(self.h, s1, s2, p(out))
        if not hit:
            return None
        k = int(out[3])
        pts = out[4:4 + 6 * k].reshape(k, 6)
        return dict(normal=out[0:3], count=k, A=pts[:, :3], B=pts[:, 3:], pen=out[28], pA=out[29:32], pB=out[32:35])
