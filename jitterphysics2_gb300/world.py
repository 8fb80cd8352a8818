"""Host-side mirror of the reference's World API for the contact hot path.

`World` plays the part of Jitter2's `World` (src/Jitter2/World.cs, World.Step.cs): it
owns a device-resident jg_world, takes bodies and shapes (as the reference's
CreateRigidBody / AddShape / SetMassInertia / CreateConstraint calls would leave them)
and steps with `step(dt)`, which raises the reference's exception types on the same
conditions (ArgumentException for a negative dt, World.Step.cs:157-165).  Everything
is routed through the C ABI; there is no CPU code path.
"""
import ctypes

import numpy as np

from . import abi
from .abi import check, ptr


class ArgumentException(ValueError):
    """World.Step's ArgumentException for an invalid time step."""


class World:
    def __init__(self, substeps=1, solver_iterations=6, relax_iterations=4, gravity=(0.0, -9.81, 0.0),
                 max_bodies=1024, max_shapes=None, max_pairs=None, max_arbiters=None, max_constraints=1024,
                 n_worlds=1, **params):
        lib = abi.load()
        max_shapes = max_shapes or max_bodies
        p = abi.default_params(substeps=substeps, solver_iterations=solver_iterations,
                               relax_iterations=relax_iterations, gravity=gravity, max_bodies=max_bodies,
                               max_shapes=max_shapes, max_pairs=max_pairs or max(4096, 24 * max_shapes),
                               max_arbiters=max_arbiters or max(4096, 8 * max_shapes),
                               max_constraints=max_constraints, **params)
        self.params = p
        h = ctypes.c_void_p()
        if n_worlds > 1:
            check(lib.jg_batch_create(ctypes.byref(p), n_worlds, ctypes.byref(h)), "jg_batch_create")
        else:
            check(lib.jg_create(ctypes.byref(p), ctypes.byref(h)), "jg_create")
        self._h = h
        self._lib = lib
        self.n_worlds = n_worlds
        self.n_bodies = 0
        self.n_shapes = 0
        self.n_joints = 0

    # -- lifetime ------------------------------------------------------------------------
    def close(self):
        if self._h:
            self._lib.jg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- scene --------------------------------------------------------------------------
    def set_bodies(self, bodies):
        b = np.ascontiguousarray(bodies, abi.BODY_DTYPE)
        check(self._lib.jg_upload_bodies(self._h, ptr(b), len(b)), "jg_upload_bodies")
        self.n_bodies = len(b)

    def set_shapes(self, shapes, hull=None, triangles=None):
        s = np.ascontiguousarray(shapes, abi.SHAPE_DTYPE)
        h = np.ascontiguousarray(hull if hull is not None else np.zeros((0, 3)), np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(triangles if triangles is not None else np.zeros(0, abi.TRIANGLE_DTYPE),
                                 abi.TRIANGLE_DTYPE)
        check(self._lib.jg_upload_shapes(self._h, ptr(s), len(s), ptr(h), len(h), ptr(t), len(t)), "jg_upload_shapes")
        self.n_shapes = len(s)

    def add_constraint(self, kind, body1, body2, init):
        v = np.ascontiguousarray(init, np.float32)
        out = ctypes.c_int32()
        check(self._lib.jg_add_constraint(self._h, kind, body1, body2, ptr(v), ctypes.byref(out)), "jg_add_constraint")
        self.n_joints += 1
        return out.value

    def set_servo(self, constraint, target, maximum):
        """A servo's target and maximum torque / force (the servos' Target* and Maximum*
        setters): target is xyzw (AngularServo), xyz (LinearServo) or one value."""
        v = np.ascontiguousarray(np.atleast_1d(target), np.float32)
        check(self._lib.jg_set_servo(self._h, constraint, ptr(v), ctypes.c_float(maximum)), "jg_set_servo")

    def set_constraint_params(self, constraint, bias=float("nan"), softness=float("nan"),
                              limit_bias=float("nan"), limit_softness=float("nan")):
        """A constraint's Bias / Softness / LimitBias / LimitSoftness (NaN keeps a value)."""
        check(self._lib.jg_set_constraint_params(self._h, constraint, bias, softness, limit_bias, limit_softness),
              "jg_set_constraint_params")

    def load_scene(self, scene):
        self.set_bodies(scene["bodies"])
        self.set_shapes(scene["shapes"], scene["hull"], scene["triangles"])
        for kind, b1, b2, init in scene.get("joints", []):
            self.add_constraint(kind, b1, b2, np.array(init, np.float32))

    def set_body(self, index, field, value):
        fields = {"position": 0, "orientation": 1, "velocity": 2, "angular_velocity": 3, "force": 4, "torque": 5}
        v = np.ascontiguousarray(value, np.float32)
        check(self._lib.jg_set_body(self._h, index, fields[field], ptr(v)), "jg_set_body")

    def activate_body(self, index):
        """World.ActivateBodyNextStep: wakes the body's island at the next step."""
        check(self._lib.jg_activate_body(self._h, index), "jg_activate_body")

    def set_body_sleep(self, index, deactivation_time=1.0, linear_threshold=0.1 ** 0.5, angular_threshold=0.1 ** 0.5):
        """RigidBody.DeactivationTime (seconds) and DeactivationThreshold (speeds)."""
        check(self._lib.jg_set_body_sleep(self._h, index, ctypes.c_float(deactivation_time),
                                          ctypes.c_float(linear_threshold), ctypes.c_float(angular_threshold)),
              "jg_set_body_sleep")

    # -- stepping -----------------------------------------------------------------------
    def step(self, dt):
        """World.Step(dt) (World.Step.cs:141-296) on the device."""
        if not np.isfinite(dt):
            raise ArgumentException("Time step must be finite.")
        if dt < 0:
            raise ArgumentException("Time step cannot be negative.")
        if self.n_worlds > 1:  # batched worlds: one graph launch per step
            check(self._lib.jg_batch_step(self._h, ctypes.c_float(dt)), "jg_batch_step")
        else:
            check(self._lib.jg_step(self._h, ctypes.c_float(dt)), "jg_step")

    def stabilize(self, dt, solver_iterations, relaxation_iterations=0):
        """World.Stabilize (World.Step.cs:318-392): the present contacts and constraints
        re-solved at the velocity level, without detection or integration."""
        if not np.isfinite(dt):
            raise ArgumentException("Time step must be finite.")
        if dt < 0 or solver_iterations < 1 or relaxation_iterations < 0:
            raise ArgumentException("Invalid time step or iteration count.")
        check(self._lib.jg_stabilize(self._h, ctypes.c_float(dt), solver_iterations, relaxation_iterations),
              "jg_stabilize")

    def step_host(self, dt, bodies):
        """One step with the body state copied in from and back to a host array."""
        check(self._lib.jg_step_host(self._h, ctypes.c_float(dt), ptr(bodies), len(bodies)), "jg_step_host")

    # -- inspection ---------------------------------------------------------------------
    def bodies(self):
        out = np.zeros(self.n_bodies, abi.BODY_DTYPE)
        check(self._lib.jg_download_bodies(self._h, ptr(out), self.n_bodies), "jg_download_bodies")
        return out

    def collide_pairs(self, pairs, noalloc=False):
        """Batched NarrowPhase.MprEpa on shape-index pairs at the current poses.
        Returns (hit[n] bool, pointA[n,3], pointB[n,3], normal[n,3], penetration[n]).
        noalloc=True calls jg_collide_pairs_noalloc (fixed device scratch, at most
        abi.COLLIDE_NOALLOC_MAX_PAIRS pairs per call)."""
        pr = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
        n = len(pr)
        out = np.zeros((max(n, 1), 10), np.float32)
        hit = np.zeros(max(n, 1), np.int32)
        name = "jg_collide_pairs_noalloc" if noalloc else "jg_collide_pairs"
        check(getattr(self._lib, name)(self._h, ptr(pr), n, ptr(out), ptr(hit)), name)
        return hit[:n] != 0, out[:n, 0:3], out[:n, 3:6], out[:n, 6:9], out[:n, 9]

    def manifold_pairs(self, pairs, points):
        """CollisionManifold.BuildManifold for shape-index pairs at the current poses, given
        (pointA, pointB, normal) per pair.  Returns a list of (A [k,3], B [k,3]) arrays."""
        pr = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 9)
        n = len(pr)
        out = np.zeros((max(n, 1), 4, 6), np.float32)
        cnt = np.zeros(max(n, 1), np.int32)
        check(self._lib.jg_manifold_pairs(self._h, ptr(pr), n, ptr(pts), ptr(out), ptr(cnt)), "jg_manifold_pairs")
        return [(out[i, :cnt[i], :3].copy(), out[i, :cnt[i], 3:].copy()) for i in range(n)]

    def pairs(self):
        """The broadphase pair list of the last step, [n, 2] shape indices."""
        n = ctypes.c_int32()
        check(self._lib.jg_get_pairs(self._h, None, 0, ctypes.byref(n)), "jg_get_pairs")
        out = np.zeros((max(n.value, 1), 2), np.int32)
        check(self._lib.jg_get_pairs(self._h, ptr(out), n.value, ctypes.byref(n)), "jg_get_pairs")
        return out[:n.value]

    def contacts(self):
        n = ctypes.c_int32()
        check(self._lib.jg_get_contacts(self._h, None, 0, ctypes.byref(n)), "jg_get_contacts")
        out = np.zeros(max(n.value, 1), abi.CONTACT_DTYPE)
        check(self._lib.jg_get_contacts(self._h, ptr(out), len(out), ctypes.byref(n)), "jg_get_contacts")
        return out[:n.value]

    def constraints(self):
        """(order keys [n], accumulated impulses [n,3]) of the constraints, creation order."""
        n = ctypes.c_int32()
        check(self._lib.jg_get_constraints(self._h, None, None, 0, ctypes.byref(n)), "jg_get_constraints")
        keys = np.zeros(max(n.value, 1), np.int32)
        imp = np.zeros((max(n.value, 1), 3), np.float32)
        check(self._lib.jg_get_constraints(self._h, ptr(keys), ptr(imp), n.value, ctypes.byref(n)), "jg_get_constraints")
        return keys[:n.value], imp[:n.value]

    def counters(self):
        buf = np.zeros(len(abi.COUNTER_NAMES), np.int64)
        check(self._lib.jg_get_counters(self._h, ptr(buf)), "jg_get_counters")
        return dict(zip(abi.COUNTER_NAMES, buf.tolist()))

    def timings(self):
        buf = np.zeros(len(abi.TIMING_NAMES), np.float32)
        check(self._lib.jg_get_timings(self._h, ptr(buf)), "jg_get_timings")
        return dict(zip(abi.TIMING_NAMES, buf.tolist()))

    def residuals(self):
        buf = np.zeros(abi.RESID_MAX, np.float32)
        n = ctypes.c_int32()
        check(self._lib.jg_get_residuals(self._h, ptr(buf), abi.RESID_MAX, ctypes.byref(n)), "jg_get_residuals")
        return buf[:n.value].copy()

    def arbiter_events(self):
        cap = 1 << 20
        created = np.zeros((cap, 2), np.int32)
        removed = np.zeros((cap, 2), np.int32)
        nc, nr = ctypes.c_int32(), ctypes.c_int32()
        check(self._lib.jg_get_arbiter_events(self._h, ptr(created), cap, ctypes.byref(nc), ptr(removed), cap,
                                              ctypes.byref(nr)), "jg_get_arbiter_events")
        return created[:nc.value].copy(), removed[:nr.value].copy()

    def export_state(self):
        size = ctypes.c_int64()
        check(self._lib.jg_export_state(self._h, None, 0, ctypes.byref(size)), "jg_export_state")
        buf = np.zeros(size.value, np.uint8)
        check(self._lib.jg_export_state(self._h, ptr(buf), size.value, ctypes.byref(size)), "jg_export_state")
        return buf

    def import_state(self, buf):
        b = np.ascontiguousarray(buf, np.uint8)
        check(self._lib.jg_import_state(self._h, ptr(b), len(b)), "jg_import_state")

    def autotune(self, dt, steps=3):
        chosen = abi.WorldParams()
        check(self._lib.jg_autotune(self._h, ctypes.c_float(dt), steps, ctypes.byref(chosen)), "jg_autotune")
        return {k: getattr(chosen, k) for k in ("solver_block", "solver_ctas_per_sm", "narrow_tile", "partitioned_solve",
                                                "sched_cells_per_sm")}

    # -- learned warm start (no reference counterpart) ------------------------------------
    def mlp_load(self, params):
        p = np.ascontiguousarray(params, np.float32)
        check(self._lib.jg_mlp_load(self._h, ptr(p), len(p)), "jg_mlp_load")

    def mlp_export(self):
        n = ctypes.c_int32()
        check(self._lib.jg_mlp_export(self._h, None, 0, ctypes.byref(n)), "jg_mlp_export")
        out = np.zeros(n.value, np.float32)
        check(self._lib.jg_mlp_export(self._h, ptr(out), len(out), ctypes.byref(n)), "jg_mlp_export")
        return out

    def mlp_predict(self, features):
        x = np.ascontiguousarray(features, np.float32).reshape(-1, abi.MLP_IN)
        out = np.zeros((len(x), abi.MLP_OUT), np.float32)
        check(self._lib.jg_mlp_predict(self._h, ptr(x), len(x), ptr(out)), "jg_mlp_predict")
        return out

    def mlp_gradients(self, features, targets):
        x = np.ascontiguousarray(features, np.float32).reshape(-1, abi.MLP_IN)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, abi.MLP_OUT)
        g = np.zeros(abi.MLP_NW, np.float32)
        loss = ctypes.c_float()
        check(self._lib.jg_mlp_gradients(self._h, ptr(x), ptr(t), len(x), ptr(g), len(g), ctypes.byref(loss)),
              "jg_mlp_gradients")
        return g, loss.value

    def mlp_train_step(self, features, targets, lr):
        x = np.ascontiguousarray(features, np.float32).reshape(-1, abi.MLP_IN)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, abi.MLP_OUT)
        loss = ctypes.c_float()
        check(self._lib.jg_mlp_train_step(self._h, ptr(x), ptr(t), len(x), ctypes.c_float(lr), ctypes.byref(loss)),
              "jg_mlp_train_step")
        return loss.value

    def collect_training(self, capacity=1 << 20):
        """(features [n,24], converged impulses [n,3]) of the contacts the last step created.
        The first call arms the recording and returns empty arrays."""
        f = np.zeros((capacity, abi.MLP_IN), np.float32)
        t = np.zeros((capacity, abi.MLP_OUT), np.float32)
        n = ctypes.c_int32()
        check(self._lib.jg_collect_training(self._h, ptr(f), ptr(t), capacity, ctypes.byref(n)), "jg_collect_training")
        return f[:n.value].copy(), t[:n.value].copy()

    @property
    def handle(self):
        return self._h


def world_for_scene(scene, **overrides):
    """A World sized for a scene from jitterphysics2_gb300.scenes, with its solver settings."""
    nb, ns = len(scene["bodies"]), len(scene["shapes"])
    # the workloads are stepped without deactivation unless a scene asks for it
    kw = dict(dict(allow_deactivation=0), **scene.get("params", {}))
    kw.update(overrides)
    w = World(max_bodies=nb, max_shapes=ns, max_constraints=max(16, len(scene.get("joints", []))),
              n_worlds=scene.get("n_worlds", 1), **kw)
    w.load_scene(scene)
    return w
