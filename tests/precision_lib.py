"""FP32 device results against the FP64 oracle (test infrastructure: used by the precision
tests and by bench.py's precision section).

one_step_errors: one step from the device's state replayed by the double-precision oracle
  in the device's solve order; per contact slot present on both sides the errors of the
  contact normal, the penetration depth at the end of the step, the local contact point and
  the accumulated impulses, and per dynamic body the velocity and position errors.
drift: the device and the double-precision oracle stepping the same scene for many steps;
  total linear momentum, kinetic energy and potential energy of both, per step.
"""
import numpy as np

import oracle_lib as O
from jitterphysics2_gb300 import abi


def _quat_rotate(q, v):
    x, y, z, w = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    u = np.stack([x, y, z], -1)
    t = 2 * np.cross(u, v)
    return v + w[..., None] * t + np.cross(u, t)


def _index(rows):
    return {(int(r["shape1"]), int(r["shape2"]), int(r["slot"])): r for r in rows}


def _stats(e, tol):
    e = np.asarray(e, np.float64)
    if len(e) == 0:
        return {"n": 0}
    return {"n": int(len(e)), "median": float(np.median(e)), "max": float(e.max()),
            "within": float(np.mean(e < tol)), "tolerance": tol}


def one_step_errors(scene, b0, c0, c1, b1):
    """b0, c0: device bodies and contacts before the step; c1, b1: after it."""
    o = O.OracleWorld(scene, real="d", external_order=True)
    o.set_bodies(b0)
    o.set_contacts(c0)
    o.narrowphase()
    for c in c1:
        o.set_arbiter_color(c["shape1"], c["shape2"], c["color"])
    o.step(scene["dt"], narrow=False)
    ob = o.bodies_d()
    oc = o.contacts()
    G, D = _index(c1), _index(oc)
    keys = sorted(set(G) & set(D))
    nrm, dep, pt, imp = [], [], [], []
    for k in keys:
        g, d = G[k], D[k]
        nrm.append(np.abs(g["normal"].astype(np.float64) - d["normal"]).max())
        pt.append(np.abs(g["pos1_local"].astype(np.float64) - d["pos1_local"]).max() / max(1.0, np.abs(d["pos1_local"]).max()))
        acc = np.abs(d["accumulated"]).max()
        imp.append(np.abs(g["accumulated"].astype(np.float64) - d["accumulated"]).max() / max(1.0, acc))
        b1g, b2g = int(g["body1"]), int(g["body2"])
        pg = (b1["position"][b1g].astype(np.float64) + g["rel_pos1"]) - (b1["position"][b2g] + g["rel_pos2"])
        pd = (ob["position"][b1g] + d["rel_pos1"]) - (ob["position"][b2g] + d["rel_pos2"])
        dep.append(abs(pg @ g["normal"] - pd @ d["normal"]))
    dyn = b1["motion_type"] == abi.MOTION_DYNAMIC
    dv = np.maximum(np.abs(b1["velocity"][dyn] - ob["velocity"][dyn]).max(1),
                    np.abs(b1["angular_velocity"][dyn] - ob["angular_velocity"][dyn]).max(1))
    dx = np.abs(b1["position"][dyn] - ob["position"][dyn]).max(1)
    return {"contacts_compared": len(keys), "contacts_only_fp32": len(set(G) - set(D)),
            "contacts_only_fp64": len(set(D) - set(G)),
            "normal": _stats(nrm, 1e-4), "depth": _stats(dep, 1e-4), "point": _stats(pt, 1e-4),
            "impulse": _stats(imp, 1e-3), "velocity": _stats(dv, 1e-3), "position": _stats(dx, 1e-4)}


def invariants(bodies, inv_inertia_local, gravity):
    """Total linear momentum [3], kinetic energy and potential energy of the dynamic bodies."""
    dyn = bodies["motion_type"] == abi.MOTION_DYNAMIC
    m = 1.0 / np.asarray(bodies["inv_mass"][dyn], np.float64)
    v = np.asarray(bodies["velocity"][dyn], np.float64)
    w = np.asarray(bodies["angular_velocity"][dyn], np.float64)
    q = np.asarray(bodies["orientation"][dyn], np.float64)
    il = np.asarray(inv_inertia_local[dyn], np.float64)
    Il = np.linalg.inv(np.stack([np.stack([il[:, 0], il[:, 1], il[:, 2]], -1), np.stack([il[:, 1], il[:, 3], il[:, 4]], -1),
                                 np.stack([il[:, 2], il[:, 4], il[:, 5]], -1)], 1))
    wl = _quat_rotate(q * np.array([-1, -1, -1, 1.0]), w)          # angular velocity in the body frame
    e_rot = 0.5 * np.einsum("ni,nij,nj->n", wl, Il, wl).sum()
    e_lin = 0.5 * (m * (v * v).sum(1)).sum()
    y = np.asarray(bodies["position"][dyn], np.float64)
    e_pot = -(m[:, None] * y * np.asarray(gravity, np.float64)).sum()
    return (m[:, None] * v).sum(0), e_lin + e_rot, e_pot


def drift(scene, gpu_world, steps, threads=1):
    """Steps the device world and the FP64 oracle from the same scene; returns per-step
    arrays (momentum [steps, 3], kinetic, potential) for both."""
    o = O.OracleWorld(scene, real="d")
    inv_local = scene["bodies"]["inv_inertia"]
    g = scene["params"].get("gravity", (0.0, -9.81, 0.0))
    out = {k: [] for k in ("p_gpu", "k_gpu", "u_gpu", "p_fp64", "k_fp64", "u_fp64")}
    for _ in range(steps):
        gpu_world.step(scene["dt"])
        if threads > 1:
            o.step_mt(scene["dt"], threads)
        else:
            o.step(scene["dt"])
        for tag, b in (("gpu", gpu_world.bodies()), ("fp64", o.bodies_d())):
            p, k, u = invariants(b, inv_local, g)
            out["p_" + tag].append(p)
            out["k_" + tag].append(k)
            out["u_" + tag].append(u)
    return {k: np.array(v) for k, v in out.items()}
