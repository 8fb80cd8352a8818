"""Seeded synthetic scenes for the five workloads the contact pipeline is measured on.

No public dataset is involved: every scene is generated from numpy's PCG64 with seed
12345 + workload index, with the shapes, sizes and value distributions the workloads
state.  A scene is a dict of numpy structured arrays (BODY_DTYPE, SHAPE_DTYPE,
TRIANGLE_DTYPE), a flat point-cloud vertex array and a joint list, and feeds both the GPU
world and the CPU oracle.

  box_grid        1000 unit boxes, mass 1, 10x10x10 grid (spacing 1.5, from y = 2,
                  +-0.05 jitter) on a static 200x1x200 ground box
  mixed_pile      n bodies drawn uniformly from box / sphere / capsule / cylinder / cone /
                  32-point hull, uniform positions and orientations, density 1, on a ground
                  box plus a 64x64-cell heightfield of amplitude 2
  batched_worlds  n worlds with log-uniform body counts in [8, 512], half of them carrying
                  chains of 4-16 capsules joined by ball-socket + hinge-angle joints
  towers_rubble   50 towers of 20 unit boxes plus rubble of mixed shapes
"""
import numpy as np

from . import abi, massprops

GROUND_FLAGS = abi.BODY_ACTIVE


def _body(n):
    b = np.zeros(n, abi.BODY_DTYPE)
    b["orientation"][:, 3] = 1.0
    b["friction"] = 0.2
    b["restitution"] = 0.0
    b["linear_damping"] = 0.998
    b["angular_damping"] = 0.995
    b["flags"] = abi.BODY_ACTIVE
    b["motion_type"] = abi.MOTION_DYNAMIC
    return b


def random_quaternions(rng, n):
    """Uniform random unit quaternions (x, y, z, w)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    q = np.stack([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)], axis=1)
    return q.astype(np.float32)


def inverse_sym(I6):
    m = np.array([[I6[0], I6[1], I6[2]], [I6[1], I6[3], I6[4]], [I6[2], I6[4], I6[5]]], np.float64)
    inv = np.linalg.inv(m)
    return np.array([inv[0, 0], inv[0, 1], inv[0, 2], inv[1, 1], inv[1, 2], inv[2, 2]], np.float32)


def set_mass(bodies, shapes, hull, body_index, shape_index, mass=None):
    """RigidBody.SetMassInertia() / SetMassInertia(mass) (RigidBody.cs:1575-1633) for a
    body with one shape."""
    I6, com, m = mass_inertia(shapes[shape_index], hull)
    inv = inverse_sym(I6)
    inv_mass = 1.0 / m
    if mass is not None:
        inv = inv * np.float32(1.0 / (inv_mass * mass))
        inv_mass = 1.0 / mass
    bodies["inv_inertia"][body_index] = inv
    bodies["inv_mass"][body_index] = inv_mass
    return com


def ground(bodies, shapes, bi, si, size=(200.0, 1.0, 200.0), y=-0.5):
    bodies["position"][bi] = (0.0, y, 0.0)
    bodies["motion_type"][bi] = abi.MOTION_STATIC
    bodies["inv_mass"][bi] = 0.0
    bodies["inv_inertia"][bi] = 0.0
    shapes["kind"][si] = abi.SHAPE_BOX
    shapes["body"][si] = bi
    shapes["dims"][si, :3] = (size[0] / 2, size[1] / 2, size[2] / 2)


def box_grid(n_side=10, spacing=1.5, y0=2.0, jitter=0.05, friction=0.6, seed=12345):
    """1000 BoxShape(1,1,1), mass 1, on a static 200x1x200 ground box."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = n_side ** 3
    bodies = _body(n + 1)
    shapes = np.zeros(n + 1, abi.SHAPE_DTYPE)
    ground(bodies, shapes, 0, 0)
    idx = np.arange(n)
    gx, gy, gz = idx % n_side, (idx // n_side) % n_side, idx // (n_side * n_side)
    pos = np.stack([(gx - (n_side - 1) / 2) * spacing, y0 + gy * spacing, (gz - (n_side - 1) / 2) * spacing], 1)
    pos += rng.uniform(-jitter, jitter, size=pos.shape)
    bodies["position"][1:] = pos.astype(np.float32)
    shapes["kind"][1:] = abi.SHAPE_BOX
    shapes["body"][1:] = np.arange(1, n + 1)
    shapes["dims"][1:, :3] = 0.5
    set_mass(bodies, shapes, None, 1, 1, mass=1.0)
    bodies["inv_inertia"][1:] = bodies["inv_inertia"][1]
    bodies["inv_mass"][1:] = bodies["inv_mass"][1]
    bodies["friction"][:] = friction
    return dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32),
                triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=[],
                params=dict(substeps=4, solver_iterations=8, relax_iterations=4), dt=1.0 / 100.0)


def heightfield(cells=64, extent=60.0, amplitude=2.0, rng=None, base=2.0):
    """TriangleMesh of a cells x cells grid (two triangles per cell), normals and
    neighbours as TriangleMesh.BuildFromIndexed / AssignNeighbors compute them
    (Collision/Shapes/TriangleMesh.cs:238-319)."""
    phase = rng.uniform(0, 2 * np.pi, 2) if rng is not None else np.zeros(2)
    k = 2 * np.pi * 3.0 / extent
    xs = np.linspace(-extent / 2, extent / 2, cells + 1)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    H = base + amplitude * np.sin(k * X + phase[0]) * np.cos(k * Z + phase[1])
    V = np.stack([X, H, Z], -1).reshape(-1, 3).astype(np.float32)

    def vid(i, j):
        return i * (cells + 1) + j

    tri = []
    for i in range(cells):
        for j in range(cells):
            p00, p10, p01, p11 = vid(i, j), vid(i + 1, j), vid(i, j + 1), vid(i + 1, j + 1)
            tri.append((p00, p01, p10))
            tri.append((p10, p01, p11))
    T = np.array(tri, np.int64)
    out = np.zeros(len(T), abi.TRIANGLE_DTYPE)
    a, b, c = V[T[:, 0]], V[T[:, 1]], V[T[:, 2]]
    nrm = np.cross(b - a, c - a)
    nrm = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
    out["a"], out["b"], out["c"], out["normal"] = a, b, c, nrm.astype(np.float32)
    edge = {}
    for t, (ia, ib, ic) in enumerate(T):
        for e in ((ia, ib), (ib, ic), (ic, ia)):
            edge.setdefault(e, t)
    for t, (ia, ib, ic) in enumerate(T):
        out["neighbor"][t] = (edge.get((ic, ib), -1), edge.get((ia, ic), -1), edge.get((ib, ia), -1))
    return out


KINDS = [abi.SHAPE_BOX, abi.SHAPE_SPHERE, abi.SHAPE_CAPSULE, abi.SHAPE_CYLINDER, abi.SHAPE_CONE, abi.SHAPE_POINTCLOUD]


def _mixed_shapes(rng, n, hull_list, hull_base):
    """Shape records for n mixed bodies: kinds uniform over the six shape kinds."""
    kinds = rng.integers(0, 6, n)
    recs = np.zeros(n, abi.SHAPE_DTYPE)
    recs["kind"] = np.array(KINDS)[kinds]
    for i in range(n):
        k = recs["kind"][i]
        if k == abi.SHAPE_BOX:
            recs["dims"][i, :3] = rng.uniform(0.5, 1.5, 3) / 2
        elif k == abi.SHAPE_SPHERE:
            recs["dims"][i, 0] = rng.uniform(0.25, 0.75)
        elif k == abi.SHAPE_CAPSULE:
            recs["dims"][i, 0] = rng.uniform(0.25, 0.75)
            recs["dims"][i, 1] = rng.uniform(0.5, 1.5) / 2
        elif k in (abi.SHAPE_CYLINDER, abi.SHAPE_CONE):
            recs["dims"][i, 0] = rng.uniform(0.25, 0.75)
            recs["dims"][i, 1] = rng.uniform(0.5, 1.5)
        else:
            pts = rng.normal(size=(32, 3))
            pts = pts / np.linalg.norm(pts, axis=1, keepdims=True) * rng.uniform(0.5, 1.5)
            recs["data_offset"][i] = hull_base + sum(len(h) for h in hull_list)
            recs["data_count"][i] = 32
            hull_list.append(pts.astype(np.float32))
    return recs


def mass_inertia(rec, hull=None):
    """(inertia6, centre, mass) of one shape record: CalculateMassInertia of its shape at
    density 1 (jitterphysics2_gb300.massprops)."""
    if rec["kind"] == abi.SHAPE_POINTCLOUD:
        o, n = int(rec["data_offset"]), int(rec["data_count"])
        I6, com, m = massprops.hull_mass_properties(np.asarray(hull, np.float32)[None, o:o + n], rec["dims"][:3])
        return I6[0], com[0], m[0]
    return massprops.analytic_mass_properties(int(rec["kind"]), rec["dims"])


def _finish_mass(bodies, shapes, hull, first_body, first_shape, count):
    """RigidBody.SetMassInertia() of bodies with one shape each (density 1); point-cloud
    shapes also get their centre of mass (GetCenter)."""
    cache = {}
    recs = shapes[first_shape:first_shape + count]
    clouds = np.nonzero(recs["kind"] == abi.SHAPE_POINTCLOUD)[0]
    if len(clouds):
        counts = recs["data_count"][clouds]
        assert (counts == counts[0]).all(), "point clouds of one scene share a vertex count"
        idx = recs["data_offset"][clouds][:, None] + np.arange(counts[0])[None, :]
        I6, com, m = massprops.hull_mass_properties(np.asarray(hull, np.float32)[idx])
        for j, i in enumerate(clouds):
            bodies["inv_inertia"][first_body + i] = inverse_sym(I6[j])
            bodies["inv_mass"][first_body + i] = 1.0 / m[j]
            shapes["center"][first_shape + i] = com[j]
    for i in np.nonzero(recs["kind"] != abi.SHAPE_POINTCLOUD)[0]:
        rec = recs[i]
        key = (int(rec["kind"]), tuple(rec["dims"].tolist()))
        if key not in cache:
            I6, com, m = massprops.analytic_mass_properties(int(rec["kind"]), rec["dims"])
            cache[key] = (inverse_sym(I6), 1.0 / m)
        bodies["inv_inertia"][first_body + i], bodies["inv_mass"][first_body + i] = cache[key]


def mixed_pile(n=20000, box=(60.0, 120.0, 60.0), y0=2.0, seed=12346, cells=64, amplitude=2.0, friction=0.6,
               ground_size=None, lattice=None):
    """n mixed bodies in a box x-z footprint from y0, on a ground box + heightfield.
    Positions are uniform in the box (bodies may start overlapping, as the workload
    states), or, with lattice=spacing, on a jittered lattice with no initial overlap."""
    rng = np.random.Generator(np.random.PCG64(seed))
    tris = heightfield(cells, box[0], amplitude, rng)
    nt = len(tris)
    nb = n + 2
    bodies = _body(nb)
    shapes = np.zeros(n + 1 + nt, abi.SHAPE_DTYPE)
    gs = ground_size or (max(200.0, 3 * box[0]), 1.0, max(200.0, 3 * box[2]))
    ground(bodies, shapes, 0, 0, size=gs)
    # heightfield body (static), shapes 1..nt
    bodies["position"][1] = (0, 0, 0)
    bodies["motion_type"][1] = abi.MOTION_STATIC
    bodies["inv_mass"][1] = 0
    shapes["kind"][1:1 + nt] = abi.SHAPE_TRIANGLE
    shapes["body"][1:1 + nt] = 1
    shapes["data_offset"][1:1 + nt] = np.arange(nt)
    hull_list = []
    recs = _mixed_shapes(rng, n, hull_list, 0)
    hull = np.concatenate(hull_list) if hull_list else np.zeros((0, 3), np.float32)
    s0 = 1 + nt
    shapes[s0:] = recs
    shapes["body"][s0:] = np.arange(2, nb)
    if lattice:
        nx = max(1, int(box[0] // lattice))
        nz = max(1, int(box[2] // lattice))
        i = np.arange(n)
        gx, gz, gy = i % nx, (i // nx) % nz, i // (nx * nz)
        pos = np.stack([(gx - (nx - 1) / 2) * lattice, y0 + 4.0 + gy * lattice, (gz - (nz - 1) / 2) * lattice], 1)
        pos += rng.uniform(-0.05, 0.05, pos.shape)
    else:
        pos = np.stack([rng.uniform(-box[0] / 2, box[0] / 2, n), y0 + 4.0 + rng.uniform(0, box[1], n),
                        rng.uniform(-box[2] / 2, box[2] / 2, n)], 1)
    bodies["position"][2:] = pos.astype(np.float32)
    bodies["orientation"][2:] = random_quaternions(rng, n)
    _finish_mass(bodies, shapes, hull, 2, s0, n)
    bodies["friction"][:] = friction
    return dict(bodies=bodies, shapes=shapes, hull=hull, triangles=tris, joints=[],
                params=dict(substeps=4, solver_iterations=8, relax_iterations=4), dt=1.0 / 100.0)


def towers_rubble(n_towers=50, height=20, n_rubble=49000, seed=12349, friction=0.6):
    """50 towers of 20 unit boxes plus rubble of mixed shapes."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nbox = n_towers * height
    n = nbox + n_rubble
    bodies = _body(n + 1)
    shapes = np.zeros(n + 1, abi.SHAPE_DTYPE)
    side = int(np.ceil(np.sqrt(n_towers)))
    area = 160.0
    ground(bodies, shapes, 0, 0, size=(3 * area, 1.0, 3 * area))
    t = np.arange(nbox)
    tw, lv = t // height, t % height
    tx = (tw % side - (side - 1) / 2) * (area / side)
    tz = (tw // side - (side - 1) / 2) * (area / side)
    bodies["position"][1:nbox + 1] = np.stack([tx, 0.5 + lv * 1.0, tz], 1).astype(np.float32)
    shapes["kind"][1:nbox + 1] = abi.SHAPE_BOX
    shapes["dims"][1:nbox + 1, :3] = 0.5
    hull_list = []
    recs = _mixed_shapes(rng, n_rubble, hull_list, 0)
    hull = np.concatenate(hull_list) if hull_list else np.zeros((0, 3), np.float32)
    shapes[nbox + 1:] = recs
    shapes["body"][:] = np.arange(n + 1)
    # rubble between the towers, a few layers high
    rp = np.stack([rng.uniform(-area / 2, area / 2, n_rubble), 1.0 + rng.uniform(0, 12.0, n_rubble),
                   rng.uniform(-area / 2, area / 2, n_rubble)], 1)
    bodies["position"][nbox + 1:] = rp.astype(np.float32)
    bodies["orientation"][nbox + 1:] = random_quaternions(rng, n_rubble)
    _finish_mass(bodies, shapes, hull, 1, 1, n)
    bodies["friction"][:] = friction
    return dict(bodies=bodies, shapes=shapes, hull=hull, triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=[],
                params=dict(substeps=4, solver_iterations=8, relax_iterations=4), dt=1.0 / 100.0)


def batched_worlds(n_worlds=4096, lo=8, hi=512, seed=12348):
    """n independent worlds, body counts log-uniform in [lo, hi] (mixed shapes in a small
    pile); even worlds also carry 1-4 chains of 4-16 capsules (r 0.2, length 1) linked
    by BallSocket + HingeAngle (limit +-60 degrees)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.exp(rng.uniform(np.log(lo), np.log(hi), n_worlds)).astype(int)
    body_list, shape_list, hull_list, joints = [], [], [], []
    nb_total = 0
    hull_n = 0
    for w in range(n_worlds):
        nw = int(counts[w])
        chains = []
        if w % 2 == 0:
            chains = [int(rng.integers(4, 17)) for _ in range(int(rng.integers(1, 5)))]
        n_chain = sum(chains)
        n_free = max(nw - n_chain, 1)
        nbw = 1 + n_free + n_chain
        b = _body(nbw)
        s = np.zeros(nbw, abi.SHAPE_DTYPE)
        ground(b, s, 0, 0, size=(60.0, 1.0, 60.0))
        ext = max(4.0, np.cbrt(n_free) * 1.6)
        hl = []
        recs = _mixed_shapes(rng, n_free, hl, hull_n)
        s[1:1 + n_free] = recs
        b["position"][1:1 + n_free] = np.stack([rng.uniform(-ext / 2, ext / 2, n_free), 1.0 + rng.uniform(0, ext, n_free),
                                                rng.uniform(-ext / 2, ext / 2, n_free)], 1)
        b["orientation"][1:1 + n_free] = random_quaternions(rng, n_free)
        if hl:
            hull_list.extend(hl)
            hull_n += sum(len(h) for h in hl)
        k = 1 + n_free
        cz = -ext / 2 - 2.0
        for ci, L in enumerate(chains):
            x0 = -L / 2.0
            for l in range(L):
                bi = k + l
                s["kind"][bi] = abi.SHAPE_CAPSULE
                s["dims"][bi, 0] = 0.2
                s["dims"][bi, 1] = 0.5
                # capsule axis along x: rotate y onto x (90 degrees about z)
                b["orientation"][bi] = (0.0, 0.0, -np.sin(np.pi / 4), np.cos(np.pi / 4))
                b["position"][bi] = (x0 + l * 1.4 + 0.7, 3.0 + ci * 1.0, cz - ci * 1.2)
                if l > 0:
                    anchor = (x0 + l * 1.4, 3.0 + ci * 1.0, cz - ci * 1.2)
                    joints.append((abi.CONSTRAINT_BALLSOCKET, nb_total + bi - 1, nb_total + bi, anchor))
                    joints.append((abi.CONSTRAINT_HINGEANGLE, nb_total + bi - 1, nb_total + bi,
                                   (0.0, 0.0, 1.0, -np.pi / 3, np.pi / 3)))
            k += L
        s["body"] = np.arange(nbw)
        b["world"] = w
        body_list.append(b)
        shape_list.append(s)
        nb_total += nbw
    bodies = np.concatenate(body_list)
    shapes = np.concatenate(shape_list)
    off = 0
    for s in shape_list:
        off += 0
    # shape body indices are per world; make them global
    base = 0
    gi = 0
    for b, s in zip(body_list, shape_list):
        shapes["body"][gi:gi + len(s)] = s["body"] + base
        gi += len(s)
        base += len(b)
    hull = np.concatenate(hull_list) if hull_list else np.zeros((0, 3), np.float32)
    _finish_mass(bodies, shapes, hull, 0, 0, len(bodies))
    static = bodies["motion_type"] == abi.MOTION_STATIC
    bodies["inv_mass"][static] = 0
    bodies["inv_inertia"][static] = 0
    return dict(bodies=bodies, shapes=shapes, hull=hull, triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=joints,
                n_worlds=n_worlds, params=dict(substeps=4, solver_iterations=8, relax_iterations=4), dt=1.0 / 120.0)


def free_cluster(n=300, spacing=3.2, speed=2.0, seed=12350):
    """n mixed bodies in free space (no gravity, no damping, no static body) thrown toward
    a common centre: contacts are the only forces, so linear and angular momentum are
    conserved and kinetic energy can only fall (restitution 0)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    bodies = _body(n)
    bodies["linear_damping"] = 1.0
    bodies["angular_damping"] = 1.0
    bodies["flags"] = abi.BODY_ACTIVE | abi.BODY_NO_GRAVITY
    hull_list = []
    shapes = _mixed_shapes(rng, n, hull_list, 0)
    shapes["body"] = np.arange(n)
    hull = np.concatenate(hull_list) if hull_list else np.zeros((0, 3), np.float32)
    # jittered lattice inside a sphere; the spacing exceeds every body's extent (no initial overlap)
    side = int(np.ceil(np.cbrt(n * 6.0 / np.pi))) + 1
    g = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3) - (side - 1) / 2.0
    g = g[np.argsort(np.linalg.norm(g, axis=1), kind="stable")][:n] * spacing
    pos = g + rng.uniform(-0.05, 0.05, g.shape)
    bodies["position"] = pos.astype(np.float32)
    bodies["orientation"] = random_quaternions(rng, n)
    d = -pos / np.maximum(np.linalg.norm(pos, axis=1, keepdims=True), 1e-3)
    bodies["velocity"] = (d * speed + rng.normal(0, 0.3 * speed, pos.shape)).astype(np.float32)
    bodies["angular_velocity"] = rng.normal(0, 1.0, pos.shape).astype(np.float32)
    _finish_mass(bodies, shapes, hull, 0, 0, n)
    bodies["friction"] = 0.5
    return dict(bodies=bodies, shapes=shapes, hull=hull, triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=[],
                params=dict(substeps=4, solver_iterations=8, relax_iterations=4, gravity=(0.0, 0.0, 0.0)),
                dt=1.0 / 100.0)


def bullets(n=256, speed=(60.0, 150.0), speculative=True, seed=12351, spacing=1.2):
    """Fast small bodies (spheres, boxes, capsules) fired down at a thin static slab
    (0.1 thick), the case speculative contacts exist for: in one step of 1/60 s each body
    covers 1 to 2.5 m, so without a sweep most pass through the slab between two steps
    (World.Detect.cs:98-122).  Body 0 is the slab."""
    rng = np.random.Generator(np.random.PCG64(seed))
    side = int(np.ceil(np.sqrt(n)))
    bodies = _body(n + 1)
    shapes = np.zeros(n + 1, abi.SHAPE_DTYPE)
    half = side * spacing / 2 + 1.0
    ground(bodies, shapes, 0, 0, size=(2 * half, 0.1, 2 * half), y=0.0)
    k = np.arange(n)
    kinds = np.array([abi.SHAPE_SPHERE, abi.SHAPE_BOX, abi.SHAPE_CAPSULE])[k % 3]
    shapes["kind"][1:] = kinds
    shapes["body"][1:] = k + 1
    shapes["dims"][1:][kinds == abi.SHAPE_SPHERE, 0] = 0.15
    shapes["dims"][1:][kinds == abi.SHAPE_BOX, :3] = 0.12
    shapes["dims"][1:][kinds == abi.SHAPE_CAPSULE, 0] = 0.1
    shapes["dims"][1:][kinds == abi.SHAPE_CAPSULE, 1] = 0.1
    gx, gz = np.meshgrid(np.arange(side), np.arange(side), indexing="ij")
    xz = (np.stack([gx.ravel(), gz.ravel()], 1)[:n] - (side - 1) / 2.0) * spacing
    pos = np.zeros((n, 3))
    pos[:, 0], pos[:, 2] = xz[:, 0], xz[:, 1]
    pos[:, 1] = rng.uniform(1.0, 3.0, n)
    bodies["position"][1:] = pos.astype(np.float32)
    bodies["orientation"][1:] = random_quaternions(rng, n)
    vel = np.zeros((n, 3))
    vel[:, 1] = -rng.uniform(speed[0], speed[1], n)
    vel[:, [0, 2]] = rng.normal(0.0, 0.5, (n, 2))
    bodies["velocity"][1:] = vel.astype(np.float32)
    if speculative:
        bodies["flags"][1:] |= abi.BODY_SPECULATIVE
    _finish_mass(bodies, shapes, np.zeros((0, 3), np.float32), 1, 1, n)
    return dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32),
                triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=[],
                params=dict(substeps=2, solver_iterations=8, relax_iterations=4), dt=1.0 / 60.0)


def mechanism_chains(n_chains=16, seed=12353, spacing=1.0):
    """Chains of four boxes hanging from static anchors, one of each device row kind the
    limb chains do not use: link 1 hangs on a BallSocket and is spun about the chain axis by
    an AngularMotor; link 2 is welded to it (BallSocket + FixedAngle); link 3 is held on
    link 2's horizontal plane by a fixed PointOnPlane, kept at its distance by a fixed
    DistanceLimit and pushed along the chain by a LinearMotor; link 4 is welded to link 3.
    Links are 0.6 long with 0.4 gaps and the chains are 8 apart: no contacts."""
    rng = np.random.Generator(np.random.PCG64(seed))
    per = 5
    n = n_chains * per
    bodies = _body(n)
    shapes = np.zeros(n, abi.SHAPE_DTYPE)
    joints = []
    x_axis, y_axis = (1.0, 0.0, 0.0), (0.0, 1.0, 0.0)
    for c in range(n_chains):
        a = c * per
        base = np.array([0.0, 10.0, 8.0 * c])
        bodies["position"][a] = base
        bodies["motion_type"][a] = abi.MOTION_STATIC
        bodies["inv_mass"][a] = 0.0
        bodies["inv_inertia"][a] = 0.0
        shapes["kind"][a] = abi.SHAPE_BOX
        shapes["body"][a] = a
        shapes["dims"][a, :3] = (0.2, 0.2, 0.2)
        for k in range(1, per):
            i = a + k
            bodies["position"][i] = base + (spacing * k, 0.0, 0.0)
            bodies["angular_velocity"][i] = rng.normal(0.0, 1.0, 3)
            shapes["kind"][i] = abi.SHAPE_BOX
            shapes["body"][i] = i
            shapes["dims"][i, :3] = (0.3, 0.12, 0.12)
        mid = lambda k: tuple(base + (spacing * (k - 0.5), 0.0, 0.0))
        pos = lambda k: tuple(base + (spacing * k, 0.0, 0.0))
        joints.append((abi.CONSTRAINT_BALLSOCKET, a, a + 1, mid(1)))
        joints.append((abi.CONSTRAINT_ANGULARMOTOR, a, a + 1, x_axis + x_axis + (2.0, 5.0)))
        joints.append((abi.CONSTRAINT_BALLSOCKET, a + 1, a + 2, mid(2)))
        joints.append((abi.CONSTRAINT_FIXEDANGLE, a + 1, a + 2, (0.0,)))
        joints.append((abi.CONSTRAINT_POINTONPLANE, a + 2, a + 3, y_axis + pos(2) + pos(3) + (0.0, 0.0)))
        joints.append((abi.CONSTRAINT_DISTANCELIMIT, a + 2, a + 3, pos(2) + pos(3) + (1e-6, -1e-6)))
        joints.append((abi.CONSTRAINT_LINEARMOTOR, a + 2, a + 3, x_axis + x_axis + (0.5, 3.0)))
        joints.append((abi.CONSTRAINT_BALLSOCKET, a + 3, a + 4, mid(4)))
        joints.append((abi.CONSTRAINT_FIXEDANGLE, a + 3, a + 4, (0.0,)))
    _finish_mass(bodies, shapes, np.zeros((0, 3), np.float32), 0, 0, n)
    return dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32),
                triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=joints,
                params=dict(substeps=4, solver_iterations=8, relax_iterations=4), dt=1.0 / 100.0)


def servo_chains(n_chains=16, seed=12354, spacing=1.0):
    """Chains of four boxes hanging from static anchors, one servo of each kind and a slider:
    link 1 hangs
    on a BallSocket and is turned by an AngularServo towards a rotation of 0.3 rad about z
    (maximum torque 5); link 2 is held by a LinearServo at an offset of (1, 0.2, 0) from link
    1 in link 1's frame (maximum force 20); link 3 hangs on a BallSocket from link 2 and is
    twisted about the chain axis by a TwistServo towards 0.6 rad (maximum torque 3); link 4
    slides on a PointOnLine along link 3's x axis (limited to 0.8-1.3) and is pushed along it
    by a LinearAxisServo towards 1.1 (maximum force 10).  Links are 0.6 long with 0.4 gaps
    and the chains are 8 apart: no contacts."""
    rng = np.random.Generator(np.random.PCG64(seed))
    per = 5
    n = n_chains * per
    bodies = _body(n)
    shapes = np.zeros(n, abi.SHAPE_DTYPE)
    joints = []
    x_axis = (1.0, 0.0, 0.0)
    h = 0.15
    q_target = (0.0, 0.0, float(np.sin(h)), float(np.cos(h)))
    for c in range(n_chains):
        a = c * per
        base = np.array([0.0, 10.0, 8.0 * c])
        bodies["position"][a] = base
        bodies["motion_type"][a] = abi.MOTION_STATIC
        bodies["inv_mass"][a] = 0.0
        bodies["inv_inertia"][a] = 0.0
        shapes["kind"][a] = abi.SHAPE_BOX
        shapes["body"][a] = a
        shapes["dims"][a, :3] = (0.2, 0.2, 0.2)
        for k in range(1, per):
            i = a + k
            bodies["position"][i] = base + (spacing * k, 0.0, 0.0)
            bodies["angular_velocity"][i] = rng.normal(0.0, 1.0, 3)
            shapes["kind"][i] = abi.SHAPE_BOX
            shapes["body"][i] = i
            shapes["dims"][i, :3] = (0.3, 0.12, 0.12)
        mid = lambda k: tuple(base + (spacing * (k - 0.5), 0.0, 0.0))
        pos = lambda k: tuple(base + (spacing * k, 0.0, 0.0))
        joints.append((abi.CONSTRAINT_BALLSOCKET, a, a + 1, mid(1)))
        joints.append((abi.CONSTRAINT_ANGULARSERVO, a, a + 1, q_target + (5.0,)))
        joints.append((abi.CONSTRAINT_LINEARSERVO, a + 1, a + 2, pos(1) + pos(2) + (spacing, 0.2, 0.0, 20.0)))
        joints.append((abi.CONSTRAINT_BALLSOCKET, a + 2, a + 3, mid(3)))
        joints.append((abi.CONSTRAINT_TWISTSERVO, a + 2, a + 3, x_axis + x_axis + (0.6, 3.0)))
        joints.append((abi.CONSTRAINT_LINEARAXISSERVO, a + 3, a + 4, x_axis + pos(3) + pos(4) + (1.1 * spacing, 10.0)))
        joints.append((abi.CONSTRAINT_POINTONLINE, a + 3, a + 4, x_axis + pos(3) + pos(4) + (0.8, 1.3)))
    _finish_mass(bodies, shapes, np.zeros((0, 3), np.float32), 0, 0, n)
    return dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32),
                triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=joints,
                params=dict(substeps=4, solver_iterations=8, relax_iterations=4), dt=1.0 / 100.0)


def limb_chains(n_chains=16, links=6, seed=12352, spacing=1.0):
    """Chains of boxes hanging from static anchors, each link joined to the next the way a
    ragdoll limb is: BallSocket at the midpoint, ConeLimit on the chain axis (0 to 0.5 rad)
    and TwistAngle about it (-0.3 to 0.3 rad); a DistanceLimit from the anchor to the last
    link keeps it within its initial distance and beyond half of it.  The chains start
    horizontal with random spin about their axes, so they swing down against the cone
    limits and twist against the twist limits.  Links are 0.6 long with 0.4 gaps: no
    contacts inside a chain, and the chains are 8 apart."""
    rng = np.random.Generator(np.random.PCG64(seed))
    per = links + 1
    n = n_chains * per
    bodies = _body(n)
    shapes = np.zeros(n, abi.SHAPE_DTYPE)
    joints = []
    x_axis = (1.0, 0.0, 0.0)
    for c in range(n_chains):
        a = c * per
        base = np.array([0.0, 10.0, 8.0 * c])
        bodies["position"][a] = base
        bodies["motion_type"][a] = abi.MOTION_STATIC
        bodies["inv_mass"][a] = 0.0
        bodies["inv_inertia"][a] = 0.0
        shapes["kind"][a] = abi.SHAPE_BOX
        shapes["body"][a] = a
        shapes["dims"][a, :3] = (0.2, 0.2, 0.2)
        for k in range(1, per):
            i = a + k
            bodies["position"][i] = base + (spacing * k, 0.0, 0.0)
            bodies["angular_velocity"][i] = (rng.normal(0.0, 3.0), rng.normal(0.0, 0.5), rng.normal(0.0, 0.5))
            shapes["kind"][i] = abi.SHAPE_BOX
            shapes["body"][i] = i
            shapes["dims"][i, :3] = (0.3, 0.12, 0.12)
            mid = base + (spacing * (k - 0.5), 0.0, 0.0)
            joints.append((abi.CONSTRAINT_BALLSOCKET, i - 1, i, tuple(mid)))
            joints.append((abi.CONSTRAINT_CONELIMIT, i - 1, i, x_axis + x_axis + (0.0, 0.5)))
            joints.append((abi.CONSTRAINT_TWISTANGLE, i - 1, i, x_axis + x_axis + (-0.3, 0.3)))
        last = a + links
        d = spacing * links
        joints.append((abi.CONSTRAINT_DISTANCELIMIT, a, last,
                       tuple(base) + tuple(base + (d, 0.0, 0.0)) + (-0.5 * d, 0.0)))
    _finish_mass(bodies, shapes, np.zeros((0, 3), np.float32), 0, 0, n)
    for c in range(n_chains):
        a = c * per
        bodies["inv_mass"][a] = 0.0
        bodies["inv_inertia"][a] = 0.0
    return dict(bodies=bodies, shapes=shapes, hull=np.zeros((0, 3), np.float32),
                triangles=np.zeros(0, abi.TRIANGLE_DTYPE), joints=joints,
                params=dict(substeps=4, solver_iterations=8, relax_iterations=2), dt=1.0 / 60.0)
