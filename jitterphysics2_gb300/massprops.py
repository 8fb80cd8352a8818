"""Shape mass properties for scene construction, in numpy (no native library).

The same formulas the C ABI's jg_shape_mass_inertia evaluates, each shape's
CalculateMassInertia at density 1: BoxShape.cs:188-199, SphereShape.cs:100-111,
CapsuleShape.cs:112-129, CylinderShape.cs:122-133, ConeShape.cs:128-138, and for point
clouds the tessellation integral of ShapeHelper.CalculateMassInertia (ShapeHelper.cs:
86-135 tessellation of the support map at four levels, :356-412 signed-tetrahedron sums).
Analytic shapes are evaluated in float32 in the same operation order; the point-cloud
sums are accumulated in float64 as the library does.  Scenes are built with this module,
so that the GPU world, the oracle and the CPU baseline all start from identical inputs
without loading any compiled library.
"""
import numpy as np

from . import abi

F = np.float32
_PI = F(3.14159265358979323846)
_GOLD = F(1.6180339887498948482045)
_ICO_V = np.array([[0, 1, _GOLD], [0, -1, _GOLD], [0, 1, -_GOLD], [0, -1, -_GOLD], [1, _GOLD, 0], [1, -_GOLD, 0],
                   [-1, _GOLD, 0], [-1, -_GOLD, 0], [_GOLD, 0, 1], [_GOLD, 0, -1], [-_GOLD, 0, 1], [-_GOLD, 0, -1]],
                  np.float32)
_ICO_I = [(1, 0, 10), (0, 1, 8), (0, 4, 6), (4, 0, 8), (0, 6, 10), (5, 1, 7), (1, 5, 8), (7, 1, 10), (2, 3, 11),
          (3, 2, 9), (4, 2, 6), (2, 4, 9), (6, 2, 11), (3, 5, 7), (5, 3, 9), (3, 7, 11), (4, 8, 9), (8, 5, 9),
          (10, 6, 11), (7, 10, 11)]
_LEVELS = 4


def _leaf_directions():
    """Corner directions of the emitted triangles, in emission order: each of the 20
    icosahedron faces split three times at unnormalised edge midpoints."""
    out = []

    def split(v1, v2, v3, level):
        if level <= 1:
            out.append((v1, v2, v3))
            return
        h1 = (v1 + v2) * F(0.5)
        h2 = (v2 + v3) * F(0.5)
        h3 = (v3 + v1) * F(0.5)
        split(v1, h1, h3, level - 1)
        split(h1, v2, h2, level - 1)
        split(h3, h2, v3, level - 1)
        split(h2, h3, h1, level - 1)

    for a, b, c in _ICO_I:
        split(_ICO_V[a], _ICO_V[b], _ICO_V[c], _LEVELS)
    d = np.array(out, np.float32)                          # [T, 3 corners, 3]
    uniq, inv = np.unique(d.reshape(-1, 3), axis=0, return_inverse=True)
    return uniq, inv.reshape(-1, 3)


_DIRS, _CORNER = _leaf_directions()


def _hull_support(points, dirs):
    """VertexSupportMap: the point with the largest dx + (dy + dz), the last one on a tie.
    points [H, n, 3], dirs [D, 3] -> [H, D, 3] (float32)."""
    rev = np.ascontiguousarray(points[:, ::-1].transpose(0, 2, 1))     # [H, 3, n], last point first
    dx = dirs[None, :, 0, None] * rev[:, None, 0, :]
    dy = dirs[None, :, 1, None] * rev[:, None, 1, :]
    dy += dirs[None, :, 2, None] * rev[:, None, 2, :]
    dx += dy                                               # dx + (dy + dz): [H, D, n]
    n = points.shape[1]
    last = n - 1 - np.argmax(dx, axis=2)                   # the first maximum of the reversed order
    return np.take_along_axis(points, last.reshape(points.shape[0], -1, 1).repeat(3, axis=2), axis=1)


def hull_mass_properties(points, shift=(0.0, 0.0, 0.0), chunk=64):
    """(inertia6 about the origin, centre of mass, mass) of point clouds [H, n, 3]."""
    points = np.asarray(points, np.float32)
    if len(points) > chunk:
        parts = [hull_mass_properties(points[i:i + chunk], shift, chunk) for i in range(0, len(points), chunk)]
        return tuple(np.concatenate([q[k] for q in parts]) for k in range(3))
    sp = _hull_support(points, _DIRS) + np.asarray(shift, np.float32)   # [H, D, 3]
    p = sp[:, _CORNER]                                     # [H, T, 3 corners, 3]
    p1, p2, p3 = p[:, :, 0], p[:, :, 1], p[:, :, 2]
    a, b = p3 - p1, p2 - p1
    cr = np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1], a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                   a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], -1)
    keep = (cr[..., 0] * cr[..., 0] + cr[..., 1] * cr[..., 1] + cr[..., 2] * cr[..., 2]) > F(1e-16)
    q1, q2, q3 = p1.astype(np.float64), p2.astype(np.float64), p3.astype(np.float64)
    # determinant of the matrix whose columns are the corners (the signed tetrahedron
    # with the origin, six times its volume)
    det = (q1[..., 0] * (q2[..., 1] * q3[..., 2] - q3[..., 1] * q2[..., 2])
           - q2[..., 0] * (q1[..., 1] * q3[..., 2] - q3[..., 1] * q1[..., 2])
           + q3[..., 0] * (q1[..., 1] * q2[..., 2] - q2[..., 1] * q1[..., 2]))
    det = np.where(keep, det, 0.0)
    # A C A^T with the canonical tetrahedron's second moments C = (I + 1 1^T) / 120:
    # (sum of the corners' outer products + the outer product of their sum) / 120
    s = q1 + q2 + q3
    w = det / 120.0
    Isum = np.empty((points.shape[0], 3, 3))
    for i in range(3):
        for j in range(i, 3):
            Isum[:, i, j] = (w * (q1[..., i] * q1[..., j] + q2[..., i] * q2[..., j] + q3[..., i] * q3[..., j]
                                  + s[..., i] * s[..., j])).sum(axis=1)
    m = det / 6.0
    com = (m[..., None] * 0.25 * s).sum(axis=1)
    mass = m.sum(axis=1)
    tr = Isum[:, 0, 0] + Isum[:, 1, 1] + Isum[:, 2, 2]
    I6 = np.stack([tr - Isum[:, 0, 0], -Isum[:, 0, 1], -Isum[:, 0, 2], tr - Isum[:, 1, 1], -Isum[:, 1, 2],
                   tr - Isum[:, 2, 2]], 1).astype(np.float32)
    return I6, (com / mass[:, None]).astype(np.float32), mass.astype(np.float32)


def analytic_mass_properties(kind, dims):
    """(inertia6, centre, mass) of a box, sphere, capsule, cylinder or cone (float32)."""
    d = [F(x) for x in dims]
    I6 = np.zeros(6, np.float32)
    c12, c25, c14, c38, c13, c43 = F(1.0 / 12.0), F(2.0 / 5.0), F(1.0 / 4.0), F(3.0 / 8.0), F(1.0 / 3.0), F(4.0 / 3.0)
    if kind == abi.SHAPE_BOX:
        sx, sy, sz = d[0] * F(2), d[1] * F(2), d[2] * F(2)
        m = sx * sy * sz
        I6[0] = c12 * m * (sy * sy + sz * sz)
        I6[3] = c12 * m * (sx * sx + sz * sz)
        I6[5] = c12 * m * (sx * sx + sy * sy)
    elif kind == abi.SHAPE_SPHERE:
        r = d[0]
        m = c43 * _PI * r * r * r
        I6[0] = I6[3] = I6[5] = c25 * m * r * r
    elif kind == abi.SHAPE_CAPSULE:
        r, ln = d[0], F(2) * d[1]
        ms = c43 * _PI * r * r * r
        mc = _PI * r * r * ln
        ixx = mc * (c12 * ln * ln + c14 * r * r) + ms * (c25 * r * r + c14 * ln * ln + c38 * ln * r)
        I6[0] = I6[5] = ixx
        I6[3] = F(0.5) * mc * r * r + c25 * ms * r * r
        m = mc + ms
    elif kind == abi.SHAPE_CYLINDER:
        r, h = d[0], d[1]
        m = _PI * r * r * h
        I6[0] = I6[5] = c14 * m * r * r + c12 * m * h * h
        I6[3] = F(0.5) * m * r * r
    elif kind == abi.SHAPE_CONE:
        r, h = d[0], d[1]
        m = c13 * _PI * r * r * h
        I6[0] = I6[5] = m * (F(3.0 / 20.0) * r * r + F(3.0 / 80.0) * h * h)
        I6[3] = F(3.0 / 10.0) * m * r * r
    else:
        raise ValueError("shape kind %d has no analytic mass" % kind)
    return I6, np.zeros(3, np.float32), F(m)
