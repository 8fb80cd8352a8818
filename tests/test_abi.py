"""CPU checks of the C-ABI library: it loads without a GPU, exports every entry point the
header declares, and its host utilities (shape mass properties) agree with the
reference's formulas.  No device compute runs here."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle_lib as O
from jitterphysics2_gb300 import abi, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "jitter_gpu.h")).read()
    return sorted(set(re.findall(r"^(?:int|const char\*)\s+(jg_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(built_lib):
    syms = declared_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(built_lib, s), s
    assert set(syms) == set(abi.SIGNATURES), set(syms) ^ set(abi.SIGNATURES)


def test_library_reports_version_and_no_device(built_lib):
    assert b"sm_103a" in built_lib.jg_version()
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("device present")
    except ImportError:
        pass
    p = abi.default_params()
    h = ctypes.c_void_p()
    rc = built_lib.jg_create(ctypes.byref(p), ctypes.byref(h))
    assert rc == abi.JG_ERR_NOT_SUPPORTED


def test_default_params_match_world_defaults(built_lib):
    # World.cs:333-416 and World.Detect.cs:88-122
    p = abi.default_params()
    assert tuple(p.gravity) == pytest.approx((0, -9.81, 0))
    assert (p.substeps, p.solver_iterations, p.relax_iterations) == (1, 6, 4)
    assert p.enable_auxiliary_contacts == 1 and p.persistent_manifold == 1
    assert p.speculative_relaxation == pytest.approx(0.9)
    assert p.speculative_threshold == pytest.approx(10.0)


def test_python_params_equal_the_library_defaults(built_lib):
    # the oracle and the benchmark's reference arm fill jg_world_params without the library
    a, b = abi.default_params(), abi.params_struct()
    for name, _ in abi.WorldParams._fields_:
        va, vb = getattr(a, name), getattr(b, name)
        if name == "gravity":
            va, vb = tuple(va), tuple(vb)
        assert va == vb, name


def test_scene_mass_properties_agree_with_the_library(built_lib):
    # scenes take their mass properties from numpy (massprops); the C ABI's host utility
    # evaluates the same formulas: analytic shapes bit for bit, point clouds to summation order
    from jitterphysics2_gb300 import massprops
    rng = np.random.default_rng(3)
    for kind in (abi.SHAPE_BOX, abi.SHAPE_SPHERE, abi.SHAPE_CAPSULE, abi.SHAPE_CYLINDER, abi.SHAPE_CONE):
        for _ in range(20):
            rec = np.zeros(1, abi.SHAPE_DTYPE)
            rec["kind"] = kind
            rec["dims"][0, :3] = rng.uniform(0.2, 1.5, 3)
            I6, com, m = abi.mass_inertia(rec[0])
            J6, com2, m2 = massprops.analytic_mass_properties(kind, rec["dims"][0])
            assert np.array_equal(I6, J6) and np.float32(m) == m2
    pts = rng.normal(size=(40, 32, 3))
    pts = (pts / np.linalg.norm(pts, axis=2, keepdims=True) * rng.uniform(0.5, 1.5, (40, 1, 1))).astype(np.float32)
    J6, com2, m2 = massprops.hull_mass_properties(pts)
    for h in range(40):
        rec = np.zeros(1, abi.SHAPE_DTYPE)
        rec["kind"], rec["data_count"] = abi.SHAPE_POINTCLOUD, 32
        I6, com, m = abi.mass_inertia(rec[0], pts[h])
        assert np.allclose(I6, J6[h], rtol=1e-6, atol=1e-7) and np.allclose(com, com2[h], atol=1e-6)
        assert abs(m - m2[h]) <= 1e-6 * m


def test_invalid_arguments_are_rejected_without_a_device(built_lib):
    assert built_lib.jg_create(None, None) == abi.JG_ERR_INVALID_ARG
    assert built_lib.jg_step(None, ctypes.c_float(0.01)) == abi.JG_ERR_INVALID_ARG
    bad = abi.default_params(substeps=0)
    h = ctypes.c_void_p()
    assert built_lib.jg_create(ctypes.byref(bad), ctypes.byref(h)) == abi.JG_ERR_INVALID_ARG


@pytest.mark.parametrize("kind,dims,mass,diag", [
    # BoxShape.CalculateMassInertia (BoxShape.cs:188-199): size (1,2,3)
    (abi.SHAPE_BOX, (0.5, 1.0, 1.5), 6.0, (6 / 12 * (4 + 9), 6 / 12 * (1 + 9), 6 / 12 * (1 + 4))),
    # SphereShape (SphereShape.cs:100-111)
    (abi.SHAPE_SPHERE, (0.7,), 4 / 3 * np.pi * 0.343, None),
    # CylinderShape (CylinderShape.cs:122-133): r 0.5, h 2
    (abi.SHAPE_CYLINDER, (0.5, 2.0), np.pi * 0.25 * 2, None),
    # ConeShape (ConeShape.cs:128-138)
    (abi.SHAPE_CONE, (0.5, 1.0), np.pi * 0.25 / 3, None),
])
def test_analytic_mass_properties(built_lib, kind, dims, mass, diag):
    s = O.shape(kind, dims)
    I6, com, m = abi.mass_inertia(s[0])
    assert m == pytest.approx(mass, rel=1e-6)
    if diag is not None:
        assert (I6[0], I6[3], I6[5]) == pytest.approx(diag, rel=1e-6)
    assert np.allclose(com, 0)


def test_point_cloud_mass_matches_box_limit(built_lib):
    # ShapeHelper.CalculateMassInertia on the 8 corners of a unit cube reproduces the
    # box's analytic mass and inertia (the tessellated hull of a box is the box).
    pts = np.array([[x, y, z] for x in (-0.5, 0.5) for y in (-0.5, 0.5) for z in (-0.5, 0.5)], np.float32)
    s, _ = O.hull(pts)
    I6, com, m = abi.mass_inertia(s[0], pts)
    assert m == pytest.approx(1.0, rel=1e-5)
    assert (I6[0], I6[3], I6[5]) == pytest.approx((1 / 6, 1 / 6, 1 / 6), rel=1e-4)
    assert np.abs(I6[[1, 2, 4]]).max() < 1e-6
    assert np.abs(com).max() < 1e-6


def test_box_grid_scene_layout(built_lib):
    sc = scenes.box_grid()
    b, s = sc["bodies"], sc["shapes"]
    assert len(b) == 1001 and b["motion_type"][0] == abi.MOTION_STATIC
    assert np.allclose(b["inv_mass"][1:], 1.0)
    assert b["position"][1:, 1].min() >= 2 - 0.05 - 1e-6
    assert np.allclose(s["dims"][1:, :3], 0.5)


def test_heightfield_neighbours_are_symmetric():
    t = scenes.heightfield(cells=8, extent=8.0, amplitude=1.0, rng=np.random.default_rng(0))
    assert len(t) == 128
    assert np.all(t["normal"][:, 1] > 0)
    for i, nb in enumerate(t["neighbor"]):
        for j in nb:
            if j >= 0:
                assert i in t["neighbor"][j]


JOINT_RECORD_BYTES = 304  # JointDev: a kind/bodies/colour header and 18 float4 rows


def state_blob(nb, keys, bodies, joints):
    """A state blob in the jg_export_state layout: header, body descriptors, arbiters
    (key, bodies, info, material, 32 contact float4), joint records."""
    narb, nj = len(keys), len(joints)
    hdr = np.array([0x4a475331, 1, nb, narb, nj, 16], np.int32).tobytes()
    b = np.zeros(nb, abi.BODY_DTYPE).tobytes()
    arb = (np.asarray(keys, np.int32).reshape(-1, 2).tobytes() + np.asarray(bodies, np.int32).reshape(-1, 2).tobytes()
           + np.zeros((narb, 4), np.int32).tobytes() + np.zeros((narb, 4), np.float32).tobytes()
           + np.zeros((32, narb, 4), np.float32).tobytes())
    jr = b""
    for kind, b1, b2 in joints:
        rec = np.zeros(JOINT_RECORD_BYTES // 4, np.int32)
        rec[:4] = (kind, b1, b2, 0)
        jr += rec.tobytes()
    return np.frombuffer(hdr + b + arb + jr, np.uint8).copy()


def test_state_blob_checks_without_a_device(built_lib):
    """jg_import_state validates a blob on the host before touching the world: sizes,
    counts and every arbiter's and constraint's indices."""
    nb, ns = 4, 5
    check = lambda blob, n=None: built_lib.jg_check_state(abi.ptr(blob), len(blob) if n is None else n, nb, ns, 16, 16)
    good = state_blob(nb, [(0, 1), (2, 4)], [(0, 1), (2, 3)], [(abi.CONSTRAINT_BALLSOCKET, 1, 2)])
    assert check(good) == abi.JG_OK
    assert check(good, len(good) - 1) == abi.JG_ERR_INVALID_ARG          # truncated
    assert check(good[:20]) == abi.JG_ERR_INVALID_ARG                    # shorter than the header
    neg = good.copy()
    neg[12:16] = np.frombuffer(np.int32(-3).tobytes(), np.uint8)         # negative arbiter count
    assert check(neg) == abi.JG_ERR_INVALID_ARG
    assert check(state_blob(nb, [(0, 1)], [(0, 4)], [])) == abi.JG_ERR_INVALID_ARG    # body out of range
    assert check(state_blob(nb, [(0, 5)], [(0, 1)], [])) == abi.JG_ERR_INVALID_ARG    # shape out of range
    assert check(state_blob(nb, [(0, 1)], [(-1, 1)], [])) == abi.JG_ERR_INVALID_ARG   # negative body
    assert check(state_blob(nb, [], [], [(abi.CONSTRAINT_BALLSOCKET, 0, 9)])) == abi.JG_ERR_INVALID_ARG
    assert check(state_blob(nb, [], [], [(99, 0, 1)])) == abi.JG_ERR_INVALID_ARG       # unknown kind
    for kind in range(abi.CONSTRAINT_BALLSOCKET, abi.CONSTRAINT_ELLIPTICALCONELIMIT + 1):  # every kind
        assert check(state_blob(nb, [], [], [(kind, 0, 1)])) == 0, kind
    assert check(state_blob(nb, [], [], [(abi.CONSTRAINT_ELLIPTICALCONELIMIT + 1, 0, 1)])) == abi.JG_ERR_INVALID_ARG
    assert check(state_blob(3, [], [], [])) == abi.JG_ERR_INVALID_ARG                   # other body count
    many = state_blob(nb, [(0, 1)] * 17, [(0, 1)] * 17, [])
    assert check(many) == abi.JG_ERR_CAPACITY
