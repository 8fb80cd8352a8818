// Device support maps, centres and world bounding boxes of the seven shape kinds.
// Within the narrowphase a warp handles one pair: every lane holds the same shape
// record and evaluates analytic support maps redundantly, while point-cloud support maps
// are split across the lanes (one vertex per lane, shuffle arg-max).
#pragma once
#include "jg_world.cuh"

// Compact shape record (kept small: the MPR stage runs one pair per thread).
//   analytic shapes: d = dims (box half extents; r, half length; r, height), b = centre
//   point cloud:     d = shift, b = centre of mass, hull / nhull = vertices
//   triangle:        d, b, c = mesh-local vertices, tri = triangle id
struct ShapeRef {
    int kind;
    v3 d, b, c;
    const float4* hull;
    int nhull;
    int tri;
};

__device__ __forceinline__ ShapeRef load_shape(const WorldDev& w, int s) {
    ShapeRef r;
    int4 info = w.sinfo[s];
    r.kind = info.x;
    r.hull = nullptr;
    r.nhull = 0;
    r.tri = -1;
    r.c = mk3(0.f);
    if (r.kind == JG_SHAPE_TRIANGLE) {
        const TriDev& t = w.tris[info.z];
        r.tri = info.z;
        r.d = mk3(t.a); r.b = mk3(t.b); r.c = mk3(t.c);
    } else {
        float4 d = w.sdims[s];
        float4 c = w.scenter[s];
        r.d = mk3(d.x, d.y, d.z);
        r.b = mk3(c.x, c.y, c.z);
        if (r.kind == JG_SHAPE_POINTCLOUD) {
            r.hull = w.hull + info.z;
            r.nhull = info.w;
        }
    }
    return r;
}

// GetCenter: the uploaded centre (zero for analytic shapes, the centre of mass for point
// clouds) or the triangle centroid (TriangleShape.GetCenter, TriangleShape.cs:158-165).
__device__ __forceinline__ v3 shape_center(const ShapeRef& s) {
    if (s.kind == JG_SHAPE_TRIANGLE) return (1.0f / 3.0f) * (s.d + s.b + s.c);
    return s.b;
}

// Warp-cooperative VertexSupportMap.SupportMapScalar (VertexSupportMap.cs:127-147):
// dot = dx + (dy + dz); ties resolved to the highest index ("last maximum wins").
__device__ __forceinline__ v3 hull_support_warp(const float4* hull, int n, v3 d) {
    const int lane = threadIdx.x & 31;
    float best = -3.402823466e+38f;
    int bi = 0x7fffffff;
    bool have = false;
    for (int i = lane; i < n; i += 32) {
        float4 p = __ldg(hull + i);
        float dx = p.x * d.x, dy = p.y * d.y, dz = p.z * d.z;
        float dp = dx + (dy + dz);
        if (!have || dp >= best) { best = dp; bi = i; have = true; }
    }
    if (!have) { best = -3.402823466e+38f; bi = -1; }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        float ob = __shfl_xor_sync(0xffffffffu, best, off);
        int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi > bi)) { best = ob; bi = oi; }
    }
    if (bi < 0) bi = 0;
    float4 p = __ldg(hull + bi);
    return mk3(p.x, p.y, p.z);
}

// Support maps (BoxShape.cs:86-91, SphereShape.cs:54-58, CapsuleShape.cs:74-88,
// CylinderShape.cs:81-97, ConeShape.cs:74-94, PointCloudShape.SupportMap,
// TriangleShape.cs:167-192).  Must be called by all 32 lanes with identical arguments.
__device__ __forceinline__ v3 support(const ShapeRef& s, v3 d) {
    switch (s.kind) {
        case JG_SHAPE_BOX:
            return mk3(sign_bit(d.x) * s.d.x, sign_bit(d.y) * s.d.y, sign_bit(d.z) * s.d.z);
        case JG_SHAPE_SPHERE:
            return normalize(d) * s.d.x;
        case JG_SHAPE_CAPSULE: {
            v3 r = normalize(d) * s.d.x;
            r.y += sgnf(d.y) * s.d.y;
            return r;
        }
        case JG_SHAPE_CYLINDER: {
            float sigma = sqrtf(d.x * d.x + d.z * d.z);
            float hy = sgnf(d.y) * s.d.y * 0.5f;
            if (sigma > 0.0f) return mk3(d.x / sigma * s.d.x, hy, d.z / sigma * s.d.x);
            return mk3(0.0f, hy, 0.0f);
        }
        case JG_SHAPE_CONE: {
            v3 base = normalize_safe(mk3(d.x, 0.0f, d.z), 1e-12f) * s.d.x;
            base.y = -0.25f * s.d.y;
            if (dot(d, base) >= d.y * 0.75f * s.d.y) return base;
            return mk3(0.0f, 0.75f * s.d.y, 0.0f);
        }
        case JG_SHAPE_POINTCLOUD:
            return hull_support_warp(s.hull, s.nhull, d) + s.d;
        default: {
            float mn = dot(s.d, d);
            float dt = dot(s.b, d);
            v3 r = s.d;
            if (dt > mn) { mn = dt; r = s.b; }
            dt = dot(s.c, d);
            if (dt > mn) r = s.c;
            return r;
        }
    }
}

// Single-thread support map (no warp cooperation), for the per-lane manifold sampling of
// analytic shapes.
__device__ __forceinline__ v3 support_lane(const ShapeRef& s, v3 d) {
    if (s.kind == JG_SHAPE_POINTCLOUD) {
        float best = -3.402823466e+38f;
        int bi = 0;
        for (int i = 0; i < s.nhull; i++) {
            float4 p = __ldg(s.hull + i);
            float dx = p.x * d.x, dy = p.y * d.y, dz = p.z * d.z;
            float dp = dx + (dy + dz);
            if (dp < best) continue;
            best = dp; bi = i;
        }
        float4 p = __ldg(s.hull + bi);
        return mk3(p.x, p.y, p.z) + s.d;
    }
    switch (s.kind) {
        case JG_SHAPE_BOX:
            return mk3(sign_bit(d.x) * s.d.x, sign_bit(d.y) * s.d.y, sign_bit(d.z) * s.d.z);
        case JG_SHAPE_SPHERE:
            return normalize(d) * s.d.x;
        case JG_SHAPE_CAPSULE: {
            v3 r = normalize(d) * s.d.x;
            r.y += sgnf(d.y) * s.d.y;
            return r;
        }
        case JG_SHAPE_CYLINDER: {
            float sigma = sqrtf(d.x * d.x + d.z * d.z);
            float hy = sgnf(d.y) * s.d.y * 0.5f;
            if (sigma > 0.0f) return mk3(d.x / sigma * s.d.x, hy, d.z / sigma * s.d.x);
            return mk3(0.0f, hy, 0.0f);
        }
        case JG_SHAPE_CONE: {
            v3 base = normalize_safe(mk3(d.x, 0.0f, d.z), 1e-12f) * s.d.x;
            base.y = -0.25f * s.d.y;
            if (dot(d, base) >= d.y * 0.75f * s.d.y) return base;
            return mk3(0.0f, 0.75f * s.d.y, 0.0f);
        }
        default: {
            float mn = dot(s.d, d);
            float dt = dot(s.b, d);
            v3 r = s.d;
            if (dt > mn) { mn = dt; r = s.b; }
            dt = dot(s.c, d);
            if (dt > mn) r = s.c;
            return r;
        }
    }
}

// World AABBs (BoxShape.cs:176-182, SphereShape.cs:66-72, CapsuleShape.cs:96-106,
// CylinderShape.cs:103-120, ConeShape.cs:100-124, PointCloudShape.CalculateBoundingBox,
// TriangleShape.cs:122-143).  Single thread per shape.
__device__ __forceinline__ void shape_aabb(const ShapeRef& s, q4 q, v3 p, v3& mn, v3& mx) {
    switch (s.kind) {
        case JG_SHAPE_BOX: {
            m33 a = mat_abs(mat_from_quat(q));
            v3 t = mat_mul(a, s.d);
            mn = p - t; mx = p + t;
            break;
        }
        case JG_SHAPE_SPHERE:
            mn = mk3(-s.d.x) + p; mx = mk3(s.d.x) + p;
            break;
        case JG_SHAPE_CAPSULE: {
            v3 delta = s.d.y * basis_y(q);
            mx = mk3(s.d.x + fabsf(delta.x), s.d.x + fabsf(delta.y), s.d.x + fabsf(delta.z));
            mn = -mx;
            mn = mn + p; mx = mx + p;
            break;
        }
        case JG_SHAPE_CYLINDER: {
            v3 u = basis_y(q);
            float xx = u.x * u.x, yy = u.y * u.y, zz = u.z * u.z;
            v3 ext = mk3(sqrtf(yy + zz) * s.d.x, sqrtf(xx + zz) * s.d.x, sqrtf(xx + yy) * s.d.x);
            v3 p1 = -0.5f * s.d.y * u, p2 = 0.5f * s.d.y * u;
            v3 delta = vmax(p1, p2) + ext;
            mn = p - delta; mx = p + delta;
            break;
        }
        case JG_SHAPE_CONE: {
            v3 u = basis_y(q);
            float xx = u.x * u.x, yy = u.y * u.y, zz = u.z * u.z;
            v3 ext = mk3(sqrtf(yy + zz) * s.d.x, sqrtf(xx + zz) * s.d.x, sqrtf(xx + yy) * s.d.x);
            v3 p1 = -0.25f * s.d.y * u, p2 = 0.75f * s.d.y * u;
            mn = p1 - ext; mx = p1 + ext;
            mx = vmax(mx, p2); mn = vmin(mn, p2);
            mn = mn + p; mx = mx + p;
            break;
        }
        case JG_SHAPE_POINTCLOUD: {
            v3 lmx, lmn;
            lmx.x = support_lane(s, mk3(1.f, 0.f, 0.f)).x;
            lmx.y = support_lane(s, mk3(0.f, 1.f, 0.f)).y;
            lmx.z = support_lane(s, mk3(0.f, 0.f, 1.f)).z;
            lmn.x = support_lane(s, mk3(-1.f, 0.f, 0.f)).x;
            lmn.y = support_lane(s, mk3(0.f, -1.f, 0.f)).y;
            lmn.z = support_lane(s, mk3(0.f, 0.f, -1.f)).z;
            v3 half = 0.5f * (lmx - lmn), cen = 0.5f * (lmx + lmn);
            m33 a = mat_abs(mat_from_quat(q));
            v3 t = mat_mul(a, half), t2 = rotate(cen, q);
            mx = t; mn = -t;
            mn = mn + (p + t2); mx = mx + (p + t2);
            break;
        }
        default: {
            v3 a = rotate(s.d, q), b = rotate(s.b, q), c = rotate(s.c, q);
            mn = mk3(3.402823466e+38f);
            mx = mk3(-3.402823466e+38f);
            mx = vmax(mx, a); mn = vmin(mn, a);
            mx = vmax(mx, b); mn = vmin(mn, b);
            mx = vmax(mx, c); mn = vmin(mn, c);
            v3 extra = mk3(0.01f);
            mn = mn + (p - extra); mx = mx + (p + extra);
            break;
        }
    }
}
