// Host utilities: mass properties of the shape kinds, as each shape's
// CalculateMassInertia computes them (BoxShape.cs:188-199, SphereShape.cs:100-111,
// CapsuleShape.cs:112-129, CylinderShape.cs:122-133, ConeShape.cs:128-138), and the
// tessellation integral used for point clouds (ShapeHelper.Tessellate /
// CalculateMassInertia, ShapeHelper.cs:60-120, :380-412).  Host code; the device never
// needs mass properties other than the uploaded inverse mass and inverse inertia.
#include "../../include/jitter_gpu.h"
#include <cmath>
#include <vector>

namespace {

struct V { float x, y, z; };
V add(V a, V b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V sub(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V mul(V a, float s) { return {a.x * s, a.y * s, a.z * s}; }
float dotv(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V crossv(V a, V b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

// VertexSupportMap support with the reference's "last maximum wins" rule
V hull_support(const float* v, int n, V s, V d) {
    float best = -3.402823466e+38f;
    int bi = 0;
    for (int i = 0; i < n; i++) {
        float dx = v[3 * i] * d.x, dy = v[3 * i + 1] * d.y, dz = v[3 * i + 2] * d.z;
        float dp = dx + (dy + dz);
        if (dp < best) continue;
        best = dp;
        bi = i;
    }
    return add(V{v[3 * bi], v[3 * bi + 1], v[3 * bi + 2]}, s);
}

struct Sink {
    double I[6] = {0, 0, 0, 0, 0, 0};  // m11 m12 m13 m22 m23 m33 of the covariance-like sum
    double com[3] = {0, 0, 0};
    double mass = 0;
    // ShapeHelper.MassInertiaSink.Add: signed tetrahedron (origin, p1, p2, p3)
    void add_tri(V a, V b, V c) {
        double A[3][3] = {{a.x, b.x, c.x}, {a.y, b.y, c.y}, {a.z, b.z, c.z}};
        double det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                     A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
        // canonical tetrahedron covariance: diag 1/60, off-diagonal 1/120
        double C[3][3] = {{1.0 / 60, 1.0 / 120, 1.0 / 120}, {1.0 / 120, 1.0 / 60, 1.0 / 120}, {1.0 / 120, 1.0 / 120, 1.0 / 60}};
        double T[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double s = 0;
                for (int k = 0; k < 3; k++)
                    for (int l = 0; l < 3; l++) s += A[i][k] * C[k][l] * A[j][l];
                T[i][j] = s * det;
            }
        I[0] += T[0][0]; I[1] += T[0][1]; I[2] += T[0][2]; I[3] += T[1][1]; I[4] += T[1][2]; I[5] += T[2][2];
        double m = det / 6.0;
        com[0] += m * 0.25 * (a.x + b.x + c.x);
        com[1] += m * 0.25 * (a.y + b.y + c.y);
        com[2] += m * 0.25 * (a.z + b.z + c.z);
        mass += m;
    }
};

void subdivide(const float* hv, int n, V shift, Sink& sink, V v1, V v2, V v3, V p1, V p2, V p3, int level) {
    if (level <= 1) {
        V cr = crossv(sub(p3, p1), sub(p2, p1));
        if (dotv(cr, cr) > 1e-16f) sink.add_tri(p1, p2, p3);
        return;
    }
    V h1 = mul(add(v1, v2), 0.5f), h2 = mul(add(v2, v3), 0.5f), h3 = mul(add(v3, v1), 0.5f);
    V s1 = hull_support(hv, n, shift, h1), s2 = hull_support(hv, n, shift, h2), s3 = hull_support(hv, n, shift, h3);
    level -= 1;
    subdivide(hv, n, shift, sink, v1, h1, h3, p1, s1, s3, level);
    subdivide(hv, n, shift, sink, h1, v2, h2, s1, p2, s2, level);
    subdivide(hv, n, shift, sink, h3, h2, v3, s3, s2, p3, level);
    subdivide(hv, n, shift, sink, h2, h3, h1, s2, s3, s1, level);
}

}  // namespace

extern "C" int jg_shape_mass_inertia(const jg_shape_desc* s, const float* hull, float* I6, float* com, float* mass) {
    if (!s || !I6 || !com || !mass) return JG_ERR_INVALID_ARG;
    const float PI = 3.14159265358979323846f;
    for (int i = 0; i < 6; i++) I6[i] = 0;
    com[0] = com[1] = com[2] = 0;
    switch (s->kind) {
        case JG_SHAPE_BOX: {
            float sx = s->dims[0] * 2.0f, sy = s->dims[1] * 2.0f, sz = s->dims[2] * 2.0f;
            float m = sx * sy * sz;
            *mass = m;
            I6[0] = (float)(1.0 / 12.0) * m * (sy * sy + sz * sz);
            I6[3] = (float)(1.0 / 12.0) * m * (sx * sx + sz * sz);
            I6[5] = (float)(1.0 / 12.0) * m * (sx * sx + sy * sy);
            return JG_OK;
        }
        case JG_SHAPE_SPHERE: {
            float r = s->dims[0];
            float m = (float)(4.0 / 3.0) * PI * r * r * r;
            *mass = m;
            I6[0] = I6[3] = I6[5] = (float)(2.0 / 5.0) * m * r * r;
            return JG_OK;
        }
        case JG_SHAPE_CAPSULE: {
            float r = s->dims[0], len = 2.0f * s->dims[1];
            float ms = (float)(4.0 / 3.0) * PI * r * r * r;
            float mc = PI * r * r * len;
            float ixx = mc * ((float)(1.0 / 12.0) * len * len + (float)(1.0 / 4.0) * r * r) +
                        ms * ((float)(2.0 / 5.0) * r * r + (float)(1.0 / 4.0) * len * len + (float)(3.0 / 8.0) * len * r);
            I6[0] = ixx;
            I6[3] = (float)(1.0 / 2.0) * mc * r * r + (float)(2.0 / 5.0) * ms * r * r;
            I6[5] = ixx;
            *mass = mc + ms;
            return JG_OK;
        }
        case JG_SHAPE_CYLINDER: {
            float r = s->dims[0], h = s->dims[1];
            float m = PI * r * r * h;
            *mass = m;
            I6[0] = (float)(1.0 / 4.0) * m * r * r + (float)(1.0 / 12.0) * m * h * h;
            I6[3] = (float)(1.0 / 2.0) * m * r * r;
            I6[5] = I6[0];
            return JG_OK;
        }
        case JG_SHAPE_CONE: {
            float r = s->dims[0], h = s->dims[1];
            float m = (float)(1.0 / 3.0) * PI * r * r * h;
            *mass = m;
            I6[0] = m * ((float)(3.0 / 20.0) * r * r + (float)(3.0 / 80.0) * h * h);
            I6[3] = (float)(3.0 / 10.0) * m * r * r;
            I6[5] = I6[0];
            return JG_OK;
        }
        case JG_SHAPE_POINTCLOUD: {
            if (!hull || s->data_count < 1) return JG_ERR_INVALID_ARG;
            const float* hv = hull + 3 * (size_t)s->data_offset;
            int n = s->data_count;
            V shift{s->dims[0], s->dims[1], s->dims[2]};
            const float g = 1.6180339887498948482045f;
            const V ico[12] = {{0, 1, g}, {0, -1, g}, {0, 1, -g}, {0, -1, -g}, {1, g, 0}, {1, -g, 0},
                               {-1, g, 0}, {-1, -g, 0}, {g, 0, 1}, {g, 0, -1}, {-g, 0, 1}, {-g, 0, -1}};
            const int idx[20][3] = {{1, 0, 10}, {0, 1, 8}, {0, 4, 6}, {4, 0, 8}, {0, 6, 10}, {5, 1, 7}, {1, 5, 8},
                                    {7, 1, 10}, {2, 3, 11}, {3, 2, 9}, {4, 2, 6}, {2, 4, 9}, {6, 2, 11}, {3, 5, 7},
                                    {5, 3, 9}, {3, 7, 11}, {4, 8, 9}, {8, 5, 9}, {10, 6, 11}, {7, 10, 11}};
            Sink sink;
            for (int i = 0; i < 20; i++) {
                V v1 = ico[idx[i][0]], v2 = ico[idx[i][1]], v3 = ico[idx[i][2]];
                subdivide(hv, n, shift, sink, v1, v2, v3, hull_support(hv, n, shift, v1), hull_support(hv, n, shift, v2),
                          hull_support(hv, n, shift, v3), 4);
            }
            if (!(sink.mass > 1e-12)) return JG_ERR_INVALID_ARG;
            double tr = sink.I[0] + sink.I[3] + sink.I[5];
            I6[0] = (float)(tr - sink.I[0]); I6[1] = (float)(-sink.I[1]); I6[2] = (float)(-sink.I[2]);
            I6[3] = (float)(tr - sink.I[3]); I6[4] = (float)(-sink.I[4]); I6[5] = (float)(tr - sink.I[5]);
            com[0] = (float)(sink.com[0] / sink.mass);
            com[1] = (float)(sink.com[1] / sink.mass);
            com[2] = (float)(sink.com[2] / sink.mass);
            *mass = (float)sink.mass;
            return JG_OK;
        }
        default:
            return JG_ERR_INVALID_SHAPE;  // TriangleShape has no mass (TriangleShape.cs:95-101)
    }
}
