// Oracle (test infrastructure only): CPU restatement of Jitter2's narrowphase for the
// contact hot path: shape support maps and bounding boxes, MPR (XenoCollide-derived),
// EPA with the filtered exact orientation predicates, the one-shot contact manifold and
// the triangle-edge filter.  Each function cites the reference lines it follows.
//
// The MPR restatement follows code the reference adapted from XenoCollide, which is
// available under the zlib license:
//   XenoCollide Collision Detection and Physics Library
//   Copyright (c) 2007-2014 Gary Snethen http://xenocollide.com
//   This software is provided 'as-is', without any express or implied warranty.  In no
//   event will the authors be held liable for any damages arising from the use of this
//   software.  Permission is granted to anyone to use this software for any purpose,
//   including commercial applications, and to alter it and redistribute it freely,
//   subject to the following restrictions: 1. The origin of this software must not be
//   misrepresented; you must not claim that you wrote the original software. If you use
//   this software in a product, an acknowledgment in the product documentation would be
//   appreciated but is not required. 2. Altered source versions must be plainly marked as
//   such, and must not be misrepresented as being the original software. 3. This notice
//   may not be removed or altered from any source distribution.
// The exact expansion arithmetic follows Jonathan Richard Shewchuk's public-domain
// predicates (error-free sums), as the reference does.
#pragma once
#include "jor_math.hpp"
#include <vector>

namespace jor {

enum ShapeKind { BOX = 0, SPHERE = 1, CAPSULE = 2, CYLINDER = 3, CONE = 4, POINTCLOUD = 5, TRIANGLE = 6 };

template <class R> struct Shape {
    int kind = BOX;
    R d0 = 0, d1 = 0, d2 = 0;      // dims: box half extents / radius / radius, half length ...
    V3<R> shift;                   // point cloud shift (PointCloudShape.cs Shift)
    V3<R> center;                  // GetCenter()
    const R* verts = nullptr;      // point cloud vertices xyz
    int nverts = 0;
    V3<R> ta, tb, tc;              // triangle vertices (mesh local)
    V3<R> tnormal;                 // triangle normal (mesh local)
    V3<R> nbr_normal[3];           // neighbour normals across edges A, B, C
    bool nbr_valid[3] = {false, false, false};
    bool is_triangle() const { return kind == TRIANGLE; }
};

// ---- support maps ---------------------------------------------------------------------
// BoxShape.SupportMap (Collision/Shapes/BoxShape.cs:86-91)
// SphereShape.SupportMap (SphereShape.cs:54-58)
// CapsuleShape.SupportMap (CapsuleShape.cs:74-88)
// CylinderShape.SupportMap (CylinderShape.cs:81-97)
// ConeShape.SupportMap (ConeShape.cs:74-94)
// PointCloudShape.SupportMap -> VertexSupportMap.SupportMapScalar (VertexSupportMap.cs:127-147)
// TriangleShape.SupportMap (TriangleShape.cs:167-192)
template <class R> V3<R> support(const Shape<R>& s, V3<R> d) {
    switch (s.kind) {
        case BOX:
            return {(R)sign_bit(d.x) * s.d0, (R)sign_bit(d.y) * s.d1, (R)sign_bit(d.z) * s.d2};
        case SPHERE:
            return normalize(d) * s.d0;
        case CAPSULE: {
            V3<R> r = normalize(d) * s.d0;
            r.y += (R)sgn(d.y) * s.d1;
            return r;
        }
        case CYLINDER: {
            R sigma = (R)std::sqrt((double)(d.x * d.x + d.z * d.z));
            R hy = (R)sgn(d.y) * s.d1 * (R)0.5;
            if (sigma > (R)0.0) return {d.x / sigma * s.d0, hy, d.z / sigma * s.d0};
            return {(R)0.0, hy, (R)0.0};
        }
        case CONE: {
            V3<R> base(d.x, (R)0.0, d.z);
            base = normalize_safe(base, (R)1e-12) * s.d0;
            base.y = -(R)0.25 * s.d1;
            if (dot(d, base) >= d.y * (R)0.75 * s.d1) return base;
            return {(R)0, (R)0.75 * s.d1, (R)0};
        }
        case POINTCLOUD: {
            R maxd = -std::numeric_limits<R>::max();
            int idx = 0;
            for (int i = 0; i < s.nverts; i++) {
                R dx = s.verts[3 * i] * d.x, dy = s.verts[3 * i + 1] * d.y, dz = s.verts[3 * i + 2] * d.z;
                R dp = dx + (dy + dz);
                if (dp < maxd) continue;
                maxd = dp;
                idx = i;
            }
            return V3<R>(s.verts[3 * idx], s.verts[3 * idx + 1], s.verts[3 * idx + 2]) + s.shift;
        }
        default: {  // TRIANGLE
            R mn = dot(s.ta, d);
            R dt = dot(s.tb, d);
            V3<R> r = s.ta;
            if (dt > mn) { mn = dt; r = s.tb; }
            dt = dot(s.tc, d);
            if (dt > mn) r = s.tc;
            return r;
        }
    }
}
// GetCenter: zero for the analytic shapes, centre of mass for point clouds
// (PointCloudShape.cs GetCenter), centroid for triangles (TriangleShape.cs:158-165).
template <class R> V3<R> shape_center(const Shape<R>& s) {
    if (s.kind == TRIANGLE) return (R)(1.0 / 3.0) * (s.ta + s.tb + s.tc);
    return s.center;
}

template <class R> struct Box3 { V3<R> mn, mx; };
// CalculateBoundingBox of each shape: BoxShape.cs:176-182, SphereShape.cs:66-72,
// CapsuleShape.cs:96-106, CylinderShape.cs:103-120, ConeShape.cs:100-124,
// PointCloudShape.cs CalculateBoundingBox, TriangleShape.cs:122-143.
template <class R> Box3<R> shape_aabb(const Shape<R>& s, Q4<R> q, V3<R> p, Box3<R>* local_cache = nullptr) {
    Box3<R> b;
    switch (s.kind) {
        case BOX: {
            M3<R> a = mat_abs(mat_from_quat(q));
            V3<R> t = mat_mul(a, V3<R>(s.d0, s.d1, s.d2));
            b.mn = p - t; b.mx = p + t;
            break;
        }
        case SPHERE:
            b.mn = V3<R>(-s.d0) + p; b.mx = V3<R>(s.d0) + p;
            break;
        case CAPSULE: {
            V3<R> delta = s.d1 * basis_y(q);
            b.mx = V3<R>(s.d0 + std::abs(delta.x), s.d0 + std::abs(delta.y), s.d0 + std::abs(delta.z));
            b.mn = -b.mx;
            b.mn = b.mn + p; b.mx = b.mx + p;
            break;
        }
        case CYLINDER: {
            V3<R> u = basis_y(q);
            R xx = u.x * u.x, yy = u.y * u.y, zz = u.z * u.z;
            V3<R> ext(std::sqrt(yy + zz) * s.d0, std::sqrt(xx + zz) * s.d0, std::sqrt(xx + yy) * s.d0);
            V3<R> p1 = -(R)0.5 * s.d1 * u, p2 = (R)0.5 * s.d1 * u;
            V3<R> delta = vmax(p1, p2) + ext;
            b.mn = p - delta; b.mx = p + delta;
            break;
        }
        case CONE: {
            V3<R> u = basis_y(q);
            R xx = u.x * u.x, yy = u.y * u.y, zz = u.z * u.z;
            V3<R> ext(std::sqrt(yy + zz) * s.d0, std::sqrt(xx + zz) * s.d0, std::sqrt(xx + yy) * s.d0);
            V3<R> p1 = -(R)0.25 * s.d1 * u, p2 = (R)0.75 * s.d1 * u;
            b.mn = p1 - ext; b.mx = p1 + ext;
            b.mx = vmax(b.mx, p2); b.mn = vmin(b.mn, p2);
            b.mn = b.mn + p; b.mx = b.mx + p;
            break;
        }
        case POINTCLOUD: {
            Box3<R> lc;
            lc.mx.x = support(s, V3<R>(1, 0, 0)).x;
            lc.mx.y = support(s, V3<R>(0, 1, 0)).y;
            lc.mx.z = support(s, V3<R>(0, 0, 1)).z;
            lc.mn.x = support(s, V3<R>(-1, 0, 0)).x;
            lc.mn.y = support(s, V3<R>(0, -1, 0)).y;
            lc.mn.z = support(s, V3<R>(0, 0, -1)).z;
            if (local_cache) *local_cache = lc;
            V3<R> half = (R)0.5 * (lc.mx - lc.mn), cen = (R)0.5 * (lc.mx + lc.mn);
            M3<R> a = mat_abs(mat_from_quat(q));
            V3<R> t = mat_mul(a, half), t2 = rotate(cen, q);
            b.mx = t; b.mn = -t;
            b.mn = b.mn + (p + t2); b.mx = b.mx + (p + t2);
            break;
        }
        default: {
            V3<R> a = rotate(s.ta, q), bb = rotate(s.tb, q), c = rotate(s.tc, q);
            b.mn = V3<R>(std::numeric_limits<R>::max());
            b.mx = V3<R>(-std::numeric_limits<R>::max());
            b.mx = vmax(b.mx, a); b.mn = vmin(b.mn, a);
            b.mx = vmax(b.mx, bb); b.mn = vmin(b.mn, bb);
            b.mx = vmax(b.mx, c); b.mn = vmin(b.mn, c);
            V3<R> extra((R)0.01);
            b.mn = b.mn + (p - extra); b.mx = b.mx + (p + extra);
            break;
        }
    }
    return b;
}
// JBoundingBox.Disjoint (LinearMath/JBoundingBox.cs:314-318)
template <class R> bool disjoint(const Box3<R>& l, const Box3<R>& r) {
    return l.mx.x < r.mn.x || l.mn.x > r.mx.x || l.mx.y < r.mn.y || l.mn.y > r.mx.y ||
           l.mx.z < r.mn.z || l.mn.z > r.mx.z;
}

// ---- Minkowski difference (MinkowskiDifference.cs:57-90) -------------------------------
template <class R> struct Vertex { V3<R> V, A, B; };
template <class R> inline void mk_support(const Shape<R>& sa, const Shape<R>& sb, Q4<R> qb, V3<R> pb, V3<R> d, Vertex<R>& v) {
    V3<R> tmp = -d;
    v.A = support(sa, d);
    V3<R> tmp2 = rotate_inv(tmp, qb);
    v.B = support(sb, tmp2);
    v.B = rotate(v.B, qb);
    v.B = v.B + pb;
    v.V = v.A - v.B;
}
template <class R> inline void mk_center(const Shape<R>& sa, const Shape<R>& sb, Q4<R> qb, V3<R> pb, Vertex<R>& c) {
    c.A = shape_center(sa);
    c.B = shape_center(sb);
    c.B = rotate(c.B, qb);
    c.B = pb + c.B;
    c.V = c.A - c.B;
}

// ---- exact arithmetic (ExactArithmetic/ExpansionArithmetic.cs:18-117) -------------------
struct Expansion {
    static int difference(double a, double b, double* out) {
        double v = a - b;
        double vb = a - v;
        double res = (a - (v + vb)) + (vb - b);
        int n = 0;
        if (res != 0) out[n++] = res;
        if (v != 0) out[n++] = v;
        return n;
    }
    static int grow(double* e, int len, double value) {
        int count = 0;
        for (int i = 0; i < len; i++) {
            double part = e[i];
            double sum = value + part;
            double vpart = sum - value;
            double res = (value - (sum - vpart)) + (part - vpart);
            if (res != 0) e[count++] = res;
            value = sum;
        }
        if (value != 0) e[count++] = value;
        return count;
    }
    static int add_product(double* r, int len, const double* a, int na, const double* b, int nb, bool neg) {
        for (int i = 0; i < na; i++)
            for (int j = 0; j < nb; j++) {
                double x = a[i], y = b[j];
                double p = x * y;
                double res = std::fma(x, y, -p);
                if (neg) { p = -p; res = -res; }
                if (res != 0) len = grow(r, len, res);
                if (p != 0) len = grow(r, len, p);
            }
        return len;
    }
    static int crossterm(const double* a, int na, const double* b, int nb, const double* c, int nc,
                         const double* d, int nd, double* out) {
        int len = add_product(out, 0, a, na, b, nb, false);
        return add_product(out, len, c, nc, d, nd, true);
    }
    template <class R> static int side(V3<R> a, V3<R> b, V3<R> c, V3<R> p) {
        double ux[2], uy[2], uz[2], vx[2], vy[2], vz[2], dx[2], dy[2], dz[2];
        int nx = difference(a.x, b.x, ux), ny = difference(a.y, b.y, uy), nz = difference(a.z, b.z, uz);
        int mx = difference(a.x, c.x, vx), my = difference(a.y, c.y, vy), mz = difference(a.z, c.z, vz);
        int px = difference(p.x, a.x, dx), py = difference(p.y, a.y, dy), pz = difference(p.z, a.z, dz);
        double cr[16], det[192];
        int len = crossterm(uy, ny, vz, mz, uz, nz, vy, my, cr);
        int count = add_product(det, 0, cr, len, dx, px, false);
        len = crossterm(uz, nz, vx, mx, ux, nx, vz, mz, cr);
        count = add_product(det, count, cr, len, dy, py, false);
        len = crossterm(ux, nx, vy, my, uy, ny, vx, mx, cr);
        count = add_product(det, count, cr, len, dz, pz, false);
        if (count == 0) return 0;
        double top = det[count - 1];
        return top > 0 ? 1 : (top < 0 ? -1 : 0);
    }
    static double estimate(const double* e, int n) { double v = 0; for (int i = 0; i < n; i++) v += e[i]; return v; }
    template <class R> static void normal(V3<R> a, V3<R> b, V3<R> c, double& x, double& y, double& z) {
        double ux[2], uy[2], uz[2], vx[2], vy[2], vz[2], cr[16];
        int nx = difference(a.x, b.x, ux), ny = difference(a.y, b.y, uy), nz = difference(a.z, b.z, uz);
        int mx = difference(a.x, c.x, vx), my = difference(a.y, c.y, vy), mz = difference(a.z, c.z, vz);
        x = estimate(cr, crossterm(uy, ny, vz, mz, uz, nz, vy, my, cr));
        y = estimate(cr, crossterm(uz, nz, vx, mx, ux, nx, vz, mz, cr));
        z = estimate(cr, crossterm(ux, nx, vy, my, uy, ny, vx, mx, cr));
    }
};

// ---- PlaneFilter (ExactArithmetic/PlaneFilter.cs:17-78) ----------------------------------
struct PlaneFilter {
    static constexpr double U = 1.1102230246251565e-16;
    static constexpr double EF = 16 * U;
    double ex = 0, ey = 0, ez = 0, nx = 0, ny = 0, nz = 0;
    bool reliable_normal() const {
        return std::max(std::abs(nx), std::max(std::abs(ny), std::abs(nz))) > 1048576 * std::max(ex, std::max(ey, ez));
    }
    template <class R> void init(V3<R> a, V3<R> b, V3<R> c) {
        double ux = (double)a.x - b.x, uy = (double)a.y - b.y, uz = (double)a.z - b.z;
        double vx = (double)a.x - c.x, vy = (double)a.y - c.y, vz = (double)a.z - c.z;
        double yz = uy * vz, zy = uz * vy, zx = uz * vx, xz = ux * vz, xy = ux * vy, yx = uy * vx;
        nx = yz - zy; ny = zx - xz; nz = xy - yx;
        ex = EF * (std::abs(yz) + std::abs(zy));
        ey = EF * (std::abs(zx) + std::abs(xz));
        ez = EF * (std::abs(xy) + std::abs(yx));
    }
    void negate() { nx = -nx; ny = -ny; nz = -nz; }
    template <class R> bool try_side(V3<R> anchor, V3<R> p, int& sign) const {
        sign = 0;
        double dx = (double)p.x - anchor.x, dy = (double)p.y - anchor.y, dz = (double)p.z - anchor.z;
        double x = nx * dx, y = ny * dy, z = nz * dz;
        double value = (x + y) + z;
        double roundoff = EF * ((std::abs(x) + std::abs(y)) + std::abs(z));
        double coef = (ex * std::abs(dx) + ey * std::abs(dy)) + ez * std::abs(dz);
        double bound = roundoff + 2 * coef;
        if (std::abs(value) <= bound) return false;
        sign = value > 0 ? 1 : -1;
        return true;
    }
    static bool safe_coord(double v) { return v == 0 || (std::abs(v) >= 6.223015277861142e-61 && std::abs(v) <= 1.6069380442589903e60); }
    template <class R> static bool is_safe(V3<R> p) { return safe_coord(p.x) && safe_coord(p.y) && safe_coord(p.z); }
};

// ---- EPA polytope (Collision/NarrowPhase/ConvexPolytope.cs:27-398) ----------------------
template <class R> struct Polytope {
    enum Result { ADDED, NO_HORIZON, DEGENERATE, CAPACITY, NUMERICAL };
    static const int MaxV = 128, MaxT = 256;
    struct Tri { short a, b, c; bool facing; V3<R> normal, closest; R normal_sq, closest_sq; };
    struct Face { PlaneFilter filter; double ba, bb, bc; double dist2; };
    struct D3 { double x, y, z; };
    Vertex<R> verts[MaxV];
    Tri tris[MaxT];
    Face faces[MaxT];
    short nv = 0, nt = 0;
    bool enclosed = false;
    int exact_calls = 0;

    static D3 d3(V3<R> v) { return {(double)v.x, (double)v.y, (double)v.z}; }
    static double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
    static D3 dcross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
    static D3 dsub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
    static D3 dadd(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
    static D3 dmul(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
    static bool dfinite(D3 a) { return std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(a.z); }

    // InitTetrahedron (ConvexPolytope.cs:113-132)
    bool init_tetrahedron() {
        nv = 4; nt = 0; enclosed = false;
        for (int i = 0; i < 4; i++) if (!PlaneFilter::is_safe(verts[i].V)) return false;
        static const short idx[12] = {0, 2, 1, 0, 1, 3, 0, 3, 2, 1, 2, 3};
        for (int i = 0; i < 4; i++)
            if (create_triangle(idx[3 * i], idx[3 * i + 1], idx[3 * i + 2], tris[i], faces[i]) != ADDED) return false;
        nt = 4;
        return true;
    }
    // InitTetrahedron(point) (ConvexPolytope.cs:136-144)
    bool init_tetrahedron(V3<R> p) {
        const R sc = (R)1e-2;
        verts[0] = Vertex<R>{p + sc * V3<R>(std::sqrt((R)(8.0 / 9.0)), 0, -(R)(1.0 / 3.0)), {}, {}};
        verts[1] = Vertex<R>{p + sc * V3<R>(-std::sqrt((R)(2.0 / 9.0)), std::sqrt((R)(2.0 / 3.0)), -(R)(1.0 / 3.0)), {}, {}};
        verts[2] = Vertex<R>{p + sc * V3<R>(-std::sqrt((R)(2.0 / 9.0)), -std::sqrt((R)(2.0 / 3.0)), -(R)(1.0 / 3.0)), {}, {}};
        verts[3] = Vertex<R>{p + sc * V3<R>(0, 0, 1), {}, {}};
        return init_tetrahedron();
    }
    // GetClosestTriangle (ConvexPolytope.cs:147-166)
    int closest_triangle() {
        int best = 0;
        double mn = std::numeric_limits<double>::infinity();
        bool skip = enclosed;
        enclosed = true;
        for (int i = 0; i < nt; i++) {
            if (faces[i].dist2 < mn) { mn = faces[i].dist2; best = i; }
            if (!tris[i].facing) enclosed = skip;
        }
        return best;
    }
    // CalculatePoints (ConvexPolytope.cs:169-185)
    bool calculate_points(const Tri& t, V3<R>& pa, V3<R>& pb) {
        for (int i = 0; i < nt; i++) {
            if (tris[i].a != t.a || tris[i].b != t.b || tris[i].c != t.c) continue;
            const Face& f = faces[i];
            D3 a = dadd(dadd(dmul(d3(verts[t.a].A), f.ba), dmul(d3(verts[t.b].A), f.bb)), dmul(d3(verts[t.c].A), f.bc));
            D3 b = dadd(dadd(dmul(d3(verts[t.a].B), f.ba), dmul(d3(verts[t.b].B), f.bb)), dmul(d3(verts[t.c].B), f.bc));
            pa = V3<R>((R)a.x, (R)a.y, (R)a.z);
            pb = V3<R>((R)b.x, (R)b.y, (R)b.z);
            return true;
        }
        return false;
    }
    // Side (ConvexPolytope.cs:321-327)
    int side(const Face& f, short a, short b, short c, short pi) {
        V3<R> p = pi < 0 ? V3<R>() : verts[pi].V;
        if (p == verts[a].V || p == verts[b].V || p == verts[c].V) return 0;
        int s;
        if (f.filter.try_side(verts[a].V, p, s)) return s;
        exact_calls++;
        return Expansion::side(verts[a].V, verts[b].V, verts[c].V, p);
    }
    // CalcBarycentric (ConvexPolytope.cs:328-395)
    static bool calc_bary(D3 a, D3 b, D3 c, D3 n, double nscale, double nsq, D3& out) {
        D3 u = dsub(a, b), v = dsub(a, c);
        double gamma = (ddot(dcross(u, a), n) / nsq) / nscale;
        double beta = (ddot(dcross(a, v), n) / nsq) / nscale;
        double alpha = 1 - gamma - beta;
        bool clamped = false;
        if (alpha >= 0 && beta < 0) {
            double t = ddot(a, u);
            if (gamma < 0 && t > 0) { beta = std::min(1.0, t / ddot(u, u)); alpha = 1 - beta; gamma = 0; }
            else { gamma = std::clamp(ddot(a, v) / ddot(v, v), 0.0, 1.0); alpha = 1 - gamma; beta = 0; }
            clamped = true;
        } else if (beta >= 0 && gamma < 0) {
            D3 w = dsub(b, c);
            double t = ddot(b, w);
            if (alpha < 0 && t > 0) { gamma = std::min(1.0, t / ddot(w, w)); beta = 1 - gamma; alpha = 0; }
            else { alpha = std::clamp(-ddot(b, u) / ddot(u, u), 0.0, 1.0); beta = 1 - alpha; gamma = 0; }
            clamped = true;
        } else if (gamma >= 0 && alpha < 0) {
            D3 w = dsub(b, c);
            double t = -ddot(c, v);
            if (beta < 0 && t > 0) { alpha = std::min(1.0, t / ddot(v, v)); gamma = 1 - alpha; beta = 0; }
            else { beta = std::clamp(-ddot(c, w) / ddot(w, w), 0.0, 1.0); gamma = 1 - beta; alpha = 0; }
            clamped = true;
        }
        out = {alpha, beta, gamma};
        return clamped;
    }
    // CreateTriangle (ConvexPolytope.cs:267-318)
    Result create_triangle(short a, short b, short c, Tri& t, Face& f) {
        t = Tri{};
        f = Face{};
        f.filter.init(verts[a].V, verts[b].V, verts[c].V);
        int orient = 0;
        for (short i = 0; i < 4 && orient == 0; i++) {
            if (i == a || i == b || i == c) continue;
            orient = -side(f, a, b, c, i);
        }
        if (orient == 0) return DEGENERATE;
        if (orient < 0) { std::swap(a, b); f.filter.negate(); }
        bool facing = side(f, a, b, c, -1) <= 0;
        D3 raw{f.filter.nx, f.filter.ny, f.filter.nz};
        if (!f.filter.reliable_normal()) {
            exact_calls++;
            Expansion::normal(verts[a].V, verts[b].V, verts[c].V, raw.x, raw.y, raw.z);
        }
        double ns = std::max(std::abs(raw.x), std::max(std::abs(raw.y), std::abs(raw.z)));
        if (!(ns > 0) || !std::isfinite(ns)) return NUMERICAL;
        D3 sn{raw.x / ns, raw.y / ns, raw.z / ns};
        double nsq = ddot(sn, sn);
        D3 va = d3(verts[a].V), vb = d3(verts[b].V), vc = d3(verts[c].V);
        D3 bc;
        bool clamped = calc_bary(va, vb, vc, sn, ns, nsq, bc);
        f.ba = bc.x; f.bb = bc.y; f.bc = bc.z;
        D3 cl = clamped ? dadd(dadd(dmul(va, bc.x), dmul(vb, bc.y)), dmul(vc, bc.z)) : dmul(sn, ddot(sn, va) / nsq);
        f.dist2 = ddot(cl, cl);
        if (!dfinite(cl) || !dfinite(bc) || !std::isfinite(f.dist2)) return NUMERICAL;
        t.a = a; t.b = b; t.c = c; t.facing = facing;
        t.normal = V3<R>((R)sn.x, (R)sn.y, (R)sn.z);
        t.normal_sq = len2(t.normal);
        t.closest = V3<R>((R)cl.x, (R)cl.y, (R)cl.z);
        t.closest_sq = (R)f.dist2;
        bool ok = std::isfinite(t.closest.x) && std::isfinite(t.closest.y) && std::isfinite(t.closest.z) && std::isfinite(t.closest_sq);
        return ok ? ADDED : NUMERICAL;
    }
    // AddVertexDetailed (ConvexPolytope.cs:199-265)
    Result add_vertex(const Vertex<R>& v) {
        if (nt == 0 || !PlaneFilter::is_safe(v.V)) return NUMERICAL;
        if (nv == MaxV) return CAPACITY;
        verts[nv] = v;
        bool lit[MaxT];
        short ea[3 * MaxT], eb[3 * MaxT];
        int ne = 0, nlit = 0;
        for (int index = nt; index-- > 0;) {
            const Tri& tr = tris[index];
            lit[index] = side(faces[index], tr.a, tr.b, tr.c, nv) > 0;
            if (!lit[index]) continue;
            nlit++;
            short cs[3] = {tr.a, tr.b, tr.c};
            for (int k = 0; k < 3; k++) {
                short A = cs[k], B = cs[(k + 1) % 3];
                bool added = true;
                for (int e = ne; e-- > 0;) {
                    bool match = (ea[e] == A && eb[e] == B) || (ea[e] == B && eb[e] == A);
                    if (!match) continue;
                    --ne;
                    ea[e] = ea[ne]; eb[e] = eb[ne];
                    added = false;
                    break;
                }
                if (added) { ea[ne] = A; eb[ne] = B; ne++; }
            }
        }
        if (ne == 0) return NO_HORIZON;
        if (nt - nlit + ne > MaxT) return CAPACITY;
        int surv = 0;
        for (int i = 0; i < nt; i++) {
            if (lit[i]) continue;
            if (surv != i) { tris[surv] = tris[i]; faces[surv] = faces[i]; }
            surv++;
        }
        for (int i = 0; i < ne; i++) {
            int index = surv + i;
            Result r = create_triangle(ea[i], eb[i], nv, tris[index], faces[index]);
            if (r != ADDED) { nt = 0; enclosed = false; return r; }
        }
        nt = (short)(surv + ne);
        nv++;
        return ADDED;
    }
};

// ---- MPR / EPA (Collision/NarrowPhase/NarrowPhase.cs) ------------------------------------
template <class R> struct MprEpa {
    static constexpr R NumericEpsilon = (R)1e-16;
    Polytope<R> poly;
    int epa_calls = 0, epa_failures = 0;

    // MprEpaSolver.SolveMprEpa (NarrowPhase.cs:39-95)
    bool solve_mpr_epa(const Shape<R>& sa, const Shape<R>& sb, Q4<R> qb, V3<R> pb,
                       V3<R>& p1, V3<R>& p2, V3<R>& n, R& pen) {
        const R eps = (R)1e-5;
        const int maxIter = 85;
        if (!poly.init_tetrahedron()) return false;
        int iter = 0;
        typename Polytope<R>::Tri ctri{};
        while (++iter < maxIter) {
            ctri = poly.tris[poly.closest_triangle()];
            V3<R> sd = ctri.closest;
            R sdsq = ctri.closest_sq;
            if (!poly.enclosed) sd = -sd;
            if (ctri.closest_sq < NumericEpsilon) { sd = ctri.normal; sdsq = ctri.normal_sq; }
            Vertex<R> v;
            mk_support(sa, sb, qb, pb, sd, v);
            R delta = dot(ctri.closest - v.V, sd);
            if (delta * delta <= eps * eps * sdsq) goto converged;
            {
                auto r = poly.add_vertex(v);
                if (r == Polytope<R>::NO_HORIZON) goto converged;
                if (r != Polytope<R>::ADDED) return false;
            }
        }
        return false;
    converged:
        if (!poly.enclosed) return false;
        poly.calculate_points(ctri, p1, p2);
        n = ctri.normal * ((R)1.0 / std::sqrt(ctri.normal_sq));
        pen = std::sqrt(ctri.closest_sq);
        return true;
    }

    // MprEpaSolver.SolveMpr (NarrowPhase.cs:98-347)
    bool solve_mpr(const Shape<R>& sa, const Shape<R>& sb, Q4<R> qb, V3<R> pb, R epa_threshold,
                   V3<R>& pA, V3<R>& pB, V3<R>& normal, R& pen) {
        const R eps = (R)1e-5;
        const int maxIter = 34;
        Vertex<R> v0, v1, v2, v3, v4;
        V3<R> t1, t2, t3;
        pen = (R)0.0;
        mk_center(sa, sb, qb, pb, v0);
        if (std::abs(v0.V.x) < NumericEpsilon && std::abs(v0.V.y) < NumericEpsilon && std::abs(v0.V.z) < NumericEpsilon)
            v0.V.x = (R)1e-05;
        normal = -v0.V;
        mk_support(sa, sb, qb, pb, normal, v1);
        pA = v1.A; pB = v1.B;
        if (dot(v1.V, normal) <= (R)0.0) return false;
        normal = cross(v1.V, v0.V);
        if (len2(normal) < (R)1e-12) {
            normal = v1.V - v0.V;
            normal = normalize(normal);
            t1 = v1.A - v1.B;
            pen = dot(t1, normal);
            return true;
        }
        mk_support(sa, sb, qb, pb, normal, v2);
        if (dot(v2.V, normal) <= (R)0.0) return false;
        t1 = v1.V - v0.V;
        t2 = v2.V - v0.V;
        normal = cross(t1, t2);
        R dist = dot(normal, v0.V);
        if (dist > (R)0.0) {
            std::swap(v1.V, v2.V); std::swap(v1.A, v2.A); std::swap(v1.B, v2.B);
            normal = -normal;
        }
        int phase2 = 0, phase1 = 0;
        bool hit = false;
        while (true) {
            if (phase1 > maxIter) return false;
            phase1++;
            mk_support(sa, sb, qb, pb, normal, v3);
            if (dot(v3.V, normal) <= (R)0.0) return false;
            t1 = cross(v1.V, v3.V);
            if (dot(t1, v0.V) < (R)0.0) {
                v2 = v3;
                t1 = v1.V - v0.V; t2 = v3.V - v0.V;
                normal = cross(t1, t2);
                continue;
            }
            t1 = cross(v3.V, v2.V);
            if (dot(t1, v0.V) < (R)0.0) {
                v1 = v3;
                t1 = v3.V - v0.V; t2 = v2.V - v0.V;
                normal = cross(t1, t2);
                continue;
            }
            break;
        }
        while (true) {
            phase2++;
            t1 = v2.V - v1.V;
            t2 = v3.V - v1.V;
            normal = cross(t1, t2);
            R nsq = len2(normal);
            if (nsq < NumericEpsilon) return false;
            if (!hit) {
                R d = dot(normal, v1.V);
                hit = d >= 0;
            }
            mk_support(sa, sb, qb, pb, normal, v4);
            t3 = v4.V - v3.V;
            R delta = dot(t3, normal);
            pen = dot(v4.V, normal);
            if (delta * delta <= eps * eps * nsq || pen <= (R)0.0 || phase2 > maxIter) {
                if (hit) {
                    R invn = (R)1.0 / std::sqrt(nsq);
                    pen *= invn;
                    if (pen > epa_threshold) {
                        poly.verts[0] = v0; poly.verts[1] = v1; poly.verts[2] = v2; poly.verts[3] = v3;
                        epa_calls++;
                        if (solve_mpr_epa(sa, sb, qb, pb, pA, pB, normal, pen)) return true;
                        epa_failures++;
                    }
                    normal = normal * invn;
                    t3 = cross(v1.V, t1);
                    R gamma = dot(t3, normal) * invn;
                    t3 = cross(t2, v1.V);
                    R beta = dot(t3, normal) * invn;
                    R alpha = (R)1.0 - gamma - beta;
                    pA = alpha * v1.A + beta * v2.A + gamma * v3.A;
                    pB = alpha * v1.B + beta * v2.B + gamma * v3.B;
                }
                return hit;
            }
            t1 = cross(v4.V, v0.V);
            R d = dot(t1, v1.V);
            if (d >= (R)0.0) {
                d = dot(t1, v2.V);
                if (d >= (R)0.0) v1 = v4; else v3 = v4;
            } else {
                d = dot(t1, v3.V);
                if (d >= (R)0.0) v2 = v4; else v1 = v4;
            }
        }
    }

    // MprEpaSolver.Collision, standalone EPA (NarrowPhase.cs:350-431)
    bool collision(const Shape<R>& sa, const Shape<R>& sb, Q4<R> qb, V3<R> pb,
                   V3<R>& p1, V3<R>& p2, V3<R>& n, R& pen) {
        const R eps = (R)1e-4;
        const int maxIter = 85;
        Vertex<R> cv;
        mk_center(sa, sb, qb, pb, cv);
        if (!poly.init_tetrahedron(cv.V)) { p1 = p2 = n = V3<R>(); pen = 0; return false; }
        int iter = 0;
        typename Polytope<R>::Tri ctri{};
        while (++iter < maxIter) {
            ctri = poly.tris[poly.closest_triangle()];
            V3<R> sd = ctri.closest;
            R sdsq = ctri.closest_sq;
            if (!poly.enclosed) sd = -sd;
            if (ctri.closest_sq < NumericEpsilon) { sd = ctri.normal; sdsq = ctri.normal_sq; }
            Vertex<R> v;
            mk_support(sa, sb, qb, pb, sd, v);
            R delta = dot(ctri.closest - v.V, sd);
            if (delta * delta <= eps * eps * sdsq) goto converged;
            {
                auto r = poly.add_vertex(v);
                if (r == Polytope<R>::NO_HORIZON) goto converged;
                if (r != Polytope<R>::ADDED) { p1 = p2 = n = V3<R>(); pen = 0; return false; }
            }
        }
        p1 = p2 = n = V3<R>();
        pen = 0;
        return false;
    converged:
        poly.calculate_points(ctri, p1, p2);
        pen = std::sqrt(ctri.closest_sq);
        if (!poly.enclosed) pen *= -(R)1.0;
        if (std::abs(pen) > NumericEpsilon) n = ctri.closest * ((R)1.0 / pen);
        else n = ctri.normal * ((R)1.0 / std::sqrt(ctri.normal_sq));
        return true;
    }

    // NarrowPhase.MprEpa, world-space wrapper (NarrowPhase.cs:902-927)
    bool mpr_epa_world(const Shape<R>& sa, const Shape<R>& sb, Q4<R> qa, Q4<R> qb, V3<R> pa, V3<R> pb,
                       V3<R>& pointA, V3<R>& pointB, V3<R>& normal, R& pen, R epa_threshold = (R)0.02) {
        Q4<R> q = qconjmul(qa, qb);
        V3<R> p = pb - pa;
        p = rotate_inv(p, qa);
        bool res = solve_mpr(sa, sb, q, p, epa_threshold, pointA, pointB, normal, pen);
        pointA = rotate(pointA, qa); pointA = pointA + pa;
        pointB = rotate(pointB, qa); pointB = pointB + pa;
        normal = rotate(normal, qa);
        return res;
    }
    // NarrowPhase.Collision world-space wrapper (NarrowPhase.cs Collision overload with two poses)
    bool collision_world(const Shape<R>& sa, const Shape<R>& sb, Q4<R> qa, Q4<R> qb, V3<R> pa, V3<R> pb,
                         V3<R>& pointA, V3<R>& pointB, V3<R>& normal, R& pen) {
        Q4<R> q = qconjmul(qa, qb);
        V3<R> p = pb - pa;
        p = rotate_inv(p, qa);
        bool res = collision(sa, sb, q, p, pointA, pointB, normal, pen);
        pointA = rotate(pointA, qa); pointA = pointA + pa;
        pointB = rotate(pointB, qa); pointB = pointB + pa;
        normal = rotate(normal, qa);
        return res;
    }
};

// ---- GJK simplex with witness points (Collision/NarrowPhase/SimplexSolverAB.cs:28-359) ---
// The simplex keeps up to four Minkowski vertices with their support points on A and B,
// the barycentric weights of the point closest to the origin, and a mask of the vertices
// that span it.  Each sub-simplex test reduces to the feature nearest the origin; the
// returned search point is computed directly (not from the weights) as the reference does.
template <class R> struct SimplexAB {
    static constexpr R Eps = (R)1e-8;
    Vertex<R> v[4];
    R bc[4];
    unsigned mask = 0;

    // ClosestSegment (SimplexSolverAB.cs:60-100)
    V3<R> segment(int i0, int i1, R* w, unsigned& m) const {
        V3<R> a = v[i0].V, b = v[i1].V;
        V3<R> d = b - a;
        R dd = len2(d);
        if (dd < Eps) { m = 1u << i1; w[i0] = 0; w[i1] = 1; return b; }
        R t = -dot(a, d) / dd;
        if (t > (R)1.0) { m = 1u << i1; w[i0] = 0; w[i1] = 1; return b; }
        if (t < (R)0.0) { m = 1u << i0; w[i0] = 1; w[i1] = 0; return a; }
        w[i0] = (R)1.0 - t; w[i1] = t;
        m = (1u << i0) | (1u << i1);
        return cross(d, cross(a, d)) * ((R)1.0 / dd);
    }
    // ClosestTriangle (SimplexSolverAB.cs:102-176): the interior when all three weights are
    // non-negative and the triangle is not degenerate, else the nearest of the edges whose
    // opposite weight is negative (all three when degenerate).
    V3<R> triangle(int i0, int i1, int i2, R* w, unsigned& m) const {
        m = 0;
        V3<R> a = v[i0].V, b = v[i1].V, c = v[i2].V;
        V3<R> u = a - b, e = a - c;
        V3<R> nrm = cross(u, e);
        R t = len2(nrm);
        R it = (R)1.0 / t;
        bool degenerate = t < Eps;
        R l2 = dot(cross(u, a), nrm) * it;
        R l1 = dot(cross(a, e), nrm) * it;
        R l0 = (R)1.0 - l2 - l1;
        R best = std::numeric_limits<R>::max();
        V3<R> cp;
        R tmp[4];
        const int edges[3][2] = {{i1, i2}, {i0, i2}, {i0, i1}};
        const R lam[3] = {l0, l1, l2};
        for (int k = 0; k < 3; k++) {
            if (!(lam[k] < (R)0.0 || degenerate)) continue;
            unsigned mk;
            V3<R> q = segment(edges[k][0], edges[k][1], tmp, mk);
            R dist = len2(q);
            if (dist < best) {
                for (int j = 0; j < 4; j++) w[j] = tmp[j];
                m = mk; cp = q;
                best = dist;
            }
        }
        if (m != 0) return cp;
        w[i0] = l0; w[i1] = l1; w[i2] = l2;
        m = (1u << i0) | (1u << i1) | (1u << i2);
        return nrm * (dot(nrm, a) * it);
    }
    static R det(V3<R> a, V3<R> b, V3<R> c, V3<R> d) { return dot(b - a, cross(c - a, d - a)); }
    // ClosestTetrahedron (SimplexSolverAB.cs:178-276)
    V3<R> tetra(R* w, unsigned& m) const {
        R dt = det(v[0].V, v[1].V, v[2].V, v[3].V);
        R idt = (R)1.0 / dt;
        bool degenerate = dt * dt < Eps;
        V3<R> z;
        R l0 = det(z, v[1].V, v[2].V, v[3].V) * idt;
        R l1 = det(v[0].V, z, v[2].V, v[3].V) * idt;
        R l2 = det(v[0].V, v[1].V, z, v[3].V) * idt;
        R l3 = (R)1.0 - l0 - l1 - l2;
        R best = std::numeric_limits<R>::max();
        V3<R> cp;
        R tmp[4];
        m = 0;
        const int faces[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
        const R lam[4] = {l0, l1, l2, l3};
        for (int k = 0; k < 4; k++) {
            if (!(lam[k] < (R)0.0 || degenerate)) continue;
            unsigned mk;
            V3<R> q = triangle(faces[k][0], faces[k][1], faces[k][2], tmp, mk);
            R dist = len2(q);
            if (dist < best) {
                for (int j = 0; j < 4; j++) w[j] = tmp[j];
                m = mk; cp = q;
                best = dist;
            }
        }
        if (m != 0) return cp;
        w[0] = l0; w[1] = l1; w[2] = l2; w[3] = l3;
        m = 15;
        return V3<R>();
    }
    // AddVertex (SimplexSolverAB.cs:300-357): false when the origin is enclosed.
    bool add(const Vertex<R>& x, V3<R>& closest) {
        int ix[4], used = 0, free_slot = 0;
        for (int i = 0; i < 4; i++) {
            if (mask & (1u << i)) ix[used++] = i;
            else free_slot = i;
        }
        ix[used++] = free_slot;
        v[free_slot] = x;
        switch (used) {
            case 1: closest = v[ix[0]].V; mask = 1u << ix[0]; bc[ix[0]] = 1; return true;
            case 2: closest = segment(ix[0], ix[1], bc, mask); return true;
            case 3: closest = triangle(ix[0], ix[1], ix[2], bc, mask); return true;
            default: closest = tetra(bc, mask); return mask != 15;
        }
    }
    // GetClosest (SimplexSolverAB.cs:278-293)
    void closest_points(V3<R>& pA, V3<R>& pB) const {
        pA = V3<R>(); pB = V3<R>();
        for (int i = 0; i < 4; i++) {
            if (!(mask & (1u << i))) continue;
            pA = pA + bc[i] * v[i].A;
            pB = pB + bc[i] * v[i].B;
        }
    }
};

// ---- time of impact (NarrowPhase.Sweep, NarrowPhase.cs:1100-1222) -------------------------
// Conservative advancement on the Minkowski difference, shape A fixed at the origin: B moves
// along `sweep`; each support point in front of the current search direction advances the
// time of impact lambda to the plane it spans, and the simplex is rebuilt around the
// moved B.  Returns false when B moves away from the current separating plane (no hit);
// true with lambda = 0 for shapes that already overlap.
template <class R> bool sweep_local(const Shape<R>& sa, const Shape<R>& sb, Q4<R> qb, V3<R> pb, V3<R> sweep,
                                    V3<R>& pA, V3<R>& pB, V3<R>& normal, R& lambda) {
    const R eps = (R)1e-4;
    int iter = 34;
    SimplexAB<R> sx;
    Vertex<R> c;
    mk_center(sa, sb, qb, pb, c);
    V3<R> pos = pb;
    lambda = 0;
    pA = pB = V3<R>();
    V3<R> r = sweep;
    V3<R> v = -c.V;
    normal = V3<R>();
    R d2 = len2(v);
    while (d2 > eps * eps && iter-- != 0) {
        Vertex<R> x;
        mk_support(sa, sb, qb, pos, v, x);
        R vw = -dot(v, x.V);
        if (vw > (R)0.0) {
            R vr = dot(v, r);
            if (vr >= -(R)1e-12) { lambda = std::numeric_limits<R>::infinity(); return false; }
            lambda -= vw / vr;
            pos = pb + lambda * r;
            normal = v;
        }
        if (!sx.add(x, v)) break;
        v = -v;
        d2 = len2(v);
    }
    sx.closest_points(pA, pB);
    normal = normalize_safe(normal, (R)1e-16);
    return true;
}
// World-space Sweep (NarrowPhase.cs:1100-1136): both bodies move with their linear
// velocities; the points come back at the bodies' current poses.
template <class R> bool sweep_world(const Shape<R>& sa, const Shape<R>& sb, Q4<R> qa, Q4<R> qb, V3<R> pa, V3<R> pb,
                                    V3<R> va, V3<R> vb, V3<R>& pA, V3<R>& pB, V3<R>& normal, R& lambda) {
    Q4<R> q = qconjmul(qa, qb);
    V3<R> p = rotate_inv(pb - pa, qa);
    V3<R> s = rotate_inv(vb - va, qa);
    if (!sweep_local(sa, sb, q, p, s, pA, pB, normal, lambda)) return false;
    pA = rotate(pA, qa); pA = pA + pa;
    pB = rotate(pB, qa); pB = pB + pa;
    normal = rotate(normal, qa);
    pB = pB + lambda * (va - vb);
    return true;
}

// ---- one-shot manifold (Collision/NarrowPhase/CollisionManifold.cs:22-586) ---------------
template <class R> struct Manifold {
    static const int MaxSupport = 6, MaxPoints = 12, SolverLimit = 4;
    static constexpr R DupSq = (R)0.001;
    static constexpr R Sqrt3Over2 = (R)0.86602540378;
    static constexpr R Perturbation = (R)0.01;
    V3<R> A[MaxPoints], B[MaxPoints];
    int count = 0;
    int lc = 0, rc = 0;

    static const R* hexagon() {
        static const R h[12] = {(R)1.0, (R)0.0, (R)0.5, Sqrt3Over2, -(R)0.5, Sqrt3Over2,
                                -(R)1.0, (R)0.0, -(R)0.5, -Sqrt3Over2, (R)0.5, -Sqrt3Over2};
        return h;
    }
    // PushLeft/PushRight (CollisionManifold.cs:64-96)
    static void push(V3<R>* arr, int& cnt, V3<R> v) {
        if (cnt > 0 && len2(arr[0] - v) < DupSq) return;
        if (cnt > 1 && len2(arr[cnt - 1] - v) < DupSq) return;
        arr[cnt++] = v;
    }
    // TryGetPolygonSign (CollisionManifold.cs:100-124)
    static bool polygon_sign(const V3<R>* poly, int cnt, V3<R> n, R& sign) {
        const R eps = (R)1e-6;
        R area = (R)0.0;
        V3<R> prev = poly[cnt - 1];
        for (int i = 0; i < cnt; i++) { V3<R> cur = poly[i]; area += dot(cross(prev, cur), n); prev = cur; }
        if (std::abs(area) <= eps) { sign = 0; return false; }
        sign = area < (R)0.0 ? -(R)1.0 : (R)1.0;
        return true;
    }
    // ContainsPoint (CollisionManifold.cs:127-142)
    static bool contains(const V3<R>* poly, int cnt, V3<R> p, V3<R> n, R sign) {
        const R eps = (R)1e-3;
        V3<R> prev = poly[cnt - 1];
        for (int i = 0; i < cnt; i++) {
            V3<R> cur = poly[i];
            R sd = sign * dot(cross(cur - prev, p - prev), n);
            if (sd < -eps) return false;
            prev = cur;
        }
        return true;
    }
    // ClipSegmentAgainstPolygon (CollisionManifold.cs:144-193)
    static int clip_segment(V3<R> s, V3<R> e, const V3<R>* poly, int pc, V3<R> n, R sign, V3<R>* out) {
        const R eps = (R)1e-3;
        R enter = (R)0.0, exit = (R)1.0;
        V3<R> delta = e - s;
        for (int i = 0; i < pc; i++) {
            V3<R> es = poly[i], ee = poly[(i + 1) % pc];
            R ss = sign * dot(cross(ee - es, s - es), n);
            R se = sign * dot(cross(ee - es, e - es), n);
            bool si = ss >= -eps, ei = se >= -eps;
            if (!si && !ei) return 0;
            if (si && ei) continue;
            R den = ss - se;
            if (std::abs(den) <= eps) return 0;
            R t = std::clamp(ss / den, (R)0.0, (R)1.0);
            if (!si) enter = std::max(enter, t); else exit = std::min(exit, t);
            if (exit < enter) return 0;
        }
        out[0] = s + enter * delta;
        if (len2(s + exit * delta - out[0]) < eps) return 1;
        out[1] = s + exit * delta;
        return 2;
    }
    static R cross_along(V3<R> l, V3<R> r, V3<R> n) { return dot(cross(l, r), n); }
    // IntersectSegments (CollisionManifold.cs:204-264)
    static int intersect(V3<R> sA, V3<R> eA, V3<R> sB, V3<R> eB, V3<R> n, V3<R>* cA, V3<R>* cB) {
        const R eps = (R)1e-3;
        V3<R> dA = eA - sA, dB = eB - sB, off = sB - sA;
        R cr = cross_along(dA, dB, n);
        if (std::abs(cr) <= eps) {
            if (std::abs(cross_along(off, dA, n)) > eps) return 0;
            R la = len2(dA), lb = len2(dB);
            if (la <= eps || lb <= eps) return 0;
            R b0 = dot(sB - sA, dA) / la, b1 = dot(eB - sA, dA) / la;
            R enter = std::max((R)0.0, std::min(b0, b1));
            R exit = std::min((R)1.0, std::max(b0, b1));
            if (exit < enter - eps) return 0;
            cA[0] = sA + enter * dA;
            R a0 = std::clamp(dot(cA[0] - sB, dB) / lb, (R)0.0, (R)1.0);
            cB[0] = sB + a0 * dB;
            cA[1] = sA + exit * dA;
            if (len2(cA[1] - cA[0]) <= eps) return 1;
            R a1 = std::clamp(dot(cA[1] - sB, dB) / lb, (R)0.0, (R)1.0);
            cB[1] = sB + a1 * dB;
            return 2;
        }
        R t = cross_along(off, dB, n) / cr;
        R u = cross_along(off, dA, n) / cr;
        if (t < -eps || t > (R)1.0 + eps || u < -eps || u > (R)1.0 + eps) return 0;
        t = std::clamp(t, (R)0.0, (R)1.0);
        u = std::clamp(u, (R)0.0, (R)1.0);
        cA[0] = sA + t * dA;
        cB[0] = sB + u * dB;
        return 1;
    }
    static bool is_dup(const V3<R>* m, int cnt, V3<R> p) {
        for (int i = 0; i < cnt; i++) if (len2(m[i] - p) < DupSq) return true;
        return false;
    }
    // AddPointOnA / AddPointOnB / AddPointPair (CollisionManifold.cs:277-318)
    void add_on_a(V3<R> p, V3<R> pB, V3<R> n) {
        if (count == MaxPoints) return;
        R diff = dot(p - pB, n);
        if (diff < (R)0.0) return;
        if (is_dup(A, count, p)) return;
        A[count] = p; B[count++] = p - diff * n;
    }
    void add_on_b(V3<R> p, V3<R> pA, V3<R> n) {
        if (count == MaxPoints) return;
        R diff = dot(p - pA, n);
        if (diff > (R)0.0) return;
        if (is_dup(B, count, p)) return;
        B[count] = p; A[count++] = p - diff * n;
    }
    void add_pair(V3<R> pa, V3<R> pb, V3<R> n) {
        if (count == MaxPoints) return;
        if (dot(pa - pb, n) < (R)0.0) return;
        if (is_dup(A, count, pa)) return;
        if (is_dup(B, count, pb)) return;
        A[count] = pa; B[count++] = pb;
    }
    // ReduceManifold (CollisionManifold.cs:321-375)
    void reduce(V3<R> n) {
        if (count <= SolverLimit) return;
        V3<R> c;
        for (int i = 0; i < count; i++) c = c + A[i];
        c = c * (R)(1.0 / count);
        V3<R> t1 = create_orthonormal(n);
        V3<R> t2 = cross(n, t1);
        double ang[MaxPoints];
        int order[MaxPoints];
        for (int i = 0; i < count; i++) {
            V3<R> d = A[i] - c;
            ang[i] = (double)StableMath<R>::atan2(dot(d, t2), dot(d, t1));
            order[i] = i;
        }
        for (int i = 1; i < count; i++) {
            int cur = order[i];
            double ca = ang[cur];
            int j = i - 1;
            while (j >= 0 && ang[order[j]] > ca) { order[j + 1] = order[j]; j--; }
            order[j + 1] = cur;
        }
        V3<R> rA[SolverLimit], rB[SolverLimit];
        for (int i = 0; i < SolverLimit; i++) {
            int sel = order[((2 * i + 1) * count) / (2 * SolverLimit)];
            rA[i] = A[sel]; rB[i] = B[sel];
        }
        for (int i = 0; i < SolverLimit; i++) { A[i] = rA[i]; B[i] = rB[i]; }
        count = SolverLimit;
    }
    // BuildManifold (CollisionManifold.cs:393-566)
    void build(const Shape<R>& sa, const Shape<R>& sb, Q4<R> qa, Q4<R> qb, V3<R> pa, V3<R> pb,
               V3<R> pA, V3<R> pB, V3<R> n) {
        lc = 0; rc = 0; count = 0;
        V3<R> c1 = create_orthonormal(n);
        V3<R> c2 = cross(n, c1);
        V3<R> relB = pb - pa, pAl = pA - pa, pBl = pB - pa;
        V3<R> left[MaxSupport], right[MaxSupport];
        const R* hx = hexagon();
        for (int e = 0; e < MaxSupport; e++) {
            V3<R> pn = n + hx[2 * e + 0] * Perturbation * c1 + hx[2 * e + 1] * Perturbation * c2;
            V3<R> tmp = rotate_inv(pn, qa);
            V3<R> np1 = support(sa, tmp);
            np1 = rotate(np1, qa);
            push(left, lc, np1);
            pn = -pn;
            tmp = rotate_inv(pn, qb);
            V3<R> np2 = support(sb, tmp);
            np2 = rotate(np2, qb);
            np2 = np2 + relB;
            push(right, rc, np2);
        }
        R ls = 0, rs = 0;
        bool lp = lc > 2 && polygon_sign(left, lc, n, ls);
        bool rp = rc > 2 && polygon_sign(right, rc, n, rs);
        if (lp) {
            for (int e = 0; e < rc; e++) {
                V3<R> p = right[e];
                if (!contains(left, lc, p, n, ls)) continue;
                add_on_b(p, pAl, n);
                if (count == MaxPoints) goto finalize;
            }
            if (rc == 2) {
                V3<R> cl[2];
                int k = clip_segment(right[0], right[1], left, lc, n, ls, cl);
                for (int i = 0; i < k; i++) { add_on_b(cl[i], pAl, n); if (count == MaxPoints) goto finalize; }
            }
        }
        if (rp) {
            for (int e = 0; e < lc; e++) {
                V3<R> p = left[e];
                if (!contains(right, rc, p, n, rs)) continue;
                add_on_a(p, pBl, n);
                if (count == MaxPoints) goto finalize;
            }
            if (lc == 2) {
                V3<R> cl[2];
                int k = clip_segment(left[0], left[1], right, rc, n, rs, cl);
                for (int i = 0; i < k; i++) { add_on_a(cl[i], pBl, n); if (count == MaxPoints) goto finalize; }
            }
        }
        if (lc == 2 && rc == 2) {
            V3<R> cA[2], cB[2];
            int k = intersect(left[0], left[1], right[0], right[1], n, cA, cB);
            for (int i = 0; i < k; i++) { add_pair(cA[i], cB[i], n); if (count == MaxPoints) goto finalize; }
        }
        if (lp && rp) {
            for (int i = 0; i < lc; i++) {
                V3<R> sA = left[i], eA = left[(i + 1) % lc];
                for (int j = 0; j < rc; j++) {
                    V3<R> sB = right[j], eB = right[(j + 1) % rc];
                    V3<R> cA[2], cB[2];
                    int k = intersect(sA, eA, sB, eB, n, cA, cB);
                    for (int m = 0; m < k; m++) { add_pair(cA[m], cB[m], n); if (count == MaxPoints) goto finalize; }
                }
            }
        }
        if (count <= 1) { A[0] = pAl; B[0] = pBl; count = 1; }
        else if (count < SolverLimit) { A[count] = pAl; B[count] = pBl; count++; }
    finalize:
        reduce(n);
        for (int i = 0; i < count; i++) { A[i] = A[i] + pa; B[i] = B[i] + pa; }
    }
};

// ---- TriangleEdgeCollisionFilter (CollisionFilter/TriangleEdgeCollisionFilter.cs:119-420) --
template <class R> struct EdgeFilter {
    enum Eval { KEEP, DISCARD, EDGE };
    R edge_threshold = (R)0.01, cos_angle = (R)0.999, projection_threshold = (R)0.5;
    bool filter_dynamic = false;

    static void project_on_plane(V3<R>& p, V3<R> a, V3<R> b, V3<R> c) {
        V3<R> ab = b - a, ac = c - a;
        V3<R> n = cross(ab, ac);
        n = normalize(n);
        V3<R> ap = p - a;
        R d = dot(ap, n);
        p = p - d * n;
    }
    // EvaluateTriangleContact (TriangleEdgeCollisionFilter.cs:183-240)
    Eval evaluate(const Shape<R>& tri, Q4<R> tq, V3<R> tp, bool tri_is_b, V3<R> cp, V3<R> n,
                  V3<R>& tn, V3<R>& nn) const {
        tn = rotate(tri.tnormal, tq);
        nn = V3<R>();
        if (tri_is_b) tn = -tn;
        if (dot(n, tn) < -cos_angle) return DISCARD;
        V3<R> a = rotate(tri.ta, tq) + tp, b = rotate(tri.tb, tq) + tp, c = rotate(tri.tc, tq) + tp;
        V3<R> pc = cp;
        project_on_plane(pc, a, b, c);
        V3<R> e = b - a, pma = pc - a;
        R d0 = len2(pma - dot(pma, e) * e * ((R)1.0 / len2(e)));
        e = c - a; pma = pc - a;
        R d1 = len2(pma - dot(pma, e) * e * ((R)1.0 / len2(e)));
        e = c - b; pma = pc - b;
        R d2 = len2(pma - dot(pma, e) * e * ((R)1.0 / len2(e)));
        if (std::min(std::min(d0, d1), d2) > edge_threshold * edge_threshold) return KEEP;
        int which;
        if (d0 < d1 && d0 < d2) which = 2;       // NeighborC
        else if (d1 < d2) which = 1;             // NeighborB
        else which = 0;                          // NeighborA
        if (!tri.nbr_valid[which]) return KEEP;
        nn = rotate(tri.nbr_normal[which], tq);
        if (tri_is_b) nn = -nn;
        return EDGE;
    }
    // Filter (TriangleEdgeCollisionFilter.cs:243-420).  body_dynamic: whether the triangle's
    // body is dynamic.  Returns false to discard the contact.
    bool filter(const Shape<R>& sa, const Shape<R>& sb, Q4<R> qa, Q4<R> qb, V3<R> pa, V3<R> pb,
                bool tri_body_dynamic, MprEpa<R>& solver, V3<R>& pA, V3<R>& pB, V3<R>& n, R& pen) const {
        bool c1 = sa.is_triangle(), c2 = sb.is_triangle();
        if (c1 == c2) return true;
        const Shape<R>& ts = c1 ? sa : sb;
        Q4<R> tq = c1 ? qa : qb;
        V3<R> tp = c1 ? pa : pb;
        if (tri_body_dynamic && !filter_dynamic) return true;
        V3<R> tn, nn;
        Eval ev = evaluate(ts, tq, tp, c2, c1 ? pA : pB, n, tn, nn);
        if (ev == DISCARD) return false;
        if (ev == KEEP) return true;
        bool spec = pen < (R)0.0;
        if (!spec) {
            bool res = solver.mpr_epa_world(sa, sb, qa, qb, pa, pb, pA, pB, n, pen, (R)0.0);
            if (!res) return false;
            ev = evaluate(ts, tq, tp, c2, c1 ? pA : pB, n, tn, nn);
            if (ev == DISCARD) return false;
            if (ev == KEEP) return true;
        }
        V3<R> mid = (R)0.5 * (pA + pB);
        if (dot(tn, nn) > cos_angle) {
            R f5 = dot(n, nn), f6 = dot(n, tn);
            if (!spec) { pen = 0; pA = pB = mid; }
            n = f5 > f6 ? nn : tn;
            return true;
        }
        V3<R> cr = cross(nn, tn);
        R crl = len2(cr);
        V3<R> proj = n - (dot(cr, n) / crl) * cr;
        if (len2(proj) < projection_threshold * projection_threshold) return false;
        R f1 = dot(cross(proj, nn), cr);
        R f2 = dot(cross(proj, tn), cr);
        bool between = f1 <= (R)0.0 && f2 >= (R)0.0;
        if (!between) {
            R f3 = dot(n, nn), f4 = dot(n, tn);
            if (!spec) { pen = 0; pA = pB = mid; }
            n = f3 > f4 ? nn : tn;
        }
        return true;
    }
};

}  // namespace jor
