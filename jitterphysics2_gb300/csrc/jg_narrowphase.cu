// Narrowphase: one warp per broadphase pair.  MPR (NarrowPhase.cs:98-347), EPA with the
// polytope in shared memory (NarrowPhase.cs:39-95, ConvexPolytope.cs), the triangle-edge
// filter (TriangleEdgeCollisionFilter.cs:243-420) and the one-shot manifold
// (CollisionManifold.cs:393-566) run fused; colliding pairs append one record (key,
// normal, up to four point pairs) to the compacted contact stream.
//
// Lanes of a warp hold identical copies of the MPR state; point-cloud support maps, the
// EPA face scans (closest face, visibility, fan construction) and the manifold's segment
// intersections are split across lanes.  EPA keeps its face data in FP32; FP64 is used
// only when a face normal is too cancelled to trust (exact expansion recomputation, as
// the reference's ExpansionArithmetic.Normal) and when the FP32 orientation filter cannot
// prove a sign (the reference's double filter, then exact expansions).  The device
// polytope holds 64 vertices / 128 faces (the reference: 128 / 256); running out ends
// EPA with the MPR result, the reference's behaviour on any EPA failure.
//
// The MPR follows code the reference adapted from XenoCollide (zlib license, (c) 2007-2014
// Gary Snethen, http://xenocollide.com): provided 'as-is', without any express or implied
// warranty; altered source versions must be plainly marked as such; this notice may not
// be removed or altered from any source distribution.
#include "jg_shapes.cuh"
#include <math_constants.h>

namespace {

constexpr unsigned FULL = 0xffffffffu;

struct MV { v3 V, A, B; };

// MinkowskiDifference.Support (MinkowskiDifference.cs:57-69).  WARP: the 32 lanes of a
// warp evaluate it together (point clouds split across lanes); otherwise one thread.
template <bool WARP>
__device__ __forceinline__ void mk_support_t(const ShapeRef& sa, const ShapeRef& sb, q4 qb, v3 pb, v3 d, MV& v) {
    v3 tmp = -d;
    v.A = WARP ? support(sa, d) : support_lane(sa, d);
    v3 tmp2 = rotate_inv(tmp, qb);
    v.B = WARP ? support(sb, tmp2) : support_lane(sb, tmp2);
    v.B = rotate(v.B, qb);
    v.B = v.B + pb;
    v.V = v.A - v.B;
}
__device__ __forceinline__ void mk_support(const ShapeRef& sa, const ShapeRef& sb, q4 qb, v3 pb, v3 d, MV& v) {
    mk_support_t<true>(sa, sb, qb, pb, d, v);
}
__device__ __forceinline__ void mk_center(const ShapeRef& sa, const ShapeRef& sb, q4 qb, v3 pb, MV& c) {
    c.A = shape_center(sa);
    c.B = rotate(shape_center(sb), qb);
    c.B = pb + c.B;
    c.V = c.A - c.B;
}

// ---- exact arithmetic (double expansions), used only on unresolved EPA predicates -------
struct Exp {
    __device__ static int diff(double a, double b, double* o) {
        double v = a - b, vb = a - v;
        double res = (a - (v + vb)) + (vb - b);
        int n = 0;
        if (res != 0) o[n++] = res;
        if (v != 0) o[n++] = v;
        return n;
    }
    __device__ static int grow(double* e, int len, double value) {
        int cnt = 0;
        for (int i = 0; i < len; i++) {
            double part = e[i];
            double sum = value + part;
            double vp = sum - value;
            double res = (value - (sum - vp)) + (part - vp);
            if (res != 0) e[cnt++] = res;
            value = sum;
        }
        if (value != 0) e[cnt++] = value;
        return cnt;
    }
    __device__ static int addp(double* r, int len, const double* a, int na, const double* b, int nb, bool neg, int cap) {
        for (int i = 0; i < na; i++)
            for (int j = 0; j < nb; j++) {
                double x = a[i], y = b[j];
                double p = __dmul_rn(x, y);
                double res = fma(x, y, -p);
                if (neg) { p = -p; res = -res; }
                if (res != 0 && len < cap) len = grow(r, len, res);
                if (p != 0 && len < cap) len = grow(r, len, p);
            }
        return len;
    }
    __device__ static int crossterm(const double* a, int na, const double* b, int nb, const double* c, int nc,
                                    const double* d, int nd, double* o) {
        int len = addp(o, 0, a, na, b, nb, false, 16);
        return addp(o, len, c, nc, d, nd, true, 16);
    }
    // ExpansionArithmetic.Side (ExactArithmetic/ExpansionArithmetic.cs:20-41)
    __device__ __noinline__ static int side(v3 a, v3 b, v3 c, v3 p) {
        double ux[2], uy[2], uz[2], vx[2], vy[2], vz[2], dx[2], dy[2], dz[2];
        int nx = diff(a.x, b.x, ux), ny = diff(a.y, b.y, uy), nz = diff(a.z, b.z, uz);
        int mx = diff(a.x, c.x, vx), my = diff(a.y, c.y, vy), mz = diff(a.z, c.z, vz);
        int px = diff(p.x, a.x, dx), py = diff(p.y, a.y, dy), pz = diff(p.z, a.z, dz);
        double cr[16], det[192];
        int len = crossterm(uy, ny, vz, mz, uz, nz, vy, my, cr);
        int cnt = addp(det, 0, cr, len, dx, px, false, 192);
        len = crossterm(uz, nz, vx, mx, ux, nx, vz, mz, cr);
        cnt = addp(det, cnt, cr, len, dy, py, false, 192);
        len = crossterm(ux, nx, vy, my, uy, ny, vx, mx, cr);
        cnt = addp(det, cnt, cr, len, dz, pz, false, 192);
        if (cnt == 0) return 0;
        double t = det[cnt - 1];
        return t > 0 ? 1 : (t < 0 ? -1 : 0);
    }
    // ExpansionArithmetic.Normal (ExpansionArithmetic.cs:43-55): each component of
    // (a-b) x (a-c) as an exact expansion, summed from the least significant part up
    __device__ __noinline__ static void normal(v3 a, v3 b, v3 c, double& x, double& y, double& z) {
        double ux[2], uy[2], uz[2], vx[2], vy[2], vz[2], cr[16];
        int nx = diff(a.x, b.x, ux), ny = diff(a.y, b.y, uy), nz = diff(a.z, b.z, uz);
        int mx = diff(a.x, c.x, vx), my = diff(a.y, c.y, vy), mz = diff(a.z, c.z, vz);
        double r[3];
        int len = crossterm(uy, ny, vz, mz, uz, nz, vy, my, cr);
        double s = 0; for (int i = 0; i < len; i++) s += cr[i]; r[0] = s;
        len = crossterm(uz, nz, vx, mx, ux, nx, vz, mz, cr);
        s = 0; for (int i = 0; i < len; i++) s += cr[i]; r[1] = s;
        len = crossterm(ux, nx, vy, my, uy, ny, vx, mx, cr);
        s = 0; for (int i = 0; i < len; i++) s += cr[i]; r[2] = s;
        x = r[0]; y = r[1]; z = r[2];
    }
};

// PlaneFilter in double (ExactArithmetic/PlaneFilter.cs:29-70); the FP32 filter below
// tries first.
__device__ __noinline__ bool dfilter_side(v3 a, v3 b, v3 c, v3 p, int& sign) {
    const double EF = 16 * 1.1102230246251565e-16;
    double ux = (double)a.x - b.x, uy = (double)a.y - b.y, uz = (double)a.z - b.z;
    double vx = (double)a.x - c.x, vy = (double)a.y - c.y, vz = (double)a.z - c.z;
    double yz = uy * vz, zy = uz * vy, zx = uz * vx, xz = ux * vz, xy = ux * vy, yx = uy * vx;
    double nx = yz - zy, ny = zx - xz, nz = xy - yx;
    double ex = EF * (fabs(yz) + fabs(zy)), ey = EF * (fabs(zx) + fabs(xz)), ez = EF * (fabs(xy) + fabs(yx));
    double dx = (double)p.x - a.x, dy = (double)p.y - a.y, dz = (double)p.z - a.z;
    double x = nx * dx, y = ny * dy, z = nz * dz;
    double value = (x + y) + z;
    double round = EF * ((fabs(x) + fabs(y)) + fabs(z));
    double coef = (ex * fabs(dx) + ey * fabs(dy)) + ez * fabs(dz);
    if (fabs(value) <= round + 2 * coef) return false;
    sign = value > 0 ? 1 : -1;
    return true;
}

// FP32 version of the same filter: identical bound structure with u = 2^-24.
__device__ __forceinline__ bool ffilter_side(v3 a, v3 b, v3 c, v3 p, int& sign) {
    const float EF = 16.0f * 5.9604645e-08f;
    float ux = a.x - b.x, uy = a.y - b.y, uz = a.z - b.z;
    float vx = a.x - c.x, vy = a.y - c.y, vz = a.z - c.z;
    float yz = uy * vz, zy = uz * vy, zx = uz * vx, xz = ux * vz, xy = ux * vy, yx = uy * vx;
    float nx = yz - zy, ny = zx - xz, nz = xy - yx;
    float ex = EF * (fabsf(yz) + fabsf(zy)), ey = EF * (fabsf(zx) + fabsf(xz)), ez = EF * (fabsf(xy) + fabsf(yx));
    float dx = p.x - a.x, dy = p.y - a.y, dz = p.z - a.z;
    float x = nx * dx, y = ny * dy, z = nz * dz;
    float value = (x + y) + z;
    float round = EF * ((fabsf(x) + fabsf(y)) + fabsf(z));
    float coef = (ex * fabsf(dx) + ey * fabsf(dy)) + ez * fabsf(dz);
    // the difference of two float coordinates is inexact in float: widen the bound for
    // the extra rounding of the displacement (covered by the factor 4)
    if (fabsf(value) <= 4.0f * (round + 2.0f * coef) || !isfinite(value)) return false;
    sign = value > 0 ? 1 : -1;
    return true;
}

// Per-warp EPA polytope, in dynamic shared memory.  Vertices and faces at the reference's
// capacity (ConvexPolytope.cs:53-54).  Each face keeps what the reference's Triangle and
// FaceData keep for the search: the squared distance of its closest point in FP64 (the
// closest-face choice compares these), and the closest point and its squared distance
// rounded to FP32 (the support direction and the convergence test).  Everything else a
// face has in FP64 (plane normal, barycentric coordinates) is a deterministic function of
// its corners and is recomputed, bit for bit, where it is needed: for the rare search
// along a face normal and for the witness points of the final face.
struct EpaSmem {
    float4 vV[JG_EPA_MAXV], vA[JG_EPA_MAXV], vB[JG_EPA_MAXV];
    double fd[JG_EPA_MAXT];     // squared distance of the closest point (FP64)
    float4 fc[JG_EPA_MAXT];     // closest point xyz, squared distance (both rounded to FP32)
    uchar4 fi[JG_EPA_MAXT];     // a, b, c, flags (1: facing the origin, 2: corners swapped)
    unsigned char ea[3 * JG_EPA_MAXT], eb[3 * JG_EPA_MAXT];
    unsigned lit[JG_EPA_MAXT / 32];
    int nv, nt, ne, enclosed;
    // manifold scratch
    float4 mA[12], mB[12];
    float4 left[6], right[6];
};
#define EPA_FACING 1
#define EPA_SWAPPED 2

enum { ADDED = 0, NO_HORIZON = 1, DEGENERATE = 2, CAPACITY = 3, NUMERICAL = 4 };

struct NpStats { int exact; };

// ConvexPolytope.Side (ConvexPolytope.cs:321-327): orientation of point p relative to face
// (a,b,c).  Every filter that answers is certified, so the sign is the exact one whichever
// answers: the FP32 filter first, then the reference's FP64 filter, then exact expansions.
__device__ __forceinline__ int side_pt(v3 a, v3 b, v3 c, v3 p, NpStats& st) {
    if (p == a || p == b || p == c) return 0;
    int s;
    if (ffilter_side(a, b, c, p, s)) return s;
    st.exact++;
    if (dfilter_side(a, b, c, p, s)) return s;
    return Exp::side(a, b, c, p);
}

// PlaneFilter.IsSafe (ExactArithmetic/PlaneFilter.cs:73-77) for float coordinates.
__device__ __forceinline__ bool safe_coord(float v) {
    float a = fabsf(v);
    return v == 0.f || (a >= 1e-30f && a <= 1e30f);
}
__device__ __forceinline__ bool is_safe(v3 p) { return safe_coord(p.x) && safe_coord(p.y) && safe_coord(p.z); }

// FP64 vector helpers in the reference's evaluation order (ConvexPolytope.Double3).
struct d3 { double x, y, z; };
__device__ __forceinline__ d3 dv(v3 v) { return d3{(double)v.x, (double)v.y, (double)v.z}; }
__device__ __forceinline__ double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ d3 dcross(d3 a, d3 b) { return d3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ d3 dsub(d3 a, d3 b) { return d3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ d3 dadd(d3 a, d3 b) { return d3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ d3 dmul(d3 a, double s) { return d3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ bool dfinite(d3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }
__device__ __forceinline__ double dclamp01(double x) { return x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x); }

// ConvexPolytope.CalcBarycentric (ConvexPolytope.cs:328-395), FP64.
__device__ bool calc_bary(d3 a, d3 b, d3 c, d3 n, double nscale, double nsq, d3& out) {
    d3 u = dsub(a, b), v = dsub(a, c);
    double gamma = (ddot(dcross(u, a), n) / nsq) / nscale;
    double beta = (ddot(dcross(a, v), n) / nsq) / nscale;
    double alpha = 1.0 - gamma - beta;
    bool clamped = false;
    if (alpha >= 0 && beta < 0) {
        double t = ddot(a, u);
        if (gamma < 0 && t > 0) { beta = fmin(1.0, t / ddot(u, u)); alpha = 1 - beta; gamma = 0; }
        else { gamma = dclamp01(ddot(a, v) / ddot(v, v)); alpha = 1 - gamma; beta = 0; }
        clamped = true;
    } else if (beta >= 0 && gamma < 0) {
        d3 w = dsub(b, c);
        double t = ddot(b, w);
        if (alpha < 0 && t > 0) { gamma = fmin(1.0, t / ddot(w, w)); beta = 1 - gamma; alpha = 0; }
        else { alpha = dclamp01(-ddot(b, u) / ddot(u, u)); beta = 1 - alpha; gamma = 0; }
        clamped = true;
    } else if (gamma >= 0 && alpha < 0) {
        d3 w = dsub(b, c);
        double t = -ddot(c, v);
        if (beta < 0 && t > 0) { alpha = fmin(1.0, t / ddot(v, v)); gamma = 1 - alpha; beta = 0; }
        else { beta = dclamp01(-ddot(c, w) / ddot(w, w)); gamma = 1 - beta; alpha = 0; }
        clamped = true;
    }
    out = d3{alpha, beta, gamma};
    return clamped;
}

// The FP64 geometry of a face (ConvexPolytope.CreateTriangle, ConvexPolytope.cs:267-318):
// p0, p1, p2 are the corners in creation order; `swapped` when the orientation test
// exchanged the first two.  The raw normal is the FP64 plane filter's cross product of the
// creation order (PlaneFilter.cs:29-45), negated on a swap, and replaced by the exact
// expansion normal of the final order when the filter calls it unreliable
// (PlaneFilter.cs:24-27).  Returns false on a numerical failure.
struct FaceGeo { d3 sn; double nscale, nsq; d3 bc, cl; double d2; };
__device__ __noinline__ bool face_geo(v3 p0, v3 p1, v3 p2, bool swapped, FaceGeo& g, NpStats& st) {
    const double EF = 16 * 1.1102230246251565e-16;
    double ux = (double)p0.x - p1.x, uy = (double)p0.y - p1.y, uz = (double)p0.z - p1.z;
    double vx = (double)p0.x - p2.x, vy = (double)p0.y - p2.y, vz = (double)p0.z - p2.z;
    double yz = uy * vz, zy = uz * vy, zx = uz * vx, xz = ux * vz, xy = ux * vy, yx = uy * vx;
    d3 raw{yz - zy, zx - xz, xy - yx};
    double ex = EF * (fabs(yz) + fabs(zy)), ey = EF * (fabs(zx) + fabs(xz)), ez = EF * (fabs(xy) + fabs(yx));
    if (swapped) raw = d3{-raw.x, -raw.y, -raw.z};
    v3 a = swapped ? p1 : p0, b = swapped ? p0 : p1, c = p2;
    if (!(fmax(fabs(raw.x), fmax(fabs(raw.y), fabs(raw.z))) > 1048576 * fmax(ex, fmax(ey, ez)))) {
        st.exact++;
        Exp::normal(a, b, c, raw.x, raw.y, raw.z);
    }
    double ns = fmax(fabs(raw.x), fmax(fabs(raw.y), fabs(raw.z)));
    if (!(ns > 0) || !isfinite(ns)) return false;
    g.nscale = ns;
    g.sn = d3{raw.x / ns, raw.y / ns, raw.z / ns};
    g.nsq = ddot(g.sn, g.sn);
    d3 va = dv(a), vb = dv(b), vc = dv(c);
    bool clamped = calc_bary(va, vb, vc, g.sn, ns, g.nsq, g.bc);
    g.cl = clamped ? dadd(dadd(dmul(va, g.bc.x), dmul(vb, g.bc.y)), dmul(vc, g.bc.z))
                   : dmul(g.sn, ddot(g.sn, va) / g.nsq);
    g.d2 = ddot(g.cl, g.cl);
    return dfinite(g.cl) && dfinite(g.bc) && isfinite(g.d2);
}

// The face's geometry from its stored corners and flags.
__device__ __forceinline__ bool face_geo_of(const EpaSmem& E, int f, FaceGeo& g, NpStats& st) {
    uchar4 t = E.fi[f];
    bool sw = (t.w & EPA_SWAPPED) != 0;
    int p0 = sw ? t.y : t.x, p1 = sw ? t.x : t.y;
    return face_geo(mk3(E.vV[p0]), mk3(E.vV[p1]), mk3(E.vV[t.z]), sw, g, st);
}

// The FP32 normal of a face and its squared length (Triangle.Normal / NormalSq).
__device__ __forceinline__ float4 face_normal32(const FaceGeo& g) {
    v3 n = mk3((float)g.sn.x, (float)g.sn.y, (float)g.sn.z);
    return f4(n, len2(n));
}

// ConvexPolytope.CreateTriangle (ConvexPolytope.cs:267-318), one lane per face.
__device__ __noinline__ int create_tri(EpaSmem& E, int a, int b, int c, int slot, NpStats& st) {
    v3 va = mk3(E.vV[a]), vb = mk3(E.vV[b]), vc = mk3(E.vV[c]);
    v3 p0 = va, p1 = vb;
    int orient = 0;
    for (int i = 0; i < 4 && orient == 0; i++) {
        if (i == a || i == b || i == c) continue;
        orient = -side_pt(va, vb, vc, mk3(E.vV[i]), st);
    }
    if (orient == 0) return DEGENERATE;
    const bool swapped = orient < 0;
    if (swapped) { int t = a; a = b; b = t; v3 tv = va; va = vb; vb = tv; }
    bool facing = side_pt(va, vb, vc, mk3(0.f), st) <= 0;
    FaceGeo g;
    if (!face_geo(p0, p1, vc, swapped, g, st)) return NUMERICAL;
    v3 cl = mk3((float)g.cl.x, (float)g.cl.y, (float)g.cl.z);
    float d2 = (float)g.d2;
    if (!isfinite(cl.x) || !isfinite(cl.y) || !isfinite(cl.z) || !isfinite(d2)) return NUMERICAL;
    E.fi[slot] = make_uchar4((unsigned char)a, (unsigned char)b, (unsigned char)c,
                             (unsigned char)((facing ? EPA_FACING : 0) | (swapped ? EPA_SWAPPED : 0)));
    E.fd[slot] = g.d2;
    E.fc[slot] = f4(cl, d2);
    return ADDED;
}

// ConvexPolytope.InitTetrahedron (ConvexPolytope.cs:113-132)
__device__ bool epa_init(EpaSmem& E, NpStats& st) {
    const int lane = threadIdx.x & 31;
    if (lane == 0) { E.nv = 4; E.nt = 0; E.enclosed = 0; }
    __syncwarp();
    bool safe = true;
    for (int i = 0; i < 4; i++) safe = safe && is_safe(mk3(E.vV[i]));
    if (!safe) return false;
    const int idx[12] = {0, 2, 1, 0, 1, 3, 0, 3, 2, 1, 2, 3};
    int r = ADDED;
    if (lane < 4) r = create_tri(E, idx[3 * lane], idx[3 * lane + 1], idx[3 * lane + 2], lane, st);
    bool ok = __all_sync(FULL, r == ADDED);
    __syncwarp();
    if (ok && lane == 0) E.nt = 4;
    __syncwarp();
    return ok;
}

// ConvexPolytope.GetClosestTriangle (ConvexPolytope.cs:147-166): the smallest FP64 squared
// distance, the first such face on a tie.
__device__ int epa_closest(EpaSmem& E) {
    const int lane = threadIdx.x & 31;
    double best = CUDART_INF;
    int bi = 0x7fffffff;
    bool notfacing = false;
    int nt = E.nt;
    for (int i = lane; i < nt; i += 32) {
        double d = E.fd[i];
        if (d < best) { best = d; bi = i; }
        if (!(E.fi[i].w & EPA_FACING)) notfacing = true;
    }
    for (int off = 16; off > 0; off >>= 1) {
        double ob = __shfl_xor_sync(FULL, best, off);
        int oi = __shfl_xor_sync(FULL, bi, off);
        if (ob < best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    bool any_nf = __any_sync(FULL, notfacing);
    bool skip = E.enclosed != 0;
    __syncwarp();
    if (lane == 0) E.enclosed = any_nf ? (skip ? 1 : 0) : 1;
    __syncwarp();
    if (bi == 0x7fffffff) bi = 0;
    return bi;
}

// ConvexPolytope.AddVertexDetailed (ConvexPolytope.cs:199-265)
__device__ __noinline__ int epa_add(EpaSmem& E, const MV& v, NpStats& st) {
    const int lane = threadIdx.x & 31;
    if (E.nt == 0 || !is_safe(v.V)) return NUMERICAL;
    int nv = E.nv;
    if (nv == JG_EPA_MAXV) return CAPACITY;
    if (lane == 0) { E.vV[nv] = f4(v.V, 0.f); E.vA[nv] = f4(v.A, 0.f); E.vB[nv] = f4(v.B, 0.f); }
    __syncwarp();
    int nt = E.nt;
    // visibility of every face, lanes in parallel
    for (int base = 0; base < nt; base += 32) {
        int i = base + lane;
        bool lit = false;
        if (i < nt) {
            uchar4 f = E.fi[i];
            lit = side_pt(mk3(E.vV[f.x]), mk3(E.vV[f.y]), mk3(E.vV[f.z]), v.V, st) > 0;
        }
        unsigned m = __ballot_sync(FULL, lit);
        if (lane == 0) E.lit[base >> 5] = m;
    }
    __syncwarp();
    // horizon edges in the reference's order (faces from last to first), one lane
    if (lane == 0) {
        int ne = 0;
        for (int index = nt; index-- > 0;) {
            if (!((E.lit[index >> 5] >> (index & 31)) & 1u)) continue;
            uchar4 f = E.fi[index];
            unsigned char cs[3] = {f.x, f.y, f.z};
            for (int k = 0; k < 3; k++) {
                unsigned char A = cs[k], B = cs[(k + 1) % 3];
                bool added = true;
                for (int e = ne; e-- > 0;) {
                    bool match = (E.ea[e] == A && E.eb[e] == B) || (E.ea[e] == B && E.eb[e] == A);
                    if (!match) continue;
                    --ne;
                    E.ea[e] = E.ea[ne]; E.eb[e] = E.eb[ne];
                    added = false;
                    break;
                }
                if (added && ne < 3 * JG_EPA_MAXT) { E.ea[ne] = A; E.eb[ne] = B; ne++; }
            }
        }
        E.ne = ne;
    }
    __syncwarp();
    int ne = E.ne;
    if (ne == 0) return NO_HORIZON;
    int nlit = 0;
    for (int k = 0; k < (nt + 31) / 32; k++) nlit += __popc(E.lit[k] & (k * 32 + 32 <= nt ? 0xffffffffu : ((1u << (nt & 31)) - 1u)));
    if (nt - nlit + ne > JG_EPA_MAXT) return CAPACITY;
    // order-preserving compaction of the surviving faces
    int surv = 0;
    for (int base = 0; base < nt; base += 32) {
        int i = base + lane;
        bool keep = i < nt && !((E.lit[i >> 5] >> (i & 31)) & 1u);
        uchar4 fi; float4 fc; double fd;
        if (keep) { fi = E.fi[i]; fc = E.fc[i]; fd = E.fd[i]; }
        unsigned m = __ballot_sync(FULL, keep);
        int dst = surv + __popc(m & ((1u << lane) - 1u));
        __syncwarp();
        if (keep) { E.fi[dst] = fi; E.fc[dst] = fc; E.fd[dst] = fd; }
        surv += __popc(m);
        __syncwarp();
    }
    // the new fan, one face per lane
    int res = ADDED;
    for (int base = 0; base < ne; base += 32) {
        int e = base + lane;
        int r = ADDED;
        if (e < ne) r = create_tri(E, E.ea[e], E.eb[e], nv, surv + e, st);
        for (int off = 16; off > 0; off >>= 1) {
            int o = __shfl_xor_sync(FULL, r, off);
            if (o != ADDED && (r == ADDED || o < r)) r = o;
        }
        if (r != ADDED && res == ADDED) res = r;
    }
    __syncwarp();
    if (res != ADDED) {
        if (lane == 0) { E.nt = 0; E.enclosed = 0; }
        __syncwarp();
        return res;
    }
    if (lane == 0) { E.nt = surv + ne; E.nv = nv + 1; }
    __syncwarp();
    return ADDED;
}

// MprEpaSolver.SolveMprEpa (NarrowPhase.cs:39-95).  Seed vertices are in E.v*[0..3].
__device__ __noinline__ bool solve_epa(EpaSmem& E, const ShapeRef& sa, const ShapeRef& sb, q4 qb, v3 pb,
                          v3& p1, v3& p2, v3& n, float& pen, NpStats& st) {
    const float eps = 1e-5f;
    const int maxIter = 85;
    if (!epa_init(E, st)) return false;
    int iter = 0;
    int ci = 0;
    while (++iter < maxIter) {
        ci = epa_closest(E);
        float4 fc = E.fc[ci];
        v3 sd = mk3(fc), cl = mk3(fc);
        float sdsq = fc.w;
        if (!E.enclosed) sd = -sd;
        if (fc.w < 1e-16f) {
            // search along the face normal (Triangle.Normal / NormalSq)
            FaceGeo g;
            face_geo_of(E, ci, g, st);
            float4 fn = face_normal32(g);
            sd = mk3(fn); sdsq = fn.w;
        }
        MV v;
        mk_support(sa, sb, qb, pb, sd, v);
        float delta = dot(cl - v.V, sd);
        if (delta * delta <= eps * eps * sdsq) goto converged;
        {
            int r = epa_add(E, v, st);
            if (r == NO_HORIZON) goto converged;
            if (r != ADDED) return false;
        }
    }
    return false;
converged:
    if (!E.enclosed) return false;
    {
        // ConvexPolytope.CalculatePoints (ConvexPolytope.cs:169-185): the FP64 barycentric
        // combination of the corners' support points, rounded to FP32
        uchar4 f = E.fi[ci];
        FaceGeo g;
        face_geo_of(E, ci, g, st);
        d3 a = dadd(dadd(dmul(dv(mk3(E.vA[f.x])), g.bc.x), dmul(dv(mk3(E.vA[f.y])), g.bc.y)), dmul(dv(mk3(E.vA[f.z])), g.bc.z));
        d3 b = dadd(dadd(dmul(dv(mk3(E.vB[f.x])), g.bc.x), dmul(dv(mk3(E.vB[f.y])), g.bc.y)), dmul(dv(mk3(E.vB[f.z])), g.bc.z));
        p1 = mk3((float)a.x, (float)a.y, (float)a.z);
        p2 = mk3((float)b.x, (float)b.y, (float)b.z);
        float4 fn = face_normal32(g);
        n = mk3(fn) * (1.0f / sqrtf(fn.w));
        pen = sqrtf(E.fc[ci].w);
    }
    return true;
}

// MprEpaSolver.SolveMpr (NarrowPhase.cs:98-347) up to the EPA hand-off.  Returns 0 (no
// overlap), 1 (overlap, result final) or 2 (overlap deeper than epa_threshold: the MPR
// result is in pA/pB/normal/pen as the fallback, and `portal` holds the tetrahedron EPA
// starts from).  WARP: evaluated redundantly by a whole warp; otherwise one thread.
template <bool WARP>
__device__ int mpr_core(const ShapeRef& sa, const ShapeRef& sb, q4 qb, v3 pb, float epa_threshold,
                        v3& pA, v3& pB, v3& normal, float& pen, MV* portal) {
    const float eps = 1e-5f;
    const int maxIter = 34;
    const float NumericEpsilon = 1e-16f;
    MV v0, v1, v2, v3v, v4;
    v3 t1, t2, t3;
    pen = 0.0f;
    mk_center(sa, sb, qb, pb, v0);
    if (fabsf(v0.V.x) < NumericEpsilon && fabsf(v0.V.y) < NumericEpsilon && fabsf(v0.V.z) < NumericEpsilon) v0.V.x = 1e-05f;
    normal = -v0.V;
    mk_support_t<WARP>(sa, sb, qb, pb, normal, v1);
    pA = v1.A; pB = v1.B;
    if (dot(v1.V, normal) <= 0.0f) return 0;
    normal = cross(v1.V, v0.V);
    if (len2(normal) < 1e-12f) {
        normal = v1.V - v0.V;
        normal = normalize(normal);
        t1 = v1.A - v1.B;
        pen = dot(t1, normal);
        return 1;
    }
    mk_support_t<WARP>(sa, sb, qb, pb, normal, v2);
    if (dot(v2.V, normal) <= 0.0f) return 0;
    t1 = v1.V - v0.V;
    t2 = v2.V - v0.V;
    normal = cross(t1, t2);
    float dist = dot(normal, v0.V);
    if (dist > 0.0f) {
        MV t = v1;
        v1 = v2; v2 = t;
        normal = -normal;
    }
    int phase2 = 0, phase1 = 0;
    bool hit = false;
    while (true) {
        if (phase1 > maxIter) return 0;
        phase1++;
        mk_support_t<WARP>(sa, sb, qb, pb, normal, v3v);
        if (dot(v3v.V, normal) <= 0.0f) return 0;
        t1 = cross(v1.V, v3v.V);
        if (dot(t1, v0.V) < 0.0f) {
            v2 = v3v;
            t1 = v1.V - v0.V; t2 = v3v.V - v0.V;
            normal = cross(t1, t2);
            continue;
        }
        t1 = cross(v3v.V, v2.V);
        if (dot(t1, v0.V) < 0.0f) {
            v1 = v3v;
            t1 = v3v.V - v0.V; t2 = v2.V - v0.V;
            normal = cross(t1, t2);
            continue;
        }
        break;
    }
    while (true) {
        phase2++;
        t1 = v2.V - v1.V;
        t2 = v3v.V - v1.V;
        normal = cross(t1, t2);
        float nsq = len2(normal);
        if (nsq < NumericEpsilon) return 0;
        if (!hit) {
            float d = dot(normal, v1.V);
            hit = d >= 0;
        }
        mk_support_t<WARP>(sa, sb, qb, pb, normal, v4);
        t3 = v4.V - v3v.V;
        float delta = dot(t3, normal);
        pen = dot(v4.V, normal);
        if (delta * delta <= eps * eps * nsq || pen <= 0.0f || phase2 > maxIter) {
            if (!hit) return 0;
            float invn = 1.0f / sqrtf(nsq);
            pen *= invn;
            int code = 1;
            if (pen > epa_threshold) {
                portal[0] = v0; portal[1] = v1; portal[2] = v2; portal[3] = v3v;
                code = 2;
            }
            normal = normal * invn;
            t3 = cross(v1.V, t1);
            float gamma = dot(t3, normal) * invn;
            t3 = cross(t2, v1.V);
            float beta = dot(t3, normal) * invn;
            float alpha = 1.0f - gamma - beta;
            pA = alpha * v1.A + beta * v2.A + gamma * v3v.A;
            pB = alpha * v1.B + beta * v2.B + gamma * v3v.B;
            return code;
        }
        t1 = cross(v4.V, v0.V);
        float d = dot(t1, v1.V);
        if (d >= 0.0f) {
            d = dot(t1, v2.V);
            if (d >= 0.0f) v1 = v4; else v3v = v4;
        } else {
            d = dot(t1, v3v.V);
            if (d >= 0.0f) v2 = v4; else v1 = v4;
        }
    }
}

// EPA from a saved MPR portal, by the whole warp; on failure the MPR result stands
// (NarrowPhase.cs:287-298).
__device__ void run_epa(EpaSmem& E, const ShapeRef& sa, const ShapeRef& sb, q4 qb, v3 pb, const MV* portal,
                        v3& pA, v3& pB, v3& normal, float& pen, NpStats& st, int& epa_calls, int& epa_fail) {
    const int lane = threadIdx.x & 31;
    if (lane < 4) {
        E.vV[lane] = f4(portal[lane].V, 0.f);
        E.vA[lane] = f4(portal[lane].A, 0.f);
        E.vB[lane] = f4(portal[lane].B, 0.f);
    }
    __syncwarp();
    epa_calls++;
    v3 a, b, n;
    float p;
    if (solve_epa(E, sa, sb, qb, pb, a, b, n, p, st)) { pA = a; pB = b; normal = n; pen = p; }
    else epa_fail++;
}

// MprEpaSolver.SolveMpr with its EPA refinement, whole warp (the edge filter's rerun).
__device__ __noinline__ bool solve_mpr(EpaSmem& E, const ShapeRef& sa, const ShapeRef& sb, q4 qb, v3 pb, float epa_threshold,
                          v3& pA, v3& pB, v3& normal, float& pen, NpStats& st, int& epa_calls, int& epa_fail) {
    MV portal[4];
    int code = mpr_core<true>(sa, sb, qb, pb, epa_threshold, pA, pB, normal, pen, portal);
    if (code == 2) run_epa(E, sa, sb, qb, pb, portal, pA, pB, normal, pen, st, epa_calls, epa_fail);
    return code != 0;
}

// NarrowPhase.MprEpa world-space wrapper (NarrowPhase.cs:902-927)
__device__ bool mpr_epa_world(EpaSmem& E, const ShapeRef& sa, const ShapeRef& sb, q4 qa, q4 qb, v3 pa, v3 pb,
                              v3& pA, v3& pB, v3& n, float& pen, float threshold, NpStats& st, int& ec, int& ef) {
    q4 q = qmul(qconj(qa), qb);
    v3 p = rotate_inv(pb - pa, qa);
    bool res = solve_mpr(E, sa, sb, q, p, threshold, pA, pB, n, pen, st, ec, ef);
    pA = rotate(pA, qa); pA = pA + pa;
    pB = rotate(pB, qa); pB = pB + pa;
    n = rotate(n, qa);
    return res;
}

// ---- TriangleEdgeCollisionFilter (TriangleEdgeCollisionFilter.cs:183-420) ---------------
enum { KEEP = 0, DISCARD = 1, EDGE = 2 };
__device__ __noinline__ int edge_evaluate(const WorldDev& w, int tri, q4 tq, v3 tp, bool tri_is_b, v3 cp, v3 n, v3& tn, v3& nn) {
    const TriDev& T = w.tris[tri];
    const float cosAngle = 0.999f, edgeThreshold = 0.01f;
    tn = rotate(mk3(T.n), tq);
    nn = mk3(0.f);
    if (tri_is_b) tn = -tn;
    if (dot(n, tn) < -cosAngle) return DISCARD;
    v3 a = rotate(mk3(T.a), tq) + tp, b = rotate(mk3(T.b), tq) + tp, c = rotate(mk3(T.c), tq) + tp;
    v3 pc = cp;
    {
        v3 ab = b - a, ac = c - a;
        v3 pn = normalize(cross(ab, ac));
        v3 ap = pc - a;
        float d = dot(ap, pn);
        pc = pc - d * pn;
    }
    v3 e = b - a, pma = pc - a;
    float d0 = len2(pma - dot(pma, e) * e * (1.0f / len2(e)));
    e = c - a; pma = pc - a;
    float d1 = len2(pma - dot(pma, e) * e * (1.0f / len2(e)));
    e = c - b; pma = pc - b;
    float d2 = len2(pma - dot(pma, e) * e * (1.0f / len2(e)));
    if (fminf(fminf(d0, d1), d2) > edgeThreshold * edgeThreshold) return KEEP;
    int which;
    if (d0 < d1 && d0 < d2) which = 2;
    else if (d1 < d2) which = 1;
    else which = 0;
    float4 nb = T.nb[which];
    if (nb.w == 0.f) return KEEP;
    nn = rotate(mk3(nb), tq);
    if (tri_is_b) nn = -nn;
    return EDGE;
}

// ---- one-shot manifold (CollisionManifold.cs) --------------------------------------------
__device__ __forceinline__ void push_pt(float4* arr, int& cnt, v3 v) {
    if (cnt > 0 && len2(mk3(arr[0]) - v) < 0.001f) return;
    if (cnt > 1 && len2(mk3(arr[cnt - 1]) - v) < 0.001f) return;
    if ((threadIdx.x & 31) == 0) arr[cnt] = f4(v, 0.f);
    cnt++;
    __syncwarp();
}
__device__ bool polygon_sign(const float4* poly, int cnt, v3 n, float& sign) {
    float area = 0.0f;
    v3 prev = mk3(poly[cnt - 1]);
    for (int i = 0; i < cnt; i++) { v3 cur = mk3(poly[i]); area += dot(cross(prev, cur), n); prev = cur; }
    if (fabsf(area) <= 1e-6f) { sign = 0.f; return false; }
    sign = area < 0.0f ? -1.0f : 1.0f;
    return true;
}
__device__ bool contains_pt(const float4* poly, int cnt, v3 p, v3 n, float sign) {
    v3 prev = mk3(poly[cnt - 1]);
    for (int i = 0; i < cnt; i++) {
        v3 cur = mk3(poly[i]);
        float sd = sign * dot(cross(cur - prev, p - prev), n);
        if (sd < -1e-3f) return false;
        prev = cur;
    }
    return true;
}
__device__ int clip_segment(v3 s, v3 e, const float4* poly, int pc, v3 n, float sign, v3* out) {
    const float eps = 1e-3f;
    float enter = 0.0f, exit = 1.0f;
    v3 delta = e - s;
    for (int i = 0; i < pc; i++) {
        v3 es = mk3(poly[i]), ee = mk3(poly[(i + 1) % pc]);
        float ss = sign * dot(cross(ee - es, s - es), n);
        float se = sign * dot(cross(ee - es, e - es), n);
        bool si = ss >= -eps, ei = se >= -eps;
        if (!si && !ei) return 0;
        if (si && ei) continue;
        float den = ss - se;
        if (fabsf(den) <= eps) return 0;
        float t = fminf(fmaxf(ss / den, 0.0f), 1.0f);
        if (!si) enter = fmaxf(enter, t); else exit = fminf(exit, t);
        if (exit < enter) return 0;
    }
    out[0] = s + enter * delta;
    if (len2(s + exit * delta - out[0]) < eps) return 1;
    out[1] = s + exit * delta;
    return 2;
}
__device__ __forceinline__ float cross_along(v3 l, v3 r, v3 n) { return dot(cross(l, r), n); }
__device__ int intersect_seg(v3 sA, v3 eA, v3 sB, v3 eB, v3 n, v3* cA, v3* cB) {
    const float eps = 1e-3f;
    v3 dA = eA - sA, dB = eB - sB, off = sB - sA;
    float cr = cross_along(dA, dB, n);
    if (fabsf(cr) <= eps) {
        if (fabsf(cross_along(off, dA, n)) > eps) return 0;
        float la = len2(dA), lb = len2(dB);
        if (la <= eps || lb <= eps) return 0;
        float b0 = dot(sB - sA, dA) / la, b1 = dot(eB - sA, dA) / la;
        float enter = fmaxf(0.0f, fminf(b0, b1));
        float exit = fminf(1.0f, fmaxf(b0, b1));
        if (exit < enter - eps) return 0;
        cA[0] = sA + enter * dA;
        float a0 = fminf(fmaxf(dot(cA[0] - sB, dB) / lb, 0.0f), 1.0f);
        cB[0] = sB + a0 * dB;
        cA[1] = sA + exit * dA;
        if (len2(cA[1] - cA[0]) <= eps) return 1;
        float a1 = fminf(fmaxf(dot(cA[1] - sB, dB) / lb, 0.0f), 1.0f);
        cB[1] = sB + a1 * dB;
        return 2;
    }
    float t = cross_along(off, dB, n) / cr;
    float u = cross_along(off, dA, n) / cr;
    if (t < -eps || t > 1.0f + eps || u < -eps || u > 1.0f + eps) return 0;
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    u = fminf(fmaxf(u, 0.0f), 1.0f);
    cA[0] = sA + t * dA;
    cB[0] = sB + u * dB;
    return 1;
}
__device__ bool is_dup(const float4* m, int cnt, v3 p) {
    for (int i = 0; i < cnt; i++) if (len2(mk3(m[i]) - p) < 0.001f) return true;
    return false;
}
struct MF {
    EpaSmem* E;
    int count;
    __device__ void set(int i, v3 a, v3 b) {
        if ((threadIdx.x & 31) == 0) { E->mA[i] = f4(a, 0.f); E->mB[i] = f4(b, 0.f); }
        __syncwarp();
    }
    __device__ void on_a(v3 p, v3 pB, v3 n) {
        if (count == 12) return;
        float diff = dot(p - pB, n);
        if (diff < 0.0f) return;
        if (is_dup(E->mA, count, p)) return;
        set(count, p, p - diff * n);
        count++;
    }
    __device__ void on_b(v3 p, v3 pA, v3 n) {
        if (count == 12) return;
        float diff = dot(p - pA, n);
        if (diff > 0.0f) return;
        if (is_dup(E->mB, count, p)) return;
        set(count, p - diff * n, p);
        count++;
    }
    __device__ void pair(v3 a, v3 b, v3 n) {
        if (count == 12) return;
        if (dot(a - b, n) < 0.0f) return;
        if (is_dup(E->mA, count, a)) return;
        if (is_dup(E->mB, count, b)) return;
        set(count, a, b);
        count++;
    }
};

__device__ __noinline__ int build_manifold(EpaSmem& E, const ShapeRef& sa, const ShapeRef& sb, q4 qa, q4 qb, v3 pa, v3 pb,
                              v3 pA, v3 pB, v3 n, v3* outA, v3* outB) {
    const int lane = threadIdx.x & 31;
    const float P = 0.01f, S = 0.86602540378f;
    const float hx[12] = {1.0f, 0.0f, 0.5f, S, -0.5f, S, -1.0f, 0.0f, -0.5f, -S, 0.5f, -S};
    v3 c1 = create_orthonormal(n);
    v3 c2 = cross(n, c1);
    v3 relB = pb - pa, pAl = pA - pa, pBl = pB - pa;
    int lc = 0, rc = 0;
    for (int e = 0; e < 6; e++) {
        v3 pn = n + hx[2 * e + 0] * P * c1 + hx[2 * e + 1] * P * c2;
        v3 np1 = rotate(support(sa, rotate_inv(pn, qa)), qa);
        push_pt(E.left, lc, np1);
        pn = -pn;
        v3 np2 = rotate(support(sb, rotate_inv(pn, qb)), qb) + relB;
        push_pt(E.right, rc, np2);
    }
    float ls = 0.f, rs = 0.f;
    bool lp = lc > 2 && polygon_sign(E.left, lc, n, ls);
    bool rp = rc > 2 && polygon_sign(E.right, rc, n, rs);
    MF m; m.E = &E; m.count = 0;
    if (lp) {
        for (int e = 0; e < rc; e++) {
            v3 p = mk3(E.right[e]);
            if (!contains_pt(E.left, lc, p, n, ls)) continue;
            m.on_b(p, pAl, n);
            if (m.count == 12) goto finalize;
        }
        if (rc == 2) {
            v3 cl[2];
            int k = clip_segment(mk3(E.right[0]), mk3(E.right[1]), E.left, lc, n, ls, cl);
            for (int i = 0; i < k; i++) { m.on_b(cl[i], pAl, n); if (m.count == 12) goto finalize; }
        }
    }
    if (rp) {
        for (int e = 0; e < lc; e++) {
            v3 p = mk3(E.left[e]);
            if (!contains_pt(E.right, rc, p, n, rs)) continue;
            m.on_a(p, pBl, n);
            if (m.count == 12) goto finalize;
        }
        if (lc == 2) {
            v3 cl[2];
            int k = clip_segment(mk3(E.left[0]), mk3(E.left[1]), E.right, rc, n, rs, cl);
            for (int i = 0; i < k; i++) { m.on_a(cl[i], pBl, n); if (m.count == 12) goto finalize; }
        }
    }
    if (lc == 2 && rc == 2) {
        v3 cA[2], cB[2];
        int k = intersect_seg(mk3(E.left[0]), mk3(E.left[1]), mk3(E.right[0]), mk3(E.right[1]), n, cA, cB);
        for (int i = 0; i < k; i++) { m.pair(cA[i], cB[i], n); if (m.count == 12) goto finalize; }
    }
    if (lp && rp) {
        // every (left edge, right edge) intersection, one lane per edge pair, inserted in
        // the reference's (i, j) order
        int total = lc * rc;
        for (int base = 0; base < total; base += 32) {
            int idx = base + lane;
            v3 cA[2], cB[2];
            int k = 0;
            if (idx < total) {
                int i = idx / rc, j = idx % rc;
                k = intersect_seg(mk3(E.left[i]), mk3(E.left[(i + 1) % lc]), mk3(E.right[j]), mk3(E.right[(j + 1) % rc]), n, cA, cB);
            }
            unsigned any = __ballot_sync(FULL, k > 0);
            while (any) {
                int src = __ffs(any) - 1;
                any &= any - 1;
                int kk = __shfl_sync(FULL, k, src);
                for (int q = 0; q < kk; q++) {
                    v3 a, b;
                    a.x = __shfl_sync(FULL, cA[q].x, src); a.y = __shfl_sync(FULL, cA[q].y, src); a.z = __shfl_sync(FULL, cA[q].z, src);
                    b.x = __shfl_sync(FULL, cB[q].x, src); b.y = __shfl_sync(FULL, cB[q].y, src); b.z = __shfl_sync(FULL, cB[q].z, src);
                    m.pair(a, b, n);
                    if (m.count == 12) goto finalize;
                }
            }
        }
    }
    if (m.count <= 1) { m.set(0, pAl, pBl); m.count = 1; }
    else if (m.count < 4) { m.set(m.count, pAl, pBl); m.count++; }
finalize:
    int count = m.count;
    if (count > 4) {
        // ReduceManifold (CollisionManifold.cs:321-375)
        v3 c = mk3(0.f);
        for (int i = 0; i < count; i++) c = c + mk3(E.mA[i]);
        c = c * (float)(1.0 / count);
        v3 t1 = create_orthonormal(n);
        v3 t2 = cross(n, t1);
        float ang[12];
        int order[12];
        for (int i = 0; i < count; i++) {
            v3 d = mk3(E.mA[i]) - c;
            ang[i] = StableMathF::atan2(dot(d, t2), dot(d, t1));
            order[i] = i;
        }
        for (int i = 1; i < count; i++) {
            int cur = order[i];
            float ca = ang[cur];
            int j = i - 1;
            while (j >= 0 && ang[order[j]] > ca) { order[j + 1] = order[j]; j--; }
            order[j + 1] = cur;
        }
        for (int i = 0; i < 4; i++) {
            int sel = order[((2 * i + 1) * count) / 8];
            outA[i] = mk3(E.mA[sel]) + pa;
            outB[i] = mk3(E.mB[sel]) + pa;
        }
        __syncwarp();
        return 4;
    }
    for (int i = 0; i < count; i++) { outA[i] = mk3(E.mA[i]) + pa; outB[i] = mk3(E.mB[i]) + pa; }
    __syncwarp();
    return count;
}

// ---- one-shot manifold, one thread per pair ----------------------------------------------
// The same steps as build_manifold (CollisionManifold.cs:393-566) with the candidate lists
// in thread-local storage, for analytic shapes and point clouds alike.
struct MFT {
    float4 A[12], B[12];
    int count;
    __device__ void on_a(v3 p, v3 pB, v3 n) {
        if (count == 12) return;
        float diff = dot(p - pB, n);
        if (diff < 0.0f) return;
        if (is_dup(A, count, p)) return;
        A[count] = f4(p, 0.f); B[count] = f4(p - diff * n, 0.f); count++;
    }
    __device__ void on_b(v3 p, v3 pA, v3 n) {
        if (count == 12) return;
        float diff = dot(p - pA, n);
        if (diff > 0.0f) return;
        if (is_dup(B, count, p)) return;
        A[count] = f4(p - diff * n, 0.f); B[count] = f4(p, 0.f); count++;
    }
    __device__ void pair(v3 a, v3 b, v3 n) {
        if (count == 12) return;
        if (dot(a - b, n) < 0.0f) return;
        if (is_dup(A, count, a)) return;
        if (is_dup(B, count, b)) return;
        A[count] = f4(a, 0.f); B[count] = f4(b, 0.f); count++;
    }
};
__device__ __forceinline__ void push_local(float4* arr, int& cnt, v3 v) {
    if (cnt > 0 && len2(mk3(arr[0]) - v) < 0.001f) return;
    if (cnt > 1 && len2(mk3(arr[cnt - 1]) - v) < 0.001f) return;
    arr[cnt++] = f4(v, 0.f);
}

__device__ __noinline__ int manifold_thread(const ShapeRef& sa, const ShapeRef& sb, q4 qa, q4 qb, v3 pa, v3 pb,
                                            v3 pA, v3 pB, v3 n, float4* outA, float4* outB) {
    const float P = 0.01f, S = 0.86602540378f;
    const float hx[12] = {1.0f, 0.0f, 0.5f, S, -0.5f, S, -1.0f, 0.0f, -0.5f, -S, 0.5f, -S};
    v3 c1 = create_orthonormal(n);
    v3 c2 = cross(n, c1);
    v3 relB = pb - pa, pAl = pA - pa, pBl = pB - pa;
    float4 left[6], right[6];
    int lc = 0, rc = 0;
    for (int e = 0; e < 6; e++) {
        v3 pn = n + hx[2 * e + 0] * P * c1 + hx[2 * e + 1] * P * c2;
        push_local(left, lc, rotate(support_lane(sa, rotate_inv(pn, qa)), qa));
        pn = -pn;
        push_local(right, rc, rotate(support_lane(sb, rotate_inv(pn, qb)), qb) + relB);
    }
    float ls = 0.f, rs = 0.f;
    bool lp = lc > 2 && polygon_sign(left, lc, n, ls);
    bool rp = rc > 2 && polygon_sign(right, rc, n, rs);
    MFT m;
    m.count = 0;
    if (lp) {
        for (int e = 0; e < rc; e++) {
            v3 p = mk3(right[e]);
            if (!contains_pt(left, lc, p, n, ls)) continue;
            m.on_b(p, pAl, n);
            if (m.count == 12) goto finalize;
        }
        if (rc == 2) {
            v3 cl[2];
            int k = clip_segment(mk3(right[0]), mk3(right[1]), left, lc, n, ls, cl);
            for (int i = 0; i < k; i++) { m.on_b(cl[i], pAl, n); if (m.count == 12) goto finalize; }
        }
    }
    if (rp) {
        for (int e = 0; e < lc; e++) {
            v3 p = mk3(left[e]);
            if (!contains_pt(right, rc, p, n, rs)) continue;
            m.on_a(p, pBl, n);
            if (m.count == 12) goto finalize;
        }
        if (lc == 2) {
            v3 cl[2];
            int k = clip_segment(mk3(left[0]), mk3(left[1]), right, rc, n, rs, cl);
            for (int i = 0; i < k; i++) { m.on_a(cl[i], pBl, n); if (m.count == 12) goto finalize; }
        }
    }
    if (lc == 2 && rc == 2) {
        v3 cA[2], cB[2];
        int k = intersect_seg(mk3(left[0]), mk3(left[1]), mk3(right[0]), mk3(right[1]), n, cA, cB);
        for (int i = 0; i < k; i++) { m.pair(cA[i], cB[i], n); if (m.count == 12) goto finalize; }
    }
    if (lp && rp) {
        for (int i = 0; i < lc; i++) {
            v3 sA = mk3(left[i]), eA = mk3(left[(i + 1) % lc]);
            for (int j = 0; j < rc; j++) {
                v3 cA[2], cB[2];
                int k = intersect_seg(sA, eA, mk3(right[j]), mk3(right[(j + 1) % rc]), n, cA, cB);
                for (int q = 0; q < k; q++) { m.pair(cA[q], cB[q], n); if (m.count == 12) goto finalize; }
            }
        }
    }
    if (m.count <= 1) { m.A[0] = f4(pAl, 0.f); m.B[0] = f4(pBl, 0.f); m.count = 1; }
    else if (m.count < 4) { m.A[m.count] = f4(pAl, 0.f); m.B[m.count] = f4(pBl, 0.f); m.count++; }
finalize:
    int count = m.count;
    if (count > 4) {
        // ReduceManifold (CollisionManifold.cs:321-375)
        v3 c = mk3(0.f);
        for (int i = 0; i < count; i++) c = c + mk3(m.A[i]);
        c = c * (float)(1.0 / count);
        v3 t1 = create_orthonormal(n);
        v3 t2 = cross(n, t1);
        float ang[12];
        int order[12];
        for (int i = 0; i < count; i++) {
            v3 d = mk3(m.A[i]) - c;
            ang[i] = StableMathF::atan2(dot(d, t2), dot(d, t1));
            order[i] = i;
        }
        for (int i = 1; i < count; i++) {
            int cur = order[i];
            float ca = ang[cur];
            int j = i - 1;
            while (j >= 0 && ang[order[j]] > ca) { order[j + 1] = order[j]; j--; }
            order[j + 1] = cur;
        }
        for (int i = 0; i < 4; i++) {
            int sel = order[((2 * i + 1) * count) / 8];
            outA[i] = f4(mk3(m.A[sel]) + pa, 0.f);
            outB[i] = f4(mk3(m.B[sel]) + pa, 0.f);
        }
        return 4;
    }
    for (int i = 0; i < count; i++) { outA[i] = f4(mk3(m.A[i]) + pa, 0.f); outB[i] = f4(mk3(m.B[i]) + pa, 0.f); }
    return count;
}

constexpr int NP_WARPS = 4;

__device__ __forceinline__ int warp_append(int* counter, bool pred) {
    const int lane = threadIdx.x & 31;
    unsigned m = __ballot_sync(FULL, pred);
    if (!m) return -1;
    int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(FULL, base, leader);
    return pred ? base + __popc(m & ((1u << lane) - 1u)) : -1;
}

// Pairs grouped by the kinds of their two shapes (a counting sort over the 64 kind
// combinations), so that the threads of a warp run the same support maps in MPR.  The
// order inside a group does not matter: results do not depend on the pair order.
__device__ __forceinline__ int pair_kind_key(const WorldDev& w, int p) {
    int2 pr = w.pairs[p];
    return ((w.sinfo[pr.x].x & 7) << 3) | (w.sinfo[pr.y].x & 7);
}
__global__ void k_pair_hist(WorldDev w) {
    __shared__ int h[64];
    if (threadIdx.x < 64) h[threadIdx.x] = 0;
    __syncthreads();
    const int n = min(w.ctr->npairs, w.cap_pairs);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        atomicAdd(&h[pair_kind_key(w, p)], 1);
    __syncthreads();
    if (threadIdx.x < 64 && h[threadIdx.x]) atomicAdd(&w.pair_kind[threadIdx.x], h[threadIdx.x]);
}
__global__ void k_pair_offsets(WorldDev w) {
    int acc = 0;
    for (int k = 0; k < 64; k++) { w.pair_kind[64 + k] = acc; acc += w.pair_kind[k]; }
}
__global__ void k_pair_scatter(WorldDev w) {
    const int n = min(w.ctr->npairs, w.cap_pairs);
    const int lane = threadIdx.x & 31;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int key = pair_kind_key(w, p);
        const unsigned act = __activemask();
        const unsigned same = __match_any_sync(act, key);
        const int leader = __ffs(same) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&w.pair_kind[64 + key], __popc(same));
        base = __shfl_sync(act, base, leader);
        w.pair_order[base + __popc(same & ((1u << lane) - 1u))] = p;
    }
}

// Stage 1, one thread per broadphase pair: the MPR overlap test in A's frame
// (NarrowPhase.MprEpa, NarrowPhase.cs:902-927, up to the EPA hand-off).  Overlapping pairs
// are appended to the colliding list with their MPR result; deeper than the EPA threshold,
// also to the EPA list with the MPR portal EPA starts from.  Separated pairs with a
// speculative body go to the sweep list (World.Detect.cs:162-170).
__global__ void __launch_bounds__(256, 2) k_mpr(WorldDev w) {
    const int npairs = min(w.ctr->npairs, w.cap_pairs);
    const int cap = w.cap_arb;
    for (int base = blockIdx.x * blockDim.x; base < npairs; base += gridDim.x * blockDim.x) {
        const int q = base + threadIdx.x;
        const int p = q < npairs ? w.pair_order[q] : npairs;
        int code = 0;
        bool sweep = false;
        v3 pA, pB, n;
        float pen = 0.f;
        MV portal[4];
        if (p < npairs) {
            int2 pr = w.pairs[p];
            int s1 = pr.x, s2 = pr.y;  // s1 < s2: ShapeId order (World.Detect.cs:141-144)
            int b1 = w.sinfo[s1].y, b2 = w.sinfo[s2].y;
            int4 i1 = w.binfo[b1], i2 = w.binfo[b2];
            bool skip = (!(i1.y & JG_BODY_ACTIVE) && !(i2.y & JG_BODY_ACTIVE)) ||
                        (i1.x != JG_MOTION_DYNAMIC && i2.x != JG_MOTION_DYNAMIC);
            if (!skip) {
                ShapeRef sa = load_shape(w, s1), sb = load_shape(w, s2);
                q4 qa = mkq(w.q[b1]), qb = mkq(w.q[b2]);
                v3 pa = mk3(w.pos[b1]), pb = mk3(w.pos[b2]);
                q4 q = qmul(qconj(qa), qb);
                v3 pr_ = rotate_inv(pb - pa, qa);
                const bool spec_body = ((i1.y | i2.y) & JG_BODY_SPECULATIVE) != 0;
                code = mpr_core<false>(sa, sb, q, pr_, 0.02f, pA, pB, n, pen, portal);
                sweep = code == 0 && spec_body;
            }
        }
        int si = warp_append(&w.ctr->nspec, sweep);
        if (si >= 0) w.spec_list[si] = p;
        int c = warp_append(&w.ctr->ncol, code != 0);
        if (c >= cap) { atomicCAS(&w.ctr->status, 0, JG_ERR_CAPACITY); c = -1; }
        if (c >= 0) {
            w.col_pair[c] = make_int2(p, code);
            w.col_res[3 * c + 0] = f4(pA, 0.f);
            w.col_res[3 * c + 1] = f4(pB, 0.f);
            w.col_res[3 * c + 2] = f4(n, pen);
        }
        int e = warp_append(&w.ctr->nepa_list, code == 2 && c >= 0);
        if (e >= 0) {
            w.epa_list[e] = c;
            for (int k = 0; k < 4; k++) {
                w.col_portal[12 * e + 3 * k + 0] = f4(portal[k].V, 0.f);
                w.col_portal[12 * e + 3 * k + 1] = f4(portal[k].A, 0.f);
                w.col_portal[12 * e + 3 * k + 2] = f4(portal[k].B, 0.f);
            }
        }
    }
}

// ---- speculative contacts: time of impact by conservative advancement --------------------
// GJK simplex with witness points (SimplexSolverAB.cs:28-359), one thread: up to four
// Minkowski vertices with their support points on A and B, the barycentric weights of the
// point nearest the origin, and the mask of the vertices spanning it.
struct SimplexAB {
    MV v[4];
    float bc[4];
    unsigned mask;

    // ClosestSegment (SimplexSolverAB.cs:60-100)
    __device__ v3 segment(int i0, int i1, float* w, unsigned& m) const {
        v3 a = v[i0].V, b = v[i1].V;
        v3 d = b - a;
        float dd = len2(d);
        if (dd < 1e-8f) { m = 1u << i1; w[i0] = 0.f; w[i1] = 1.f; return b; }
        float t = -dot(a, d) / dd;
        if (t > 1.0f) { m = 1u << i1; w[i0] = 0.f; w[i1] = 1.f; return b; }
        if (t < 0.0f) { m = 1u << i0; w[i0] = 1.f; w[i1] = 0.f; return a; }
        w[i0] = 1.0f - t; w[i1] = t;
        m = (1u << i0) | (1u << i1);
        return cross(d, cross(a, d)) * (1.0f / dd);
    }
    // ClosestTriangle (SimplexSolverAB.cs:102-176): the interior when every weight is
    // non-negative and the triangle is not degenerate, else the nearest edge among those
    // opposite a negative weight (all three edges when degenerate).
    __device__ v3 triangle(int i0, int i1, int i2, float* w, unsigned& m) const {
        m = 0;
        v3 a = v[i0].V, b = v[i1].V, c = v[i2].V;
        v3 u = a - b, e = a - c;
        v3 nrm = cross(u, e);
        float t = len2(nrm);
        float it = 1.0f / t;
        bool degenerate = t < 1e-8f;
        float l2 = dot(cross(u, a), nrm) * it;
        float l1 = dot(cross(a, e), nrm) * it;
        float l0 = 1.0f - l2 - l1;
        const int ea[3] = {i1, i0, i0}, eb[3] = {i2, i2, i1};
        const float lam[3] = {l0, l1, l2};
        float best = 3.402823466e+38f;
        v3 cp = mk3(0.f);
        float tmp[4];
        for (int k = 0; k < 3; k++) {
            if (!(lam[k] < 0.0f || degenerate)) continue;
            unsigned mk;
            v3 q = segment(ea[k], eb[k], tmp, mk);
            float dist = len2(q);
            if (dist < best) {
                for (int j = 0; j < 4; j++) w[j] = tmp[j];
                m = mk; cp = q; best = dist;
            }
        }
        if (m != 0) return cp;
        w[i0] = l0; w[i1] = l1; w[i2] = l2;
        m = (1u << i0) | (1u << i1) | (1u << i2);
        return nrm * (dot(nrm, a) * it);
    }
    __device__ static float det(v3 a, v3 b, v3 c, v3 d) { return dot(b - a, cross(c - a, d - a)); }
    // ClosestTetrahedron (SimplexSolverAB.cs:178-276)
    __device__ v3 tetra(float* w, unsigned& m) const {
        float dt = det(v[0].V, v[1].V, v[2].V, v[3].V);
        float idt = 1.0f / dt;
        bool degenerate = dt * dt < 1e-8f;
        v3 z = mk3(0.f);
        float l0 = det(z, v[1].V, v[2].V, v[3].V) * idt;
        float l1 = det(v[0].V, z, v[2].V, v[3].V) * idt;
        float l2 = det(v[0].V, v[1].V, z, v[3].V) * idt;
        float l3 = 1.0f - l0 - l1 - l2;
        const int fa[4] = {1, 0, 0, 0}, fb[4] = {2, 2, 1, 1}, fc[4] = {3, 3, 3, 2};
        const float lam[4] = {l0, l1, l2, l3};
        float best = 3.402823466e+38f;
        v3 cp = mk3(0.f);
        float tmp[4];
        m = 0;
        for (int k = 0; k < 4; k++) {
            if (!(lam[k] < 0.0f || degenerate)) continue;
            unsigned mk;
            v3 q = triangle(fa[k], fb[k], fc[k], tmp, mk);
            float dist = len2(q);
            if (dist < best) {
                for (int j = 0; j < 4; j++) w[j] = tmp[j];
                m = mk; cp = q; best = dist;
            }
        }
        if (m != 0) return cp;
        w[0] = l0; w[1] = l1; w[2] = l2; w[3] = l3;
        m = 15u;
        return mk3(0.f);
    }
    // AddVertex (SimplexSolverAB.cs:300-357): false when the tetrahedron encloses the origin.
    __device__ bool add(const MV& x, v3& closest) {
        int ix[4], used = 0, free_slot = 0;
        for (int i = 0; i < 4; i++) {
            if (mask & (1u << i)) ix[used++] = i;
            else free_slot = i;
        }
        ix[used++] = free_slot;
        v[free_slot] = x;
        if (used == 1) { closest = v[ix[0]].V; mask = 1u << ix[0]; bc[ix[0]] = 1.0f; return true; }
        if (used == 2) { closest = segment(ix[0], ix[1], bc, mask); return true; }
        if (used == 3) { closest = triangle(ix[0], ix[1], ix[2], bc, mask); return true; }
        closest = tetra(bc, mask);
        return mask != 15u;
    }
    // GetClosest (SimplexSolverAB.cs:278-293)
    __device__ void closest_points(v3& pA, v3& pB) const {
        pA = mk3(0.f); pB = mk3(0.f);
        for (int i = 0; i < 4; i++) {
            if (!(mask & (1u << i))) continue;
            pA = pA + bc[i] * v[i].A;
            pB = pB + bc[i] * v[i].B;
        }
    }
};

// NarrowPhase.Sweep with A at the origin (NarrowPhase.cs:1155-1222): B moves along `sweep`;
// a support point in front of the search direction advances the time of impact to the
// plane it spans.  False when B moves away from that plane (no hit); lambda = 0 when the
// shapes already overlap.  At most 34 support evaluations.
__device__ bool sweep_local(const ShapeRef& sa, const ShapeRef& sb, q4 qb, v3 pb, v3 sweep, v3& pA, v3& pB,
                            v3& normal, float& lambda) {
    SimplexAB sx;
    sx.mask = 0;
    MV c;
    mk_center(sa, sb, qb, pb, c);
    v3 pos = pb;
    lambda = 0.0f;
    v3 v = -c.V;
    normal = mk3(0.f);
    int iter = 34;
    float d2 = len2(v);
    while (d2 > 1e-4f * 1e-4f && iter-- != 0) {
        MV x;
        mk_support_t<false>(sa, sb, qb, pos, v, x);
        float vw = -dot(v, x.V);
        if (vw > 0.0f) {
            float vr = dot(v, sweep);
            if (vr >= -1e-12f) { lambda = __int_as_float(0x7f800000); return false; }
            lambda -= vw / vr;
            pos = pb + lambda * sweep;
            normal = v;
        }
        if (!sx.add(x, v)) break;
        v = -v;
        d2 = len2(v);
    }
    sx.closest_points(pA, pB);
    normal = normalize_safe(normal, 1e-16f);
    return true;
}

// Stage 1b, one thread per pair the MPR stage found separated with a speculative body
// (World.Detect.cs:168-196): pairs closing slower than the threshold speed are dropped; the
// rest run the sweep in A's frame (NarrowPhase.cs:1100-1136) and are kept when it hits
// within the step (0 < toi <= dt).  The record goes to the colliding list in world space
// with kind 3, penetration n . (pA - pB) * SpeculativeRelaxationFactor.
__global__ void __launch_bounds__(128) k_sweep(WorldDev w, StepParams sp) {
    const int ns = min(w.ctr->nspec, w.cap_pairs);
    const int cap = w.cap_arb;
    for (int base = blockIdx.x * blockDim.x; base < ns; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        bool hit = false;
        int p = 0;
        v3 pA = mk3(0.f), pB = mk3(0.f), n = mk3(0.f);
        float pen = 0.f;
        if (i < ns) {
            p = w.spec_list[i];
            int2 pr = w.pairs[p];
            int b1 = w.sinfo[pr.x].y, b2 = w.sinfo[pr.y].y;
            ShapeRef sa = load_shape(w, pr.x), sb = load_shape(w, pr.y);
            q4 qa = mkq(w.q[b1]), qb = mkq(w.q[b2]);
            v3 pa = mk3(w.pos[b1]), pb = mk3(w.pos[b2]);
            v3 va = mk3(w.body[b1].v), vb = mk3(w.body[b2].v);
            v3 dv = vb - va;
            q4 q = qmul(qconj(qa), qb);
            v3 prl = rotate_inv(pb - pa, qa);
            v3 swl = rotate_inv(dv, qa);
            float toi;
            if (!(len2(dv) < sp.spec_threshold * sp.spec_threshold) &&
                sweep_local(sa, sb, q, prl, swl, pA, pB, n, toi)) {
                pA = rotate(pA, qa); pA = pA + pa;
                pB = rotate(pB, qa); pB = pB + pa;
                n = rotate(n, qa);
                pB = pB + toi * (va - vb);
                hit = !(toi > sp.dt) && toi != 0.0f;
                pen = dot(n, pA - pB) * sp.spec_relax;
            }
        }
        int c = warp_append(&w.ctr->ncol, hit);
        if (c >= cap) { atomicCAS(&w.ctr->status, 0, JG_ERR_CAPACITY); c = -1; }
        if (c >= 0) {
            w.col_pair[c] = make_int2(p, 3);
            w.col_res[3 * c + 0] = f4(pA, 0.f);
            w.col_res[3 * c + 1] = f4(pB, 0.f);
            w.col_res[3 * c + 2] = f4(n, pen);
        }
    }
}

// Stage 2, one warp per deep pair: EPA from the saved portal (NarrowPhase.cs:39-95); on
// success the colliding record takes the EPA result, otherwise the MPR result stands.
// Next work item of a warp: lane 0 takes it from the cursor, every lane gets it.
__device__ __forceinline__ int next_item(int* cursor, int lane) {
    int e = 0;
    if (lane == 0) e = atomicAdd(cursor, 1);
    return __shfl_sync(0xffffffffu, e, 0);
}

__global__ void __launch_bounds__(NP_WARPS * 32) k_epa(WorldDev w) {
    extern __shared__ __align__(16) unsigned char np_smem_raw[];
    EpaSmem* smem = reinterpret_cast<EpaSmem*>(np_smem_raw);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    EpaSmem& E = smem[wib];
    NpStats st; st.exact = 0;
    int epa_calls = 0, epa_fail = 0;
    const int ne = min(w.ctr->nepa_list, w.cap_arb);
    // pairs handed out one at a time: EPA's cost varies by an order of magnitude between
    // pairs, so a fixed share per warp would leave most warps idle behind a few
    for (int e = next_item(&w.ctr->epa_next, lane); e < ne; e = next_item(&w.ctr->epa_next, lane)) {
        int c = w.epa_list[e];
        int2 pr = w.pairs[w.col_pair[c].x];
        ShapeRef sa = load_shape(w, pr.x), sb = load_shape(w, pr.y);
        int b1 = w.sinfo[pr.x].y, b2 = w.sinfo[pr.y].y;
        q4 qa = mkq(w.q[b1]), qb = mkq(w.q[b2]);
        v3 pa = mk3(w.pos[b1]), pb = mk3(w.pos[b2]);
        MV portal[4];
        for (int k = 0; k < 4; k++) {
            portal[k].V = mk3(w.col_portal[12 * e + 3 * k + 0]);
            portal[k].A = mk3(w.col_portal[12 * e + 3 * k + 1]);
            portal[k].B = mk3(w.col_portal[12 * e + 3 * k + 2]);
        }
        v3 pA = mk3(w.col_res[3 * c + 0]), pB = mk3(w.col_res[3 * c + 1]);
        float4 nr = w.col_res[3 * c + 2];
        v3 n = mk3(nr);
        float pen = nr.w;
        q4 q = qmul(qconj(qa), qb);
        v3 prl = rotate_inv(pb - pa, qa);
        run_epa(E, sa, sb, q, prl, portal, pA, pB, n, pen, st, epa_calls, epa_fail);
        if (lane == 0) {
            w.col_res[3 * c + 0] = f4(pA, 0.f);
            w.col_res[3 * c + 1] = f4(pB, 0.f);
            w.col_res[3 * c + 2] = f4(n, pen);
        }
    }
    if (lane == 0) {
        if (epa_calls) atomicAdd(&w.ctr->nepa, epa_calls);
        if (epa_fail) atomicAdd(&w.ctr->epa_fail, epa_fail);
    }
    int ex = st.exact;
    for (int off = 16; off > 0; off >>= 1) ex += __shfl_xor_sync(FULL, ex, off);
    if (lane == 0 && ex) atomicAdd(&w.ctr->exact, ex);
}

// Contact stream record: shape pair, normal with the point count (low byte) and
// JG_STREAM_SPECULATIVE, and the points.
__device__ __forceinline__ void write_stream(WorldDev& w, int idx, int s1, int s2, v3 n, int cnt, bool spec,
                                             const float4* oA, const float4* oB) {
    if (idx >= w.cap_pairs) { atomicCAS(&w.ctr->status, 0, JG_ERR_CAPACITY); return; }
    w.cs_key[idx] = make_int2(s1, s2);
    w.cs_n[idx] = f4(n, __int_as_float(cnt | (spec ? JG_STREAM_SPECULATIVE : 0)));
    for (int k = 0; k < cnt; k++) { w.cs_pa[4 * idx + k] = oA[k]; w.cs_pb[4 * idx + k] = oB[k]; }
}

// Stage 3, one thread per colliding record: world transform, the first test of the
// triangle-edge filter (TriangleEdgeCollisionFilter.cs:183-240; pairs near a mesh edge
// move to stage 4) and the one-shot manifold; appends the contact stream record.  A
// speculative record (kind 3, already in world space) registers its one point
// (World.Detect.cs:185-196).
__global__ void __launch_bounds__(128) k_manifold(WorldDev w, StepParams sp) {
    const int ncol = min(w.ctr->ncol, w.cap_arb);
    int pts = 0;
    for (int base = blockIdx.x * blockDim.x; base < ncol; base += gridDim.x * blockDim.x) {
        int c = base + threadIdx.x;
        bool emit = false, to_edge = false, spec = false;
        int s1 = 0, s2 = 0, cnt = 0;
        v3 n = mk3(0.f);
        float4 oA[4], oB[4];
        if (c < ncol) {
            int2 cp = w.col_pair[c];
            spec = cp.y == 3;
            int2 pr = w.pairs[cp.x];
            s1 = pr.x; s2 = pr.y;
            ShapeRef sa = load_shape(w, s1), sb = load_shape(w, s2);
            int b1 = w.sinfo[s1].y, b2 = w.sinfo[s2].y;
            q4 qa = mkq(w.q[b1]), qb = mkq(w.q[b2]);
            v3 pa = mk3(w.pos[b1]), pb = mk3(w.pos[b2]);
            v3 pA = mk3(w.col_res[3 * c + 0]), pB = mk3(w.col_res[3 * c + 1]);
            float4 nr = w.col_res[3 * c + 2];
            n = mk3(nr);
            float pen = nr.w;
            if (!spec) {
                pA = rotate(pA, qa); pA = pA + pa;
                pB = rotate(pB, qa); pB = pB + pa;
                n = rotate(n, qa);
            }
            emit = true;
            bool c1 = sa.kind == JG_SHAPE_TRIANGLE, c2 = sb.kind == JG_SHAPE_TRIANGLE;
            if (sp.edge_filter && c1 != c2) {
                int4 i1 = w.binfo[b1], i2 = w.binfo[b2];
                bool tri_dyn = c1 ? i1.x == JG_MOTION_DYNAMIC : i2.x == JG_MOTION_DYNAMIC;
                if (!tri_dyn) {
                    v3 tn, nn;
                    int ev = edge_evaluate(w, c1 ? sa.tri : sb.tri, c1 ? qa : qb, c1 ? pa : pb, c2, c1 ? pA : pB, n, tn, nn);
                    if (ev == DISCARD) emit = false;
                    else if (ev == EDGE) { emit = false; to_edge = true; }
                }
            }
            (void)pen;
            if (emit) {
                if (sp.aux_contacts && !spec) cnt = manifold_thread(sa, sb, qa, qb, pa, pb, pA, pB, n, oA, oB);
                else { cnt = 1; oA[0] = f4(pA, 0.f); oB[0] = f4(pB, 0.f); }
            }
        }
        int idx = warp_append(&w.ctr->nstream, emit);
        if (idx >= 0) { write_stream(w, idx, s1, s2, n, cnt, spec, oA, oB); pts += cnt; }
        int ei = warp_append(&w.ctr->nedge, to_edge);
        if (ei >= 0) w.edge_list[ei] = c;
    }
    for (int off = 16; off > 0; off >>= 1) pts += __shfl_xor_sync(FULL, pts, off);
    if ((threadIdx.x & 31) == 0 && pts) atomicAdd(&w.ctr->points, pts);
}

// Stage 4, one warp per pair near a mesh edge: the rest of the triangle-edge filter
// (rerun of MPR/EPA with threshold zero, normal snapping; TriangleEdgeCollisionFilter.cs:
// 294-420) and the manifold.
__global__ void __launch_bounds__(NP_WARPS * 32) k_edge(WorldDev w, StepParams sp) {
    extern __shared__ __align__(16) unsigned char np_smem_raw[];
    EpaSmem* smem = reinterpret_cast<EpaSmem*>(np_smem_raw);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    EpaSmem& E = smem[wib];
    NpStats st; st.exact = 0;
    int epa_calls = 0, epa_fail = 0, pts = 0;
    const int ne = min(w.ctr->nedge, w.cap_arb);
    for (int e = next_item(&w.ctr->edge_next, lane); e < ne; e = next_item(&w.ctr->edge_next, lane)) {
        int c = w.edge_list[e];
        int2 cp = w.col_pair[c];
        const bool from_sweep = cp.y == 3;
        int2 pr = w.pairs[cp.x];
        int s1 = pr.x, s2 = pr.y;
        ShapeRef sa = load_shape(w, s1), sb = load_shape(w, s2);
        int b1 = w.sinfo[s1].y, b2 = w.sinfo[s2].y;
        q4 qa = mkq(w.q[b1]), qb = mkq(w.q[b2]);
        v3 pa = mk3(w.pos[b1]), pb = mk3(w.pos[b2]);
        v3 pA = mk3(w.col_res[3 * c + 0]), pB = mk3(w.col_res[3 * c + 1]);
        float4 nr = w.col_res[3 * c + 2];
        v3 n = mk3(nr);
        float pen = nr.w;
        if (!from_sweep) {
            pA = rotate(pA, qa); pA = pA + pa;
            pB = rotate(pB, qa); pB = pB + pa;
            n = rotate(n, qa);
        }
        bool c1 = sa.kind == JG_SHAPE_TRIANGLE, c2 = sb.kind == JG_SHAPE_TRIANGLE;
        int tri = c1 ? sa.tri : sb.tri;
        q4 tq = c1 ? qa : qb;
        v3 tp = c1 ? pa : pb;
        v3 tn, nn;
        int ev = edge_evaluate(w, tri, tq, tp, c2, c1 ? pA : pB, n, tn, nn);
        bool spec = pen < 0.0f;
        bool keep = true, done = false;
        if (!spec) {
            bool res = mpr_epa_world(E, sa, sb, qa, qb, pa, pb, pA, pB, n, pen, 0.0f, st, epa_calls, epa_fail);
            if (!res) keep = false;
            else {
                ev = edge_evaluate(w, tri, tq, tp, c2, c1 ? pA : pB, n, tn, nn);
                if (ev == DISCARD) keep = false;
                else if (ev == KEEP) done = true;
            }
        }
        if (!keep) continue;
        if (!done) {
            v3 mid = 0.5f * (pA + pB);
            if (dot(tn, nn) > 0.999f) {
                float f5 = dot(n, nn), f6 = dot(n, tn);
                if (!spec) { pen = 0; pA = pB = mid; }
                n = f5 > f6 ? nn : tn;
            } else {
                v3 cr = cross(nn, tn);
                float crl = len2(cr);
                v3 proj = n - (dot(cr, n) / crl) * cr;
                if (len2(proj) < 0.5f * 0.5f) continue;
                float f1 = dot(cross(proj, nn), cr);
                float f2 = dot(cross(proj, tn), cr);
                bool between = f1 <= 0.0f && f2 >= 0.0f;
                if (!between) {
                    float f3 = dot(n, nn), f4v = dot(n, tn);
                    if (!spec) { pen = 0; pA = pB = mid; }
                    n = f3 > f4v ? nn : tn;
                }
            }
        }
        v3 oA[4], oB[4];
        int cnt;
        if (sp.aux_contacts && !from_sweep) cnt = build_manifold(E, sa, sb, qa, qb, pa, pb, pA, pB, n, oA, oB);
        else { cnt = 1; oA[0] = pA; oB[0] = pB; }
        if (lane == 0) {
            int idx = atomicAdd(&w.ctr->nstream, 1);
            float4 fa[4], fb[4];
            for (int k = 0; k < cnt; k++) { fa[k] = f4(oA[k], 0.f); fb[k] = f4(oB[k], 0.f); }
            write_stream(w, idx, s1, s2, n, cnt, from_sweep, fa, fb);
        }
        pts += cnt;
    }
    if (lane == 0) {
        if (epa_calls) atomicAdd(&w.ctr->nepa, epa_calls);
        if (epa_fail) atomicAdd(&w.ctr->epa_fail, epa_fail);
        if (pts) atomicAdd(&w.ctr->points, pts);
    }
    int ex = st.exact;
    for (int off = 16; off > 0; off >>= 1) ex += __shfl_xor_sync(FULL, ex, off);
    if (lane == 0 && ex) atomicAdd(&w.ctr->exact, ex);
}

// Batched NarrowPhase.MprEpa query (NarrowPhase.cs:902-927), one warp per shape pair, on
// the world's shapes and body poses.  out holds 10 floats per pair (pointA, pointB,
// normal, penetration, world frame) and hit the method's return value; every slot is
// written, so neither buffer needs clearing.
__global__ void __launch_bounds__(NP_WARPS * 32) k_collide_query(WorldDev w, const int2* pairs, int n, float threshold,
                                                                 float* out, int* hit) {
    extern __shared__ __align__(16) unsigned char np_smem_raw[];
    EpaSmem* smem = reinterpret_cast<EpaSmem*>(np_smem_raw);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    EpaSmem& E = smem[wib];
    NpStats st; st.exact = 0;
    int ec = 0, ef = 0;
    for (int i = blockIdx.x * NP_WARPS + wib; i < n; i += gridDim.x * NP_WARPS) {
        int2 pr = pairs[i];
        ShapeRef sa = load_shape(w, pr.x), sb = load_shape(w, pr.y);
        int b1 = w.sinfo[pr.x].y, b2 = w.sinfo[pr.y].y;
        q4 qa = mkq(w.q[b1]), qb = mkq(w.q[b2]);
        v3 pa = mk3(w.pos[b1]), pb = mk3(w.pos[b2]);
        v3 pA = mk3(0.f), pB = mk3(0.f), nn = mk3(0.f);
        float pen = 0.f;
        bool h = mpr_epa_world(E, sa, sb, qa, qb, pa, pb, pA, pB, nn, pen, threshold, st, ec, ef);
        if (lane == 0) {
            float* o = out + 10 * (size_t)i;
            o[0] = pA.x; o[1] = pA.y; o[2] = pA.z;
            o[3] = pB.x; o[4] = pB.y; o[5] = pB.z;
            o[6] = nn.x; o[7] = nn.y; o[8] = nn.z;
            o[9] = pen;
            hit[i] = h ? 1 : 0;
        }
    }
}

// Batched CollisionManifold.BuildManifold (CollisionManifold.cs:393-566) for given witness
// points, one thread per pair, the same function the step's manifold stage runs.  in holds
// 9 floats per pair (pointA, pointB, normal, world frame); out receives 24 floats per pair
// (up to four point pairs A, B) and count the number of pairs.
__global__ void __launch_bounds__(128) k_manifold_query(WorldDev w, const int2* pairs, int n, const float* in, float* out,
                                                        int* count) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int2 pr = pairs[i];
        ShapeRef sa = load_shape(w, pr.x), sb = load_shape(w, pr.y);
        int b1 = w.sinfo[pr.x].y, b2 = w.sinfo[pr.y].y;
        q4 qa = mkq(w.q[b1]), qb = mkq(w.q[b2]);
        v3 pa = mk3(w.pos[b1]), pb = mk3(w.pos[b2]);
        const float* c = in + 9 * (size_t)i;
        float4 oA[4], oB[4];
        int cnt = manifold_thread(sa, sb, qa, qb, pa, pb, mk3(c[0], c[1], c[2]), mk3(c[3], c[4], c[5]), mk3(c[6], c[7], c[8]),
                                  oA, oB);
        float* o = out + 24 * (size_t)i;
        for (int k = 0; k < 4; k++) {
            float4 a = k < cnt ? oA[k] : make_float4(0.f, 0.f, 0.f, 0.f), b = k < cnt ? oB[k] : make_float4(0.f, 0.f, 0.f, 0.f);
            o[6 * k + 0] = a.x; o[6 * k + 1] = a.y; o[6 * k + 2] = a.z;
            o[6 * k + 3] = b.x; o[6 * k + 4] = b.y; o[6 * k + 5] = b.z;
        }
        count[i] = cnt;
    }
}

// Dynamic shared memory of the warp-per-pair kernels: one polytope per warp.
constexpr int kNpSmem = NP_WARPS * (int)sizeof(EpaSmem);

}  // namespace

// Lets the warp-per-pair kernels take their polytopes' shared memory (above the 48 KB
// default) on the current device; called when a world is created.
int jg_narrowphase_init() {
    cudaError_t e = cudaFuncSetAttribute(k_epa, cudaFuncAttributeMaxDynamicSharedMemorySize, kNpSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_edge, cudaFuncAttributeMaxDynamicSharedMemorySize, kNpSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_collide_query, cudaFuncAttributeMaxDynamicSharedMemorySize, kNpSmem);
    return e == cudaSuccess ? 0 : -1;
}

void jg_launch_manifold_query(WorldDev& w, const int2* pairs, int n, const float* in, float* out, int* count,
                              cudaStream_t s, int nsm) {
    if (n <= 0) return;
    int blocks = (n + 127) / 128;
    if (blocks > nsm * 8) blocks = nsm * 8;
    k_manifold_query<<<blocks, 128, 0, s>>>(w, pairs, n, in, out, count);
}

void jg_launch_collide_query(WorldDev& w, const int2* pairs, int n, float threshold, float* out, int* hit,
                             cudaStream_t s, int nsm) {
    if (n <= 0) return;
    int blocks = (n + NP_WARPS - 1) / NP_WARPS;
    if (blocks > nsm * 4) blocks = nsm * 4;
    k_collide_query<<<blocks, NP_WARPS * 32, kNpSmem, s>>>(w, pairs, n, threshold, out, hit);
}

void jg_launch_narrowphase(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm, int tile) {
    (void)tile;
    cudaMemsetAsync(w.pair_kind, 0, sizeof(int) * 64, s);
    k_pair_hist<<<nsm * 4, 256, 0, s>>>(w);
    k_pair_offsets<<<1, 1, 0, s>>>(w);
    k_pair_scatter<<<nsm * 4, 256, 0, s>>>(w);
    k_mpr<<<nsm * 8, 256, 0, s>>>(w);
    k_sweep<<<nsm * 2, 128, 0, s>>>(w, p);
    k_epa<<<nsm * 4, NP_WARPS * 32, kNpSmem, s>>>(w);
    k_manifold<<<nsm * 16, 128, 0, s>>>(w, p);
    k_edge<<<nsm * 4, NP_WARPS * 32, kNpSmem, s>>>(w, p);
}
