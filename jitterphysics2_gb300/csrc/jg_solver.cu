// Substepped sequential-impulse solve in one persistent, cooperatively launched kernel:
//   for each substep (World.Step.cs:234-253):
//     IntegrateForces (World.Step.cs:1060-1072)                       bodies, grid-stride
//     Prepare, colour by colour (Contact.cs:802-924, BallSocket.cs:140-183, HingeAngle.cs:133-220)
//     iterations x colours: Iterate (Contact.cs:931-1018, BallSocket.cs:223-252, HingeAngle.cs:313-364)
//     IntegrateVelocities (World.Step.cs:1106-1133)                   bodies, grid-stride
//     relaxation x colours: Iterate without bias (World.Step.cs:1135-1153)
// Rows of one colour share no dynamic body, so a colour is solved in parallel with no
// atomics.  Two kernels: k_solve runs global colours with a grid barrier between them;
// k_solve_tasks runs the partitioned schedule (spatial tasks with their bodies in shared
// memory and a block barrier between local colours, the three grid phases handed off task
// by task, and the remainder in global colours).  Arbiters are stored colour-sorted, so each
// colour is a contiguous range of coalesced float4 rows.  The per-step body update
// (RigidBody.Update, RigidBody.cs:716-764) is a separate kernel.
#include "jg_sync.cuh"
#include <algorithm>

namespace {

constexpr float MaximumBias = 100.0f, BiasFactor = 0.2f, AllowedPenetration = 0.01f, BreakThreshold = 0.02f;

struct LBody {
    v3 v, w;
    v3 im;     // inverse mass vector
    sym6 I;    // world inverse inertia
    int flags;
};
__device__ __forceinline__ LBody load_body(const SBody* B, int i) {
    SBody s = B[i];
    LBody b;
    b.v = mk3(s.v); b.w = mk3(s.w);
    b.im = mk3(s.v.w, s.w.w, s.i1.z);
    b.I.m11 = s.i0.x; b.I.m12 = s.i0.y; b.I.m13 = s.i0.z; b.I.m22 = s.i0.w; b.I.m23 = s.i1.x; b.I.m33 = s.i1.y;
    b.flags = __float_as_int(s.i1.w);
    return b;
}
__device__ __forceinline__ void store_vel(SBody* B, int i, const LBody& b) {
    B[i].v = f4(b.v, b.im.x);
    B[i].w = f4(b.w, b.im.y);
}

// Contact.PrepareForIteration (Contact.cs:802-924)
__device__ __forceinline__ void prepare_contact(const ArbStore& A, int i, int mode, float spec_relax, LBody& b1, LBody& b2,
                                                v3 pos1, q4 q1, v3 pos2, q4 q2, const StepParams& sp) {
    float4 cn = A.cn[i], ct1 = A.ct1[i], ct2 = A.ct2[i], cr1 = A.cr1[i], cr2 = A.cr2[i], ca = A.cacc[i];
    float4 cp1 = A.cp1[i], cp2 = A.cp2[i];
    int flag = __float_as_int(ct2.w);
    float an = ca.x, at1 = ca.y, at2 = ca.z;
    bool skip = (flag & 4) != 0;
    flag &= ~4;
    if (skip) { an = 0; at1 = 0; at2 = 0; }
    v3 n = mk3(cn), t1 = mk3(ct1), t2 = mk3(ct2), rel1 = mk3(cr1), rel2 = mk3(cr2);
    float bias = cn.w;
    v3 cur1 = rotate(mk3(cp1), q1), cur2 = rotate(mk3(cp2), q2);
    v3 imv = mk3(0.f);
    if (mode & 1) imv = b1.im;
    if (mode & 4) imv = imv + b2.im;
    float im = imv.x;
    if ((flag & 2) == 0) bias = 0;
    v3 p1 = cur1 + pos1, p2 = cur2 + pos2;
    v3 dist = p1 - p2;
    float pen = dot(dist, n);
    if (pen < -BreakThreshold) bias = pen * sp.inv_dt * spec_relax;
    flag &= ~2;
    float kt1 = im, kt2 = im, kn = im;
    if ((b1.flags | b2.flags) & SB_LINLOCK) {
        kn = dot(cmul(imv, n), n);
        kt1 = dot(cmul(imv, t1), t1);
        kt2 = dot(cmul(imv, t2), t2);
    }
    v3 ancN = mk3(0.f), ancT1 = mk3(0.f), ancT2 = mk3(0.f);
    v3 imp = an * n;
    imp = imp + at1 * t1;
    imp = imp + at2 * t2;
    if (mode & 1) b1.v = b1.v - cmul(imp, b1.im);
    if (mode & 2) {
        v3 aN = sym_mul(b1.I, cross(rel1, n)), aT1 = sym_mul(b1.I, cross(rel1, t1)), aT2 = sym_mul(b1.I, cross(rel1, t2));
        ancN = ancN + cross(aN, rel1);
        ancT1 = ancT1 + cross(aT1, rel1);
        ancT2 = ancT2 + cross(aT2, rel1);
        v3 ai = an * aN;
        ai = ai + at1 * aT1;
        ai = ai + at2 * aT2;
        b1.w = b1.w - ai;
    }
    if (mode & 4) b2.v = b2.v + cmul(imp, b2.im);
    if (mode & 8) {
        v3 aN = sym_mul(b2.I, cross(rel2, n)), aT1 = sym_mul(b2.I, cross(rel2, t1)), aT2 = sym_mul(b2.I, cross(rel2, t2));
        ancN = ancN + cross(aN, rel2);
        ancT1 = ancT1 + cross(aT1, rel2);
        ancT2 = ancT2 + cross(aT2, rel2);
        v3 ai = an * aN;
        ai = ai + at1 * aT1;
        ai = ai + at2 * aT2;
        b2.w = b2.w + ai;
    }
    kn += dot(n, ancN);
    kt1 += dot(t1, ancT1);
    kt2 += dot(t2, ancT2);
    float mT1 = kt1 > 0 ? 1.0f / kt1 : 0.f;
    float mT2 = kt2 > 0 ? 1.0f / kt2 : 0.f;
    float mN = kn > 0 ? 1.0f / kn : 0.f;
    float pb = BiasFactor * sp.inv_dt * fmaxf(0.0f, pen - AllowedPenetration);
    pb = fminf(pb, MaximumBias);
    A.cn[i] = f4(n, bias);
    A.ct1[i] = f4(t1, pb);
    A.ct2[i] = f4(t2, __int_as_float(flag));
    A.cr1[i] = f4(rel1, mN);
    A.cr2[i] = f4(rel2, mT1);
    A.cacc[i] = make_float4(ca.x, ca.y, ca.z, mT2);
}

// Contact.Iterate (Contact.cs:931-1018) on one contact row held in registers; returns the
// new accumulated impulses (with the tangent-2 mass) and, with kResid, adds the squared
// impulse change and squared impulse to d2, l2 for the residual metric.
template <bool kResid = true>
__device__ __forceinline__ float4 iterate_row(float4 cn, float4 ct1, float4 ct2, float4 cr1, float4 cr2, float4 ca, int mode,
                                              float friction, LBody& b1, LBody& b2, bool apply_bias, float& d2, float& l2) {
    float mN = cr1.w, mT1 = cr2.w, mT2 = ca.w;
    float aN = ca.x, aT1 = ca.y, aT2 = ca.z;
    v3 n = mk3(cn), t1 = mk3(ct1), t2 = mk3(ct2), rel1 = mk3(cr1), rel2 = mk3(cr2);
    v3 dv = b2.v - b1.v;
    if (mode & (2 | 8)) {
        dv = b2.v + cross(b2.w, rel2);
        dv = dv - (b1.v + cross(b1.w, rel1));
    }
    float bias = cn.w;
    float penalty = ct1.w;
    if (apply_bias && penalty > 0) bias = fmaxf(penalty, cn.w);
    float vn = dot(n, dv), vt1 = dot(t1, dv), vt2 = dot(t2, dv);
    float ni = -vn + bias;
    ni *= mN;
    float oldN = aN;
    aN = fmaxf(oldN + ni, 0.0f);
    ni = aN - oldN;
    float maxT = friction * oldN;
    float ti1 = mT1 * -vt1, ti2 = mT2 * -vt2;
    float oldT1 = aT1;
    aT1 = oldT1 + ti1;
    aT1 = fminf(fmaxf(aT1, -maxT), maxT);
    ti1 = aT1 - oldT1;
    float oldT2 = aT2;
    aT2 = oldT2 + ti2;
    aT2 = fminf(fmaxf(aT2, -maxT), maxT);
    ti2 = aT2 - oldT2;
    if (kResid) {
        d2 += ni * ni + ti1 * ti1 + ti2 * ti2;
        l2 += aN * aN + aT1 * aT1 + aT2 * aT2;
    }
    v3 imp = ni * n;
    imp = imp + ti1 * t1;
    imp = imp + ti2 * t2;
    if (mode & 1) b1.v = b1.v - cmul(imp, b1.im);
    if (mode & 2) b1.w = b1.w - sym_mul(b1.I, cross(rel1, imp));
    if (mode & 4) b2.v = b2.v + cmul(imp, b2.im);
    if (mode & 8) b2.w = b2.w + sym_mul(b2.I, cross(rel2, imp));
    return make_float4(aN, aT1, aT2, mT2);
}

__device__ __forceinline__ void iterate_contact(const ArbStore& A, int i, int mode, float friction, LBody& b1, LBody& b2,
                                                bool apply_bias, float& d2, float& l2) {
    A.cacc[i] = iterate_row(A.cn[i], A.ct1[i], A.ct2[i], A.cr1[i], A.cr2[i], A.cacc[i], mode, friction, b1, b2, apply_bias,
                            d2, l2);
}

#include "jg_joints.cuh"

__device__ __forceinline__ void solve_arbiter(const WorldDev& w, const ArbStore& A, int a, int phase, const StepParams& sp,
                                              bool bias, float& d2, float& l2) {
    int4 info = A.info[a];
    int usage = info.x & 15;
    if (!usage || (info.y & JG_ARB_ASLEEP)) return;
    int mode = info.y & 15;
    int2 bb = A.body[a];
    LBody b1 = load_body(w.body, bb.x), b2 = load_body(w.body, bb.y);
    const int cap = w.cap_arb;
    if (phase == 0) {
        float spec = A.mat[a].z;
        v3 pos1 = mk3(w.pos[bb.x]), pos2 = mk3(w.pos[bb.y]);
        q4 q1 = mkq(w.q[bb.x]), q2 = mkq(w.q[bb.y]);
        for (int k = 0; k < 4; k++)
            if (usage & (1 << k)) prepare_contact(A, k * cap + a, mode, spec, b1, b2, pos1, q1, pos2, q2, sp);
    } else {
        float fr = A.mat[a].x;
        for (int k = 0; k < 4; k++)
            if (usage & (1 << k)) iterate_contact(A, k * cap + a, mode, fr, b1, b2, bias, d2, l2);
    }
    if (mode & 3) store_vel(w.body, bb.x, b1);
    if (mode & 12) store_vel(w.body, bb.y, b2);
}

__device__ __forceinline__ void block_reduce_add(float a, float b, float* out) {
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0 && (a != 0.f || b != 0.f)) {
        atomicAdd(out, a);
        atomicAdd(out + 1, b);
    }
}

// IntegrateForces (World.Step.cs:1060-1072): v += dv, w += dw for dynamic bodies.
__device__ __forceinline__ void integrate_forces_all(const WorldDev& w, const StepParams& sp, int tid, int nth) {
    for (int i = tid; i < w.nb; i += nth) {
        const int4 bi = w.binfo[i];
        if (bi.x != JG_MOTION_DYNAMIC || (sp.allow_deact && !(bi.y & JG_BODY_ACTIVE))) continue;
        SBody b = w.body[i];
        float4 dv = w.dv[i], dw = w.dw[i];
        b.w = make_float4(b.w.x + dw.x, b.w.y + dw.y, b.w.z + dw.z, b.w.w);
        b.v = make_float4(b.v.x + dv.x, b.v.y + dv.y, b.v.z + dv.z, b.v.w);
        w.body[i].v = b.v;
        w.body[i].w = b.w;
    }
}

// float.IsNormal
__device__ __forceinline__ bool is_normal_f(float x) { return isfinite(x) && fabsf(x) >= 1.17549435e-38f; }

// JSymmetricMatrix.TryInverseUnscaled / Inverse (JSymmetricMatrix.cs:104-178): zero when
// neither the matrix nor its scaled copy inverts
__device__ bool sym_try_inverse_unscaled(const sym6& m, sym6& o) {
    float det = m.m11 * (m.m22 * m.m33 - m.m23 * m.m23) + m.m12 * (m.m23 * m.m13 - m.m12 * m.m33) +
                m.m13 * (m.m12 * m.m23 - m.m22 * m.m13);
    float idet = 1.0f / det;
    if (!is_normal_f(idet)) return false;
    o.m11 = (m.m22 * m.m33 - m.m23 * m.m23) * idet;
    o.m12 = (m.m13 * m.m23 - m.m12 * m.m33) * idet;
    o.m13 = (m.m12 * m.m23 - m.m22 * m.m13) * idet;
    o.m22 = (m.m11 * m.m33 - m.m13 * m.m13) * idet;
    o.m23 = (m.m13 * m.m12 - m.m23 * m.m11) * idet;
    o.m33 = (m.m11 * m.m22 - m.m12 * m.m12) * idet;
    return isfinite(o.m11) && isfinite(o.m12) && isfinite(o.m13) && isfinite(o.m22) && isfinite(o.m23) && isfinite(o.m33);
}
__device__ sym6 sym_inverse_ref(const sym6& m) {
    sym6 o;
    if (sym_try_inverse_unscaled(m, o)) return o;
    float s = fmaxf(fabsf(m.m11), fmaxf(fabsf(m.m12), fabsf(m.m13)));
    s = fmaxf(s, fmaxf(fabsf(m.m22), fmaxf(fabsf(m.m23), fabsf(m.m33))));
    if (s > 0 && isfinite(s)) {
        sym6 n{m.m11 / s, m.m12 / s, m.m13 / s, m.m22 / s, m.m23 / s, m.m33 / s};
        if (sym_try_inverse_unscaled(n, o)) {
            o = sym6{o.m11 / s, o.m12 / s, o.m13 / s, o.m22 / s, o.m23 / s, o.m33 / s};
            if (isfinite(o.m11) && isfinite(o.m12) && isfinite(o.m13) && isfinite(o.m22) && isfinite(o.m23) && isfinite(o.m33))
                return o;
        }
    }
    return sym6{0, 0, 0, 0, 0, 0};
}

// JMatrix.Determinant / TryInverseUnscaled / Inverse (JMatrix.cs:391-478)
__device__ bool mat_try_inverse_unscaled(const float M[3][3], float o[3][3]) {
    float det = M[0][0] * M[1][1] * M[2][2] + M[0][1] * M[1][2] * M[2][0] + M[0][2] * M[1][0] * M[2][1] -
                M[2][0] * M[1][1] * M[0][2] - M[2][1] * M[1][2] * M[0][0] - M[2][2] * M[1][0] * M[0][1];
    float idet = 1.0f / det;
    if (!is_normal_f(idet)) return false;
    float n[3][3];
    n[0][0] = M[1][1] * M[2][2] - M[1][2] * M[2][1];
    n[0][1] = M[0][2] * M[2][1] - M[0][1] * M[2][2];
    n[0][2] = M[0][1] * M[1][2] - M[1][1] * M[0][2];
    n[1][0] = M[1][2] * M[2][0] - M[2][2] * M[1][0];
    n[1][1] = M[0][0] * M[2][2] - M[2][0] * M[0][2];
    n[1][2] = M[0][2] * M[1][0] - M[1][2] * M[0][0];
    n[2][0] = M[1][0] * M[2][1] - M[2][0] * M[1][1];
    n[2][1] = M[0][1] * M[2][0] - M[2][1] * M[0][0];
    n[2][2] = M[0][0] * M[1][1] - M[1][0] * M[0][1];
    bool fin = true;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) { o[r][c] = n[r][c] * idet; fin = fin && isfinite(o[r][c]); }
    return fin;
}
__device__ bool mat_inverse(const float M[3][3], float o[3][3]) {
    if (mat_try_inverse_unscaled(M, o)) return true;
    float s = fmaxf(fabsf(M[0][0]), fmaxf(fabsf(M[0][1]), fabsf(M[0][2])));
    s = fmaxf(s, fmaxf(fabsf(M[1][0]), fmaxf(fabsf(M[1][1]), fabsf(M[1][2]))));
    s = fmaxf(s, fmaxf(fabsf(M[2][0]), fmaxf(fabsf(M[2][1]), fabsf(M[2][2]))));
    if (!(s > 0 && isfinite(s))) return false;
    float nm[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) nm[r][c] = M[r][c] / s;
    if (!mat_try_inverse_unscaled(nm, o)) return false;
    bool fin = true;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) { o[r][c] = o[r][c] / s; fin = fin && isfinite(o[r][c]); }
    return fin;
}

// World.SolveGyroscopic (World.Step.cs:1075-1104): one implicit Newton step on the
// gyroscopic term with the world inertia held fixed
__device__ __noinline__ v3 solve_gyroscopic(const sym6& I, v3 av, float dt) {
    v3 Iw = sym_mul(I, av);
    v3 f = dt * cross(av, Iw);
    const float M[3][3] = {{I.m11, I.m12, I.m13}, {I.m12, I.m22, I.m23}, {I.m13, I.m23, I.m33}};
    const float W[3][3] = {{0, -av.z, av.y}, {av.z, 0, -av.x}, {-av.y, av.x, 0}};
    const float L[3][3] = {{0, -Iw.z, Iw.y}, {Iw.z, 0, -Iw.x}, {-Iw.y, Iw.x, 0}};
    float J[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) J[r][c] = M[r][c] + dt * ((W[r][0] * M[0][c] + W[r][1] * M[1][c] + W[r][2] * M[2][c]) - L[r][c]);
    float inv[3][3];
    if (!mat_inverse(J, inv)) return av;
    v3 d = mk3(inv[0][0] * f.x + inv[0][1] * f.y + inv[0][2] * f.z, inv[1][0] * f.x + inv[1][1] * f.y + inv[1][2] * f.z,
               inv[2][0] * f.x + inv[2][1] * f.y + inv[2][2] * f.z);
    return av - d;
}

// IntegrateVelocities (World.Step.cs:1106-1133) with SolveGyroscopic (World.Step.cs:1075-1104).
__device__ __forceinline__ void integrate_velocities_all(const WorldDev& w, const StepParams& sp, int tid, int nth) {
    for (int i = tid; i < w.nb; i += nth) {
        int4 bi = w.binfo[i];
        if (bi.x == JG_MOTION_STATIC || (sp.allow_deact && !(bi.y & JG_BODY_ACTIVE))) continue;
        SBody b = w.body[i];
        v3 lv = mk3(b.v), av = mk3(b.w);
        float4 p = w.pos[i];
        w.pos[i] = make_float4(p.x + lv.x * sp.sub_dt, p.y + lv.y * sp.sub_dt, p.z + lv.z * sp.sub_dt, p.w);
        q4 rq = rotation_quaternion(av, sp.sub_dt);
        q4 q = qnormalize(qmul(rq, mkq(w.q[i])));
        w.q[i] = f4(q);
        if ((bi.y & JG_BODY_GYROSCOPIC) && ((bi.y >> 4) & 63) == 0) {
            // JSymmetricMatrix.Inverse of the world inverse inertia, then SolveGyroscopic
            sym6 Ii;
            Ii.m11 = b.i0.x; Ii.m12 = b.i0.y; Ii.m13 = b.i0.z; Ii.m22 = b.i0.w; Ii.m23 = b.i1.x; Ii.m33 = b.i1.y;
            w.body[i].w = f4(solve_gyroscopic(sym_inverse_ref(Ii), av, sp.sub_dt), b.w.w);
        }
    }
}

// Global-colour passes (all constraints when the solve is not partitioned, else the
// remainder): one grid barrier per non-empty colour.
__device__ __forceinline__ bool remainder_pass(const WorldDev& w, const ArbStore& A, const StepParams& sp, int phase,
                                               bool bias, bool joints, int tid, int nth, float& d2, float& l2) {
    const int ncol = w.ctr->ncolors;
    int* status = &w.ctr->status;
    for (int c = 0; c < ncol; c++) {
        int beg = w.color_start[c], end = w.color_start[c + 1];
        int jb = joints ? w.jcolor_start[c] : 0, je = joints ? w.jcolor_start[c + 1] : 0;
        if (beg == end && jb == je) continue;
        for (int a = beg + tid; a < end; a += nth) solve_arbiter(w, A, a, phase, sp, bias, d2, l2);
        for (int j = jb + tid; j < je; j += nth) {
            const int jj = w.jorder[j];
            if (sp.allow_deact) {  // a constraint is solved while one of its bodies is awake and non-static
                const int4 h = w.joints[jj].hdr, i1 = w.binfo[h.y], i2 = w.binfo[h.z];
                if (!((i1.x != JG_MOTION_STATIC && (i1.y & JG_BODY_ACTIVE)) || (i2.x != JG_MOTION_STATIC && (i2.y & JG_BODY_ACTIVE))))
                    continue;
            }
            if (phase == 0) joint_prepare(w, jj, sp);
            else joint_iterate(w, jj, sp);
        }
        if (!grid_sync(w.bar_count, w.bar_gen, status)) return false;
    }
    return true;
}

// Training targets of the learned warm start: the accumulated impulses of this step's
// new contacts once the first substep's iterations have converged them (the impulse a
// warm start of that substep should have supplied).
__device__ __forceinline__ void record_targets(const WorldDev& w, const ArbStore& A, int tid, int nth) {
    const int n = min(*w.rec_count, w.rec_cap), cap = w.cap_arb;
    for (int e = tid; e < n; e += nth) {
        int2 ak = w.rec_fidx[e];
        int d = w.rec_dst[ak.x];
        float4 c = d >= 0 ? A.cacc[ak.y * cap + d] : make_float4(0.f, 0.f, 0.f, 0.f);
        w.rec_tgt[3 * e] = c.x; w.rec_tgt[3 * e + 1] = c.y; w.rec_tgt[3 * e + 2] = c.z;
    }
}

__global__ void k_solve(WorldDev w, StepParams sp) {
    const ArbStore& A = w.arb[w.cur];
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    int* status = &w.ctr->status;
    for (int s = 0; s < sp.substeps; s++) {
        if (!sp.stabilize) integrate_forces_all(w, sp, tid, nth);
        if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
        for (int it = 0; it < 1 + sp.iterations; it++) {
            float d2 = 0.f, l2 = 0.f;
            if (!remainder_pass(w, A, sp, it == 0 ? 0 : 1, true, true, tid, nth, d2, l2)) return;
            if (sp.record_residual && s == 0 && it > 0 && it <= JG_RESID_MAX) block_reduce_add(d2, l2, w.resid + 2 * (it - 1));
        }
        if (w.rec_on && s == 0) record_targets(w, A, tid, nth);
        if (!sp.stabilize) integrate_velocities_all(w, sp, tid, nth);
        if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
        for (int it = 0; it < sp.relax; it++) {
            float d2 = 0.f, l2 = 0.f;
            if (!remainder_pass(w, A, sp, 1, false, false, tid, nth, d2, l2)) return;
        }
    }
}

// ---- partitioned solve ---------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" :: "r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
// the oldest of the JG_TASK_RING groups in flight has landed
__device__ __forceinline__ void cp_async_wait_ring() { asm volatile("cp.async.wait_group %0;" :: "n"(JG_TASK_RING - 1) : "memory"); }
// everything but the JG_TASK_RING most recent groups (the ring prologue) has landed
__device__ __forceinline__ void cp_async_wait_bodies() { asm volatile("cp.async.wait_group %0;" :: "n"(JG_TASK_RING) : "memory"); }

// Staged arbiter (JG_TASK_STAGE_F4 float4): the header (body slots, usage | mode << 4 |
// non-dynamic << 8, friction), the non-dynamic body's v and w (copied only when there is
// one), then 5 rows per contact slot (cn, ct1, cr1, cr2, cacc; tangent 2 is cross(t1, n),
// as the contact was created with, recomputed by the consumer).  Only the contact
// slots in the usage mask are copied; the others keep stale data that the staged mask
// tells the consumer to skip.  `hz` is the header's third word.
__device__ __forceinline__ void stage_arbiter(float4* dst, const ArbStore& A, int d, int cap, int hz) {
    cp_async16(dst + 0, &A.lslot[d]);
    if (hz & 256) {
        cp_async16(dst + 1, &A.sv[d]);
        cp_async16(dst + 2, &A.sv[cap + d]);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (!(hz & (1 << k))) continue;
        int i = k * cap + d;
        float4* q = dst + 3 + 5 * k;
        cp_async16(q + 0, &A.cn[i]); cp_async16(q + 1, &A.ct1[i]);
        cp_async16(q + 2, &A.cr1[i]); cp_async16(q + 3, &A.cr2[i]); cp_async16(q + 4, &A.cacc[i]);
    }
}

// Staged task bodies in shared memory as four arrays of `stride` float4 (v, w, i0, i1 of
// SBody): random slots spread over all banks, where 64-byte records would meet in two.
__device__ __forceinline__ LBody sbody_load(const float4* sb, int slot, int stride) {
    float4 v = sb[slot], wv = sb[stride + slot], i0 = sb[2 * stride + slot], i1 = sb[3 * stride + slot];
    LBody b;
    b.v = mk3(v); b.w = mk3(wv);
    b.im = mk3(v.w, wv.w, i1.z);
    b.I.m11 = i0.x; b.I.m12 = i0.y; b.I.m13 = i0.z; b.I.m22 = i0.w; b.I.m23 = i1.x; b.I.m33 = i1.y;
    b.flags = __float_as_int(i1.w);
    return b;
}
__device__ __forceinline__ void sbody_store(float4* sb, int slot, int stride, const LBody& b) {
    sb[slot] = f4(b.v, b.im.x);
    sb[stride + slot] = f4(b.w, b.im.y);
}
// A non-dynamic body: velocities only (zero inverse mass and inertia, as its SBody holds).
__device__ __forceinline__ LBody fixed_body(float4 v, float4 wv) {
    LBody b;
    b.v = mk3(v); b.w = mk3(wv);
    b.im = mk3(v.w, wv.w, 0.f);
    b.I.m11 = b.I.m12 = b.I.m13 = b.I.m22 = b.I.m23 = b.I.m33 = 0.f;
    b.flags = 0;
    return b;
}

enum { PASS_PREPARE = 0, PASS_ITERATE = 1, PASS_RELAX = 2 };

// Order inside a task.  sver[slot] (shared memory) counts the task arbiters on that body
// finished in the current pass.  A task arbiter carries, per dynamic body, the body's slot
// and its rank among the body's arbiters in colour order (slot | rank << 16, -1 for a
// non-dynamic body); it runs once each body's count equals its rank, then raises it.  So
// every body sees its arbiters in colour order, the order a block barrier between colours
// gives, and the results are the same bits, but an arbiter waits only for the earlier
// arbiters on its own two bodies.
__device__ __forceinline__ int slot_of(int packed) { return packed & 0xffff; }
__device__ __forceinline__ int rank_of(int packed) { return packed >> 16; }
__device__ __forceinline__ bool deps_ready(const volatile int* sver, int p1, int p2) {
    return (p1 < 0 || sver[slot_of(p1)] == rank_of(p1)) && (p2 < 0 || sver[slot_of(p2)] == rank_of(p2));
}
__device__ __forceinline__ void deps_release(volatile int* sver, int p1, int p2) {
    __threadfence_block();  // the bodies' new velocities before the counts
    if (p1 >= 0) sver[slot_of(p1)] = rank_of(p1) + 1;
    if (p2 >= 0) sver[slot_of(p2)] = rank_of(p2) + 1;
}
// A warp that could run none of its lanes' arbiters backs off; after about 2^20 such
// rounds (far beyond any legitimate wait) the task is abandoned with JG_ERR_TIMEOUT.
__device__ __forceinline__ bool backoff(unsigned& idle, volatile int* abort_flag, int* status) {
    if (*abort_flag) return false;
    if (++idle > (1u << 20)) {
        *abort_flag = 1;
        atomicCAS(status, 0, JG_ERR_TIMEOUT);
        return false;
    }
    __nanosleep(idle < 8 ? 16 : 64);
    return true;
}

// Iterate / relax pass of one task (its bodies already staged or in flight).  Returns
// false when the task was abandoned.
template <bool kResid>
__device__ __forceinline__ bool iterate_task(const WorldDev& w, const ArbStore& A, int4 T, bool bias, float4* sbody,
                                             int sst, float4* ring, volatile int* sver, volatile int* abort_flag,
                                             int* status, float& d2, float& l2) {
    const int cap = w.cap_arb, bs = blockDim.x, tid = threadIdx.x;
    // Thread tid owns the task's arbiters tid, tid + bs, tid + 2 bs, ... (colour order)
    // and runs them in that order.  Each thread keeps its next JG_TASK_RING arbiters in
    // flight (one cp.async group per arbiter, empty groups past the end keep the count
    // uniform).  Every wait is on an arbiter of a smaller index, whose owner runs its
    // arbiters in order too, so the smallest unfinished arbiter can always run.
    const int n = T.y;
    for (int m = 0; m < JG_TASK_RING; m++) {
        int j = m * bs + tid;
        if (j < n) stage_arbiter(ring + ((size_t)m * bs + tid) * JG_TASK_STAGE_F4, A, T.x + j, cap, A.lslot[T.x + j].z);
        cp_async_commit();
    }
    cp_async_wait_bodies();  // this thread's body copies have landed
    __syncthreads();         // ... and everyone's, with the zeroed counts
    int m = 0;               // next owned arbiter: j = m * bs + tid
    unsigned idle = 0;
    for (;;) {
        const int j = m * bs + tid;
        const bool active = j < n;
        if (!__any_sync(0xffffffffu, active)) break;
        float4* r = ring + ((size_t)(m % JG_TASK_RING) * bs + tid) * JG_TASK_STAGE_F4;
        bool go = false;
        float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (active) {
            cp_async_wait_ring();
            r0 = r[0];
            go = deps_ready(sver, __float_as_int(r0.x), __float_as_int(r0.y));
        }
        if (go) {
            __threadfence_block();  // the counts before the bodies they guard
            const int d = T.x + j;
            // header word of the arbiter this slot is refilled with, loaded now and used
            // after the compute below, so its latency stays off the critical path
            const int jn = j + JG_TASK_RING * bs;
            const int un = jn < n ? __ldg(&A.lslot[T.x + jn].z) : 0;
            const int p1 = __float_as_int(r0.x), p2 = __float_as_int(r0.y), hz = __float_as_int(r0.z);
            const int l1 = p1 >= 0 ? slot_of(p1) : -1, l2s = p2 >= 0 ? slot_of(p2) : -1;
            const int usage = (hz & JG_TASK_ASLEEP) ? 0 : hz & 15, mode = (hz >> 4) & 15;
            const float fr = r0.w;
            LBody b1 = l1 >= 0 ? sbody_load(sbody, l1, sst) : fixed_body(r[1], r[2]);
            LBody b2 = l2s >= 0 ? sbody_load(sbody, l2s, sst) : fixed_body(r[1], r[2]);
            // over the set usage bits only: a warp runs as many rows as its fullest arbiter
            // has contacts, not one per slot position any of its lanes uses
            for (unsigned um = (unsigned)usage; um; um &= um - 1) {
                const int k = __ffs(um) - 1;
                const float4* q = r + 3 + 5 * k;
                const float4 cn = q[0], ct1 = q[1];
                const float4 ct2 = f4(cross(mk3(ct1), mk3(cn)), 0.f);  // bit-identical to the stored tangent 2
                A.cacc[k * cap + d] = iterate_row<kResid>(cn, ct1, ct2, q[2], q[3], q[4], mode, fr, b1, b2, bias, d2, l2);
            }
            if ((mode & 3) && l1 >= 0) sbody_store(sbody, l1, sst, b1);
            if ((mode & 12) && l2s >= 0) sbody_store(sbody, l2s, sst, b2);
            deps_release(sver, p1, p2);
            // refill the slot just consumed (its values are in registers by now)
            if (jn < n) stage_arbiter(r, A, T.x + jn, cap, un);
            cp_async_commit();
            m++;
        }
        if (__any_sync(0xffffffffu, go)) idle = 0;
        else if (!backoff(idle, abort_flag, status)) return false;
    }
    return true;
}

// Prepare pass of one task (bodies, positions and orientations staged).
__device__ __forceinline__ bool prepare_task(const WorldDev& w, const ArbStore& A, const StepParams& sp, int4 T,
                                             float4* sbody, int sst, const float4* spos, const float4* sq, bool staged,
                                             volatile int* sver, volatile int* abort_flag, int* status) {
    const int cap = w.cap_arb, bs = blockDim.x, tid = threadIdx.x;
    int m = 0;
    unsigned idle = 0;
    int4 ls = make_int4(-1, -1, 0, 0);
    int loaded = -1;
    for (;;) {
        const int j = m * bs + tid;
        const bool active = j < T.y;
        if (!__any_sync(0xffffffffu, active)) break;
        const int d = T.x + j;
        bool go = false;
        if (active) {
            if (loaded != m) { ls = A.lslot[d]; loaded = m; }
            go = deps_ready(sver, ls.x, ls.y);
        }
        if (go) {
            __threadfence_block();
            int4 info = A.info[d];
            int usage = (info.y & JG_ARB_ASLEEP) ? 0 : info.x & 15, mode = info.y & 15;
            int2 bb = A.body[d];
            const int l1 = ls.x >= 0 ? slot_of(ls.x) : -1, l2 = ls.y >= 0 ? slot_of(ls.y) : -1;
            LBody b1 = l1 >= 0 ? sbody_load(sbody, l1, sst) : fixed_body(A.sv[d], A.sv[cap + d]);
            LBody b2 = l2 >= 0 ? sbody_load(sbody, l2, sst) : fixed_body(A.sv[d], A.sv[cap + d]);
            float spec = A.mat[d].z;
            const bool s1 = staged && l1 >= 0, s2 = staged && l2 >= 0;
            v3 pos1 = mk3(s1 ? spos[l1] : w.pos[bb.x]), pos2 = mk3(s2 ? spos[l2] : w.pos[bb.y]);
            q4 q1 = mkq(s1 ? sq[l1] : w.q[bb.x]), q2 = mkq(s2 ? sq[l2] : w.q[bb.y]);
            for (unsigned um = (unsigned)usage; um; um &= um - 1) {
                const int k = __ffs(um) - 1;
                prepare_contact(A, k * cap + d, mode, spec, b1, b2, pos1, q1, pos2, q2, sp);
            }
            if ((mode & 3) && l1 >= 0) sbody_store(sbody, l1, sst, b1);
            if ((mode & 12) && l2 >= 0) sbody_store(sbody, l2, sst, b2);
            deps_release(sver, ls.x, ls.y);
            m++;
        }
        if (__any_sync(0xffffffffu, go)) idle = 0;
        else if (!backoff(idle, abort_flag, status)) return false;
    }
    return true;
}

// One task in one pass: bodies staged into shared memory, arbiters in per-body colour
// order, bodies written back.  Iterations stage each thread's next arbiter's rows with
// cp.async while the current one computes.  Returns false when the task was abandoned
// (JG_ERR_TIMEOUT recorded).
__device__ __forceinline__ bool run_task(const WorldDev& w, const ArbStore& A, const StepParams& sp, int t, int kind,
                                         float4* sbody, float4* ring, volatile int* sver, volatile int* abort_flag,
                                         float& d2, float& l2) {
    const int4 T = w.sc_task[t];
    const int bs = blockDim.x, tid = threadIdx.x;
    const int sst = sp.task_maxb;  // stride of the staged body arrays
    int* status = &w.ctr->status;
    for (int i = tid; i < T.w; i += bs) sver[i] = 0;
    // the task's bodies, one cp.async group per thread (the arbiter ring, in iterations,
    // follows as later groups so that both loads are in flight together)
    for (int i = tid; i < T.w; i += bs) {
        const float4* src = (const float4*)&w.body[w.sc_tbody[T.z + i]];
        cp_async16(&sbody[i], src); cp_async16(&sbody[sst + i], src + 1);
        cp_async16(&sbody[2 * sst + i], src + 2); cp_async16(&sbody[3 * sst + i], src + 3);
    }
    // (the bodies' group: committed with the positions below in Prepare, here otherwise,
    // so that the arbiter ring of the iterations follows as later groups)
    if (kind != PASS_PREPARE) cp_async_commit();
    bool ok = true;
    if (kind == PASS_PREPARE) {
        // Prepare also needs the bodies' positions and orientations: staged into the
        // arbiter ring, which Prepare does not use, when they fit
        float4* spos = ring;
        float4* sq = ring + T.w;
        const bool staged = 2 * T.w <= JG_TASK_RING * bs * JG_TASK_STAGE_F4;
        if (staged)
            for (int i = tid; i < T.w; i += bs) {
                const int b = w.sc_tbody[T.z + i];
                cp_async16(&spos[i], &w.pos[b]);
                cp_async16(&sq[i], &w.q[b]);
            }
        cp_async_commit();
        cp_async_wait_0();
        __syncthreads();
        ok = prepare_task(w, A, sp, T, sbody, sst, spos, sq, staged, sver, abort_flag, status);
    } else if (T.y > 0) {
        if (sp.record_residual)
            ok = iterate_task<true>(w, A, T, kind == PASS_ITERATE, sbody, sst, ring, sver, abort_flag, status, d2, l2);
        else
            ok = iterate_task<false>(w, A, T, kind == PASS_ITERATE, sbody, sst, ring, sver, abort_flag, status, d2, l2);
    }
    cp_async_wait_0();  // no copy into shared memory outlives the task
    __syncthreads();
    for (int i = tid; i < T.w; i += bs) {
        float4* dst = (float4*)&w.body[w.sc_tbody[T.z + i]];
        dst[0] = sbody[i];
        dst[1] = sbody[sst + i];
    }
    __syncthreads();
    return ok && !*abort_flag;
}

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

// Waits until the tasks of the two grid phases before this one that may share a body with
// task t have completed them (phase level - 1, counter >= level; phase level - 2, counter
// >= level - 1) and task t its previous pass (counter >= level - 2); with these the last
// earlier access to each of t's bodies is finished.  False after about a second
// (JG_ERR_TIMEOUT recorded), or when another block has recorded a timeout.
__device__ __forceinline__ bool wait_deps(const WorldDev& w, int t, unsigned level, int* status) {
    __shared__ int dep_ok;
    if (threadIdx.x < 32) {  // warp 0: one dependency per lane, polled together
        const int lane = threadIdx.x;
        // lanes 0-3: grid phase level - 1; 4-7: level - 2; 8: the task itself, whose
        // previous pass (level - 3) another block may have run
        int n = -1;
        unsigned need = 0;
        if (lane < 8) {
            const int4 dep = w.sc_tdep[2 * t + (lane >> 2)];
            n = (&dep.x)[lane & 3];
            need = lane < 4 ? level : level - 1;
            if (lane >= 4 && level < 2) n = -1;
        } else if (lane == 8 && level >= 3) {
            n = t;
            need = level - 2;
        }
        const unsigned long long t0 = globaltimer_ns();
        int ok = 1;
        for (unsigned spins = 0;; ++spins) {
            const bool ready = n < 0 || (int)(ld_acquire(&w.sc_done[n]) - need) >= 0;
            if (__all_sync(0xffffffffu, ready)) break;
            if ((spins & 63) == 63) {
                int bad = 0;
                if (lane == 0) {
                    if (ld_relaxed_int(status) == JG_ERR_TIMEOUT) bad = 1;
                    else if (globaltimer_ns() - t0 > 1000000000ull) { atomicCAS(status, 0, JG_ERR_TIMEOUT); bad = 1; }
                }
                if (__shfl_sync(0xffffffffu, bad, 0)) { ok = 0; break; }
            }
            __nanosleep(spins < 4 ? 20 : 80);
        }
        if (lane == 0) dep_ok = ok;
    }
    __syncthreads();
    return dep_ok != 0;
}

// Partitioned solve: the schedule's three grids run as three phases of tasks per pass,
// then the remainder in global colours; integration phases are grid-stride.
__global__ void k_solve_tasks(WorldDev w, StepParams sp) {
    extern __shared__ float4 solve_smem[];
    float4* sbody = solve_smem;
    float4* ring = solve_smem + 4 * sp.task_maxb;
    volatile int* sver = (volatile int*)(ring + (size_t)JG_TASK_RING * blockDim.x * JG_TASK_STAGE_F4);
    __shared__ int s_abort;
    if (threadIdx.x == 0) s_abort = 0;
    __syncthreads();
    const ArbStore& A = w.arb[w.cur];
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    int* status = &w.ctr->status;
    int ntask[JG_SCHED_GRIDS], tbase[JG_SCHED_GRIDS];
    for (int g = 0; g < JG_SCHED_GRIDS; g++) { ntask[g] = w.sc->ntask[g]; tbase[g] = w.sc->task_base[g]; }
    const int ntasks = ntask[0] + ntask[1] + ntask[2];
    const int npass = 1 + sp.iterations + sp.relax;
    // With no remainder, consecutive grid phases hand off task by task instead of waiting at
    // a grid barrier: a task waits only for the tasks of the two phases before it that may
    // share its bodies (their completion counters), so a slow task delays its neighbours,
    // not the whole pass.  Grid barriers stay around the whole-body integration steps.
    // Every block runs its tasks in phase order and each awaited task belongs to an earlier
    // phase, so the waits end.  (Tasks go to blocks in cell order: a longest-first order,
    // static or claimed from a queue, measured slower.)
    if (w.ctr->ncolors == 0) {
        unsigned level = 0;  // grid phases started so far in this launch
        for (int s = 0; s < sp.substeps; s++) {
            if (!sp.stabilize) integrate_forces_all(w, sp, tid, nth);
            if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
            for (int pass = 0; pass < npass; pass++) {
                const bool relax = pass > sp.iterations;
                const int kind = pass == 0 ? PASS_PREPARE : (relax ? PASS_RELAX : PASS_ITERATE);
                float d2 = 0.f, l2 = 0.f;
                for (int g = 0; g < JG_SCHED_GRIDS; g++, level++) {
                    for (int t = tbase[g] + blockIdx.x; t < tbase[g] + ntask[g]; t += gridDim.x) {
                        if (!wait_deps(w, t, level, status)) return;
                        if (!run_task(w, A, sp, t, kind, sbody, ring, sver, &s_abort, d2, l2)) return;
                        if (threadIdx.x == 0) {  // run_task ended with a block barrier
                            __threadfence();
                            st_release_u32(&w.sc_done[t], level + 1);
                        }
                    }
                }
                if (sp.record_residual && s == 0 && pass > 0 && !relax && pass <= JG_RESID_MAX)
                    block_reduce_add(d2, l2, w.resid + 2 * (pass - 1));
                if (pass == sp.iterations) {  // after the last biased iteration (World.Step.cs:244-246)
                    if (!grid_sync(w.bar_count, w.bar_gen, status)) return;  // every task of the pass
                    if (w.rec_on && s == 0) record_targets(w, A, tid, nth);
                    if (!sp.stabilize) integrate_velocities_all(w, sp, tid, nth);
                    if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
                }
            }
            if (!grid_sync(w.bar_count, w.bar_gen, status)) return;  // before the next IntegrateForces
        }
        return;
    }
    // With a remainder: the three grids as three phases per pass with a grid barrier after
    // each, then the remainder in global colours.
    for (int s = 0; s < sp.substeps; s++) {
        if (!sp.stabilize) integrate_forces_all(w, sp, tid, nth);
        if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
        for (int pass = 0; pass < npass; pass++) {
            const bool relax = pass > sp.iterations;
            const int kind = pass == 0 ? PASS_PREPARE : (relax ? PASS_RELAX : PASS_ITERATE);
            float d2 = 0.f, l2 = 0.f;
            for (int g = 0; g < JG_SCHED_GRIDS; g++) {
                if (ntask[g] == 0) continue;
                for (int t = tbase[g] + blockIdx.x; t < tbase[g] + ntask[g]; t += gridDim.x)
                    if (!run_task(w, A, sp, t, kind, sbody, ring, sver, &s_abort, d2, l2)) return;
                if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
            }
            if (!remainder_pass(w, A, sp, pass == 0 ? 0 : 1, !relax, !relax, tid, nth, d2, l2)) return;
            if (sp.record_residual && s == 0 && pass > 0 && !relax && pass <= JG_RESID_MAX) block_reduce_add(d2, l2, w.resid + 2 * (pass - 1));
            if (pass == sp.iterations) {  // after the last biased iteration (World.Step.cs:244-246)
                if (w.rec_on && s == 0) record_targets(w, A, tid, nth);
                if (!sp.stabilize) integrate_velocities_all(w, sp, tid, nth);
                if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
            }
        }
    }
}

// RigidBody.Update (RigidBody.cs:716-764) + UpdateWorldInertia (RigidBody.cs:903-923)
__global__ void k_update_bodies(WorldDev w, StepParams sp) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.nb; i += gridDim.x * blockDim.x) {
        int4 bi = w.binfo[i];
        if (sp.allow_deact && !(bi.y & JG_BODY_ACTIVE)) continue;  // only active bodies update
        SBody b = w.body[i];
        int axes = 63 ^ ((bi.y >> 4) & 63);
        v3 v = mk3(b.v), av = mk3(b.w);
        if ((axes & 7) != 7) { if (!(axes & 1)) v.x = 0; if (!(axes & 2)) v.y = 0; if (!(axes & 4)) v.z = 0; }
        if ((axes & 56) != 56) { if (!(axes & 8)) av.x = 0; if (!(axes & 16)) av.y = 0; if (!(axes & 32)) av.z = 0; }
        if (sp.allow_deact) {
            // the rest test of RigidBody.Update (RigidBody.cs:723-743): a kinematic body rests only
            // when it does not move, a dynamic one below the thresholds; resting accumulates the
            // sleep time, and a body that moved or has not rested long enough marks its island
            float4 sl = w.sleep[i];
            const bool kin = bi.x == JG_MOTION_KINEMATIC;
            const v3 zero = mk3(0.f);
            const bool resting = kin ? (av == zero && v == zero) : (len2(av) < sl.w && len2(v) < sl.z);
            sl.x = resting ? sl.x + sp.dt : 0.f;
            w.sleep[i].x = sl.x;
            if ((kin && !resting) || sl.x < sl.y) w.binfo[i].w = bi.w | 1;
        }
        if (bi.x == JG_MOTION_DYNAMIC) {
            float4 il0 = w.il0[i], il1 = w.il1[i];
            sym6 L; L.m11 = il0.x; L.m12 = il0.y; L.m13 = il0.z; L.m22 = il0.w; L.m23 = il1.x; L.m33 = il1.y;
            sym6 I = sym_transform(L, mat_from_quat(mkq(w.q[i])));
            if ((bi.y >> 4) & 56) {
                // RigidBody.RestrictAngularMotion on the inverse inertia (Schur complements)
                if ((axes & 56) == 0) { I.m11 = I.m12 = I.m13 = I.m22 = I.m23 = I.m33 = 0; }
                else {
                    if (!(axes & 8)) {
                        if (I.m11 > 0) { float xy = I.m12 / I.m11, xz = I.m13 / I.m11; I.m22 -= xy * I.m12; I.m23 -= xy * I.m13; I.m33 -= xz * I.m13; }
                        I.m11 = I.m12 = I.m13 = 0;
                    }
                    if (!(axes & 16)) {
                        if (I.m22 > 0) { float xy = I.m12 / I.m22, yz = I.m23 / I.m22; I.m11 -= xy * I.m12; I.m13 -= xy * I.m23; I.m33 -= yz * I.m23; }
                        I.m12 = I.m22 = I.m23 = 0;
                    }
                    if (!(axes & 32)) {
                        if (I.m33 > 0) { float xz = I.m13 / I.m33, yz = I.m23 / I.m33; I.m11 -= xz * I.m13; I.m12 -= xz * I.m23; I.m22 -= yz * I.m23; }
                        I.m13 = I.m23 = I.m33 = 0;
                    }
                }
            }
            float im = il1.z;
            v3 imv = mk3(im);
            if ((axes & 7) != 7) { if (!(axes & 1)) imv.x = 0; if (!(axes & 2)) imv.y = 0; if (!(axes & 4)) imv.z = 0; }
            float4 mt = w.mat[i];
            av = av * mt.w;
            v = v * mt.z;
            v3 force = mk3(w.force[i]), torque = mk3(w.torque[i]);
            v3 dv = cmul(force, imv) * sp.sub_dt;
            v3 dw = sym_mul(I, torque) * sp.sub_dt;
            if (!(bi.y & JG_BODY_NO_GRAVITY)) {
                v3 g = mk3(sp.gravity.x, sp.gravity.y, sp.gravity.z);
                if ((axes & 7) != 7) { if (!(axes & 1)) g.x = 0; if (!(axes & 2)) g.y = 0; if (!(axes & 4)) g.z = 0; }
                dv = dv + g * sp.sub_dt;
            }
            w.dv[i] = f4(dv, 0.f);
            w.dw[i] = f4(dw, 0.f);
            w.force[i] = make_float4(0, 0, 0, 0);
            w.torque[i] = make_float4(0, 0, 0, 0);
            int fl = SB_DYNAMIC | ((bi.y >> 4) & 7 ? SB_LINLOCK : 0);
            b.i0 = make_float4(I.m11, I.m12, I.m13, I.m22);
            b.i1 = make_float4(I.m23, I.m33, imv.z, __int_as_float(fl));
            b.v = f4(v, imv.x);
            b.w = f4(av, imv.y);
        } else {
            b.v = f4(v, 0.f);
            b.w = f4(av, 0.f);
            b.i0 = make_float4(0, 0, 0, 0);
            b.i1 = make_float4(0, 0, 0, __int_as_float(0));
        }
        w.body[i] = b;
    }
}

}  // namespace

// Shared memory limits of the current device.
static void smem_limits(int& per_block, int& per_sm) {
    int b = 0, m = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&m, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (b <= 0) b = 48 * 1024;
    if (m <= 0) m = b;
    per_block = b; per_sm = m;
}

// Lets the task solve take all the dynamic shared memory the current device allows, once
// per device (called when a world is created), so that worlds with different launch
// shapes never have to change the attribute under each other.
int jg_solver_init() {
    int pb, psm;
    smem_limits(pb, psm);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, (const void*)k_solve_tasks) != cudaSuccess) return -1;
    int dyn = pb - (int)fa.sharedSizeBytes;
    return cudaFuncSetAttribute(k_solve_tasks, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) == cudaSuccess ? 0 : -1;
}

// Bodies a task can stage next to the arbiter ring of `block` threads when
// `ctas_per_sm` task CTAs share an SM (1 KB per CTA is reserved by the runtime).
int jg_solver_task_maxb(int block, int ctas_per_sm) {
    int pb, psm;
    smem_limits(pb, psm);
    if (ctas_per_sm < 1) ctas_per_sm = 1;
    long long avail = std::min<long long>(pb, psm / ctas_per_sm - 1024);
    long long ring = (long long)JG_TASK_RING * block * JG_TASK_STAGE_F4 * 16;
    long long m = (avail - ring - 256) / 68;  // 64 B of staged body and a 4 B order count per slot
    if (m > 4096) m = 4096;
    return m > 0 ? (int)m : 0;
}

static size_t task_smem(const StepParams& p, int block) {
    return ((size_t)4 * p.task_maxb + (size_t)JG_TASK_RING * block * JG_TASK_STAGE_F4) * 16 + (size_t)4 * p.task_maxb;
}

// The cooperative grid of each solve kernel is sized once per world (its device, block,
// shared memory and CTAs per SM) and kept in the world's launch cache.
int jg_launch_solve(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm, int block, int ctas_per_sm) {
    if (p.partition) {
        if (block <= 0) block = JG_TASK_BLOCK;
        if (ctas_per_sm <= 0) ctas_per_sm = JG_TASK_CTAS;
        size_t smem = task_smem(p, block);
        if (w.lc_tasks_block != block || w.lc_tasks_smem != smem || w.lc_tasks_ctas != ctas_per_sm || w.lc_tasks_grid == 0) {
            int occ = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_solve_tasks, block, smem);
            if (occ < 1) return -1;
            if (occ > ctas_per_sm) occ = ctas_per_sm;
            w.lc_tasks_grid = nsm * occ;
            w.lc_tasks_block = block;
            w.lc_tasks_smem = smem;
            w.lc_tasks_ctas = ctas_per_sm;
        }
        cudaMemsetAsync(w.bar_count, 0, sizeof(unsigned) * 2, s);
        StepParams sp = p;
        void* args[] = {(void*)&w, (void*)&sp};
        cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_solve_tasks, dim3(w.lc_tasks_grid), dim3(block), args, smem, s);
        return e == cudaSuccess ? w.lc_tasks_grid : -1;
    }
    if (block <= 0) block = 256;
    if (ctas_per_sm <= 0) ctas_per_sm = 2;
    if (w.lc_solve_block != block || w.lc_solve_ctas != ctas_per_sm || w.lc_solve_grid == 0) {
        int occ = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_solve, block, 0);
        if (occ < 1) occ = 1;
        w.lc_solve_grid = nsm * (ctas_per_sm > occ ? occ : ctas_per_sm);
        w.lc_solve_block = block;
        w.lc_solve_ctas = ctas_per_sm;
    }
    cudaMemsetAsync(w.bar_count, 0, sizeof(unsigned) * 2, s);
    StepParams sp = p;
    void* args[] = {(void*)&w, (void*)&sp};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_solve, dim3(w.lc_solve_grid), dim3(block), args, 0, s);
    return e == cudaSuccess ? w.lc_solve_grid : -1;
}

void jg_launch_update(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm) {
    k_update_bodies<<<nsm * 4, 256, 0, s>>>(w, p);
}

void jg_solver_reset_launch_cache(WorldDev& w) { w.lc_solve_grid = 0; w.lc_tasks_grid = 0; w.lc_color_grid = 0; }
