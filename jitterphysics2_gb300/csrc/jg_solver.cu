// Substepped sequential-impulse solve in one persistent, cooperatively launched kernel:
//   for each substep (World.Step.cs:234-253):
//     IntegrateForces (World.Step.cs:1060-1072)                       bodies, grid-stride
//     Prepare, colour by colour (Contact.cs:802-924, BallSocket.cs:140-183, HingeAngle.cs:133-220)
//     iterations x colours: Iterate (Contact.cs:931-1018, BallSocket.cs:223-252, HingeAngle.cs:313-364)
//     IntegrateVelocities (World.Step.cs:1106-1133)                   bodies, grid-stride
//     relaxation x colours: Iterate without bias (World.Step.cs:1135-1153)
// Rows of one colour share no dynamic body, so a colour is solved in parallel with no
// atomics; a grid barrier separates colours.  Arbiters are stored colour-sorted, so each
// colour is a contiguous range: row loads are coalesced float4s, body loads are 64-byte
// records.  The per-step body update (RigidBody.Update, RigidBody.cs:716-764) is a
// separate kernel.
#include "jg_sync.cuh"

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

// Contact.Iterate (Contact.cs:931-1018).  Returns the squared impulse change for the
// residual metric.
__device__ __forceinline__ void iterate_contact(const ArbStore& A, int i, int mode, float friction, LBody& b1, LBody& b2,
                                                bool apply_bias, float& d2, float& l2) {
    float4 cn = A.cn[i], ct1 = A.ct1[i], ct2 = A.ct2[i], cr1 = A.cr1[i], cr2 = A.cr2[i], ca = A.cacc[i];
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
    A.cacc[i] = make_float4(aN, aT1, aT2, mT2);
    d2 += ni * ni + ti1 * ti1 + ti2 * ti2;
    l2 += aN * aN + aT1 * aT1 + aT2 * aT2;
    v3 imp = ni * n;
    imp = imp + ti1 * t1;
    imp = imp + ti2 * t2;
    if (mode & 1) b1.v = b1.v - cmul(imp, b1.im);
    if (mode & 2) b1.w = b1.w - sym_mul(b1.I, cross(rel1, imp));
    if (mode & 4) b2.v = b2.v + cmul(imp, b2.im);
    if (mode & 8) b2.w = b2.w + sym_mul(b2.I, cross(rel2, imp));
}

#include "jg_joints.cuh"

__device__ __forceinline__ void solve_arbiter(const WorldDev& w, const ArbStore& A, int a, int phase, const StepParams& sp,
                                              bool bias, float& d2, float& l2) {
    int4 info = A.info[a];
    int usage = info.x & 15;
    if (!usage) return;
    int mode = info.y;
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

__global__ void k_solve(WorldDev w, StepParams sp) {
    const ArbStore& A = w.arb[w.cur];
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int ncol = w.ctr->ncolors;
    int* status = &w.ctr->status;
    const int nb = w.nb;
    for (int s = 0; s < sp.substeps; s++) {
        // IntegrateForces
        for (int i = tid; i < nb; i += nth) {
            if (w.binfo[i].x != JG_MOTION_DYNAMIC) continue;
            SBody b = w.body[i];
            float4 dv = w.dv[i], dw = w.dw[i];
            b.w = make_float4(b.w.x + dw.x, b.w.y + dw.y, b.w.z + dw.z, b.w.w);
            b.v = make_float4(b.v.x + dv.x, b.v.y + dv.y, b.v.z + dv.z, b.v.w);
            w.body[i].v = b.v;
            w.body[i].w = b.w;
        }
        if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
        const int total_iters = 1 + sp.iterations;
        for (int it = 0; it < total_iters; it++) {
            float d2 = 0.f, l2 = 0.f;
            for (int c = 0; c < ncol; c++) {
                int beg = w.color_start[c], end = w.color_start[c + 1];
                for (int a = beg + tid; a < end; a += nth) solve_arbiter(w, A, a, it == 0 ? 0 : 1, sp, true, d2, l2);
                int jb = w.jcolor_start[c], je = w.jcolor_start[c + 1];
                for (int j = jb + tid; j < je; j += nth) {
                    if (it == 0) joint_prepare(w, w.jorder[j], sp);
                    else joint_iterate(w, w.jorder[j], sp);
                }
                if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
            }
            if (sp.record_residual && s == 0 && it > 0 && it <= 64) block_reduce_add(d2, l2, w.resid + 2 * (it - 1));
        }
        // IntegrateVelocities
        for (int i = tid; i < nb; i += nth) {
            int4 bi = w.binfo[i];
            if (bi.x == JG_MOTION_STATIC) continue;
            SBody b = w.body[i];
            v3 lv = mk3(b.v), av = mk3(b.w);
            float4 p = w.pos[i];
            w.pos[i] = make_float4(p.x + lv.x * sp.sub_dt, p.y + lv.y * sp.sub_dt, p.z + lv.z * sp.sub_dt, p.w);
            q4 rq = rotation_quaternion(av, sp.sub_dt);
            q4 q = qnormalize(qmul(rq, mkq(w.q[i])));
            w.q[i] = f4(q);
            if ((bi.y & JG_BODY_GYROSCOPIC) && ((bi.y >> 4) & 63) == 0) {
                // SolveGyroscopic (World.Step.cs:1075-1104): one implicit Newton step
                sym6 Ii;
                Ii.m11 = b.i0.x; Ii.m12 = b.i0.y; Ii.m13 = b.i0.z; Ii.m22 = b.i0.w; Ii.m23 = b.i1.x; Ii.m33 = b.i1.y;
                float det = Ii.m11 * (Ii.m22 * Ii.m33 - Ii.m23 * Ii.m23) + Ii.m12 * (Ii.m23 * Ii.m13 - Ii.m12 * Ii.m33) +
                            Ii.m13 * (Ii.m12 * Ii.m23 - Ii.m22 * Ii.m13);
                float id = 1.0f / det;
                if (isfinite(id) && id != 0.f) {
                    sym6 I;
                    I.m11 = (Ii.m22 * Ii.m33 - Ii.m23 * Ii.m23) * id; I.m12 = (Ii.m13 * Ii.m23 - Ii.m12 * Ii.m33) * id;
                    I.m13 = (Ii.m12 * Ii.m23 - Ii.m22 * Ii.m13) * id; I.m22 = (Ii.m11 * Ii.m33 - Ii.m13 * Ii.m13) * id;
                    I.m23 = (Ii.m13 * Ii.m12 - Ii.m23 * Ii.m11) * id; I.m33 = (Ii.m11 * Ii.m22 - Ii.m12 * Ii.m12) * id;
                    v3 Iw = sym_mul(I, av);
                    v3 f = sp.sub_dt * cross(av, Iw);
                    float M[3][3] = {{I.m11, I.m12, I.m13}, {I.m12, I.m22, I.m23}, {I.m13, I.m23, I.m33}};
                    float W[3][3] = {{0, -av.z, av.y}, {av.z, 0, -av.x}, {-av.y, av.x, 0}};
                    float L[3][3] = {{0, -Iw.z, Iw.y}, {Iw.z, 0, -Iw.x}, {-Iw.y, Iw.x, 0}};
                    float J[3][3];
                    for (int r = 0; r < 3; r++)
                        for (int c = 0; c < 3; c++)
                            J[r][c] = M[r][c] + sp.sub_dt * ((W[r][0] * M[0][c] + W[r][1] * M[1][c] + W[r][2] * M[2][c]) - L[r][c]);
                    float jd = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                               J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
                    if (jd != 0.f && isfinite(jd)) {
                        float ij = 1.0f / jd;
                        float inv[3][3];
                        inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * ij;
                        inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * ij;
                        inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * ij;
                        inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * ij;
                        inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * ij;
                        inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * ij;
                        inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * ij;
                        inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * ij;
                        inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * ij;
                        v3 d = mk3(f.x * inv[0][0] + f.y * inv[0][1] + f.z * inv[0][2], f.x * inv[1][0] + f.y * inv[1][1] + f.z * inv[1][2],
                                   f.x * inv[2][0] + f.y * inv[2][1] + f.z * inv[2][2]);
                        v3 nw = av - d;
                        w.body[i].w = f4(nw, b.w.w);
                    }
                }
            }
        }
        if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
        for (int it = 0; it < sp.relax; it++) {
            float d2 = 0.f, l2 = 0.f;
            for (int c = 0; c < ncol; c++) {
                int beg = w.color_start[c], end = w.color_start[c + 1];
                for (int a = beg + tid; a < end; a += nth) solve_arbiter(w, A, a, 1, sp, false, d2, l2);
                if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
            }
        }
    }
}

// RigidBody.Update (RigidBody.cs:716-764) + UpdateWorldInertia (RigidBody.cs:903-923)
__global__ void k_update_bodies(WorldDev w, StepParams sp) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.nb; i += gridDim.x * blockDim.x) {
        int4 bi = w.binfo[i];
        SBody b = w.body[i];
        int axes = 63 ^ ((bi.y >> 4) & 63);
        v3 v = mk3(b.v), av = mk3(b.w);
        if ((axes & 7) != 7) { if (!(axes & 1)) v.x = 0; if (!(axes & 2)) v.y = 0; if (!(axes & 4)) v.z = 0; }
        if ((axes & 56) != 56) { if (!(axes & 8)) av.x = 0; if (!(axes & 16)) av.y = 0; if (!(axes & 32)) av.z = 0; }
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

static int g_solve_grid = 0, g_solve_block = 0;
int jg_launch_solve(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm, int block, int ctas_per_sm) {
    if (block <= 0) block = 256;
    if (ctas_per_sm <= 0) ctas_per_sm = 2;
    if (g_solve_block != block || g_solve_grid == 0) {
        int occ = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_solve, block, 0);
        if (occ < 1) occ = 1;
        if (ctas_per_sm > occ) ctas_per_sm = occ;
        g_solve_grid = nsm * ctas_per_sm;
        g_solve_block = block;
    }
    cudaMemsetAsync(w.bar_count, 0, sizeof(unsigned) * 2, s);
    StepParams sp = p;
    void* args[] = {(void*)&w, (void*)&sp};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_solve, dim3(g_solve_grid), dim3(block), args, 0, s);
    return e == cudaSuccess ? g_solve_grid : -1;
}

void jg_launch_update(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm) {
    k_update_bodies<<<nsm * 4, 256, 0, s>>>(w, p);
}

void jg_solver_reset_launch_cache() { g_solve_grid = 0; }
