// Device constraint rows, solved in the same colours as the contacts: BallSocket
// (Dynamics/Constraints/BallSocket.cs:140-252), HingeAngle (HingeAngle.cs:133-364),
// DistanceLimit (DistanceLimit.cs:227-391), ConeLimit (ConeLimit.cs:262-404), TwistAngle
// (TwistAngle.cs:170-323), FixedAngle (FixedAngle.cs:87-181), PointOnPlane
// (PointOnPlane.cs:128-256), AngularMotor (AngularMotor.cs:128-180), LinearMotor
// (LinearMotor.cs:152-231), AngularServo (AngularServo.cs:125-172), LinearServo
// (LinearServo.cs:149-201), LinearAxisServo (LinearAxisServo.cs:169-224) and TwistServo
// (TwistServo.cs:150-192), PointOnLine (PointOnLine.cs:149-465) and EllipticalConeLimit
// (EllipticalConeLimit.cs:257-429).  Included by the solver translation unit.  Matrices are
// row-major float[3][3].
//
// JointDev fields of the one-row kinds: la1/la2 anchors (DistanceLimit) or local axes
// (ConeLimit); axis / q0 the twist axis and reference rotation (TwistAngle); lim = (min, max,
// distance or fixed angle, clamp); prm = (bias factor, softness); acc.x the accumulated
// impulse, bias.x the bias, bil.x the effective mass, bil.w the hemisphere (TwistAngle);
// Jacobian blocks in eff[0..2] and jac[0] (the ConeLimit block persists between steps).
#pragma once

struct M3x { float a[3][3]; };
__device__ __forceinline__ M3x mzero() { M3x m; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) m.a[i][j] = 0.f; return m; }
__device__ __forceinline__ M3x mskew(v3 v) {
    M3x m = mzero();
    m.a[0][1] = -v.z; m.a[0][2] = v.y; m.a[1][0] = v.z; m.a[1][2] = -v.x; m.a[2][0] = -v.y; m.a[2][1] = v.x;
    return m;
}
__device__ __forceinline__ v3 mv(const M3x& M, v3 v) {
    return mk3(v.x * M.a[0][0] + v.y * M.a[0][1] + v.z * M.a[0][2], v.x * M.a[1][0] + v.y * M.a[1][1] + v.z * M.a[1][2],
               v.x * M.a[2][0] + v.y * M.a[2][1] + v.z * M.a[2][2]);
}
__device__ __forceinline__ v3 mtv(const M3x& M, v3 v) {
    return mk3(v.x * M.a[0][0] + v.y * M.a[1][0] + v.z * M.a[2][0], v.x * M.a[0][1] + v.y * M.a[1][1] + v.z * M.a[2][1],
               v.x * M.a[0][2] + v.y * M.a[1][2] + v.z * M.a[2][2]);
}
__device__ __forceinline__ M3x mmulx(const M3x& x, const M3x& y) {
    M3x o;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) o.a[i][j] = x.a[i][0] * y.a[0][j] + x.a[i][1] * y.a[1][j] + x.a[i][2] * y.a[2][j];
    return o;
}
__device__ __forceinline__ float mdetx(const M3x& m) {
    const auto& a = m.a;
    return a[0][0] * a[1][1] * a[2][2] + a[0][1] * a[1][2] * a[2][0] + a[0][2] * a[1][0] * a[2][1] -
           a[2][0] * a[1][1] * a[0][2] - a[2][1] * a[1][2] * a[0][0] - a[2][2] * a[1][0] * a[0][1];
}
__device__ __forceinline__ bool mfin(const M3x& m) {
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) if (!isfinite(m.a[i][j])) return false;
    return true;
}
// JMatrix.TryInverseUnscaled / Inverse (JMatrix.cs:404-478)
__device__ bool minv_u(const M3x& m, M3x& o) {
    float idet = 1.0f / mdetx(m);
    if (!(isfinite(idet) && fabsf(idet) >= 1.17549435e-38f)) { o = mzero(); return false; }
    const auto& a = m.a;
    o.a[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) * idet;
    o.a[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * idet;
    o.a[0][2] = (a[0][1] * a[1][2] - a[1][1] * a[0][2]) * idet;
    o.a[1][0] = (a[1][2] * a[2][0] - a[2][2] * a[1][0]) * idet;
    o.a[1][1] = (a[0][0] * a[2][2] - a[2][0] * a[0][2]) * idet;
    o.a[1][2] = (a[0][2] * a[1][0] - a[1][2] * a[0][0]) * idet;
    o.a[2][0] = (a[1][0] * a[2][1] - a[2][0] * a[1][1]) * idet;
    o.a[2][1] = (a[0][1] * a[2][0] - a[2][1] * a[0][0]) * idet;
    o.a[2][2] = (a[0][0] * a[1][1] - a[1][0] * a[0][1]) * idet;
    return mfin(o);
}
__device__ bool minvx(const M3x& m, M3x& o) {
    if (minv_u(m, o)) return true;
    float s = 0.f;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) s = fmaxf(s, fabsf(m.a[i][j]));
    if (s > 0 && isfinite(s)) {
        M3x n;
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) n.a[i][j] = m.a[i][j] / s;
        if (minv_u(n, o)) {
            for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.a[i][j] /= s;
            if (mfin(o)) return true;
        }
    }
    o = mzero();
    return false;
}
// MathHelper.JacobiRotate (MathHelper.cs:374-406)
__device__ bool jacobi(float* a, float* basis, int p, int q, float tol) {
    float off = a[3 * p + q];
    if (fabsf(off) <= tol) return false;
    float tau = (a[3 * q + q] - a[3 * p + p]) / (2.0f * off);
    float tg = copysignf(1.0f, tau) / (fabsf(tau) + sqrtf(1.0f + tau * tau));
    float cs = 1.0f / sqrtf(1.0f + tg * tg);
    float sn = tg * cs;
    a[3 * p + p] -= tg * off;
    a[3 * q + q] += tg * off;
    a[3 * p + q] = a[3 * q + p] = 0;
    for (int k = 0; k < 3; k++) {
        if (k != p && k != q) {
            float akp = a[3 * k + p], akq = a[3 * k + q];
            a[3 * k + p] = a[3 * p + k] = cs * akp - sn * akq;
            a[3 * k + q] = a[3 * q + k] = sn * akp + cs * akq;
        }
        float vkp = basis[3 * k + p], vkq = basis[3 * k + q];
        basis[3 * k + p] = cs * vkp - sn * vkq;
        basis[3 * k + q] = sn * vkp + cs * vkq;
    }
    return true;
}
// MathHelper.PseudoInverseSymmetric (MathHelper.cs:282-325)
__device__ M3x pinv_sym(const M3x& m) {
    float s = fmaxf(fabsf(m.a[0][0]), fmaxf(fabsf(m.a[1][1]), fabsf(m.a[2][2])));
    if (!(s > 0) || !isfinite(s)) return mzero();
    float n11 = m.a[0][0] / s, n12 = m.a[0][1] / s, n13 = m.a[0][2] / s, n22 = m.a[1][1] / s, n23 = m.a[1][2] / s, n33 = m.a[2][2] / s;
    const float tol = 1e-6f;
    float nd = n11 * (n22 * n33 - n23 * n23) + n12 * (n23 * n13 - n12 * n33) + n13 * (n12 * n23 - n22 * n13);
    M3x inv;
    if (fabsf(nd) > tol && minvx(m, inv)) return inv;
    float a[9] = {n11, n12, n13, n12, n22, n23, n13, n23, n33};
    float basis[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int sw = 0; sw < 8; sw++) {
        bool ch = jacobi(a, basis, 0, 1, tol);
        ch |= jacobi(a, basis, 0, 2, tol);
        ch |= jacobi(a, basis, 1, 2, tol);
        if (!ch) break;
    }
    float r11 = 0, r12 = 0, r13 = 0, r22 = 0, r23 = 0, r33 = 0;
    for (int i = 0; i < 3; i++) {
        float ev = a[3 * i + i];
        if (!(ev > tol)) continue;
        float wgt = (1.0f / ev) / s;
        v3 ax = mk3(basis[i], basis[3 + i], basis[6 + i]);
        r11 += wgt * (ax.x * ax.x); r12 += wgt * (ax.x * ax.y); r13 += wgt * (ax.x * ax.z);
        r22 += wgt * (ax.y * ax.y); r23 += wgt * (ax.y * ax.z); r33 += wgt * (ax.z * ax.z);
    }
    M3x o;
    o.a[0][0] = r11; o.a[0][1] = r12; o.a[0][2] = r13;
    o.a[1][0] = r12; o.a[1][1] = r22; o.a[1][2] = r23;
    o.a[2][0] = r13; o.a[2][1] = r23; o.a[2][2] = r33;
    return o;
}
// MathHelper.InverseSymmetric (MathHelper.cs:328-365)
__device__ M3x inv_symmetric(const M3x& m) {
    const float tol = 1e-6f;
    float dp = m.a[0][0] * m.a[1][1] * m.a[2][2];
    M3x inv;
    if (mdetx(m) / dp > tol && minvx(m, inv)) return inv;
    float x = m.a[0][0] > 0 ? sqrtf(m.a[0][0]) : 0, y = m.a[1][1] > 0 ? sqrtf(m.a[1][1]) : 0, z = m.a[2][2] > 0 ? sqrtf(m.a[2][2]) : 0;
    if (x == 0 && y == 0 && z == 0) return mzero();
    float xy = x > 0 && y > 0 ? m.a[0][1] / x / y : 0, xz = x > 0 && z > 0 ? m.a[0][2] / x / z : 0, yz = y > 0 && z > 0 ? m.a[1][2] / y / z : 0;
    M3x nrm;
    nrm.a[0][0] = 1; nrm.a[0][1] = xy; nrm.a[0][2] = xz;
    nrm.a[1][0] = xy; nrm.a[1][1] = 1; nrm.a[1][2] = yz;
    nrm.a[2][0] = xz; nrm.a[2][1] = yz; nrm.a[2][2] = 1;
    M3x r = pinv_sym(nrm);
    xy = x > 0 && y > 0 ? r.a[0][1] / x / y : 0;
    xz = x > 0 && z > 0 ? r.a[0][2] / x / z : 0;
    yz = y > 0 && z > 0 ? r.a[1][2] / y / z : 0;
    M3x o;
    o.a[0][0] = x > 0 ? r.a[0][0] / x / x : 0; o.a[0][1] = xy; o.a[0][2] = xz;
    o.a[1][0] = xy; o.a[1][1] = y > 0 ? r.a[1][1] / y / y : 0; o.a[1][2] = yz;
    o.a[2][0] = xz; o.a[2][1] = yz; o.a[2][2] = z > 0 ? r.a[2][2] / z / z : 0;
    return mfin(o) ? o : mzero();
}

__device__ __forceinline__ void jstore_m(float4* dst, const M3x& m) {
    for (int r = 0; r < 3; r++) dst[r] = make_float4(m.a[r][0], m.a[r][1], m.a[r][2], 0.f);
}
__device__ __forceinline__ M3x jload_m(const float4* src) {
    M3x m;
    for (int r = 0; r < 3; r++) { float4 v = src[r]; m.a[r][0] = v.x; m.a[r][1] = v.y; m.a[r][2] = v.z; }
    return m;
}
// JSymmetricMatrix.Transform(S, T) = T S T^T with a full T (JSymmetricMatrix.cs:247-260)
__device__ __forceinline__ M3x sym_transform_full(const sym6& S, const M3x& T) {
    m33 t;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) t.m[i][j] = T.a[i][j];
    sym6 r = sym_transform(S, t);
    M3x o;
    o.a[0][0] = r.m11; o.a[0][1] = r.m12; o.a[0][2] = r.m13;
    o.a[1][0] = r.m12; o.a[1][1] = r.m22; o.a[1][2] = r.m23;
    o.a[2][0] = r.m13; o.a[2][1] = r.m23; o.a[2][2] = r.m33;
    return o;
}

// BallSocket.PrepareForIterationBallSocket (BallSocket.cs:140-183)
__device__ void ballsocket_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    q4 q1 = mkq(w.q[i1]), q2 = mkq(w.q[i2]);
    v3 r1 = rotate(mk3(J.la1), q1), r2 = rotate(mk3(J.la2), q2);
    v3 p1 = mk3(w.pos[i1]) + r1, p2 = mk3(w.pos[i2]) + r2;
    M3x cr1 = mskew(r1), cr2 = mskew(r2);
    M3x t1 = sym_transform_full(b1.I, cr1), t2 = sym_transform_full(b2.I, cr2);
    // ((Scale(m1) + T1) + Scale(m2)) + T2, component-wise, in the reference's order
    M3x e;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) e.a[i][j] = t1.a[i][j] + t2.a[i][j];
    e.a[0][0] = ((b1.im.x + t1.a[0][0]) + b2.im.x) + t2.a[0][0];
    e.a[1][1] = ((b1.im.y + t1.a[1][1]) + b2.im.y) + t2.a[1][1];
    e.a[2][2] = ((b1.im.z + t1.a[2][2]) + b2.im.z) + t2.a[2][2];
    float soft = J.prm.y * sp.inv_sub_dt;
    e.a[0][0] += soft; e.a[1][1] += soft; e.a[2][2] += soft;
    M3x eff = inv_symmetric(e);
    v3 bias = (p2 - p1) * J.prm.x * sp.inv_dt;
    v3 acc = mk3(J.acc);
    if (b1.flags & SB_DYNAMIC) {
        b1.v = b1.v - cmul(acc, b1.im);
        b1.w = b1.w - sym_mul(b1.I, mv(cr1, acc));
        store_vel(w.body, i1, b1);
    }
    if (b2.flags & SB_DYNAMIC) {
        b2.v = b2.v + cmul(acc, b2.im);
        b2.w = b2.w + sym_mul(b2.I, mv(cr2, acc));
        store_vel(w.body, i2, b2);
    }
    J.r1 = f4(r1, 0.f); J.r2 = f4(r2, 0.f);
    J.bias = f4(bias, 0.f);
    jstore_m(J.eff, eff);
}
// BallSocket.IterateBallSocket (BallSocket.cs:223-252)
__device__ void ballsocket_iterate(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    M3x cr1 = mskew(mk3(J.r1)), cr2 = mskew(mk3(J.r2));
    v3 acc = mk3(J.acc);
    v3 sv = acc * J.prm.y * sp.inv_sub_dt;
    v3 jv = -b1.v + mv(cr1, b1.w) + b2.v - mv(cr2, b2.w);
    M3x eff = jload_m(J.eff);
    v3 lambda = -1.0f * mv(eff, jv + mk3(J.bias) + sv);
    J.acc = f4(acc + lambda, 0.f);
    if (b1.flags & SB_DYNAMIC) {
        b1.v = b1.v - cmul(lambda, b1.im);
        b1.w = b1.w - sym_mul(b1.I, mv(cr1, lambda));
        store_vel(w.body, i1, b1);
    }
    if (b2.flags & SB_DYNAMIC) {
        b2.v = b2.v + cmul(lambda, b2.im);
        b2.w = b2.w + sym_mul(b2.I, mv(cr2, lambda));
        store_vel(w.body, i2, b2);
    }
}

// AngularConstraintMath.CalculateJacobian (AngularConstraintMath.cs:65-95)
__device__ M3x calc_jacobian(q4 left, q4 right, v3& err, int& hemi) {
    q4 q = qmul(left, right);
    hemi = q.w < 0 ? -1 : 1;
    if (q.w < 0) { q.x = -q.x; q.y = -q.y; q.z = -q.z; q.w = -q.w; }
    v3 qv = mk3(q.x, q.y, q.z);
    float sine = sqrtf(len2(qv));
    M3x der;
    if (sine > 0) {
        float half = StableMathF::atan2(sine, q.w);
        v3 ax = qv * (1.0f / sine);
        err = ax * half;
        float diag = half * q.w / sine;
        float od = 1.0f - diag;
        M3x sk = mskew(err);
        float outer[3][3] = {{ax.x * ax.x, ax.x * ax.y, ax.x * ax.z}, {ax.x * ax.y, ax.y * ax.y, ax.y * ax.z}, {ax.x * ax.z, ax.y * ax.z, ax.z * ax.z}};
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) der.a[i][j] = ((i == j ? diag : 0.f) + od * outer[i][j]) - sk.a[i][j];
    } else {
        err = mk3(0.f);
        der = mzero();
        der.a[0][0] = der.a[1][1] = der.a[2][2] = 1.f;
    }
    m33 R = mat_from_quat(left);
    M3x Rm;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) Rm.a[i][j] = R.m[i][j];
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) der.a[i][j] = -0.5f * der.a[i][j];
    return mmulx(der, Rm);
}

// HingeAngle.PrepareForIterationHingeAngle (HingeAngle.cs:133-220)
__device__ void hinge_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    q4 q1 = mkq(w.q[i1]), q2 = mkq(w.q[i2]);
    v3 axis = mk3(J.axis);
    v3 p0 = create_orthonormal(axis);
    v3 p1 = cross(axis, p0);
    v3 rot;
    int hemi;
    M3x m0 = calc_jacobian(qmul(mkq(J.q0), qconj(q1)), q2, rot, hemi);
    v3 acc = mk3(J.acc);
    int old_hemi = (int)J.bil.w;
    if (old_hemi != 0 && old_hemi != hemi) acc = mk3(0.f);
    v3 err = mk3(dot(p0, rot), dot(p1, rot), dot(axis, rot));
    int clamp = 0;
    v3 c0 = mtv(m0, p0), c1 = mtv(m0, p1), c2 = mtv(m0, axis);
    M3x jac;  // columns c0 c1 c2 (JMatrix column-major UnsafeGet, JMatrix.cs:62-79)
    jac.a[0][0] = c0.x; jac.a[1][0] = c0.y; jac.a[2][0] = c0.z;
    jac.a[0][1] = c1.x; jac.a[1][1] = c1.y; jac.a[2][1] = c1.z;
    jac.a[0][2] = c2.x; jac.a[1][2] = c2.y; jac.a[2][2] = c2.z;
    sym6 Is;
    Is.m11 = b1.I.m11 + b2.I.m11; Is.m12 = b1.I.m12 + b2.I.m12; Is.m13 = b1.I.m13 + b2.I.m13;
    Is.m22 = b1.I.m22 + b2.I.m22; Is.m23 = b1.I.m23 + b2.I.m23; Is.m33 = b1.I.m33 + b2.I.m33;
    M3x jt;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) jt.a[i][j] = jac.a[j][i];
    M3x eff = sym_transform_full(Is, jt);
    float soft = J.prm.y, lsoft = J.prm.w, bias_f = J.prm.x, lbias = J.prm.z;
    eff.a[0][0] += soft * sp.inv_sub_dt;
    eff.a[1][1] += soft * sp.inv_sub_dt;
    eff.a[2][2] += lsoft * sp.inv_sub_dt;
    float minA = J.lim.x, maxA = J.lim.y, fixedA = J.lim.z;
    const float PI = 3.14159265358979323846f;
    bool full = minA <= -PI / 2 && maxA >= PI / 2;
    if (minA >= maxA) {
        clamp = 3;
        float ang = err.z - fixedA, half = PI / 2;
        if (!(ang >= -half && ang <= half)) {
            float period = 2 * half;
            ang = fmodf(ang, period);
            if (ang > half) ang -= period; else if (ang < -half) ang += period;
        }
        err.z = ang;
    } else if (!full && err.z >= maxA) {
        clamp = 1;
        err.z -= maxA;
    } else if (!full && err.z <= minA) {
        clamp = 2;
        err.z -= minA;
    } else {
        acc.z = 0;
        eff.a[2][2] = 0;
        eff.a[2][0] = eff.a[0][2] = 0;
        eff.a[2][1] = eff.a[1][2] = 0;
        jac.a[0][2] = jac.a[1][2] = jac.a[2][2] = 0;
    }
    v3 bil = mk3(0.f);
    float cx = 0.f, cy = 0.f;
    if (clamp == 1 || clamp == 2) {
        acc.z = clamp == 1 ? fminf(acc.z, 0.f) : fmaxf(acc.z, 0.f);
        M3x blk = mzero();
        blk.a[0][0] = eff.a[0][0]; blk.a[0][1] = eff.a[0][1]; blk.a[1][0] = eff.a[0][1]; blk.a[1][1] = eff.a[1][1];
        M3x bi = inv_symmetric(blk);
        bil = mk3(bi.a[0][0], bi.a[0][1], bi.a[1][1]);
        cx = eff.a[0][2];
        cy = eff.a[1][2];
    }
    eff = inv_symmetric(eff);
    v3 bias = err * sp.inv_dt;
    bias.x *= bias_f; bias.y *= bias_f; bias.z *= lbias;
    if (b1.flags & SB_DYNAMIC) { b1.w = b1.w + sym_mul(b1.I, mv(jac, acc)); store_vel(w.body, i1, b1); }
    if (b2.flags & SB_DYNAMIC) { b2.w = b2.w - sym_mul(b2.I, mv(jac, acc)); store_vel(w.body, i2, b2); }
    J.acc = f4(acc, 0.f);
    J.bias = f4(bias, 0.f);
    jstore_m(J.eff, eff);
    jstore_m(J.jac, jac);
    J.lim.w = (float)clamp;
    J.bil = make_float4(bil.x, bil.y, bil.z, (float)hemi);
    J.cpl = make_float4(cx, cy, 0.f, 0.f);
}
// HingeAngle.IterateHingeAngle (HingeAngle.cs:313-364)
__device__ void hinge_iterate(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    M3x jac = jload_m(J.jac), eff = jload_m(J.eff);
    v3 jv = mtv(jac, b1.w - b2.w);
    v3 acc = mk3(J.acc);
    v3 soft = acc * sp.inv_sub_dt;
    soft.x *= J.prm.y; soft.y *= J.prm.y; soft.z *= J.prm.w;
    v3 res = jv + mk3(J.bias) + soft;
    v3 lambda = -1.0f * mv(eff, res);
    v3 orig = acc;
    acc = acc + lambda;
    int clamp = (int)J.lim.w;
    if ((clamp == 1 && acc.z > 0) || (clamp == 2 && acc.z < 0)) {
        lambda.z = -orig.z;
        float x = res.x + J.cpl.x * lambda.z;
        float y = res.y + J.cpl.y * lambda.z;
        lambda.x = -(J.bil.x * x + J.bil.y * y);
        lambda.y = -(J.bil.y * x + J.bil.z * y);
        acc.x = orig.x + lambda.x;
        acc.y = orig.y + lambda.y;
        acc.z = 0;
    } else if (clamp == 0) {
        orig.z = 0;
        acc.z = 0;
    }
    lambda = acc - orig;
    J.acc = f4(acc, 0.f);
    if (b1.flags & SB_DYNAMIC) { b1.w = b1.w + sym_mul(b1.I, mv(jac, lambda)); store_vel(w.body, i1, b1); }
    if (b2.flags & SB_DYNAMIC) { b2.w = b2.w - sym_mul(b2.I, mv(jac, lambda)); store_vel(w.body, i2, b2); }
}

// ---- one-row limits ---------------------------------------------------------------------
__device__ __forceinline__ float clamp_impulse(int clamp, float acc) {
    if (clamp == 1) return fminf(acc, 0.0f);
    if (clamp == 2) return fmaxf(acc, 0.0f);
    return acc;
}
__device__ __forceinline__ float row_mass(float m, float softness, const StepParams& sp) {
    m += softness * sp.inv_sub_dt;
    return m > 0 ? 1.0f / m : 0.0f;
}
__device__ __forceinline__ sym6 sym_add(const sym6& a, const sym6& b) {
    sym6 o;
    o.m11 = a.m11 + b.m11; o.m12 = a.m12 + b.m12; o.m13 = a.m13 + b.m13;
    o.m22 = a.m22 + b.m22; o.m23 = a.m23 + b.m23; o.m33 = a.m33 + b.m33;
    return o;
}

// DistanceLimit.PrepareForIterationDistanceLimit (DistanceLimit.cs:227-306): the distance
// between the anchors against [distance + min, distance + max]
__device__ void distance_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    v3 r1 = rotate(mk3(J.la1), mkq(w.q[i1])), r2 = rotate(mk3(J.la2), mkq(w.q[i2]));
    v3 dp = (mk3(w.pos[i2]) + r2) - (mk3(w.pos[i1]) + r1);
    float dist = sqrtf(len2(dp));
    float err = dist - J.lim.z;
    const float lo = J.lim.x, hi = J.lim.y;
    int clamp;
    if (lo >= hi) { err -= 0.5f * lo + 0.5f * hi; clamp = 3; }
    else if (err >= hi) { clamp = 1; err -= hi; }
    else if (err <= lo) { clamp = 2; err -= lo; }
    else { J.lim.w = 0.f; J.acc.x = 0.f; return; }
    if (dist == 0.0f) { J.lim.w = 0.f; J.acc.x = 0.f; return; }
    J.lim.w = (float)clamp;
    v3 n = dp * (1.0f / dist);
    v3 j0 = -1.0f * n, j1 = -1.0f * cross(r1, n), j2 = 1.0f * n, j3 = cross(r2, n);
    float m = dot(cmul(j0, b1.im), j0) + dot(cmul(j2, b2.im), j2) + dot(sym_mul(b1.I, j1), j1) + dot(sym_mul(b2.I, j3), j3);
    float eff = row_mass(m, J.prm.y, sp);
    float a = eff == 0.0f ? 0.0f : J.acc.x;
    J.acc.x = a;
    J.bil.x = eff;
    J.bias.x = err * J.prm.x * sp.inv_dt;
    J.eff[0] = f4(j0, 0.f); J.eff[1] = f4(j1, 0.f); J.eff[2] = f4(j2, 0.f); J.jac[0] = f4(j3, 0.f);
    if (b1.flags & SB_DYNAMIC) {
        b1.v = b1.v + cmul(a * j0, b1.im);
        b1.w = b1.w + sym_mul(b1.I, a * j1);
        store_vel(w.body, i1, b1);
    }
    if (b2.flags & SB_DYNAMIC) {
        b2.v = b2.v + cmul(a * j2, b2.im);
        b2.w = b2.w + sym_mul(b2.I, a * j3);
        store_vel(w.body, i2, b2);
    }
}
// DistanceLimit.IterateDistanceLimit (DistanceLimit.cs:344-391)
__device__ void distance_iterate(const WorldDev& w, JointDev& J, const StepParams& sp) {
    const int clamp = (int)J.lim.w;
    if (clamp == 0) return;
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    v3 j0 = mk3(J.eff[0]), j1 = mk3(J.eff[1]), j2 = mk3(J.eff[2]), j3 = mk3(J.jac[0]);
    float jv = dot(b1.v, j0) + dot(b1.w, j1) + dot(b2.v, j2) + dot(b2.w, j3);
    float soft = J.acc.x * J.prm.y * sp.inv_sub_dt;
    float lambda = -J.bil.x * (jv + J.bias.x + soft);
    float old = J.acc.x;
    J.acc.x = clamp_impulse(clamp, J.acc.x + lambda);
    lambda = J.acc.x - old;
    if (b1.flags & SB_DYNAMIC) {
        b1.v = b1.v + cmul(lambda * j0, b1.im);
        b1.w = b1.w + sym_mul(b1.I, lambda * j1);
        store_vel(w.body, i1, b1);
    }
    if (b2.flags & SB_DYNAMIC) {
        b2.v = b2.v + cmul(lambda * j2, b2.im);
        b2.w = b2.w + sym_mul(b2.I, lambda * j3);
        store_vel(w.body, i2, b2);
    }
}

// ConeLimit.PrepareForIterationConeLimit (ConeLimit.cs:262-356): the angle between the
// bodies' axes against [min, max]; the Jacobian row persists, and its sign flip drops the
// cached impulse
__device__ void cone_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    v3 a1 = rotate(mk3(J.la1), mkq(w.q[i1])), a2 = rotate(mk3(J.la2), mkq(w.q[i2]));
    v3 prev = mk3(J.eff[0]);
    v3 j0 = cross(a2, a1);
    float cosine = dot(a1, a2);
    const float minA = J.lim.x, maxA = J.lim.y;
    float lower = -minA, upper = -maxA;
    float sine = sqrtf(len2(j0));
    if (sine > 0) {
        j0 = j0 * (1.0f / sine);
    } else {
        v3 axis = create_orthonormal(a1);
        v3 other = cross(a1, axis);
        sym6 I = sym_add(b1.I, b2.I);
        j0 = dot(sym_mul(I, axis), axis) >= dot(sym_mul(I, other), other) ? axis : other;
    }
    v3 j1 = -j0;
    J.eff[0] = f4(j0, 0.f); J.eff[1] = f4(j1, 0.f);
    float acc = J.acc.x;
    if (dot(prev, j0) < 0) acc = 0.f;
    float err = -StableMathF::atan2(sine, cosine);
    const float PI = 3.14159265358979323846f;
    int clamp;
    if (lower == upper) { clamp = 3; err -= upper; }
    else if (err <= upper && maxA < PI) { clamp = 1; err -= upper; }
    else if (err >= lower && minA > 0) { clamp = 2; err -= lower; }
    else { J.lim.w = 0.f; J.acc.x = 0.f; return; }
    J.lim.w = (float)clamp;
    acc = clamp_impulse(clamp, acc);
    float m = dot(sym_mul(b1.I, j0), j0) + dot(sym_mul(b2.I, j1), j1);
    float eff = row_mass(m, J.prm.y, sp);
    if (eff == 0.0f) acc = 0.f;
    J.acc.x = acc;
    J.bil.x = eff;
    J.bias.x = -err * J.prm.x * sp.inv_dt;
    if (b1.flags & SB_DYNAMIC) { b1.w = b1.w + sym_mul(b1.I, acc * j0); store_vel(w.body, i1, b1); }
    if (b2.flags & SB_DYNAMIC) { b2.w = b2.w + sym_mul(b2.I, acc * j1); store_vel(w.body, i2, b2); }
}
// ConeLimit.IterateConeLimit (ConeLimit.cs:378-404)
__device__ void cone_iterate(const WorldDev& w, JointDev& J, const StepParams& sp) {
    const int clamp = (int)J.lim.w;
    if (clamp == 0) return;
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    v3 j0 = mk3(J.eff[0]), j1 = mk3(J.eff[1]);
    float jv = dot(b1.w, j0) + dot(b2.w, j1);
    float soft = J.acc.x * J.prm.y * sp.inv_sub_dt;
    float lambda = -J.bil.x * (jv + J.bias.x + soft);
    float old = J.acc.x;
    J.acc.x = clamp_impulse(clamp, J.acc.x + lambda);
    lambda = J.acc.x - old;
    if (b1.flags & SB_DYNAMIC) { b1.w = b1.w + sym_mul(b1.I, lambda * j0); store_vel(w.body, i1, b1); }
    if (b2.flags & SB_DYNAMIC) { b2.w = b2.w + sym_mul(b2.I, lambda * j1); store_vel(w.body, i2, b2); }
}

// QMatrix.ProjectMultiplyLeftRight (QMatrix.cs:112-125): the vector block (rows and columns
// 1..3) of L(left) R(right), the quaternions' left- and right-multiplication matrices in
// (w, x, y, z) order, each entry summed over k = 0..3 in order
__device__ M3x project_left_right(q4 l, q4 r) {
    const float L[4][4] = {{l.w, -l.x, -l.y, -l.z}, {l.x, l.w, -l.z, l.y}, {l.y, l.z, l.w, -l.x}, {l.z, -l.y, l.x, l.w}};
    const float Rm[4][4] = {{r.w, -r.x, -r.y, -r.z}, {r.x, r.w, r.z, -r.y}, {r.y, -r.z, r.w, r.x}, {r.z, r.y, -r.x, r.w}};
    M3x o;
    for (int i = 1; i < 4; i++)
        for (int c = 1; c < 4; c++) {
            float acc = L[i][0] * Rm[0][c];
            for (int k = 1; k < 4; k++) acc += L[i][k] * Rm[k][c];
            o.a[i - 1][c - 1] = acc;
        }
    return o;
}
// AngularConstraintMath.CalculateTwist (AngularConstraintMath.cs:33-64)
__device__ float calc_twist(q4 left, q4 right, v3 axis, v3& jac, int& hemi) {
    M3x m = project_left_right(left, right);
    for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) m.a[i][k] = -0.5f * m.a[i][k];
    q4 q = qmul(left, right);
    jac = mtv(m, axis);
    float proj = dot(axis, mk3(q.x, q.y, q.z));
    hemi = q.w < 0 ? -1 : 1;
    if (q.w < 0) {
        q.x = -q.x; q.y = -q.y; q.z = -q.z; q.w = -q.w;
        proj = proj * -1.0f;
        jac = jac * -1.0f;
    }
    float d2 = len2(jac);
    if (d2 > 0) jac = jac * (1.0f / sqrtf(d2));
    else jac = -rotate(axis, right);
    v3 perp = mk3(q.x, q.y, q.z) - axis * proj;
    float cosine = sqrtf(q.w * q.w + len2(perp));
    return 2.0f * StableMathF::atan2(proj, cosine);
}
// TwistAngle.PrepareForIterationTwistAngle (TwistAngle.cs:170-233)
__device__ void twist_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    q4 q1 = mkq(w.q[i1]), q2 = mkq(w.q[i2]);
    v3 jr;
    int hemi;
    float err = calc_twist(qmul(mkq(J.q0), qconj(q1)), q2, mk3(J.axis), jr, hemi);
    J.eff[0] = f4(jr, 0.f);
    const float lower = J.lim.x, upper = J.lim.y;
    float acc = J.acc.x;
    int old_hemi = (int)J.bil.w;
    if (old_hemi != 0 && old_hemi != hemi) acc = 0.f;
    J.bil.w = (float)hemi;
    const float PI = 3.14159265358979323846f;
    bool full = lower <= -PI && upper >= PI;
    int clamp;
    if (lower >= upper) {
        clamp = 3;
        float ang = err - J.lim.z;
        if (!(ang >= -PI && ang <= PI)) {
            float period = 2 * PI;
            ang = fmodf(ang, period);
            if (ang > PI) ang -= period; else if (ang < -PI) ang += period;
        }
        err = ang;
    } else if (!full && err >= upper) { clamp = 1; err -= upper; }
    else if (!full && err <= lower) { clamp = 2; err -= lower; }
    else { J.lim.w = 0.f; J.acc.x = 0.f; return; }
    J.lim.w = (float)clamp;
    acc = clamp_impulse(clamp, acc);
    float eff = row_mass(dot(sym_mul(sym_add(b1.I, b2.I), jr), jr), J.prm.y, sp);
    if (eff == 0.0f) acc = 0.f;
    J.acc.x = acc;
    J.bil.x = eff;
    J.bias.x = err * J.prm.x * sp.inv_dt;
    if (b1.flags & SB_DYNAMIC) { b1.w = b1.w + sym_mul(b1.I, acc * jr); store_vel(w.body, i1, b1); }
    if (b2.flags & SB_DYNAMIC) { b2.w = b2.w - sym_mul(b2.I, acc * jr); store_vel(w.body, i2, b2); }
}
// TwistAngle.IterateTwistAngle (TwistAngle.cs:296-323)
__device__ void twist_iterate(const WorldDev& w, JointDev& J, const StepParams& sp) {
    const int clamp = (int)J.lim.w;
    if (clamp == 0) return;
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    v3 jr = mk3(J.eff[0]);
    float jv = dot(b1.w - b2.w, jr);
    float soft = J.acc.x * (J.prm.y * sp.inv_sub_dt);
    float lambda = -J.bil.x * (jv + J.bias.x + soft);
    float old = J.acc.x;
    J.acc.x = clamp_impulse(clamp, J.acc.x + lambda);
    lambda = J.acc.x - old;
    if (b1.flags & SB_DYNAMIC) { b1.w = b1.w + sym_mul(b1.I, lambda * jr); store_vel(w.body, i1, b1); }
    if (b2.flags & SB_DYNAMIC) { b2.w = b2.w - sym_mul(b2.I, lambda * jr); store_vel(w.body, i2, b2); }
}

// ---- FixedAngle, PointOnPlane, AngularMotor, LinearMotor ------------------------------------
// FixedAngle.PrepareForIterationFixedAngle (FixedAngle.cs:87-128): three angular rows, the
// Jacobian -2 x the rotation-log derivative of Q0 conj(q1) q2 (q0), softness prm.y, bias
// factor prm.x; Jacobian in jac[0..2], inverse effective mass in eff[0..2], hemisphere bil.w
__device__ void fixed_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    v3 err;
    int hemi;
    M3x m = calc_jacobian(qmul(mkq(J.q0), qconj(mkq(w.q[i1]))), mkq(w.q[i2]), err, hemi);
    M3x jac;
    for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) jac.a[i][k] = -2.0f * m.a[i][k];
    v3 acc = mk3(J.acc);
    int old_hemi = (int)J.bil.w;
    if (old_hemi != 0 && old_hemi != hemi) acc = mk3(0.f);
    M3x eff = sym_transform_full(sym_add(b1.I, b2.I), jac);
    float soft = J.prm.y * sp.inv_sub_dt;
    eff.a[0][0] += soft; eff.a[1][1] += soft; eff.a[2][2] += soft;
    eff = inv_symmetric(eff);
    v3 bias = (-err) * J.prm.x * sp.inv_dt;
    v3 imp = mtv(jac, acc);
    if (b1.flags & SB_DYNAMIC) { b1.w = b1.w + sym_mul(b1.I, imp); store_vel(w.body, i1, b1); }
    if (b2.flags & SB_DYNAMIC) { b2.w = b2.w - sym_mul(b2.I, imp); store_vel(w.body, i2, b2); }
    J.acc = f4(acc, 0.f);
    J.bias = f4(bias, 0.f);
    jstore_m(J.eff, eff);
    jstore_m(J.jac, jac);
    J.bil = make_float4(0.f, 0.f, 0.f, (float)hemi);
}
// FixedAngle.IterateFixedAngle (FixedAngle.cs:159-181)
__device__ void fixed_iterate(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    M3x jac = jload_m(J.jac), eff = jload_m(J.eff);
    v3 jv = mv(jac, b1.w - b2.w);
    v3 acc = mk3(J.acc);
    v3 soft = acc * (J.prm.y * sp.inv_sub_dt);
    v3 lambda = -1.0f * mv(eff, (jv + mk3(J.bias)) + soft);
    J.acc = f4(acc + lambda, 0.f);
    v3 imp = mtv(jac, lambda);
    if (b1.flags & SB_DYNAMIC) { b1.w = b1.w + sym_mul(b1.I, imp); store_vel(w.body, i1, b1); }
    if (b2.flags & SB_DYNAMIC) { b2.w = b2.w - sym_mul(b2.I, imp); store_vel(w.body, i2, b2); }
}

// PointOnPlane.PrepareForIterationPointOnPlane (PointOnPlane.cs:128-200): one row along the
// plane normal (axis, local to body 1), the arm of body 1 measured to the second anchor; the
// same row layout and iteration as DistanceLimit (PointOnPlane.cs:218-256)
__device__ void plane_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    q4 q1 = mkq(w.q[i1]), q2 = mkq(w.q[i2]);
    v3 axis = rotate(mk3(J.axis), q1);
    v3 r1 = rotate(mk3(J.la1), q1), r2 = rotate(mk3(J.la2), q2);
    v3 u = (mk3(w.pos[i2]) + r2) - (mk3(w.pos[i1]) + r1);
    v3 j0 = -axis, j1 = -cross(r1 + u, axis), j2 = axis, j3 = cross(r2, axis);
    J.eff[0] = f4(j0, 0.f); J.eff[1] = f4(j1, 0.f); J.eff[2] = f4(j2, 0.f); J.jac[0] = f4(j3, 0.f);
    float err = dot(u, axis);
    const float lo = J.lim.x, hi = J.lim.y;
    int clamp;
    if (lo >= hi) { err -= 0.5f * lo + 0.5f * hi; clamp = 3; }
    else if (err >= hi) { err -= hi; clamp = 1; }
    else if (err <= lo) { err -= lo; clamp = 2; }
    else { J.lim.w = 0.f; J.acc.x = 0.f; J.bil.x = 1.0f; return; }
    J.lim.w = (float)clamp;
    float m = dot(cmul(j0, b1.im), j0) + dot(cmul(j2, b2.im), j2) + dot(sym_mul(b1.I, j1), j1) + dot(sym_mul(b2.I, j3), j3);
    float eff = row_mass(m, J.prm.y, sp);
    if (eff == 0.0f) J.acc.x = 0.f;
    J.bil.x = eff;
    J.bias.x = err * J.prm.x * sp.inv_dt;
    const float a = J.acc.x;
    if (b1.flags & SB_DYNAMIC) {
        b1.v = b1.v + cmul(j0 * a, b1.im);
        b1.w = b1.w + sym_mul(b1.I, j1 * a);
        store_vel(w.body, i1, b1);
    }
    if (b2.flags & SB_DYNAMIC) {
        b2.v = b2.v + cmul(j2 * a, b2.im);
        b2.w = b2.w + sym_mul(b2.I, j3 * a);
        store_vel(w.body, i2, b2);
    }
}

// AngularMotor (AngularMotor.cs:128-180) and LinearMotor (LinearMotor.cs:152-231): a velocity
// drive about (along) an axis of each body (la1, la2 local); lim = (impulse limit of the
// substep, maximum torque or force, target velocity); the world axes in eff[0], eff[1], the
// effective mass in bil.x, the accumulated impulse in acc.x
__device__ __forceinline__ float motor_response(const LBody& b, v3 a, bool linear) {
    return linear ? dot(cmul(a, b.im), a) : dot(sym_mul(b.I, a), a);
}
__device__ __forceinline__ void motor_push(LBody& b, v3 imp, bool linear) {
    if (linear) b.v = b.v + cmul(imp, b.im);
    else b.w = b.w + sym_mul(b.I, imp);
}
__device__ void motor_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    const bool lin = J.hdr.x == JG_CONSTRAINT_LINEARMOTOR;
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    v3 j1 = rotate(mk3(J.la1), mkq(w.q[i1])), j2 = rotate(mk3(J.la2), mkq(w.q[i2]));
    float m = motor_response(b1, j1, lin) + motor_response(b2, j2, lin);
    float eff = m > 0 ? 1.0f / m : 0.0f;
    if (eff == 0.0f) J.acc.x = 0.f;
    J.bil.x = eff;
    J.lim.x = sp.sub_dt * J.lim.y;
    J.eff[0] = f4(j1, 0.f); J.eff[1] = f4(j2, 0.f);
    const float a = J.acc.x;
    if (b1.flags & SB_DYNAMIC) { motor_push(b1, -(j1 * a), lin); store_vel(w.body, i1, b1); }
    if (b2.flags & SB_DYNAMIC) { motor_push(b2, j2 * a, lin); store_vel(w.body, i2, b2); }
}
__device__ void motor_iterate(const WorldDev& w, JointDev& J, const StepParams& sp) {
    const bool lin = J.hdr.x == JG_CONSTRAINT_LINEARMOTOR;
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    v3 j1 = mk3(J.eff[0]), j2 = mk3(J.eff[1]);
    float jv = lin ? dot(-j1, b1.v) + dot(j2, b2.v) : dot(-j1, b1.w) + dot(j2, b2.w);
    float lambda = -(jv - J.lim.z) * J.bil.x;
    float old = J.acc.x;
    J.acc.x = fminf(fmaxf(J.acc.x + lambda, -J.lim.x), J.lim.x);
    lambda = J.acc.x - old;
    if (b1.flags & SB_DYNAMIC) { motor_push(b1, -(j1 * lambda), lin); store_vel(w.body, i1, b1); }
    if (b2.flags & SB_DYNAMIC) { motor_push(b2, j2 * lambda, lin); store_vel(w.body, i2, b2); }
}

// ---- servos: AngularServo, LinearServo, LinearAxisServo, TwistServo ------------------------
// ServoMath (Internal/ServoMath.cs:30-49): the impulse limit of a substep, and the clamps of a
// vector impulse (its length) and of an angular one (the length of J^T imp)
__device__ __forceinline__ float servo_max_impulse(float maximum, float dt) { return dt > 0.f ? maximum * dt : 0.f; }
__device__ __forceinline__ float net_clamp(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }
__device__ __forceinline__ bool pos_inf(float x) { return isinf(x) && x > 0.f; }
__device__ __forceinline__ v3 servo_clamp_magnitude(v3 imp, float maxi) {
    if (pos_inf(maxi)) return imp;
    const float l2 = dot(imp, imp);
    return l2 > maxi * maxi ? imp * (maxi / sqrtf(l2)) : imp;
}
__device__ __forceinline__ v3 servo_clamp_angular(v3 imp, const M3x& jac, float maxi) {
    if (pos_inf(maxi)) return imp;
    const v3 a = mtv(jac, imp);
    const float l2 = dot(a, a);
    return l2 > maxi * maxi ? imp * (maxi / sqrtf(l2)) : imp;
}

// AngularServo (AngularServo.cs:125-172): three angular rows towards the target relative
// orientation q0; Jacobian in jac[0..2], inverse effective mass in eff[0..2], maximum torque
// lim.y, hemisphere bil.w
__device__ void angular_servo_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    v3 err;
    int hemi;
    M3x m = calc_jacobian(qmul(qconj(mkq(J.q0)), qconj(mkq(w.q[i1]))), mkq(w.q[i2]), err, hemi);
    M3x jac;
    for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) jac.a[i][k] = -2.0f * m.a[i][k];
    v3 acc = mk3(J.acc);
    int old_hemi = (int)J.bil.w;
    if (old_hemi != 0 && old_hemi != hemi) acc = mk3(0.f);
    M3x eff = sym_transform_full(sym_add(b1.I, b2.I), jac);
    float soft = J.prm.y * sp.inv_sub_dt;
    eff.a[0][0] += soft; eff.a[1][1] += soft; eff.a[2][2] += soft;
    eff = inv_symmetric(eff);
    v3 bias = (-err) * J.prm.x * sp.inv_dt;
    acc = servo_clamp_angular(acc, jac, servo_max_impulse(J.lim.y, sp.sub_dt));
    v3 imp = mtv(jac, acc);
    if (b1.flags & SB_DYNAMIC) { b1.w = b1.w + sym_mul(b1.I, imp); store_vel(w.body, i1, b1); }
    if (b2.flags & SB_DYNAMIC) { b2.w = b2.w - sym_mul(b2.I, imp); store_vel(w.body, i2, b2); }
    J.acc = f4(acc, 0.f);
    J.bias = f4(bias, 0.f);
    jstore_m(J.eff, eff);
    jstore_m(J.jac, jac);
    J.bil = make_float4(0.f, 0.f, 0.f, (float)hemi);
}
__device__ void angular_servo_iterate(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    M3x jac = jload_m(J.jac), eff = jload_m(J.eff);
    v3 jv = mv(jac, b1.w - b2.w);
    v3 acc = mk3(J.acc);
    v3 soft = acc * (J.prm.y * sp.inv_sub_dt);
    v3 lambda = -1.0f * mv(eff, (jv + mk3(J.bias)) + soft);
    v3 next = servo_clamp_angular(acc + lambda, jac, servo_max_impulse(J.lim.y, sp.sub_dt));
    J.acc = f4(next, 0.f);
    v3 imp = mtv(jac, next - acc);
    if (b1.flags & SB_DYNAMIC) { b1.w = b1.w + sym_mul(b1.I, imp); store_vel(w.body, i1, b1); }
    if (b2.flags & SB_DYNAMIC) { b2.w = b2.w - sym_mul(b2.I, imp); store_vel(w.body, i2, b2); }
}

// LinearServo (LinearServo.cs:149-201): three linear rows pulling anchor 2 to anchor 1 offset
// by the target (axis, body 1's frame); arms in r1, r2, inverse effective mass in eff[0..2],
// maximum force lim.y
__device__ __forceinline__ void linear_servo_apply(const WorldDev& w, const JointDev& J, LBody& b1, LBody& b2, v3 r1,
                                                   v3 r2, v3 imp) {
    if (b1.flags & SB_DYNAMIC) {
        b1.v = b1.v - cmul(imp, b1.im);
        b1.w = b1.w - sym_mul(b1.I, cross(r1, imp));
        store_vel(w.body, J.hdr.y, b1);
    }
    if (b2.flags & SB_DYNAMIC) {
        b2.v = b2.v + cmul(imp, b2.im);
        b2.w = b2.w + sym_mul(b2.I, cross(r2, imp));
        store_vel(w.body, J.hdr.z, b2);
    }
}
__device__ void linear_servo_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    q4 q1 = mkq(w.q[i1]), q2 = mkq(w.q[i2]);
    v3 r1 = rotate(mk3(J.la1) + mk3(J.axis), q1), r2 = rotate(mk3(J.la2), q2);
    M3x cr1 = mskew(r1), cr2 = mskew(r2);
    M3x t1 = sym_transform_full(b1.I, cr1), t2 = sym_transform_full(b2.I, cr2);
    // ((Scale(m1) + T1) + Scale(m2)) + T2, component-wise, in the reference's order
    M3x e;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) e.a[i][j] = t1.a[i][j] + t2.a[i][j];
    e.a[0][0] = ((b1.im.x + t1.a[0][0]) + b2.im.x) + t2.a[0][0];
    e.a[1][1] = ((b1.im.y + t1.a[1][1]) + b2.im.y) + t2.a[1][1];
    e.a[2][2] = ((b1.im.z + t1.a[2][2]) + b2.im.z) + t2.a[2][2];
    float soft = J.prm.y * sp.inv_sub_dt;
    e.a[0][0] += soft; e.a[1][1] += soft; e.a[2][2] += soft;
    jstore_m(J.eff, inv_symmetric(e));
    v3 bias = (((mk3(w.pos[i2]) + r2) - mk3(w.pos[i1])) - r1) * (J.prm.x * sp.inv_dt);
    v3 acc = servo_clamp_magnitude(mk3(J.acc), servo_max_impulse(J.lim.y, sp.sub_dt));
    linear_servo_apply(w, J, b1, b2, r1, r2, acc);
    J.r1 = f4(r1, 0.f); J.r2 = f4(r2, 0.f);
    J.acc = f4(acc, 0.f);
    J.bias = f4(bias, 0.f);
}
__device__ void linear_servo_iterate(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    v3 r1 = mk3(J.r1), r2 = mk3(J.r2);
    v3 jv = ((-b1.v - cross(b1.w, r1)) + b2.v) + cross(b2.w, r2);
    v3 acc = mk3(J.acc);
    v3 soft = acc * (J.prm.y * sp.inv_sub_dt);
    v3 lambda = -1.0f * mv(jload_m(J.eff), (jv + mk3(J.bias)) + soft);
    v3 next = servo_clamp_magnitude(acc + lambda, servo_max_impulse(J.lim.y, sp.sub_dt));
    J.acc = f4(next, 0.f);
    linear_servo_apply(w, J, b1, b2, r1, r2, next - acc);
}

// LinearAxisServo (LinearAxisServo.cs:169-224): one row along an axis of body 1 (axis, local),
// target position lim.z, maximum force lim.y; Jacobian blocks in eff[0..2] and jac[0], the
// effective mass in bil.x
__device__ __forceinline__ void axis_servo_apply(const WorldDev& w, const JointDev& J, LBody& b1, LBody& b2, float a) {
    if (b1.flags & SB_DYNAMIC) {
        b1.v = b1.v + cmul(mk3(J.eff[0]) * a, b1.im);
        b1.w = b1.w + sym_mul(b1.I, mk3(J.eff[1]) * a);
        store_vel(w.body, J.hdr.y, b1);
    }
    if (b2.flags & SB_DYNAMIC) {
        b2.v = b2.v + cmul(mk3(J.eff[2]) * a, b2.im);
        b2.w = b2.w + sym_mul(b2.I, mk3(J.jac[0]) * a);
        store_vel(w.body, J.hdr.z, b2);
    }
}
__device__ void linear_axis_servo_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    q4 q1 = mkq(w.q[i1]), q2 = mkq(w.q[i2]);
    v3 axis = rotate(mk3(J.axis), q1);
    v3 r1 = rotate(mk3(J.la1), q1), r2 = rotate(mk3(J.la2), q2);
    v3 sep = ((mk3(w.pos[i2]) + r2) - mk3(w.pos[i1])) - r1;
    v3 j0 = -axis, j1 = -cross(r1 + sep, axis), j2 = axis, j3 = cross(r2, axis);
    J.eff[0] = f4(j0, 0.f); J.eff[1] = f4(j1, 0.f); J.eff[2] = f4(j2, 0.f); J.jac[0] = f4(j3, 0.f);
    float m = dot(cmul(j0, b1.im), j0) + dot(cmul(j2, b2.im), j2) + dot(sym_mul(b1.I, j1), j1) + dot(sym_mul(b2.I, j3), j3) +
              J.prm.y * sp.inv_sub_dt;
    float eff = m > 0.f ? 1.0f / m : 0.0f;
    float acc = eff == 0.0f ? 0.0f : J.acc.x;
    J.bil.x = eff;
    J.bias.x = (dot(sep, axis) - J.lim.z) * J.prm.x * sp.inv_dt;
    const float maxi = servo_max_impulse(J.lim.y, sp.sub_dt);
    acc = net_clamp(acc, -maxi, maxi);
    J.acc.x = acc;
    axis_servo_apply(w, J, b1, b2, acc);
}
__device__ void linear_axis_servo_iterate(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    float jv = dot(mk3(J.eff[0]), b1.v) + dot(mk3(J.eff[1]), b1.w) + dot(mk3(J.eff[2]), b2.v) + dot(mk3(J.jac[0]), b2.w);
    float lambda = -(jv + J.bias.x + J.acc.x * J.prm.y * sp.inv_sub_dt) * J.bil.x;
    const float prev = J.acc.x, maxi = servo_max_impulse(J.lim.y, sp.sub_dt);
    J.acc.x = net_clamp(prev + lambda, -maxi, maxi);
    axis_servo_apply(w, J, b1, b2, J.acc.x - prev);
}

// TwistServo (TwistServo.cs:150-192): the twist about body 2's axis (axis, local) towards the
// target angle lim.z, reference rotation q0, maximum torque lim.y; Jacobian row jac[0],
// effective mass bil.x, hemisphere bil.w
__device__ __forceinline__ void twist_servo_apply(const WorldDev& w, const JointDev& J, LBody& b1, LBody& b2, float a) {
    const v3 jr = mk3(J.jac[0]);
    if (b1.flags & SB_DYNAMIC) { b1.w = b1.w + sym_mul(b1.I, jr * a); store_vel(w.body, J.hdr.y, b1); }
    if (b2.flags & SB_DYNAMIC) { b2.w = b2.w - sym_mul(b2.I, jr * a); store_vel(w.body, J.hdr.z, b2); }
}
__device__ void twist_servo_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    v3 jr;
    int hemi;
    float angle = calc_twist(qmul(mkq(J.q0), qconj(mkq(w.q[i1]))), mkq(w.q[i2]), mk3(J.axis), jr, hemi);
    float acc = J.acc.x;
    int old_hemi = (int)J.bil.w;
    if (old_hemi != 0 && old_hemi != hemi) acc = 0.f;
    float m = dot(sym_mul(sym_add(b1.I, b2.I), jr), jr) + J.prm.y * sp.inv_sub_dt;
    float eff = m > 0.f ? 1.0f / m : 0.0f;
    if (eff == 0.0f) acc = 0.f;
    J.jac[0] = f4(jr, 0.f);
    J.bil = make_float4(eff, 0.f, 0.f, (float)hemi);
    float error = angle - J.lim.z;
    J.bias.x = error * J.prm.x * sp.inv_dt;
    const float maxi = servo_max_impulse(J.lim.y, sp.sub_dt);
    acc = net_clamp(acc, -maxi, maxi);
    J.acc.x = acc;
    twist_servo_apply(w, J, b1, b2, acc);
}
__device__ void twist_servo_iterate(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    float jv = dot(b1.w - b2.w, mk3(J.jac[0]));
    float lambda = -J.bil.x * (jv + J.bias.x + J.acc.x * J.prm.y * sp.inv_sub_dt);
    const float prev = J.acc.x, maxi = servo_max_impulse(J.lim.y, sp.sub_dt);
    J.acc.x = net_clamp(prev + lambda, -maxi, maxi);
    twist_servo_apply(w, J, b1, b2, J.acc.x - prev);
}

// ---- PointOnLine (PointOnLine.cs:149-465) ------------------------------------------------------
// Math.Min / Math.Max as .NET defines them for floating point: NaN wins, and of two equal
// values Min returns the negative zero, Max the positive one
__device__ __forceinline__ float net_min(float a, float b) {
    if (a != b) return isnan(a) ? a : (a < b ? a : b);
    return signbit(b) ? b : a;
}
__device__ __forceinline__ float net_max(float a, float b) {
    if (a != b) return isnan(a) ? a : (a > b ? a : b);
    return signbit(b) ? a : b;
}
// The twelve Jacobian blocks (two rows across the line and one along it, each for v1, w1,
// v2, w2) and the error, from the current poses (PointOnLine.cs:155-185, :378-408); the line's
// direction (axis) and anchors (la1, la2) are local
__device__ __forceinline__ v3 line_jacobian(const WorldDev& w, const JointDev& J, v3* jb) {
    const int i1 = J.hdr.y, i2 = J.hdr.z;
    const q4 q1 = mkq(w.q[i1]), q2 = mkq(w.q[i2]);
    const v3 aw = rotate(mk3(J.axis), q1);
    const v3 n1 = rotate(create_orthonormal(mk3(J.axis)), q1);
    const v3 n2 = cross(aw, n1);
    const v3 r1 = rotate(mk3(J.la1), q1), r2 = rotate(mk3(J.la2), q2);
    const v3 p1 = mk3(w.pos[i1]) + r1, p2 = mk3(w.pos[i2]) + r2;
    const v3 u = p2 - p1;
    jb[0] = -n1; jb[1] = -cross(r1 + u, n1); jb[2] = n1; jb[3] = cross(r2, n1);
    jb[4] = -n2; jb[5] = -cross(r1 + u, n2); jb[6] = n2; jb[7] = cross(r2, n2);
    jb[8] = -aw; jb[9] = -cross(r1 + u, aw); jb[10] = aw; jb[11] = cross(r2, aw);
    return mk3(dot(u, n1), dot(u, n2), dot(u, aw));
}
__device__ __forceinline__ void line_apply(const WorldDev& w, const JointDev& J, LBody& b1, LBody& b2, const v3* jb, v3 a) {
    if (b1.flags & SB_DYNAMIC) {
        b1.v = b1.v + cmul(jb[0] * a.x + jb[4] * a.y + jb[8] * a.z, b1.im);
        b1.w = b1.w + sym_mul(b1.I, jb[1] * a.x + jb[5] * a.y + jb[9] * a.z);
        store_vel(w.body, J.hdr.y, b1);
    }
    if (b2.flags & SB_DYNAMIC) {
        b2.v = b2.v + cmul(jb[2] * a.x + jb[6] * a.y + jb[10] * a.z, b2.im);
        b2.w = b2.w + sym_mul(b2.I, jb[3] * a.x + jb[7] * a.y + jb[11] * a.z);
        store_vel(w.body, J.hdr.z, b2);
    }
}
// Prepare: prm = (bias, softness, limit bias, limit softness), lim = (min, max, -, clamp),
// inverse effective mass in eff[0..2], bilateral block inverse in bil, couplings in cpl
__device__ void line_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    LBody b1 = load_body(w.body, J.hdr.y), b2 = load_body(w.body, J.hdr.z);
    v3 jb[12];
    v3 err = line_jacobian(w, J, jb);
    const sym6 I1 = b1.I, I2 = b2.I;
    const v3 m1 = b1.im, m2 = b2.im;
    M3x M = mzero();
    M.a[0][0] = dot(cmul(jb[0], m1), jb[0]) + dot(cmul(jb[2], m2), jb[2]) + dot(sym_mul(I1, jb[1]), jb[1]) +
                dot(sym_mul(I2, jb[3]), jb[3]);
    M.a[1][1] = dot(cmul(jb[4], m1), jb[4]) + dot(cmul(jb[6], m2), jb[6]) + dot(sym_mul(I1, jb[5]), jb[5]) +
                dot(sym_mul(I2, jb[7]), jb[7]);
    M.a[2][2] = 1.0f;
    M.a[0][1] = dot(sym_mul(I1, jb[1]), jb[5]) + dot(sym_mul(I2, jb[3]), jb[7]);
    M.a[1][0] = dot(sym_mul(I1, jb[5]), jb[1]) + dot(sym_mul(I2, jb[7]), jb[3]);
    const float c12 = dot(cmul(jb[0], m1), jb[4]) + dot(cmul(jb[2], m2), jb[6]);
    M.a[0][1] += c12;
    M.a[1][0] += c12;
    v3 acc = mk3(J.acc);
    const float lo = J.lim.x, hi = J.lim.y;
    int clamp = 0;
    if (lo >= hi) { err.z -= 0.5f * lo + 0.5f * hi; clamp = 3; }
    else if (err.z >= hi) { err.z -= hi; clamp = 1; }
    else if (err.z <= lo) { err.z -= lo; clamp = 2; }
    else acc.z = 0.f;
    if (clamp != 0) {
        M.a[2][2] = dot(cmul(jb[8], m1), jb[8]) + dot(cmul(jb[10], m2), jb[10]) + dot(sym_mul(I1, jb[9]), jb[9]) +
                    dot(sym_mul(I2, jb[11]), jb[11]);
        M.a[0][2] = dot(sym_mul(I1, jb[1]), jb[9]) + dot(sym_mul(I2, jb[3]), jb[11]);
        M.a[2][0] = dot(sym_mul(I1, jb[9]), jb[1]) + dot(sym_mul(I2, jb[11]), jb[3]);
        M.a[1][2] = dot(sym_mul(I1, jb[5]), jb[9]) + dot(sym_mul(I2, jb[7]), jb[11]);
        M.a[2][1] = dot(sym_mul(I1, jb[9]), jb[5]) + dot(sym_mul(I2, jb[11]), jb[7]);
        const float c13 = dot(cmul(jb[0], m1), jb[8]) + dot(cmul(jb[2], m2), jb[10]);
        const float c23 = dot(cmul(jb[4], m1), jb[8]) + dot(cmul(jb[6], m2), jb[10]);
        M.a[0][2] += c13; M.a[2][0] += c13;
        M.a[1][2] += c23; M.a[2][1] += c23;
    }
    M.a[0][0] += J.prm.y * sp.inv_sub_dt;
    M.a[1][1] += J.prm.y * sp.inv_sub_dt;
    M.a[2][2] += J.prm.w * sp.inv_sub_dt;
    v3 bil = mk3(0.f);
    float cx = 0.f, cy = 0.f;
    if (clamp == 1 || clamp == 2) {
        M3x blk = mzero();
        blk.a[0][0] = M.a[0][0]; blk.a[0][1] = M.a[0][1]; blk.a[1][0] = M.a[0][1]; blk.a[1][1] = M.a[1][1];
        M3x bi = inv_symmetric(blk);
        bil = mk3(bi.a[0][0], bi.a[0][1], bi.a[1][1]);
        cx = M.a[0][2];
        cy = M.a[1][2];
    }
    if (clamp == 0) M.a[2][2] = 0.f;
    jstore_m(J.eff, inv_symmetric(M));
    v3 bias = err * sp.inv_dt;
    bias.x *= J.prm.x; bias.y *= J.prm.x; bias.z *= J.prm.z;
    if (clamp == 1) acc.z = net_min(0.f, acc.z);
    else if (clamp == 2) acc.z = net_max(0.f, acc.z);
    line_apply(w, J, b1, b2, jb, acc);
    J.acc = f4(acc, 0.f);
    J.bias = f4(bias, 0.f);
    J.lim.w = (float)clamp;
    J.bil = make_float4(bil.x, bil.y, bil.z, 0.f);
    J.cpl = make_float4(cx, cy, 0.f, 0.f);
}
__device__ void line_iterate(const WorldDev& w, JointDev& J, const StepParams& sp) {
    LBody b1 = load_body(w.body, J.hdr.y), b2 = load_body(w.body, J.hdr.z);
    v3 jb[12];
    line_jacobian(w, J, jb);
    v3 jv = mk3(dot(jb[0], b1.v) + dot(jb[1], b1.w) + dot(jb[2], b2.v) + dot(jb[3], b2.w),
                dot(jb[4], b1.v) + dot(jb[5], b1.w) + dot(jb[6], b2.v) + dot(jb[7], b2.w),
                dot(jb[8], b1.v) + dot(jb[9], b1.w) + dot(jb[10], b2.v) + dot(jb[11], b2.w));
    v3 acc = mk3(J.acc);
    v3 soft = acc * sp.inv_sub_dt;
    soft.x *= J.prm.y; soft.y *= J.prm.y; soft.z *= J.prm.w;
    v3 res = jv + mk3(J.bias) + soft;
    v3 lambda = -1.0f * mv(jload_m(J.eff), res);
    v3 orig = acc;
    acc = acc + lambda;
    const int clamp = (int)J.lim.w;
    if ((clamp == 1 && acc.z > 0) || (clamp == 2 && acc.z < 0)) {
        lambda.z = -orig.z;
        float x = res.x + J.cpl.x * lambda.z;
        float y = res.y + J.cpl.y * lambda.z;
        lambda.x = -(J.bil.x * x + J.bil.y * y);
        lambda.y = -(J.bil.y * x + J.bil.z * y);
        acc.x = orig.x + lambda.x;
        acc.y = orig.y + lambda.y;
        acc.z = 0;
    } else if (clamp == 0) {
        acc.z = 0;
        orig.z = 0;
    }
    J.acc = f4(acc, 0.f);
    line_apply(w, J, b1, b2, jb, acc - orig);
}

// ---- EllipticalConeLimit (EllipticalConeLimit.cs:257-429) -----------------------------------------
// la1, la2 the cone axes (local), axis body 1's reference direction (local), lim = (min1, max1,
// min2, max2), prm = (bias factor, softness); the Jacobian row in jac[0] and the clamp state in
// bil.w persist between steps, the effective mass is bil.x
__device__ __forceinline__ float ellipse_radius(float a, float b, float c, float s, float& derivative) {
    const float scale = net_min(a, b);
    const float u = scale / a, v = scale / b;
    const float sq = c * c * u * u + s * s * v * v;
    derivative = c * s * (v * v - u * u) / sq;
    return scale / sqrtf(sq);
}
__device__ __forceinline__ void elliptical_apply(const WorldDev& w, const JointDev& J, LBody& b1, LBody& b2, v3 jac, float a) {
    if (b1.flags & SB_DYNAMIC) { b1.w = b1.w + sym_mul(b1.I, a * jac); store_vel(w.body, J.hdr.y, b1); }
    if (b2.flags & SB_DYNAMIC) { b2.w = b2.w - sym_mul(b2.I, a * jac); store_vel(w.body, J.hdr.z, b2); }
}
__device__ void elliptical_prepare(const WorldDev& w, JointDev& J, const StepParams& sp) {
    int i1 = J.hdr.y, i2 = J.hdr.z;
    LBody b1 = load_body(w.body, i1), b2 = load_body(w.body, i2);
    const q4 q1 = mkq(w.q[i1]), q2 = mkq(w.q[i2]);
    const v3 axis = rotate(mk3(J.la1), q1);
    const v3 reference = rotate(mk3(J.axis), q1);
    const v3 other = cross(axis, reference);
    const v3 target = rotate(mk3(J.la2), q2);
    const float x = dot(target, reference), y = dot(target, other), z = dot(target, axis);
    const float sine = sqrtf(x * x + y * y);
    const float angle = StableMathF::atan2(sine, z);
    float ca, sa;
    if (sine > 0.f) {
        ca = x / sine;
        sa = y / sine;
    } else {
        // no unique direction at either pole: the principal direction with the more
        // responsive angular axis
        const sym6 I = sym_add(b1.I, b2.I);
        const bool use_ref = dot(sym_mul(I, other), other) >= dot(sym_mul(I, reference), reference);
        ca = use_ref ? 1.f : 0.f;
        sa = use_ref ? 0.f : 1.f;
    }
    float derivative;
    const float outer = ellipse_radius(J.lim.y, J.lim.w, ca, sa, derivative);
    const bool fixed_cone = J.lim.x == J.lim.y && J.lim.z == J.lim.w;
    float boundary = outer;
    int clamp = 0;
    if (fixed_cone) clamp = 3;
    else if (angle >= outer) clamp = 1;
    else if (J.lim.x > 0.f) {
        float inner_d;
        const float inner = ellipse_radius(J.lim.x, J.lim.z, ca, sa, inner_d);
        if (angle <= inner) {
            clamp = 2;
            boundary = inner;
            derivative = inner_d;
        }
    }
    const int previous = (int)J.bil.w;
    J.bil.w = (float)clamp;
    if (clamp == 0) {
        J.acc.x = 0.f;
        return;
    }
    const v3 tilt = ca * reference + sa * other;
    const v3 azimuth = cross(axis, tilt);
    const v3 angle_dir = z * tilt - sine * axis;
    const float az = sine > 0.f ? angle / sine * derivative : 0.f;
    const float scale = net_max(1.f, fabsf(az));
    v3 jac = (-azimuth) * (1.f / scale) + (az / scale) * angle_dir;
    float inv_len = 1.f / sqrtf(dot(jac, jac));
    jac = jac * inv_len;
    inv_len /= scale;
    float acc = J.acc.x;
    if (previous != clamp || dot(mk3(J.jac[0]), jac) < 0.f) acc = 0.f;
    J.jac[0] = f4(jac, 0.f);
    if (clamp == 1) acc = net_min(acc, 0.f);
    else if (clamp == 2) acc = net_max(acc, 0.f);
    const float mass = dot(sym_mul(b1.I, jac), jac) + dot(sym_mul(b2.I, jac), jac) + J.prm.y * sp.inv_sub_dt;
    const float eff = mass > 0.f ? 1.f / mass : 0.f;
    if (eff == 0.f) acc = 0.f;
    J.bil.x = eff;
    J.bias.x = (angle - boundary) * inv_len * J.prm.x * sp.inv_dt;
    J.acc.x = acc;
    elliptical_apply(w, J, b1, b2, jac, acc);
}
__device__ void elliptical_iterate(const WorldDev& w, JointDev& J, const StepParams& sp) {
    const int clamp = (int)J.bil.w;
    if (clamp == 0) return;
    LBody b1 = load_body(w.body, J.hdr.y), b2 = load_body(w.body, J.hdr.z);
    const v3 jac = mk3(J.jac[0]);
    const float jv = dot(b1.w - b2.w, jac);
    const float lambda = -J.bil.x * (jv + J.bias.x + J.acc.x * J.prm.y * sp.inv_sub_dt);
    const float old = J.acc.x;
    float acc = old + lambda;
    if (clamp == 1) acc = net_min(acc, 0.f);
    else if (clamp == 2) acc = net_max(acc, 0.f);
    J.acc.x = acc;
    elliptical_apply(w, J, b1, b2, jac, acc - old);
}

__device__ __forceinline__ void joint_prepare(const WorldDev& w, int j, const StepParams& sp) {
    JointDev& J = w.joints[j];
    switch (J.hdr.x) {
        case JG_CONSTRAINT_BALLSOCKET: ballsocket_prepare(w, J, sp); break;
        case JG_CONSTRAINT_HINGEANGLE: hinge_prepare(w, J, sp); break;
        case JG_CONSTRAINT_DISTANCELIMIT: distance_prepare(w, J, sp); break;
        case JG_CONSTRAINT_CONELIMIT: cone_prepare(w, J, sp); break;
        case JG_CONSTRAINT_FIXEDANGLE: fixed_prepare(w, J, sp); break;
        case JG_CONSTRAINT_POINTONPLANE: plane_prepare(w, J, sp); break;
        case JG_CONSTRAINT_ANGULARMOTOR: case JG_CONSTRAINT_LINEARMOTOR: motor_prepare(w, J, sp); break;
        case JG_CONSTRAINT_ANGULARSERVO: angular_servo_prepare(w, J, sp); break;
        case JG_CONSTRAINT_LINEARSERVO: linear_servo_prepare(w, J, sp); break;
        case JG_CONSTRAINT_LINEARAXISSERVO: linear_axis_servo_prepare(w, J, sp); break;
        case JG_CONSTRAINT_TWISTSERVO: twist_servo_prepare(w, J, sp); break;
        case JG_CONSTRAINT_POINTONLINE: line_prepare(w, J, sp); break;
        case JG_CONSTRAINT_ELLIPTICALCONELIMIT: elliptical_prepare(w, J, sp); break;
        default: twist_prepare(w, J, sp); break;
    }
}
__device__ __forceinline__ void joint_iterate(const WorldDev& w, int j, const StepParams& sp) {
    JointDev& J = w.joints[j];
    switch (J.hdr.x) {
        case JG_CONSTRAINT_BALLSOCKET: ballsocket_iterate(w, J, sp); break;
        case JG_CONSTRAINT_HINGEANGLE: hinge_iterate(w, J, sp); break;
        case JG_CONSTRAINT_DISTANCELIMIT: distance_iterate(w, J, sp); break;
        case JG_CONSTRAINT_CONELIMIT: cone_iterate(w, J, sp); break;
        case JG_CONSTRAINT_FIXEDANGLE: fixed_iterate(w, J, sp); break;
        case JG_CONSTRAINT_POINTONPLANE: distance_iterate(w, J, sp); break;
        case JG_CONSTRAINT_ANGULARMOTOR: case JG_CONSTRAINT_LINEARMOTOR: motor_iterate(w, J, sp); break;
        case JG_CONSTRAINT_ANGULARSERVO: angular_servo_iterate(w, J, sp); break;
        case JG_CONSTRAINT_LINEARSERVO: linear_servo_iterate(w, J, sp); break;
        case JG_CONSTRAINT_LINEARAXISSERVO: linear_axis_servo_iterate(w, J, sp); break;
        case JG_CONSTRAINT_TWISTSERVO: twist_servo_iterate(w, J, sp); break;
        case JG_CONSTRAINT_POINTONLINE: line_iterate(w, J, sp); break;
        case JG_CONSTRAINT_ELLIPTICALCONELIMIT: elliptical_iterate(w, J, sp); break;
        default: twist_iterate(w, J, sp); break;
    }
}
