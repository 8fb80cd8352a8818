// Oracle (test infrastructure only): CPU restatement of the joint kinds on the device:
// BallSocket (Dynamics/Constraints/BallSocket.cs:140-252), HingeAngle
// (Dynamics/Constraints/HingeAngle.cs:84-364), DistanceLimit (DistanceLimit.cs:92-391),
// ConeLimit (ConeLimit.cs:92-404), TwistAngle (TwistAngle.cs:85-323), FixedAngle, PointOnPlane,
// the motors, the servos (AngularServo, LinearServo, LinearAxisServo, TwistServo) and
// PointOnLine and EllipticalConeLimit, with their math
// helpers (AngularConstraintMath.cs:13-95, QMatrix.cs:112-125, MathHelper.cs:282-372,
// JMatrix.cs:391-478, JQuaternion.cs:84-101).
#pragma once
#include "jor_dynamics.hpp"

namespace jor {

template <class R> struct Mat {
    R a[3][3];
    Mat() { for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) a[i][j] = 0; }
    static Mat ident() { Mat m; m.a[0][0] = m.a[1][1] = m.a[2][2] = 1; return m; }
    static Mat skew(V3<R> v) { Mat m; m.a[0][1] = -v.z; m.a[0][2] = v.y; m.a[1][0] = v.z; m.a[1][2] = -v.x; m.a[2][0] = -v.y; m.a[2][1] = v.x; return m; }
    static Mat from_sym(const Sym3<R>& s) {
        Mat m;
        m.a[0][0] = s.m11; m.a[0][1] = s.m12; m.a[0][2] = s.m13;
        m.a[1][0] = s.m12; m.a[1][1] = s.m22; m.a[1][2] = s.m23;
        m.a[2][0] = s.m13; m.a[2][1] = s.m23; m.a[2][2] = s.m33;
        return m;
    }
    static Mat from_m3(const M3<R>& s) { Mat m; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) m.a[i][j] = s.m[i][j]; return m; }
};
// JMatrix.Multiply (JMatrix.cs:156-180)
template <class R> Mat<R> mmul(const Mat<R>& x, const Mat<R>& y) {
    Mat<R> o;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) o.a[i][j] = x.a[i][0] * y.a[0][j] + x.a[i][1] * y.a[1][j] + x.a[i][2] * y.a[2][j];
    return o;
}
template <class R> Mat<R> madd(const Mat<R>& x, const Mat<R>& y) { Mat<R> o; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.a[i][j] = x.a[i][j] + y.a[i][j]; return o; }
template <class R> Mat<R> msub(const Mat<R>& x, const Mat<R>& y) { Mat<R> o; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.a[i][j] = x.a[i][j] - y.a[i][j]; return o; }
template <class R> Mat<R> mscale(R s, const Mat<R>& x) { Mat<R> o; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.a[i][j] = s * x.a[i][j]; return o; }
template <class R> Mat<R> mtrans(const Mat<R>& x) { Mat<R> o; for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.a[i][j] = x.a[j][i]; return o; }
template <class R> V3<R> mvec(const Mat<R>& M, V3<R> v) {
    return {v.x * M.a[0][0] + v.y * M.a[0][1] + v.z * M.a[0][2], v.x * M.a[1][0] + v.y * M.a[1][1] + v.z * M.a[1][2],
            v.x * M.a[2][0] + v.y * M.a[2][1] + v.z * M.a[2][2]};
}
template <class R> V3<R> mtvec(const Mat<R>& M, V3<R> v) {
    return {v.x * M.a[0][0] + v.y * M.a[1][0] + v.z * M.a[2][0], v.x * M.a[0][1] + v.y * M.a[1][1] + v.z * M.a[2][1],
            v.x * M.a[0][2] + v.y * M.a[1][2] + v.z * M.a[2][2]};
}
// JMatrix.Determinant (JMatrix.cs:391-395)
template <class R> R mdet(const Mat<R>& m) {
    const auto& a = m.a;
    return a[0][0] * a[1][1] * a[2][2] + a[0][1] * a[1][2] * a[2][0] + a[0][2] * a[1][0] * a[2][1] -
           a[2][0] * a[1][1] * a[0][2] - a[2][1] * a[1][2] * a[0][0] - a[2][2] * a[1][0] * a[0][1];
}
template <class R> bool mfinite(const Mat<R>& m) { for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) if (!std::isfinite(m.a[i][j])) return false; return true; }
// JMatrix.TryInverseUnscaled (JMatrix.cs:448-480)
template <class R> bool minv_unscaled(const Mat<R>& m, Mat<R>& o) {
    R idet = (R)1.0 / mdet(m);
    if (!std::isnormal(idet)) { o = Mat<R>(); return false; }
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
    return mfinite(o);
}
// JMatrix.Inverse (JMatrix.cs:404-437)
template <class R> bool minv(const Mat<R>& m, Mat<R>& o) {
    if (minv_unscaled(m, o)) return true;
    R s = 0;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) s = std::max(s, std::abs(m.a[i][j]));
    if (s > 0 && std::isfinite(s)) {
        Mat<R> n;
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) n.a[i][j] = m.a[i][j] / s;
        if (minv_unscaled(n, o)) {
            for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.a[i][j] /= s;
            if (mfinite(o)) return true;
        }
    }
    o = Mat<R>();
    return false;
}
template <class R> R tol() { return sizeof(R) == 8 ? (R)1e-12 : (R)1e-6; }
// MathHelper.JacobiRotate (MathHelper.cs:374-406)
template <class R> bool jacobi_rotate(R* a, R* basis, int p, int q, R t) {
    R off = a[3 * p + q];
    if (std::abs(off) <= t) return false;
    R tau = (a[3 * q + q] - a[3 * p + p]) / ((R)2.0 * off);
    R tg = std::copysign((R)1.0, tau) / (std::abs(tau) + std::sqrt((R)1.0 + tau * tau));
    R cs = (R)1.0 / std::sqrt((R)1.0 + tg * tg);
    R sn = tg * cs;
    a[3 * p + p] -= tg * off;
    a[3 * q + q] += tg * off;
    a[3 * p + q] = a[3 * q + p] = 0;
    for (int k = 0; k < 3; k++) {
        if (k != p && k != q) {
            R akp = a[3 * k + p], akq = a[3 * k + q];
            a[3 * k + p] = a[3 * p + k] = cs * akp - sn * akq;
            a[3 * k + q] = a[3 * q + k] = sn * akp + cs * akq;
        }
        R vkp = basis[3 * k + p], vkq = basis[3 * k + q];
        basis[3 * k + p] = cs * vkp - sn * vkq;
        basis[3 * k + q] = sn * vkp + cs * vkq;
    }
    return true;
}
// MathHelper.PseudoInverseSymmetric (MathHelper.cs:282-325)
template <class R> Mat<R> pinv_sym(const Mat<R>& m) {
    R s = std::max(std::abs(m.a[0][0]), std::max(std::abs(m.a[1][1]), std::abs(m.a[2][2])));
    if (!(s > 0) || !std::isfinite(s)) return Mat<R>();
    Sym3<R> n(m.a[0][0] / s, m.a[0][1] / s, m.a[0][2] / s, m.a[1][1] / s, m.a[1][2] / s, m.a[2][2] / s);
    R t = tol<R>();
    Mat<R> inv;
    if (std::abs(sym_det(n)) > t && minv(m, inv)) return inv;
    R a[9] = {n.m11, n.m12, n.m13, n.m12, n.m22, n.m23, n.m13, n.m23, n.m33};
    R basis[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int sw = 0; sw < 8; sw++) {
        bool ch = jacobi_rotate(a, basis, 0, 1, t);
        ch |= jacobi_rotate(a, basis, 0, 2, t);
        ch |= jacobi_rotate(a, basis, 1, 2, t);
        if (!ch) break;
    }
    Sym3<R> r;
    for (int i = 0; i < 3; i++) {
        R ev = a[3 * i + i];
        if (!(ev > t)) continue;
        R wgt = ((R)1.0 / ev) / s;
        V3<R> ax(basis[i], basis[3 + i], basis[6 + i]);
        r.m11 += wgt * (ax.x * ax.x); r.m12 += wgt * (ax.x * ax.y); r.m13 += wgt * (ax.x * ax.z);
        r.m22 += wgt * (ax.y * ax.y); r.m23 += wgt * (ax.y * ax.z); r.m33 += wgt * (ax.z * ax.z);
    }
    return Mat<R>::from_sym(r);
}
// MathHelper.InverseSymmetric (MathHelper.cs:328-365)
template <class R> Mat<R> inverse_symmetric(const Mat<R>& m) {
    R t = tol<R>();
    R dp = m.a[0][0] * m.a[1][1] * m.a[2][2];
    Mat<R> inv;
    if (mdet(m) / dp > t && minv(m, inv)) return inv;
    R x = m.a[0][0] > 0 ? std::sqrt(m.a[0][0]) : 0;
    R y = m.a[1][1] > 0 ? std::sqrt(m.a[1][1]) : 0;
    R z = m.a[2][2] > 0 ? std::sqrt(m.a[2][2]) : 0;
    if (x == 0 && y == 0 && z == 0) return Mat<R>();
    R xy = x > 0 && y > 0 ? m.a[0][1] / x / y : 0;
    R xz = x > 0 && z > 0 ? m.a[0][2] / x / z : 0;
    R yz = y > 0 && z > 0 ? m.a[1][2] / y / z : 0;
    Mat<R> nrm;
    nrm.a[0][0] = 1; nrm.a[0][1] = xy; nrm.a[0][2] = xz;
    nrm.a[1][0] = xy; nrm.a[1][1] = 1; nrm.a[1][2] = yz;
    nrm.a[2][0] = xz; nrm.a[2][1] = yz; nrm.a[2][2] = 1;
    Mat<R> resp = pinv_sym(nrm);
    xy = x > 0 && y > 0 ? resp.a[0][1] / x / y : 0;
    xz = x > 0 && z > 0 ? resp.a[0][2] / x / z : 0;
    yz = y > 0 && z > 0 ? resp.a[1][2] / y / z : 0;
    Mat<R> r;
    r.a[0][0] = x > 0 ? resp.a[0][0] / x / x : 0; r.a[0][1] = xy; r.a[0][2] = xz;
    r.a[1][0] = xy; r.a[1][1] = y > 0 ? resp.a[1][1] / y / y : 0; r.a[1][2] = yz;
    r.a[2][0] = xz; r.a[2][1] = yz; r.a[2][2] = z > 0 ? resp.a[2][2] / z / z : 0;
    return mfinite(r) ? r : Mat<R>();
}
// MathHelper.InverseBilateralBlock (MathHelper.cs:367-372)
template <class R> V3<R> inverse_bilateral(const Mat<R>& m) {
    Mat<R> b;
    b.a[0][0] = m.a[0][0]; b.a[0][1] = m.a[0][1]; b.a[1][0] = m.a[0][1]; b.a[1][1] = m.a[1][1];
    Mat<R> inv = inverse_symmetric(b);
    return V3<R>(inv.a[0][0], inv.a[0][1], inv.a[1][1]);
}
// AngularConstraintMath.ShortestAngle (AngularConstraintMath.cs:13-21)
template <class R> R shortest_angle(R angle, R half) {
    if (angle >= -half && angle <= half) return angle;
    R period = (R)2 * half;
    angle = std::fmod(angle, period);
    if (angle > half) angle -= period;
    else if (angle < -half) angle += period;
    return angle;
}
// AngularConstraintMath.CalculateJacobian (AngularConstraintMath.cs:65-95)
template <class R> Mat<R> calc_jacobian(Q4<R> left, Q4<R> right, V3<R>& err, short& hemi) {
    Q4<R> q = qmul(left, right);
    hemi = q.w < 0 ? (short)-1 : (short)1;
    if (q.w < 0) q = Q4<R>(-q.x, -q.y, -q.z, -q.w);
    V3<R> qv(q.x, q.y, q.z);
    R sine = std::sqrt(len2(qv));
    Mat<R> der;
    if (sine > 0) {
        R half = StableMath<R>::atan2(sine, q.w);
        V3<R> ax = qv * ((R)1 / sine);
        err = ax * half;
        R diag = half * q.w / sine;
        Sym3<R> outer(ax.x * ax.x, ax.x * ax.y, ax.x * ax.z, ax.y * ax.y, ax.y * ax.z, ax.z * ax.z);
        der = msub(madd(mscale(diag, Mat<R>::ident()), mscale((R)1 - diag, Mat<R>::from_sym(outer))), Mat<R>::skew(err));
    } else {
        err = V3<R>();
        der = Mat<R>::ident();
    }
    return mmul(mscale(-(R)0.5, der), Mat<R>::from_m3(mat_from_quat(left)));
}

enum JointKind { BALLSOCKET = 1, HINGEANGLE = 2, DISTANCELIMIT = 3, CONELIMIT = 4, TWISTANGLE = 5, FIXEDANGLE = 6,
                 POINTONPLANE = 7, ANGULARMOTOR = 8, LINEARMOTOR = 9, ANGULARSERVO = 10, LINEARSERVO = 11,
                 LINEARAXISSERVO = 12, TWISTSERVO = 13, POINTONLINE = 14, ELLIPTICALCONELIMIT = 15 };
template <class R> struct Joint {
    int kind = BALLSOCKET;
    int b1 = 0, b2 = 0;
    int color = 0;
    // BallSocketData (BallSocket.cs:32-60)
    V3<R> la1, la2, r1, r2, acc, bias;
    R bias_factor = (R)0.2, softness = (R)0.00001;
    Mat<R> eff;
    // HingeAngleData (HingeAngle.cs:32-70)
    R min_angle = 0, max_angle = 0, fixed_angle = 0, limit_bias = (R)0.1, limit_softness = (R)0.001;
    V3<R> axis;
    Q4<R> q0;
    Mat<R> jac;
    V3<R> bilateral;
    R coupling_x = 0, coupling_y = 0;
    int clamp = 0;
    short hemisphere = 0;
    // one-row kinds (DistanceLimitData, ConeLimitData, TwistLimitData): limits in
    // min_angle / max_angle (and fixed_angle), the row's Jacobian blocks, its effective mass;
    // the accumulated impulse and bias in acc.x / bias.x
    R target = 0;                     // DistanceLimit.Distance; a servo's target position or angle
    V3<R> jr[4];
    R eff1 = 0;
    // servos (AngularServoData, LinearServoData, LinearAxisServoData, TwistServoData):
    // MaximumTorque / MaximumForce, LinearServo.TargetPosition
    R maximum = 0;
    V3<R> target_pos;
    // EllipticalConeLimitData: MinAngle2 / MaxAngle2 (the first pair in min_angle / max_angle),
    // LocalReference1 (in target_pos), the Jacobian kept from the last Prepare (jr[0])
    R min_angle2 = 0, max_angle2 = 0;
};

// BallSocket.Initialize (BallSocket.cs:120-138)
template <class R> void ballsocket_init(Joint<R>& j, const std::vector<Body<R>>& b, V3<R> anchor) {
    j.kind = BALLSOCKET;
    j.la1 = rotate_inv(anchor - b[j.b1].pos, b[j.b1].q);
    j.la2 = rotate_inv(anchor - b[j.b2].pos, b[j.b2].q);
    j.bias_factor = (R)0.2;
    j.softness = (R)0.00001;
}
// HingeAngle.Initialize (HingeAngle.cs:84-110)
template <class R> void hinge_init(Joint<R>& j, const std::vector<Body<R>>& b, V3<R> axis, R from, R to) {
    j.kind = HINGEANGLE;
    j.softness = (R)0.001; j.limit_softness = (R)0.001;
    j.bias_factor = (R)0.2; j.limit_bias = (R)0.1;
    j.min_angle = from / (R)2.0;
    j.max_angle = to / (R)2.0;
    j.fixed_angle = (R)0.25 * from + (R)0.25 * to;
    axis = normalize(axis);
    j.axis = rotate_inv(axis, b[j.b2].q);
    j.q0 = qmul(qconj(b[j.b2].q), b[j.b1].q);
}

// ((Scale(m1) + Transform(I1, [r1]x)) + Scale(m2)) + Transform(I2, [r2]x), component-wise
// in the reference's left-to-right order (BallSocket.cs:158-161)
template <class R> Mat<R> ballsocket_mass(const Body<R>& b1, V3<R> r1, const Body<R>& b2, V3<R> r2) {
    auto tr = [](const Body<R>& bd, V3<R> r) {
        Mat<R> cr = Mat<R>::skew(r);
        M3<R> c3;
        for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) c3.m[i][k] = cr.a[i][k];
        return sym_transform(bd.inv_inertia_world, c3);
    };
    Sym3<R> t1 = tr(b1, r1), t2 = tr(b2, r2);
    Sym3<R> o;
    o.m11 = ((b1.inv_mass_vec.x + t1.m11) + b2.inv_mass_vec.x) + t2.m11;
    o.m12 = ((0 + t1.m12) + 0) + t2.m12;
    o.m13 = ((0 + t1.m13) + 0) + t2.m13;
    o.m22 = ((b1.inv_mass_vec.y + t1.m22) + b2.inv_mass_vec.y) + t2.m22;
    o.m23 = ((0 + t1.m23) + 0) + t2.m23;
    o.m33 = ((b1.inv_mass_vec.z + t1.m33) + b2.inv_mass_vec.z) + t2.m33;
    return Mat<R>::from_sym(o);
}

// BallSocket.PrepareForIterationBallSocket (BallSocket.cs:140-183)
template <class R> void ballsocket_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    j.r1 = rotate(j.la1, b1.q);
    j.r2 = rotate(j.la2, b2.q);
    V3<R> p1 = b1.pos + j.r1, p2 = b2.pos + j.r2;
    Mat<R> cr1 = Mat<R>::skew(j.r1), cr2 = Mat<R>::skew(j.r2);
    Mat<R> e = ballsocket_mass(b1, j.r1, b2, j.r2);
    R soft = j.softness * ts.inv_sub_dt;
    e.a[0][0] += soft; e.a[1][1] += soft; e.a[2][2] += soft;
    j.eff = inverse_symmetric(e);
    j.bias = (p2 - p1) * j.bias_factor * ts.inv_dt;
    V3<R> acc = j.acc;
    if (b1.motion == DYNAMIC) {
        b1.vel = b1.vel - cmul(acc, b1.inv_mass_vec);
        b1.angvel = b1.angvel - sym_mul(b1.inv_inertia_world, mvec(cr1, acc));
    }
    if (b2.motion == DYNAMIC) {
        b2.vel = b2.vel + cmul(acc, b2.inv_mass_vec);
        b2.angvel = b2.angvel + sym_mul(b2.inv_inertia_world, mvec(cr2, acc));
    }
}
// BallSocket.IterateBallSocket (BallSocket.cs:223-252)
template <class R> void ballsocket_iterate(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    Mat<R> cr1 = Mat<R>::skew(j.r1), cr2 = Mat<R>::skew(j.r2);
    V3<R> sv = j.acc * j.softness * ts.inv_sub_dt;
    V3<R> jv = -b1.vel + mvec(cr1, b1.angvel) + b2.vel - mvec(cr2, b2.angvel);
    V3<R> lambda = -(R)1.0 * mvec(j.eff, jv + j.bias + sv);
    j.acc = j.acc + lambda;
    if (b1.motion == DYNAMIC) {
        b1.vel = b1.vel - cmul(lambda, b1.inv_mass_vec);
        b1.angvel = b1.angvel - sym_mul(b1.inv_inertia_world, mvec(cr1, lambda));
    }
    if (b2.motion == DYNAMIC) {
        b2.vel = b2.vel + cmul(lambda, b2.inv_mass_vec);
        b2.angvel = b2.angvel + sym_mul(b2.inv_inertia_world, mvec(cr2, lambda));
    }
}
// HingeAngle.PrepareForIterationHingeAngle (HingeAngle.cs:133-220)
template <class R> void hinge_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> p0 = create_orthonormal(j.axis);
    V3<R> p1 = cross(j.axis, p0);
    V3<R> rot;
    short hemi;
    Mat<R> m0 = calc_jacobian(qmul(j.q0, qconj(b1.q)), b2.q, rot, hemi);
    if (j.hemisphere != 0 && j.hemisphere != hemi) j.acc = V3<R>();
    j.hemisphere = hemi;
    V3<R> err(dot(p0, rot), dot(p1, rot), dot(j.axis, rot));
    j.clamp = 0;
    V3<R> r0 = mtvec(m0, p0), r1 = mtvec(m0, p1), r2 = mtvec(m0, j.axis);
    // JMatrix is column-major: UnsafeGet(i) is column i (JMatrix.cs:62-79).
    for (int k = 0; k < 3; k++) { j.jac.a[k][0] = (&r0.x)[k]; j.jac.a[k][1] = (&r1.x)[k]; j.jac.a[k][2] = (&r2.x)[k]; }
    Sym3<R> isum(b1.inv_inertia_world.m11 + b2.inv_inertia_world.m11, b1.inv_inertia_world.m12 + b2.inv_inertia_world.m12,
                 b1.inv_inertia_world.m13 + b2.inv_inertia_world.m13, b1.inv_inertia_world.m22 + b2.inv_inertia_world.m22,
                 b1.inv_inertia_world.m23 + b2.inv_inertia_world.m23, b1.inv_inertia_world.m33 + b2.inv_inertia_world.m33);
    Mat<R> jt = mtrans(j.jac);
    M3<R> jt3;
    for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) jt3.m[i][k] = jt.a[i][k];
    j.eff = Mat<R>::from_sym(sym_transform(isum, jt3));
    j.eff.a[0][0] += j.softness * ts.inv_sub_dt;
    j.eff.a[1][1] += j.softness * ts.inv_sub_dt;
    j.eff.a[2][2] += j.limit_softness * ts.inv_sub_dt;
    R maxA = j.max_angle, minA = j.min_angle;
    const R PI = (R)3.14159265358979323846;
    bool full = minA <= -PI / 2 && maxA >= PI / 2;
    if (minA >= maxA) {
        j.clamp = 3;
        err.z = shortest_angle(err.z - j.fixed_angle, PI / 2);
    } else if (!full && err.z >= maxA) {
        j.clamp = 1;
        err.z -= maxA;
    } else if (!full && err.z <= minA) {
        j.clamp = 2;
        err.z -= minA;
    } else {
        j.acc.z = 0;
        j.eff.a[2][2] = 0;
        j.eff.a[2][0] = j.eff.a[0][2] = 0;
        j.eff.a[2][1] = j.eff.a[1][2] = 0;
        j.jac.a[0][2] = j.jac.a[1][2] = j.jac.a[2][2] = 0;
    }
    if (j.clamp == 1 || j.clamp == 2) {
        j.acc.z = j.clamp == 1 ? std::min(j.acc.z, (R)0) : std::max(j.acc.z, (R)0);
        j.bilateral = inverse_bilateral(j.eff);
        j.coupling_x = j.eff.a[0][2];
        j.coupling_y = j.eff.a[1][2];
    }
    j.eff = inverse_symmetric(j.eff);
    j.bias = err * ts.inv_dt;
    j.bias.x *= j.bias_factor;
    j.bias.y *= j.bias_factor;
    j.bias.z *= j.limit_bias;
    if (b1.motion == DYNAMIC) b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, mvec(j.jac, j.acc));
    if (b2.motion == DYNAMIC) b2.angvel = b2.angvel - sym_mul(b2.inv_inertia_world, mvec(j.jac, j.acc));
}
// HingeAngle.IterateHingeAngle (HingeAngle.cs:313-364)
template <class R> void hinge_iterate(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> jv = mtvec(j.jac, b1.angvel - b2.angvel);
    V3<R> soft = j.acc * ts.inv_sub_dt;
    soft.x *= j.softness; soft.y *= j.softness; soft.z *= j.limit_softness;
    V3<R> res = jv + j.bias + soft;
    V3<R> lambda = -(R)1.0 * mvec(j.eff, res);
    V3<R> orig = j.acc;
    j.acc = j.acc + lambda;
    if ((j.clamp == 1 && j.acc.z > 0) || (j.clamp == 2 && j.acc.z < 0)) {
        lambda.z = -orig.z;
        R x = res.x + j.coupling_x * lambda.z;
        R y = res.y + j.coupling_y * lambda.z;
        lambda.x = -(j.bilateral.x * x + j.bilateral.y * y);
        lambda.y = -(j.bilateral.y * x + j.bilateral.z * y);
        j.acc.x = orig.x + lambda.x;
        j.acc.y = orig.y + lambda.y;
        j.acc.z = 0;
    } else if (j.clamp == 0) {
        orig.z = 0;
        j.acc.z = 0;
    }
    lambda = j.acc - orig;
    if (b1.motion == DYNAMIC) b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, mvec(j.jac, lambda));
    if (b2.motion == DYNAMIC) b2.angvel = b2.angvel - sym_mul(b2.inv_inertia_world, mvec(j.jac, lambda));
}
// ---- one-row limits ---------------------------------------------------------------------
// Shared by DistanceLimit, ConeLimit and TwistAngle: the row's clamp rule for the
// accumulated impulse (1: at the upper limit, impulse <= 0; 2: lower, >= 0; 3: fixed).
template <class R> R clamp_impulse(int clamp, R acc) {
    if (clamp == 1) return std::min(acc, (R)0.0);
    if (clamp == 2) return std::max(acc, (R)0.0);
    return acc;
}
template <class R> R row_mass(R m, R softness, const TimeStep<R>& ts) {
    m += softness * ts.inv_sub_dt;
    return m > 0 ? (R)1.0 / m : (R)0.0;
}

// DistanceLimit.Initialize (DistanceLimit.cs:92-117); limit (min, max), LinearLimit.Fixed
// is (1e-6, -1e-6)
template <class R> void distance_init(Joint<R>& j, const std::vector<Body<R>>& b, V3<R> a1, V3<R> a2, R lo, R hi) {
    j.kind = DISTANCELIMIT;
    j.la1 = rotate_inv(a1 - b[j.b1].pos, b[j.b1].q);
    j.la2 = rotate_inv(a2 - b[j.b2].pos, b[j.b2].q);
    j.softness = (R)0.00001;
    j.bias_factor = (R)0.2;
    j.target = std::sqrt(len2(a2 - a1));
    j.min_angle = lo; j.max_angle = hi;
}
// DistanceLimit.PrepareForIterationDistanceLimit (DistanceLimit.cs:227-306)
template <class R> void distance_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> r1 = rotate(j.la1, b1.q), r2 = rotate(j.la2, b2.q);
    V3<R> dp = (b2.pos + r2) - (b1.pos + r1);
    R dist = std::sqrt(len2(dp));
    R err = dist - j.target;
    j.clamp = 0;
    if (j.min_angle >= j.max_angle) { err -= (R)0.5 * j.min_angle + (R)0.5 * j.max_angle; j.clamp = 3; }
    else if (err >= j.max_angle) { j.clamp = 1; err -= j.max_angle; }
    else if (err <= j.min_angle) { j.clamp = 2; err -= j.min_angle; }
    else { j.acc.x = 0; return; }
    if (dist == 0) { j.clamp = 0; j.acc.x = 0; return; }
    V3<R> n = dp * ((R)1.0 / dist);
    j.jr[0] = -(R)1.0 * n;
    j.jr[1] = -(R)1.0 * cross(r1, n);
    j.jr[2] = (R)1.0 * n;
    j.jr[3] = cross(r2, n);
    R m = dot(cmul(j.jr[0], b1.inv_mass_vec), j.jr[0]) + dot(cmul(j.jr[2], b2.inv_mass_vec), j.jr[2]) +
          dot(sym_mul(b1.inv_inertia_world, j.jr[1]), j.jr[1]) + dot(sym_mul(b2.inv_inertia_world, j.jr[3]), j.jr[3]);
    j.eff1 = row_mass(m, j.softness, ts);
    if (j.eff1 == 0) j.acc.x = 0;
    j.bias.x = err * j.bias_factor * ts.inv_dt;
    R a = j.acc.x;
    if (b1.motion == DYNAMIC) {
        b1.vel = b1.vel + cmul(a * j.jr[0], b1.inv_mass_vec);
        b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, a * j.jr[1]);
    }
    if (b2.motion == DYNAMIC) {
        b2.vel = b2.vel + cmul(a * j.jr[2], b2.inv_mass_vec);
        b2.angvel = b2.angvel + sym_mul(b2.inv_inertia_world, a * j.jr[3]);
    }
}
// DistanceLimit.IterateDistanceLimit (DistanceLimit.cs:344-391)
template <class R> void distance_iterate(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    if (j.clamp == 0) return;
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    R jv = dot(b1.vel, j.jr[0]) + dot(b1.angvel, j.jr[1]) + dot(b2.vel, j.jr[2]) + dot(b2.angvel, j.jr[3]);
    R soft = j.acc.x * j.softness * ts.inv_sub_dt;
    R lambda = -j.eff1 * (jv + j.bias.x + soft);
    R old = j.acc.x;
    j.acc.x = clamp_impulse(j.clamp, j.acc.x + lambda);
    lambda = j.acc.x - old;
    if (b1.motion == DYNAMIC) {
        b1.vel = b1.vel + cmul(lambda * j.jr[0], b1.inv_mass_vec);
        b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, lambda * j.jr[1]);
    }
    if (b2.motion == DYNAMIC) {
        b2.vel = b2.vel + cmul(lambda * j.jr[2], b2.inv_mass_vec);
        b2.angvel = b2.angvel + sym_mul(b2.inv_inertia_world, lambda * j.jr[3]);
    }
}

// ConeLimit.Initialize (ConeLimit.cs:92-118): world axes of the two bodies, limit (min, max)
// in radians within [0, pi]
template <class R> void cone_init(Joint<R>& j, const std::vector<Body<R>>& b, V3<R> ax1, V3<R> ax2, R lo, R hi) {
    j.kind = CONELIMIT;
    j.la1 = rotate_inv(normalize(ax1), b[j.b1].q);
    j.la2 = rotate_inv(normalize(ax2), b[j.b2].q);
    j.softness = (R)0.001;
    j.bias_factor = (R)0.2;
    j.min_angle = lo; j.max_angle = hi;
}
// ConeLimit.PrepareForIterationConeLimit (ConeLimit.cs:262-356).  The row is the angle
// between the two axes; its Jacobian persists between steps, and a sign flip of it drops
// the cached impulse.
template <class R> void cone_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> a1 = rotate(j.la1, b1.q), a2 = rotate(j.la2, b2.q);
    V3<R> prev = j.jr[0];
    j.jr[0] = cross(a2, a1);
    j.clamp = 0;
    R cosine = dot(a1, a2);
    R lower = -j.min_angle, upper = -j.max_angle;
    R sine = std::sqrt(len2(j.jr[0]));
    if (sine > 0) {
        j.jr[0] = j.jr[0] * ((R)1.0 / sine);
    } else {
        // at a cusp: the perpendicular axis with the larger response
        V3<R> axis = create_orthonormal(a1);
        V3<R> other = cross(a1, axis);
        Sym3<R> I(b1.inv_inertia_world.m11 + b2.inv_inertia_world.m11, b1.inv_inertia_world.m12 + b2.inv_inertia_world.m12,
                  b1.inv_inertia_world.m13 + b2.inv_inertia_world.m13, b1.inv_inertia_world.m22 + b2.inv_inertia_world.m22,
                  b1.inv_inertia_world.m23 + b2.inv_inertia_world.m23, b1.inv_inertia_world.m33 + b2.inv_inertia_world.m33);
        j.jr[0] = dot(sym_mul(I, axis), axis) >= dot(sym_mul(I, other), other) ? axis : other;
    }
    j.jr[1] = -j.jr[0];
    if (dot(prev, j.jr[0]) < 0) j.acc.x = 0;
    R err = -StableMath<R>::atan2(sine, cosine);
    const R PI = (R)3.14159265358979323846;
    if (lower == upper) { j.clamp = 3; err -= upper; }
    else if (err <= upper && j.max_angle < PI) { j.clamp = 1; err -= upper; }
    else if (err >= lower && j.min_angle > 0) { j.clamp = 2; err -= lower; }
    else { j.acc.x = 0; return; }
    j.acc.x = clamp_impulse(j.clamp, j.acc.x);
    R m = dot(sym_mul(b1.inv_inertia_world, j.jr[0]), j.jr[0]) + dot(sym_mul(b2.inv_inertia_world, j.jr[1]), j.jr[1]);
    j.eff1 = row_mass(m, j.softness, ts);
    if (j.eff1 == 0) j.acc.x = 0;
    j.bias.x = -err * j.bias_factor * ts.inv_dt;
    if (b1.motion == DYNAMIC) b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, j.acc.x * j.jr[0]);
    if (b2.motion == DYNAMIC) b2.angvel = b2.angvel + sym_mul(b2.inv_inertia_world, j.acc.x * j.jr[1]);
}
// ConeLimit.IterateConeLimit (ConeLimit.cs:378-404)
template <class R> void cone_iterate(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    if (j.clamp == 0) return;
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    R jv = dot(b1.angvel, j.jr[0]) + dot(b2.angvel, j.jr[1]);
    R soft = j.acc.x * j.softness * ts.inv_sub_dt;
    R lambda = -j.eff1 * (jv + j.bias.x + soft);
    R old = j.acc.x;
    j.acc.x = clamp_impulse(j.clamp, j.acc.x + lambda);
    lambda = j.acc.x - old;
    if (b1.motion == DYNAMIC) b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, lambda * j.jr[0]);
    if (b2.motion == DYNAMIC) b2.angvel = b2.angvel + sym_mul(b2.inv_inertia_world, lambda * j.jr[1]);
}

// JQuaternion.CreateFromToRotation (JQuaternion.cs:84-101)
template <class R> Q4<R> from_to_rotation(V3<R> from, V3<R> to) {
    R d = dot(from, to);
    if (d < -(R)1.0 + (R)1e-6) {
        V3<R> ax = create_orthonormal(from);
        return Q4<R>(ax.x, ax.y, ax.z, 0);
    }
    R s = std::sqrt(((R)1.0 + d) * (R)2.0);
    R is = (R)1.0 / s;
    V3<R> c = cross(from, to);
    V3<R> v = c * is;
    return Q4<R>(v.x, v.y, v.z, s * (R)0.5);
}
// QMatrix.ProjectMultiplyLeftRight (QMatrix.cs:112-125): the vector block (rows and
// columns 1..3) of L(left) R(right), the left- and right-multiplication matrices of the
// two quaternions in (w, x, y, z) order, each entry summed over k = 0..3 in order.
template <class R> Mat<R> project_left_right(Q4<R> l, Q4<R> r) {
    const R L[4][4] = {{l.w, -l.x, -l.y, -l.z}, {l.x, l.w, -l.z, l.y}, {l.y, l.z, l.w, -l.x}, {l.z, -l.y, l.x, l.w}};
    const R Rm[4][4] = {{r.w, -r.x, -r.y, -r.z}, {r.x, r.w, r.z, -r.y}, {r.y, -r.z, r.w, r.x}, {r.z, r.y, -r.x, r.w}};
    Mat<R> o;
    for (int i = 1; i < 4; i++)
        for (int c = 1; c < 4; c++) {
            R acc = L[i][0] * Rm[0][c];
            for (int k = 1; k < 4; k++) acc += L[i][k] * Rm[k][c];
            o.a[i - 1][c - 1] = acc;
        }
    return o;
}
// AngularConstraintMath.CalculateTwist (AngularConstraintMath.cs:33-64): the twist angle of
// left * right about `axis` and its unit Jacobian row
template <class R> R calc_twist(Q4<R> left, Q4<R> right, V3<R> axis, V3<R>& jac, short& hemi) {
    Mat<R> m = mscale(-(R)0.5, project_left_right(left, right));
    Q4<R> q = qmul(left, right);
    jac = mtvec(m, axis);
    R proj = dot(axis, V3<R>(q.x, q.y, q.z));
    hemi = q.w < 0 ? (short)-1 : (short)1;
    if (q.w < 0) {
        q = Q4<R>(-q.x, -q.y, -q.z, -q.w);
        proj = proj * -(R)1;
        jac = jac * (R)-1;
    }
    R d2 = len2(jac);
    if (d2 > 0) jac = jac * ((R)1 / std::sqrt(d2));
    else jac = -rotate(axis, right);
    V3<R> perp = V3<R>(q.x, q.y, q.z) - axis * proj;
    R cosine = std::sqrt(q.w * q.w + len2(perp));
    return (R)2 * StableMath<R>::atan2(proj, cosine);
}
// TwistAngle.Initialize (TwistAngle.cs:85-128): world axes of the two bodies, limit
// (min, max) in radians; Q0 is the initial relative rotation with the axes aligned
template <class R> void twist_init(Joint<R>& j, const std::vector<Body<R>>& b, V3<R> ax1, V3<R> ax2, R lo, R hi) {
    j.kind = TWISTANGLE;
    j.softness = (R)0.001;
    j.bias_factor = (R)0.2;
    ax1 = normalize(ax1); ax2 = normalize(ax2);
    j.min_angle = lo; j.max_angle = hi;
    j.fixed_angle = (R)0.5 * lo + (R)0.5 * hi;
    Q4<R> q1 = b[j.b1].q, q2 = b[j.b2].q;
    V3<R> u1 = rotate_inv(ax1, q1);
    j.axis = rotate_inv(ax2, q2);
    Q4<R> rel = qmul(qconj(q2), q1);
    V3<R> u1b2 = rotate(u1, rel);
    j.q0 = qmul(from_to_rotation(u1b2, j.axis), rel);
}
// TwistAngle.PrepareForIterationTwistAngle (TwistAngle.cs:170-233)
template <class R> void twist_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    short hemi;
    R err = calc_twist(qmul(j.q0, qconj(b1.q)), b2.q, j.axis, j.jr[0], hemi);
    R lower = j.min_angle, upper = j.max_angle;
    if (j.hemisphere != 0 && j.hemisphere != hemi) j.acc.x = 0;
    j.hemisphere = hemi;
    j.clamp = 0;
    const R PI = (R)3.14159265358979323846;
    bool full = lower <= -PI && upper >= PI;
    if (lower >= upper) { j.clamp = 3; err = shortest_angle(err - j.fixed_angle, PI); }
    else if (!full && err >= upper) { j.clamp = 1; err -= upper; }
    else if (!full && err <= lower) { j.clamp = 2; err -= lower; }
    else { j.acc.x = 0; return; }
    j.acc.x = clamp_impulse(j.clamp, j.acc.x);
    Sym3<R> I(b1.inv_inertia_world.m11 + b2.inv_inertia_world.m11, b1.inv_inertia_world.m12 + b2.inv_inertia_world.m12,
              b1.inv_inertia_world.m13 + b2.inv_inertia_world.m13, b1.inv_inertia_world.m22 + b2.inv_inertia_world.m22,
              b1.inv_inertia_world.m23 + b2.inv_inertia_world.m23, b1.inv_inertia_world.m33 + b2.inv_inertia_world.m33);
    j.eff1 = row_mass(dot(sym_mul(I, j.jr[0]), j.jr[0]), j.softness, ts);
    if (j.eff1 == 0) j.acc.x = 0;
    j.bias.x = err * j.bias_factor * ts.inv_dt;
    if (b1.motion == DYNAMIC) b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, j.acc.x * j.jr[0]);
    if (b2.motion == DYNAMIC) b2.angvel = b2.angvel - sym_mul(b2.inv_inertia_world, j.acc.x * j.jr[0]);
}
// TwistAngle.IterateTwistAngle (TwistAngle.cs:296-323)
template <class R> void twist_iterate(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    if (j.clamp == 0) return;
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    R jv = dot(b1.angvel - b2.angvel, j.jr[0]);
    R soft = j.acc.x * (j.softness * ts.inv_sub_dt);
    R lambda = -j.eff1 * (jv + j.bias.x + soft);
    R old = j.acc.x;
    j.acc.x = clamp_impulse(j.clamp, j.acc.x + lambda);
    lambda = j.acc.x - old;
    if (b1.motion == DYNAMIC) b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, lambda * j.jr[0]);
    if (b2.motion == DYNAMIC) b2.angvel = b2.angvel - sym_mul(b2.inv_inertia_world, lambda * j.jr[0]);
}

// ConeLimit.Angle (ConeLimit.cs:137-149) and TwistAngle.Angle (TwistAngle.cs:240-258): the
// joint's current angle as its public getter reports it (0 for the other kinds).
template <class R> R joint_angle(const Joint<R>& j, const std::vector<Body<R>>& b) {
    if (j.kind == CONELIMIT) {
        V3<R> a1 = rotate(j.la1, b[j.b1].q), a2 = rotate(j.la2, b[j.b2].q);
        return StableMath<R>::atan2(std::sqrt(len2(cross(a1, a2))), dot(a1, a2));
    }
    if (j.kind == TWISTANGLE) {
        Q4<R> q = qmul(qmul(j.q0, qconj(b[j.b1].q)), b[j.b2].q);
        if (q.w < (R)0.0) q = Q4<R>(-q.x, -q.y, -q.z, -q.w);
        V3<R> v(q.x, q.y, q.z);
        R proj = dot(j.axis, v);
        V3<R> perp = v - j.axis * proj;
        return (R)2.0 * StableMath<R>::atan2(proj, std::sqrt(q.w * q.w + len2(perp)));
    }
    return 0;
}

// FixedAngle.Initialize (FixedAngle.cs:72-85): Q0 is the initial relative rotation
template <class R> void fixed_init(Joint<R>& j, const std::vector<Body<R>>& b) {
    j.kind = FIXEDANGLE;
    j.softness = (R)0.001;
    j.bias_factor = (R)0.2;
    j.q0 = qmul(qconj(b[j.b2].q), b[j.b1].q);
}
// FixedAngle.PrepareForIterationFixedAngle (FixedAngle.cs:87-128): three angular rows, the
// Jacobian -2 x the rotation-log derivative of Q0 conj(q1) q2
template <class R> void fixed_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> err;
    short hemi;
    j.jac = mscale(-(R)2, calc_jacobian(qmul(j.q0, qconj(b1.q)), b2.q, err, hemi));
    if (j.hemisphere != 0 && j.hemisphere != hemi) j.acc = V3<R>();
    j.hemisphere = hemi;
    Sym3<R> isum(b1.inv_inertia_world.m11 + b2.inv_inertia_world.m11, b1.inv_inertia_world.m12 + b2.inv_inertia_world.m12,
                 b1.inv_inertia_world.m13 + b2.inv_inertia_world.m13, b1.inv_inertia_world.m22 + b2.inv_inertia_world.m22,
                 b1.inv_inertia_world.m23 + b2.inv_inertia_world.m23, b1.inv_inertia_world.m33 + b2.inv_inertia_world.m33);
    M3<R> jt3;
    for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) jt3.m[i][k] = j.jac.a[i][k];
    j.eff = Mat<R>::from_sym(sym_transform(isum, jt3));
    R soft = j.softness * ts.inv_sub_dt;
    j.eff.a[0][0] += soft; j.eff.a[1][1] += soft; j.eff.a[2][2] += soft;
    j.eff = inverse_symmetric(j.eff);
    j.bias = -err * j.bias_factor * ts.inv_dt;
    V3<R> imp = mtvec(j.jac, j.acc);
    if (b1.motion == DYNAMIC) b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, imp);
    if (b2.motion == DYNAMIC) b2.angvel = b2.angvel - sym_mul(b2.inv_inertia_world, imp);
}
// FixedAngle.IterateFixedAngle (FixedAngle.cs:159-181)
template <class R> void fixed_iterate(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> jv = mvec(j.jac, b1.angvel - b2.angvel);
    V3<R> soft = j.acc * (j.softness * ts.inv_sub_dt);
    V3<R> lambda = -(R)1.0 * mvec(j.eff, jv + j.bias + soft);
    j.acc = j.acc + lambda;
    V3<R> imp = mtvec(j.jac, lambda);
    if (b1.motion == DYNAMIC) b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, imp);
    if (b2.motion == DYNAMIC) b2.angvel = b2.angvel - sym_mul(b2.inv_inertia_world, imp);
}

// PointOnPlane.Initialize (PointOnPlane.cs:96-126): the plane's normal fixed in body 1, an
// anchor on each body, the signed distance limited to [min, max] (min >= max fixes it)
template <class R> void plane_init(Joint<R>& j, const std::vector<Body<R>>& b, V3<R> axis, V3<R> a1, V3<R> a2, R lo, R hi) {
    j.kind = POINTONPLANE;
    axis = normalize(axis);
    j.la1 = rotate_inv(a1 - b[j.b1].pos, b[j.b1].q);
    j.la2 = rotate_inv(a2 - b[j.b2].pos, b[j.b2].q);
    j.axis = rotate_inv(axis, b[j.b1].q);
    j.bias_factor = (R)0.2;
    j.softness = (R)0.00001;
    j.min_angle = lo; j.max_angle = hi;
}
// PointOnPlane.PrepareForIterationPointOnPlane (PointOnPlane.cs:128-200): one row along the
// plane normal, the arm of body 1 measured to the second anchor
template <class R> void plane_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> axis = rotate(j.axis, b1.q);
    V3<R> r1 = rotate(j.la1, b1.q), r2 = rotate(j.la2, b2.q);
    V3<R> u = (b2.pos + r2) - (b1.pos + r1);
    j.clamp = 0;
    j.jr[0] = -axis;
    j.jr[1] = -cross(r1 + u, axis);
    j.jr[2] = axis;
    j.jr[3] = cross(r2, axis);
    R err = dot(u, axis);
    j.eff1 = 1;
    if (j.min_angle >= j.max_angle) { err -= (R)0.5 * j.min_angle + (R)0.5 * j.max_angle; j.clamp = 3; }
    else if (err >= j.max_angle) { err -= j.max_angle; j.clamp = 1; }
    else if (err <= j.min_angle) { err -= j.min_angle; j.clamp = 2; }
    else { j.acc.x = 0; return; }
    R m = dot(cmul(j.jr[0], b1.inv_mass_vec), j.jr[0]) + dot(cmul(j.jr[2], b2.inv_mass_vec), j.jr[2]) +
          dot(sym_mul(b1.inv_inertia_world, j.jr[1]), j.jr[1]) + dot(sym_mul(b2.inv_inertia_world, j.jr[3]), j.jr[3]);
    j.eff1 = row_mass(m, j.softness, ts);
    if (j.eff1 == 0) j.acc.x = 0;
    j.bias.x = err * j.bias_factor * ts.inv_dt;
    R a = j.acc.x;
    if (b1.motion == DYNAMIC) {
        b1.vel = b1.vel + cmul(j.jr[0] * a, b1.inv_mass_vec);
        b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, j.jr[1] * a);
    }
    if (b2.motion == DYNAMIC) {
        b2.vel = b2.vel + cmul(j.jr[2] * a, b2.inv_mass_vec);
        b2.angvel = b2.angvel + sym_mul(b2.inv_inertia_world, j.jr[3] * a);
    }
}

// AngularMotor.Initialize (AngularMotor.cs:62-82) and LinearMotor.Initialize
// (LinearMotor.cs:97-115) with TargetVelocity and MaximumTorque / MaximumForce: a velocity
// drive about (along) an axis of each body (the target in target, the torque or force limit
// in max_angle, the impulse limit of a substep in min_angle once prepared)
template <class R> void motor_init(Joint<R>& j, const std::vector<Body<R>>& b, V3<R> ax1, V3<R> ax2, R velocity, R torque,
                                   bool linear = false) {
    j.kind = linear ? LINEARMOTOR : ANGULARMOTOR;
    j.la1 = rotate_inv(normalize(ax1), b[j.b1].q);
    j.la2 = rotate_inv(normalize(ax2), b[j.b2].q);
    j.target = velocity;
    j.max_angle = torque;
}
// the response of a body along / about an axis, and the velocity change of an impulse
template <class R> R motor_response(const Body<R>& b, V3<R> a, bool linear) {
    return linear ? dot(cmul(a, b.inv_mass_vec), a) : dot(sym_mul(b.inv_inertia_world, a), a);
}
template <class R> void motor_push(Body<R>& b, V3<R> imp, bool linear) {
    if (linear) b.vel = b.vel + cmul(imp, b.inv_mass_vec);
    else b.angvel = b.angvel + sym_mul(b.inv_inertia_world, imp);
}
// AngularMotor.PrepareForIterationAngularMotor (AngularMotor.cs:128-152),
// LinearMotor.PrepareForIterationLinearMotor (LinearMotor.cs:152-176)
template <class R> void motor_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    const bool lin = j.kind == LINEARMOTOR;
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> j1 = rotate(j.la1, b1.q), j2 = rotate(j.la2, b2.q);
    R m = motor_response(b1, j1, lin) + motor_response(b2, j2, lin);
    j.eff1 = m > 0 ? (R)1.0 / m : (R)0;
    if (j.eff1 == 0) j.acc.x = 0;
    j.min_angle = ts.sub_dt * j.max_angle;
    if (b1.motion == DYNAMIC) motor_push(b1, -(j1 * j.acc.x), lin);
    if (b2.motion == DYNAMIC) motor_push(b2, j2 * j.acc.x, lin);
}
// AngularMotor.IterateAngularMotor (AngularMotor.cs:154-180),
// LinearMotor.IterateLinearMotor (LinearMotor.cs:203-231)
template <class R> void motor_iterate(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>&) {
    const bool lin = j.kind == LINEARMOTOR;
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> j1 = rotate(j.la1, b1.q), j2 = rotate(j.la2, b2.q);
    R jv = lin ? dot(-j1, b1.vel) + dot(j2, b2.vel) : dot(-j1, b1.angvel) + dot(j2, b2.angvel);
    R lambda = -(jv - j.target) * j.eff1;
    R old = j.acc.x;
    j.acc.x = std::min(std::max(j.acc.x + lambda, -j.min_angle), j.min_angle);
    lambda = j.acc.x - old;
    if (b1.motion == DYNAMIC) motor_push(b1, -(j1 * lambda), lin);
    if (b2.motion == DYNAMIC) motor_push(b2, j2 * lambda, lin);
}


// ---- servos (Dynamics/Constraints/*Servo.cs, Internal/ServoMath.cs) --------------------------
// ServoMath.MaximumImpulse (ServoMath.cs:30)
template <class R> R servo_max_impulse(R maximum, R dt) { return dt > 0 ? maximum * dt : (R)0; }
// Math.Clamp as .NET defines it (value < min -> min, value > max -> max, else value)
template <class R> R net_clamp(R v, R lo, R hi) { return v < lo ? lo : (v > hi ? hi : v); }
// ServoMath.ClampMagnitude (ServoMath.cs:32-38)
template <class R> void servo_clamp_magnitude(V3<R>& imp, R maxi) {
    if (std::isinf(maxi) && maxi > 0) return;
    R l2 = dot(imp, imp);
    if (l2 > maxi * maxi) imp = imp * (maxi / std::sqrt(l2));
}
// ServoMath.ClampAngular (ServoMath.cs:40-49): the applied angular impulse J^T imp limited
template <class R> void servo_clamp_angular(V3<R>& imp, const Mat<R>& jac, R maxi) {
    if (std::isinf(maxi) && maxi > 0) return;
    V3<R> a = mtvec(jac, imp);
    R l2 = dot(a, a);
    if (l2 > maxi * maxi) imp = imp * (maxi / std::sqrt(l2));
}

// AngularServo.Initialize (AngularServo.cs:55-77): the target relative orientation (body 2 in
// body 1's frame), MaximumTorque
template <class R> void angular_servo_init(Joint<R>& j, Q4<R> target, R maximum) {
    j.kind = ANGULARSERVO;
    j.q0 = target;
    j.maximum = maximum;
    j.softness = (R)0.001;
    j.bias_factor = (R)0.2;
    j.hemisphere = 0;
}
template <class R> void angular_servo_apply(Joint<R>& j, Body<R>& b1, Body<R>& b2, V3<R> imp) {
    if (b1.motion == DYNAMIC) b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, imp);
    if (b2.motion == DYNAMIC) b2.angvel = b2.angvel - sym_mul(b2.inv_inertia_world, imp);
}
// AngularServo.PrepareForIterationAngularServo (AngularServo.cs:125-149), ApplyImpulse (:164-172)
template <class R> void angular_servo_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> err;
    short hemi;
    j.jac = mscale(-(R)2, calc_jacobian(qmul(qconj(j.q0), qconj(b1.q)), b2.q, err, hemi));
    if (j.hemisphere != 0 && j.hemisphere != hemi) j.acc = V3<R>();
    j.hemisphere = hemi;
    Sym3<R> isum(b1.inv_inertia_world.m11 + b2.inv_inertia_world.m11, b1.inv_inertia_world.m12 + b2.inv_inertia_world.m12,
                 b1.inv_inertia_world.m13 + b2.inv_inertia_world.m13, b1.inv_inertia_world.m22 + b2.inv_inertia_world.m22,
                 b1.inv_inertia_world.m23 + b2.inv_inertia_world.m23, b1.inv_inertia_world.m33 + b2.inv_inertia_world.m33);
    M3<R> jt3;
    for (int i = 0; i < 3; i++) for (int k = 0; k < 3; k++) jt3.m[i][k] = j.jac.a[i][k];
    j.eff = Mat<R>::from_sym(sym_transform(isum, jt3));
    R soft = j.softness * ts.inv_sub_dt;
    j.eff.a[0][0] += soft; j.eff.a[1][1] += soft; j.eff.a[2][2] += soft;
    j.eff = inverse_symmetric(j.eff);
    j.bias = -err * j.bias_factor * ts.inv_dt;
    servo_clamp_angular(j.acc, j.jac, servo_max_impulse(j.maximum, ts.sub_dt));
    angular_servo_apply(j, b1, b2, mtvec(j.jac, j.acc));
}
// AngularServo.IterateAngularServo (AngularServo.cs:151-162)
template <class R> void angular_servo_iterate(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> jv = mvec(j.jac, b1.angvel - b2.angvel);
    V3<R> soft = j.acc * (j.softness * ts.inv_sub_dt);
    V3<R> lambda = -(R)1.0 * mvec(j.eff, jv + j.bias + soft);
    V3<R> prev = j.acc;
    j.acc = j.acc + lambda;
    servo_clamp_angular(j.acc, j.jac, servo_max_impulse(j.maximum, ts.sub_dt));
    angular_servo_apply(j, b1, b2, mtvec(j.jac, j.acc - prev));
}

// LinearServo.Initialize (LinearServo.cs:60-73) with TargetPosition and MaximumForce: anchors on both bodies, the target offset of
// anchor 2 from anchor 1 in body 1's frame, MaximumForce
template <class R> void linear_servo_init(Joint<R>& j, const std::vector<Body<R>>& b, V3<R> a1, V3<R> a2, V3<R> target,
                                          R maximum) {
    j.kind = LINEARSERVO;
    j.la1 = rotate_inv(a1 - b[j.b1].pos, b[j.b1].q);
    j.la2 = rotate_inv(a2 - b[j.b2].pos, b[j.b2].q);
    j.target_pos = target;
    j.maximum = maximum;
    j.softness = (R)0.00001;
    j.bias_factor = (R)0.2;
}
template <class R> void linear_servo_apply(Joint<R>& j, Body<R>& b1, Body<R>& b2, V3<R> imp) {
    if (b1.motion == DYNAMIC) {
        b1.vel = b1.vel - cmul(imp, b1.inv_mass_vec);
        b1.angvel = b1.angvel - sym_mul(b1.inv_inertia_world, cross(j.r1, imp));
    }
    if (b2.motion == DYNAMIC) {
        b2.vel = b2.vel + cmul(imp, b2.inv_mass_vec);
        b2.angvel = b2.angvel + sym_mul(b2.inv_inertia_world, cross(j.r2, imp));
    }
}
// LinearServo.PrepareForIterationLinearServo (LinearServo.cs:149-171), ApplyImpulse (:189-201)
template <class R> void linear_servo_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    j.r1 = rotate(j.la1 + j.target_pos, b1.q);
    j.r2 = rotate(j.la2, b2.q);
    Mat<R> e = ballsocket_mass(b1, j.r1, b2, j.r2);
    R soft = j.softness * ts.inv_sub_dt;
    e.a[0][0] += soft; e.a[1][1] += soft; e.a[2][2] += soft;
    j.eff = inverse_symmetric(e);
    j.bias = (((b2.pos + j.r2) - b1.pos) - j.r1) * (j.bias_factor * ts.inv_dt);
    servo_clamp_magnitude(j.acc, servo_max_impulse(j.maximum, ts.sub_dt));
    linear_servo_apply(j, b1, b2, j.acc);
}
// LinearServo.IterateLinearServo (LinearServo.cs:173-187)
template <class R> void linear_servo_iterate(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> jv = ((-b1.vel - cross(b1.angvel, j.r1)) + b2.vel) + cross(b2.angvel, j.r2);
    V3<R> soft = j.acc * (j.softness * ts.inv_sub_dt);
    V3<R> lambda = -(R)1.0 * mvec(j.eff, jv + j.bias + soft);
    V3<R> prev = j.acc;
    j.acc = j.acc + lambda;
    servo_clamp_magnitude(j.acc, servo_max_impulse(j.maximum, ts.sub_dt));
    linear_servo_apply(j, b1, b2, j.acc - prev);
}

// LinearAxisServo.Initialize (LinearAxisServo.cs:61-78) with MaximumForce: an axis fixed in body 1, anchors on
// both bodies, the target signed position of anchor 2 along the axis, MaximumForce
template <class R> void linear_axis_servo_init(Joint<R>& j, const std::vector<Body<R>>& b, V3<R> axis, V3<R> a1, V3<R> a2,
                                               R target, R maximum) {
    j.kind = LINEARAXISSERVO;
    axis = normalize(axis);
    j.axis = rotate_inv(axis, b[j.b1].q);
    j.la1 = rotate_inv(a1 - b[j.b1].pos, b[j.b1].q);
    j.la2 = rotate_inv(a2 - b[j.b2].pos, b[j.b2].q);
    j.target = target;
    j.maximum = maximum;
    j.softness = (R)0.00001;
    j.bias_factor = (R)0.2;
}
template <class R> void axis_servo_apply(Joint<R>& j, Body<R>& b1, Body<R>& b2, R a) {
    if (b1.motion == DYNAMIC) {
        b1.vel = b1.vel + cmul(j.jr[0] * a, b1.inv_mass_vec);
        b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, j.jr[1] * a);
    }
    if (b2.motion == DYNAMIC) {
        b2.vel = b2.vel + cmul(j.jr[2] * a, b2.inv_mass_vec);
        b2.angvel = b2.angvel + sym_mul(b2.inv_inertia_world, j.jr[3] * a);
    }
}
// LinearAxisServo.PrepareForIterationLinearAxisServo (LinearAxisServo.cs:169-194), ApplyImpulse (:211-224)
template <class R> void linear_axis_servo_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> axis = rotate(j.axis, b1.q);
    V3<R> r1 = rotate(j.la1, b1.q), r2 = rotate(j.la2, b2.q);
    V3<R> sep = ((b2.pos + r2) - b1.pos) - r1;
    j.jr[0] = -axis;
    j.jr[1] = -cross(r1 + sep, axis);
    j.jr[2] = axis;
    j.jr[3] = cross(r2, axis);
    R m = dot(cmul(j.jr[0], b1.inv_mass_vec), j.jr[0]) + dot(cmul(j.jr[2], b2.inv_mass_vec), j.jr[2]) +
          dot(sym_mul(b1.inv_inertia_world, j.jr[1]), j.jr[1]) + dot(sym_mul(b2.inv_inertia_world, j.jr[3]), j.jr[3]) +
          j.softness * ts.inv_sub_dt;
    j.eff1 = m > 0 ? (R)1 / m : (R)0;
    if (j.eff1 == 0) j.acc.x = 0;
    j.bias.x = (dot(sep, axis) - j.target) * j.bias_factor * ts.inv_dt;
    R maxi = servo_max_impulse(j.maximum, ts.sub_dt);
    j.acc.x = net_clamp(j.acc.x, -maxi, maxi);
    axis_servo_apply(j, b1, b2, j.acc.x);
}
// LinearAxisServo.IterateLinearAxisServo (LinearAxisServo.cs:196-209)
template <class R> void linear_axis_servo_iterate(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    R jv = dot(j.jr[0], b1.vel) + dot(j.jr[1], b1.angvel) + dot(j.jr[2], b2.vel) + dot(j.jr[3], b2.angvel);
    R lambda = -(jv + j.bias.x + j.acc.x * j.softness * ts.inv_sub_dt) * j.eff1;
    R prev = j.acc.x;
    R maxi = servo_max_impulse(j.maximum, ts.sub_dt);
    j.acc.x = net_clamp(prev + lambda, -maxi, maxi);
    axis_servo_apply(j, b1, b2, j.acc.x - prev);
}

// TwistServo.Initialize (TwistServo.cs:69-87) with MaximumTorque: body 2's axis, the reference rotation that
// turns body 1's axis onto it, the target twist angle in [-pi, pi], MaximumTorque
template <class R> void twist_servo_init(Joint<R>& j, const std::vector<Body<R>>& b, V3<R> ax1, V3<R> ax2, R target,
                                         R maximum) {
    j.kind = TWISTSERVO;
    ax1 = normalize(ax1);
    ax2 = normalize(ax2);
    const Q4<R> q1 = b[j.b1].q, q2 = b[j.b2].q;
    j.axis = rotate_inv(ax2, q2);
    V3<R> first = rotate_inv(ax1, q2);
    j.q0 = qmul(from_to_rotation(first, j.axis), qmul(qconj(q2), q1));
    j.target = target;
    j.maximum = maximum;
    j.softness = (R)0.001;
    j.bias_factor = (R)0.2;
    j.hemisphere = 0;
}
template <class R> void twist_servo_apply(Joint<R>& j, Body<R>& b1, Body<R>& b2, R a) {
    if (b1.motion == DYNAMIC) b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, j.jr[0] * a);
    if (b2.motion == DYNAMIC) b2.angvel = b2.angvel - sym_mul(b2.inv_inertia_world, j.jr[0] * a);
}
// TwistServo.PrepareForIterationTwistServo (TwistServo.cs:150-170), ApplyImpulse (:184-192)
template <class R> void twist_servo_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    short hemi;
    R angle = calc_twist(qmul(j.q0, qconj(b1.q)), b2.q, j.axis, j.jr[0], hemi);
    if (j.hemisphere != 0 && j.hemisphere != hemi) j.acc.x = 0;
    j.hemisphere = hemi;
    Sym3<R> isum(b1.inv_inertia_world.m11 + b2.inv_inertia_world.m11, b1.inv_inertia_world.m12 + b2.inv_inertia_world.m12,
                 b1.inv_inertia_world.m13 + b2.inv_inertia_world.m13, b1.inv_inertia_world.m22 + b2.inv_inertia_world.m22,
                 b1.inv_inertia_world.m23 + b2.inv_inertia_world.m23, b1.inv_inertia_world.m33 + b2.inv_inertia_world.m33);
    R m = dot(sym_mul(isum, j.jr[0]), j.jr[0]) + j.softness * ts.inv_sub_dt;
    j.eff1 = m > 0 ? (R)1 / m : (R)0;
    if (j.eff1 == 0) j.acc.x = 0;
    R error = angle - j.target;
    j.bias.x = error * j.bias_factor * ts.inv_dt;
    R maxi = servo_max_impulse(j.maximum, ts.sub_dt);
    j.acc.x = net_clamp(j.acc.x, -maxi, maxi);
    twist_servo_apply(j, b1, b2, j.acc.x);
}
// TwistServo.IterateTwistServo (TwistServo.cs:172-182)
template <class R> void twist_servo_iterate(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    R jv = dot(b1.angvel - b2.angvel, j.jr[0]);
    R lambda = -j.eff1 * (jv + j.bias.x + j.acc.x * j.softness * ts.inv_sub_dt);
    R prev = j.acc.x;
    R maxi = servo_max_impulse(j.maximum, ts.sub_dt);
    j.acc.x = net_clamp(prev + lambda, -maxi, maxi);
    twist_servo_apply(j, b1, b2, j.acc.x - prev);
}

// ---- PointOnLine (Dynamics/Constraints/PointOnLine.cs) ---------------------------------------
// Math.Min / Math.Max as .NET defines them for floating point: NaN wins, and of two equal
// values Min returns the negative zero, Max the positive one
template <class R> R net_min(R a, R b) {
    if (a != b) return std::isnan(a) ? a : (a < b ? a : b);
    return std::signbit(b) ? b : a;
}
template <class R> R net_max(R a, R b) {
    if (a != b) return std::isnan(a) ? a : (a > b ? a : b);
    return std::signbit(b) ? a : b;
}
// PointOnLine.Initialize (PointOnLine.cs:92-121): the line's direction fixed in body 1
// through anchor 1, anchor 2 on body 2, the position along the line limited to [min, max]
// (min >= max fixes it)
template <class R> void line_init(Joint<R>& j, const std::vector<Body<R>>& b, V3<R> axis, V3<R> a1, V3<R> a2, R lo, R hi) {
    j.kind = POINTONLINE;
    axis = normalize(axis);
    j.la1 = rotate_inv(a1 - b[j.b1].pos, b[j.b1].q);
    j.la2 = rotate_inv(a2 - b[j.b2].pos, b[j.b2].q);
    j.axis = rotate_inv(axis, b[j.b1].q);
    j.bias_factor = (R)0.2;
    j.softness = (R)0.00001;
    j.limit_softness = (R)0.0001;
    j.limit_bias = (R)0.2;
    j.min_angle = lo; j.max_angle = hi;
}
// the twelve Jacobian blocks (two perpendicular rows and the row along the line, each for
// v1, w1, v2, w2) and the error (PointOnLine.cs:155-185, recomputed in :378-408)
template <class R> V3<R> line_jacobian(const Joint<R>& j, const Body<R>& b1, const Body<R>& b2, V3<R>* J) {
    V3<R> aw = rotate(j.axis, b1.q);
    V3<R> n1 = rotate(create_orthonormal(j.axis), b1.q);
    V3<R> n2 = cross(aw, n1);
    V3<R> r1 = rotate(j.la1, b1.q), r2 = rotate(j.la2, b2.q);
    V3<R> p1 = b1.pos + r1, p2 = b2.pos + r2;
    V3<R> u = p2 - p1;
    J[0] = -n1; J[1] = -cross(r1 + u, n1); J[2] = n1; J[3] = cross(r2, n1);
    J[4] = -n2; J[5] = -cross(r1 + u, n2); J[6] = n2; J[7] = cross(r2, n2);
    J[8] = -aw; J[9] = -cross(r1 + u, aw); J[10] = aw; J[11] = cross(r2, aw);
    return V3<R>(dot(u, n1), dot(u, n2), dot(u, aw));
}
template <class R> void line_apply(Body<R>& b1, Body<R>& b2, const V3<R>* J, V3<R> a) {
    if (b1.motion == DYNAMIC) {
        b1.vel = b1.vel + cmul(J[0] * a.x + J[4] * a.y + J[8] * a.z, b1.inv_mass_vec);
        b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, J[1] * a.x + J[5] * a.y + J[9] * a.z);
    }
    if (b2.motion == DYNAMIC) {
        b2.vel = b2.vel + cmul(J[2] * a.x + J[6] * a.y + J[10] * a.z, b2.inv_mass_vec);
        b2.angvel = b2.angvel + sym_mul(b2.inv_inertia_world, J[3] * a.x + J[7] * a.y + J[11] * a.z);
    }
}
// PointOnLine.PrepareForIterationPointOnLine (PointOnLine.cs:149-300)
template <class R> void line_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> J[12];
    V3<R> err = line_jacobian(j, b1, b2, J);
    const Sym3<R>& I1 = b1.inv_inertia_world;
    const Sym3<R>& I2 = b2.inv_inertia_world;
    const V3<R> m1 = b1.inv_mass_vec, m2 = b2.inv_mass_vec;
    j.clamp = 0;
    Mat<R> M = Mat<R>::ident();
    M.a[0][0] = dot(cmul(J[0], m1), J[0]) + dot(cmul(J[2], m2), J[2]) + dot(sym_mul(I1, J[1]), J[1]) + dot(sym_mul(I2, J[3]), J[3]);
    M.a[1][1] = dot(cmul(J[4], m1), J[4]) + dot(cmul(J[6], m2), J[6]) + dot(sym_mul(I1, J[5]), J[5]) + dot(sym_mul(I2, J[7]), J[7]);
    M.a[0][1] = dot(sym_mul(I1, J[1]), J[5]) + dot(sym_mul(I2, J[3]), J[7]);
    M.a[1][0] = dot(sym_mul(I1, J[5]), J[1]) + dot(sym_mul(I2, J[7]), J[3]);
    R c12 = dot(cmul(J[0], m1), J[4]) + dot(cmul(J[2], m2), J[6]);
    M.a[0][1] += c12;
    M.a[1][0] += c12;
    if (j.min_angle >= j.max_angle) { err.z -= (R)0.5 * j.min_angle + (R)0.5 * j.max_angle; j.clamp = 3; }
    else if (err.z >= j.max_angle) { err.z -= j.max_angle; j.clamp = 1; }
    else if (err.z <= j.min_angle) { err.z -= j.min_angle; j.clamp = 2; }
    else j.acc.z = 0;
    if (j.clamp != 0) {
        M.a[2][2] = dot(cmul(J[8], m1), J[8]) + dot(cmul(J[10], m2), J[10]) + dot(sym_mul(I1, J[9]), J[9]) + dot(sym_mul(I2, J[11]), J[11]);
        M.a[0][2] = dot(sym_mul(I1, J[1]), J[9]) + dot(sym_mul(I2, J[3]), J[11]);
        M.a[2][0] = dot(sym_mul(I1, J[9]), J[1]) + dot(sym_mul(I2, J[11]), J[3]);
        M.a[1][2] = dot(sym_mul(I1, J[5]), J[9]) + dot(sym_mul(I2, J[7]), J[11]);
        M.a[2][1] = dot(sym_mul(I1, J[9]), J[5]) + dot(sym_mul(I2, J[11]), J[7]);
        R c13 = dot(cmul(J[0], m1), J[8]) + dot(cmul(J[2], m2), J[10]);
        R c23 = dot(cmul(J[4], m1), J[8]) + dot(cmul(J[6], m2), J[10]);
        M.a[0][2] += c13; M.a[2][0] += c13;
        M.a[1][2] += c23; M.a[2][1] += c23;
    }
    M.a[0][0] += j.softness * ts.inv_sub_dt;
    M.a[1][1] += j.softness * ts.inv_sub_dt;
    M.a[2][2] += j.limit_softness * ts.inv_sub_dt;
    if (j.clamp == 1 || j.clamp == 2) {
        j.bilateral = inverse_bilateral(M);
        j.coupling_x = M.a[0][2];
        j.coupling_y = M.a[1][2];
    }
    if (j.clamp == 0) M.a[2][2] = 0;
    j.eff = inverse_symmetric(M);
    j.bias = err * ts.inv_dt;
    j.bias.x *= j.bias_factor;
    j.bias.y *= j.bias_factor;
    j.bias.z *= j.limit_bias;
    if (j.clamp == 1) j.acc.z = net_min((R)0, j.acc.z);
    else if (j.clamp == 2) j.acc.z = net_max((R)0, j.acc.z);
    line_apply(b1, b2, J, j.acc);
}
// PointOnLine.IteratePointOnLine (PointOnLine.cs:372-465)
template <class R> void line_iterate(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> J[12];
    line_jacobian(j, b1, b2, J);
    V3<R> jv(dot(J[0], b1.vel) + dot(J[1], b1.angvel) + dot(J[2], b2.vel) + dot(J[3], b2.angvel),
             dot(J[4], b1.vel) + dot(J[5], b1.angvel) + dot(J[6], b2.vel) + dot(J[7], b2.angvel),
             dot(J[8], b1.vel) + dot(J[9], b1.angvel) + dot(J[10], b2.vel) + dot(J[11], b2.angvel));
    V3<R> sv = j.acc * ts.inv_sub_dt;
    sv.x *= j.softness;
    sv.y *= j.softness;
    sv.z *= j.limit_softness;
    V3<R> res = jv + j.bias + sv;
    V3<R> lambda = -(R)1.0 * mvec(j.eff, res);
    V3<R> orig = j.acc;
    j.acc = j.acc + lambda;
    if ((j.clamp == 1 && j.acc.z > 0) || (j.clamp == 2 && j.acc.z < 0)) {
        lambda.z = -orig.z;
        R x = res.x + j.coupling_x * lambda.z;
        R y = res.y + j.coupling_y * lambda.z;
        lambda.x = -(j.bilateral.x * x + j.bilateral.y * y);
        lambda.y = -(j.bilateral.y * x + j.bilateral.z * y);
        j.acc.x = orig.x + lambda.x;
        j.acc.y = orig.y + lambda.y;
        j.acc.z = 0;
    } else if (j.clamp == 0) {
        j.acc.z = 0;
        orig.z = 0;
    }
    line_apply(b1, b2, J, j.acc - orig);
}

// ---- EllipticalConeLimit (Dynamics/Constraints/EllipticalConeLimit.cs) -----------------------
// EllipticalConeLimit.Initialize (EllipticalConeLimit.cs:92-126) and SetLimits (:163-176): the
// cone axes of both bodies, a reference direction of body 1 made perpendicular to its axis,
// the swing limits along the reference [min1, max1] and across it [min2, max2]
template <class R> void elliptical_init(Joint<R>& j, const std::vector<Body<R>>& b, V3<R> ax1, V3<R> ax2, V3<R> ref,
                                        R min1, R max1, R min2, R max2) {
    j.kind = ELLIPTICALCONELIMIT;
    ax1 = normalize(ax1);
    ax2 = normalize(ax2);
    ref = normalize(ref);
    ref = ref - ax1 * dot(ax1, ref);
    ref = normalize(ref);
    j.la1 = rotate_inv(ax1, b[j.b1].q);
    j.la2 = rotate_inv(ax2, b[j.b2].q);
    j.target_pos = rotate_inv(ref, b[j.b1].q);
    j.softness = (R)0.001;
    j.bias_factor = (R)0.2;
    j.jr[0] = V3<R>();
    j.min_angle = min1; j.max_angle = max1;
    j.min_angle2 = min2; j.max_angle2 = max2;
    j.acc.x = 0;
    j.clamp = 0;
}
// EllipticalConeLimit.EllipseRadius (EllipticalConeLimit.cs:257-267): the radius of the
// ellipse with semiaxes a, b at an azimuth, and its logarithmic azimuth derivative
template <class R> R ellipse_radius(R a, R b, R c, R s, R& derivative) {
    R scale = net_min(a, b);
    R u = scale / a;
    R v = scale / b;
    R sq = c * c * u * u + s * s * v * v;
    derivative = c * s * (v * v - u * u) / sq;
    return scale / std::sqrt(sq);
}
// EllipticalConeLimit.GetSwing (EllipticalConeLimit.cs:206-221): the swing along the
// reference and across it
template <class R> void elliptical_swing(const Joint<R>& j, const std::vector<Body<R>>& bodies, R& along, R& across) {
    const Body<R>& b1 = bodies[j.b1];
    const Body<R>& b2 = bodies[j.b2];
    V3<R> axis = rotate(j.la1, b1.q);
    V3<R> reference = rotate(j.target_pos, b1.q);
    V3<R> other = cross(axis, reference);
    V3<R> target = rotate(j.la2, b2.q);
    R x = dot(target, reference);
    R y = dot(target, other);
    R sine = std::sqrt(x * x + y * y);
    R angle = StableMath<R>::atan2(sine, dot(target, axis));
    R factor = sine > 0 ? angle / sine : (R)0;
    along = sine > 0 ? x * factor : angle;
    across = y * factor;
}
template <class R> void elliptical_apply(Body<R>& b1, Body<R>& b2, V3<R> jac, R a) {
    if (b1.motion == DYNAMIC) b1.angvel = b1.angvel + sym_mul(b1.inv_inertia_world, a * jac);
    if (b2.motion == DYNAMIC) b2.angvel = b2.angvel - sym_mul(b2.inv_inertia_world, a * jac);
}
// EllipticalConeLimit.PrepareForIterationEllipticalConeLimit (EllipticalConeLimit.cs:269-392)
template <class R> void elliptical_prepare(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    V3<R> axis = rotate(j.la1, b1.q);
    V3<R> reference = rotate(j.target_pos, b1.q);
    V3<R> other = cross(axis, reference);
    V3<R> target = rotate(j.la2, b2.q);
    R x = dot(target, reference);
    R y = dot(target, other);
    R z = dot(target, axis);
    R sine = std::sqrt(x * x + y * y);
    R angle = StableMath<R>::atan2(sine, z);
    R ca, sa;
    if (sine > 0) {
        ca = x / sine;
        sa = y / sine;
    } else {
        Sym3<R> I(b1.inv_inertia_world.m11 + b2.inv_inertia_world.m11, b1.inv_inertia_world.m12 + b2.inv_inertia_world.m12,
                  b1.inv_inertia_world.m13 + b2.inv_inertia_world.m13, b1.inv_inertia_world.m22 + b2.inv_inertia_world.m22,
                  b1.inv_inertia_world.m23 + b2.inv_inertia_world.m23, b1.inv_inertia_world.m33 + b2.inv_inertia_world.m33);
        bool use_ref = dot(sym_mul(I, other), other) >= dot(sym_mul(I, reference), reference);
        ca = use_ref ? (R)1 : (R)0;
        sa = use_ref ? (R)0 : (R)1;
    }
    R derivative;
    R outer = ellipse_radius(j.max_angle, j.max_angle2, ca, sa, derivative);
    bool fixed_cone = j.min_angle == j.max_angle && j.min_angle2 == j.max_angle2;
    R boundary = outer;
    int clamp = 0;
    if (fixed_cone) clamp = 3;
    else if (angle >= outer) clamp = 1;
    else if (j.min_angle > 0) {
        R inner_d;
        R inner = ellipse_radius(j.min_angle, j.min_angle2, ca, sa, inner_d);
        if (angle <= inner) {
            clamp = 2;
            boundary = inner;
            derivative = inner_d;
        }
    }
    int previous = j.clamp;
    j.clamp = clamp;
    if (clamp == 0) {
        j.acc.x = 0;
        return;
    }
    V3<R> tilt = ca * reference + sa * other;
    V3<R> azimuth = cross(axis, tilt);
    V3<R> angle_dir = z * tilt - sine * axis;
    R az = sine > 0 ? angle / sine * derivative : (R)0;
    R scale = net_max((R)1, std::fabs(az));
    V3<R> jac = -azimuth * ((R)1 / scale) + (az / scale) * angle_dir;
    R inv_len = (R)1 / std::sqrt(dot(jac, jac));
    jac = jac * inv_len;
    inv_len /= scale;
    if (previous != clamp || dot(j.jr[0], jac) < 0) j.acc.x = 0;
    j.jr[0] = jac;
    if (clamp == 1) j.acc.x = net_min(j.acc.x, (R)0);
    else if (clamp == 2) j.acc.x = net_max(j.acc.x, (R)0);
    R mass = dot(sym_mul(b1.inv_inertia_world, jac), jac) + dot(sym_mul(b2.inv_inertia_world, jac), jac) +
             j.softness * ts.inv_sub_dt;
    j.eff1 = mass > 0 ? (R)1 / mass : (R)0;
    if (j.eff1 == 0) j.acc.x = 0;
    j.bias.x = (angle - boundary) * inv_len * j.bias_factor * ts.inv_dt;
    elliptical_apply(b1, b2, jac, j.acc.x);
}
// EllipticalConeLimit.IterateEllipticalConeLimit (EllipticalConeLimit.cs:394-429)
template <class R> void elliptical_iterate(Joint<R>& j, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    if (j.clamp == 0) return;
    Body<R>& b1 = bodies[j.b1];
    Body<R>& b2 = bodies[j.b2];
    R jv = dot(b1.angvel - b2.angvel, j.jr[0]);
    R lambda = -j.eff1 * (jv + j.bias.x + j.acc.x * j.softness * ts.inv_sub_dt);
    R old = j.acc.x;
    j.acc.x = j.acc.x + lambda;
    if (j.clamp == 1) j.acc.x = net_min(j.acc.x, (R)0);
    else if (j.clamp == 2) j.acc.x = net_max(j.acc.x, (R)0);
    elliptical_apply(b1, b2, j.jr[0], j.acc.x - old);
}

template <class R> void joint_prepare(Joint<R>& j, std::vector<Body<R>>& b, const TimeStep<R>& ts) {
    switch (j.kind) {
        case BALLSOCKET: ballsocket_prepare(j, b, ts); break;
        case HINGEANGLE: hinge_prepare(j, b, ts); break;
        case DISTANCELIMIT: distance_prepare(j, b, ts); break;
        case CONELIMIT: cone_prepare(j, b, ts); break;
        case FIXEDANGLE: fixed_prepare(j, b, ts); break;
        case POINTONPLANE: plane_prepare(j, b, ts); break;
        case ANGULARMOTOR: case LINEARMOTOR: motor_prepare(j, b, ts); break;
        case ANGULARSERVO: angular_servo_prepare(j, b, ts); break;
        case LINEARSERVO: linear_servo_prepare(j, b, ts); break;
        case LINEARAXISSERVO: linear_axis_servo_prepare(j, b, ts); break;
        case TWISTSERVO: twist_servo_prepare(j, b, ts); break;
        case POINTONLINE: line_prepare(j, b, ts); break;
        case ELLIPTICALCONELIMIT: elliptical_prepare(j, b, ts); break;
        default: twist_prepare(j, b, ts); break;
    }
}
template <class R> void joint_iterate(Joint<R>& j, std::vector<Body<R>>& b, const TimeStep<R>& ts) {
    switch (j.kind) {
        case BALLSOCKET: ballsocket_iterate(j, b, ts); break;
        case HINGEANGLE: hinge_iterate(j, b, ts); break;
        case DISTANCELIMIT: distance_iterate(j, b, ts); break;
        case CONELIMIT: cone_iterate(j, b, ts); break;
        case FIXEDANGLE: fixed_iterate(j, b, ts); break;
        case POINTONPLANE: distance_iterate(j, b, ts); break;   // PointOnPlane.cs:218-256: the same one-row update
        case ANGULARMOTOR: case LINEARMOTOR: motor_iterate(j, b, ts); break;
        case ANGULARSERVO: angular_servo_iterate(j, b, ts); break;
        case LINEARSERVO: linear_servo_iterate(j, b, ts); break;
        case LINEARAXISSERVO: linear_axis_servo_iterate(j, b, ts); break;
        case TWISTSERVO: twist_servo_iterate(j, b, ts); break;
        case POINTONLINE: line_iterate(j, b, ts); break;
        case ELLIPTICALCONELIMIT: elliptical_iterate(j, b, ts); break;
        default: twist_iterate(j, b, ts); break;
    }
}

}  // namespace jor
