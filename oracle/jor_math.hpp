// Oracle (test infrastructure only): CPU restatement of the Jitter2 linear-math subset
// used by the per-step contact pipeline.  Templated on the reference's `Real`
// (float = Jitter2, double = Jitter2.Double, src/Jitter2/Precision.cs:14-28).
// Compile with -ffp-contract=off so float arithmetic follows .NET's non-fused IEEE
// evaluation.  Expression order follows the cited reference lines.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <algorithm>

namespace jor {

template <class R> struct V3 {
    R x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(R a, R b, R c) : x(a), y(b), z(c) {}
    explicit V3(R a) : x(a), y(a), z(a) {}
};
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> inline bool operator==(V3<R> a, V3<R> b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
// JVector.Dot / operator* (LinearMath/JVector.cs)
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// JVector.Cross / operator% (LinearMath/JVector.cs)
template <class R> inline V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> inline R len2(V3<R> a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
// JVector.Multiply(vector, vector): component-wise
template <class R> inline V3<R> cmul(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline R rsq(R v) { return (R)1.0 / std::sqrt(v); }
// JVector.Normalize (JVector.cs:600-607)
template <class R> inline V3<R> normalize(V3<R> v) {
    R n2 = v.x * v.x + v.y * v.y + v.z * v.z;
    R inv = (R)1.0 / std::sqrt(n2);
    return {v.x * inv, v.y * inv, v.z * inv};
}
// JVector.NormalizeSafe (JVector.cs:561-567)
template <class R> inline V3<R> normalize_safe(V3<R> v, R eps2) {
    R n2 = v.x * v.x + v.y * v.y + v.z * v.z;
    if (n2 < eps2) return V3<R>();
    R inv = (R)1.0 / std::sqrt(n2);
    return inv * v;
}
template <class R> inline V3<R> vmin(V3<R> a, V3<R> b) { return {std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)}; }
template <class R> inline V3<R> vmax(V3<R> a, V3<R> b) { return {std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; }

template <class R> struct Q4 {
    R x, y, z, w;
    Q4() : x(0), y(0), z(0), w(1) {}
    Q4(R a, R b, R c, R d) : x(a), y(b), z(c), w(d) {}
};
// JVector.Transform(vector, quaternion) (JVector.cs:326-338)
template <class R> inline V3<R> rotate(V3<R> v, Q4<R> q) {
    R n0 = (R)2.0 * (q.y * v.z - q.z * v.y);
    R n1 = (R)2.0 * (q.z * v.x - q.x * v.z);
    R n2 = (R)2.0 * (q.x * v.y - q.y * v.x);
    R n00 = q.y * n2 - q.z * n1;
    R n11 = q.z * n0 - q.x * n2;
    R n22 = q.x * n1 - q.y * n0;
    return {v.x + q.w * n0 + n00, v.y + q.w * n1 + n11, v.z + q.w * n2 + n22};
}
// JVector.ConjugatedTransform (JVector.cs:347-360)
template <class R> inline V3<R> rotate_inv(V3<R> v, Q4<R> q) {
    R n0 = (R)2.0 * (q.z * v.y - q.y * v.z);
    R n1 = (R)2.0 * (q.x * v.z - q.z * v.x);
    R n2 = (R)2.0 * (q.y * v.x - q.x * v.y);
    R n00 = q.z * n1 - q.y * n2;
    R n11 = q.x * n2 - q.z * n0;
    R n22 = q.y * n0 - q.x * n1;
    return {v.x + q.w * n0 + n00, v.y + q.w * n1 + n11, v.z + q.w * n2 + n22};
}
// JQuaternion.Multiply (JQuaternion.cs:353-369)
template <class R> inline Q4<R> qmul(Q4<R> a, Q4<R> b) {
    R r1 = a.w, i1 = a.x, j1 = a.y, k1 = a.z;
    R r2 = b.w, i2 = b.x, j2 = b.y, k2 = b.z;
    Q4<R> o;
    o.w = r1 * r2 - (i1 * i2 + j1 * j2 + k1 * k2);
    o.x = r1 * i2 + r2 * i1 + j1 * k2 - k1 * j2;
    o.y = r1 * j2 + r2 * j1 + k1 * i2 - i1 * k2;
    o.z = r1 * k2 + r2 * k1 + i1 * j2 - j1 * i2;
    return o;
}
template <class R> inline Q4<R> qconj(Q4<R> a) { return {-a.x, -a.y, -a.z, a.w}; }
// JQuaternion.ConjugateMultiply (JQuaternion.cs:378-394)
template <class R> inline Q4<R> qconjmul(Q4<R> a, Q4<R> b) { return qmul(qconj(a), b); }
// JQuaternion.Normalize (JQuaternion.cs:521-529)
template <class R> inline Q4<R> qnormalize(Q4<R> v) {
    R n2 = v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w;
    R inv = (R)1.0 / std::sqrt(n2);
    return {v.x * inv, v.y * inv, v.z * inv, v.w * inv};
}
// JQuaternion.GetBasisY (JQuaternion.cs:233-240)
template <class R> inline V3<R> basis_y(Q4<R> q) {
    return {(R)2.0 * (q.x * q.y - q.z * q.w), (R)1.0 - (R)2.0 * (q.x * q.x + q.z * q.z), (R)2.0 * (q.y * q.z + q.x * q.w)};
}

template <class R> struct M3 { R m[3][3]; };
// JMatrix.CreateFromQuaternion (JMatrix.cs:553-569)
template <class R> inline M3<R> mat_from_quat(Q4<R> q) {
    R r = q.w, i = q.x, j = q.y, k = q.z;
    M3<R> o;
    o.m[0][0] = (R)1.0 - (R)2.0 * (j * j + k * k);
    o.m[0][1] = (R)2.0 * (i * j - k * r);
    o.m[0][2] = (R)2.0 * (i * k + j * r);
    o.m[1][0] = (R)2.0 * (i * j + k * r);
    o.m[1][1] = (R)1.0 - (R)2.0 * (i * i + k * k);
    o.m[1][2] = (R)2.0 * (j * k - i * r);
    o.m[2][0] = (R)2.0 * (i * k - j * r);
    o.m[2][1] = (R)2.0 * (j * k + i * r);
    o.m[2][2] = (R)1.0 - (R)2.0 * (i * i + j * j);
    return o;
}
// JVector.Transform(vector, matrix) = M v (JVector.cs:290-299)
template <class R> inline V3<R> mat_mul(const M3<R>& M, V3<R> v) {
    return {v.x * M.m[0][0] + v.y * M.m[0][1] + v.z * M.m[0][2],
            v.x * M.m[1][0] + v.y * M.m[1][1] + v.z * M.m[1][2],
            v.x * M.m[2][0] + v.y * M.m[2][1] + v.z * M.m[2][2]};
}
// JVector.TransposedTransform = M^T v (JVector.cs:306-316)
template <class R> inline V3<R> mat_tmul(const M3<R>& M, V3<R> v) {
    return {v.x * M.m[0][0] + v.y * M.m[1][0] + v.z * M.m[2][0],
            v.x * M.m[0][1] + v.y * M.m[1][1] + v.z * M.m[2][1],
            v.x * M.m[0][2] + v.y * M.m[1][2] + v.z * M.m[2][2]};
}
template <class R> inline M3<R> mat_abs(const M3<R>& M) {
    M3<R> o;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.m[i][j] = std::abs(M.m[i][j]);
    return o;
}

// JSymmetricMatrix (LinearMath/JSymmetricMatrix.cs:20-40): M11 M12 M13 M22 M23 M33
template <class R> struct Sym3 {
    R m11, m12, m13, m22, m23, m33;
    Sym3() : m11(0), m12(0), m13(0), m22(0), m23(0), m33(0) {}
    Sym3(R a, R b, R c, R d, R e, R f) : m11(a), m12(b), m13(c), m22(d), m23(e), m33(f) {}
};
// JVector.Transform(vector, JSymmetricMatrix) (JVector.cs:233-242)
template <class R> inline V3<R> sym_mul(const Sym3<R>& M, V3<R> v) {
    return {v.x * M.m11 + v.y * M.m12 + v.z * M.m13,
            v.x * M.m12 + v.y * M.m22 + v.z * M.m23,
            v.x * M.m13 + v.y * M.m23 + v.z * M.m33};
}
// Contact.TransformSymmetricInertia (Contact.cs:1027-1036)
template <class R> inline V3<R> sym_mul_inertia(const Sym3<R>& M, V3<R> v) {
    return {v.x * M.m11 + v.y * M.m12 + v.z * M.m13,
            v.x * M.m12 + v.y * M.m22 + v.z * M.m23,
            v.x * M.m13 + v.y * M.m23 + v.z * M.m33};
}
// JSymmetricMatrix.Transform(matrix, transform) = T S T^T (JSymmetricMatrix.cs:247-260)
template <class R> inline Sym3<R> sym_transform(const Sym3<R>& S, const M3<R>& T) {
    V3<R> r1(T.m[0][0], T.m[0][1], T.m[0][2]);
    V3<R> r2(T.m[1][0], T.m[1][1], T.m[1][2]);
    V3<R> r3(T.m[2][0], T.m[2][1], T.m[2][2]);
    V3<R> p1 = sym_mul(S, r1), p2 = sym_mul(S, r2), p3 = sym_mul(S, r3);
    return Sym3<R>(dot(p1, r1), dot(p1, r2), dot(p1, r3), dot(p2, r2), dot(p2, r3), dot(p3, r3));
}
// JSymmetricMatrix.Determinant (JSymmetricMatrix.cs:104-109)
template <class R> inline R sym_det(const Sym3<R>& m) {
    return m.m11 * (m.m22 * m.m33 - m.m23 * m.m23) +
           m.m12 * (m.m23 * m.m13 - m.m12 * m.m33) +
           m.m13 * (m.m12 * m.m23 - m.m22 * m.m13);
}
template <class R> inline bool is_normal(R v) { return std::isnormal(v); }
// JSymmetricMatrix.TryInverseUnscaled (JSymmetricMatrix.cs:157-178)
template <class R> inline bool sym_try_inverse_unscaled(const Sym3<R>& m, Sym3<R>& out) {
    R idet = (R)1.0 / sym_det(m);
    if (!is_normal(idet)) { out = Sym3<R>(); return false; }
    R a11 = m.m22 * m.m33 - m.m23 * m.m23;
    R a12 = m.m13 * m.m23 - m.m12 * m.m33;
    R a13 = m.m12 * m.m23 - m.m22 * m.m13;
    R a22 = m.m11 * m.m33 - m.m13 * m.m13;
    R a23 = m.m13 * m.m12 - m.m23 * m.m11;
    R a33 = m.m11 * m.m22 - m.m12 * m.m12;
    out = Sym3<R>(a11 * idet, a12 * idet, a13 * idet, a22 * idet, a23 * idet, a33 * idet);
    return std::isfinite(out.m11) && std::isfinite(out.m12) && std::isfinite(out.m13) &&
           std::isfinite(out.m22) && std::isfinite(out.m23) && std::isfinite(out.m33);
}
// JSymmetricMatrix.Inverse (JSymmetricMatrix.cs:119-147)
template <class R> inline bool sym_inverse(const Sym3<R>& m, Sym3<R>& out) {
    if (sym_try_inverse_unscaled(m, out)) return true;
    R s = std::max(std::abs(m.m11), std::max(std::abs(m.m12), std::abs(m.m13)));
    s = std::max(s, std::max(std::abs(m.m22), std::max(std::abs(m.m23), std::abs(m.m33))));
    if (s > 0 && std::isfinite(s)) {
        Sym3<R> n(m.m11 / s, m.m12 / s, m.m13 / s, m.m22 / s, m.m23 / s, m.m33 / s);
        Sym3<R> inv;
        if (sym_try_inverse_unscaled(n, inv)) {
            out = Sym3<R>(inv.m11 / s, inv.m12 / s, inv.m13 / s, inv.m22 / s, inv.m23 / s, inv.m33 / s);
            return true;
        }
    }
    out = Sym3<R>();
    return false;
}

// MathHelper.SignBit (MathHelper.cs:28-38): +1 or -1 from the sign bit (-0 -> -1)
inline int sign_bit(float v) { return std::signbit(v) ? -1 : 1; }
inline int sign_bit(double v) { return std::signbit(v) ? -1 : 1; }
// Math.Sign: -1, 0, +1
template <class R> inline int sgn(R v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }

// MathHelper.CreateOrthonormal (MathHelper.cs:204-254)
template <class R> inline V3<R> create_orthonormal(V3<R> v) {
    R ax = std::abs(v.x), ay = std::abs(v.y), az = std::abs(v.z);
    V3<R> r;
    if (ax <= ay && ax <= az) {
        R y = v.z, z = -v.y;
        R inv = (R)1.0 / std::sqrt(y * y + z * z);
        r = V3<R>(0, y * inv, z * inv);
    } else if (ay <= az) {
        R x = -v.z, z = v.x;
        R inv = (R)1.0 / std::sqrt(x * x + z * z);
        r = V3<R>(x * inv, 0, z * inv);
    } else {
        R x = v.y, y = -v.x;
        R inv = (R)1.0 / std::sqrt(x * x + y * y);
        r = V3<R>(x * inv, y * inv, 0);
    }
    return r;
}

// StableMath (LinearMath/StableMath.cs:21-314): the reference's own polynomial
// sin/cos/atan2, restated so that angle-dependent branches and the manifold's angular
// ordering see the same values as the reference.
template <class R> struct StableMath {
    static constexpr R Pi = (R)3.141592653589793238462643383279502884;
    static constexpr R HalfPi = (R)1.570796326794896619231321691639751442;
    static constexpr R QuarterPi = (R)0.785398163397448309615660845819875721;
    static constexpr R TwoPi = (R)6.283185307179586476925286766559005768;
    static constexpr R TanPiOver8 = (R)0.414213562373095048801688724209698079;
    static int floor_to_int(R v) { int i = (int)v; return v < (R)i ? i - 1 : i; }
    static R reduce_angle(R a) {
        int periods = floor_to_int((a + Pi) / TwoPi);
        a -= (R)periods * TwoPi;
        if (a > Pi) a -= TwoPi;
        else if (a <= -Pi) a += TwoPi;
        return a;
    }
    static void reduce_quadrant(R a, int& quadrant, R& reduced) {
        a = reduce_angle(a);
        int q = floor_to_int((a + QuarterPi) / HalfPi);
        reduced = a - (R)q * HalfPi;
        quadrant = q & 3;
    }
    static R sin_poly(R x) {
        R x2 = x * x;
        R p = -(R)(1.0 / 6227020800.0);
        p = p * x2 + (R)(1.0 / 39916800.0);
        p = p * x2 - (R)(1.0 / 362880.0);
        p = p * x2 + (R)(1.0 / 5040.0);
        p = p * x2 - (R)(1.0 / 120.0);
        p = p * x2 + (R)(1.0 / 6.0);
        p = p * x2 - (R)1.0;
        return -x * p;
    }
    static R cos_poly(R x) {
        R x2 = x * x;
        R p = -(R)(1.0 / 479001600.0);
        p = p * x2 + (R)(1.0 / 3628800.0);
        p = p * x2 - (R)(1.0 / 40320.0);
        p = p * x2 + (R)(1.0 / 720.0);
        p = p * x2 - (R)(1.0 / 24.0);
        p = p * x2 + (R)(1.0 / 2.0);
        p = p * x2 - (R)1.0;
        return -p;
    }
    static void sincos(R a, R& s, R& c) {
        if (a >= -QuarterPi && a <= QuarterPi) { s = sin_poly(a); c = cos_poly(a); return; }
        int q; R r;
        reduce_quadrant(a, q, r);
        R sn = sin_poly(r), cs = cos_poly(r);
        switch (q) {
            case 0: s = sn; c = cs; break;
            case 1: s = cs; c = -sn; break;
            case 2: s = -sn; c = -cs; break;
            default: s = -cs; c = sn; break;
        }
    }
    static R atan_taylor(R v) {
        R x2 = v * v;
        R p = (R)(1.0 / 17.0);
        p = p * x2 - (R)(1.0 / 15.0);
        p = p * x2 + (R)(1.0 / 13.0);
        p = p * x2 - (R)(1.0 / 11.0);
        p = p * x2 + (R)(1.0 / 9.0);
        p = p * x2 - (R)(1.0 / 7.0);
        p = p * x2 + (R)(1.0 / 5.0);
        p = p * x2 - (R)(1.0 / 3.0);
        p = p * x2 + (R)1.0;
        return v * p;
    }
    static R atan(R v) {
        if (v < (R)0.0) return -atan(-v);
        if (v > (R)1.0) return HalfPi - atan((R)1.0 / v);
        if (v > TanPiOver8) return QuarterPi + atan_taylor((v - (R)1.0) / (v + (R)1.0));
        return atan_taylor(v);
    }
    static R atan2(R y, R x) {
        if (x > (R)0.0) return atan(y / x);
        if (x < (R)0.0) return y >= (R)0.0 ? atan(y / x) + Pi : atan(y / x) - Pi;
        if (y > (R)0.0) return HalfPi;
        if (y < (R)0.0) return -HalfPi;
        return (R)0.0;
    }
};

// MathHelper.RotationQuaternion (MathHelper.cs:47-78)
template <class R> inline Q4<R> rotation_quaternion(V3<R> omega, R dt) {
    R angle = std::sqrt(len2(omega));
    R theta = angle * dt;
    if (theta < (R)1e-3) {
        R theta2 = theta * theta;
        R scale = (R)0.5 * dt * ((R)1.0 - theta2 / (R)24.0);
        V3<R> a = omega * scale;
        R c = (R)1.0 - ((R)1.0 / (R)8.0) * theta2;
        return Q4<R>(a.x, a.y, a.z, c);
    }
    R half = (R)0.5 * angle * dt;
    R s, c;
    StableMath<R>::sincos(half, s, c);
    R scale = s / angle;
    V3<R> a = omega * scale;
    return Q4<R>(a.x, a.y, a.z, c);
}

}  // namespace jor
