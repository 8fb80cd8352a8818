// Device math for the contact pipeline.  Operation order follows the reference's
// linear-math code (src/Jitter2/LinearMath/*.cs); the library is compiled with
// -fmad=false and IEEE division/sqrt so that FP32 results round like .NET's
// non-fused float arithmetic.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define JG_HD __host__ __device__ __forceinline__

struct v3 { float x, y, z; };
struct q4 { float x, y, z, w; };
struct sym6 { float m11, m12, m13, m22, m23, m33; };

JG_HD v3 mk3(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
JG_HD v3 mk3(float a) { return mk3(a, a, a); }
JG_HD v3 mk3(float4 a) { return mk3(a.x, a.y, a.z); }
JG_HD q4 mkq(float4 a) { q4 q; q.x = a.x; q.y = a.y; q.z = a.z; q.w = a.w; return q; }
JG_HD float4 f4(v3 a, float w) { return make_float4(a.x, a.y, a.z, w); }
JG_HD float4 f4(q4 a) { return make_float4(a.x, a.y, a.z, a.w); }
JG_HD v3 operator+(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
JG_HD v3 operator-(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
JG_HD v3 operator-(v3 a) { return mk3(-a.x, -a.y, -a.z); }
JG_HD v3 operator*(v3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
JG_HD v3 operator*(float s, v3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
JG_HD bool operator==(v3 a, v3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
JG_HD float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
JG_HD v3 cross(v3 a, v3 b) { return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
JG_HD float len2(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
JG_HD v3 cmul(v3 a, v3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
JG_HD v3 vmin(v3 a, v3 b) { return mk3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
JG_HD v3 vmax(v3 a, v3 b) { return mk3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
// JVector.Normalize (JVector.cs:600-607)
JG_HD v3 normalize(v3 v) {
    float n2 = v.x * v.x + v.y * v.y + v.z * v.z;
    float inv = 1.0f / sqrtf(n2);
    return mk3(v.x * inv, v.y * inv, v.z * inv);
}
// JVector.NormalizeSafe (JVector.cs:561-567)
JG_HD v3 normalize_safe(v3 v, float eps2) {
    float n2 = v.x * v.x + v.y * v.y + v.z * v.z;
    if (n2 < eps2) return mk3(0.f);
    float inv = 1.0f / sqrtf(n2);
    return inv * v;
}
// JVector.Transform(v, quaternion) (JVector.cs:326-338)
JG_HD v3 rotate(v3 v, q4 q) {
    float n0 = 2.0f * (q.y * v.z - q.z * v.y);
    float n1 = 2.0f * (q.z * v.x - q.x * v.z);
    float n2 = 2.0f * (q.x * v.y - q.y * v.x);
    float n00 = q.y * n2 - q.z * n1;
    float n11 = q.z * n0 - q.x * n2;
    float n22 = q.x * n1 - q.y * n0;
    return mk3(v.x + q.w * n0 + n00, v.y + q.w * n1 + n11, v.z + q.w * n2 + n22);
}
// JVector.ConjugatedTransform (JVector.cs:347-360)
JG_HD v3 rotate_inv(v3 v, q4 q) {
    float n0 = 2.0f * (q.z * v.y - q.y * v.z);
    float n1 = 2.0f * (q.x * v.z - q.z * v.x);
    float n2 = 2.0f * (q.y * v.x - q.x * v.y);
    float n00 = q.z * n1 - q.y * n2;
    float n11 = q.x * n2 - q.z * n0;
    float n22 = q.y * n0 - q.x * n1;
    return mk3(v.x + q.w * n0 + n00, v.y + q.w * n1 + n11, v.z + q.w * n2 + n22);
}
// JQuaternion.Multiply (JQuaternion.cs:353-369)
JG_HD q4 qmul(q4 a, q4 b) {
    q4 o;
    o.w = a.w * b.w - (a.x * b.x + a.y * b.y + a.z * b.z);
    o.x = a.w * b.x + b.w * a.x + a.y * b.z - a.z * b.y;
    o.y = a.w * b.y + b.w * a.y + a.z * b.x - a.x * b.z;
    o.z = a.w * b.z + b.w * a.z + a.x * b.y - a.y * b.x;
    return o;
}
JG_HD q4 qconj(q4 a) { q4 o; o.x = -a.x; o.y = -a.y; o.z = -a.z; o.w = a.w; return o; }
JG_HD q4 qnormalize(q4 v) {
    float n2 = v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w;
    float inv = 1.0f / sqrtf(n2);
    q4 o; o.x = v.x * inv; o.y = v.y * inv; o.z = v.z * inv; o.w = v.w * inv;
    return o;
}
// JQuaternion.GetBasisY (JQuaternion.cs:233-240)
JG_HD v3 basis_y(q4 q) {
    return mk3(2.0f * (q.x * q.y - q.z * q.w), 1.0f - 2.0f * (q.x * q.x + q.z * q.z), 2.0f * (q.y * q.z + q.x * q.w));
}
struct m33 { float m[3][3]; };
// JMatrix.CreateFromQuaternion (JMatrix.cs:553-569)
JG_HD m33 mat_from_quat(q4 q) {
    float r = q.w, i = q.x, j = q.y, k = q.z;
    m33 o;
    o.m[0][0] = 1.0f - 2.0f * (j * j + k * k);
    o.m[0][1] = 2.0f * (i * j - k * r);
    o.m[0][2] = 2.0f * (i * k + j * r);
    o.m[1][0] = 2.0f * (i * j + k * r);
    o.m[1][1] = 1.0f - 2.0f * (i * i + k * k);
    o.m[1][2] = 2.0f * (j * k - i * r);
    o.m[2][0] = 2.0f * (i * k - j * r);
    o.m[2][1] = 2.0f * (j * k + i * r);
    o.m[2][2] = 1.0f - 2.0f * (i * i + j * j);
    return o;
}
JG_HD v3 mat_mul(const m33& M, v3 v) {
    return mk3(v.x * M.m[0][0] + v.y * M.m[0][1] + v.z * M.m[0][2],
               v.x * M.m[1][0] + v.y * M.m[1][1] + v.z * M.m[1][2],
               v.x * M.m[2][0] + v.y * M.m[2][1] + v.z * M.m[2][2]);
}
JG_HD v3 mat_tmul(const m33& M, v3 v) {
    return mk3(v.x * M.m[0][0] + v.y * M.m[1][0] + v.z * M.m[2][0],
               v.x * M.m[0][1] + v.y * M.m[1][1] + v.z * M.m[2][1],
               v.x * M.m[0][2] + v.y * M.m[1][2] + v.z * M.m[2][2]);
}
JG_HD m33 mat_abs(const m33& M) {
    m33 o;
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.m[i][j] = fabsf(M.m[i][j]);
    return o;
}
// JVector.Transform(v, JSymmetricMatrix) (JVector.cs:233-242) and
// Contact.TransformSymmetricInertia (Contact.cs:1027-1036): same expression order.
JG_HD v3 sym_mul(const sym6& M, v3 v) {
    return mk3(v.x * M.m11 + v.y * M.m12 + v.z * M.m13,
               v.x * M.m12 + v.y * M.m22 + v.z * M.m23,
               v.x * M.m13 + v.y * M.m23 + v.z * M.m33);
}
// JSymmetricMatrix.Transform(S, T) = T S T^T (JSymmetricMatrix.cs:247-260)
JG_HD sym6 sym_transform(const sym6& S, const m33& T) {
    v3 r1 = mk3(T.m[0][0], T.m[0][1], T.m[0][2]);
    v3 r2 = mk3(T.m[1][0], T.m[1][1], T.m[1][2]);
    v3 r3 = mk3(T.m[2][0], T.m[2][1], T.m[2][2]);
    v3 p1 = sym_mul(S, r1), p2 = sym_mul(S, r2), p3 = sym_mul(S, r3);
    sym6 o;
    o.m11 = dot(p1, r1); o.m12 = dot(p1, r2); o.m13 = dot(p1, r3);
    o.m22 = dot(p2, r2); o.m23 = dot(p2, r3); o.m33 = dot(p3, r3);
    return o;
}
// MathHelper.SignBit (MathHelper.cs:28-38): +1 / -1 from the sign bit
JG_HD float sign_bit(float v) { return signbit(v) ? -1.0f : 1.0f; }
JG_HD float sgnf(float v) { return v > 0.f ? 1.f : (v < 0.f ? -1.f : 0.f); }
// MathHelper.CreateOrthonormal (MathHelper.cs:204-254)
JG_HD v3 create_orthonormal(v3 v) {
    float ax = fabsf(v.x), ay = fabsf(v.y), az = fabsf(v.z);
    if (ax <= ay && ax <= az) {
        float y = v.z, z = -v.y;
        float inv = 1.0f / sqrtf(y * y + z * z);
        return mk3(0.f, y * inv, z * inv);
    } else if (ay <= az) {
        float x = -v.z, z = v.x;
        float inv = 1.0f / sqrtf(x * x + z * z);
        return mk3(x * inv, 0.f, z * inv);
    }
    float x = v.y, y = -v.x;
    float inv = 1.0f / sqrtf(x * x + y * y);
    return mk3(x * inv, y * inv, 0.f);
}

// The reference's own polynomial trigonometry (LinearMath/StableMath.cs:21-314), so
// angle-dependent decisions (the manifold's angular ordering, rotation quaternions)
// see the same values as the reference.
struct StableMathF {
    static constexpr float Pi = 3.141592653589793238462643383279502884f;
    static constexpr float HalfPi = 1.570796326794896619231321691639751442f;
    static constexpr float QuarterPi = 0.785398163397448309615660845819875721f;
    static constexpr float TwoPi = 6.283185307179586476925286766559005768f;
    static constexpr float TanPiOver8 = 0.414213562373095048801688724209698079f;
    JG_HD static int floor_to_int(float v) { int i = (int)v; return v < (float)i ? i - 1 : i; }
    JG_HD static float sin_poly(float x) {
        float x2 = x * x;
        float p = -(float)(1.0 / 6227020800.0);
        p = p * x2 + (float)(1.0 / 39916800.0);
        p = p * x2 - (float)(1.0 / 362880.0);
        p = p * x2 + (float)(1.0 / 5040.0);
        p = p * x2 - (float)(1.0 / 120.0);
        p = p * x2 + (float)(1.0 / 6.0);
        p = p * x2 - 1.0f;
        return -x * p;
    }
    JG_HD static float cos_poly(float x) {
        float x2 = x * x;
        float p = -(float)(1.0 / 479001600.0);
        p = p * x2 + (float)(1.0 / 3628800.0);
        p = p * x2 - (float)(1.0 / 40320.0);
        p = p * x2 + (float)(1.0 / 720.0);
        p = p * x2 - (float)(1.0 / 24.0);
        p = p * x2 + (float)(1.0 / 2.0);
        p = p * x2 - 1.0f;
        return -p;
    }
    JG_HD static void sincos(float a, float& s, float& c) {
        if (a >= -QuarterPi && a <= QuarterPi) { s = sin_poly(a); c = cos_poly(a); return; }
        int periods = floor_to_int((a + Pi) / TwoPi);
        a -= (float)periods * TwoPi;
        if (a > Pi) a -= TwoPi;
        else if (a <= -Pi) a += TwoPi;
        int q = floor_to_int((a + QuarterPi) / HalfPi);
        float r = a - (float)q * HalfPi;
        q &= 3;
        float sn = sin_poly(r), cs = cos_poly(r);
        if (q == 0) { s = sn; c = cs; }
        else if (q == 1) { s = cs; c = -sn; }
        else if (q == 2) { s = -sn; c = -cs; }
        else { s = -cs; c = sn; }
    }
    JG_HD static float atan_taylor(float v) {
        float x2 = v * v;
        float p = (float)(1.0 / 17.0);
        p = p * x2 - (float)(1.0 / 15.0);
        p = p * x2 + (float)(1.0 / 13.0);
        p = p * x2 - (float)(1.0 / 11.0);
        p = p * x2 + (float)(1.0 / 9.0);
        p = p * x2 - (float)(1.0 / 7.0);
        p = p * x2 + (float)(1.0 / 5.0);
        p = p * x2 - (float)(1.0 / 3.0);
        p = p * x2 + 1.0f;
        return v * p;
    }
    JG_HD static float atan(float v) {
        float sign = 1.f;
        if (v < 0.f) { v = -v; sign = -1.f; }
        float r;
        if (v > 1.0f) {
            float w = 1.0f / v;
            float inner = w > TanPiOver8 ? QuarterPi + atan_taylor((w - 1.0f) / (w + 1.0f)) : atan_taylor(w);
            r = HalfPi - inner;
        } else if (v > TanPiOver8) {
            r = QuarterPi + atan_taylor((v - 1.0f) / (v + 1.0f));
        } else {
            r = atan_taylor(v);
        }
        return sign * r;
    }
    JG_HD static float atan2(float y, float x) {
        if (x > 0.f) return atan(y / x);
        if (x < 0.f) return y >= 0.f ? atan(y / x) + Pi : atan(y / x) - Pi;
        if (y > 0.f) return HalfPi;
        if (y < 0.f) return -HalfPi;
        return 0.f;
    }
};

// MathHelper.RotationQuaternion (MathHelper.cs:47-78)
JG_HD q4 rotation_quaternion(v3 omega, float dt) {
    float angle = sqrtf(len2(omega));
    float theta = angle * dt;
    q4 o;
    if (theta < 1e-3f) {
        float theta2 = theta * theta;
        float scale = 0.5f * dt * (1.0f - theta2 / 24.0f);
        v3 a = omega * scale;
        o.x = a.x; o.y = a.y; o.z = a.z; o.w = 1.0f - (1.0f / 8.0f) * theta2;
        return o;
    }
    float half = 0.5f * angle * dt;
    float s, c;
    StableMathF::sincos(half, s, c);
    float scale = s / angle;
    v3 a = omega * scale;
    o.x = a.x; o.y = a.y; o.z = a.z; o.w = c;
    return o;
}
