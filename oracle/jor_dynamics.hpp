// Oracle (test infrastructure only): CPU restatement of Jitter2's contact cache, contact
// solver, body integration and per-step update, plus a world step that runs them in
// either the reference's deterministic order (World.Deterministic.cs:142-313: contacts
// sorted by arbiter key) or an externally supplied colour order (the GPU solver's).
//
// The contact-cache restatement (AddContact / SortCachedPoints) follows code the
// reference derived from the Bullet Physics Engine, zlib license:
//   Bullet Continuous Collision Detection and Physics Library Copyright (c) 2003-2006
//   Erwin Coumans https://bulletphysics.org
//   This software is provided 'as-is', without any express or implied warranty. In no
//   event will the authors be held liable for any damages arising from the use of this
//   software. Permission is granted to anyone to use this software for any purpose,
//   including commercial applications, and to alter it and redistribute it freely,
//   subject to the following restrictions: 1. The origin of this software must not be
//   misrepresented; you must not claim that you wrote the original software. If you use
//   this software in a product, an acknowledgment in the product documentation would be
//   appreciated but is not required. 2. Altered source versions must be plainly marked as
//   such, and must not be misrepresented as being the original software. 3. This notice
//   may not be removed or altered from any source distribution.
#pragma once
#include "jor_collision.hpp"
#include <map>
#include <unordered_map>
#include <vector>
#include <thread>
#include <atomic>
#include <mutex>
#include <functional>

namespace jor {

enum Motion { DYNAMIC = 0, KINEMATIC = 1, STATIC = 2 };

// RigidBodyData (Dynamics/RigidBody.cs:107-250) + the RigidBody fields Update reads.
template <class R> struct Body {
    V3<R> pos, vel, angvel, dvel, dangvel;
    Q4<R> q;
    Sym3<R> inv_inertia_world;
    V3<R> inv_mass_vec;
    int flags = 4;                  // bit 2 active, bit 3 gyroscopic, bits 4..9 locked axes
    int motion = DYNAMIC;
    Sym3<R> inv_inertia_local = Sym3<R>(1, 0, 0, 1, 0, 1);
    R inv_mass = 1;
    R friction = (R)0.2, restitution = 0;
    R lin_damp = (R)0.998, ang_damp = (R)0.995;
    V3<R> force, torque;
    bool gravity = true;
    bool speculative = false;       // RigidBody.EnableSpeculativeContacts
    int world = 0;
    // deactivation (RigidBody.cs:315, :398-400; Island.cs): time at rest, and the two island
    // flags kept per body (an island's flag is the OR over its bodies): MarkedAsActive and
    // membership of the active island partition
    R sleep_time = 0;
    R deactivation_time = (R)1.0;   // RigidBody.DeactivationTime (RigidBody.cs:400, :476-483)
    R sleep_lin2 = (R)0.1, sleep_ang2 = (R)0.1;  // squared rest thresholds (RigidBody.cs:398-399, :497-508)
    bool marked = true, island_active = true;
    bool active() const { return (flags & 4) != 0; }
    bool gyroscopic() const { return (flags & 8) != 0; }
    bool has_linear_locks() const { return (flags & (7 << 4)) != 0; }
    bool has_angular_locks() const { return (flags & (56 << 4)) != 0; }
    bool has_motion_locks() const { return (flags & (63 << 4)) != 0; }
    int allowed() const { return 63 ^ ((flags >> 4) & 63); }
};

template <class R> inline void restrict_linear(V3<R>& v, int axes) {
    if ((axes & 7) == 7) return;
    if ((axes & 1) == 0) v.x = 0;
    if ((axes & 2) == 0) v.y = 0;
    if ((axes & 4) == 0) v.z = 0;
}
template <class R> inline void restrict_angular(V3<R>& v, int axes) {
    if ((axes & 56) == 56) return;
    if ((axes & 8) == 0) v.x = 0;
    if ((axes & 16) == 0) v.y = 0;
    if ((axes & 32) == 0) v.z = 0;
}
// RigidBody.RestrictAngularMotion(ref JSymmetricMatrix) (RigidBody.cs:560-610)
template <class R> inline void restrict_inertia(Sym3<R>& I, int axes) {
    if ((axes & 56) == 0) { I = Sym3<R>(); return; }
    if ((axes & 8) == 0) {
        if (I.m11 > 0) { R xy = I.m12 / I.m11, xz = I.m13 / I.m11; I.m22 -= xy * I.m12; I.m23 -= xy * I.m13; I.m33 -= xz * I.m13; }
        I.m11 = I.m12 = I.m13 = 0;
    }
    if ((axes & 16) == 0) {
        if (I.m22 > 0) { R xy = I.m12 / I.m22, yz = I.m23 / I.m22; I.m11 -= xy * I.m12; I.m13 -= xy * I.m23; I.m33 -= yz * I.m23; }
        I.m12 = I.m22 = I.m23 = 0;
    }
    if ((axes & 32) == 0) {
        if (I.m33 > 0) { R xz = I.m13 / I.m33, yz = I.m23 / I.m33; I.m11 -= xz * I.m13; I.m12 -= xz * I.m23; I.m22 -= yz * I.m23; }
        I.m13 = I.m23 = I.m33 = 0;
    }
}
// RigidBody.UpdateWorldInertia (RigidBody.cs:903-923)
template <class R> inline void update_world_inertia(Body<R>& b) {
    if (b.motion == DYNAMIC) {
        M3<R> ori = mat_from_quat(b.q);
        b.inv_inertia_world = sym_transform(b.inv_inertia_local, ori);
        if (b.has_angular_locks()) restrict_inertia(b.inv_inertia_world, b.allowed());
        b.inv_mass_vec = V3<R>(b.inv_mass);
        restrict_linear(b.inv_mass_vec, b.allowed());
    } else {
        b.inv_inertia_world = Sym3<R>();
        b.inv_mass_vec = V3<R>();
    }
}

template <class R> struct TimeStep {
    R dt, sub_dt, inv_dt, inv_sub_dt;
    int substeps;
    // TimeStep (TimeStep.cs:36-46)
    TimeStep(R d, int n) : dt(d), sub_dt(d / n), inv_dt(d > 0 ? (R)1.0 / d : 0), substeps(n) {
        inv_sub_dt = sub_dt > 0 ? (R)1.0 / sub_dt : 0;
    }
};

// Contact (Dynamics/Contact.cs:585-1250)
template <class R> struct Contact {
    static constexpr R MaximumBias = (R)100.0, BiasFactor = (R)0.2, AllowedPenetration = (R)0.01, BreakThreshold = (R)0.02;
    enum { NewContact = 2, SkipWarmStart = 4 };
    int flag = 0;
    R bias = 0, penalty_bias = 0;
    V3<R> n, t1, t2;
    R mass[3] = {0, 0, 0};
    R acc[3] = {0, 0, 0};
    V3<R> pos1, pos2;       // local
    V3<R> rel1, rel2;       // world offsets
};

template <class R> struct ContactData {
    enum Mode { LinearBody1 = 1, AngularBody1 = 2, LinearBody2 = 4, AngularBody2 = 8 };
    unsigned usage = 0;
    int b1 = -1, b2 = -1;
    int key1 = -1, key2 = -1;
    R restitution = 0, friction = 0, spec_relax = (R)0.9;
    int mode = 0;
    Contact<R> c[4];
    int color = 0;
};

// Contact.Initialize (Contact.cs:703-759)
template <class R> void contact_initialize(ContactData<R>& cd, Contact<R>& c, std::vector<Body<R>>& bodies,
                                           V3<R> p1, V3<R> p2, V3<R> n, bool is_new) {
    Body<R>& b1 = bodies[cd.b1];
    Body<R>& b2 = bodies[cd.b2];
    c.rel1 = p1 - b1.pos;
    c.rel2 = p2 - b2.pos;
    c.pos1 = rotate_inv(c.rel1, b1.q);
    c.pos2 = rotate_inv(c.rel2, b2.q);
    if (!is_new) return;
    c.flag = Contact<R>::NewContact;
    c.acc[0] = c.acc[1] = c.acc[2] = 0;
    V3<R> dv = b2.vel - b1.vel;
    if (cd.mode == 0 || (cd.mode & (ContactData<R>::AngularBody1 | ContactData<R>::AngularBody2)) != 0) {
        dv = b2.vel + cross(b2.angvel, c.rel2);
        dv = dv - (b1.vel + cross(b1.angvel, c.rel1));
    }
    R rnv = dot(dv, n);
    c.bias = 0;
    if (rnv < (R)(-1.0)) c.bias = -cd.restitution * rnv;
    V3<R> t1 = dv - n * rnv;
    R num = len2(t1);
    if (num > (R)1e-12) {
        num = (R)1.0 / std::sqrt(num);
        t1 = t1 * num;
    } else {
        t1 = create_orthonormal(n);
    }
    V3<R> t2 = cross(t1, n);
    c.n = n; c.t1 = t1; c.t2 = t2;
}

// ContactData.CalcArea4Points / SelectCachedPointReplacementMask (Contact.cs:418-480)
template <class R> R area4(V3<R> p0, V3<R> p1, V3<R> p2, V3<R> p3) {
    V3<R> a0 = p0 - p1, a1 = p0 - p2, a2 = p0 - p3;
    V3<R> b0 = p2 - p3, b1 = p1 - p3, b2 = p1 - p2;
    V3<R> t0 = cross(a0, b0), t1 = cross(a1, b1), t2 = cross(a2, b2);
    return std::max(std::max(len2(t0), len2(t1)), len2(t2));
}
template <class R> unsigned replacement_mask(V3<R> np, V3<R> c0, V3<R> c1, V3<R> c2, V3<R> c3) {
    R ar[4] = {area4(np, c1, c2, c3), area4(np, c0, c2, c3), area4(np, c0, c1, c3), area4(np, c0, c1, c2)};
    const R eps = -(R)0.0001;
    R big = 0;
    unsigned mask = 0;
    if (ar[0] > big + eps) { big = ar[0]; mask = 1; }
    if (ar[1] > big + eps) { big = ar[1]; mask = 2; }
    if (ar[2] > big + eps) { big = ar[2]; mask = 4; }
    if (ar[3] > big + eps) { mask = 8; }
    return mask;
}

// ContactData.AddContact + SortCachedPoints (Contact.cs:329-416, :555-580)
template <class R> void add_contact(ContactData<R>& cd, std::vector<Body<R>>& bodies, V3<R> p1, V3<R> p2, V3<R> n) {
    if ((cd.usage & 15u) == 15u) {
        V3<R> rp1 = p1 - bodies[cd.b1].pos;
        unsigned mask = replacement_mask(rp1, cd.c[0].rel1, cd.c[1].rel1, cd.c[2].rel1, cd.c[3].rel1);
        int k = mask == 2 ? 1 : (mask == 4 ? 2 : (mask == 8 ? 3 : 0));
        contact_initialize(cd, cd.c[k], bodies, p1, p2, n, false);
        cd.usage |= mask;
        return;
    }
    int closest = -1;
    R dist = std::numeric_limits<R>::max();
    V3<R> rp1 = p1 - bodies[cd.b1].pos;
    for (int k = 0; k < 4; k++) {
        if ((cd.usage & (1u << k)) == 0) continue;
        R d = len2(cd.c[k].rel1 - rp1);
        if (d < dist) { dist = d; closest = k; }
    }
    if (dist < Contact<R>::BreakThreshold * Contact<R>::BreakThreshold) {
        contact_initialize(cd, cd.c[closest], bodies, p1, p2, n, false);
        return;
    }
    for (int k = 0; k < 4; k++) {
        if ((cd.usage & (1u << k)) == 0) {
            contact_initialize(cd, cd.c[k], bodies, p1, p2, n, true);
            cd.usage |= 1u << k;
            return;
        }
    }
}

// Contact.UpdatePosition (Contact.cs:762-797)
template <class R> bool contact_update_position(ContactData<R>& cd, Contact<R>& c, std::vector<Body<R>>& bodies) {
    Body<R>& b1 = bodies[cd.b1];
    Body<R>& b2 = bodies[cd.b2];
    c.rel1 = rotate(c.pos1, b1.q);
    V3<R> p1 = c.rel1 + b1.pos;
    c.rel2 = rotate(c.pos2, b2.q);
    V3<R> p2 = c.rel2 + b2.pos;
    V3<R> dist = p1 - p2;
    R pen = dot(dist, c.n);
    if (pen < -Contact<R>::BreakThreshold * (R)0.1) return false;
    dist = dist - pen * c.n;
    if (len2(dist) > Contact<R>::BreakThreshold * Contact<R>::BreakThreshold) return false;
    return true;
}
// ContactData.UpdatePosition (Contact.cs:238-264)
template <class R> void contactdata_update_position(ContactData<R>& cd, std::vector<Body<R>>& bodies) {
    cd.usage &= 15u;
    cd.usage |= cd.usage << 4;
    for (int k = 0; k < 4; k++)
        if ((cd.usage & (1u << k)) != 0 && !contact_update_position(cd, cd.c[k], bodies)) cd.usage &= ~(1u << k);
}

// Contact.PrepareForIteration, scalar path (Contact.cs:802-924); the SIMD path
// (:1039-1180) is bitwise identical (ReproducibilityTest.cs:58-105).
template <class R> void contact_prepare(ContactData<R>& cd, Contact<R>& c, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    R an = c.acc[0], at1 = c.acc[1], at2 = c.acc[2];
    bool skip = (c.flag & Contact<R>::SkipWarmStart) != 0;
    c.flag &= ~Contact<R>::SkipWarmStart;
    if (skip) { an = 0; at1 = 0; at2 = 0; }
    Body<R>& b1 = bodies[cd.b1];
    Body<R>& b2 = bodies[cd.b2];
    V3<R> n = c.n, t1 = c.t1, t2 = c.t2;
    V3<R> cr1 = rotate(c.pos1, b1.q);
    V3<R> cr2 = rotate(c.pos2, b2.q);
    V3<R> imv;
    if (cd.mode & ContactData<R>::LinearBody1) imv = b1.inv_mass_vec;
    if (cd.mode & ContactData<R>::LinearBody2) imv = imv + b2.inv_mass_vec;
    R im = imv.x;
    if ((c.flag & Contact<R>::NewContact) == 0) c.bias = 0;
    V3<R> p1 = cr1 + b1.pos, p2 = cr2 + b2.pos;
    V3<R> dist = p1 - p2;
    R pen = dot(dist, n);
    if (pen < -Contact<R>::BreakThreshold) c.bias = pen * ts.inv_dt * cd.spec_relax;
    c.flag &= ~Contact<R>::NewContact;
    R kt1 = im, kt2 = im, kn = im;
    if (b1.has_linear_locks() || b2.has_linear_locks()) {
        kn = dot(cmul(imv, n), n);
        kt1 = dot(cmul(imv, t1), t1);
        kt2 = dot(cmul(imv, t2), t2);
    }
    V3<R> ancN, ancT1, ancT2;
    V3<R> imp = an * n;
    imp = imp + at1 * t1;
    imp = imp + at2 * t2;
    if (cd.mode & ContactData<R>::LinearBody1) b1.vel = b1.vel - cmul(imp, b1.inv_mass_vec);
    if (cd.mode & ContactData<R>::AngularBody1) {
        V3<R> aN = sym_mul_inertia(b1.inv_inertia_world, cross(c.rel1, n));
        V3<R> aT1 = sym_mul_inertia(b1.inv_inertia_world, cross(c.rel1, t1));
        V3<R> aT2 = sym_mul_inertia(b1.inv_inertia_world, cross(c.rel1, t2));
        ancN = ancN + cross(aN, c.rel1);
        ancT1 = ancT1 + cross(aT1, c.rel1);
        ancT2 = ancT2 + cross(aT2, c.rel1);
        V3<R> ai = an * aN;
        ai = ai + at1 * aT1;
        ai = ai + at2 * aT2;
        b1.angvel = b1.angvel - ai;
    }
    if (cd.mode & ContactData<R>::LinearBody2) b2.vel = b2.vel + cmul(imp, b2.inv_mass_vec);
    if (cd.mode & ContactData<R>::AngularBody2) {
        V3<R> aN = sym_mul_inertia(b2.inv_inertia_world, cross(c.rel2, n));
        V3<R> aT1 = sym_mul_inertia(b2.inv_inertia_world, cross(c.rel2, t1));
        V3<R> aT2 = sym_mul_inertia(b2.inv_inertia_world, cross(c.rel2, t2));
        ancN = ancN + cross(aN, c.rel2);
        ancT1 = ancT1 + cross(aT1, c.rel2);
        ancT2 = ancT2 + cross(aT2, c.rel2);
        V3<R> ai = an * aN;
        ai = ai + at1 * aT1;
        ai = ai + at2 * aT2;
        b2.angvel = b2.angvel + ai;
    }
    kn += dot(n, ancN);
    kt1 += dot(t1, ancT1);
    kt2 += dot(t2, ancT2);
    c.mass[1] = kt1 > 0 ? (R)1.0 / kt1 : 0;
    c.mass[2] = kt2 > 0 ? (R)1.0 / kt2 : 0;
    c.mass[0] = kn > 0 ? (R)1.0 / kn : 0;
    c.penalty_bias = Contact<R>::BiasFactor * ts.inv_dt * std::max((R)0.0, pen - Contact<R>::AllowedPenetration);
    c.penalty_bias = std::min(c.penalty_bias, Contact<R>::MaximumBias);
}

// Contact.Iterate, scalar path (Contact.cs:931-1018)
template <class R> void contact_iterate(ContactData<R>& cd, Contact<R>& c, std::vector<Body<R>>& bodies, bool apply_bias) {
    R mN = c.mass[0], mT1 = c.mass[1], mT2 = c.mass[2];
    R aN = c.acc[0], aT1 = c.acc[1], aT2 = c.acc[2];
    Body<R>& b1 = bodies[cd.b1];
    Body<R>& b2 = bodies[cd.b2];
    V3<R> n = c.n, t1 = c.t1, t2 = c.t2;
    V3<R> dv = b2.vel - b1.vel;
    if (cd.mode & (ContactData<R>::AngularBody1 | ContactData<R>::AngularBody2)) {
        dv = b2.vel + cross(b2.angvel, c.rel2);
        dv = dv - (b1.vel + cross(b1.angvel, c.rel1));
    }
    R bias = c.bias;
    if (apply_bias && c.penalty_bias > 0) bias = std::max(c.penalty_bias, c.bias);
    R vn = dot(n, dv), vt1 = dot(t1, dv), vt2 = dot(t2, dv);
    R ni = -vn + bias;
    ni *= mN;
    R oldN = aN;
    aN = std::max(oldN + ni, (R)0.0);
    ni = aN - oldN;
    R maxT = cd.friction * oldN;
    R ti1 = mT1 * -vt1, ti2 = mT2 * -vt2;
    R oldT1 = aT1;
    aT1 = oldT1 + ti1;
    aT1 = std::clamp(aT1, -maxT, maxT);
    ti1 = aT1 - oldT1;
    R oldT2 = aT2;
    aT2 = oldT2 + ti2;
    aT2 = std::clamp(aT2, -maxT, maxT);
    ti2 = aT2 - oldT2;
    c.acc[0] = aN; c.acc[1] = aT1; c.acc[2] = aT2;
    V3<R> imp = ni * n;
    imp = imp + ti1 * t1;
    imp = imp + ti2 * t2;
    if (cd.mode & ContactData<R>::LinearBody1) b1.vel = b1.vel - cmul(imp, b1.inv_mass_vec);
    if (cd.mode & ContactData<R>::AngularBody1) b1.angvel = b1.angvel - sym_mul_inertia(b1.inv_inertia_world, cross(c.rel1, imp));
    if (cd.mode & ContactData<R>::LinearBody2) b2.vel = b2.vel + cmul(imp, b2.inv_mass_vec);
    if (cd.mode & ContactData<R>::AngularBody2) b2.angvel = b2.angvel + sym_mul_inertia(b2.inv_inertia_world, cross(c.rel2, imp));
}

template <class R> void contactdata_prepare(ContactData<R>& cd, std::vector<Body<R>>& bodies, const TimeStep<R>& ts) {
    for (int k = 0; k < 4; k++) if (cd.usage & (1u << k)) contact_prepare(cd, cd.c[k], bodies, ts);
}
template <class R> void contactdata_iterate(ContactData<R>& cd, std::vector<Body<R>>& bodies, bool bias) {
    for (int k = 0; k < 4; k++) if (cd.usage & (1u << k)) contact_iterate(cd, cd.c[k], bodies, bias);
}

// World.IntegrateForces (World.Step.cs:1060-1072)
template <class R> void integrate_forces(Body<R>& b) {
    if (b.motion != DYNAMIC) return;
    b.angvel = b.angvel + b.dangvel;
    b.vel = b.vel + b.dvel;
}
// JMatrix.Determinant (JMatrix.cs:391-395) and JMatrix.TryInverseUnscaled (JMatrix.cs:448-478)
template <class R> R mat_det(const R M[3][3]) {
    return M[0][0] * M[1][1] * M[2][2] + M[0][1] * M[1][2] * M[2][0] + M[0][2] * M[1][0] * M[2][1] -
           M[2][0] * M[1][1] * M[0][2] - M[2][1] * M[1][2] * M[0][0] - M[2][2] * M[1][0] * M[0][1];
}
template <class R> bool mat_try_inverse_unscaled(const R M[3][3], R out[3][3]) {
    R idet = (R)1.0 / mat_det(M);
    if (!std::isnormal(idet)) return false;
    R n[3][3];
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
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) { out[i][j] = n[i][j] * idet; fin = fin && std::isfinite(out[i][j]); }
    return fin;
}
// JMatrix.Inverse (JMatrix.cs:404-440): unscaled, else on the matrix scaled by its largest entry
template <class R> bool mat_inverse(const R M[3][3], R out[3][3]) {
    if (mat_try_inverse_unscaled(M, out)) return true;
    R s = std::max(std::abs(M[0][0]), std::max(std::abs(M[0][1]), std::abs(M[0][2])));
    s = std::max(s, std::max(std::abs(M[1][0]), std::max(std::abs(M[1][1]), std::abs(M[1][2]))));
    s = std::max(s, std::max(std::abs(M[2][0]), std::max(std::abs(M[2][1]), std::abs(M[2][2]))));
    if (s > 0 && std::isfinite(s)) {
        R nm[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) nm[i][j] = M[i][j] / s;
        if (mat_try_inverse_unscaled(nm, out)) {
            bool fin = true;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) { out[i][j] /= s; fin = fin && std::isfinite(out[i][j]); }
            if (fin) return true;
        }
    }
    return false;
}
// World.SolveGyroscopic (World.Step.cs:1075-1104): one implicit Newton step
template <class R> V3<R> solve_gyroscopic(const Sym3<R>& Iw, V3<R> w, R dt) {
    V3<R> Iwv = sym_mul(Iw, w);
    V3<R> f = dt * cross(w, Iwv);
    R I[3][3] = {{Iw.m11, Iw.m12, Iw.m13}, {Iw.m12, Iw.m22, Iw.m23}, {Iw.m13, Iw.m23, Iw.m33}};
    R W[3][3] = {{0, -w.z, w.y}, {w.z, 0, -w.x}, {-w.y, w.x, 0}};
    R L[3][3] = {{0, -Iwv.z, Iwv.y}, {Iwv.z, 0, -Iwv.x}, {-Iwv.y, Iwv.x, 0}};
    R J[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            R wi = W[i][0] * I[0][j] + W[i][1] * I[1][j] + W[i][2] * I[2][j];
            J[i][j] = I[i][j] + dt * (wi - L[i][j]);
        }
    R inv[3][3];
    if (!mat_inverse(J, inv)) return w;
    V3<R> d(inv[0][0] * f.x + inv[0][1] * f.y + inv[0][2] * f.z, inv[1][0] * f.x + inv[1][1] * f.y + inv[1][2] * f.z,
            inv[2][0] * f.x + inv[2][1] * f.y + inv[2][2] * f.z);
    return w - d;
}
// World.IntegrateVelocities (World.Step.cs:1106-1133)
template <class R> void integrate_velocities(Body<R>& b, const TimeStep<R>& ts) {
    if (b.motion == STATIC) return;
    V3<R> lv = b.vel, av = b.angvel;
    b.pos = b.pos + lv * ts.sub_dt;
    Q4<R> q = rotation_quaternion(av, ts.sub_dt);
    b.q = qnormalize(qmul(q, b.q));
    if (!b.gyroscopic() || b.has_motion_locks()) return;
    Sym3<R> Iw;
    sym_inverse(b.inv_inertia_world, Iw);
    b.angvel = solve_gyroscopic(Iw, av, ts.sub_dt);
}
// RigidBody.Update (RigidBody.cs:716-764); sleeping bookkeeping is not restated.
template <class R> void body_update(Body<R>& b, const TimeStep<R>& ts, V3<R> gravity) {
    int axes = b.allowed();
    restrict_linear(b.vel, axes);
    restrict_angular(b.angvel, axes);
    if (b.motion == DYNAMIC) {
        update_world_inertia(b);
        b.angvel = b.angvel * b.ang_damp;
        b.vel = b.vel * b.lin_damp;
        b.dvel = cmul(b.force, b.inv_mass_vec) * ts.sub_dt;
        b.dangvel = sym_mul(b.inv_inertia_world, b.torque) * ts.sub_dt;
        if (b.gravity) {
            V3<R> g = gravity;
            restrict_linear(g, axes);
            b.dvel = b.dvel + g * ts.sub_dt;
        }
        b.force = V3<R>();
        b.torque = V3<R>();
    }
}

}  // namespace jor
