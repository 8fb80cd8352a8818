// Oracle (test infrastructure only): extern "C" surface of the CPU restatement for the
// Python tests and the CPU baseline.  Every function exists twice, suffix _f (Real =
// float, the reference's default build) and _d (Real = double, Jitter2.Double).  The
// plain data structs are the ones the GPU library's header declares, so one scene
// description feeds both.
#include "jor_world.hpp"
#include "../include/jitter_gpu.h"
#include <chrono>

using namespace jor;

// Constraint kinds the oracle restates ahead of the device (ids past the header's).
#define JOR_CONSTRAINT_FIXEDANGLE 6
#define JOR_CONSTRAINT_POINTONPLANE 7
#define JOR_CONSTRAINT_ANGULARMOTOR 8
#define JOR_CONSTRAINT_LINEARMOTOR 9
#define JOR_CONSTRAINT_ANGULARSERVO 10
#define JOR_CONSTRAINT_LINEARSERVO 11
#define JOR_CONSTRAINT_LINEARAXISSERVO 12
#define JOR_CONSTRAINT_TWISTSERVO 13
#define JOR_CONSTRAINT_POINTONLINE 14
#define JOR_CONSTRAINT_ELLIPTICALCONELIMIT 15

namespace {

template <class R> Shape<R> make_shape(const jg_shape_desc& d, const float* hull, const jg_triangle_desc* tris,
                                       std::vector<R>& hull_store, size_t hull_base) {
    Shape<R> s;
    s.kind = d.kind;
    s.d0 = (R)d.dims[0]; s.d1 = (R)d.dims[1]; s.d2 = (R)d.dims[2];
    s.center = V3<R>((R)d.center[0], (R)d.center[1], (R)d.center[2]);
    if (d.kind == POINTCLOUD) {
        s.shift = V3<R>((R)d.dims[0], (R)d.dims[1], (R)d.dims[2]);
        s.d0 = s.d1 = s.d2 = 0;
        s.nverts = d.data_count;
        (void)hull; (void)hull_store;
        s.verts = nullptr;  // patched by the caller once hull_store is final
        (void)hull_base;
    }
    if (d.kind == TRIANGLE) {
        const jg_triangle_desc& t = tris[d.data_offset];
        s.ta = V3<R>((R)t.a[0], (R)t.a[1], (R)t.a[2]);
        s.tb = V3<R>((R)t.b[0], (R)t.b[1], (R)t.b[2]);
        s.tc = V3<R>((R)t.c[0], (R)t.c[1], (R)t.c[2]);
        s.tnormal = V3<R>((R)t.normal[0], (R)t.normal[1], (R)t.normal[2]);
        for (int k = 0; k < 3; k++) {
            int nb = t.neighbor[k];
            s.nbr_valid[k] = nb >= 0;
            if (nb >= 0) s.nbr_normal[k] = V3<R>((R)tris[nb].normal[0], (R)tris[nb].normal[1], (R)tris[nb].normal[2]);
        }
    }
    return s;
}

template <class R> void set_shapes(World<R>& w, const jg_shape_desc* d, int n, const float* hull, int nh,
                                   const jg_triangle_desc* tris, int nt) {
    (void)nt;
    w.hull.assign(hull, hull + 3 * (size_t)nh);
    w.shapes.clear();
    w.shape_body.clear();
    for (int i = 0; i < n; i++) {
        Shape<R> s = make_shape<R>(d[i], hull, tris, w.hull, 0);
        if (d[i].kind == POINTCLOUD) s.verts = w.hull.data() + 3 * (size_t)d[i].data_offset;
        w.shapes.push_back(s);
        w.shape_body.push_back(d[i].body);
    }
    w.arbiters.clear();
    w.arb_index.clear();
}

template <class R> void set_bodies(World<R>& w, const jg_body_desc* d, int n) {
    w.bodies.resize(n);
    for (int i = 0; i < n; i++) {
        Body<R>& b = w.bodies[i];
        const jg_body_desc& s = d[i];
        b.pos = V3<R>(s.position[0], s.position[1], s.position[2]);
        b.q = Q4<R>(s.orientation[0], s.orientation[1], s.orientation[2], s.orientation[3]);
        b.vel = V3<R>(s.velocity[0], s.velocity[1], s.velocity[2]);
        b.angvel = V3<R>(s.angular_velocity[0], s.angular_velocity[1], s.angular_velocity[2]);
        b.inv_inertia_local = Sym3<R>(s.inv_inertia[0], s.inv_inertia[1], s.inv_inertia[2], s.inv_inertia[3], s.inv_inertia[4], s.inv_inertia[5]);
        b.inv_mass = s.inv_mass;
        b.friction = s.friction; b.restitution = s.restitution;
        b.lin_damp = s.linear_damping; b.ang_damp = s.angular_damping;
        b.force = V3<R>(s.force[0], s.force[1], s.force[2]);
        b.torque = V3<R>(s.torque[0], s.torque[1], s.torque[2]);
        b.motion = s.motion_type;
        b.flags = (s.flags & 0x3f0) | (s.flags & JG_BODY_ACTIVE) | (s.flags & JG_BODY_GYROSCOPIC);
        b.gravity = (s.flags & JG_BODY_NO_GRAVITY) == 0;
        b.speculative = (s.flags & JG_BODY_SPECULATIVE) != 0;
        // a body made static is deactivated at the next step (DeactivateBodyNextStep,
        // World.cs:797-800, from the MotionType setter, RigidBody.cs:959-968)
        if (b.motion == STATIC) b.sleep_time = std::numeric_limits<R>::infinity();
        b.world = s.world;
        // DeltaVelocity/DeltaAngularVelocity: the velocity change queued by the last
        // RigidBody.Update (zero for a body that has not been stepped yet).
        b.dvel = V3<R>(s.delta_velocity[0], s.delta_velocity[1], s.delta_velocity[2]);
        b.dangvel = V3<R>(s.delta_angular_velocity[0], s.delta_angular_velocity[1], s.delta_angular_velocity[2]);
        update_world_inertia(b);
    }
}

template <class R> void get_bodies(const World<R>& w, jg_body_desc* d, int n) {
    for (int i = 0; i < n && i < (int)w.bodies.size(); i++) {
        const Body<R>& b = w.bodies[i];
        jg_body_desc& s = d[i];
        s.position[0] = (float)b.pos.x; s.position[1] = (float)b.pos.y; s.position[2] = (float)b.pos.z;
        s.orientation[0] = (float)b.q.x; s.orientation[1] = (float)b.q.y; s.orientation[2] = (float)b.q.z; s.orientation[3] = (float)b.q.w;
        s.velocity[0] = (float)b.vel.x; s.velocity[1] = (float)b.vel.y; s.velocity[2] = (float)b.vel.z;
        s.angular_velocity[0] = (float)b.angvel.x; s.angular_velocity[1] = (float)b.angvel.y; s.angular_velocity[2] = (float)b.angvel.z;
        s.delta_velocity[0] = (float)b.dvel.x; s.delta_velocity[1] = (float)b.dvel.y; s.delta_velocity[2] = (float)b.dvel.z;
        s.delta_angular_velocity[0] = (float)b.dangvel.x; s.delta_angular_velocity[1] = (float)b.dangvel.y; s.delta_angular_velocity[2] = (float)b.dangvel.z;
        s.motion_type = b.motion;
        s.world = b.world;
        const Sym3<R>& L = b.inv_inertia_local;
        s.inv_inertia[0] = (float)L.m11; s.inv_inertia[1] = (float)L.m12; s.inv_inertia[2] = (float)L.m13;
        s.inv_inertia[3] = (float)L.m22; s.inv_inertia[4] = (float)L.m23; s.inv_inertia[5] = (float)L.m33;
        s.inv_mass = (float)b.inv_mass;
        s.friction = (float)b.friction; s.restitution = (float)b.restitution;
        s.linear_damping = (float)b.lin_damp; s.angular_damping = (float)b.ang_damp;
        s.force[0] = (float)b.force.x; s.force[1] = (float)b.force.y; s.force[2] = (float)b.force.z;
        s.torque[0] = (float)b.torque.x; s.torque[1] = (float)b.torque.y; s.torque[2] = (float)b.torque.z;
        s.flags = b.flags | (b.gravity ? 0 : JG_BODY_NO_GRAVITY) | (b.speculative ? JG_BODY_SPECULATIVE : 0);
    }
}

template <class R> int get_contacts(const World<R>& w, jg_contact_view* out, int cap) {
    int n = 0;
    for (auto& a : w.arbiters)
        for (int k = 0; k < 4; k++) {
            if (!(a.usage & (0x11u << k))) continue;
            if (n < cap) {
                jg_contact_view& v = out[n];
                const Contact<R>& c = a.c[k];
                v.shape1 = a.key1; v.shape2 = a.key2; v.body1 = a.b1; v.body2 = a.b2;
                v.slot = k; v.usage_mask = (int)a.usage; v.color = a.color; v.flags = c.flag;
                auto put = [](float* o, V3<R> x) { o[0] = (float)x.x; o[1] = (float)x.y; o[2] = (float)x.z; };
                put(v.normal, c.n); put(v.tangent1, c.t1); put(v.tangent2, c.t2);
                put(v.rel_pos1, c.rel1); put(v.rel_pos2, c.rel2); put(v.pos1_local, c.pos1); put(v.pos2_local, c.pos2);
                for (int r = 0; r < 3; r++) { v.accumulated[r] = (float)c.acc[r]; v.mass[r] = (float)c.mass[r]; }
                v.bias = (float)c.bias; v.penalty_bias = (float)c.penalty_bias;
                v.friction = (float)a.friction; v.restitution = (float)a.restitution;
            }
            n++;
        }
    return n;
}

// Rebuilds the arbiter cache from contact views (state import, one-step comparisons).
template <class R> void set_contacts(World<R>& w, const jg_contact_view* in, int n) {
    w.arbiters.clear();
    w.arb_index.clear();
    for (int i = 0; i < n; i++) {
        const jg_contact_view& v = in[i];
        int ai = w.find_or_create(v.shape1, v.shape2);
        ContactData<R>& a = w.arbiters[ai];
        a.usage = (unsigned)v.usage_mask;
        a.color = v.color;
        a.friction = v.friction; a.restitution = v.restitution;
        w.reset_mode(a);
        Contact<R>& c = a.c[v.slot];
        auto get = [](const float* o) { return V3<R>(o[0], o[1], o[2]); };
        c.n = get(v.normal); c.t1 = get(v.tangent1); c.t2 = get(v.tangent2);
        c.rel1 = get(v.rel_pos1); c.rel2 = get(v.rel_pos2); c.pos1 = get(v.pos1_local); c.pos2 = get(v.pos2_local);
        for (int r = 0; r < 3; r++) { c.acc[r] = v.accumulated[r]; c.mass[r] = v.mass[r]; }
        c.bias = v.bias; c.penalty_bias = v.penalty_bias; c.flag = v.flags;
    }
}

template <class R> void desc_to_shape(const jg_shape_desc* d, const float* verts, Shape<R>& s, std::vector<R>& store) {
    jg_triangle_desc dummy{};
    s = make_shape<R>(*d, verts, &dummy, store, 0);
    if (d->kind == POINTCLOUD) {
        store.assign(verts, verts + 3 * (size_t)d->data_count);
        s.verts = store.data();
    }
}
template <class R> void put3(float* o, V3<R> v) { o[0] = (float)v.x; o[1] = (float)v.y; o[2] = (float)v.z; }
template <class R> V3<R> get3(const float* v) { return V3<R>(v[0], v[1], v[2]); }
template <class R> Q4<R> get4(const float* v) { return Q4<R>(v[0], v[1], v[2], v[3]); }
template <class R> void put3d(double* o, V3<R> v) { o[0] = (double)v.x; o[1] = (double)v.y; o[2] = (double)v.z; }
template <class R> V3<R> get3d(const double* v) { return V3<R>((R)v[0], (R)v[1], (R)v[2]); }
template <class R> Q4<R> get4d(const double* v) { return Q4<R>((R)v[0], (R)v[1], (R)v[2], (R)v[3]); }

template <class R> struct Handle {
    World<R> w;
};

}  // namespace

#define JOR_DEFINE(SUF, R)                                                                                       \
    extern "C" void* jor_world_create_##SUF(void) { return new Handle<R>(); }                                     \
    extern "C" void jor_world_destroy_##SUF(void* h) { delete (Handle<R>*)h; }                                    \
    extern "C" void jor_world_config_##SUF(void* h, const jg_world_params* p) {                                   \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        w.gravity = V3<R>(p->gravity[0], p->gravity[1], p->gravity[2]);                                            \
        w.substeps = p->substeps; w.iterations = p->solver_iterations; w.relax = p->relax_iterations;             \
        w.aux_contacts = p->enable_auxiliary_contacts != 0; w.persistent = p->persistent_manifold != 0;           \
        w.spec_relax = p->speculative_relaxation; w.edge_filter = p->edge_filter != 0;                             \
        w.spec_threshold = p->speculative_threshold;                                                               \
        w.record_residual = p->record_residual != 0;                                                               \
    }                                                                                                              \
    extern "C" void jor_world_set_bodies_##SUF(void* h, const jg_body_desc* d, int n) { set_bodies(((Handle<R>*)h)->w, d, n); } \
    extern "C" void jor_world_get_bodies_##SUF(void* h, jg_body_desc* d, int n) { get_bodies(((Handle<R>*)h)->w, d, n); } \
    extern "C" void jor_world_get_bodies_d_##SUF(void* h, double* out, int n) {                                   \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        for (int i = 0; i < n && i < (int)w.bodies.size(); i++) {                                                  \
            const Body<R>& b = w.bodies[i]; double* o = out + 13 * (size_t)i;                                       \
            put3d(o, b.pos); o[3] = b.q.x; o[4] = b.q.y; o[5] = b.q.z; o[6] = b.q.w; put3d(o + 7, b.vel); put3d(o + 10, b.angvel); \
        }                                                                                                          \
    }                                                                                                              \
    extern "C" void jor_world_set_shapes_##SUF(void* h, const jg_shape_desc* d, int n, const float* hull, int nh, \
                                               const jg_triangle_desc* t, int nt) {                                \
        set_shapes(((Handle<R>*)h)->w, d, n, hull, nh, t, nt);                                                     \
    }                                                                                                              \
    extern "C" int jor_world_add_joint_##SUF(void* h, int kind, int b1, int b2, const float* init) {             \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        Joint<R> j; j.b1 = b1; j.b2 = b2;                                                                          \
        if (kind == JG_CONSTRAINT_BALLSOCKET) ballsocket_init(j, w.bodies, get3<R>(init));                         \
        else if (kind == JG_CONSTRAINT_HINGEANGLE) hinge_init(j, w.bodies, get3<R>(init), (R)init[3], (R)init[4]);  \
        else if (kind == JG_CONSTRAINT_DISTANCELIMIT)                                                              \
            distance_init(j, w.bodies, get3<R>(init), get3<R>(init + 3), (R)init[6], (R)init[7]);                 \
        else if (kind == JG_CONSTRAINT_CONELIMIT)                                                                  \
            cone_init(j, w.bodies, get3<R>(init), get3<R>(init + 3), (R)init[6], (R)init[7]);                     \
        else if (kind == JG_CONSTRAINT_TWISTANGLE)                                                                 \
            twist_init(j, w.bodies, get3<R>(init), get3<R>(init + 3), (R)init[6], (R)init[7]);                    \
        else if (kind == JOR_CONSTRAINT_FIXEDANGLE) fixed_init(j, w.bodies);                                       \
        else if (kind == JOR_CONSTRAINT_ANGULARMOTOR || kind == JOR_CONSTRAINT_LINEARMOTOR)                        \
            motor_init(j, w.bodies, get3<R>(init), get3<R>(init + 3), (R)init[6], (R)init[7],                     \
                       kind == JOR_CONSTRAINT_LINEARMOTOR);                                                        \
        else if (kind == JOR_CONSTRAINT_POINTONPLANE)                                                              \
            plane_init(j, w.bodies, get3<R>(init), get3<R>(init + 3), get3<R>(init + 6), (R)init[9], (R)init[10]); \
        else if (kind == JOR_CONSTRAINT_ANGULARSERVO) {                                                            \
            Q4<R> t((R)init[0], (R)init[1], (R)init[2], (R)init[3]);                                               \
            if (init[0] == 0 && init[1] == 0 && init[2] == 0 && init[3] == 0)                                      \
                t = qmul(qconj(w.bodies[b1].q), w.bodies[b2].q);                                                   \
            angular_servo_init(j, t, (R)init[4]);                                                                  \
        } else if (kind == JOR_CONSTRAINT_LINEARSERVO)                                                             \
            linear_servo_init(j, w.bodies, get3<R>(init), get3<R>(init + 3), get3<R>(init + 6), (R)init[9]);       \
        else if (kind == JOR_CONSTRAINT_LINEARAXISSERVO)                                                           \
            linear_axis_servo_init(j, w.bodies, get3<R>(init), get3<R>(init + 3), get3<R>(init + 6), (R)init[9],  \
                                   (R)init[10]);                                                                   \
        else if (kind == JOR_CONSTRAINT_TWISTSERVO)                                                                \
            twist_servo_init(j, w.bodies, get3<R>(init), get3<R>(init + 3), (R)init[6], (R)init[7]);              \
        else if (kind == JOR_CONSTRAINT_POINTONLINE)                                                               \
            line_init(j, w.bodies, get3<R>(init), get3<R>(init + 3), get3<R>(init + 6), (R)init[9], (R)init[10]);  \
        else if (kind == JOR_CONSTRAINT_ELLIPTICALCONELIMIT)                                                       \
            elliptical_init(j, w.bodies, get3<R>(init), get3<R>(init + 3), get3<R>(init + 6), (R)init[9],        \
                            (R)init[10], (R)init[11], (R)init[12]);                                                \
        w.joints.push_back(j);                                                                                     \
        return (int)w.joints.size() - 1;                                                                           \
    }                                                                                                              \
    /* one Prepare (and, with iterate set, one Iterate) of joint j alone at step dt, bias factor \
       and softness overridden: the constraint-level calls the reference's own tests make */     \
    extern "C" void jor_world_joint_solve_##SUF(void* h, int j, float dt, float bias, float soft, int iterate) { \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        Joint<R>& jt = w.joints[j];                                                                                \
        jt.bias_factor = (R)bias; jt.softness = (R)soft;                                                           \
        TimeStep<R> ts((R)dt, 1);                                                                                  \
        joint_prepare(jt, w.bodies, ts);                                                                           \
        if (iterate) joint_iterate(jt, w.bodies, ts);                                                              \
    }                                                                                                              \
    /* one Prepare and `iterations` Iterates of joint j alone under TimeStep(dt, substeps), its own \
       bias and softness: the Solve helper of the reference's ServoTests (ServoTests.cs:51-56) */    \
    extern "C" void jor_world_joint_run_##SUF(void* h, int j, float dt, int substeps, int prepare, int iterations) { \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        TimeStep<R> ts((R)dt, substeps);                                                                           \
        if (prepare) joint_prepare(w.joints[j], w.bodies, ts);                                                     \
        for (int i = 0; i < iterations; i++) joint_iterate(w.joints[j], w.bodies, ts);                             \
    }                                                                                                              \
    /* PointOnLine.Distance (PointOnLine.cs:123-146): anchor 2's position along the line */                     \
    extern "C" double jor_world_line_distance_##SUF(void* h, int j) {                                              \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        const Joint<R>& jt = w.joints[j];                                                                          \
        V3<R> J[12];                                                                                               \
        return (double)line_jacobian(jt, w.bodies[jt.b1], w.bodies[jt.b2], J).z;                                   \
    }                                                                                                              \
    /* EllipticalConeLimit.GetSwing (EllipticalConeLimit.cs:206-221): out = along, across */                     \
    extern "C" void jor_world_elliptical_swing_##SUF(void* h, int j, double* out) {                                \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        R x, y;                                                                                                    \
        elliptical_swing(w.joints[j], w.bodies, x, y);                                                             \
        out[0] = (double)x; out[1] = (double)y;                                                                    \
    }                                                                                                              \
    /* a joint's accumulated impulse (acc xyz) */                                                                \
    extern "C" void jor_world_joint_impulse_##SUF(void* h, int j, double* out) {                                   \
        put3d(out, ((Handle<R>*)h)->w.joints[j].acc);                                                              \
    }                                                                                                              \
    /* a servo's target and maximum, as jg_set_servo: a changed target drops the warm start (and   \
       the AngularServo's hemisphere) */                                                              \
    extern "C" void jor_world_set_servo_##SUF(void* h, int j, const float* target, float maximum) {                \
        Joint<R>& jt = ((Handle<R>*)h)->w.joints[j];                                                               \
        bool changed;                                                                                              \
        if (jt.kind == ANGULARSERVO) {                                                                             \
            Q4<R> t((R)target[0], (R)target[1], (R)target[2], (R)target[3]);                                       \
            changed = t.x != jt.q0.x || t.y != jt.q0.y || t.z != jt.q0.z || t.w != jt.q0.w;                        \
            jt.q0 = t;                                                                                             \
            if (changed) jt.hemisphere = 0;                                                                        \
        } else if (jt.kind == LINEARSERVO) {                                                                       \
            V3<R> t = get3<R>(target);                                                                             \
            changed = t.x != jt.target_pos.x || t.y != jt.target_pos.y || t.z != jt.target_pos.z;                  \
            jt.target_pos = t;                                                                                     \
        } else {                                                                                                   \
            changed = (R)target[0] != jt.target;                                                                   \
            jt.target = (R)target[0];                                                                              \
        }                                                                                                          \
        if (changed) jt.acc = V3<R>();                                                                             \
        jt.maximum = (R)maximum;                                                                                   \
    }                                                                                                              \
    /* one Iterate of joint j alone (after a Prepare) at step dt */                                              \
    extern "C" void jor_world_joint_iterate_##SUF(void* h, int j, float dt) {                                      \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        TimeStep<R> ts((R)dt, 1);                                                                                  \
        joint_iterate(w.joints[j], w.bodies, ts);                                                                  \
    }                                                                                                              \
    /* joint row after its last Prepare: out = jr[0], jr[1], effective mass, clamp, impulse */                \
    extern "C" void jor_world_joint_data_##SUF(void* h, int j, double* out) {                                      \
        const Joint<R>& jt = ((Handle<R>*)h)->w.joints[j];                                                         \
        put3d(out, jt.jr[0]); put3d(out + 3, jt.jr[1]);                                                            \
        out[6] = (double)jt.eff1; out[7] = jt.clamp; out[8] = (double)jt.acc.x; put3d(out + 9, jt.bias);          \
    }                                                                                                              \
    /* Bias / Softness setters of a joint (ConeLimit.cs:358-376, TwistAngle.cs:262-294, ...) */                   \
    extern "C" void jor_world_joint_params_##SUF(void* h, int j, double bias, double soft) {                       \
        Joint<R>& jt = ((Handle<R>*)h)->w.joints[j];                                                               \
        jt.bias_factor = (R)bias; jt.softness = (R)soft;                                                           \
    }                                                                                                              \
    /* HingeAngle LimitBias / LimitSoftness setters (HingeAngle.cs:270-300) */                                   \
    extern "C" void jor_world_joint_limit_params_##SUF(void* h, int j, double bias, double soft) {                 \
        Joint<R>& jt = ((Handle<R>*)h)->w.joints[j];                                                               \
        jt.limit_bias = (R)bias; jt.limit_softness = (R)soft;                                                      \
    }                                                                                                              \
    /* three-row joint state after its last Prepare: out = Jacobian (3x3, row-major as stored), \
       Q0 (x y z w), local axis */                                                                                 \
    extern "C" void jor_world_joint_matrix_##SUF(void* h, int j, double* out) {                                    \
        const Joint<R>& jt = ((Handle<R>*)h)->w.joints[j];                                                         \
        for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) out[3 * r + c] = (double)jt.jac.a[r][c];           \
        out[9] = jt.q0.x; out[10] = jt.q0.y; out[11] = jt.q0.z; out[12] = jt.q0.w;                                 \
        put3d(out + 13, jt.axis);                                                                                  \
    }                                                                                                              \
    extern "C" double jor_world_joint_angle_##SUF(void* h, int j) {                                                \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        return (double)joint_angle(w.joints[j], w.bodies);                                                         \
    }                                                                                                              \
    /* ConeLimit.Limit / TwistAngle.Limit setters (ConeLimit.cs:196-206, TwistAngle.cs:130-143) */               \
    extern "C" void jor_world_joint_set_limit_##SUF(void* h, int j, double lo, double hi) {                       \
        Joint<R>& jt = ((Handle<R>*)h)->w.joints[j];                                                               \
        jt.min_angle = (R)lo; jt.max_angle = (R)hi;                                                                \
        jt.fixed_angle = (R)0.5 * (R)lo + (R)0.5 * (R)hi;                                                          \
    }                                                                                                              \
    extern "C" void jor_world_set_joint_colors_##SUF(void* h, const int* colors, int n) {                         \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        for (int i = 0; i < n && i < (int)w.joints.size(); i++) w.joints[i].color = colors[i];                     \
    }                                                                                                              \
    extern "C" void jor_world_get_joint_impulses_##SUF(void* h, float* out, int n) {                               \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        for (int i = 0; i < n && i < (int)w.joints.size(); i++) put3(out + 3 * i, w.joints[i].acc);                \
    }                                                                                                              \
    extern "C" void jor_world_set_joint_impulses_##SUF(void* h, const float* in, int n) {                          \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        for (int i = 0; i < n && i < (int)w.joints.size(); i++)                                                    \
            w.joints[i].acc = V3<R>((R)in[3 * i], (R)in[3 * i + 1], (R)in[3 * i + 2]);                             \
    }                                                                                                              \
    extern "C" void jor_world_external_order_##SUF(void* h, int on) { ((Handle<R>*)h)->w.external_order = on != 0; } \
    extern "C" void jor_world_set_contacts_##SUF(void* h, const jg_contact_view* v, int n) { set_contacts(((Handle<R>*)h)->w, v, n); } \
    extern "C" int jor_world_get_contacts_##SUF(void* h, jg_contact_view* v, int cap) { return get_contacts(((Handle<R>*)h)->w, v, cap); } \
    extern "C" void jor_world_set_arbiter_color_##SUF(void* h, int s1, int s2, int color) {                       \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        auto it = w.arb_index.find(World<R>::key(s1, s2));                                                         \
        if (it != w.arb_index.end()) w.arbiters[it->second].color = color;                                         \
    }                                                                                                              \
    extern "C" void jor_world_register_contact_##SUF(void* h, int s1, int s2, const float* p1, const float* p2,   \
                                                     const float* n) {                                             \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        typename World<R>::DetectResult r; r.hit = true; r.count = 1;                                               \
        r.A[0] = get3<R>(p1); r.B[0] = get3<R>(p2); r.n = get3<R>(n);                                              \
        w.register_contact(s1, s2, r);                                                                             \
    }                                                                                                              \
    /* RegisterContact of a manifold (World.Detect.cs:294-324): n points on A and on B */                        \
    extern "C" void jor_world_register_manifold_##SUF(void* h, int s1, int s2, const float* pa, const float* pb,   \
                                                      int n, const float* nrm) {                                   \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        typename World<R>::DetectResult r; r.hit = true; r.count = std::min(n, 4); r.n = get3<R>(nrm);              \
        for (int i = 0; i < r.count; i++) { r.A[i] = get3<R>(pa + 3 * i); r.B[i] = get3<R>(pb + 3 * i); }           \
        w.register_contact(s1, s2, r);                                                                             \
    }                                                                                                              \
    /* RegisterContact with SolveMode.Angular removed (World.Detect.cs:246-262, removeFlags) */                 \
    extern "C" void jor_world_register_linear_contact_##SUF(void* h, int s1, int s2, const float* p1,              \
                                                            const float* p2, const float* n) {                     \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        typename World<R>::DetectResult r; r.hit = true; r.count = 1; r.speculative = true;                        \
        r.A[0] = get3<R>(p1); r.B[0] = get3<R>(p2); r.n = get3<R>(n);                                              \
        w.register_contact(s1, s2, r);                                                                             \
    }                                                                                                              \
    extern "C" void jor_world_narrowphase_##SUF(void* h) { ((Handle<R>*)h)->w.narrowphase(); }                    \
    extern "C" void jor_world_body_deactivation_time_##SUF(void* h, int i, double seconds) {                      \
        ((Handle<R>*)h)->w.bodies[i].deactivation_time = (R)seconds;                                               \
    }                                                                                                              \
    extern "C" void jor_world_activate_body_##SUF(void* h, int i) { ((Handle<R>*)h)->w.activate_body(i); }        \
    extern "C" void jor_world_body_sleep_thresholds_##SUF(void* h, int i, double lin, double ang) {                \
        ((Handle<R>*)h)->w.bodies[i].sleep_lin2 = (R)(lin * lin);                                                   \
        ((Handle<R>*)h)->w.bodies[i].sleep_ang2 = (R)(ang * ang);                                                   \
    }                                                                                                              \
    /* World.AllowDeactivation (World.cs:333) for the oracle's island restatement */                           \
    extern "C" void jor_world_set_deactivation_##SUF(void* h, int on) { ((Handle<R>*)h)->w.allow_deactivation = on != 0; } \
    /* world bounding box of shape s as the step of length dt sees it (out = min, max) */                        \
    extern "C" void jor_world_shape_box_##SUF(void* h, int s, float dt, double* out) {                            \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        w.step_dt = (R)dt;                                                                                         \
        Box3<R> b = w.aabbs()[s]; put3d(out, b.mn); put3d(out + 3, b.mx);                                          \
    }                                                                                                              \
    extern "C" void jor_world_set_step_dt_##SUF(void* h, float dt) { ((Handle<R>*)h)->w.step_dt = (R)dt; }        \
    /* ContactData.PrepareForIteration / Iterate on every arbiter, key order (tests) */                            \
    extern "C" void jor_world_prepare_##SUF(void* h, float dt, int substeps) {                                    \
        World<R>& w = ((Handle<R>*)h)->w; TimeStep<R> ts((R)dt, substeps);                                         \
        for (auto& a : w.arbiters) contactdata_prepare(a, w.bodies, ts);                                           \
    }                                                                                                              \
    extern "C" void jor_world_iterate_##SUF(void* h, int bias) {                                                  \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        for (auto& a : w.arbiters) contactdata_iterate(a, w.bodies, bias != 0);                                    \
    }                                                                                                              \
    /* ContactData.Mode of arbiter a (Contact.cs:37-60): which body velocities the rows update */           \
    extern "C" void jor_world_set_arbiter_mode_##SUF(void* h, int a, int mode) { ((Handle<R>*)h)->w.arbiters[a].mode = mode; } \
    extern "C" void jor_world_set_penalty_##SUF(void* h, int arb, int slot, double value) {                       \
        ((Handle<R>*)h)->w.arbiters[arb].c[slot].penalty_bias = (R)value;                                         \
    }                                                                                                              \
    extern "C" void jor_world_set_orientation_##SUF(void* h, int b, const float* q) {                             \
        World<R>& w = ((Handle<R>*)h)->w; w.bodies[b].q = Q4<R>(q[0], q[1], q[2], q[3]);                           \
        update_world_inertia(w.bodies[b]);                                                                         \
    }                                                                                                              \
    extern "C" void jor_world_set_orientation_d_##SUF(void* h, int b, const double* q) {                          \
        World<R>& w = ((Handle<R>*)h)->w; w.bodies[b].q = Q4<R>((R)q[0], (R)q[1], (R)q[2], (R)q[3]);               \
        update_world_inertia(w.bodies[b]);                                                                         \
    }                                                                                                              \
    extern "C" void jor_world_inertia_world_##SUF(void* h, int b, double* out) {                                  \
        const Sym3<R>& I = ((Handle<R>*)h)->w.bodies[b].inv_inertia_world;                                        \
        out[0] = I.m11; out[1] = I.m12; out[2] = I.m13; out[3] = I.m22; out[4] = I.m23; out[5] = I.m33;            \
    }                                                                                                              \
    extern "C" void jor_world_step_##SUF(void* h, float dt, int narrow) { ((Handle<R>*)h)->w.step((R)dt, narrow != 0); } \
    extern "C" void jor_world_stabilize_##SUF(void* h, float dt, int iterations, int relax) {                    \
        ((Handle<R>*)h)->w.stabilize((R)dt, iterations, relax);                                                    \
    }                                                                                                              \
    extern "C" double jor_world_step_mt_##SUF(void* h, float dt, int threads) {                                   \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        w.nthreads = threads;                                                                                      \
        auto t0 = std::chrono::steady_clock::now();                                                                \
        RegularSolver<R> rs(w); rs.step((R)dt);                                                                    \
        auto t1 = std::chrono::steady_clock::now();                                                                \
        w.nthreads = 1;                                                                                            \
        return std::chrono::duration<double>(t1 - t0).count();                                                     \
    }                                                                                                              \
    extern "C" void jor_world_counters_##SUF(void* h, long long* out) {                                           \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        long long pts = 0;                                                                                         \
        for (auto& a : w.arbiters) pts += __builtin_popcount(a.usage & 15u);                                       \
        out[0] = w.n_pairs; out[1] = w.n_colliding; out[2] = w.n_points; out[3] = (long long)w.arbiters.size();    \
        out[4] = pts; out[5] = w.solver.epa_calls; out[6] = w.solver.epa_failures; out[7] = w.n_speculative;      \
    }                                                                                                              \
    extern "C" int jor_world_pairs_##SUF(void* h, int* out, int cap) {                                            \
        auto p = ((Handle<R>*)h)->w.find_pairs();                                                                  \
        for (int i = 0; i < (int)p.size() && i < cap; i++) { out[2 * i] = p[i].first; out[2 * i + 1] = p[i].second; } \
        return (int)p.size();                                                                                      \
    }                                                                                                              \
    extern "C" int jor_world_pairs_sweep_##SUF(void* h, int* out, int cap) {                                      \
        auto p = ((Handle<R>*)h)->w.find_pairs_sweep();                                                            \
        for (int i = 0; i < (int)p.size() && i < cap; i++) { out[2 * i] = p[i].first; out[2 * i + 1] = p[i].second; } \
        return (int)p.size();                                                                                      \
    }                                                                                                              \
    extern "C" int jor_world_residuals_##SUF(void* h, float* out, int cap) {                                      \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        for (int i = 0; i < (int)w.residuals.size() && i < cap; i++) out[i] = (float)w.residuals[i];              \
        return (int)w.residuals.size();                                                                            \
    }                                                                                                              \
    /* Detect on one pair of shapes of the world: returns hit; out = n, count, 4x(A,B), pen, pA, pB */            \
    extern "C" int jor_world_detect_##SUF(void* h, int s1, int s2, double* out) {                                 \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        auto r = w.detect(s1, s2, w.solver);                                                                       \
        if (!r.hit) return 0;                                                                                      \
        put3d(out, r.n); out[3] = r.count;                                                                         \
        for (int i = 0; i < r.count; i++) { put3d(out + 4 + 6 * i, r.A[i]); put3d(out + 7 + 6 * i, r.B[i]); }       \
        out[28] = (double)r.pen; put3d(out + 29, r.pA); put3d(out + 32, r.pB);                                     \
        return 1;                                                                                                  \
    }                                                                                                              \
    /* NarrowPhase.MprEpa (NarrowPhase.cs:902-927) on two shapes of the world at their     \
       bodies' poses: out = pA, pB, n, pen */                                                                      \
    extern "C" int jor_world_collide_##SUF(void* h, int s1, int s2, double* out) {                                \
        World<R>& w = ((Handle<R>*)h)->w;                                                                          \
        const Body<R>& b1 = w.bodies[w.shape_body[s1]];                                                            \
        const Body<R>& b2 = w.bodies[w.shape_body[s2]];                                                            \
        MprEpa<R> sol; V3<R> pA, pB, n; R pen = 0;                                                                 \
        bool hit = sol.mpr_epa_world(w.shapes[s1], w.shapes[s2], b1.q, b2.q, b1.pos, b2.pos, pA, pB, n, pen);      \
        put3d(out, pA); put3d(out + 3, pB); put3d(out + 6, n); out[9] = (double)pen;                              \
        return hit ? 1 : 0;                                                                                        \
    }                                                                                                              \
    extern "C" void jor_support_##SUF(const jg_shape_desc* d, const float* verts, const double* dir, double* out) { \
        Shape<R> s; std::vector<R> st; desc_to_shape<R>(d, verts, s, st);                                          \
        put3d(out, support(s, get3d<R>(dir)));                                                                     \
    }                                                                                                              \
    extern "C" void jor_aabb_##SUF(const jg_shape_desc* d, const float* verts, const double* q, const double* p, double* out) { \
        Shape<R> s; std::vector<R> st; desc_to_shape<R>(d, verts, s, st);                                          \
        Box3<R> b = shape_aabb(s, get4d<R>(q), get3d<R>(p)); put3d(out, b.mn); put3d(out + 3, b.mx);               \
    }                                                                                                              \
    /* mode 0: MprEpa world (NarrowPhase.cs:902-927); mode 1: Collision (EPA, NarrowPhase.cs:350-431) */          \
    extern "C" int jor_collide_##SUF(const jg_shape_desc* da, const float* va, const jg_shape_desc* db,          \
                                     const float* vb, const double* qa, const double* qb, const double* pa,       \
                                     const double* pb, double threshold, int mode, double* out) {                 \
        Shape<R> sa, sb; std::vector<R> s1, s2; desc_to_shape<R>(da, va, sa, s1); desc_to_shape<R>(db, vb, sb, s2); \
        MprEpa<R> sol; V3<R> pA, pB, n; R pen = 0;                                                                 \
        bool hit = mode == 0 ? sol.mpr_epa_world(sa, sb, get4d<R>(qa), get4d<R>(qb), get3d<R>(pa), get3d<R>(pb), pA, pB, n, pen, (R)threshold) \
                             : sol.collision_world(sa, sb, get4d<R>(qa), get4d<R>(qb), get3d<R>(pa), get3d<R>(pb), pA, pB, n, pen); \
        put3d(out, pA); put3d(out + 3, pB); put3d(out + 6, n); out[9] = (double)pen;                             \
        out[10] = sol.epa_calls; out[11] = sol.epa_failures;                                                       \
        return hit ? 1 : 0;                                                                                        \
    }                                                                                                              \
    /* NarrowPhase.Sweep (NarrowPhase.cs:1100-1136): out = pA, pB, n, toi */                                     \
    extern "C" int jor_sweep_##SUF(const jg_shape_desc* da, const float* va, const jg_shape_desc* db,            \
                                   const float* vb, const double* qa, const double* qb, const double* pa,         \
                                   const double* pb, const double* sa_, const double* sb_, double* out) {          \
        Shape<R> sa, sb; std::vector<R> s1, s2; desc_to_shape<R>(da, va, sa, s1); desc_to_shape<R>(db, vb, sb, s2); \
        V3<R> pA, pB, n; R toi = 0;                                                                                \
        bool hit = sweep_world(sa, sb, get4d<R>(qa), get4d<R>(qb), get3d<R>(pa), get3d<R>(pb), get3d<R>(sa_),     \
                               get3d<R>(sb_), pA, pB, n, toi);                                                     \
        put3d(out, pA); put3d(out + 3, pB); put3d(out + 6, n); out[9] = (double)toi;                              \
        return hit ? 1 : 0;                                                                                        \
    }                                                                                                              \
    /* SimplexSolverAB.AddVertex over n Minkowski vertices (witness points zero): returns the     \
       last call's result, out = the closest point it reports */                                   \
    extern "C" int jor_simplex_##SUF(const double* verts, int n, double* out) {                                    \
        SimplexAB<R> sx; V3<R> c; bool r = true;                                                                   \
        for (int i = 0; i < n; i++) { Vertex<R> v; v.V = get3d<R>(verts + 3 * i); r = sx.add(v, c); }           \
        put3d(out, c);                                                                                             \
        return r ? 1 : 0;                                                                                          \
    }                                                                                                              \
    extern "C" int jor_manifold_##SUF(const jg_shape_desc* da, const float* va, const jg_shape_desc* db,         \
                                      const float* vb, const double* qa, const double* qb, const double* pa,      \
                                      const double* pb, const double* pA, const double* pB, const double* n,      \
                                      double* out) {                                                              \
        Shape<R> sa, sb; std::vector<R> s1, s2; desc_to_shape<R>(da, va, sa, s1); desc_to_shape<R>(db, vb, sb, s2); \
        Manifold<R> m;                                                                                             \
        m.build(sa, sb, get4d<R>(qa), get4d<R>(qb), get3d<R>(pa), get3d<R>(pb), get3d<R>(pA), get3d<R>(pB), get3d<R>(n)); \
        for (int i = 0; i < m.count; i++) { put3d(out + 6 * i, m.A[i]); put3d(out + 6 * i + 3, m.B[i]); }          \
        return m.count;                                                                                            \
    }                                                                                                              \
    extern "C" int jor_exact_side_##SUF(const double* a, const double* b, const double* c, const double* p) {     \
        return Expansion::side(get3d<R>(a), get3d<R>(b), get3d<R>(c), get3d<R>(p));                               \
    }                                                                                                              \
    extern "C" int jor_filter_side_##SUF(const double* a, const double* b, const double* c, const double* p, int* sign) { \
        PlaneFilter f; f.init(get3d<R>(a), get3d<R>(b), get3d<R>(c));                                              \
        return f.try_side(get3d<R>(a), get3d<R>(p), *sign) ? 1 : 0;                                                \
    }                                                                                                              \
    extern "C" void jor_stable_sincos_##SUF(double a, double* s, double* c) {                                     \
        R ss, cc; StableMath<R>::sincos((R)a, ss, cc); *s = ss; *c = cc;                                           \
    }                                                                                                              \
    extern "C" double jor_shortest_angle_##SUF(double a, double half) { return (double)shortest_angle((R)a, (R)half); } \
    extern "C" double jor_stable_atan2_##SUF(double y, double x) { return (double)StableMath<R>::atan2((R)y, (R)x); }

JOR_DEFINE(f, float)
JOR_DEFINE(d, double)

extern "C" const char* jor_version(void) { return "jitter oracle 1 (restates Jitter2 2.12.0 hot path)"; }
