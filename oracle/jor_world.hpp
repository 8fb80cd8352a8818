// Oracle (test infrastructure only): a CPU world that strings the restated stages
// together the way World.StepInternal does (World.Step.cs:153-296) with deactivation
// disabled.  Pairs are every shape pair with non-disjoint exact world AABBs on different
// bodies (DynamicTree.cs:266-286 + World.cs:447-455), found with a uniform grid.  Solve
// order: the reference's deterministic order (contacts sorted by arbiter key, then
// constraints by id; World.Deterministic.cs:142-203) or an external colour order
// (colour by colour; inside a colour rows share no dynamic body, so their order does
// not change the result).  A multithreaded variant restates the Regular mode's
// batch + try-lock scheme (World.Step.cs:428-526, :924-986) for the CPU baseline.
#pragma once
#include "jor_dynamics.hpp"
#include "jor_joints.hpp"
#include <algorithm>
#include <numeric>
#include <condition_variable>
#include <mutex>
#include <atomic>
#include <thread>
#include <functional>

namespace jor {

template <class R> struct World {
    std::vector<Body<R>> bodies;
    std::vector<Shape<R>> shapes;
    std::vector<int> shape_body;
    std::vector<R> hull;                       // point cloud vertices
    std::vector<ContactData<R>> arbiters;
    std::unordered_map<uint64_t, int> arb_index;
    std::vector<Joint<R>> joints;
    V3<R> gravity = V3<R>(0, -(R)9.81, 0);
    int substeps = 1, iterations = 6, relax = 4;
    bool aux_contacts = true, persistent = true, edge_filter = true;
    R spec_relax = (R)0.9;
    R spec_threshold = (R)10.0;                // SpeculativeVelocityThreshold
    R step_dt = 0;                             // dt of the step in progress
    // World.AllowDeactivation (World.cs:333; the reference's default is on) with the bodies'
    // default thresholds (RigidBody.cs:398-400)
    bool allow_deactivation = false;
    R sleep_lin2 = (R)0.1, sleep_ang2 = (R)0.1;
    std::vector<int> created;                  // arbiters created by this step's detection
    bool external_order = false;               // use ContactData::color / Joint::color
    bool record_residual = false;
    std::vector<R> residuals;                  // first substep, one value per iteration
    MprEpa<R> solver;
    EdgeFilter<R> efilter;
    int64_t n_pairs = 0, n_colliding = 0, n_points = 0, n_speculative = 0;
    int nthreads = 1;

    static uint64_t key(int a, int b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; }

    int find_or_create(int s1, int s2) {
        uint64_t k = key(s1, s2);
        auto it = arb_index.find(k);
        if (it != arb_index.end()) return it->second;
        ContactData<R> cd;
        int b1 = shape_body[s1], b2 = shape_body[s2];
        // ContactData.Init (Contact.cs:271-286)
        cd.b1 = b1; cd.b2 = b2; cd.key1 = s1; cd.key2 = s2;
        cd.friction = std::max(bodies[b1].friction, bodies[b2].friction);
        cd.restitution = std::max(bodies[b1].restitution, bodies[b2].restitution);
        cd.spec_relax = spec_relax;
        cd.mode = 0; cd.usage = 0;
        arbiters.push_back(cd);
        int idx = (int)arbiters.size() - 1;
        arb_index[k] = idx;
        created.push_back(idx);
        return idx;
    }
    // ContactData.ResetMode (Contact.cs:288-296)
    void reset_mode(ContactData<R>& cd) {
        cd.mode = (bodies[cd.b1].motion == DYNAMIC) ? 3 : 0;
        cd.mode |= (bodies[cd.b2].motion == DYNAMIC) ? 12 : 0;
    }

    std::vector<Box3<R>> aabbs() {
        std::vector<Box3<R>> out(shapes.size());
        for (size_t i = 0; i < shapes.size(); i++) {
            const Body<R>& b = bodies[shape_body[i]];
            out[i] = shape_aabb(shapes[i], b.q, b.pos);
            if (b.speculative) {
                // RigidBodyShape.UpdateWorldBoundingBox (RigidBodyShape.cs:37-57): grown by the
                // distance the linear velocity covers in one step
                R swept = step_dt * std::sqrt(len2(b.vel));
                out[i].mn = out[i].mn - V3<R>(swept);
                out[i].mx = out[i].mx + V3<R>(swept);
            }
        }
        return out;
    }
    // The reference's pair contract (DynamicTree.EnumerateOverlapsCallback with the
    // default filter, DynamicTree.cs:266-286, World.cs:447-455): every shape pair with
    // non-disjoint world AABBs, on different bodies of one world, at least one active and
    // one dynamic.  Evaluated with a uniform grid (the reference's tree gives the same
    // set): shapes spanning more than 8 cells on an axis are tested against all others,
    // the rest are binned by the cells their AABB covers and each pair is reported by the
    // cell that holds the lower corner of the two AABBs' intersection.
    // The same contract by sort-and-sweep on x: quadratic in dense scenes, kept to check
    // the grid against.
    std::vector<std::pair<int, int>> find_pairs_sweep() {
        auto box = aabbs();
        std::vector<int> ord(shapes.size());
        std::iota(ord.begin(), ord.end(), 0);
        std::sort(ord.begin(), ord.end(), [&](int a, int b) { return box[a].mn.x < box[b].mn.x; });
        std::vector<std::pair<int, int>> pairs;
        for (size_t ii = 0; ii < ord.size(); ii++) {
            int i = ord[ii];
            for (size_t jj = ii + 1; jj < ord.size(); jj++) {
                int j = ord[jj];
                if (box[j].mn.x > box[i].mx.x) break;
                if (disjoint(box[i], box[j]) || !pair_ok(i, j)) continue;
                pairs.push_back(i < j ? std::make_pair(i, j) : std::make_pair(j, i));
            }
        }
        std::sort(pairs.begin(), pairs.end());
        return pairs;
    }
    bool pair_ok(int i, int j) const {
        int bi = shape_body[i], bj = shape_body[j];
        if (bi == bj) return false;
        if (bodies[bi].world != bodies[bj].world) return false;
        if (!bodies[bi].active() && !bodies[bj].active()) return false;
        if (bodies[bi].motion != DYNAMIC && bodies[bj].motion != DYNAMIC) return false;
        return true;
    }
    std::vector<std::pair<int, int>> find_pairs() {
        auto box = aabbs();
        const int n = (int)shapes.size();
        std::vector<std::pair<int, int>> pairs;
        if (n < 2) return pairs;
        // cell size: twice the median largest AABB extent
        std::vector<double> ext(n);
        for (int i = 0; i < n; i++) {
            V3<R> d = box[i].mx - box[i].mn;
            ext[i] = std::max((double)d.x, std::max((double)d.y, (double)d.z));
        }
        std::vector<double> tmp(ext);
        std::nth_element(tmp.begin(), tmp.begin() + n / 2, tmp.end());
        const double cell = std::max(2.0 * tmp[n / 2], 1e-3);
        auto cidx = [&](double v) { return (long long)std::floor(v / cell); };
        std::vector<int> big;
        std::vector<std::pair<unsigned long long, int>> ent;
        ent.reserve((size_t)n * 4);
        // cell key: world id and cell coordinates (different worlds never share a cell;
        // coordinates wrap at 2^14 cells, which only adds candidate pairs)
        auto key = [](int world, long long x, long long y, long long z) {
            return ((unsigned long long)(x & 0x3FFF) << 50) | ((unsigned long long)(y & 0x3FFF) << 36) |
                   ((unsigned long long)(z & 0x3FFF) << 22) | (unsigned long long)(world & 0x3FFFFF);
        };
        auto wld = [&](int i) { return bodies[shape_body[i]].world; };
        for (int i = 0; i < n; i++) {
            long long x0 = cidx(box[i].mn.x), x1 = cidx(box[i].mx.x), y0 = cidx(box[i].mn.y), y1 = cidx(box[i].mx.y),
                      z0 = cidx(box[i].mn.z), z1 = cidx(box[i].mx.z);
            if (x1 - x0 > 8 || y1 - y0 > 8 || z1 - z0 > 8 || !(box[i].mx.x - box[i].mn.x < 1e30)) {
                big.push_back(i);
                continue;
            }
            for (long long x = x0; x <= x1; x++)
                for (long long y = y0; y <= y1; y++)
                    for (long long z = z0; z <= z1; z++) ent.push_back({key(wld(i), x, y, z), i});
        }
        std::sort(ent.begin(), ent.end());
        std::vector<std::pair<size_t, size_t>> runs;
        for (size_t s = 0; s < ent.size();) {
            size_t e = s + 1;
            while (e < ent.size() && ent[e].first == ent[s].first) e++;
            if (e - s > 1) runs.push_back({s, e});
            s = e;
        }
        const int nt = std::max(1, nthreads);
        std::vector<std::vector<std::pair<int, int>>> part(nt);
        std::atomic<int> slot{0};
        parallel_for((int)runs.size(), 64, [&](int b, int e) {
            thread_local std::vector<std::pair<int, int>> local;
            local.clear();
            for (int r = b; r < e; r++) {
                auto [s0, s1] = runs[r];
                unsigned long long ck = ent[s0].first;
                for (size_t a = s0; a < s1; a++)
                    for (size_t c = a + 1; c < s1; c++) {
                        int i = ent[a].second, j = ent[c].second;
                        if (disjoint(box[i], box[j]) || !pair_ok(i, j)) continue;
                        // report once: the cell of the intersection's lower corner
                        double lx = std::max((double)box[i].mn.x, (double)box[j].mn.x);
                        double ly = std::max((double)box[i].mn.y, (double)box[j].mn.y);
                        double lz = std::max((double)box[i].mn.z, (double)box[j].mn.z);
                        if (key(wld(i), cidx(lx), cidx(ly), cidx(lz)) != ck) continue;
                        local.push_back(i < j ? std::make_pair(i, j) : std::make_pair(j, i));
                    }
            }
            int k = slot.fetch_add(1);
            std::vector<std::pair<int, int>>& dst = part[k % nt];
            static std::mutex mu;
            std::lock_guard<std::mutex> lock(mu);
            dst.insert(dst.end(), local.begin(), local.end());
        });
        for (auto& p : part) pairs.insert(pairs.end(), p.begin(), p.end());
        // large shapes against every shape of their world
        if (!big.empty()) {
            std::vector<int> by_world(n);
            std::iota(by_world.begin(), by_world.end(), 0);
            std::stable_sort(by_world.begin(), by_world.end(), [&](int a, int b) { return wld(a) < wld(b); });
            for (int i : big) {
                auto lo = std::lower_bound(by_world.begin(), by_world.end(), wld(i), [&](int s, int w) { return wld(s) < w; });
                for (auto it = lo; it != by_world.end() && wld(*it) == wld(i); ++it) {
                    int j = *it;
                    if (j == i || (std::binary_search(big.begin(), big.end(), j) && j < i)) continue;
                    if (disjoint(box[i], box[j]) || !pair_ok(i, j)) continue;
                    pairs.push_back(i < j ? std::make_pair(i, j) : std::make_pair(j, i));
                }
            }
        }
        std::sort(pairs.begin(), pairs.end());
        pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
        return pairs;
    }

    struct DetectResult {
        bool hit = false;
        V3<R> n;
        int count = 0;
        V3<R> A[4], B[4];
        V3<R> pA, pB;
        R pen = 0;
        bool speculative = false;              // registered with SolveMode.Angular removed
    };
    // World.Detect (World.Detect.cs:125-218) up to, not including, RegisterContact.
    DetectResult detect(int sA, int sB, MprEpa<R>& sol) {
        DetectResult r;
        const Body<R>& b1 = bodies[shape_body[sA]];
        const Body<R>& b2 = bodies[shape_body[sB]];
        if (!b1.active() && !b2.active()) return r;
        if (b1.motion != DYNAMIC && b2.motion != DYNAMIC) return r;
        V3<R> pA, pB, n;
        R pen;
        bool hit = sol.mpr_epa_world(shapes[sA], shapes[sB], b1.q, b2.q, b1.pos, b2.pos, pA, pB, n, pen);
        if (!hit) {
            // speculative branch (World.Detect.cs:168-196): a sweep along the relative linear
            // velocity; a hit within the step registers its one point, linear terms only
            if (!b1.speculative && !b2.speculative) return r;
            V3<R> dv = b2.vel - b1.vel;
            if (len2(dv) < spec_threshold * spec_threshold) return r;
            R toi;
            bool ok = sweep_world(shapes[sA], shapes[sB], b1.q, b2.q, b1.pos, b2.pos, b1.vel, b2.vel, pA, pB, n, toi);
            if (!ok || toi > step_dt || toi == (R)0.0) return r;
            pen = dot(n, pA - pB) * spec_relax;
            if (edge_filter) {
                bool tri_dyn = shapes[sA].is_triangle() ? b1.motion == DYNAMIC : b2.motion == DYNAMIC;
                if (!efilter.filter(shapes[sA], shapes[sB], b1.q, b2.q, b1.pos, b2.pos, tri_dyn, sol, pA, pB, n, pen)) return r;
            }
            r.hit = true; r.speculative = true; r.n = n; r.pA = pA; r.pB = pB; r.pen = pen;
            r.count = 1; r.A[0] = pA; r.B[0] = pB;
            return r;
        }
        if (edge_filter) {
            bool tri_dyn = shapes[sA].is_triangle() ? b1.motion == DYNAMIC : b2.motion == DYNAMIC;
            if (!efilter.filter(shapes[sA], shapes[sB], b1.q, b2.q, b1.pos, b2.pos, tri_dyn, sol, pA, pB, n, pen)) return r;
        }
        r.hit = true; r.n = n; r.pA = pA; r.pB = pB; r.pen = pen;
        if (aux_contacts) {
            Manifold<R> m;
            m.build(shapes[sA], shapes[sB], b1.q, b2.q, b1.pos, b2.pos, pA, pB, n);
            r.count = m.count;
            for (int i = 0; i < m.count; i++) { r.A[i] = m.A[i]; r.B[i] = m.B[i]; }
        } else {
            r.count = 1; r.A[0] = pA; r.B[0] = pB;
        }
        return r;
    }
    // RegisterContact (World.Detect.cs:294-324)
    void register_contact(int sA, int sB, const DetectResult& r) {
        int ai = find_or_create(sA, sB);
        ContactData<R>& cd = arbiters[ai];
        if (!persistent) cd.usage = 0;
        reset_mode(cd);
        if (r.speculative) cd.mode &= ~(ContactData<R>::AngularBody1 | ContactData<R>::AngularBody2);
        for (int e = 0; e < r.count; e++) add_contact(cd, bodies, r.A[e], r.B[e], r.n);
    }

    void narrowphase() {
        created.clear();
        auto pairs = find_pairs();
        n_pairs = (int64_t)pairs.size();
        n_colliding = 0; n_points = 0; n_speculative = 0;
        if (nthreads <= 1) {
            for (auto& p : pairs) {
                DetectResult r = detect(p.first, p.second, solver);
                if (!r.hit) continue;
                n_colliding++; n_points += r.count; n_speculative += r.speculative;
                register_contact(p.first, p.second, r);
            }
            return;
        }
        std::vector<DetectResult> res(pairs.size());
        parallel_for((int)pairs.size(), 64, [&](int b, int e) {
            MprEpa<R> local;
            for (int i = b; i < e; i++) res[i] = detect(pairs[i].first, pairs[i].second, local);
        });
        for (size_t i = 0; i < pairs.size(); i++) {
            if (!res[i].hit) continue;
            n_colliding++; n_points += res[i].count; n_speculative += res[i].speculative;
            register_contact(pairs[i].first, pairs[i].second, res[i]);
        }
    }

    // ---- islands and deactivation --------------------------------------------------------
    // The reference keeps islands incrementally (IslandHelper.cs: merge on a new connection,
    // breadth-first split on a removed one); they are the connected components of the graph
    // of non-static bodies joined by arbiters and constraints, static bodies alone.  Their
    // two flags are kept per body here: MarkedAsActive (set by a body still moving,
    // RigidBody.cs:740-743, and by AddToActiveList) and membership of the active partition
    // (set by AddToActiveList, World.cs:903-910, cleared when the island goes to sleep).  A
    // merge ORs both flags and always comes with AddToActiveList; a split copies them to both
    // parts, and the splits of a step (RemoveBrokenArbiters) follow AddToActiveList on both
    // bodies of the removed arbiter, so the OR over a component's bodies is the island's flag.
    static bool non_static(const Body<R>& b) { return b.motion != STATIC; }
    // AddToActiveList (World.cs:903-910) on the island of body i
    void add_to_active(int i) { bodies[i].marked = true; bodies[i].island_active = true; }
    // a row is solved while its non-static bodies are awake (memContacts / constraint
    // activation follows DeactivateBodyForSleep and activation, World.Step.cs:1247-1275, :1325-1345)
    bool row_awake(int b1, int b2) const {
        return (non_static(bodies[b1]) && bodies[b1].active()) || (non_static(bodies[b2]) && bodies[b2].active());
    }
    int uf_find(std::vector<int>& p, int x) {
        while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; }
        return x;
    }
    // CheckDeactivation (World.Step.cs:1289-1371) on the components of the connection graph
    void check_deactivation() {
        const int n = (int)bodies.size();
        std::vector<int> parent(n);
        std::iota(parent.begin(), parent.end(), 0);
        auto join = [&](int a, int b) {
            if (!non_static(bodies[a]) || !non_static(bodies[b])) return;
            a = uf_find(parent, a); b = uf_find(parent, b);
            if (a != b) parent[std::max(a, b)] = std::min(a, b);
        };
        for (auto& a : arbiters) join(a.b1, a.b2);
        for (auto& j : joints) join(j.b1, j.b2);
        std::vector<char> any_active(n, 0), any_marked(n, 0);
        for (int i = 0; i < n; i++) {
            int r = uf_find(parent, i);
            any_active[r] |= bodies[i].island_active;
            any_marked[r] |= bodies[i].marked;
        }
        for (int i = 0; i < n; i++) {
            Body<R>& b = bodies[i];
            int r = uf_find(parent, i);
            if (!any_active[r]) continue;            // a sleeping island is not visited
            b.marked = false;
            if (!any_marked[r] && allow_deactivation) {
                // DeactivateBodyForSleep (World.Step.cs:1247-1287): velocities are kept
                b.flags &= ~4;
                b.island_active = false;
            } else {
                b.island_active = true;
                if (!b.active() && b.motion != STATIC) { b.flags |= 4; b.sleep_time = 0; }
            }
        }
    }
    // RigidBody.Update's rest test (RigidBody.cs:723-743)
    // (on the velocities restricted to the allowed motion axes, as Update restricts them first)
    void sleep_update(Body<R>& b, const TimeStep<R>& ts) {
        bool kin = b.motion == KINEMATIC;
        V3<R> zero, v = b.vel, av = b.angvel;
        restrict_linear(v, b.allowed());
        restrict_angular(av, b.allowed());
        bool resting = kin ? (av == zero && v == zero) : (len2(av) < b.sleep_ang2 && len2(v) < b.sleep_lin2);
        b.sleep_time = resting ? b.sleep_time + ts.dt : (R)0;
        if ((kin && !resting) || b.sleep_time < b.deactivation_time) b.marked = true;
    }
    // World.ActivateBodyNextStep (World.cs:696-720) for a dynamic or kinematic body:
    // SetActivationState(true) and the setters that wake a body
    void activate_body(int i) {
        Body<R>& b = bodies[i];
        b.sleep_time = 0;
        if (b.active() || b.motion == STATIC) return;
        add_to_active(i);
    }

    // Solve order: indices into arbiters and joints, grouped by colour.
    std::vector<std::vector<int>> order_arb, order_joint;
    void build_order() {
        order_arb.clear(); order_joint.clear();
        if (!external_order) {
            std::vector<int> a;
            for (int i = 0; i < (int)arbiters.size(); i++)
                if (!allow_deactivation || row_awake(arbiters[i].b1, arbiters[i].b2)) a.push_back(i);
            std::sort(a.begin(), a.end(), [&](int x, int y) {
                return std::make_pair(arbiters[x].key1, arbiters[x].key2) < std::make_pair(arbiters[y].key1, arbiters[y].key2);
            });
            std::vector<int> j;
            for (int i = 0; i < (int)joints.size(); i++)
                if (!allow_deactivation || row_awake(joints[i].b1, joints[i].b2)) j.push_back(i);
            order_arb.push_back(a);
            order_joint.push_back(std::vector<int>());
            order_arb.push_back(std::vector<int>());
            order_joint.push_back(j);
            return;
        }
        int nc = 0;
        for (auto& a : arbiters) nc = std::max(nc, a.color + 1);
        for (auto& j : joints) nc = std::max(nc, j.color + 1);
        order_arb.assign(nc, {});
        order_joint.assign(nc, {});
        for (size_t i = 0; i < arbiters.size(); i++)
            if (!allow_deactivation || row_awake(arbiters[i].b1, arbiters[i].b2)) order_arb[arbiters[i].color].push_back((int)i);
        for (size_t i = 0; i < joints.size(); i++)
            if (!allow_deactivation || row_awake(joints[i].b1, joints[i].b2)) order_joint[joints[i].color].push_back((int)i);
    }
    R residual_norm(std::vector<R>& prev) {
        double d2 = 0, l2 = 0;
        size_t k = 0;
        for (auto& cd : arbiters)
            for (int c = 0; c < 4; c++) {
                if (!(cd.usage & (1u << c))) continue;
                for (int r = 0; r < 3; r++) {
                    R v = cd.c[c].acc[r];
                    if (k < prev.size()) { double d = (double)v - prev[k]; d2 += d * d; prev[k] = v; }
                    else prev.push_back(v);
                    l2 += (double)v * v;
                    k++;
                }
            }
        return (R)(std::sqrt(d2) / std::max(std::sqrt(l2), 1e-12));
    }
    std::vector<R> snapshot_acc() {
        std::vector<R> v;
        for (auto& cd : arbiters)
            for (int c = 0; c < 4; c++)
                if (cd.usage & (1u << c)) for (int r = 0; r < 3; r++) v.push_back(cd.c[c].acc[r]);
        return v;
    }

    // bodies the step moves: all, or with deactivation the awake ones (memRigidBodies.Active)
    bool moves(const Body<R>& b) const { return !allow_deactivation || b.active(); }
    void solve_substep(const TimeStep<R>& ts, bool first, bool integrate = true) {
        if (integrate) for (auto& b : bodies) if (moves(b)) integrate_forces(b);
        // prepare (World.Step.cs:1155-1172)
        for (size_t c = 0; c < order_arb.size(); c++) {
            for (int i : order_arb[c]) contactdata_prepare(arbiters[i], bodies, ts);
            for (int i : order_joint[c]) joint_prepare(joints[i], bodies, ts);
        }
        std::vector<R> prev;
        if (first && record_residual) { prev = snapshot_acc(); residuals.clear(); }
        for (int it = 0; it < iterations; it++) {
            for (size_t c = 0; c < order_arb.size(); c++) {
                for (int i : order_arb[c]) contactdata_iterate(arbiters[i], bodies, true);
                for (int i : order_joint[c]) joint_iterate(joints[i], bodies, ts);
            }
            if (first && record_residual) residuals.push_back(residual_norm(prev));
        }
        if (integrate) for (auto& b : bodies) if (moves(b)) integrate_velocities(b, ts);
        for (int it = 0; it < relax; it++)
            for (size_t c = 0; c < order_arb.size(); c++)
                for (int i : order_arb[c]) contactdata_iterate(arbiters[i], bodies, false);
    }

    // World.Stabilize (World.Step.cs:318-392), Regular mode: CheckDeactivation, then per substep
    // SolveVelocities and RelaxVelocities on the present contacts and constraints, with no
    // detection and no integration
    void stabilize(R dt, int solver_iterations, int relaxation_iterations) {
        if (dt < std::numeric_limits<R>::epsilon()) return;
        TimeStep<R> ts(dt, substeps);
        step_dt = dt;
        if (allow_deactivation) check_deactivation();
        const int it = iterations, rx = relax;
        iterations = solver_iterations;
        relax = relaxation_iterations;
        build_order();
        for (int s = 0; s < substeps; s++) solve_substep(ts, false, false);
        iterations = it;
        relax = rx;
    }

    // RemoveBrokenArbiters (World.Step.cs:839-860): arbiters still without contacts.
    void remove_broken() {
        std::vector<ContactData<R>> keep;
        keep.reserve(arbiters.size());
        for (auto& a : arbiters) {
            if ((a.usage & 15u) != 0) { keep.push_back(a); continue; }
            // AddToActiveList on both islands before the arbiter goes (World.Step.cs:845-846)
            if (allow_deactivation) { add_to_active(a.b1); add_to_active(a.b2); }
        }
        arbiters.swap(keep);
        arb_index.clear();
        for (size_t i = 0; i < arbiters.size(); i++) arb_index[key(arbiters[i].key1, arbiters[i].key2)] = (int)i;
    }

    // World.StepInternal (World.Step.cs:153-296) with deactivation disabled.
    // narrow=false skips detection (the caller registered contacts itself).
    void step(R dt, bool narrow = true) {
        if (dt < std::numeric_limits<R>::epsilon()) return;
        TimeStep<R> ts(dt, substeps);
        step_dt = dt;
        if (narrow) narrowphase();
        if (allow_deactivation) {
            // HandleDeferredArbiters (World.Step.cs:880-914), then CheckDeactivation
            for (int i : created) { add_to_active(arbiters[i].b1); add_to_active(arbiters[i].b2); }
            check_deactivation();
        }
        build_order();
        for (int s = 0; s < substeps; s++) solve_substep(ts, s == 0);
        remove_broken();
        for (auto& a : arbiters)
            if (!allow_deactivation || row_awake(a.b1, a.b2)) contactdata_update_position(a, bodies);
        for (auto& b : bodies) {
            if (!moves(b)) continue;
            if (allow_deactivation) sleep_update(b, ts);
            body_update(b, ts, gravity);
        }
    }

    // --- threading for the multithreaded Regular-mode restatement ---------------------
    void parallel_for(int n, int batch, const std::function<void(int, int)>& fn) {
        std::atomic<int> next{0};
        auto worker = [&]() {
            while (true) {
                int b = next.fetch_add(batch);
                if (b >= n) break;
                fn(b, std::min(n, b + batch));
            }
        };
        std::vector<std::thread> th;
        for (int t = 1; t < nthreads; t++) th.emplace_back(worker);
        worker();
        for (auto& t : th) t.join();
    }
};

// Multithreaded Regular-mode step (World.Step.cs:428-526, :924-986): batches of 64
// arbiters per task, a per-body try-lock, and a deferred queue for locked rows.  Used
// only as the timed CPU baseline.
template <class R> struct RegularSolver {
    World<R>& w;
    std::vector<std::atomic<int>> locks;
    explicit RegularSolver(World<R>& world) : w(world), locks(world.bodies.size()) {
        for (auto& l : locks) l.store(0);
    }
    bool try_lock_two(int a, int b) {
        bool da = w.bodies[a].motion == DYNAMIC, db = w.bodies[b].motion == DYNAMIC;
        int lo = std::min(a, b), hi = std::max(a, b);
        bool dlo = lo == a ? da : db, dhi = hi == a ? da : db;
        int z = 0;
        if (dlo && !locks[lo].compare_exchange_strong(z, 1)) return false;
        z = 0;
        if (dhi && hi != lo && !locks[hi].compare_exchange_strong(z, 1)) {
            if (dlo) locks[lo].store(0);
            return false;
        }
        return true;
    }
    void unlock_two(int a, int b) {
        if (w.bodies[a].motion == DYNAMIC) locks[a].store(0);
        if (b != a && w.bodies[b].motion == DYNAMIC) locks[b].store(0);
    }
    template <class F> void sweep(const F& fn) {
        int n = (int)w.arbiters.size();
        w.parallel_for(n, 64, [&](int b, int e) {
            std::vector<int> q;
            for (int i = b; i < e; i++) {
                auto& cd = w.arbiters[i];
                if (!try_lock_two(cd.b1, cd.b2)) { q.push_back(i); continue; }
                fn(cd);
                unlock_two(cd.b1, cd.b2);
            }
            size_t h = 0;
            while (h < q.size()) {
                int i = q[h++];
                auto& cd = w.arbiters[i];
                if (!try_lock_two(cd.b1, cd.b2)) { q.push_back(i); continue; }
                fn(cd);
                unlock_two(cd.b1, cd.b2);
            }
        });
    }
    void step(R dt) {
        TimeStep<R> ts(dt, w.substeps);
        w.step_dt = dt;
        w.narrowphase();
        locks = std::vector<std::atomic<int>>(w.bodies.size());
        for (auto& l : locks) l.store(0);
        int nb = (int)w.bodies.size();
        for (int s = 0; s < w.substeps; s++) {
            w.parallel_for(nb, 256, [&](int b, int e) { for (int i = b; i < e; i++) integrate_forces(w.bodies[i]); });
            sweep([&](ContactData<R>& cd) { contactdata_prepare(cd, w.bodies, ts); });
            for (auto& j : w.joints) joint_prepare(j, w.bodies, ts);
            for (int it = 0; it < w.iterations; it++) {
                sweep([&](ContactData<R>& cd) { contactdata_iterate(cd, w.bodies, true); });
                for (auto& j : w.joints) joint_iterate(j, w.bodies, ts);
            }
            w.parallel_for(nb, 256, [&](int b, int e) { for (int i = b; i < e; i++) integrate_velocities(w.bodies[i], ts); });
            for (int it = 0; it < w.relax; it++)
                sweep([&](ContactData<R>& cd) { contactdata_iterate(cd, w.bodies, false); });
        }
        w.remove_broken();
        w.parallel_for((int)w.arbiters.size(), 256, [&](int b, int e) {
            for (int i = b; i < e; i++) contactdata_update_position(w.arbiters[i], w.bodies);
        });
        w.parallel_for(nb, 256, [&](int b, int e) { for (int i = b; i < e; i++) body_update(w.bodies[i], ts, w.gravity); });
    }
};

}  // namespace jor
