// The C ABI (include/jitter_gpu.h): world lifetime, state upload/download, the step
// driver and inspection.  One jg_world owns one CUDA stream and all of its device pools;
// every call returns a status and never throws.  The step is a fixed launch sequence
// whose sizes live in device memory, so it can be captured once per arbiter-buffer parity
// into a CUDA graph and replayed.
#include "jg_world.cuh"
#include <cstring>
#include <cmath>
#include <vector>
#include <string>
#include <algorithm>
#include <chrono>
#include <mutex>
#include <climits>

void jg_flip_store(WorldDev& w);
void jg_launch_count_contacts(WorldDev& w, cudaStream_t s, int nsm);
void jg_launch_update_contacts(WorldDev& w, cudaStream_t s, int nsm);
void jg_solver_reset_launch_cache(WorldDev& w);
int jg_solver_init();
int jg_schedule_init();
void jg_launch_activate(WorldDev& w, int body, cudaStream_t s);
void jg_launch_wake_dynamic(WorldDev& w, int body, cudaStream_t s);
void jg_launch_sleep_settings(WorldDev& w, int body, float t, float lin2, float ang2, cudaStream_t s);
void jg_launch_sleep_init(float4* sleep, int n, cudaStream_t s);
int jg_mlp_step_hook(jg_world* w, const StepParams& p);
void jg_mlp_free(void* mlp);
void jg_launch_collide_query(WorldDev& w, const int2* pairs, int n, float threshold, float* out, int* hit,
                             cudaStream_t s, int nsm);
int jg_schedule_launches(const StepParams& p);
int jg_narrowphase_init();
void jg_launch_manifold_query(WorldDev& w, const int2* pairs, int n, const float* in, float* out, int* count,
                              cudaStream_t s, int nsm);

static thread_local std::string g_err;

struct jg_world {
    jg_world_params prm{};
    WorldDev d{};
    cudaStream_t stream = nullptr;
    int device = 0, nsm = 0;
    DevCounters* h_ctr = nullptr;     // pinned
    jg_body_desc* d_desc = nullptr;   // device copy of the body descriptors (last upload, updated by downloads)
    jg_body_desc* d_stage = nullptr;  // an upload lands here and becomes d_desc once it is valid
    int* d_bad = nullptr;             // first invalid body of an upload: index * 4 + reason
    int* h_bad = nullptr;             // pinned
    std::vector<jg_body_desc> host_bodies;
    bool host_current = false;         // host_bodies equals the device state (no step since the upload)
    std::vector<jg_shape_desc> host_shapes;
    int nj_host = 0;
    std::vector<JointDev> pending_joints;  // added since the last step, uploaded in one copy
    cudaEvent_t ev[9]{};
    jg_timings timings{};
    jg_counters counters{};
    cudaGraphExec_t graph[2]{nullptr, nullptr};
    float graph_dt[2]{-1.f, -1.f};
    int nworlds = 1;
    std::vector<void*> allocs;
    bool mlp_ready = false;
    int launches = 0;
    // jg_collide_pairs scratch, grown on demand: pairs, 10 floats and a hit flag per pair
    int2* q_pairs = nullptr;
    float* q_out = nullptr;
    int* q_hit = nullptr;
    int q_cap = 0;
    void* mlp = nullptr;              // learned warm start state (jg_mlp.cu)
};

extern "C" {
static void invalidate_graphs(jg_world* w);
}

namespace {

int cuda_fail(cudaError_t e, const char* what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return JG_ERR_CUDA;
}
#define CK(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) return cuda_fail(_e, #x); } while (0)

template <class T> int dalloc(jg_world* w, T** p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    cudaMemsetAsync(*p, 0, sizeof(T) * count, w->stream);
    w->allocs.push_back(*p);
    return JG_OK;
}
#define DA(ptr, n) do { int _r = dalloc(w, &(ptr), (size_t)(n)); if (_r) return _r; } while (0)

int alloc_store(jg_world* w, ArbStore& A, int cap) {
    DA(A.key, cap); DA(A.body, cap); DA(A.info, cap); DA(A.mat, cap);
    DA(A.lslot, cap); DA(A.sv, 2 * (size_t)cap);
    DA(A.cn, 4 * cap); DA(A.ct1, 4 * cap); DA(A.ct2, 4 * cap); DA(A.cr1, 4 * cap);
    DA(A.cr2, 4 * cap); DA(A.cacc, 4 * cap); DA(A.cp1, 4 * cap); DA(A.cp2, 4 * cap);
    return JG_OK;
}

int next_pow2(int v) { int p = 1; while (p < v) p <<= 1; return p; }

int allocate(jg_world* w) {
    WorldDev& d = w->d;
    const jg_world_params& p = w->prm;
    if (p.max_bodies >= (1 << 29)) {  // the broadphase packs a body id into 29 bits
        g_err = "max_bodies must be below 2^29";
        return JG_ERR_INVALID_ARG;
    }
    d.cap_bodies = std::max(p.max_bodies, 16);
    d.cap_shapes = std::max(p.max_shapes, 16);
    d.cap_pairs = std::max(p.max_pairs, 1024);
    d.cap_arb = std::max(p.max_arbiters, 1024);
    d.cap_joints = std::max(p.max_constraints, 16);
    d.cap_hull = 64;
    d.cap_tris = 16;
    DA(d.body, d.cap_bodies); DA(d.pos, d.cap_bodies); DA(d.q, d.cap_bodies); DA(d.dv, d.cap_bodies);
    DA(d.dw, d.cap_bodies); DA(d.il0, d.cap_bodies); DA(d.il1, d.cap_bodies); DA(d.force, d.cap_bodies);
    DA(d.torque, d.cap_bodies); DA(d.mat, d.cap_bodies); DA(d.binfo, d.cap_bodies);
    DA(d.sleep, d.cap_bodies); DA(d.uf, d.cap_bodies); DA(d.ufl, d.cap_bodies);
    jg_launch_sleep_init(d.sleep, d.cap_bodies, w->stream);
    DA(d.sinfo, d.cap_shapes); DA(d.sdims, d.cap_shapes); DA(d.scenter, d.cap_shapes);
    DA(d.amin, d.cap_shapes); DA(d.amax, d.cap_shapes);
    DA(d.mkey, d.cap_shapes); DA(d.mkey_alt, d.cap_shapes); DA(d.midx, d.cap_shapes); DA(d.midx_alt, d.cap_shapes);
    int rs_blocks = (d.cap_shapes + 2047) / 2048;
    DA(d.hist, std::max(256 * rs_blocks + 1, 8192));
    DA(d.node, d.cap_shapes); DA(d.node_range, d.cap_shapes); DA(d.nmin, d.cap_shapes); DA(d.nmax, d.cap_shapes);
    DA(d.cbox, 4 * (size_t)d.cap_shapes);
    DA(d.leaf_parent, d.cap_shapes); DA(d.node_parent, d.cap_shapes); DA(d.node_flag, d.cap_shapes);
    DA(d.scene_box, 2);
    DA(d.pairs, d.cap_pairs);
    DA(d.pair_order, d.cap_pairs); DA(d.pair_kind, 2 * 64);
    DA(d.cs_key, d.cap_pairs); DA(d.cs_n, d.cap_pairs); DA(d.cs_pa, 4 * (size_t)d.cap_pairs); DA(d.cs_pb, 4 * (size_t)d.cap_pairs);
    int r;
    if ((r = alloc_store(w, d.arb[0], d.cap_arb))) return r;
    if ((r = alloc_store(w, d.arb[1], d.cap_arb))) return r;
    d.cur = 0;
    DA(d.col_pair, d.cap_arb); DA(d.col_res, 3 * (size_t)d.cap_arb); DA(d.col_portal, 12 * (size_t)d.cap_arb);
    DA(d.epa_list, d.cap_arb); DA(d.edge_list, d.cap_arb); DA(d.spec_list, d.cap_pairs);
    d.hcap = next_pow2(2 * d.cap_arb);
    DA(d.hkeys, d.hcap); DA(d.hvals, d.hcap);
    DA(d.cstat, d.cap_arb + d.cap_joints);
    DA(d.bmask, 2 * (size_t)d.cap_bodies);
    DA(d.adj_off, d.cap_bodies + 1);
    DA(d.adj, 2 * ((size_t)d.cap_arb + d.cap_joints));
    DA(d.deg, d.cap_bodies);
    DA(d.color_count, JG_MAX_COLORS + 1); DA(d.color_start, JG_MAX_COLORS + 1); DA(d.jcolor_start, JG_MAX_COLORS + 1);
    DA(d.color_cursor, JG_MAX_COLORS + 1);
    DA(d.jorder, d.cap_joints + JG_MAX_COLORS);
    DA(d.joints, d.cap_joints);
    DA(d.bar_count, 2); d.bar_gen = d.bar_count + 1;
    DA(d.resid, 2 * JG_RESID_MAX);
    DA(d.ctr, 1);
    // partitioned solve schedule
    DA(d.sc, 1);
    DA(d.sc_cell, 3 * (size_t)d.cap_bodies); DA(d.sc_stamp, 3 * (size_t)d.cap_bodies);
    DA(d.sc_bslot, 3 * (size_t)d.cap_bodies); DA(d.sc_tbody, 3 * (size_t)d.cap_bodies);
    DA(d.sc_arb, d.cap_arb); DA(d.sc_tlist, d.cap_arb); DA(d.sc_dst, d.cap_arb); DA(d.sc_lcol, d.cap_arb);
    DA(d.sc_ls, d.cap_arb);
    DA(d.sc_acount, 3 * JG_SCHED_MAXCELLS); DA(d.sc_bcount, 3 * JG_SCHED_MAXCELLS); DA(d.sc_task_of, 3 * JG_SCHED_MAXCELLS);
    DA(d.sc_task, JG_SCHED_MAXTASKS); DA(d.sc_cursor, JG_SCHED_MAXTASKS); DA(d.sc_tnc, JG_SCHED_MAXTASKS);
    DA(d.sc_tcell, JG_SCHED_MAXTASKS); DA(d.sc_tdep, 2 * JG_SCHED_MAXTASKS); DA(d.sc_done, JG_SCHED_MAXTASKS);
    DA(d.sc_tcol, (size_t)JG_SCHED_MAXTASKS * (JG_TASK_MAXC + 1));
    DA(d.ev_created, d.cap_arb); DA(d.ev_removed, d.cap_arb); DA(d.remaining, 2); DA(d.dst_index, d.cap_arb);
    CK(cudaMallocHost((void**)&w->h_ctr, sizeof(DevCounters)));
    memset(w->h_ctr, 0, sizeof(DevCounters));
    DA(w->d_desc, d.cap_bodies); DA(w->d_stage, d.cap_bodies); DA(w->d_bad, 1);
    CK(cudaMallocHost((void**)&w->h_bad, sizeof(int)));
    return JG_OK;
}

int ensure_hull(jg_world* w, int n) {
    if (n <= w->d.cap_hull && w->d.hull) return JG_OK;
    w->d.cap_hull = std::max(n, 64);
    DA(w->d.hull, w->d.cap_hull);
    return JG_OK;
}
int ensure_tris(jg_world* w, int n) {
    if (n <= w->d.cap_tris && w->d.tris) return JG_OK;
    w->d.cap_tris = std::max(n, 16);
    DA(w->d.tris, w->d.cap_tris);
    return JG_OK;
}

JG_HD bool finite3(const float* v) { return isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]); }
float host_int_as_float(int i) { float f; memcpy(&f, &i, 4); return f; }
int host_float_as_int(float f) { int i; memcpy(&i, &f, 4); return i; }

// RigidBody.UpdateWorldInertia (RigidBody.cs:903-923) on the host, for uploads.
JG_HD void body_world_inertia(const jg_body_desc& b, float* i0, float* i1, float* imv) {
    float x = b.orientation[0], y = b.orientation[1], z = b.orientation[2], ww = b.orientation[3];
    m33 R;
    R.m[0][0] = 1.0f - 2.0f * (y * y + z * z); R.m[0][1] = 2.0f * (x * y - z * ww); R.m[0][2] = 2.0f * (x * z + y * ww);
    R.m[1][0] = 2.0f * (x * y + z * ww); R.m[1][1] = 1.0f - 2.0f * (x * x + z * z); R.m[1][2] = 2.0f * (y * z - x * ww);
    R.m[2][0] = 2.0f * (x * z - y * ww); R.m[2][1] = 2.0f * (y * z + x * ww); R.m[2][2] = 1.0f - 2.0f * (x * x + y * y);
    sym6 L{b.inv_inertia[0], b.inv_inertia[1], b.inv_inertia[2], b.inv_inertia[3], b.inv_inertia[4], b.inv_inertia[5]};
    sym6 I = sym_transform(L, R);
    int axes = 63 ^ ((b.flags >> 4) & 63);
    if (((b.flags >> 4) & 56) != 0) {
        if ((axes & 56) == 0) { I = sym6{0, 0, 0, 0, 0, 0}; }
        else {
            if (!(axes & 8)) { if (I.m11 > 0) { float xy = I.m12 / I.m11, xz = I.m13 / I.m11; I.m22 -= xy * I.m12; I.m23 -= xy * I.m13; I.m33 -= xz * I.m13; } I.m11 = I.m12 = I.m13 = 0; }
            if (!(axes & 16)) { if (I.m22 > 0) { float xy = I.m12 / I.m22, yz = I.m23 / I.m22; I.m11 -= xy * I.m12; I.m13 -= xy * I.m23; I.m33 -= yz * I.m23; } I.m12 = I.m22 = I.m23 = 0; }
            if (!(axes & 32)) { if (I.m33 > 0) { float xz = I.m13 / I.m33, yz = I.m23 / I.m33; I.m11 -= xz * I.m13; I.m12 -= xz * I.m23; I.m22 -= yz * I.m23; } I.m13 = I.m23 = I.m33 = 0; }
        }
    }
    imv[0] = imv[1] = imv[2] = b.inv_mass;
    if (!(axes & 1)) imv[0] = 0;
    if (!(axes & 2)) imv[1] = 0;
    if (!(axes & 4)) imv[2] = 0;
    if (b.motion_type != JG_MOTION_DYNAMIC) { I = sym6{0, 0, 0, 0, 0, 0}; imv[0] = imv[1] = imv[2] = 0; }
    i0[0] = I.m11; i0[1] = I.m12; i0[2] = I.m13; i0[3] = I.m22;
    i1[0] = I.m23; i1[1] = I.m33;
}

__global__ void k_reset_counters(DevCounters* c) {
    int narb = c->narb;
    DevCounters z;
    memset(&z, 0, sizeof(z));
    z.narb = narb;
    *c = z;
}

// The partition's cell density: 0 (the default) or a finite value in (0, 64].
bool cells_per_sm_ok(float c) { return c == 0.f || (std::isfinite(c) && c > 0.f && c <= 64.f); }

StepParams make_params(const jg_world* w, float dt) {
    StepParams sp;
    const jg_world_params& p = w->prm;
    sp.dt = dt;
    sp.substeps = p.substeps;
    sp.sub_dt = dt / (float)p.substeps;
    sp.inv_dt = dt > 0 ? 1.0f / dt : 0;
    sp.inv_sub_dt = sp.sub_dt > 0 ? 1.0f / sp.sub_dt : 0;
    sp.gravity = make_float3(p.gravity[0], p.gravity[1], p.gravity[2]);
    sp.iterations = p.solver_iterations;
    sp.relax = p.relax_iterations;
    sp.aux_contacts = p.enable_auxiliary_contacts;
    sp.persistent = p.persistent_manifold;
    sp.edge_filter = p.edge_filter;
    sp.spec_relax = p.speculative_relaxation;
    sp.spec_threshold = p.speculative_threshold;
    sp.warm_start = p.warm_start_mode;
    sp.record_residual = p.record_residual;
    sp.partition = p.partitioned_solve ? 1 : 0;
    sp.allow_deact = p.allow_deactivation ? 1 : 0;
    sp.stabilize = 0;
    sp.task_maxb = jg_solver_task_maxb(p.solver_block > 0 ? p.solver_block : JG_TASK_BLOCK,
                                       p.solver_ctas_per_sm > 0 ? p.solver_ctas_per_sm : JG_TASK_CTAS);
    if (sp.task_maxb < 64) sp.partition = 0;  // a block too large for a useful task
    sp.cells_per_sm = p.sched_cells_per_sm;  // 0: chosen on the device (cell count and arbiter count)
    sp.solve_blocks = w->nsm * (p.solver_ctas_per_sm > 0 ? p.solver_ctas_per_sm : JG_TASK_CTAS);
    return sp;
}

// The launch sequence of one step.  `timed` records stage events (not inside graphs).
int launch_step(jg_world* w, const StepParams& sp, bool timed) {
    WorldDev& d = w->d;
    cudaStream_t s = w->stream;
    if (timed) cudaEventRecord(w->ev[0], s);
    k_reset_counters<<<1, 1, 0, s>>>(d.ctr);
    if (sp.record_residual) cudaMemsetAsync(d.resid, 0, sizeof(float) * 2 * JG_RESID_MAX, s);
    jg_launch_aabb(d, sp.dt, s);
    int passes = jg_launch_broadphase(d, s, w->nsm);
    // kernels of this sequence: reset 1, aabb 2, broadphase 1 + 3 per radix pass + 4,
    // narrowphase 3 + 5, merge 3 (+ warm-start hook), schedule, colour/permute 4, count 1,
    // solve 1, contact update 1, body update 1
    w->launches = 1 + 2 + (d.ns >= 2 ? 5 + 3 * passes : 0) + 8 + 3 + 4 + 1 + 1 + 1 + 1 + jg_schedule_launches(sp);
    if (timed) cudaEventRecord(w->ev[1], s);
    jg_launch_narrowphase(d, sp, s, w->nsm, w->prm.narrow_tile);
    if (timed) cudaEventRecord(w->ev[2], s);
    d.allow_deact = sp.allow_deact;
    jg_launch_merge(d, sp, s, w->nsm);
    w->launches += jg_mlp_step_hook(w, sp);
    if (sp.allow_deact) {
        jg_launch_islands(d, s, w->nsm);  // HandleDeferredArbiters done in the merge, then CheckDeactivation
        w->launches += 4;
    }
    if (timed) cudaEventRecord(w->ev[3], s);
    jg_launch_schedule(d, sp, s, w->nsm);
    if (jg_launch_color(d, s, w->nsm) < 0) {
        g_err = "cooperative launch of the colouring failed";
        return JG_ERR_CUDA;
    }
    jg_flip_store(d);
    if (timed) cudaEventRecord(w->ev[4], s);
    jg_launch_count_contacts(d, s, w->nsm);
    if (jg_launch_solve(d, sp, s, w->nsm, w->prm.solver_block, w->prm.solver_ctas_per_sm) < 0) {
        g_err = "cooperative launch of the solver failed";
        return JG_ERR_CUDA;
    }
    if (timed) cudaEventRecord(w->ev[5], s);
    jg_launch_update_contacts(d, s, w->nsm);
    if (timed) cudaEventRecord(w->ev[6], s);
    jg_launch_update(d, sp, s, w->nsm);
    if (timed) cudaEventRecord(w->ev[7], s);
    return JG_OK;
}

// timed: stage times from the stage events; graph_timed: only the total (a graph replay)
int finish_step(jg_world* w, bool timed, bool graph_timed = false) {
    CK(cudaMemcpyAsync(w->h_ctr, w->d.ctr, sizeof(DevCounters), cudaMemcpyDeviceToHost, w->stream));
    CK(cudaStreamSynchronize(w->stream));
    CK(cudaGetLastError());
    const DevCounters& c = *w->h_ctr;
    jg_counters& o = w->counters;
    o.pairs = c.npairs; o.colliding = c.nstream; o.manifold_points = c.points; o.arbiters = c.narb;
    o.contacts = c.contacts; o.new_contacts = c.new_contacts; o.colors = c.ncolors; o.epa_calls = c.nepa;
    o.epa_failures = c.epa_fail; o.exact_fallbacks = c.exact; o.status = c.status;
    o.created_arbiters = c.nnew; o.removed_arbiters = c.nremoved;
    o.kernel_launches = w->launches;
    o.solver_tasks = c.ntasks; o.task_arbiters = c.narb_task; o.task_colors = c.task_colors;
    o.speculative_contacts = c.nspec_hit;
    if (timed) {
        float t[8];
        for (int i = 0; i < 7; i++) cudaEventElapsedTime(&t[i], w->ev[i], w->ev[i + 1]);
        jg_timings& tm = w->timings;
        tm.broadphase = t[0]; tm.narrowphase = t[1]; tm.add_arbiter = t[2]; tm.coloring = t[3];
        tm.solve = t[4]; tm.update_contacts = t[5]; tm.update_bodies = t[6];
        cudaEventElapsedTime(&tm.total, w->ev[0], w->ev[7]);
    } else if (graph_timed) {
        jg_timings& tm = w->timings;
        tm = jg_timings{};
        cudaEventElapsedTime(&tm.total, w->ev[0], w->ev[7]);
    }
    if (c.status != 0) {
        g_err = "device status " + std::to_string(c.status);
        return c.status;
    }
    return JG_OK;
}

}  // namespace

extern "C" {

const char* jg_last_error(void) { return g_err.c_str(); }
const char* jg_version(void) { return "jitter-gb300 0.1 (sm_103a)"; }

int jg_default_params(jg_world_params* p) {
    if (!p) return JG_ERR_INVALID_ARG;
    memset(p, 0, sizeof(*p));
    p->gravity[0] = 0; p->gravity[1] = -9.81f; p->gravity[2] = 0;
    p->substeps = 1;
    p->solver_iterations = 6;
    p->relax_iterations = 4;
    p->enable_auxiliary_contacts = 1;
    p->persistent_manifold = 1;
    p->speculative_relaxation = 0.9f;
    p->speculative_threshold = 10.0f;
    p->allow_deactivation = 1;
    p->edge_filter = 1;
    p->warm_start_mode = JG_WARMSTART_CACHED;
    p->narrow_tile = 32;
    p->partitioned_solve = 1;
    return JG_OK;
}

int jg_create(const jg_world_params* params, jg_world** out) {
    if (!params || !out) return JG_ERR_INVALID_ARG;
    *out = nullptr;
    if (params->substeps < 1 || params->solver_iterations < 1 || params->relax_iterations < 0) return JG_ERR_INVALID_ARG;
    if (params->solver_iterations > 4096) return JG_ERR_INVALID_ARG;
    if (!cells_per_sm_ok(params->sched_cells_per_sm)) return JG_ERR_INVALID_ARG;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) { g_err = "no CUDA device"; return JG_ERR_NOT_SUPPORTED; }
    jg_world* w = new jg_world();
    w->prm = *params;
    cudaGetDevice(&w->device);
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, w->device);
    if (prop.major < 10) { delete w; g_err = "needs an sm_103a (Blackwell) device"; return JG_ERR_NOT_SUPPORTED; }
    w->nsm = prop.multiProcessorCount;
    if (jg_narrowphase_init() != 0 || jg_solver_init() != 0 || jg_schedule_init() != 0) {
        delete w;
        g_err = "shared memory attribute refused";
        return JG_ERR_CUDA;
    }
    if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess) { delete w; return JG_ERR_CUDA; }
    for (int i = 0; i < 9; i++) cudaEventCreate(&w->ev[i]);
    int r = allocate(w);
    if (r) { jg_destroy(w); return r; }
    w->d.nworlds = 1;
    cudaStreamSynchronize(w->stream);
    *out = w;
    return JG_OK;
}

// The World property setters (World.cs:346-403, World.Detect.cs:88-122): solver
// iterations at least one, relaxation iterations not negative, substeps at least one, a
// finite gravity; the pool capacities are fixed at creation.
int jg_set_params(jg_world* w, const jg_world_params* p) {
    if (!w || !p) return JG_ERR_INVALID_ARG;
    if (p->substeps < 1 || p->solver_iterations < 1 || p->solver_iterations > 4096 || p->relax_iterations < 0 ||
        !cells_per_sm_ok(p->sched_cells_per_sm) || !std::isfinite(p->gravity[0]) || !std::isfinite(p->gravity[1]) || !std::isfinite(p->gravity[2])) {
        g_err = "jg_set_params: invalid solver settings";
        return JG_ERR_INVALID_ARG;
    }
    const jg_world_params& c = w->prm;
    if (p->max_bodies != c.max_bodies || p->max_shapes != c.max_shapes || p->max_pairs != c.max_pairs ||
        p->max_arbiters != c.max_arbiters || p->max_constraints != c.max_constraints) {
        g_err = "jg_set_params: pool capacities are fixed when the world is created";
        return JG_ERR_INVALID_ARG;
    }
    w->prm = *p;
    invalidate_graphs(w);
    return JG_OK;
}

int jg_get_params(jg_world* w, jg_world_params* out) {
    if (!w || !out) return JG_ERR_INVALID_ARG;
    *out = w->prm;
    return JG_OK;
}

int jg_batch_create(const jg_world_params* params, int32_t n_worlds, jg_world** out) {
    if (n_worlds < 1) return JG_ERR_INVALID_ARG;
    int r = jg_create(params, out);
    if (r) return r;
    (*out)->nworlds = n_worlds;
    (*out)->d.nworlds = n_worlds;
    return JG_OK;
}

int jg_destroy(jg_world* w) {
    if (!w) return JG_ERR_INVALID_ARG;
    for (int i = 0; i < 2; i++) if (w->graph[i]) cudaGraphExecDestroy(w->graph[i]);
    if (w->stream) cudaStreamSynchronize(w->stream);
    for (void* p : w->allocs) cudaFree(p);
    cudaFree(w->q_pairs); cudaFree(w->q_out); cudaFree(w->q_hit);
    jg_mlp_free(w->mlp);
    if (w->h_ctr) cudaFreeHost(w->h_ctr);
    if (w->h_bad) cudaFreeHost(w->h_bad);
    for (int i = 0; i < 9; i++) if (w->ev[i]) cudaEventDestroy(w->ev[i]);
    if (w->stream) cudaStreamDestroy(w->stream);
    delete w;
    return JG_OK;
}

static void invalidate_graphs(jg_world* w) {
    for (int i = 0; i < 2; i++) {
        if (w->graph[i]) cudaGraphExecDestroy(w->graph[i]);
        w->graph[i] = nullptr;
        w->graph_dt[i] = -1.f;
    }
}

}  // extern "C"

namespace {

// Body descriptors in and out through the device: one copy of the caller's array each
// way, validation, conversion to the solver layout and the write-back of the state a step
// changes run as kernels.  Reasons recorded in d_bad: 1 non-finite, 2 invalid argument;
// the body with the smallest index wins, as a sequential check would report it.
__global__ void k_bodies_check(const jg_body_desc* d, int n, int nworlds, int* bad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const jg_body_desc& b = d[i];
        int why = 0;
        if (!finite3(b.position) || !finite3(b.velocity) || !finite3(b.angular_velocity) ||
            !isfinite(b.orientation[3]) || !finite3(b.orientation) || !isfinite(b.inv_mass))
            why = 1;
        else if (b.motion_type < 0 || b.motion_type > 2 || b.world < 0 || b.world >= nworlds)
            why = 2;
        if (why) atomicMin(bad, i * 4 + why);
    }
}

// keep: the upload refreshes the same bodies (the host-buffer step), so each body keeps its
// sleep time and island flags; otherwise they start afresh (sleep time 0, infinite for a
// static body, island marked and in the active list).
__global__ void k_bodies_in(const jg_body_desc* d, int n, WorldDev D, const int* bad, int keep) {
    if (*bad != INT_MAX) return;  // an invalid body: the state stays as it was
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const jg_body_desc& b = d[i];
        float i0[4], i1[2], imv[3];
        body_world_inertia(b, i0, i1, imv);
        int fl = 0;
        if (b.motion_type == JG_MOTION_DYNAMIC) fl |= SB_DYNAMIC;
        if (b.motion_type == JG_MOTION_DYNAMIC && ((b.flags >> 4) & 7)) fl |= SB_LINLOCK;
        SBody sb;
        sb.v = make_float4(b.velocity[0], b.velocity[1], b.velocity[2], imv[0]);
        sb.w = make_float4(b.angular_velocity[0], b.angular_velocity[1], b.angular_velocity[2], imv[1]);
        sb.i0 = make_float4(i0[0], i0[1], i0[2], i0[3]);
        sb.i1 = make_float4(i1[0], i1[1], imv[2], __int_as_float(fl));
        D.body[i] = sb;
        D.pos[i] = make_float4(b.position[0], b.position[1], b.position[2], 0.f);
        D.q[i] = make_float4(b.orientation[0], b.orientation[1], b.orientation[2], b.orientation[3]);
        D.dv[i] = make_float4(b.delta_velocity[0], b.delta_velocity[1], b.delta_velocity[2], 0.f);
        D.dw[i] = make_float4(b.delta_angular_velocity[0], b.delta_angular_velocity[1], b.delta_angular_velocity[2], 0.f);
        D.il0[i] = make_float4(b.inv_inertia[0], b.inv_inertia[1], b.inv_inertia[2], b.inv_inertia[3]);
        D.il1[i] = make_float4(b.inv_inertia[4], b.inv_inertia[5], b.inv_mass, 0.f);
        D.force[i] = make_float4(b.force[0], b.force[1], b.force[2], 0.f);
        D.torque[i] = make_float4(b.torque[0], b.torque[1], b.torque[2], 0.f);
        D.mat[i] = make_float4(b.friction, b.restitution, b.linear_damping, b.angular_damping);
        int island = 3;
        if (keep) island = D.binfo[i].w;
        else D.sleep[i].x = b.motion_type == JG_MOTION_STATIC ? INFINITY : 0.f;
        D.binfo[i] = make_int4(b.motion_type, b.flags, b.world, island);
    }
}

// The state a step changes, written over the stored descriptors (forces are cleared after
// each step, RigidBody.cs:760).
__global__ void k_bodies_out(jg_body_desc* d, int n, WorldDev D) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        jg_body_desc& o = d[i];
        const float4 p = D.pos[i], q = D.q[i], v = D.body[i].v, av = D.body[i].w, dv = D.dv[i], dw = D.dw[i];
        o.position[0] = p.x; o.position[1] = p.y; o.position[2] = p.z;
        o.orientation[0] = q.x; o.orientation[1] = q.y; o.orientation[2] = q.z; o.orientation[3] = q.w;
        o.velocity[0] = v.x; o.velocity[1] = v.y; o.velocity[2] = v.z;
        o.angular_velocity[0] = av.x; o.angular_velocity[1] = av.y; o.angular_velocity[2] = av.z;
        o.delta_velocity[0] = dv.x; o.delta_velocity[1] = dv.y; o.delta_velocity[2] = dv.z;
        o.delta_angular_velocity[0] = dw.x; o.delta_angular_velocity[1] = dw.y; o.delta_angular_velocity[2] = dw.z;
        o.force[0] = o.force[1] = o.force[2] = 0.f;
        o.torque[0] = o.torque[1] = o.torque[2] = 0.f;
        o.flags = D.binfo[i].y;  // RigidBody.IsActive may have changed (sleeping)
    }
}

int upload_bodies_device(jg_world* w, const jg_body_desc* b, int32_t n) {
    WorldDev& D = w->d;
    cudaStream_t s = w->stream;
    const int blocks = std::max(1, std::min((n + 255) / 256, w->nsm * 8));
    const int none = INT_MAX;
    CK(cudaMemcpyAsync(w->d_bad, &none, sizeof(int), cudaMemcpyHostToDevice, s));
    if (n > 0) {
        CK(cudaMemcpyAsync(w->d_stage, b, sizeof(jg_body_desc) * n, cudaMemcpyHostToDevice, s));
        k_bodies_check<<<blocks, 256, 0, s>>>(w->d_stage, n, w->nworlds, w->d_bad);
        k_bodies_in<<<blocks, 256, 0, s>>>(w->d_stage, n, D, w->d_bad, D.nb == n ? 1 : 0);
    }
    CK(cudaMemcpyAsync(w->h_bad, w->d_bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (*w->h_bad != INT_MAX) return (*w->h_bad & 3) == 1 ? JG_ERR_NONFINITE : JG_ERR_INVALID_ARG;
    std::swap(w->d_desc, w->d_stage);  // the accepted descriptors
    if (D.nb != n) invalidate_graphs(w);
    D.nb = n;
    return JG_OK;
}

int download_bodies_device(jg_world* w, jg_body_desc* b, int32_t n) {
    cudaStream_t s = w->stream;
    if (n > 0) {
        k_bodies_out<<<std::max(1, std::min((n + 255) / 256, w->nsm * 8)), 256, 0, s>>>(w->d_desc, n, w->d);
        CK(cudaMemcpyAsync(b, w->d_desc, sizeof(jg_body_desc) * n, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
    return JG_OK;
}

}  // namespace

extern "C" {

int jg_upload_bodies(jg_world* w, const jg_body_desc* b, int32_t n) {
    if (!w || (!b && n > 0) || n < 0) return JG_ERR_INVALID_ARG;
    if (n > w->d.cap_bodies) return JG_ERR_CAPACITY;
    int r = upload_bodies_device(w, b, n);
    if (r) return r;
    w->host_bodies.assign(b, b + n);
    w->host_current = true;
    return JG_OK;
}

int jg_download_bodies(jg_world* w, jg_body_desc* b, int32_t n) {
    if (!w || (!b && n > 0) || n < 0 || n > w->d.nb) return JG_ERR_INVALID_ARG;
    return download_bodies_device(w, b, n);
}

int jg_upload_shapes(jg_world* w, const jg_shape_desc* sh, int32_t n, const float* hull, int32_t nh,
                     const jg_triangle_desc* tris, int32_t nt) {
    if (!w || n < 0 || nh < 0 || nt < 0 || (n > 0 && !sh)) return JG_ERR_INVALID_ARG;
    if (n > w->d.cap_shapes) return JG_ERR_CAPACITY;
    std::vector<int4> info(n);
    std::vector<float4> dims(n), cen(n);
    for (int i = 0; i < n; i++) {
        const jg_shape_desc& s = sh[i];
        if (s.kind < 0 || s.kind > JG_SHAPE_TRIANGLE) { g_err = "invalid shape kind"; return JG_ERR_INVALID_SHAPE; }
        if (s.body < 0 || s.body >= w->d.nb) return JG_ERR_INVALID_ARG;
        if (s.kind == JG_SHAPE_POINTCLOUD) {
            if (s.data_offset < 0 || s.data_count < 1 || s.data_offset + s.data_count > nh) return JG_ERR_INVALID_ARG;
        }
        if (s.kind == JG_SHAPE_TRIANGLE && (s.data_offset < 0 || s.data_offset >= nt)) return JG_ERR_INVALID_ARG;
        info[i] = make_int4(s.kind, s.body, s.data_offset, s.data_count);
        dims[i] = make_float4(s.dims[0], s.dims[1], s.dims[2], s.dims[3]);
        cen[i] = make_float4(s.center[0], s.center[1], s.center[2], 0.f);
    }
    int r;
    if ((r = ensure_hull(w, nh))) return r;
    if ((r = ensure_tris(w, nt))) return r;
    std::vector<float4> hv(nh);
    for (int i = 0; i < nh; i++) hv[i] = make_float4(hull[3 * i], hull[3 * i + 1], hull[3 * i + 2], 0.f);
    std::vector<TriDev> td(nt);
    for (int i = 0; i < nt; i++) {
        const jg_triangle_desc& t = tris[i];
        td[i].a = make_float4(t.a[0], t.a[1], t.a[2], 0.f);
        td[i].b = make_float4(t.b[0], t.b[1], t.b[2], 0.f);
        td[i].c = make_float4(t.c[0], t.c[1], t.c[2], 0.f);
        td[i].n = make_float4(t.normal[0], t.normal[1], t.normal[2], 0.f);
        for (int k = 0; k < 3; k++) {
            int nb = t.neighbor[k];
            if (nb >= 0 && nb < nt) td[i].nb[k] = make_float4(tris[nb].normal[0], tris[nb].normal[1], tris[nb].normal[2], 1.f);
            else td[i].nb[k] = make_float4(0, 0, 0, 0.f);
        }
    }
    WorldDev& D = w->d;
    cudaStream_t s = w->stream;
    CK(cudaMemcpyAsync(D.sinfo, info.data(), sizeof(int4) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(D.sdims, dims.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(D.scenter, cen.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s));
    if (nh) CK(cudaMemcpyAsync(D.hull, hv.data(), sizeof(float4) * nh, cudaMemcpyHostToDevice, s));
    if (nt) CK(cudaMemcpyAsync(D.tris, td.data(), sizeof(TriDev) * nt, cudaMemcpyHostToDevice, s));
    // new shape ids: the contact cache starts empty
    int zero = 0;
    CK(cudaMemcpyAsync(&D.ctr->narb, &zero, sizeof(int), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    D.ns = n; D.nhull = nh; D.ntris = nt;
    w->host_shapes.assign(sh, sh + n);
    invalidate_graphs(w);
    return JG_OK;
}

int jg_set_body(jg_world* w, int32_t body, int32_t field, const float* v) {
    if (!w || !v || body < 0 || body >= w->d.nb || field < 0 || field > 5) return JG_ERR_INVALID_ARG;
    jg_body_desc d;
    int r = jg_download_bodies(w, w->host_bodies.data(), w->d.nb);
    if (r) return r;
    d = w->host_bodies[body];
    switch (field) {
        case 0: memcpy(d.position, v, 12); break;
        case 1: memcpy(d.orientation, v, 16); break;
        case 2: memcpy(d.velocity, v, 12); break;
        case 3: memcpy(d.angular_velocity, v, 12); break;
        case 4: memcpy(d.force, v, 12); break;
        case 5: memcpy(d.torque, v, 12); break;
    }
    w->host_bodies[body] = d;
    std::vector<jg_body_desc> all = w->host_bodies;
    r = jg_upload_bodies(w, all.data(), (int)all.size());
    if (r) return r;
    if (field <= 1) {
        // RigidBody.Move (RigidBody.cs:637-648): clear the contact cache of the body
        std::vector<int2> bodies(w->d.ctr ? 0 : 0);
        WorldDev& D = w->d;
        int narb = 0;
        CK(cudaMemcpy(&narb, &D.ctr->narb, sizeof(int), cudaMemcpyDeviceToHost));
        if (narb > 0) {
            std::vector<int2> bb(narb);
            std::vector<int4> info(narb);
            const ArbStore& A = D.arb[D.cur];
            CK(cudaMemcpy(bb.data(), A.body, sizeof(int2) * narb, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(info.data(), A.info, sizeof(int4) * narb, cudaMemcpyDeviceToHost));
            for (int a = 0; a < narb; a++) if (bb[a].x == body || bb[a].y == body) info[a].x = 0;
            CK(cudaMemcpy(A.info, info.data(), sizeof(int4) * narb, cudaMemcpyHostToDevice));
        }
    }
    return JG_OK;
}

// JQuaternion.CreateFromToRotation (JQuaternion.cs:84-101)
static q4 from_to_rotation(v3 from, v3 to) {
    float d = dot(from, to);
    if (d < -1.0f + 1e-6f) {
        v3 ax = create_orthonormal(from);
        return q4{ax.x, ax.y, ax.z, 0.f};
    }
    float s = sqrtf((1.0f + d) * 2.0f);
    float is = 1.0f / s;
    v3 c = cross(from, to) * is;
    return q4{c.x, c.y, c.z, s * 0.5f};
}

// The servos' argument checks: ArgumentCheck.UnitQuaternion (ArgumentCheck.cs:157-167, squared
// length within 1e-3 of 1), NonZero and Finite vectors, a twist target in [-pi, pi]
// (TwistServo.cs:73), ServoMath.CheckMaximum (ServoMath.cs:15-20: not NaN, >= 0, +inf allowed).
static bool servo_maximum_ok(float m) { return !std::isnan(m) && m >= 0.f; }
static int check_servo_init(int kind, const float* init) {
    const float PI = 3.14159265358979323846f;
    auto finite = [&](int a, int n) { for (int i = a; i < a + n; i++) if (!std::isfinite(init[i])) return false; return true; };
    auto nonzero = [&](int a) { return finite(a, 3) && len2(mk3(init[a], init[a + 1], init[a + 2])) != 0.f; };
    switch (kind) {
        case JG_CONSTRAINT_ANGULARSERVO: {
            const bool keep = init[0] == 0.f && init[1] == 0.f && init[2] == 0.f && init[3] == 0.f;
            if (!keep) {
                if (!finite(0, 4)) return JG_ERR_INVALID_ARG;
                float l2 = init[0] * init[0] + init[1] * init[1] + init[2] * init[2] + init[3] * init[3];
                if (std::fabs(l2 - 1.0f) > 1e-3f) return JG_ERR_INVALID_ARG;
            }
            return servo_maximum_ok(init[4]) ? JG_OK : JG_ERR_INVALID_ARG;
        }
        case JG_CONSTRAINT_LINEARSERVO:
            return finite(0, 9) && servo_maximum_ok(init[9]) ? JG_OK : JG_ERR_INVALID_ARG;
        case JG_CONSTRAINT_LINEARAXISSERVO:
            return nonzero(0) && finite(3, 7) && servo_maximum_ok(init[10]) ? JG_OK : JG_ERR_INVALID_ARG;
        case JG_CONSTRAINT_TWISTSERVO:
            return nonzero(0) && nonzero(3) && std::isfinite(init[6]) && init[6] >= -PI && init[6] <= PI &&
                           servo_maximum_ok(init[7])
                       ? JG_OK
                       : JG_ERR_INVALID_ARG;
    }
    return JG_ERR_INVALID_ARG;
}

int jg_add_constraint(jg_world* w, int32_t kind, int32_t b1, int32_t b2, const float* init, int32_t* out_id) {
    if (!w || !init) return JG_ERR_INVALID_ARG;
    if (kind < JG_CONSTRAINT_BALLSOCKET || kind > JG_CONSTRAINT_ELLIPTICALCONELIMIT) return JG_ERR_INVALID_ARG;
    v3 ell_ref = mk3(0.f);
    if (kind == JG_CONSTRAINT_ELLIPTICALCONELIMIT) {
        // EllipticalConeLimit.Initialize (EllipticalConeLimit.cs:92-113) and ValidateLimits
        // (:178-200): finite non-zero directions, 0 <= min <= max < pi with max > 0 for both
        // swings, the inner semiaxes both zero or both positive, and a reference direction
        // that is not along body 1's axis
        for (int i = 0; i < 9; i++) if (!std::isfinite(init[i])) return JG_ERR_INVALID_ARG;
        for (int a = 0; a < 9; a += 3) if (len2(mk3(init[a], init[a + 1], init[a + 2])) == 0.f) return JG_ERR_INVALID_ARG;
        const float PI = 3.14159265358979323846f;
        for (int a = 9; a < 13; a += 2) {
            const float lo = init[a], hi = init[a + 1];
            if (!std::isfinite(lo) || !std::isfinite(hi) || lo < 0.f || hi <= 0.f || hi >= PI || lo > hi)
                return JG_ERR_INVALID_ARG;
        }
        if ((init[9] == 0.f) != (init[11] == 0.f)) return JG_ERR_INVALID_ARG;
        v3 ax1 = normalize(mk3(init[0], init[1], init[2]));
        v3 r = normalize(mk3(init[6], init[7], init[8]));
        r = r - ax1 * dot(ax1, r);
        if (len2(r) < 1e-12f) return JG_ERR_INVALID_ARG;
        ell_ref = normalize(r);
    }
    if (kind >= JG_CONSTRAINT_ANGULARSERVO && kind <= JG_CONSTRAINT_TWISTSERVO) {
        int r = check_servo_init(kind, init);
        if (r) return r;
    } else if (kind == JG_CONSTRAINT_POINTONPLANE || kind == JG_CONSTRAINT_POINTONLINE) {
        // PointOnPlane.Initialize (PointOnPlane.cs:89-100), PointOnLine.Initialize
        // (PointOnLine.cs:92-100): a non-zero finite axis, finite anchors, limits that are not NaN
        for (int i = 0; i < 9; i++) if (!std::isfinite(init[i])) return JG_ERR_INVALID_ARG;
        if (len2(mk3(init[0], init[1], init[2])) == 0.f || std::isnan(init[9]) || std::isnan(init[10])) return JG_ERR_INVALID_ARG;
    } else if (kind == JG_CONSTRAINT_ANGULARMOTOR || kind == JG_CONSTRAINT_LINEARMOTOR) {
        // AngularMotor.Initialize (AngularMotor.cs:62-82), LinearMotor.Initialize
        // (LinearMotor.cs:97-115): non-zero finite axes; MaximumTorque / MaximumForce >= 0
        for (int i = 0; i < 6; i++) if (!std::isfinite(init[i])) return JG_ERR_INVALID_ARG;
        if (len2(mk3(init[0], init[1], init[2])) == 0.f || len2(mk3(init[3], init[4], init[5])) == 0.f) return JG_ERR_INVALID_ARG;
        if (!std::isfinite(init[6]) || !(init[7] >= 0.f)) return JG_ERR_INVALID_ARG;
    } else if (kind >= JG_CONSTRAINT_DISTANCELIMIT && kind <= JG_CONSTRAINT_TWISTANGLE) {
        // the reference's argument checks (DistanceLimit.cs:99-103, ConeLimit.cs:96-99 and
        // :228-238, TwistAngle.cs:88-92)
        for (int i = 0; i < 6; i++) if (!std::isfinite(init[i])) return JG_ERR_INVALID_ARG;
        float lo = init[6], hi = init[7];
        if (kind == JG_CONSTRAINT_DISTANCELIMIT) {
            if (std::isnan(lo) || std::isnan(hi)) return JG_ERR_INVALID_ARG;
        } else {
            if (len2(mk3(init[0], init[1], init[2])) == 0.f || len2(mk3(init[3], init[4], init[5])) == 0.f)
                return JG_ERR_INVALID_ARG;
            if (!std::isfinite(lo) || !std::isfinite(hi)) return JG_ERR_INVALID_ARG;
            const float PI = 3.14159265358979323846f;
            if (kind == JG_CONSTRAINT_CONELIMIT &&
                (!(lo >= 0.f && lo <= PI) || !(hi >= lo && hi <= PI) || (lo == hi && (lo == 0.f || lo == PI))))
                return JG_ERR_INVALID_ARG;
        }
    }
    if (b1 < 0 || b2 < 0 || b1 >= w->d.nb || b2 >= w->d.nb || b1 == b2) return JG_ERR_INVALID_ARG;
    if (w->nj_host >= w->d.cap_joints) return JG_ERR_CAPACITY;
    // the two bodies' current poses: from the host copy while it is current, else from the device
    float4 pq[4];
    if (w->host_current) {
        const jg_body_desc& d1 = w->host_bodies[b1];
        const jg_body_desc& d2 = w->host_bodies[b2];
        pq[0] = make_float4(d1.position[0], d1.position[1], d1.position[2], 0.f);
        pq[1] = make_float4(d1.orientation[0], d1.orientation[1], d1.orientation[2], d1.orientation[3]);
        pq[2] = make_float4(d2.position[0], d2.position[1], d2.position[2], 0.f);
        pq[3] = make_float4(d2.orientation[0], d2.orientation[1], d2.orientation[2], d2.orientation[3]);
    } else {
        CK(cudaMemcpy(&pq[0], w->d.pos + b1, sizeof(float4), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(&pq[1], w->d.q + b1, sizeof(float4), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(&pq[2], w->d.pos + b2, sizeof(float4), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(&pq[3], w->d.q + b2, sizeof(float4), cudaMemcpyDeviceToHost));
    }
    JointDev J;
    memset(&J, 0, sizeof(J));
    J.hdr = make_int4(kind, b1, b2, 0);
    q4 q1{pq[1].x, pq[1].y, pq[1].z, pq[1].w};
    q4 q2{pq[3].x, pq[3].y, pq[3].z, pq[3].w};
    v3 p1 = mk3(pq[0]);
    v3 p2 = mk3(pq[2]);
    if (kind == JG_CONSTRAINT_BALLSOCKET) {
        // BallSocket.Initialize (BallSocket.cs:120-138)
        v3 anchor = mk3(init[0], init[1], init[2]);
        J.la1 = f4(rotate_inv(anchor - p1, q1), 0.f);
        J.la2 = f4(rotate_inv(anchor - p2, q2), 0.f);
        J.prm = make_float4(0.2f, 0.00001f, 0.f, 0.f);
    } else if (kind == JG_CONSTRAINT_DISTANCELIMIT) {
        // DistanceLimit.Initialize (DistanceLimit.cs:92-117)
        v3 a1 = mk3(init[0], init[1], init[2]), a2 = mk3(init[3], init[4], init[5]);
        J.la1 = f4(rotate_inv(a1 - p1, q1), 0.f);
        J.la2 = f4(rotate_inv(a2 - p2, q2), 0.f);
        J.prm = make_float4(0.2f, 0.00001f, 0.f, 0.f);
        J.lim = make_float4(init[6], init[7], sqrtf(len2(a2 - a1)), 0.f);
    } else if (kind == JG_CONSTRAINT_CONELIMIT) {
        // ConeLimit.Initialize (ConeLimit.cs:92-118)
        J.la1 = f4(rotate_inv(normalize(mk3(init[0], init[1], init[2])), q1), 0.f);
        J.la2 = f4(rotate_inv(normalize(mk3(init[3], init[4], init[5])), q2), 0.f);
        J.prm = make_float4(0.2f, 0.001f, 0.f, 0.f);
        J.lim = make_float4(init[6], init[7], 0.f, 0.f);
    } else if (kind == JG_CONSTRAINT_FIXEDANGLE) {
        // FixedAngle.Initialize (FixedAngle.cs:72-85): Q0 is the current relative rotation
        J.prm = make_float4(0.2f, 0.001f, 0.f, 0.f);
        J.q0 = f4(qmul(qconj(q2), q1));
    } else if (kind == JG_CONSTRAINT_POINTONPLANE) {
        // PointOnPlane.Initialize (PointOnPlane.cs:100-126)
        v3 axis = normalize(mk3(init[0], init[1], init[2]));
        J.la1 = f4(rotate_inv(mk3(init[3], init[4], init[5]) - p1, q1), 0.f);
        J.la2 = f4(rotate_inv(mk3(init[6], init[7], init[8]) - p2, q2), 0.f);
        J.axis = f4(rotate_inv(axis, q1), 0.f);
        J.prm = make_float4(0.2f, 0.00001f, 0.f, 0.f);
        J.lim = make_float4(init[9], init[10], 0.f, 0.f);
    } else if (kind == JG_CONSTRAINT_ANGULARMOTOR || kind == JG_CONSTRAINT_LINEARMOTOR) {
        // AngularMotor / LinearMotor Initialize with TargetVelocity and MaximumTorque (Force)
        J.la1 = f4(rotate_inv(normalize(mk3(init[0], init[1], init[2])), q1), 0.f);
        J.la2 = f4(rotate_inv(normalize(mk3(init[3], init[4], init[5])), q2), 0.f);
        J.lim = make_float4(0.f, init[7], init[6], 0.f);
    } else if (kind == JG_CONSTRAINT_ELLIPTICALCONELIMIT) {
        // EllipticalConeLimit.Initialize (EllipticalConeLimit.cs:92-126)
        J.la1 = f4(rotate_inv(normalize(mk3(init[0], init[1], init[2])), q1), 0.f);
        J.la2 = f4(rotate_inv(normalize(mk3(init[3], init[4], init[5])), q2), 0.f);
        J.axis = f4(rotate_inv(ell_ref, q1), 0.f);
        J.prm = make_float4(0.2f, 0.001f, 0.f, 0.f);
        J.lim = make_float4(init[9], init[10], init[11], init[12]);
    } else if (kind == JG_CONSTRAINT_POINTONLINE) {
        // PointOnLine.Initialize (PointOnLine.cs:92-121)
        v3 axis = normalize(mk3(init[0], init[1], init[2]));
        J.la1 = f4(rotate_inv(mk3(init[3], init[4], init[5]) - p1, q1), 0.f);
        J.la2 = f4(rotate_inv(mk3(init[6], init[7], init[8]) - p2, q2), 0.f);
        J.axis = f4(rotate_inv(axis, q1), 0.f);
        J.prm = make_float4(0.2f, 0.00001f, 0.2f, 0.0001f);
        J.lim = make_float4(init[9], init[10], 0.f, 0.f);
    } else if (kind == JG_CONSTRAINT_ANGULARSERVO) {
        // AngularServo.Initialize (AngularServo.cs:55-77): the given target relative
        // orientation, or the current one (conj(q1) q2) when all four are zero
        q4 t{init[0], init[1], init[2], init[3]};
        if (init[0] == 0.f && init[1] == 0.f && init[2] == 0.f && init[3] == 0.f) t = qmul(qconj(q1), q2);
        J.q0 = f4(t);
        J.prm = make_float4(0.2f, 0.001f, 0.f, 0.f);
        J.lim = make_float4(0.f, init[4], 0.f, 0.f);
    } else if (kind == JG_CONSTRAINT_LINEARSERVO) {
        // LinearServo.Initialize (LinearServo.cs:60-73) with TargetPosition and MaximumForce
        J.la1 = f4(rotate_inv(mk3(init[0], init[1], init[2]) - p1, q1), 0.f);
        J.la2 = f4(rotate_inv(mk3(init[3], init[4], init[5]) - p2, q2), 0.f);
        J.axis = make_float4(init[6], init[7], init[8], 0.f);
        J.prm = make_float4(0.2f, 0.00001f, 0.f, 0.f);
        J.lim = make_float4(0.f, init[9], 0.f, 0.f);
    } else if (kind == JG_CONSTRAINT_LINEARAXISSERVO) {
        // LinearAxisServo.Initialize (LinearAxisServo.cs:61-78) with MaximumForce
        J.axis = f4(rotate_inv(normalize(mk3(init[0], init[1], init[2])), q1), 0.f);
        J.la1 = f4(rotate_inv(mk3(init[3], init[4], init[5]) - p1, q1), 0.f);
        J.la2 = f4(rotate_inv(mk3(init[6], init[7], init[8]) - p2, q2), 0.f);
        J.prm = make_float4(0.2f, 0.00001f, 0.f, 0.f);
        J.lim = make_float4(0.f, init[10], init[9], 0.f);
    } else if (kind == JG_CONSTRAINT_TWISTSERVO) {
        // TwistServo.Initialize (TwistServo.cs:69-87) with MaximumTorque: body 2's axis, and the
        // reference rotation that turns body 1's axis (expressed in body 2's frame) onto it
        v3 ax1 = normalize(mk3(init[0], init[1], init[2])), ax2 = normalize(mk3(init[3], init[4], init[5]));
        v3 B = rotate_inv(ax2, q2);
        J.axis = f4(B, 0.f);
        J.q0 = f4(qmul(from_to_rotation(rotate_inv(ax1, q2), B), qmul(qconj(q2), q1)));
        J.prm = make_float4(0.2f, 0.001f, 0.f, 0.f);
        J.lim = make_float4(0.f, init[7], init[6], 0.f);
    } else if (kind == JG_CONSTRAINT_TWISTANGLE) {
        // TwistAngle.Initialize (TwistAngle.cs:85-128): Q0 is the initial relative rotation
        // turned so that body 1's axis lies on body 2's
        v3 ax1 = normalize(mk3(init[0], init[1], init[2])), ax2 = normalize(mk3(init[3], init[4], init[5]));
        J.prm = make_float4(0.2f, 0.001f, 0.f, 0.f);
        J.lim = make_float4(init[6], init[7], 0.5f * init[6] + 0.5f * init[7], 0.f);
        v3 u1 = rotate_inv(ax1, q1);
        v3 B = rotate_inv(ax2, q2);
        q4 rel = qmul(qconj(q2), q1);
        J.axis = f4(B, 0.f);
        J.q0 = f4(qmul(from_to_rotation(rotate(u1, rel), B), rel));
    } else {
        // HingeAngle.Initialize (HingeAngle.cs:84-110)
        v3 axis = normalize(mk3(init[0], init[1], init[2]));
        float from = init[3], to = init[4];
        J.prm = make_float4(0.2f, 0.001f, 0.1f, 0.001f);
        J.lim = make_float4(from / 2.0f, to / 2.0f, 0.25f * from + 0.25f * to, 0.f);
        J.axis = f4(rotate_inv(axis, q2), 0.f);
        J.q0 = f4(qmul(qconj(q2), q1));
    }
    w->pending_joints.push_back(J);
    if (out_id) *out_id = w->nj_host;
    w->nj_host++;
    w->d.nj = w->nj_host;
    invalidate_graphs(w);
    return JG_OK;
}

// Uploads the constraints added since the last flush in one copy.
static int flush_joints(jg_world* w) {
    if (w->pending_joints.empty()) return JG_OK;
    size_t k = w->pending_joints.size();
    CK(cudaMemcpy(w->d.joints + (w->nj_host - k), w->pending_joints.data(), sizeof(JointDev) * k, cudaMemcpyHostToDevice));
    w->pending_joints.clear();
    return JG_OK;
}

// One step as a stream of launches (stage times recorded) or, with `graph`, as the replay of
// the step captured for the current arbiter-buffer parity (recaptured when dt or the world's
// shape changes), timed as a whole.
static int step_impl(jg_world* w, float dt, bool graph) {
    if (!w) return JG_ERR_INVALID_ARG;
    if (!std::isfinite(dt)) return JG_ERR_NONFINITE;
    if (dt < 0) return JG_ERR_INVALID_ARG;
    if (dt < 1.401298e-45f) return JG_OK;
    int fr = flush_joints(w);
    if (fr) return fr;
    w->host_current = false;
    StepParams sp = make_params(w, dt);
    if (w->d.ns == 0 && w->d.nb == 0) return JG_OK;
    int parity = w->d.cur;
    if (graph) {
        if (!w->graph[parity] || w->graph_dt[parity] != dt) {
            if (w->graph[parity]) { cudaGraphExecDestroy(w->graph[parity]); w->graph[parity] = nullptr; }
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeThreadLocal));
            int r = launch_step(w, sp, false);
            cudaError_t e = cudaStreamEndCapture(w->stream, &g);
            if (r) return r;
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
            CK(cudaGraphInstantiate(&w->graph[parity], g, 0));
            cudaGraphDestroy(g);
            w->graph_dt[parity] = dt;
        } else {
            jg_flip_store(w->d);
        }
        CK(cudaEventRecord(w->ev[0], w->stream));
        CK(cudaGraphLaunch(w->graph[parity], w->stream));
        CK(cudaEventRecord(w->ev[7], w->stream));
        return finish_step(w, false, true);
    }
    int r = launch_step(w, sp, true);
    if (r) return r;
    return finish_step(w, true);
}

int jg_step(jg_world* w, float dt) { return step_impl(w, dt, w && w->prm.use_graph != 0); }

// Batched worlds always step as one graph launch: every world of the batch in the captured
// sequence, the solve one persistent cooperative kernel over all worlds (one task each).
int jg_batch_step(jg_world* w, float dt) { return step_impl(w, dt, true); }

// World.Stabilize (World.Step.cs:318-392): the island check, then per substep the prepare,
// solver_iterations iterations and relaxation_iterations relaxation passes over the present
// contacts and constraints, with no detection and no integration of forces or velocities.
int jg_stabilize(jg_world* w, float dt, int32_t iterations, int32_t relax) {
    if (!w) return JG_ERR_INVALID_ARG;
    if (!std::isfinite(dt)) return JG_ERR_NONFINITE;
    if (dt < 0 || iterations < 1 || iterations > 4096 || relax < 0) return JG_ERR_INVALID_ARG;
    if (dt < 1.401298e-45f) return JG_OK;
    int fr = flush_joints(w);
    if (fr) return fr;
    w->host_current = false;
    StepParams sp = make_params(w, dt);
    sp.iterations = iterations;
    sp.relax = relax;
    sp.stabilize = 1;
    sp.record_residual = 0;
    WorldDev& d = w->d;
    cudaStream_t s = w->stream;
    d.allow_deact = sp.allow_deact;
    k_reset_counters<<<1, 1, 0, s>>>(d.ctr);
    if (sp.allow_deact) jg_launch_islands(d, s, w->nsm);
    jg_launch_schedule(d, sp, s, w->nsm);
    if (jg_launch_color(d, s, w->nsm) < 0) { g_err = "cooperative launch of the colouring failed"; return JG_ERR_CUDA; }
    jg_flip_store(d);
    jg_launch_count_contacts(d, s, w->nsm);
    if (jg_launch_solve(d, sp, s, w->nsm, w->prm.solver_block, w->prm.solver_ctas_per_sm) < 0) {
        g_err = "cooperative launch of the solver failed";
        return JG_ERR_CUDA;
    }
    invalidate_graphs(w);  // the arbiter store parity changed outside a captured step
    return finish_step(w, false);
}

int jg_step_host(jg_world* w, float dt, jg_body_desc* bodies, int32_t n) {
    if (!w || !bodies || n != w->d.nb) return JG_ERR_INVALID_ARG;
    // one copy of the caller's array each way; validation and conversion on the device
    int r = upload_bodies_device(w, bodies, n);
    if (r) return r;
    w->host_current = false;
    r = jg_step(w, dt);
    if (r) return r;
    return download_bodies_device(w, bodies, n);
}

// The servos' TargetRelativeOrientation / TargetPosition / TargetAngle and MaximumTorque /
// MaximumForce setters (AngularServo.cs:79-98, LinearServo.cs:103-124, LinearAxisServo.cs:131-152,
// TwistServo.cs:89-112): a changed target drops the warm start (and the AngularServo's
// hemisphere), and both setters wake the servo's dynamic bodies (ServoMath.cs:22-28).
int jg_set_servo(jg_world* w, int32_t id, const float* target, float maximum) {
    if (!w || !target || id < 0) return JG_ERR_INVALID_ARG;
    int r = flush_joints(w);
    if (r) return r;
    if (id >= w->nj_host) return JG_ERR_INVALID_ARG;
    JointDev J;
    CK(cudaMemcpy(&J, w->d.joints + id, sizeof(JointDev), cudaMemcpyDeviceToHost));
    const int kind = J.hdr.x;
    if (kind < JG_CONSTRAINT_ANGULARSERVO || kind > JG_CONSTRAINT_TWISTSERVO || !servo_maximum_ok(maximum))
        return JG_ERR_INVALID_ARG;
    const float PI = 3.14159265358979323846f;
    bool changed;
    if (kind == JG_CONSTRAINT_ANGULARSERVO) {
        for (int i = 0; i < 4; i++) if (!std::isfinite(target[i])) return JG_ERR_INVALID_ARG;
        float l2 = target[0] * target[0] + target[1] * target[1] + target[2] * target[2] + target[3] * target[3];
        if (std::fabs(l2 - 1.0f) > 1e-3f) return JG_ERR_INVALID_ARG;
        float4 t = make_float4(target[0], target[1], target[2], target[3]);
        changed = memcmp(&t, &J.q0, sizeof(t)) != 0;
        J.q0 = t;
        if (changed) J.bil.w = 0.f;
    } else if (kind == JG_CONSTRAINT_LINEARSERVO) {
        for (int i = 0; i < 3; i++) if (!std::isfinite(target[i])) return JG_ERR_INVALID_ARG;
        float4 t = make_float4(target[0], target[1], target[2], 0.f);
        changed = memcmp(&t, &J.axis, sizeof(t)) != 0;
        J.axis = t;
    } else {
        if (!std::isfinite(target[0])) return JG_ERR_INVALID_ARG;
        if (kind == JG_CONSTRAINT_TWISTSERVO && !(target[0] >= -PI && target[0] <= PI)) return JG_ERR_INVALID_ARG;
        changed = memcmp(&target[0], &J.lim.z, sizeof(float)) != 0;
        J.lim.z = target[0];
    }
    if (changed) J.acc = make_float4(0.f, 0.f, 0.f, 0.f);
    J.lim.y = maximum;
    CK(cudaMemcpy(w->d.joints + id, &J, sizeof(JointDev), cudaMemcpyHostToDevice));
    for (int b : {J.hdr.y, J.hdr.z}) {
        jg_launch_wake_dynamic(w->d, b, w->stream);
        CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(w->stream));
    w->host_current = false;
    return JG_OK;
}

// The constraints' Bias, Softness, LimitBias and LimitSoftness setters (e.g. BallSocket.cs:
// 192-222, HingeAngle.cs:250-312, PointOnLine.cs:308-374, EllipticalConeLimit.cs:226-252): NaN
// keeps a value, a negative one is refused (DebugCheck.IsNonNegative).  The limit pair applies to
// HingeAngle and PointOnLine; the motors have none of the four.
int jg_set_constraint_params(jg_world* w, int32_t id, float bias, float softness, float limit_bias, float limit_softness) {
    if (!w || id < 0) return JG_ERR_INVALID_ARG;
    const float v[4] = {bias, softness, limit_bias, limit_softness};
    for (float x : v) if (!std::isnan(x) && !(x >= 0.f)) return JG_ERR_INVALID_ARG;
    int r = flush_joints(w);
    if (r) return r;
    if (id >= w->nj_host) return JG_ERR_INVALID_ARG;
    JointDev J;
    CK(cudaMemcpy(&J, w->d.joints + id, sizeof(JointDev), cudaMemcpyDeviceToHost));
    const int kind = J.hdr.x;
    if (kind == JG_CONSTRAINT_ANGULARMOTOR || kind == JG_CONSTRAINT_LINEARMOTOR) return JG_ERR_INVALID_ARG;
    const bool limits = kind == JG_CONSTRAINT_HINGEANGLE || kind == JG_CONSTRAINT_POINTONLINE;
    if (!limits && (!std::isnan(limit_bias) || !std::isnan(limit_softness))) return JG_ERR_INVALID_ARG;
    if (!std::isnan(bias)) J.prm.x = bias;
    if (!std::isnan(softness)) J.prm.y = softness;
    if (!std::isnan(limit_bias)) J.prm.z = limit_bias;
    if (!std::isnan(limit_softness)) J.prm.w = limit_softness;
    CK(cudaMemcpy(w->d.joints + id, &J, sizeof(JointDev), cudaMemcpyHostToDevice));
    return JG_OK;
}

int jg_activate_body(jg_world* w, int32_t body) {
    if (!w || body < 0 || body >= w->d.nb) return JG_ERR_INVALID_ARG;
    jg_launch_activate(w->d, body, w->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(w->stream));
    w->host_current = false;
    return JG_OK;
}

int jg_set_body_sleep(jg_world* w, int32_t body, float deactivation_time, float linear_threshold, float angular_threshold) {
    if (!w || body < 0 || body >= w->d.nb) return JG_ERR_INVALID_ARG;
    if (!(deactivation_time >= 0) || !(linear_threshold >= 0) || !(angular_threshold >= 0)) return JG_ERR_INVALID_ARG;
    jg_launch_sleep_settings(w->d, body, deactivation_time, linear_threshold * linear_threshold,
                             angular_threshold * angular_threshold, w->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(w->stream));
    return JG_OK;
}

int jg_get_constraints(jg_world* w, int32_t* keys, float* imp, int32_t cap, int32_t* count) {
    if (!w || !count || cap < 0) return JG_ERR_INVALID_ARG;
    int r = flush_joints(w);
    if (r) return r;
    const int n = w->nj_host;
    *count = n;
    const int k = std::min(n, cap);
    if (k == 0 || (!keys && !imp)) return JG_OK;
    std::vector<JointDev> J(k);
    CK(cudaMemcpy(J.data(), w->d.joints, sizeof(JointDev) * k, cudaMemcpyDeviceToHost));
    for (int i = 0; i < k; i++) {
        if (keys) keys[i] = J[i].hdr.w;
        if (imp) { imp[3 * i] = J[i].acc.x; imp[3 * i + 1] = J[i].acc.y; imp[3 * i + 2] = J[i].acc.z; }
    }
    return JG_OK;
}

int jg_get_counters(jg_world* w, jg_counters* out) {
    if (!w || !out) return JG_ERR_INVALID_ARG;
    *out = w->counters;
    return JG_OK;
}
int jg_get_timings(jg_world* w, jg_timings* out) {
    if (!w || !out) return JG_ERR_INVALID_ARG;
    *out = w->timings;
    return JG_OK;
}

int jg_get_residuals(jg_world* w, float* out, int32_t cap, int32_t* n) {
    if (!w || !out || !n) return JG_ERR_INVALID_ARG;
    std::vector<float> h(2 * JG_RESID_MAX);
    CK(cudaMemcpy(h.data(), w->d.resid, sizeof(float) * h.size(), cudaMemcpyDeviceToHost));
    int k = std::min(w->prm.solver_iterations, JG_RESID_MAX);
    *n = k;
    for (int i = 0; i < k && i < cap; i++) out[i] = (float)(std::sqrt((double)h[2 * i]) / std::max(std::sqrt((double)h[2 * i + 1]), 1e-12));
    return JG_OK;
}

static int check_query_args(const char* fn, jg_world* w, const int32_t* pairs, int32_t n, float* out, int32_t* hit) {
    if (!w || n < 0 || (n > 0 && (!pairs || !out || !hit))) {
        g_err = std::string(fn) + ": null buffer or negative count";
        return JG_ERR_INVALID_ARG;
    }
    for (int32_t i = 0; i < 2 * n; i++)
        if (pairs[i] < 0 || pairs[i] >= w->d.ns) {
            g_err = std::string(fn) + ": shape index " + std::to_string(pairs[i]) + " out of range";
            return JG_ERR_INVALID_ARG;
        }
    return JG_OK;
}

// Pairs in, results out through the world's stream; synchronous.
static int run_query(jg_world* w, const int32_t* pairs, int32_t n, float* out, int32_t* hit, int2* d_pairs,
                     float* d_out, int* d_hit) {
    cudaStream_t s = w->stream;
    CK(cudaMemcpyAsync(d_pairs, pairs, sizeof(int2) * n, cudaMemcpyHostToDevice, s));
    jg_launch_collide_query(w->d, d_pairs, n, 0.02f, d_out, d_hit, s, w->nsm);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, d_out, sizeof(float) * 10 * n, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(hit, d_hit, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return JG_OK;
}

int jg_collide_pairs(jg_world* w, const int32_t* pairs, int32_t n, float* out, int32_t* hit) {
    int r = check_query_args("jg_collide_pairs", w, pairs, n, out, hit);
    if (r || n == 0) return r;
    if (n > w->q_cap) {
        CK(cudaStreamSynchronize(w->stream));
        cudaFree(w->q_pairs); cudaFree(w->q_out); cudaFree(w->q_hit);
        w->q_pairs = nullptr; w->q_out = nullptr; w->q_hit = nullptr; w->q_cap = 0;
        CK(cudaMalloc((void**)&w->q_pairs, sizeof(int2) * n));
        CK(cudaMalloc((void**)&w->q_out, sizeof(float) * 10 * n));
        CK(cudaMalloc((void**)&w->q_hit, sizeof(int) * n));
        w->q_cap = n;
    }
    return run_query(w, pairs, n, out, hit, w->q_pairs, w->q_out, w->q_hit);
}

// jg_collide_pairs_noalloc: the same query with its scratch in a fixed device array of
// JG_COLLIDE_NOALLOC_MAX_PAIRS pairs instead of buffers grown with cudaMalloc.  Layout:
// pairs (int2), results (10 floats), hit flags (int), each region 256-byte aligned.  The
// kernel writes every result and hit slot of the batch, so nothing in the array has to
// start at zero.  The array is shared by every world of a device: calls that overlap on
// the GPU race on it.
namespace {
constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kNaPairs = 0;
constexpr size_t kNaOut = kNaPairs + align256(sizeof(int2) * JG_COLLIDE_NOALLOC_MAX_PAIRS);
constexpr size_t kNaHit = kNaOut + align256(sizeof(float) * 10 * JG_COLLIDE_NOALLOC_MAX_PAIRS);
constexpr size_t kNaBytes = kNaHit + align256(sizeof(int) * JG_COLLIDE_NOALLOC_MAX_PAIRS);
constexpr int kNaMaxDevices = 64;
}  // namespace
static __device__ __align__(256) unsigned char g_collide_scratch[kNaBytes];
static std::mutex g_collide_scratch_mu;
static void* g_collide_scratch_addr[kNaMaxDevices];  // per device, looked up on first use

int jg_collide_pairs_noalloc(jg_world* w, const int32_t* pairs, int32_t n, float* out, int32_t* hit) {
    int r = check_query_args("jg_collide_pairs_noalloc", w, pairs, n, out, hit);
    if (r || n == 0) return r;
    if (n > JG_COLLIDE_NOALLOC_MAX_PAIRS) {
        g_err = "jg_collide_pairs_noalloc: " + std::to_string(n) + " pairs exceed the fixed scratch of " +
                std::to_string(JG_COLLIDE_NOALLOC_MAX_PAIRS) + "; split the batch or call jg_collide_pairs";
        return JG_ERR_CAPACITY;
    }
    int dev = -1;
    CK(cudaGetDevice(&dev));
    if (dev != w->device || dev < 0 || dev >= kNaMaxDevices) {
        g_err = "jg_collide_pairs_noalloc: the current device is not the world's device (or above 63)";
        return JG_ERR_INVALID_ARG;
    }
    unsigned char* base;
    {
        std::lock_guard<std::mutex> lock(g_collide_scratch_mu);
        if (!g_collide_scratch_addr[dev]) {
            void* p = nullptr;
            CK(cudaGetSymbolAddress(&p, g_collide_scratch));
            g_collide_scratch_addr[dev] = p;
        }
        base = (unsigned char*)g_collide_scratch_addr[dev];
    }
    return run_query(w, pairs, n, out, hit, (int2*)(base + kNaPairs), (float*)(base + kNaOut), (int*)(base + kNaHit));
}

int jg_manifold_pairs(jg_world* w, const int32_t* pairs, int32_t n, const float* points, float* out, int32_t* counts) {
    int r = check_query_args("jg_manifold_pairs", w, pairs, n, out, counts);
    if (r || n == 0) return r;
    if (!points) { g_err = "jg_manifold_pairs: null points"; return JG_ERR_INVALID_ARG; }
    int2* d_pairs = nullptr;
    float *d_in = nullptr, *d_out = nullptr;
    int* d_cnt = nullptr;
    cudaStream_t s = w->stream;
    cudaError_t e = cudaMalloc((void**)&d_pairs, sizeof(int2) * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_in, sizeof(float) * 9 * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_out, sizeof(float) * 24 * n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_cnt, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_pairs, pairs, sizeof(int2) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_in, points, sizeof(float) * 9 * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        jg_launch_manifold_query(w->d, d_pairs, n, d_in, d_out, d_cnt, s, w->nsm);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, sizeof(float) * 24 * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(counts, d_cnt, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_pairs); cudaFree(d_in); cudaFree(d_out); cudaFree(d_cnt);
    return e == cudaSuccess ? JG_OK : cuda_fail(e, "jg_manifold_pairs");
}

int jg_get_pairs(jg_world* w, int32_t* out, int32_t cap, int32_t* count) {
    if (!w || !count || cap < 0 || (cap > 0 && !out)) return JG_ERR_INVALID_ARG;
    int n = 0;
    CK(cudaMemcpy(&n, &w->d.ctr->npairs, sizeof(int), cudaMemcpyDeviceToHost));
    n = std::min(n, w->d.cap_pairs);
    *count = n;
    if (cap > 0 && n > 0) CK(cudaMemcpy(out, w->d.pairs, sizeof(int2) * std::min(n, cap), cudaMemcpyDeviceToHost));
    return JG_OK;
}

int jg_get_contacts(jg_world* w, jg_contact_view* out, int32_t cap, int32_t* count) {
    if (!w || !count) return JG_ERR_INVALID_ARG;
    WorldDev& D = w->d;
    int narb = 0;
    CK(cudaMemcpy(&narb, &D.ctr->narb, sizeof(int), cudaMemcpyDeviceToHost));
    narb = std::min(narb, D.cap_arb);
    const ArbStore& A = D.arb[D.cur];
    int c = D.cap_arb;
    std::vector<int2> key(narb), body(narb);
    std::vector<int4> info(narb);
    std::vector<float4> mat(narb);
    std::vector<float4> f[8];
    CK(cudaMemcpy(key.data(), A.key, sizeof(int2) * narb, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(body.data(), A.body, sizeof(int2) * narb, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(info.data(), A.info, sizeof(int4) * narb, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(mat.data(), A.mat, sizeof(float4) * narb, cudaMemcpyDeviceToHost));
    float4* src[8] = {A.cn, A.ct1, A.ct2, A.cr1, A.cr2, A.cacc, A.cp1, A.cp2};
    for (int k = 0; k < 8; k++) {
        f[k].resize(4 * (size_t)narb);
        for (int s = 0; s < 4; s++)
            CK(cudaMemcpy(f[k].data() + (size_t)s * narb, src[k] + (size_t)s * c, sizeof(float4) * narb, cudaMemcpyDeviceToHost));
    }
    int n = 0;
    for (int a = 0; a < narb; a++)
        for (int s = 0; s < 4; s++) {
            if (!(info[a].x & (0x11 << s))) continue;
            if (out && n < cap) {
                jg_contact_view& v = out[n];
                size_t i = (size_t)s * narb + a;
                v.shape1 = key[a].x; v.shape2 = key[a].y; v.body1 = body[a].x; v.body2 = body[a].y;
                v.slot = s; v.usage_mask = info[a].x; v.color = info[a].z;
                v.flags = host_float_as_int(f[2][i].w);
                auto put = [](float* o, float4 x) { o[0] = x.x; o[1] = x.y; o[2] = x.z; };
                put(v.normal, f[0][i]); put(v.tangent1, f[1][i]); put(v.tangent2, f[2][i]);
                put(v.rel_pos1, f[3][i]); put(v.rel_pos2, f[4][i]); put(v.pos1_local, f[6][i]); put(v.pos2_local, f[7][i]);
                v.accumulated[0] = f[5][i].x; v.accumulated[1] = f[5][i].y; v.accumulated[2] = f[5][i].z;
                v.mass[0] = f[3][i].w; v.mass[1] = f[4][i].w; v.mass[2] = f[5][i].w;
                v.bias = f[0][i].w; v.penalty_bias = f[1][i].w;
                v.friction = mat[a].x; v.restitution = mat[a].y;
            }
            n++;
        }
    *count = n;
    return JG_OK;
}

int jg_get_arbiter_events(jg_world* w, int32_t* created, int32_t ccap, int32_t* nc, int32_t* removed, int32_t rcap,
                          int32_t* nr) {
    if (!w || !nc || !nr) return JG_ERR_INVALID_ARG;
    int a = (int)std::min<int64_t>(w->counters.created_arbiters, w->d.cap_arb);
    int b = (int)std::min<int64_t>(w->counters.removed_arbiters, w->d.cap_arb);
    *nc = a; *nr = b;
    if (created && ccap > 0) CK(cudaMemcpy(created, w->d.ev_created, sizeof(int2) * std::min(a, ccap), cudaMemcpyDeviceToHost));
    if (removed && rcap > 0) CK(cudaMemcpy(removed, w->d.ev_removed, sizeof(int2) * std::min(b, rcap), cudaMemcpyDeviceToHost));
    return JG_OK;
}

// State blob: header, bodies (jg_body_desc), arbiter store of the live buffer, joints.
struct StateHeader { int magic, version, nb, narb, nj, cap_arb; };

// Layout of a state blob: the header, nb body descriptors, narb arbiters (key, bodies,
// info, material, then 8 contact fields x 4 slots of float4) and nj joint records.
static int64_t state_blob_size(int nb, int narb, int nj) {
    const int64_t per_arb = sizeof(int2) * 2 + sizeof(int4) + sizeof(float4) + 32 * sizeof(float4);
    return (int64_t)sizeof(StateHeader) + (int64_t)sizeof(jg_body_desc) * nb + per_arb * narb +
           (int64_t)sizeof(JointDev) * nj;
}


int jg_export_state(jg_world* w, void* buf, int64_t cap, int64_t* size) {
    if (!w || !size) return JG_ERR_INVALID_ARG;
    int fr = flush_joints(w);
    if (fr) return fr;
    WorldDev& D = w->d;
    int narb = 0;
    CK(cudaMemcpy(&narb, &D.ctr->narb, sizeof(int), cudaMemcpyDeviceToHost));
    narb = std::min(narb, D.cap_arb);
    int64_t need = state_blob_size(D.nb, narb, D.nj);
    *size = need;
    if (!buf) return JG_OK;
    if (cap < need) return JG_ERR_CAPACITY;
    char* p = (char*)buf;
    StateHeader h{0x4a475331, 1, D.nb, narb, D.nj, D.cap_arb};
    memcpy(p, &h, sizeof(h)); p += sizeof(h);
    int r = jg_download_bodies(w, (jg_body_desc*)p, D.nb);
    if (r) return r;
    p += sizeof(jg_body_desc) * D.nb;
    const ArbStore& A = D.arb[D.cur];
    auto cp = [&](const void* src, size_t bytes) -> int {
        cudaError_t e = cudaMemcpy(p, src, bytes, cudaMemcpyDeviceToHost);
        p += bytes;
        return e == cudaSuccess ? 0 : cuda_fail(e, "export");
    };
    if ((r = cp(A.key, sizeof(int2) * narb))) return r;
    if ((r = cp(A.body, sizeof(int2) * narb))) return r;
    if ((r = cp(A.info, sizeof(int4) * narb))) return r;
    if ((r = cp(A.mat, sizeof(float4) * narb))) return r;
    float4* fs[8] = {A.cn, A.ct1, A.ct2, A.cr1, A.cr2, A.cacc, A.cp1, A.cp2};
    for (int k = 0; k < 8; k++)
        for (int s = 0; s < 4; s++)
            if ((r = cp(fs[k] + (size_t)s * D.cap_arb, sizeof(float4) * narb))) return r;
    if ((r = cp(D.joints, sizeof(JointDev) * D.nj))) return r;
    return JG_OK;
}

int jg_check_state(const void* buf, int64_t size, int32_t nb, int32_t ns, int32_t cap_arb, int32_t cap_joints) {
    if (!buf || size < (int64_t)sizeof(StateHeader)) { g_err = "state blob shorter than its header"; return JG_ERR_INVALID_ARG; }
    StateHeader h;
    memcpy(&h, buf, sizeof(h));
    if (h.magic != 0x4a475331 || h.version != 1) { g_err = "not a state blob of this version"; return JG_ERR_INVALID_ARG; }
    if (h.nb != nb || h.narb < 0 || h.nj < 0) { g_err = "state blob counts do not fit the world"; return JG_ERR_INVALID_ARG; }
    if (h.narb > cap_arb || h.nj > cap_joints) { g_err = "state blob exceeds the world's pools"; return JG_ERR_CAPACITY; }
    if (size < state_blob_size(h.nb, h.narb, h.nj)) { g_err = "state blob truncated"; return JG_ERR_INVALID_ARG; }
    const char* p = (const char*)buf + sizeof(StateHeader) + sizeof(jg_body_desc) * (size_t)h.nb;
    const int2* key = (const int2*)p;
    const int2* body = key + h.narb;
    for (int a = 0; a < h.narb; a++) {
        int2 k, b;
        memcpy(&k, key + a, sizeof(k));
        memcpy(&b, body + a, sizeof(b));
        if (k.x < 0 || k.x >= ns || k.y < 0 || k.y >= ns || b.x < 0 || b.x >= nb || b.y < 0 || b.y >= nb) {
            g_err = "state blob arbiter " + std::to_string(a) + " names a shape or body outside the world";
            return JG_ERR_INVALID_ARG;
        }
    }
    const char* jp = (const char*)buf + state_blob_size(h.nb, h.narb, 0);
    for (int j = 0; j < h.nj; j++) {
        int4 hd;
        memcpy(&hd, jp + sizeof(JointDev) * (size_t)j, sizeof(hd));
        if (hd.x < JG_CONSTRAINT_BALLSOCKET || hd.x > JG_CONSTRAINT_ELLIPTICALCONELIMIT || hd.y < 0 || hd.y >= nb || hd.z < 0 ||
            hd.z >= nb) {
            g_err = "state blob joint " + std::to_string(j) + " has an invalid kind or body";
            return JG_ERR_INVALID_ARG;
        }
    }
    return JG_OK;
}

int jg_import_state(jg_world* w, const void* buf, int64_t size) {
    if (!w) return JG_ERR_INVALID_ARG;
    int chk = jg_check_state(buf, size, w->d.nb, w->d.ns, w->d.cap_arb, w->d.cap_joints);
    if (chk) return chk;
    int fr = flush_joints(w);
    if (fr) return fr;
    w->host_current = false;
    const char* p = (const char*)buf;
    StateHeader h;
    memcpy(&h, p, sizeof(h)); p += sizeof(h);
    WorldDev& D = w->d;
    int r = jg_upload_bodies(w, (const jg_body_desc*)p, h.nb);
    if (r) return r;
    p += sizeof(jg_body_desc) * h.nb;
    const ArbStore& A = D.arb[D.cur];
    int narb = h.narb;
    auto cp = [&](void* dst, size_t bytes) -> int {
        cudaError_t e = cudaMemcpy(dst, p, bytes, cudaMemcpyHostToDevice);
        p += bytes;
        return e == cudaSuccess ? 0 : cuda_fail(e, "import");
    };
    if ((r = cp(A.key, sizeof(int2) * narb))) return r;
    if ((r = cp(A.body, sizeof(int2) * narb))) return r;
    if ((r = cp(A.info, sizeof(int4) * narb))) return r;
    if ((r = cp(A.mat, sizeof(float4) * narb))) return r;
    float4* fs[8] = {A.cn, A.ct1, A.ct2, A.cr1, A.cr2, A.cacc, A.cp1, A.cp2};
    for (int k = 0; k < 8; k++)
        for (int s = 0; s < 4; s++)
            if ((r = cp(fs[k] + (size_t)s * D.cap_arb, sizeof(float4) * narb))) return r;
    if ((r = cp(D.joints, sizeof(JointDev) * h.nj))) return r;
    CK(cudaMemcpy(&D.ctr->narb, &narb, sizeof(int), cudaMemcpyHostToDevice));
    D.nj = h.nj;
    w->nj_host = h.nj;
    invalidate_graphs(w);
    return JG_OK;
}

int jg_autotune(jg_world* w, float dt, int32_t steps, jg_world_params* chosen) {
    if (!w || steps < 1) return JG_ERR_INVALID_ARG;
    int64_t size = 0;
    int r = jg_export_state(w, nullptr, 0, &size);
    if (r) return r;
    std::vector<char> snap(size);
    if ((r = jg_export_state(w, snap.data(), size, &size))) return r;
    jg_world_params saved = w->prm;
    // steps from the snapshot under the current settings: milliseconds, or -1 on an error
    auto trial = [&]() -> float {
        w->prm.use_graph = 0;
        jg_solver_reset_launch_cache(w->d);
        if (jg_import_state(w, snap.data(), size)) return -1.f;
        if (jg_step(w, dt)) return -1.f;  // warm-up
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0); cudaEventCreate(&e1);
        cudaEventRecord(e0, w->stream);
        bool ok = true;
        for (int s = 0; s < steps && ok; s++) ok = jg_step(w, dt) == JG_OK;
        cudaEventRecord(e1, w->stream);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        return ok ? ms : -1.f;
    };
    // 1. the solve's form (spatial tasks with their bodies in shared memory, or global
    // colours) and its launch shape: threads per task CTA x task CTAs per SM (shared memory
    // bound), or threads per CTA x CTAs per SM
    const int pblocks[] = {64, 96, 128}, gblocks[] = {128, 256, 512};
    const int pctas[] = {1, 2}, gctas[] = {1, 2, 4};
    float best = 1e30f;
    int bp = w->prm.partitioned_solve != 0, bb = bp ? JG_TASK_BLOCK : 256, bc = bp ? JG_TASK_CTAS : 2;
    for (int part = 1; part >= 0; part--)
    for (int ib = 0; ib < 3; ib++)
        for (int ic = 0; ic < (part ? 2 : 3); ic++) {
            const int b = part ? pblocks[ib] : gblocks[ib], c = part ? pctas[ic] : gctas[ic];
            w->prm.partitioned_solve = part;
            w->prm.solver_block = b;
            w->prm.solver_ctas_per_sm = c;
            const float ms = trial();
            if (ms >= 0 && ms < best) { best = ms; bb = b; bc = c; bp = part; }
        }
    w->prm.partitioned_solve = bp;
    w->prm.solver_block = bb;
    w->prm.solver_ctas_per_sm = bc;
    // 2. for the spatial tasks, the partition's cell density (cells per grid and SM): more
    // cells make the longest task shorter and add per-task latency
    float bcell = saved.sched_cells_per_sm;
    if (bp && w->d.nworlds <= 1) {  // (batched worlds: one cell per world)
        const float cells[] = {0.f, 1.f, 2.f, 3.f, 4.5f, 6.f, 9.f};  // 0: the default rule
        float bcm = 1e30f;
        for (float c : cells) {
            w->prm.sched_cells_per_sm = c;
            const float ms = trial();
            if (ms >= 0 && ms < bcm) { bcm = ms; bcell = c; }
        }
    }
    jg_world_params out = saved;
    out.partitioned_solve = bp;
    out.solver_block = bb;
    out.solver_ctas_per_sm = bc;
    out.sched_cells_per_sm = bcell;
    w->prm = out;
    jg_solver_reset_launch_cache(w->d);
    invalidate_graphs(w);
    r = jg_import_state(w, snap.data(), size);
    if (chosen) *chosen = w->prm;
    return r;
}

}  // extern "C"

// accessors for the MLP translation unit
void*& jg_world_mlp(jg_world* w) { return w->mlp; }
void jg_world_invalidate_graphs(jg_world* w) { invalidate_graphs(w); }
int* jg_world_dst_index(jg_world* w) { return w->d.dst_index; }
void jg_set_error(const char* msg) { g_err = msg; }
WorldDev& jg_world_dev(jg_world* w) { return w->d; }
cudaStream_t jg_world_stream(jg_world* w) { return w->stream; }
int jg_world_nsm(jg_world* w) { return w->nsm; }
void jg_world_set_mlp_ready(jg_world* w, bool r) { w->mlp_ready = r; }
int jg_world_iterations(jg_world* w) { return w->prm.solver_iterations; }
