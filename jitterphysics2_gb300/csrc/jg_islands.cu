// Islands and sleeping (World.AllowDeactivation): CheckDeactivation (World.Step.cs:1289-1371)
// on the islands of the connection graph.  The reference keeps islands incrementally
// (IslandHelper.cs:54-278: merge on a new connection, split on a removed one) with two flags
// per island, MarkedAsActive and membership of the active list.  Every merge comes with
// AddToActiveList (World.cs:903-910) on both islands, and every split of a step follows
// AddToActiveList on both bodies of the removed arbiter, so an island's flag is the OR of
// per-body flags over its bodies, and the island itself is a connected component of the
// arbiters and constraints among non-static bodies (static bodies are alone).  Each step
// therefore rebuilds the components by union-find over the arbiter and joint lists, ORs the
// two flags per component root and applies the reference's rule to every body of an island
// in the active list:
//   nobody marked the island     -> its bodies deactivate (DeactivateBodyForSleep)
//   otherwise                    -> the island stays in the active list; its inactive
//                                   non-static bodies activate with their sleep time reset
// and clears each such body's mark for the next step.  Per body, binfo.w holds the flags
// (1: marked, 2: island in the active list); sleep = (sleep time, deactivation time,
// squared linear and angular rest thresholds).
#include "jg_world.cuh"

namespace {

__device__ __forceinline__ bool non_static(const WorldDev& w, int b) { return w.binfo[b].x != JG_MOTION_STATIC; }

// Root of x with path halving.  Parent indices only ever decrease (a root is linked below
// a smaller root), so a halving store races benignly with a concurrent link.
__device__ __forceinline__ int uf_find(volatile int* p, int x) {
    for (;;) {
        int px = p[x];
        if (px == x) return x;
        int gp = p[px];
        if (gp != px) p[x] = gp;
        x = px;
    }
}

// Joins the components of a and b: the larger root is linked below the smaller one with a
// compare-and-swap; a failed swap means another thread linked that root first, so the
// loop retries from the new root (each retry follows a strictly smaller root: it ends).
__device__ __forceinline__ void uf_link(int* parent, int a, int b) {
    volatile int* p = parent;
    for (;;) {
        a = uf_find(p, a);
        b = uf_find(p, b);
        if (a == b) return;
        if (a < b) { int t = a; a = b; b = t; }
        if (atomicCAS(&parent[a], a, b) == a) return;
    }
}

__global__ void k_uf_init(WorldDev w) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.nb; b += gridDim.x * blockDim.x) {
        w.uf[b] = b;
        w.ufl[b] = 0;
    }
}

// Every arbiter of the step (those about to be removed included: the reference removes them
// after this check) and every constraint joins its two bodies when both are non-static.
__global__ void k_uf_link(WorldDev w) {
    const ArbStore& A = w.arb[w.cur];
    const int narb = min(w.ctr->narb, w.cap_arb);
    const int n = narb + w.nj;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        int b1, b2;
        if (c < narb) { int2 bb = A.body[c]; b1 = bb.x; b2 = bb.y; }
        else { int4 h = w.joints[c - narb].hdr; b1 = h.y; b2 = h.z; }
        if (b1 != b2 && non_static(w, b1) && non_static(w, b2)) uf_link(w.uf, b1, b2);
    }
}

// The island flags: the OR of the bodies' flags at each root (roots stored in uf).
__global__ void k_uf_flags(WorldDev w) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.nb; b += gridDim.x * blockDim.x) {
        int r = uf_find(w.uf, b);
        w.uf[b] = r;
        int f = w.binfo[b].w & 3;
        if (f) atomicOr(&w.ufl[r], f);
    }
}

// CheckDeactivation's rule on the bodies of islands in the active list.
__global__ void k_uf_apply(WorldDev w) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.nb; b += gridDim.x * blockDim.x) {
        const int f = w.ufl[w.uf[b]];
        if (!(f & 2)) continue;  // a sleeping island is not visited
        int4 bi = w.binfo[b];
        if (!(f & 1)) {
            bi.y &= ~JG_BODY_ACTIVE;  // DeactivateBodyForSleep (World.Step.cs:1247-1287): velocities kept
            bi.w = 0;
        } else {
            bi.w = 2;
            if (!(bi.y & JG_BODY_ACTIVE) && bi.x != JG_MOTION_STATIC) {
                bi.y |= JG_BODY_ACTIVE;
                w.sleep[b].x = 0.f;
            }
        }
        w.binfo[b] = bi;
    }
}

// World.ActivateBodyNextStep (World.cs:696-720) / RigidBody.SetActivationState(true).
__global__ void k_activate(WorldDev w, int b) {
    w.sleep[b].x = 0.f;
    int4 bi = w.binfo[b];
    if ((bi.y & JG_BODY_ACTIVE) || bi.x == JG_MOTION_STATIC) return;
    bi.w |= 3;  // AddToActiveList
    w.binfo[b] = bi;
}

// ServoMath.WakeBodies (ServoMath.cs:22-28): an inactive dynamic body is activated at the
// next step; other bodies are left alone
__global__ void k_wake_dynamic(WorldDev w, int b) {
    int4 bi = w.binfo[b];
    if (bi.x != JG_MOTION_DYNAMIC || (bi.y & JG_BODY_ACTIVE)) return;
    w.sleep[b].x = 0.f;
    bi.w |= 3;  // AddToActiveList
    w.binfo[b] = bi;
}

__global__ void k_sleep_settings(WorldDev w, int b, float deactivation_time, float lin2, float ang2) {
    float4 s = w.sleep[b];
    w.sleep[b] = make_float4(s.x, deactivation_time, lin2, ang2);
}

__global__ void k_sleep_init(float4* sleep, int n) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x)
        sleep[b] = make_float4(0.f, 1.0f, 0.1f, 0.1f);  // RigidBody.cs:398-400 defaults
}

}  // namespace

void jg_launch_islands(WorldDev& w, cudaStream_t s, int nsm) {
    const int blocks = nsm * 4;
    k_uf_init<<<blocks, 256, 0, s>>>(w);
    k_uf_link<<<blocks, 256, 0, s>>>(w);
    k_uf_flags<<<blocks, 256, 0, s>>>(w);
    k_uf_apply<<<blocks, 256, 0, s>>>(w);
}
void jg_launch_activate(WorldDev& w, int body, cudaStream_t s) { k_activate<<<1, 1, 0, s>>>(w, body); }
void jg_launch_wake_dynamic(WorldDev& w, int body, cudaStream_t s) { k_wake_dynamic<<<1, 1, 0, s>>>(w, body); }
void jg_launch_sleep_settings(WorldDev& w, int body, float t, float lin2, float ang2, cudaStream_t s) {
    k_sleep_settings<<<1, 1, 0, s>>>(w, body, t, lin2, ang2);
}
void jg_launch_sleep_init(float4* sleep, int n, cudaStream_t s) { k_sleep_init<<<64, 256, 0, s>>>(sleep, n); }
