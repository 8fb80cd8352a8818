// Broadphase: world AABBs, a linear BVH rebuilt every step (Morton codes, an LSD radix
// sort written here, Karras-style hierarchy, bottom-up refit) and one traversal per
// dynamic shape that writes the pair list.
//
// Contract (the reference's, not its data structure): every shape pair on different
// bodies of the same world whose exact world AABBs are not disjoint (touching counts),
// with at least one body active and at least one dynamic
// (DynamicTree.EnumerateOverlapsCallback, Collision/DynamicTree/DynamicTree.cs:266-286;
// JBoundingBox.Disjoint, LinearMath/JBoundingBox.cs:314-318; World.DefaultDynamicTreeFilter,
// World.cs:447-455; World.Detect.cs:158-160).  The reference keeps an incremental SAH tree
// with enlarged boxes; the set of pairs handed to the narrowphase is the same, the order
// is not.
#include "jg_shapes.cuh"

namespace {

__device__ __forceinline__ unsigned f2ord(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__global__ void k_aabb(WorldDev w, unsigned* scene, float dt) {
    __shared__ unsigned smin[3], smax[3];
    if (threadIdx.x < 3) { smin[threadIdx.x] = 0xffffffffu; smax[threadIdx.x] = 0u; }
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.ns; i += gridDim.x * blockDim.x) {
        ShapeRef s = load_shape(w, i);
        int b = w.sinfo[i].y;
        float4 p4 = w.pos[b], q4v = w.q[b];
        v3 mn, mx;
        shape_aabb(s, mkq(q4v), mk3(p4), mn, mx);
        if (w.binfo[b].y & JG_BODY_SPECULATIVE) {
            // RigidBodyShape.UpdateWorldBoundingBox (RigidBodyShape.cs:37-57): a speculative
            // body's box grows by the distance its linear velocity covers in one step
            float swept = dt * sqrtf(len2(mk3(w.body[b].v)));
            mn = mn - mk3(swept);
            mx = mx + mk3(swept);
        }
        w.amin[i] = f4(mn, 0.f);
        w.amax[i] = f4(mx, 0.f);
        v3 c = 0.5f * (mn + mx);
        atomicMin(&smin[0], f2ord(c.x)); atomicMin(&smin[1], f2ord(c.y)); atomicMin(&smin[2], f2ord(c.z));
        atomicMax(&smax[0], f2ord(c.x)); atomicMax(&smax[1], f2ord(c.y)); atomicMax(&smax[2], f2ord(c.z));
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        atomicMin(&scene[threadIdx.x], smin[threadIdx.x]);
        atomicMax(&scene[3 + threadIdx.x], smax[threadIdx.x]);
    }
}

__global__ void k_scene_init(unsigned* scene) {
    if (threadIdx.x < 3) { scene[threadIdx.x] = 0xffffffffu; scene[3 + threadIdx.x] = 0u; }
}

__device__ __forceinline__ unsigned expand10(unsigned v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_morton(WorldDev w, const unsigned* scene) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.ns) return;
    v3 lo = mk3(ord2f(scene[0]), ord2f(scene[1]), ord2f(scene[2]));
    v3 hi = mk3(ord2f(scene[3]), ord2f(scene[4]), ord2f(scene[5]));
    float4 a = w.amin[i], b = w.amax[i];
    v3 c = 0.5f * (mk3(a) + mk3(b));
    v3 ext = hi - lo;
    float ex = fmaxf(ext.x, 1e-6f), ey = fmaxf(ext.y, 1e-6f), ez = fmaxf(ext.z, 1e-6f);
    unsigned x = (unsigned)fminf(fmaxf((c.x - lo.x) / ex * 1023.0f, 0.0f), 1023.0f);
    unsigned y = (unsigned)fminf(fmaxf((c.y - lo.y) / ey * 1023.0f, 0.0f), 1023.0f);
    unsigned z = (unsigned)fminf(fmaxf((c.z - lo.z) / ez * 1023.0f, 0.0f), 1023.0f);
    unsigned m = (expand10(x) << 2) | (expand10(y) << 1) | expand10(z);
    int world = w.binfo[w.sinfo[i].y].z;
    w.mkey[i] = ((unsigned long long)(unsigned)world << 32) | m;
    w.midx[i] = i;
}

// ---- LSD radix sort of (u64 key, int value), 8-bit digits ------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;

__global__ void k_rs_hist(const unsigned long long* keys, int n, int shift, int* hist, int nblocks) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    int base = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ITEMS; r++) {
        int i = base + r * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255], 1);
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_rs_scan(int* hist, int total) {
    // single block exclusive scan, 1024 threads, chunked
    __shared__ int carry;
    __shared__ int warp_sums[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < total; base += blockDim.x) {
        int i = base + threadIdx.x;
        int v = i < total ? hist[i] : 0;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) >= o) x += y;
        }
        if ((threadIdx.x & 31) == 31) warp_sums[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            int s = warp_sums[threadIdx.x];
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, s, o);
                if (threadIdx.x >= o) s += y;
            }
            warp_sums[threadIdx.x] = s;
        }
        __syncthreads();
        int warp_prefix = (threadIdx.x >= 32) ? warp_sums[(threadIdx.x >> 5) - 1] : 0;
        int excl = carry + warp_prefix + x - v;
        if (i < total) hist[i] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
}

__global__ void k_rs_scatter(const unsigned long long* keys, const int* vals, unsigned long long* okeys, int* ovals,
                             int n, int shift, const int* hist, int nblocks) {
    __shared__ int wcnt[RS_THREADS / 32][256];
    __shared__ int running[256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    running[threadIdx.x] = hist[threadIdx.x * nblocks + blockIdx.x];
    int base = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ITEMS; r++) {
        for (int k = threadIdx.x; k < (RS_THREADS / 32) * 256; k += RS_THREADS) (&wcnt[0][0])[k] = 0;
        __syncthreads();
        int i = base + r * RS_THREADS + threadIdx.x;
        bool valid = i < n;
        unsigned long long key = valid ? keys[i] : 0ull;
        int dg = valid ? (int)((key >> shift) & 255) : 256 + lane;
        unsigned peers = __match_any_sync(0xffffffffu, dg);
        int rank = __popc(peers & ((1u << lane) - 1u));
        int leader = __ffs(peers) - 1;
        if (valid && lane == leader) wcnt[warp][dg] = __popc(peers);
        __syncthreads();
        {
            int d = threadIdx.x;
            int acc = running[d];
            for (int ww = 0; ww < RS_THREADS / 32; ww++) {
                int t = wcnt[ww][d];
                wcnt[ww][d] = acc;
                acc += t;
            }
            running[d] = acc;
        }
        __syncthreads();
        if (valid) {
            int dst = wcnt[warp][dg] + rank;
            okeys[dst] = key;
            ovals[dst] = vals[i];
        }
        __syncthreads();
    }
}

// ---- Karras hierarchy -------------------------------------------------------------------
__device__ __forceinline__ int delta(const unsigned long long* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    unsigned long long a = k[i], b = k[j];
    if (a == b) return 64 + __clz(i ^ j);
    return __clzll(a ^ b);
}

__global__ void k_build(WorldDev w, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const unsigned long long* k = w.mkey;
    int d = (delta(k, n, i, i + 1) - delta(k, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(k, n, i, i - d);
    int lmax = 2;
    while (delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(k, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int g = i + s * d + min(d, 0);
    int first = min(i, j), last = max(i, j);
    int left = (first == g) ? ~g : g;
    int right = (last == g + 1) ? ~(g + 1) : (g + 1);
    w.node[i] = make_int4(left, right, 0, 0);
    w.node_range[i] = make_int2(first, last);
    if (left < 0) w.leaf_parent[~left] = i; else w.node_parent[left] = i;
    if (right < 0) w.leaf_parent[~right] = i; else w.node_parent[right] = i;
}

__global__ void k_build_init(WorldDev w, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n - 1) { w.node_parent[i] = -1; w.node_flag[i] = 0; }
}

// A leaf's body id with its motion and activity, stored beside the leaf's box:
// body | dynamic << 30 | active << 29.
constexpr int LEAF_DYN = 1 << 30, LEAF_ACTIVE = 1 << 29, LEAF_BODY = (1 << 29) - 1;
__device__ __forceinline__ int leaf_word(const WorldDev& w, int shape) {
    const int body = w.sinfo[shape].y;
    const int4 bi = w.binfo[body];
    return body | (bi.x == JG_MOTION_DYNAMIC ? LEAF_DYN : 0) | ((bi.y & JG_BODY_ACTIVE) ? LEAF_ACTIVE : 0);
}

__global__ void k_refit(WorldDev w, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int p = w.leaf_parent[i];
    while (p >= 0) {
        __threadfence();
        if (atomicAdd(&w.node_flag[p], 1) == 0) return;
        int4 nd = w.node[p];
        float4 lmn, lmx, rmn, rmx;
        int lcode, rcode;
        if (nd.x < 0) { int s = w.midx[~nd.x]; lmn = w.amin[s]; lmx = w.amax[s]; lcode = ~s; }
        else { lmn = __ldcg(&w.nmin[nd.x]); lmx = __ldcg(&w.nmax[nd.x]); lcode = nd.x; }
        if (nd.y < 0) { int s = w.midx[~nd.y]; rmn = w.amin[s]; rmx = w.amax[s]; rcode = ~s; }
        else { rmn = __ldcg(&w.nmin[nd.y]); rmx = __ldcg(&w.nmax[nd.y]); rcode = nd.y; }
        __stcg(&w.nmin[p], make_float4(fminf(lmn.x, rmn.x), fminf(lmn.y, rmn.y), fminf(lmn.z, rmn.z), 0.f));
        __stcg(&w.nmax[p], make_float4(fmaxf(lmx.x, rmx.x), fmaxf(lmx.y, rmx.y), fmaxf(lmx.z, rmx.z), 0.f));
        // both children's boxes in the parent, for the traversal (one 64-byte read per node)
        int lw = 0, rw = 0;
        if (nd.x < 0) lw = leaf_word(w, ~lcode);
        else if (w.nworlds > 1 && w.nworlds <= 65536) {
            int2 rg = w.node_range[nd.x];
            lw = (int)(w.mkey[rg.x] >> 32) | ((int)(w.mkey[rg.y] >> 32) << 16);
        }
        if (nd.y < 0) rw = leaf_word(w, ~rcode);
        else if (w.nworlds > 1 && w.nworlds <= 65536) {
            int2 rg = w.node_range[nd.y];
            rw = (int)(w.mkey[rg.x] >> 32) | ((int)(w.mkey[rg.y] >> 32) << 16);
        }
        float4* cb = w.cbox + 4 * (size_t)p;
        cb[0] = make_float4(lmn.x, lmn.y, lmn.z, __int_as_float(lcode));
        cb[1] = make_float4(lmx.x, lmx.y, lmx.z, __int_as_float(lw));
        cb[2] = make_float4(rmn.x, rmn.y, rmn.z, __int_as_float(rcode));
        cb[3] = make_float4(rmx.x, rmx.y, rmx.z, __int_as_float(rw));
        p = w.node_parent[p];
    }
}

__device__ __forceinline__ bool overlap(float4 amn, float4 amx, float4 bmn, float4 bmx) {
    // !JBoundingBox.Disjoint (touching boxes overlap)
    return !(amx.x < bmn.x || amn.x > bmx.x || amx.y < bmn.y || amn.y > bmx.y || amx.z < bmn.z || amn.z > bmx.z);
}

constexpr int PAIR_BUF = 16;

__device__ __forceinline__ void flush_pairs(WorldDev& w, int2* buf, int& nbuf) {
    if (nbuf == 0) return;
    int base = atomicAdd(&w.ctr->npairs, nbuf);
    for (int k = 0; k < nbuf; k++) {
        if (base + k < w.cap_pairs) w.pairs[base + k] = buf[k];
        else atomicCAS(&w.ctr->status, 0, JG_ERR_CAPACITY);
    }
    nbuf = 0;
}

__global__ void k_traverse(WorldDev w, int n) {
    int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n) return;
    int sa = w.midx[li];
    int4 sia = w.sinfo[sa];
    int4 bia = w.binfo[sia.y];
    if (bia.x != JG_MOTION_DYNAMIC) return;  // queries start from dynamic shapes only
    bool act_a = (bia.y & JG_BODY_ACTIVE) != 0;
    int world = bia.z;
    float4 qmn = w.amin[sa], qmx = w.amax[sa];
    int2 buf[PAIR_BUF];
    int nbuf = 0;
    int stack[64];
    int sp = 0;
    int node = 0;
    if (n == 1) return;
    const bool packed_worlds = w.nworlds <= 65536;
    while (true) {
        // both children's boxes, stored in the node by k_refit
        const float4* cb = w.cbox + 4 * (size_t)node;
        const float4 box[4] = {__ldg(cb), __ldg(cb + 1), __ldg(cb + 2), __ldg(cb + 3)};
        int push_cnt = 0;
        int next_nodes[2];
        for (int c = 0; c < 2; c++) {
            const float4 bmn = box[2 * c], bmx = box[2 * c + 1];
            const int cidx = __float_as_int(bmn.w);
            if (!overlap(qmn, qmx, bmn, bmx)) continue;
            if (cidx < 0) {
                int sb = ~cidx;
                if (sb == sa) continue;
                const int lf = __float_as_int(bmx.w);  // body, dynamic, active of the leaf
                const int body_b = lf & LEAF_BODY;
                if (body_b == sia.y) continue;
                if (w.nworlds > 1 && w.binfo[body_b].z != world) continue;
                const bool dyn_b = (lf & LEAF_DYN) != 0;
                if (dyn_b && sb < sa) continue;            // each dynamic pair once
                if (!act_a && (lf & LEAF_ACTIVE) == 0) continue;
                buf[nbuf++] = make_int2(min(sa, sb), max(sa, sb));
                if (nbuf == PAIR_BUF) flush_pairs(w, buf, nbuf);
            } else {
                if (w.nworlds > 1) {  // subtrees hold one world range (the world id leads the Morton key)
                    int wf, wl;
                    if (packed_worlds) {
                        const int wr = __float_as_int(bmx.w);
                        wf = wr & 0xffff; wl = (wr >> 16) & 0xffff;
                    } else {
                        int2 rg = w.node_range[cidx];
                        wf = (int)(w.mkey[rg.x] >> 32); wl = (int)(w.mkey[rg.y] >> 32);
                    }
                    if (world < wf || world > wl) continue;
                }
                next_nodes[push_cnt++] = cidx;
            }
        }
        if (push_cnt == 2) {
            if (sp < 64) stack[sp++] = next_nodes[1];
            else atomicCAS(&w.ctr->status, 0, JG_ERR_CAPACITY);
            node = next_nodes[0];
        } else if (push_cnt == 1) {
            node = next_nodes[0];
        } else {
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    flush_pairs(w, buf, nbuf);
}

}  // namespace

void jg_launch_aabb(WorldDev& w, float dt, cudaStream_t s) {
    if (w.ns == 0) return;
    k_scene_init<<<1, 32, 0, s>>>((unsigned*)w.scene_box);
    int blocks = (w.ns + 255) / 256;
    if (blocks > 1024) blocks = 1024;
    k_aabb<<<blocks, 256, 0, s>>>(w, (unsigned*)w.scene_box, dt);
}

int jg_launch_broadphase(WorldDev& w, cudaStream_t s, int nsm) {
    (void)nsm;
    int n = w.ns;
    if (n < 2) return 0;
    k_morton<<<(n + 255) / 256, 256, 0, s>>>(w, (const unsigned*)w.scene_box);
    int bits = 30;
    int wb = 0;
    while ((1 << wb) < w.nworlds) wb++;
    bits = 32 + wb;
    if (wb == 0) bits = 30;
    int nblocks = (n + RS_TILE - 1) / RS_TILE;
    unsigned long long *ka = w.mkey, *kb = w.mkey_alt;
    int *va = w.midx, *vb = w.midx_alt;
    int passes = 0;
    for (int shift = 0; shift < bits; shift += 8) {
        if (wb > 0 && shift >= 32 - 8 + 8 && shift < 32) { }
        k_rs_hist<<<nblocks, RS_THREADS, 0, s>>>(ka, n, shift, w.hist, nblocks);
        k_rs_scan<<<1, 1024, 0, s>>>(w.hist, 256 * nblocks);
        k_rs_scatter<<<nblocks, RS_THREADS, 0, s>>>(ka, va, kb, vb, n, shift, w.hist, nblocks);
        unsigned long long* tk = ka; ka = kb; kb = tk;
        int* tv = va; va = vb; vb = tv;
        passes++;
    }
    if (ka != w.mkey) {
        cudaMemcpyAsync(w.mkey, ka, sizeof(unsigned long long) * n, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(w.midx, va, sizeof(int) * n, cudaMemcpyDeviceToDevice, s);
    }
    k_build_init<<<(n + 255) / 256, 256, 0, s>>>(w, n);
    k_build<<<(n + 255) / 256, 256, 0, s>>>(w, n);
    k_refit<<<(n + 255) / 256, 256, 0, s>>>(w, n);
    k_traverse<<<(n + 127) / 128, 128, 0, s>>>(w, n);
    return passes;
}
