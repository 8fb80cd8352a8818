// Persistent contact cache and solver colouring.
//
// merge:   the contact stream is matched against the live arbiters through an
//          open-addressing hash on the ordered shape-id pair (ArbiterKey, Arbiter.cs:67-103);
//          unknown keys allocate a new arbiter (ContactData.Init, Contact.cs:271-286), then
//          ResetMode and AddContact run per manifold point (World.RegisterContact,
//          World.Detect.cs:294-324; ContactData.AddContact / SortCachedPoints, Contact.cs:329-580).
// colour:  Jones-Plassmann colouring of contacts and joints with per-body colour masks;
//          static and kinematic bodies never conflict because the solver never writes them.
//          It replaces the reference's per-body spin locks (World.Step.cs:924-986).
// permute: arbiters with contacts are moved to the other buffer sorted by colour; arbiters
//          left without contacts are dropped (RemoveBrokenArbiters, World.Step.cs:839-860).
// update:  ContactData.UpdatePosition (Contact.cs:238-264, :762-797) after the solve.
//
// The contact-cache rules follow code the reference derived from the Bullet Physics
// Engine (zlib license, (c) 2003-2006 Erwin Coumans, https://bulletphysics.org): provided
// 'as-is', without any express or implied warranty; altered source versions must be
// plainly marked as such; this notice may not be removed or altered from any source
// distribution.
#include "jg_sync.cuh"

namespace {

constexpr unsigned long long HEMPTY = 0xffffffffffffffffull;
constexpr float BreakThreshold = 0.02f;

__device__ __forceinline__ unsigned long long akey(int2 k) {
    return ((unsigned long long)(unsigned)k.x << 32) | (unsigned)k.y;
}
__device__ __forceinline__ unsigned hash64(unsigned long long k) {
    k ^= k >> 33; k *= 0xff51afd7ed558ccdull; k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ull; k ^= k >> 33;
    return (unsigned)k;
}

__global__ void k_hash_clear(WorldDev w) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.hcap; i += gridDim.x * blockDim.x) {
        w.hkeys[i] = HEMPTY;
        w.hvals[i] = -1;
    }
}

__device__ __forceinline__ int hash_insert(WorldDev& w, unsigned long long key, int val) {
    unsigned mask = (unsigned)w.hcap - 1u;
    unsigned h = hash64(key) & mask;
    for (int probe = 0; probe < w.hcap; probe++) {
        unsigned long long prev = atomicCAS(&w.hkeys[h], HEMPTY, key);
        if (prev == HEMPTY) { w.hvals[h] = val; return val; }
        if (prev == key) return -2;
        h = (h + 1) & mask;
    }
    return -3;
}
__device__ __forceinline__ int hash_find(const WorldDev& w, unsigned long long key) {
    unsigned mask = (unsigned)w.hcap - 1u;
    unsigned h = hash64(key) & mask;
    for (int probe = 0; probe < w.hcap; probe++) {
        unsigned long long k = w.hkeys[h];
        if (k == key) return w.hvals[h];
        if (k == HEMPTY) return -1;
        h = (h + 1) & mask;
    }
    return -1;
}

__global__ void k_hash_build(WorldDev w) {
    const ArbStore& A = w.arb[w.cur];
    int n = w.ctr->narb;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x)
        hash_insert(w, akey(A.key[a]), a);
}

// Contact.Initialize (Contact.cs:703-759)
__device__ void contact_init(const WorldDev& w, const ArbStore& A, int i, int b1, int b2, int mode, float restitution,
                             v3 p1, v3 p2, v3 n, bool is_new) {
    v3 pos1 = mk3(w.pos[b1]), pos2 = mk3(w.pos[b2]);
    q4 q1 = mkq(w.q[b1]), q2 = mkq(w.q[b2]);
    v3 rel1 = p1 - pos1, rel2 = p2 - pos2;
    A.cr1[i] = f4(rel1, A.cr1[i].w);
    A.cr2[i] = f4(rel2, A.cr2[i].w);
    A.cp1[i] = f4(rotate_inv(rel1, q1), 0.f);
    A.cp2[i] = f4(rotate_inv(rel2, q2), 0.f);
    if (!is_new) return;
    SBody B1 = w.body[b1], B2 = w.body[b2];
    v3 v1 = mk3(B1.v), v2 = mk3(B2.v), w1 = mk3(B1.w), w2 = mk3(B2.w);
    v3 dv = v2 - v1;
    if (mode == 0 || (mode & (2 | 8)) != 0) {
        dv = v2 + cross(w2, rel2);
        dv = dv - (v1 + cross(w1, rel1));
    }
    float rnv = dot(dv, n);
    float bias = 0.f;
    if (rnv < -1.0f) bias = -restitution * rnv;
    v3 t1 = dv - n * rnv;
    float num = len2(t1);
    if (num > 1e-12f) {
        num = 1.0f / sqrtf(num);
        t1 = t1 * num;
    } else {
        t1 = create_orthonormal(n);
    }
    v3 t2 = cross(t1, n);
    A.cn[i] = f4(n, bias);
    A.ct1[i] = f4(t1, 0.f);
    A.ct2[i] = f4(t2, __int_as_float(2));   // Flags.NewContact
    A.cacc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__device__ __forceinline__ float area4(v3 p0, v3 p1, v3 p2, v3 p3) {
    v3 a0 = p0 - p1, a1 = p0 - p2, a2 = p0 - p3;
    v3 b0 = p2 - p3, b1 = p1 - p3, b2 = p1 - p2;
    return fmaxf(fmaxf(len2(cross(a0, b0)), len2(cross(a1, b1))), len2(cross(a2, b2)));
}

// ContactData.AddContact + SortCachedPoints (Contact.cs:329-416, :555-580)
__device__ void add_contact(const WorldDev& w, const ArbStore& A, int a, int& usage, int b1, int b2, int mode,
                            float restitution, v3 p1, v3 p2, v3 n, int& created) {
    const int cap = w.cap_arb;
    v3 rp1 = p1 - mk3(w.pos[b1]);
    if ((usage & 15) == 15) {
        v3 c0 = mk3(A.cr1[a]), c1 = mk3(A.cr1[cap + a]), c2 = mk3(A.cr1[2 * cap + a]), c3 = mk3(A.cr1[3 * cap + a]);
        float ar0 = area4(rp1, c1, c2, c3), ar1 = area4(rp1, c0, c2, c3), ar2 = area4(rp1, c0, c1, c3), ar3 = area4(rp1, c0, c1, c2);
        const float eps = -0.0001f;
        float big = 0.f;
        int mask = 0;
        if (ar0 > big + eps) { big = ar0; mask = 1; }
        if (ar1 > big + eps) { big = ar1; mask = 2; }
        if (ar2 > big + eps) { big = ar2; mask = 4; }
        if (ar3 > big + eps) { mask = 8; }
        int k = mask == 2 ? 1 : (mask == 4 ? 2 : (mask == 8 ? 3 : 0));
        contact_init(w, A, k * cap + a, b1, b2, mode, restitution, p1, p2, n, false);
        usage |= mask;
        return;
    }
    int closest = -1;
    float dist = 3.402823466e+38f;
    for (int k = 0; k < 4; k++) {
        if (!(usage & (1 << k))) continue;
        float d = len2(mk3(A.cr1[k * cap + a]) - rp1);
        if (d < dist) { dist = d; closest = k; }
    }
    if (dist < BreakThreshold * BreakThreshold) {
        contact_init(w, A, closest * cap + a, b1, b2, mode, restitution, p1, p2, n, false);
        return;
    }
    for (int k = 0; k < 4; k++) {
        if (!(usage & (1 << k))) {
            contact_init(w, A, k * cap + a, b1, b2, mode, restitution, p1, p2, n, true);
            usage |= 1 << k;
            created++;
            return;
        }
    }
}

__global__ void k_merge(WorldDev w, StepParams sp, int2* ev_created) {
    const ArbStore& A = w.arb[w.cur];
    int ns = min(w.ctr->nstream, w.cap_pairs);
    int created_pts = 0, contacts = 0, spec = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ns; i += gridDim.x * blockDim.x) {
        int2 key = w.cs_key[i];
        unsigned long long k64 = akey(key);
        int a = hash_find(w, k64);
        int b1 = w.sinfo[key.x].y, b2 = w.sinfo[key.y].y;
        float4 m1 = w.mat[b1], m2 = w.mat[b2];
        if (a < 0) {
            a = atomicAdd(&w.ctr->narb, 1);
            if (a >= w.cap_arb) { atomicCAS(&w.ctr->status, 0, JG_ERR_CAPACITY); continue; }
            if (w.allow_deact) {  // HandleDeferredArbiters: AddToActiveList on both islands (World.Step.cs:880-914)
                atomicOr(&w.binfo[b1].w, 3);
                atomicOr(&w.binfo[b2].w, 3);
            }
            A.key[a] = key;
            A.body[a] = make_int2(b1, b2);
            A.mat[a] = make_float4(fmaxf(m1.x, m2.x), fmaxf(m1.y, m2.y), sp.spec_relax, 0.f);
            A.info[a] = make_int4(0, 0, -1, 1);
            int e = atomicAdd(&w.ctr->nnew, 1);
            if (e < w.cap_arb) ev_created[e] = key;
        }
        int4 info = A.info[a];
        float restitution = A.mat[a].y;
        int usage = info.x;
        if (!sp.persistent) usage = 0;
        // ContactData.ResetMode (Contact.cs:288-296)
        int mode = (w.binfo[b1].x == JG_MOTION_DYNAMIC ? 3 : 0) | (w.binfo[b2].x == JG_MOTION_DYNAMIC ? 12 : 0);
        float4 nc = w.cs_n[i];
        v3 n = mk3(nc);
        int cnt = __float_as_int(nc.w) & 0xff;
        // a speculative contact updates linear velocities only: ResetMode(SolveMode.Angular)
        // (World.Detect.cs:193-194)
        if (__float_as_int(nc.w) & JG_STREAM_SPECULATIVE) { mode &= ~(2 | 8); spec++; }
        // ResetMode before AddContact: Initialize reads the mode
        for (int k = 0; k < cnt; k++)
            add_contact(w, A, a, usage, b1, b2, mode, restitution, mk3(w.cs_pa[4 * i + k]), mk3(w.cs_pb[4 * i + k]), n, created_pts);
        A.info[a] = make_int4(usage, mode, info.z, info.w);
        contacts += __popc(usage & 15);
    }
    if (created_pts) atomicAdd(&w.ctr->new_contacts, created_pts);
    if (spec) atomicAdd(&w.ctr->nspec_hit, spec);
    (void)contacts;
}

// ---- colouring -----------------------------------------------------------------------------
__device__ __forceinline__ unsigned prio(unsigned long long key) { return hash64(key * 0x9E3779B97F4A7C15ull + 1); }

struct ColorCtx {
    int narb, nj, ncons;
};
__device__ __forceinline__ void cons_bodies(const WorldDev& w, const ArbStore& A, int c, int narb, int& b1, int& b2,
                                            unsigned long long& key) {
    if (c < narb) {
        int2 b = A.body[c];
        b1 = b.x; b2 = b.y;
        key = akey(A.key[c]);
    } else {
        int4 h = w.joints[c - narb].hdr;
        b1 = h.y; b2 = h.z;
        key = 0x8000000000000000ull | (unsigned long long)(c - narb);
    }
    if (w.binfo[b1].x != JG_MOTION_DYNAMIC) b1 = -1;
    if (w.binfo[b2].x != JG_MOTION_DYNAMIC) b2 = -1;
}

// Persistent cooperative kernel: adjacency build, Jones-Plassmann rounds, colour counts.
__global__ void k_color(WorldDev w, int* remaining) {
    const ArbStore& A = w.arb[w.cur];
    const int narb = w.ctr->narb < w.cap_arb ? w.ctr->narb : w.cap_arb;
    const int nj = w.nj;
    const int ncons = narb + nj;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    int* status = &w.ctr->status;
    __shared__ int s_warp[32];
    for (int b = tid; b < w.nb; b += nth) { w.deg[b] = 0; w.bmask[2 * b] = 0ull; w.bmask[2 * b + 1] = 0ull; }
    for (int c = tid; c < JG_MAX_COLORS + 1; c += nth) { w.color_count[c] = 0; w.color_cursor[c] = 0; }
    if (tid < 2) remaining[tid] = 0;
    if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
    const bool tasks = w.sc->ntasks > 0;
    for (int c = tid; c < ncons; c += nth) {
        if (c < narb && (A.info[c].x & 15) == 0) { w.cstat[c] = -2; continue; }
        if (c < narb && tasks && w.sc_dst[c] >= 0) { w.cstat[c] = -4; continue; }  // solved in a task
        int b1, b2; unsigned long long key;
        cons_bodies(w, A, c, narb, b1, b2, key);
        w.cstat[c] = -1;
        if (b1 >= 0) atomicAdd(&w.deg[b1], 1);
        if (b2 >= 0 && b2 != b1) atomicAdd(&w.deg[b2], 1);
    }
    if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
    // exclusive scan of deg -> adj_off: per-block chunk scan, then block offsets
    {
        int chunk = (w.nb + gridDim.x - 1) / gridDim.x;
        int lo = blockIdx.x * chunk, hi = min(w.nb, lo + chunk);
        // block-local scan of [lo, hi) in passes of blockDim
        int carry = 0;
        for (int base = lo; base < hi; base += blockDim.x) {
            int i = base + threadIdx.x;
            int v = i < hi ? w.deg[i] : 0;
            int x = v;
            for (int o = 1; o < 32; o <<= 1) { int y = __shfl_up_sync(0xffffffffu, x, o); if ((threadIdx.x & 31) >= o) x += y; }
            if ((threadIdx.x & 31) == 31) s_warp[threadIdx.x >> 5] = x;
            __syncthreads();
            if (threadIdx.x < 32) {
                int s = threadIdx.x < (int)(blockDim.x >> 5) ? s_warp[threadIdx.x] : 0;
                for (int o = 1; o < 32; o <<= 1) { int y = __shfl_up_sync(0xffffffffu, s, o); if ((int)threadIdx.x >= o) s += y; }
                s_warp[threadIdx.x] = s;
            }
            __syncthreads();
            int wp = (threadIdx.x >= 32) ? s_warp[(threadIdx.x >> 5) - 1] : 0;
            if (i < hi) w.adj_off[i] = carry + wp + x - v;
            int tot = s_warp[(blockDim.x >> 5) - 1];
            __syncthreads();
            carry += tot;
        }
        if (threadIdx.x == 0) w.hist[blockIdx.x] = carry;
    }
    if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int acc = 0;
        for (int b = 0; b < (int)gridDim.x; b++) { int t = w.hist[b]; w.hist[b] = acc; acc += t; }
        w.hist[gridDim.x] = acc;
    }
    if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
    {
        int chunk = (w.nb + gridDim.x - 1) / gridDim.x;
        int lo = blockIdx.x * chunk, hi = min(w.nb, lo + chunk);
        int off = w.hist[blockIdx.x];
        for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) { w.adj_off[i] += off; w.deg[i] = 0; }
        if (blockIdx.x == 0 && threadIdx.x == 0) w.adj_off[w.nb] = w.hist[gridDim.x];
    }
    if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
    for (int c = tid; c < ncons; c += nth) {
        if (w.cstat[c] < -1) continue;
        int b1, b2; unsigned long long key;
        cons_bodies(w, A, c, narb, b1, b2, key);
        if (b1 >= 0) { int s = atomicAdd(&w.deg[b1], 1); w.adj[w.adj_off[b1] + s] = c; }
        if (b2 >= 0 && b2 != b1) { int s = atomicAdd(&w.deg[b2], 1); w.adj[w.adj_off[b2] + s] = c; }
    }
    if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
    // Jones-Plassmann rounds; cstat = round * 256 + colour once coloured
    for (int round = 1; round < 4096; round++) {
        int left = 0;
        for (int c = tid; c < ncons; c += nth) {
            int st = w.cstat[c];
            if (st != -1) continue;
            int b1, b2; unsigned long long key;
            cons_bodies(w, A, c, narb, b1, b2, key);
            unsigned pc = prio(key);
            bool is_max = true;
            for (int side = 0; side < 2 && is_max; side++) {
                int b = side == 0 ? b1 : b2;
                if (b < 0) continue;
                int beg = w.adj_off[b], end = w.adj_off[b + 1];
                for (int e = beg; e < end; e++) {
                    int n = w.adj[e];
                    if (n == c) continue;
                    int sn = w.cstat[n];
                    bool unc = sn == -1 || (sn >= 0 && (sn >> 8) == round);
                    if (!unc) continue;
                    int nb1, nb2; unsigned long long nk;
                    cons_bodies(w, A, n, narb, nb1, nb2, nk);
                    unsigned pn = prio(nk);
                    if (pn > pc || (pn == pc && n > c)) { is_max = false; break; }
                }
            }
            if (!is_max) { left++; continue; }
            unsigned long long m0 = 0, m1 = 0;
            if (b1 >= 0) { m0 |= w.bmask[2 * b1]; m1 |= w.bmask[2 * b1 + 1]; }
            if (b2 >= 0) { m0 |= w.bmask[2 * b2]; m1 |= w.bmask[2 * b2 + 1]; }
            int color;
            if (~m0) color = __ffsll((long long)~m0) - 1;
            else if (~m1) color = 64 + __ffsll((long long)~m1) - 1;
            else { atomicCAS(status, 0, JG_ERR_CAPACITY); color = JG_MAX_COLORS - 1; }
            if (color >= JG_MAX_COLORS) { atomicCAS(status, 0, JG_ERR_CAPACITY); color = JG_MAX_COLORS - 1; }
            unsigned long long bit0 = color < 64 ? (1ull << color) : 0ull, bit1 = color >= 64 ? (1ull << (color - 64)) : 0ull;
            if (b1 >= 0) { if (bit0) atomicOr(&w.bmask[2 * b1], bit0); if (bit1) atomicOr(&w.bmask[2 * b1 + 1], bit1); }
            if (b2 >= 0) { if (bit0) atomicOr(&w.bmask[2 * b2], bit0); if (bit1) atomicOr(&w.bmask[2 * b2 + 1], bit1); }
            w.cstat[c] = round * 256 + color;
        }
        for (int o = 16; o > 0; o >>= 1) left += __shfl_xor_sync(0xffffffffu, left, o);
        if ((threadIdx.x & 31) == 0 && left) atomicAdd(&remaining[round & 1], left);
        if (tid == 0) remaining[(round + 1) & 1] = 0;
        if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
        int rem = ld_relaxed_int(&remaining[round & 1]);
        if (tid == 0) w.ctr->color_rounds = round;
        if (rem == 0) break;
        if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
    }
    for (int c = tid; c < ncons; c += nth) {
        int st = w.cstat[c];
        if (st < 0) continue;
        int col = st & 255;
        if (c < narb) atomicAdd(&w.color_count[col], 1);
        else atomicAdd(&w.color_cursor[col], 1);   // joint counts (cursor reset before use)
    }
    if (!grid_sync(w.bar_count, w.bar_gen, status)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int acc = tasks ? w.sc->narb_task : 0, jacc = 0, nc = 0;  // the remainder follows the tasks
        for (int c = 0; c < JG_MAX_COLORS; c++) {
            int t = w.color_count[c], jt = w.color_cursor[c];
            if (t || jt) nc = c + 1;
            w.color_start[c] = acc; acc += t;
            w.jcolor_start[c] = jacc; jacc += jt;
        }
        w.color_start[JG_MAX_COLORS] = acc;
        w.jcolor_start[JG_MAX_COLORS] = jacc;
        for (int c = nc; c < JG_MAX_COLORS; c++) { w.color_start[c] = acc; w.jcolor_start[c] = jacc; }
        w.ctr->ncolors = nc;
        for (int c = 0; c <= JG_MAX_COLORS; c++) w.color_cursor[c] = 0;
    }
}

// Moves every arbiter with contacts to the other buffer at its colour slot.
__global__ void k_permute(WorldDev w, int2* ev_removed, int* dst_index) {
    const ArbStore& S = w.arb[w.cur];
    const ArbStore& D = w.arb[1 - w.cur];
    const int narb = w.ctr->narb < w.cap_arb ? w.ctr->narb : w.cap_arb;
    const int cap = w.cap_arb;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < narb; a += gridDim.x * blockDim.x) {
        int st = w.cstat[a];
        int d, key;
        int4 ls;
        if (st == -4) {  // task arbiter: slot, order key and body slots from the schedule
            d = w.sc_dst[a];
            key = w.sc_lcol[a];
            ls = w.sc_ls[a];
        } else if (st < 0) {
            int e = atomicAdd(&w.ctr->nremoved, 1);
            if (e < cap) ev_removed[e] = S.key[a];
            dst_index[a] = -1;
            if (w.allow_deact) {  // RemoveBrokenArbiters: AddToActiveList on both islands (World.Step.cs:845-846)
                int2 bb = S.body[a];
                atomicOr(&w.binfo[bb.x].w, 3);
                atomicOr(&w.binfo[bb.y].w, 3);
            }
            continue;
        } else {
            int col = st & 255;
            d = w.color_start[col] + atomicAdd(&w.color_cursor[col], 1);
            key = JG_ORDER_REMAINDER + col;
            ls = make_int4(-1, -1, 3, 0);
        }
        dst_index[a] = d;
        int4 info = S.info[a];
        int2 bb = S.body[a];
        // a row is solved and updated while one of its bodies is an awake non-static body
        // (memContacts activation follows the bodies, World.Step.cs:1247-1275, :1325-1345)
        bool asleep = false;
        if (w.allow_deact) {
            int4 i1 = w.binfo[bb.x], i2 = w.binfo[bb.y];
            asleep = !((i1.x != JG_MOTION_STATIC && (i1.y & JG_BODY_ACTIVE)) || (i2.x != JG_MOTION_STATIC && (i2.y & JG_BODY_ACTIVE)));
        }
        D.key[d] = S.key[a];
        D.body[d] = bb;
        D.info[d] = make_int4(info.x, (info.y & 0xffff) | (asleep ? JG_ARB_ASLEEP : 0), key, info.w);
        // velocities of a non-dynamic body stay constant through the solve
        int nd = w.binfo[bb.x].x != JG_MOTION_DYNAMIC ? bb.x : (w.binfo[bb.y].x != JG_MOTION_DYNAMIC ? bb.y : -1);
        // task arbiters: what the iterations read besides the rows, in one record
        if (st == -4) ls = make_int4(ls.x, ls.y, (info.x & 15) | ((info.y & 15) << 4) | (nd >= 0 ? 256 : 0) | (asleep ? JG_TASK_ASLEEP : 0),
                                     __float_as_int(S.mat[a].x));
        D.lslot[d] = ls;
        D.sv[d] = nd >= 0 ? w.body[nd].v : make_float4(0.f, 0.f, 0.f, 0.f);
        D.sv[cap + d] = nd >= 0 ? w.body[nd].w : make_float4(0.f, 0.f, 0.f, 0.f);
        D.mat[d] = S.mat[a];
        for (int k = 0; k < 4; k++) {
            if (!(info.x & (1 << k))) continue;
            int s = k * cap + a, t = k * cap + d;
            D.cn[t] = S.cn[s]; D.ct1[t] = S.ct1[s]; D.ct2[t] = S.ct2[s]; D.cr1[t] = S.cr1[s];
            D.cr2[t] = S.cr2[s]; D.cacc[t] = S.cacc[s]; D.cp1[t] = S.cp1[s]; D.cp2[t] = S.cp2[s];
        }
    }
    const int nj = w.nj;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nj; j += gridDim.x * blockDim.x) {
        int st = w.cstat[narb + j];
        int col = st >= 0 ? (st & 255) : 0;
        int d = w.jcolor_start[col] + atomicAdd(&w.jorder[w.cap_joints + col], 1);
        w.jorder[d] = j;
        w.joints[j].hdr.w = JG_ORDER_REMAINDER + col;
    }
}

__global__ void k_permute_done(WorldDev w) {
    w.ctr->narb = w.color_start[JG_MAX_COLORS];
}

__global__ void k_count_contacts(WorldDev w) {
    const ArbStore& A = w.arb[w.cur];
    int n = w.ctr->narb;
    int c = 0;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) c += __popc(A.info[a].x & 15);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&w.ctr->contacts, c);
}

__global__ void k_jcursor_clear(WorldDev w) {
    for (int c = threadIdx.x; c < JG_MAX_COLORS; c += blockDim.x) w.jorder[w.cap_joints + c] = 0;
}

// ContactData.UpdatePosition (Contact.cs:238-264) / Contact.UpdatePosition (Contact.cs:762-797)
__global__ void k_update_contacts(WorldDev w) {
    const ArbStore& A = w.arb[w.cur];
    const int n = w.ctr->narb, cap = w.cap_arb;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
        int4 info = A.info[a];
        if (info.y & JG_ARB_ASLEEP) continue;  // sleeping contacts keep their points
        int usage = info.x & 15;
        usage |= usage << 4;
        int2 b = A.body[a];
        v3 pos1 = mk3(w.pos[b.x]), pos2 = mk3(w.pos[b.y]);
        q4 q1 = mkq(w.q[b.x]), q2 = mkq(w.q[b.y]);
        for (int k = 0; k < 4; k++) {
            if (!(usage & (1 << k))) continue;
            int i = k * cap + a;
            v3 rel1 = rotate(mk3(A.cp1[i]), q1);
            v3 p1 = rel1 + pos1;
            v3 rel2 = rotate(mk3(A.cp2[i]), q2);
            v3 p2 = rel2 + pos2;
            float4 r1 = A.cr1[i], r2 = A.cr2[i];
            A.cr1[i] = f4(rel1, r1.w);
            A.cr2[i] = f4(rel2, r2.w);
            v3 dist = p1 - p2;
            v3 nrm = mk3(A.cn[i]);
            float pen = dot(dist, nrm);
            bool keep = true;
            if (pen < -BreakThreshold * 0.1f) keep = false;
            else {
                dist = dist - pen * nrm;
                if (len2(dist) > BreakThreshold * BreakThreshold) keep = false;
            }
            if (!keep) usage &= ~(1 << k);
        }
        A.info[a] = make_int4(usage, info.y, info.z, 0);
    }
}

}  // namespace

void jg_launch_merge(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm) {
    int blocks = nsm * 4;
    k_hash_clear<<<blocks, 256, 0, s>>>(w);
    k_hash_build<<<blocks, 256, 0, s>>>(w);
    k_merge<<<blocks, 128, 0, s>>>(w, p, w.ev_created);
}

// Returns 0, or -1 when the cooperative colouring launch is refused.
int jg_launch_color(WorldDev& w, cudaStream_t s, int nsm) {
    if (w.lc_color_grid == 0) {
        int occ = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_color, 256, 0);
        if (occ < 1) occ = 1;
        w.lc_color_grid = nsm * (occ < 2 ? occ : 2);
    }
    cudaMemsetAsync(w.bar_count, 0, sizeof(unsigned) * 2, s);
    int* rem = w.remaining;
    void* args[] = {(void*)&w, (void*)&rem};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_color, dim3(w.lc_color_grid), dim3(256), args, 0, s);
    if (e != cudaSuccess) return -1;
    k_jcursor_clear<<<1, 128, 0, s>>>(w);
    k_permute<<<nsm * 4, 256, 0, s>>>(w, w.ev_removed, w.dst_index);
    k_permute_done<<<1, 1, 0, s>>>(w);
    return 0;
}

void jg_flip_store(WorldDev& w) { w.cur = 1 - w.cur; }

void jg_launch_count_contacts(WorldDev& w, cudaStream_t s, int nsm) {
    k_count_contacts<<<nsm * 2, 256, 0, s>>>(w);
}

void jg_launch_update_contacts(WorldDev& w, cudaStream_t s, int nsm) {
    k_update_contacts<<<nsm * 4, 256, 0, s>>>(w);
}
