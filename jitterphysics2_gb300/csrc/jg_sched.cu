// Schedule of the partitioned solve, rebuilt every step after the arbiter merge.
//
// The reference solves contacts in one sequential (Deterministic mode) or lock-batched
// (Regular mode) Gauss-Seidel sweep per iteration (World.Step.cs:1135-1191,
// World.Deterministic.cs:250-334).  Any order in which no two rows touching the same
// dynamic body run at once is one of those sequential orders.  This schedule builds one
// with few grid-wide synchronisations:
//   1. three staggered column grids in x-z with cell size h > 3 x the largest horizontal
//      distance between two dynamic bodies sharing an arbiter (offsets 0, h/3, 2h/3): an
//      arbiter lies inside a cell of grid 0, else of grid 1, else of grid 2 (batched
//      worlds use one cell per world, all in grid 0).  Above that bound h gives about
//      cells_per_sm cells per grid and SM (by default the narrowest cells when there are
//      no more of them than solve blocks, else as many as make about 250 arbiters a cell):
//      narrow columns keep the longest task short, which bounds every pass, at the price of
//      more tasks, each with a fixed latency;
//   2. each non-empty cell of a grid is a task: its arbiters and the dynamic bodies they
//      touch, which no other task of the same grid touches;
//   3. inside a task, arbiters get local colours (Jones-Plassmann in shared memory) and
//      are ordered by colour; the solver runs a task in one CTA with the bodies in shared
//      memory and a block barrier between colours, and the three grids one after another
//      (without a remainder a task waits only for the tasks of the two previous grid
//      phases that may share its bodies; their list is built here);
//   4. arbiters of cells too large for shared memory form the remainder, coloured
//      globally and solved as before.
// The resulting order key of an arbiter (grid * 256 + local colour, or 768 + global
// colour) describes a sequential order the oracle can replay.
#include "jg_sync.cuh"

namespace {

__device__ __forceinline__ unsigned f2ord(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}
__device__ __forceinline__ bool dyn(const WorldDev& w, int b) { return w.binfo[b].x == JG_MOTION_DYNAMIC; }

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

__global__ void k_sched_reset(WorldDev w) {
    SchedInfo* S = w.sc;
    S->span_bits = 0;
    S->bbox[0] = S->bbox[1] = 0xffffffffu;
    S->bbox[2] = S->bbox[3] = 0u;
    S->tag += 1;
    S->ntasks = 0; S->narb_task = 0; S->overflow = 0; S->maxc = 0;
    for (int g = 0; g < JG_SCHED_GRIDS; g++) { S->ntask[g] = 0; S->task_base[g] = 0; }
}

// Bounds of the dynamic bodies and the largest horizontal span of a two-dynamic arbiter.
__global__ void k_sched_bounds(WorldDev w) {
    const ArbStore& A = w.arb[w.cur];
    const int narb = min(w.ctr->narb, w.cap_arb);
    unsigned mnx = 0xffffffffu, mnz = 0xffffffffu, mxx = 0u, mxz = 0u, span = 0u;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    for (int i = tid; i < w.nb; i += nth) {
        if (!dyn(w, i)) continue;
        float4 p = w.pos[i];
        if (!isfinite(p.x) || !isfinite(p.z)) continue;
        unsigned ox = f2ord(p.x), oz = f2ord(p.z);
        mnx = min(mnx, ox); mxx = max(mxx, ox);
        mnz = min(mnz, oz); mxz = max(mxz, oz);
    }
    for (int a = tid; a < narb; a += nth) {
        if ((A.info[a].x & 15) == 0) continue;
        int2 b = A.body[a];
        if (!dyn(w, b.x) || !dyn(w, b.y)) continue;
        float4 p1 = w.pos[b.x], p2 = w.pos[b.y];
        float d = fmaxf(fabsf(p1.x - p2.x), fabsf(p1.z - p2.z));
        if (isfinite(d)) span = max(span, __float_as_uint(d));
    }
    mnx = __reduce_min_sync(0xffffffffu, mnx); mnz = __reduce_min_sync(0xffffffffu, mnz);
    mxx = __reduce_max_sync(0xffffffffu, mxx); mxz = __reduce_max_sync(0xffffffffu, mxz);
    span = __reduce_max_sync(0xffffffffu, span);
    if ((threadIdx.x & 31) == 0) {
        SchedInfo* S = w.sc;
        if (mnx != 0xffffffffu) {
            atomicMin(&S->bbox[0], mnx); atomicMin(&S->bbox[1], mnz);
            atomicMax(&S->bbox[2], mxx); atomicMax(&S->bbox[3], mxz);
        }
        if (span) atomicMax(&S->span_bits, span);
    }
}

// Cell size and grid extent (one thread).
__global__ void k_sched_setup(WorldDev w, int nsm, float cells_per_sm, int blocks) {
    SchedInfo* S = w.sc;
    if (w.nworlds > 1) {
        S->h = 0.f; S->x0 = S->z0 = 0.f; S->ncx = S->ncz = 1; S->ncells = min(w.nworlds, JG_SCHED_MAXCELLS);
        return;
    }
    if (S->bbox[0] == 0xffffffffu) { S->ncells = 0; S->ncx = S->ncz = 0; S->h = 1.f; return; }
    float xmin = ord2f(S->bbox[0]), zmin = ord2f(S->bbox[1]), xmax = ord2f(S->bbox[2]), zmax = ord2f(S->bbox[3]);
    float ex = xmax - xmin, ez = zmax - zmin;
    float span = __uint_as_float(S->span_bits);
    const float h_min = 3.0f * span * 1.001f + 1e-4f;
    float h;
    if (cells_per_sm > 0.f) {
        h = fmaxf(h_min, sqrtf(ex * ez / (cells_per_sm * (float)nsm)));
    } else if ((floorf(ex / h_min) + 3.0f) * (floorf(ez / h_min) + 3.0f) <= (float)blocks) {
        h = h_min;  // the narrowest cells still give each solve block at most one task per grid
    } else {
        // more cells than blocks: about JG_SCHED_CELL_ARBITERS arbiters per cell on average,
        // so that dense piles get narrow columns (their longest task bounds a pass) and
        // sparse scenes few tasks per block (each task costs a fixed latency)
        const float c = fminf(fmaxf((float)min(w.ctr->narb, w.cap_arb) / (JG_SCHED_CELL_ARBITERS * (float)nsm), 0.5f), 16.f);
        h = fmaxf(h_min, sqrtf(ex * ez / (c * (float)nsm)));
    }
    h = fmaxf(h, 1e-3f);
    float fx = 0.f, fz = 0.f;
    for (int k = 0; k < 256; k++) {
        fx = floorf(ex / h) + 3.0f;
        fz = floorf(ez / h) + 3.0f;
        if (fx * fz <= (float)JG_SCHED_MAXCELLS) break;
        h *= 2.0f;
    }
    S->h = h; S->x0 = xmin - h; S->z0 = zmin - h;
    S->ncx = (int)fx; S->ncz = (int)fz; S->ncells = S->ncx * S->ncz;
}

// Grid g is offset by g/3 of a cell in x and z.  An arbiter whose bodies are less than
// h/3 apart crosses the x planes of at most one grid and the z planes of at most one
// grid, so it lies inside a cell of the third.
__device__ __forceinline__ int cell_of(const SchedInfo& S, float x, float z, int g) {
    const float off = g == 0 ? 0.f : (g == 1 ? (1.0f / 3.0f) : (2.0f / 3.0f));
    int ix = (int)floorf((x - S.x0) / S.h + off);
    int iz = (int)floorf((z - S.z0) / S.h + off);
    ix = min(max(ix, 0), S.ncx - 1);
    iz = min(max(iz, 0), S.ncz - 1);
    return iz * S.ncx + ix;
}

// Cell of each dynamic body per grid; clears the per-cell counters.
__global__ void k_sched_cells(WorldDev w) {
    const SchedInfo S = *w.sc;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int cb = w.cap_bodies;
    for (int i = tid; i < JG_SCHED_GRIDS * S.ncells; i += nth) {
        int g = i / S.ncells, c = i - g * S.ncells;
        w.sc_acount[g * JG_SCHED_MAXCELLS + c] = 0;
        w.sc_bcount[g * JG_SCHED_MAXCELLS + c] = 0;
    }
    for (int i = tid; i < w.nb; i += nth) {
        int c0 = -1, c1 = -1, c2 = -1;
        if (dyn(w, i) && S.ncells > 0) {
            if (w.nworlds > 1) {
                c0 = min(w.binfo[i].z, S.ncells - 1);
            } else {
                float4 p = w.pos[i];
                if (isfinite(p.x) && isfinite(p.z)) {
                    c0 = cell_of(S, p.x, p.z, 0); c1 = cell_of(S, p.x, p.z, 1); c2 = cell_of(S, p.x, p.z, 2);
                }
            }
        }
        w.sc_cell[i] = c0; w.sc_cell[cb + i] = c1; w.sc_cell[2 * cb + i] = c2;
    }
}

// Grid and cell of each arbiter; arbiter counts per cell; each cell claims slots for the
// dynamic bodies its arbiters touch.
__global__ void k_sched_assign(WorldDev w) {
    const ArbStore& A = w.arb[w.cur];
    const int narb = min(w.ctr->narb, w.cap_arb);
    const int cb = w.cap_bodies;
    const int tag = w.sc->tag;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < narb; a += gridDim.x * blockDim.x) {
        w.sc_dst[a] = -1;
        if ((A.info[a].x & 15) == 0) { w.sc_arb[a] = make_int2(-1, -1); continue; }
        int2 b = A.body[a];
        bool d1 = dyn(w, b.x), d2 = dyn(w, b.y);
        int g = 3, cell = -1;
        for (int k = 0; k < JG_SCHED_GRIDS; k++) {
            int c1 = d1 ? w.sc_cell[k * cb + b.x] : -1, c2 = d2 ? w.sc_cell[k * cb + b.y] : -1;
            if (c1 < 0 && c2 < 0) continue;
            if ((d1 && c1 < 0) || (d2 && c2 < 0)) continue;
            if (c1 < 0 || c2 < 0 || c1 == c2) { g = k; cell = c1 >= 0 ? c1 : c2; break; }
        }
        w.sc_arb[a] = make_int2(g, cell);
        if (g >= JG_SCHED_GRIDS) continue;
        atomicAdd(&w.sc_acount[g * JG_SCHED_MAXCELLS + cell], 1);
        for (int side = 0; side < 2; side++) {
            int body = side == 0 ? b.x : b.y;
            if (!(side == 0 ? d1 : d2)) continue;
            if (atomicExch(&w.sc_stamp[g * cb + body], tag) != tag)
                w.sc_bslot[g * cb + body] = atomicAdd(&w.sc_bcount[g * JG_SCHED_MAXCELLS + cell], 1);
        }
    }
}

// Exclusive block scan of two ints (1024 threads).
__device__ __forceinline__ int2 block_scan2(int2 v, int2& total) {
    __shared__ int2 s_w[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int2 x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int yx = __shfl_up_sync(0xffffffffu, x.x, o), yy = __shfl_up_sync(0xffffffffu, x.y, o);
        if (lane >= o) { x.x += yx; x.y += yy; }
    }
    if (lane == 31) s_w[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int2 s = lane < (int)(blockDim.x >> 5) ? s_w[lane] : make_int2(0, 0);
        for (int o = 1; o < 32; o <<= 1) {
            int yx = __shfl_up_sync(0xffffffffu, s.x, o), yy = __shfl_up_sync(0xffffffffu, s.y, o);
            if (lane >= o) { s.x += yx; s.y += yy; }
        }
        s_w[lane] = s;
    }
    __syncthreads();
    int2 pre = wid > 0 ? s_w[wid - 1] : make_int2(0, 0);
    total = s_w[(blockDim.x >> 5) - 1];
    __syncthreads();
    return make_int2(pre.x + x.x - v.x, pre.y + x.y - v.y);
}

// Tasks: the non-empty cells of each grid that fit a CTA, with arbiter and body offsets
// (one block of 1024 threads).
__global__ void __launch_bounds__(1024) k_sched_tasks(WorldDev w, StepParams sp) {
    SchedInfo* S = w.sc;
    const int ncells = S->ncells;
    int t = 0, aoff = 0, boff = 0, over = 0;
    for (int g = 0; g < JG_SCHED_GRIDS; g++) {
        if (threadIdx.x == 0) S->task_base[g] = t;
        for (int base = 0; base < ncells; base += blockDim.x) {
            int cell = base + threadIdx.x;
            int ac = 0, bc = 0;
            if (cell < ncells) { ac = w.sc_acount[g * JG_SCHED_MAXCELLS + cell]; bc = w.sc_bcount[g * JG_SCHED_MAXCELLS + cell]; }
            bool ok = ac > 0 && ac <= JG_TASK_MAXA && bc <= sp.task_maxb && sp.partition;
            int2 tot;
            int2 idx = block_scan2(make_int2(ok ? 1 : 0, 0), tot);
            bool ok2 = ok && t + idx.x < JG_SCHED_MAXTASKS;
            int2 offs = block_scan2(make_int2(ok2 ? ac : 0, ok2 ? bc : 0), tot);
            if (cell < ncells) {
                w.sc_task_of[g * JG_SCHED_MAXCELLS + cell] = ok2 ? t + idx.x : -1;
                if (ok2) {
                    w.sc_task[t + idx.x] = make_int4(aoff + offs.x, ac, boff + offs.y, bc);
                    w.sc_cursor[t + idx.x] = 0;
                    w.sc_tcell[t + idx.x] = cell;
                    w.sc_done[t + idx.x] = 0u;
                }
            }
            over += __syncthreads_count(ac > 0 && !ok2);
            int2 nt;
            block_scan2(make_int2(ok2 ? 1 : 0, 0), nt);
            t += nt.x; aoff += tot.x; boff += tot.y;
        }
        if (threadIdx.x == 0) S->ntask[g] = t - S->task_base[g];
    }
    if (threadIdx.x == 0) {
        S->ntasks = t; S->narb_task = aoff; S->overflow = over;
        w.ctr->ntasks = t; w.ctr->narb_task = aoff;
    }
}

// Task arbiter and body lists; arbiters of cells without a task join the remainder.
__global__ void k_sched_scatter(WorldDev w) {
    const int narb = min(w.ctr->narb, w.cap_arb);
    const int cb = w.cap_bodies;
    const int tag = w.sc->tag;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    for (int a = tid; a < narb; a += nth) {
        int2 ga = w.sc_arb[a];
        if (ga.x < 0 || ga.x >= JG_SCHED_GRIDS) continue;
        int t = w.sc_task_of[ga.x * JG_SCHED_MAXCELLS + ga.y];
        if (t < 0) { w.sc_arb[a] = make_int2(3, -1); continue; }
        int p = atomicAdd(&w.sc_cursor[t], 1);
        w.sc_tlist[w.sc_task[t].x + p] = a;
    }
    // Dependencies of each task on the two grid phases before it (grids g - 1 and g - 2,
    // wrapping to the previous pass): the tasks of those grids that may share a body with
    // it.  A body in cell ix of grid g (offset g/3) lies in cell ix - 1 or ix of a grid with
    // a smaller offset and in ix or ix + 1 of one with a larger offset, in each axis, so at
    // most four tasks per grid.  Both grids are needed: a body's cell in the phase just
    // before may hold no task, and then only the direct wait orders the accesses.
    const SchedInfo& S = *w.sc;
    for (int t = tid; t < S.ntasks; t += nth) {
        int g = 0;
        while (g + 1 < JG_SCHED_GRIDS && t >= S.task_base[g + 1]) g++;
        for (int back = 1; back <= 2; back++) {
            int4 dep = make_int4(-1, -1, -1, -1);
            if (w.nworlds <= 1) {
                const int gp = (g + JG_SCHED_GRIDS - back) % JG_SCHED_GRIDS;
                const int c = w.sc_tcell[t], ix = c % S.ncx, iz = c / S.ncx;
                const int d0 = gp > g ? 0 : -1;
                int k = 0;
                for (int dz = d0; dz <= d0 + 1; dz++)
                    for (int dx = d0; dx <= d0 + 1; dx++) {
                        const int jx = min(max(ix + dx, 0), S.ncx - 1), jz = min(max(iz + dz, 0), S.ncz - 1);
                        const int n = w.sc_task_of[gp * JG_SCHED_MAXCELLS + jz * S.ncx + jx];
                        if (n < 0 || n == dep.x || n == dep.y || n == dep.z) continue;
                        (&dep.x)[k++] = n;
                    }
            }
            w.sc_tdep[2 * t + back - 1] = dep;
        }
    }
    for (int b = tid; b < w.nb; b += nth) {
        for (int g = 0; g < JG_SCHED_GRIDS; g++) {
            if (w.sc_stamp[g * cb + b] != tag) continue;
            int cell = w.sc_cell[g * cb + b];
            if (cell < 0) continue;
            int t = w.sc_task_of[g * JG_SCHED_MAXCELLS + cell];
            if (t < 0) continue;
            w.sc_tbody[w.sc_task[t].z + w.sc_bslot[g * cb + b]] = b;
        }
    }
}

// Local Jones-Plassmann colouring of each task in shared memory (one CTA per task at a
// time): in each round every uncoloured arbiter that holds the highest priority on all of
// its task bodies takes the smallest colour free on them.  Then the task's arbiters are
// placed by colour: final slot, local colour and body slots per arbiter.
constexpr int TC_THREADS = 256;
__global__ void __launch_bounds__(TC_THREADS) k_task_color(WorldDev w, StepParams sp) {
    extern __shared__ unsigned long long tc_smem[];
    const int maxb = sp.task_maxb;
    unsigned long long* s_mask = tc_smem;                          // [maxb]
    unsigned long long* s_own = s_mask + maxb;                      // [maxb]
    int* s_deg = (int*)(s_own + maxb);                              // [maxb] arbiters per body
    int* s_l1 = s_deg + ((maxb + 1) & ~1);                          // [MAXA]
    int* s_l2 = s_l1 + JG_TASK_MAXA;                                // [MAXA]
    int* s_a = s_l2 + JG_TASK_MAXA;                                 // [MAXA]
    unsigned char* s_col = (unsigned char*)(s_a + JG_TASK_MAXA);    // [MAXA]
    __shared__ int s_cnt[JG_TASK_MAXC + 1], s_cur[4 * JG_TASK_MAXC];
    const ArbStore& A = w.arb[w.cur];
    const SchedInfo* S = w.sc;
    const int cb = w.cap_bodies;
    const int ntasks = S->ntasks;
    for (int t = blockIdx.x; t < ntasks; t += gridDim.x) {
        const int4 T = w.sc_task[t];
        const int n = T.y, nb = T.w;
        const int g = t >= S->task_base[2] && S->ntask[2] ? 2 : (t >= S->task_base[1] && S->ntask[1] ? 1 : 0);
        for (int i = threadIdx.x; i < nb; i += blockDim.x) { s_mask[i] = 0ull; s_own[i] = 0ull; s_deg[i] = 0; }
        for (int i = threadIdx.x; i <= JG_TASK_MAXC; i += blockDim.x) s_cnt[i] = 0;
        for (int i = threadIdx.x; i < 4 * JG_TASK_MAXC; i += blockDim.x) s_cur[i] = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            int a = w.sc_tlist[T.x + i];
            int2 b = A.body[a];
            s_a[i] = a;
            int l1 = dyn(w, b.x) ? w.sc_bslot[g * cb + b.x] : -1;
            int l2 = dyn(w, b.y) ? w.sc_bslot[g * cb + b.y] : -1;
            s_l1[i] = l1;
            s_l2[i] = l2;
            s_col[i] = 0xff;
            if (l1 >= 0) atomicAdd(&s_deg[l1], 1);
            if (l2 >= 0) atomicAdd(&s_deg[l2], 1);
        }
        __syncthreads();
        // priorities, largest degree first (an arbiter's degree: the arbiters sharing one of
        // its bodies), then a hash of the arbiter key (deterministic), then the list position
        auto prio = [&](int i) -> unsigned long long {
            int l1 = s_l1[i], l2 = s_l2[i];
            unsigned long long deg = (unsigned long long)min((l1 >= 0 ? s_deg[l1] : 0) + (l2 >= 0 ? s_deg[l2] : 0), 8191);
            int2 key = A.key[s_a[i]];
            unsigned long long h = mix64(((unsigned long long)(unsigned)key.x << 32) | (unsigned)key.y) & ((1ull << 37) - 1);
            return (1ull << 63) | (deg << 50) | (h << 13) | (unsigned long long)i;
        };
        unsigned todo = 0;  // bit k: element threadIdx.x + k * blockDim.x still uncoloured
        for (int k = 0; k * (int)blockDim.x + (int)threadIdx.x < n; k++) todo |= 1u << k;
        // every round colours at least the highest-priority uncoloured arbiter, so n rounds
        // always suffice (n <= JG_TASK_MAXA)
        int left = n;
        for (int round = 0; round <= JG_TASK_MAXA && left > 0; round++) {
            for (unsigned m = todo; m; m &= m - 1) {
                int i = __ffs(m) - 1;
                i = threadIdx.x + i * blockDim.x;
                unsigned long long p = prio(i);
                if (s_l1[i] >= 0) atomicMax(&s_own[s_l1[i]], p);
                if (s_l2[i] >= 0) atomicMax(&s_own[s_l2[i]], p);
            }
            __syncthreads();
            unsigned won = 0;
            for (unsigned m = todo; m; m &= m - 1) {
                int k = __ffs(m) - 1;
                int i = threadIdx.x + k * blockDim.x;
                unsigned long long p = prio(i);
                int l1 = s_l1[i], l2 = s_l2[i];
                if ((l1 < 0 || s_own[l1] == p) && (l2 < 0 || s_own[l2] == p)) won |= 1u << k;
            }
            __syncthreads();
            for (unsigned m = todo; m; m &= m - 1) {
                int k = __ffs(m) - 1;
                int i = threadIdx.x + k * blockDim.x;
                int l1 = s_l1[i], l2 = s_l2[i];
                if (won & (1u << k)) {
                    unsigned long long used = (l1 >= 0 ? s_mask[l1] : 0ull) | (l2 >= 0 ? s_mask[l2] : 0ull);
                    int c = ~used ? __ffsll((long long)~used) - 1 : JG_TASK_MAXC - 1;
                    if (!~used) atomicCAS(&w.ctr->status, 0, JG_ERR_CAPACITY);
                    s_col[i] = (unsigned char)c;
                    if (l1 >= 0) s_mask[l1] |= 1ull << c;
                    if (l2 >= 0) s_mask[l2] |= 1ull << c;
                }
                if (l1 >= 0) s_own[l1] = 0ull;
                if (l2 >= 0) s_own[l2] = 0ull;
            }
            todo &= ~won;
            left = __syncthreads_count(todo != 0) ? 1 : 0;
        }
        // colour counts, offsets, placement.  Inside a colour the arbiters with more
        // contacts come first, so that the lanes of a warp mostly run the same number of
        // contact rows (any order inside a colour is the same solve).
        auto bucket = [&](int i) {
            int pc = __popc(A.info[s_a[i]].x & 15);
            return 4 * s_col[i] + (pc >= 4 ? 0 : (pc <= 1 ? 3 : 4 - pc));
        };
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            if (s_col[i] >= JG_TASK_MAXC) { s_col[i] = JG_TASK_MAXC - 1; atomicCAS(&w.ctr->status, 0, JG_ERR_CAPACITY); }
            atomicAdd(&s_cnt[s_col[i]], 1);
            atomicAdd(&s_cur[bucket(i)], 1);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0, nc = 0;
            for (int c = 0; c < JG_TASK_MAXC; c++) {
                if (s_cnt[c]) nc = c + 1;
                w.sc_tcol[t * (JG_TASK_MAXC + 1) + c] = acc;
                for (int q = 0; q < 4; q++) {
                    int kq = s_cur[4 * c + q];
                    s_cur[4 * c + q] = acc;
                    acc += kq;
                }
            }
            w.sc_tcol[t * (JG_TASK_MAXC + 1) + JG_TASK_MAXC] = acc;
            for (int c = nc; c <= JG_TASK_MAXC; c++) w.sc_tcol[t * (JG_TASK_MAXC + 1) + c] = acc;
            w.sc_tnc[t] = nc;
            atomicMax(&w.sc->maxc, nc);
            atomicMax(&w.ctr->task_colors, nc);
        }
        __syncthreads();
        // body slots packed with the arbiter's rank among its body's arbiters in colour
        // order (the colours a body's arbiters take are distinct, so the rank is the number
        // of the body's colours below this one): slot | rank << 16, -1 for a non-dynamic body
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            int c = s_col[i];
            int p = atomicAdd(&s_cur[bucket(i)], 1);
            int a = s_a[i];
            const unsigned long long below = (1ull << c) - 1ull;
            int l1 = s_l1[i], l2 = s_l2[i];
            int p1 = l1 >= 0 ? (l1 | __popcll(s_mask[l1] & below) << 16) : -1;
            int p2 = l2 >= 0 ? (l2 | __popcll(s_mask[l2] & below) << 16) : -1;
            w.sc_dst[a] = T.x + p;
            w.sc_lcol[a] = g * 256 + c;
            w.sc_ls[a] = make_int4(p1, p2, g, 0);
        }
        __syncthreads();
    }
}

}  // namespace

size_t jg_task_color_smem(int maxb) {
    return (size_t)maxb * 16 + (size_t)((maxb + 1) & ~1) * 4 + (size_t)JG_TASK_MAXA * 13;
}

void jg_launch_schedule(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm) {
    k_sched_reset<<<1, 1, 0, s>>>(w);
    if (p.partition) {
        k_sched_bounds<<<nsm * 4, 256, 0, s>>>(w);
        k_sched_setup<<<1, 1, 0, s>>>(w, nsm, p.cells_per_sm, p.solve_blocks);
        k_sched_cells<<<nsm * 4, 256, 0, s>>>(w);
        k_sched_assign<<<nsm * 4, 256, 0, s>>>(w);
        k_sched_tasks<<<1, 1024, 0, s>>>(w, p);
        k_sched_scatter<<<nsm * 4, 256, 0, s>>>(w);
        size_t smem = jg_task_color_smem(p.task_maxb);
        k_task_color<<<nsm * 2, TC_THREADS, smem, s>>>(w, p);
    }
}

// Lets the local colouring take all the dynamic shared memory the current device allows,
// once per device (called when a world is created).
int jg_schedule_init() {
    int dev = 0, pb = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&pb, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, (const void*)k_task_color) != cudaSuccess) return -1;
    return cudaFuncSetAttribute(k_task_color, cudaFuncAttributeMaxDynamicSharedMemorySize, pb - (int)fa.sharedSizeBytes)
               == cudaSuccess ? 0 : -1;
}

// Kernels launched by jg_launch_schedule.
int jg_schedule_launches(const StepParams& p) { return p.partition ? 8 : 1; }
