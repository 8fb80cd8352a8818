// Device-resident world state of the GB300 contact pipeline and the launch entry points
// of each stage.  Layout (all SoA or 64-byte records, 16-byte aligned):
//   bodies    SBody[nb]      64 B solver record: v|invM.x, w|invM.y, I^-1 world (6), invM.z, flags
//             pos/q/dv/dw/...  float4 per body, read by integration and the per-step update
//   shapes    int4 info + float4 dims/centre, hull vertices float4, triangles TriDev
//   arbiters  ArbStore (double-buffered): key, bodies, usage/mode/colour, material, and
//             8 float4 fields per contact slot stored as [slot * capacity + arbiter]
//   joints    JointDev records (BallSocket / HingeAngle)
// Arbiters are kept sorted by solver colour: the colouring stage permutes them into the
// other buffer, so each colour is a contiguous, coalesced range during the solve.
#pragma once
#include "jg_math.cuh"
#include "../../include/jitter_gpu.h"

#define JG_MAX_COLORS 128
#define JG_RESID_MAX 2048       // iterations whose residual a step records (record_residual)
#define JG_HULL_MAX 64          // point-cloud vertices per shape handled on the device
#define JG_EPA_MAXV 128         // EPA polytope capacity (ConvexPolytope.cs:53-54)
#define JG_EPA_MAXT 256

struct __align__(16) SBody {
    float4 v;   // velocity xyz, inverse mass x
    float4 w;   // angular velocity xyz, inverse mass y
    float4 i0;  // world inverse inertia M11 M12 M13 M22
    float4 i1;  // M23 M33, inverse mass z, flags (int bits: 1 dynamic, 2 linear locks)
};
#define SB_DYNAMIC 1
#define SB_LINLOCK 2

struct __align__(16) TriDev {
    float4 a, b, c;    // mesh-local vertices
    float4 n;          // unit normal
    float4 nb[3];      // neighbour normals across edges A, B, C; w = 1 when the neighbour exists
};

// Partitioned solve schedule.  Three staggered column grids in x-z (offsets 0, h/3, 2h/3
// of the cell size h, with h above three times the largest horizontal distance between
// two dynamic bodies sharing an arbiter): every such arbiter lies inside one cell of at
// least one grid.  A cell's arbiters form a task, solved by one CTA with the cell's
// bodies in shared memory; the three grids are three phases per solver pass, so a pass
// needs at most three grid barriers instead of one per colour (none between phases when
// tasks hand off through completion counters).  Arbiters that fit no task
// (and all joints) form the remainder, solved in global colours as before.
#define JG_SCHED_GRIDS 3
#define JG_SCHED_MAXCELLS 65536      // cells per grid
#define JG_SCHED_MAXTASKS 32768
#define JG_SCHED_CELL_ARBITERS 250.f // default partition density: arbiters per cell on average
#define JG_TASK_MAXC 64              // local colours per task
#define JG_TASK_MAXA 6144            // arbiters per task (local colouring in shared memory)
#define JG_ORDER_REMAINDER 768       // order keys: task arbiters grid * 256 + colour, remainder 768 + colour

struct SchedInfo {
    unsigned span_bits;              // largest |dx|, |dz| between two dynamic bodies of an arbiter
    unsigned bbox[4];                // dynamic body x min, z min, x max, z max (order-preserving bits)
    float h, x0, z0;                 // cell size and grid origin
    int ncx, ncz, ncells;            // cells per grid (ncells = worlds * ncx * ncz, or worlds)
    int ntask[JG_SCHED_GRIDS];       // tasks per grid
    int task_base[JG_SCHED_GRIDS];   // first task of each grid
    int ntasks;
    int narb_task;                   // arbiters placed in tasks (the remainder starts there)
    int tag;                         // step counter for the body claim stamps
    int overflow;                    // cells pushed to the remainder (too large)
    int maxc;                        // most local colours of any task
    int pad[3];
};

struct ArbStore {
    int2* key;      // shape ids (ArbiterKey)
    int2* body;     // body indices
    int4* info;     // usage mask, solve mode, order key, created-this-step flag
    int4* lslot;    // task arbiters: body slots of body 1 and 2 in the task (-1: not a task body),
                    // usage | mode << 4 | (a non-dynamic body) << 8, friction bits
    float4* sv;     // [2 * cap] velocity, angular velocity of a non-dynamic body (constant in the solve)
    float4* mat;    // friction, restitution, speculative relaxation, 0
    float4* cn;     // normal xyz, Bias
    float4* ct1;    // tangent1 xyz, PenaltyBias
    float4* ct2;    // tangent2 xyz, contact flags (int bits)
    float4* cr1;    // RelativePosition1 xyz, mass normal
    float4* cr2;    // RelativePosition2 xyz, mass tangent1
    float4* cacc;   // accumulated normal, tangent1, tangent2, mass tangent2
    float4* cp1;    // Position1 (local) xyz, 0
    float4* cp2;    // Position2 (local) xyz, 0
};

struct __align__(16) JointDev {
    int4 hdr;        // kind, body1, body2, colour
    float4 la1, la2; // BallSocket local anchors
    float4 r1, r2;   // world anchors (prepare)
    float4 acc;      // accumulated impulse
    float4 bias;
    float4 eff[3];   // effective mass rows
    float4 jac[3];   // HingeAngle Jacobian columns
    float4 axis;     // hinge axis (local to body 2)
    float4 q0;       // hinge reference rotation
    float4 lim;      // min, max, fixed angle, clamp (as float)
    float4 prm;      // bias factor, softness, limit bias, limit softness
    float4 bil;      // bilateral block inverse xyz, hemisphere
    float4 cpl;      // coupling x, coupling y
};

struct DevCounters {
    int npairs;
    int nstream;      // colliding pairs written by the narrowphase
    int nepa;         // pairs queued for EPA
    int narb;         // arbiters in the current store
    int nnew;         // arbiters created this step
    int ncolors;
    int nremoved;
    int status;       // JG_ERR_* raised on the device
    int epa_fail;
    int exact;
    int points;       // manifold points written
    int contacts;     // active contact points after the merge
    int new_contacts;
    int color_rounds;
    int ncol;         // overlapping pairs found by the MPR stage
    int nepa_list;    // of those, deeper than the EPA threshold
    int nedge;        // of those, near a mesh edge (triangle-edge filter)
    int ntasks;       // partitioned solve: tasks, arbiters in tasks, most local colours
    int narb_task;
    int task_colors;
    int epa_next;     // work cursors of the warp-per-pair narrowphase stages
    int edge_next;
    int nspec;        // speculative sweep candidates, and of those the pairs registered
    int nspec_hit;
    int pad[1];
};

struct WorldDev {
    // capacities
    int cap_bodies, cap_shapes, cap_pairs, cap_arb, cap_joints, cap_hull, cap_tris;
    int nb, ns, nj, nhull, ntris, nworlds;
    // bodies
    SBody* body;
    float4 *pos, *q, *dv, *dw, *il0, *il1, *force, *torque, *mat;
    int4* binfo;                 // motion, flags, world, island flags (1 marked, 2 in the active list)
    float4* sleep;               // sleep time, deactivation time, squared linear / angular rest thresholds
    int* uf;                     // [cap_bodies] islands: union-find parent, then root
    int* ufl;                    // [cap_bodies] island flags at each root
    int allow_deact;             // World.AllowDeactivation for this step
    // shapes
    int4* sinfo;                 // kind, body, data offset, data count
    float4 *sdims, *scenter, *hull;
    TriDev* tris;
    float4 *amin, *amax;         // world AABBs
    // broadphase
    unsigned long long *mkey, *mkey_alt;
    int *midx, *midx_alt;
    int *hist;                   // radix histograms
    int4* node;                  // internal nodes: left, right, parent, first|last packed
    int2* node_range;            // leaf range [first, last] per internal node
    float4 *nmin, *nmax;         // internal node AABBs
    float4* cbox;                // [4 * cap_shapes] per internal node, both children's boxes:
                                 // left min|code, left max|worlds, right min|code, right max|worlds
                                 // (code: internal child index, or ~shape for a leaf; worlds:
                                 // first | last << 16 of an internal child's subtree)
    int* leaf_parent;
    int* node_parent;            // parent of each internal node (-1 for the root)
    int* node_flag;
    float4* scene_box;           // [0] min, [1] max (reduction)
    int2* pairs;
    int* pair_order;             // [cap_pairs] pair indices grouped by the two shapes' kinds
    int* pair_kind;              // [2 * 64] counts, then cursors, per kind combination
    // narrowphase: overlapping pairs from the MPR stage, then the contact stream
    int2* col_pair;              // [cap_arb] pair index, MPR code (1 final, 2 needs EPA)
    float4* col_res;             // [3 * cap_arb] MPR result in A's frame: pA, pB, normal|depth
    float4* col_portal;          // [12 * cap_arb] MPR portal (4 vertices: V, A, B), by EPA-list slot
    int* epa_list;               // [cap_arb] colliding-record index of each deep pair
    int* edge_list;              // [cap_arb] colliding-record index of each pair near a mesh edge
    int* spec_list;              // [cap_pairs] pairs without overlap that qualify for the sweep
    int2* cs_key;
    float4* cs_n;                // normal xyz, count
    float4* cs_pa;               // [4 * cap_pairs]
    float4* cs_pb;
    // arbiters
    ArbStore arb[2];
    int cur;                     // which ArbStore holds the live arbiters
    unsigned long long* hkeys;   // hash table keys
    int* hvals;
    int hcap;
    // colouring
    int* cstat;                  // per constraint: colour or -1
    unsigned long long* bmask;   // per body: used colours (2 words)
    int* adj_off;                // CSR body -> constraints
    int* adj;
    int* deg;
    int* color_count;            // [JG_MAX_COLORS + 1]
    int* color_start;            // [JG_MAX_COLORS + 1] arbiters
    int* jcolor_start;           // [JG_MAX_COLORS + 1] joints
    int* color_cursor;
    int* jorder;                 // joints sorted by colour
    // joints
    JointDev* joints;
    // solver bookkeeping
    unsigned* bar_count;         // grid barrier
    unsigned* bar_gen;
    float* resid;                // per iteration: sum dlambda^2, sum lambda^2 [2 * 64]
    float* mlp_w;                // MLP parameters (device)
    DevCounters* ctr;
    // partitioned solve schedule (see SchedInfo)
    SchedInfo* sc;
    int* sc_cell;                // [3 * cap_bodies] cell of each dynamic body per grid, -1 otherwise
    int* sc_stamp;               // [3 * cap_bodies] step tag of the body's claim per grid
    int* sc_bslot;               // [3 * cap_bodies] body slot in its cell's task
    int2* sc_arb;                // [cap_arb] grid (3 = remainder, -1 = dead) and cell of each arbiter
    int* sc_acount;              // [3 * MAXCELLS] arbiters per cell
    int* sc_bcount;              // [3 * MAXCELLS] bodies claimed per cell
    int* sc_task_of;             // [3 * MAXCELLS] task of each cell, -1 if none
    int4* sc_task;               // [MAXTASKS] arbiter offset, count, body offset, count
    int* sc_cursor;              // [MAXTASKS]
    int* sc_tnc;                 // [MAXTASKS] local colours of the task
    int* sc_tcell;               // [MAXTASKS] cell of the task (in its grid)
    int4* sc_tdep;               // [2 * MAXTASKS] tasks of the previous two grid phases sharing bodies (-1: none)
    unsigned* sc_done;           // [MAXTASKS] levels (grid phases) the task has completed in the solve
    int* sc_tcol;                // [MAXTASKS * (MAXC + 1)] colour offsets inside the task
    int* sc_tlist;               // [cap_arb] arbiters of each task (pre-permute ids)
    int* sc_tbody;               // [3 * cap_bodies] bodies of each task
    int* sc_dst;                 // [cap_arb] final slot of a task arbiter, -1 for the remainder
    int* sc_lcol;                // [cap_arb] local colour of a task arbiter
    int4* sc_ls;                 // [cap_arb] body slots of a task arbiter
    // per-step scratch of the cache merge and the colour permutation (each world its own)
    int2* ev_created;            // [cap_arb] keys of the arbiters created this step
    int2* ev_removed;            // [cap_arb] keys of the arbiters removed this step
    int* remaining;              // [2] colouring: constraints still without a colour
    int* dst_index;              // [cap_arb] slot of each arbiter after the permutation, -1 if removed
    // launch shapes of the cooperative kernels, sized once per world on its device (host
    // side only; a world is driven by one host thread)
    int lc_color_grid;
    int lc_solve_grid, lc_solve_block, lc_solve_ctas;
    int lc_tasks_grid, lc_tasks_block, lc_tasks_ctas;
    size_t lc_tasks_smem;
    // learned warm start: for the contacts created this step (arbiter before the colouring
    // permutation, slot), the accumulated impulse after the first substep's iterations
    // is copied to rec_tgt (training targets); rec_on enables it
    int rec_on;
    int rec_cap;
    const int2* rec_fidx;
    const int* rec_count;
    const int* rec_dst;
    float* rec_tgt;
};

// Contact stream record flag (bits above the point count in the normal's w): the pair came
// from the speculative sweep and is solved without angular terms (SolveMode.Angular removed).
#define JG_STREAM_SPECULATIVE 0x100

struct StepParams {
    float dt, sub_dt, inv_dt, inv_sub_dt;
    float3 gravity;
    int substeps, iterations, relax;
    int aux_contacts, persistent, edge_filter;
    float spec_relax;
    float spec_threshold;        // SpeculativeVelocityThreshold
    int warm_start;
    int record_residual;
    int partition;               // 1: partitioned solve (tasks + remainder), 0: global colours only
    int allow_deact;             // World.AllowDeactivation: sleeping bodies and rows are skipped
    int stabilize;               // World.Stabilize: solve only, no force or velocity integration
    int task_maxb;               // bodies a task may hold in the solver's shared memory
    float cells_per_sm;          // partition cells per grid and SM, before the span bound (0: chosen on the device)
    int solve_blocks;            // persistent blocks of the task solve (the default density rule)
};

// Partitioned-solve launch shape: threads per CTA and bytes of shared memory per
// staged arbiter (4 contact slots x 5 float4 rows + header, 2 x non-dynamic body velocity).
#define JG_TASK_STAGE_F4 23
// Staged arbiters per thread.  Thread t owns every blockDim-th arbiter of its task, so its
// next arbiter lies blockDim positions (several colours) ahead: one slot in flight is
// enough, and the small ring lets two 128-thread task CTAs share an SM.
#define JG_TASK_RING 1
#define JG_TASK_BLOCK 128        // default threads per task CTA
#define JG_TASK_CTAS 2           // default task CTAs per SM
int jg_solver_task_maxb(int block, int ctas_per_sm);

// ---- stage launchers (each defined in its own translation unit) ------------------------
void jg_launch_aabb(WorldDev& w, float dt, cudaStream_t s);
int  jg_launch_broadphase(WorldDev& w, cudaStream_t s, int nsm);
void jg_launch_narrowphase(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm, int tile);
void jg_launch_merge(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm);
int  jg_launch_color(WorldDev& w, cudaStream_t s, int nsm);
void jg_launch_schedule(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm);
int  jg_launch_solve(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm, int block, int ctas_per_sm);
void jg_launch_update(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm);
void jg_launch_mlp_warmstart(WorldDev& w, const StepParams& p, cudaStream_t s, int nsm);
void jg_launch_islands(WorldDev& w, cudaStream_t s, int nsm);

// Arbiter mode word (ArbStore::info.y): SolveMode bits 0-3, and this bit when neither body
// is an awake non-static body (the row is neither solved nor updated while it sleeps).
#define JG_ARB_ASLEEP (1 << 16)
// Staged header bit of a task arbiter that sleeps.
#define JG_TASK_ASLEEP 512
