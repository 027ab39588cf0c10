/*
 * b2g_internal.h — device data layout of a GPU world (or batch of worlds) and the
 * launchers each kernel file exports to the host-side world (api.cu).
 *
 * Layout (all arrays in HBM, structure-of-arrays, 16-byte vectors where a kernel
 * reads several fields of one object together):
 *   bodies    b_xf(p.x,p.y,sin,cos) b_pos(c.x,c.y,a,-) b_pos0(c0.x,c0.y,a0,-)
 *             b_vel(v.x,v.y,w,sleep_time) b_force(f.x,f.y,torque,-) b_mass(m,1/m,I,1/I)
 *             b_damp(lin,ang,gravity_scale,-) b_lc(local centre) b_flags b_world b_island
 *   fixtures  f_shape (144-byte ShapeRec) and its structure-of-arrays copy for the narrowphase:
 *             f_vn (8 rows per fixture: vertex k and the normal of edge k) and f_hdr (centroid.x,
 *             centroid.y, radius, meta bits); f_body f_mat(friction,restitution,threshold,density)
 *             f_filter(category|mask<<16, group|sensor<<16) f_refid (the reference's proxy id)
 *             f_fat (fat AABB lo.x,lo.y,hi.x,hi.y) f_moved
 *   contacts  sorted by key = refid_min << 32 | refid_max (double-buffered, merged each step)
 *   solver    per constraint slot, slots grouped by colour: vc_* (velocity), pc_* (position)
 *   LBVH      sorted leaf keys/ids, internal nodes holding both child boxes
 */
#ifndef B2G_INTERNAL_H
#define B2G_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>

#include "b2g_collide.cuh"

namespace b2g {

/* body flag bits (BodyFlags, src/b2_body.rs:212-229, plus the body type) */
enum : uint32_t {
    BF_TYPE_MASK = 3u,
    BF_AWAKE = 1u << 2,
    BF_ENABLED = 1u << 3,
    BF_AUTO_SLEEP = 1u << 4,
    BF_FIXED_ROTATION = 1u << 5,
    BF_BULLET = 1u << 6,
    BF_ISLAND = 1u << 7,   /* member of an island solved this step */
};
enum { BODY_STATIC = 0, BODY_KINEMATIC = 1, BODY_DYNAMIC = 2 };

/* contact flag bits (ContactFlags, src/b2_contact.rs:283-305) */
enum : uint32_t {
    CF_TOUCHING = 1u << 0,
    CF_ENABLED = 1u << 1,
    CF_DEAD = 1u << 2,
    CF_SENSOR = 1u << 3,
    CF_FILTER = 1u << 4,   /* E_FILTER_FLAG: re-check should_collide at the next collide */
    CF_REJECT = 1u << 5,   /* the host's contact filter rejected this flagged contact (destroyed at collide) */
    CF_UPDATED = 1u << 6,  /* updated by this step's collide (kept only while a pre_solve callback is set) */
    CF_KIND_SHIFT = 8,
};

/* revolute joint flag bits (j_par.y) */
enum : uint32_t {
    JF_LIMIT = 1u << 0,
    JF_MOTOR = 1u << 1,
    JF_COLLIDE = 1u << 2,  /* collide_connected */
    JF_TYPE_SHIFT = 8,     /* the joint type (B2G_JOINT_*) sits in bits 8-15 */
    JF_GEAR_A_PRISMATIC = 1u << 16,  /* a gear joint's first joint is prismatic (else revolute) */
    JF_GEAR_B_PRISMATIC = 1u << 17,  /* its second joint is prismatic */
};

/* device status bits (sticky until read by the host) */
enum : uint32_t {
    ST_CONTACT_OVERFLOW = 1u << 0,
    ST_PAIR_OVERFLOW = 1u << 1,
    ST_EVENT_OVERFLOW = 1u << 2,
    ST_COLOUR_OVERFLOW = 1u << 3,
    ST_BARRIER_TIMEOUT = 1u << 4,
    ST_STACK_OVERFLOW = 1u << 5,
    ST_RECORD_OVERFLOW = 1u << 6,
    ST_PART_MISMATCH = 1u << 7,   /* the solver ran with other parts than its colouring */
    ST_TOI_OVERFLOW = 1u << 8,    /* a time-of-impact island, candidate, moved-proxy or new-contact
                                     list of the continuous pass overflowed */
};

/* device counters (d_cnt[]) */
enum {
    CNT_CONTACTS = 0,     /* contacts in the current table */
    CNT_CONS = 1,         /* island constraints this step */
    CNT_COLOURS = 2,      /* non-empty colours */
    CNT_NEW = 3,          /* new contacts found by the broadphase */
    CNT_EVENTS = 4,
    CNT_PAIRS = 5,        /* recorded emitted pairs (parity hook) */
    CNT_STATUS = 6,
    CNT_ALIVE = 7,        /* surviving old contacts during a merge */
    CNT_UNCOLOURED = 8,   /* 2 ints, alternating by colouring round */
    CNT_ROUNDS = 10,
    CNT_TOUCHING = 11,
    CNT_BOUNDS = 12,      /* 4 ints: ordered-int min.x, min.y, max.x, max.y of proxy centres */
    CNT_BARRIER = 16,     /* grid barrier arrivals of the running cooperative launch (zeroed per launch) */
    CNT_ISLANDS = 18,
    CNT_COLOURINGS = 19,  /* colourings done so far: the stamp of colours kept in contacts (mids.w) */
    CNT_DYN_EXTENT = 20,  /* largest half-extent of a dynamic body's fat AABB (float bits), this pass */
    CNT_INTERIOR = 21,    /* constraint slots solved part-locally this step (slots [0, n)) */
    CNT_PARTS = 22,       /* parts of this step's colouring (at most the solver's blocks), 0 if off */
    CNT_PART_NCACHE = 23, /* constraint bodies of the current partition (entries of cache_body) */
    CNT_PART_P = 24,      /* parts of the current partition (0: none) */
    CNT_PART_NF = 25,     /* proxies when the current partition was made */
    CNT_TAIL = 26,        /* colouring: constraints left to the single-block rounds */
    CNT_TOI_EVENTS = 27,  /* solid time-of-impact events solved since the world was made */
    CNT_TOI_ITERS = 28,   /* iterations of the last continuous pass */
    CNT_TOI_PASSES = 29,  /* continuous passes run (their body marks are stamped with it) */
    CNT_TOI_ROLLBACKS = 30, /* passes restarted in sequential order after a conflict */
    CNT_MERGE_FROM = 31,  /* contacts in the table the last merge started from */
    CNT_CASCADE = 40,     /* 3 ints: contacts collided per round of the wake cascade (rotating) */
    CNT_CASCADE_ROUNDS = 43, /* rounds of the last wake cascade */
    CNT_BARRIER_LIMIT = 44, /* grid-barrier wait limit in units of 1024 clock cycles (0: 2e9 cycles) */
    CNT_BARRIER_HOLD = 45,  /* extra arrivals every grid barrier waits for (0; a test's timeout hook) */
    CNT_BP_VISITS = 46,     /* hierarchy nodes the last broadphase traversal fetched */
    CNT_BP_CANDIDATES = 47, /* leaves it checked against the pair rules */
    /* continuous pass (k_continuous.cu), zeroed before every pass: */
    CNT_TOI_FIRST = 32,
    CNT_TOI_NEW = 32,     /* contacts created by the pass (table slots [n, n + this)) */
    CNT_TOI_SYNC = 33,    /* bodies with a pending sweep advance */
    CNT_TOI_MOVED = 34,   /* proxies moved by this iteration's islands */
    CNT_TOI_HITS = 35,    /* contacts whose time of impact is an event candidate this iteration */
    CNT_TOI_NEV = 36,     /* events of this iteration */
    CNT_TOI_CONFLICT = 37, /* two events of one iteration asked to advance one body to different alphas */
    CNT_TOI_SNAP_EV = 38, /* CNT_EVENTS and CNT_TOI_EVENTS when the pass's snapshot was taken */
    CNT_TOI_SNAP_TE = 39,
    CNT_TOI_LAST = 40,
    /* the broadphase hierarchy: rebuilt, or kept with its moved leaves updated in place */
    CNT_BP_REBUILD = 48,  /* this pass rebuilds the hierarchy (1) or updates it in place (0) */
    CNT_BP_AGE = 49,      /* passes since the last rebuild */
    CNT_BP_MOVED = 50,    /* proxies the solver moved since the last pass (the fixture sync counts them) */
    CNT_BP_DRIFT = 51,    /* proxies moved since the last rebuild */
    CNT_BP_FORCE = 52,    /* nonzero: the host changed proxies, the next pass rebuilds */
    CNT_BP_NF = 53,       /* proxies at the last rebuild */
    CNT_BP_SORT_N = 54,   /* keys the pass sorts: the proxies on a rebuild, 0 otherwise */
    CNT_BP_LAST_MOVED = 55, /* proxies the solver moved before the last pass */
    CNT_BP_MAX_AGE = 56,  /* passes a kept hierarchy may reach before a rebuild (0: rebuild every pass) */
    CNT_BP_WARP_VISITS = 57, /* the most node fetches one warp of the last traversal made */
    CNT_BP_WARP_CHECKS = 58, /* the most leaf checks one warp of the last traversal made */
    CNT_SIZE = 64
};

constexpr int kMaxColours = 256;   /* first-fit colours 0..63, then one per colouring round */
constexpr int kFirstFitColours = 64;
constexpr int kColourTail = 256;   /* uncoloured constraints one block finishes colouring (one per thread) */
constexpr int kMaxParts = 1024;    /* body parts of the part-local solve (at most one per solver block) */
/* default of cfg_collide_group: one lane per pair (measured on GB300 at least as fast as the 8-lane
 * segments on the mixed 100k scene, the 4096-world batch and the 250k-box pile) */
constexpr int kCollideGroup = 0;
constexpr int kKeyMortonBits = 22; /* broadphase keys: key world << 22 | Morton code (11 bits per axis) */
constexpr int kMaxPosIters = 64;
constexpr int kNoWake = 0x7f7f7f7f;  /* b_wake's "not woken" (a byte-wise memset value) */
/* continuous pass lists (k_continuous.cu): partner contacts of one event, events of one
 * iteration, contacts created in one pass */
constexpr int kMaxJointColours = 64;  /* colours of the joint colouring */
constexpr int kToiCand = 64;
constexpr int kToiEvCap = 4096;
constexpr int kToiNewCap = 4096;

struct Contacts {
    unsigned long long* key;
    int2* fix;        /* fixture A, fixture B (A = primary shape type) */
    int2* body;
    uint32_t* flags;
    float4* mat;      /* friction, restitution, restitution threshold, tangent speed */
    float4* mgeo;     /* local normal, local point */
    float4* mpts;     /* point 0 local, point 1 local */
    float4* mimp;     /* normal 0, tangent 0, normal 1, tangent 1 impulses */
    uint4* mids;      /* id 0, id 1, type | count << 8, colour | stamp << 6 (the colour this contact
                         had as a constraint of the colouring with that stamp; 0 = none) */
};

struct StepParams {
    float dt, inv_dt, dt_ratio;
    float gx, gy;
    int vi, pi;
    int warm;
    int allow_sleep;
    int auto_clear;
    int record_events;
    int record_pairs;
    int part_bodies;      /* part-local solve: bodies cached in shared memory per block */
    int part_slot_bytes;  /* part-local solve: shared memory per block for constraint slots */
    int toi_schedule;     /* continuous pass: B2G_TOI_SCHEDULE_* */
    int custom_filter;    /* the host's contact filter replaces the default one (new pairs are filtered on
                             the host, flagged contacts carry its answer in CF_REJECT) */
    int pre_solve;        /* contacts updated by collide are marked CF_UPDATED for the host's pre_solve */
    int toi_may_conflict; /* continuous pass: a kinematic or bullet body exists, so side-by-side events
                             can conflict and the pass keeps a snapshot to restart from */
};

struct DevWorld {
    int body_cap, fix_cap, contact_cap, pair_cap, event_cap, cons_cap;
    /* launch configuration (b2g_set_launch_config / b2g_autotune); results do not depend on it */
    int cfg_coop_per_sm;      /* blocks per SM of the cooperative colouring and solver kernels */
    int cfg_collide_block;    /* threads per block of the narrowphase */
    int cfg_traverse_block;   /* threads per block of the broadphase traversal */
    int cfg_solver_block;     /* threads per block of the persistent solver (256, or 512 at one block per SM) */
    int cfg_collide_group;    /* narrowphase: a warp batch with at most this many polygon pairs evaluates
                                 them eight lanes to a pair (collide_polygons_group); more, a lane each */
    int n_bodies, n_fixtures, num_worlds;
    int num_sms;              /* multiprocessors of the world's device (grid caps of the launchers) */
    int key_bits;      /* bits of the contact key (2 x refid bits) */
    int morton_world_bits;
    /* bodies */
    float4 *b_xf, *b_pos, *b_pos0, *b_vel, *b_force, *b_mass, *b_damp;
    float2* b_lc;
    uint32_t* b_flags;
    uint32_t* b_world;
    int* b_island;
    int* b_rank;                 /* smallest sorted position of the body's proxies in the last
                                    broadphase (Morton order), INT_MAX if none */
    int* b_part;                 /* part-local solve: the body's part (valid for constraint bodies) */
    int* b_cidx;                 /* part-local solve: the body's place among constraint bodies in
                                    rank order (valid for constraint bodies) */
    unsigned long long* b_cmin;  /* colouring: minimum priority of uncoloured constraints,
                                    2 round parities x 2 classes x body_cap */
    unsigned long long* b_cmask; /* colouring: colours used at this body, 2 classes x body_cap */
    uint32_t* isl_minsep;        /* 2 x body_cap: per-island max(-separation) bits, double-buffered */
    int* b_wake;                 /* collide pass of a world whose bodies may sleep: the smallest table
                                    place of a contact whose update woke the body (kNoWake: none) */
    uint8_t* b_dwake;            /* woken by a destroyed contact (applied after the pass) */
    uint8_t* c_done;             /* per contact: collided in this pass */
    uint8_t* isl_done;
    float* isl_sleep;            /* per island root: min sleep time (as ordered uint bits) */
    /* fixtures */
    ShapeRec* f_shape;
    float4* f_vn;                /* kMaxPolygonVertices rows per fixture (f * 8 + k): v.x, v.y, n.x, n.y */
    float4* f_hdr;               /* centroid.x, centroid.y, radius, meta word (bits) */
    int* f_body;
    float4* f_mat;
    uint32_t* f_filter;          /* category | mask << 16 */
    uint32_t* f_group;           /* (uint16) group | sensor << 16 */
    uint32_t* f_refid;
    float4* f_fat;
    uint8_t* f_moved;
    /* contacts: current table and the merge target */
    Contacts c, c_alt;
    int* c_rank;                 /* exclusive scan of alive flags during a merge */
    int* c_row_end;              /* per proxy id: one past the last contact of that row (same validity) */
    int* c_row;                  /* per proxy id: first contact of the sorted table whose key starts with
                                    it (valid only when that contact's key does: see k_bp_rows) */
    /* new contacts from the broadphase */
    unsigned long long* n_key;   /* keys; sorted in place */
    int2* n_fix;                 /* fixture pair per new key (before sorting) */
    uint32_t* n_idx;             /* sort payload */
    unsigned long long* n_key_alt;
    uint32_t* n_idx_alt;
    /* constraints */
    int* cons_contact;           /* unsorted: contact index per constraint */
    int* cons_colour;
    int* cons_island;
    int* s_contact;              /* slot -> contact (sorted by colour) */
    int* s_cons;                 /* slot -> constraint */
    int2* s_fix;                 /* slot -> (fixture A, fixture B): the solve order exported to the host */
    int* cons_part;              /* part of an interior constraint, -1 for a boundary one */
    int* col_tail;               /* kColourTail: the constraints the last colouring rounds took */
    int* col_off;                /* kMaxColours + 1 offsets of non-empty boundary colours */
    int* col_hist;               /* (kMaxParts + 1) x kMaxColours counts, then slot cursors:
                                    rows of the parts' interior colours, last row the boundary's */
    int* part_off;               /* kMaxParts x (kMaxColours + 1): offsets of each part's
                                    non-empty interior colours */
    int* part_ncol;              /* kMaxParts: non-empty interior colours of each part */
    int* part_tot;               /* kMaxParts + 1: slots of each histogram row */
    unsigned long long* rank_x;  /* per Morton rank: constraint endpoints << 32 | has-any, then
                                    its exclusive prefix within the scanning block's chunk */
    unsigned long long* blk_tot; /* per block of a cooperative launch (at least kMaxParts and 8 per SM): chunk
                                    totals of that scan and of k_islands' constraint count */
    int* cache_body;             /* constraint bodies in rank order */
    int* part_cbeg;              /* kMaxParts: each part's first entry of cache_body */
    int* part_cend;              /* kMaxParts: one past its last */
    int* part_rbeg;              /* kMaxParts: each part's first Morton rank when the partition was
                                    made (ascending); places bodies outside it by their rank */
    int4* vc_idx;                /* ia, ib, point count, flags (bit0 A dynamic, bit1 B dynamic) */
    int2* vc_code;               /* part-local solve: the slot's bodies as its block addresses them
                                    (cache entry, or -(body + 1) in global memory), for slots read
                                    from global memory */
    float4 *vc_inv, *vc_nf, *vc_r0, *vc_r1, *vc_m0, *vc_m1, *vc_imp, *vc_k;
    float4 *pc_lp, *pc_geo, *pc_lc, *pc_inv, *pc_meta;
    int* vc_island;
    /* broadphase */
    unsigned long long* bp_key;
    uint32_t* bp_val;
    unsigned long long* bp_key_alt;
    uint32_t* bp_val_alt;
    float4* bp_leaf;             /* leaf fat AABB in sorted order */
    float4* bp_node_b0;          /* internal node: child 0 box */
    float4* bp_node_b1;          /* internal node: child 1 box */
    int2* bp_node_child;         /* child indices; leaves encoded as ~leaf */
    int* bp_parent;              /* parent of internal nodes [0,n-1) and leaves [n-1, 2n-1) */
    uint32_t* bp_flag;           /* refit arrival counters */
    float4* bp_quad_box;         /* internal node: its grandchildren's boxes (4 per node; a leaf child
                                    stands for itself), so a walk descends two levels per fetch */
    int4* bp_quad_child;         /* the 4 entries (encoded like children; INT_MIN: none) */
    int* bp_world_root;          /* per key world (2 x num_worlds): root node (encoded like children), or
                                    INT_MIN if empty; key world w + num_worlds holds world w's large
                                    static proxies (see k_bp_keys) */
    int* bp_world_first;         /* per key world: first sorted leaf */
    /* joints (revolute): definitions, impulses kept across steps, the step's temporaries, the
     * joints sorted by colour (j_order, j_coff: n_jcolours + 1 offsets) and body -> joints */
    int n_joints, n_jcolours;
    int2* j_body;
    int2* j_body2;               /* a gear joint's bodies C and D (the first bodies of its two joints) */
    float4 *j_anchor, *j_lim, *j_par, *j_imp, *j_imp2, *j_rr, *j_k, *j_m, *j_x;
    float2* j_s;
    int *j_order, *j_coff;
    int *b_jnt_off, *b_jnt;
    /* continuous physics: the time-of-impact pass (k_continuous.cu) */
    int* b_fix_off;              /* body -> fixtures: offsets into b_fix (n_bodies + 1) */
    int* b_fix;                  /* fixtures grouped by body */
    float* b_alpha0;             /* the body sweep's alpha0 during the pass */
    int* b_stamp;                /* pass iteration that last put the body in an event's island */
    int* b_event;                /* that event's slot */
    int* b_inval;                /* pass iteration whose island displaced the body (its contacts' times
                                    of impact are stale) */
    int* b_cx;                   /* the pass (CNT_TOI_PASSES) in which the body was found touching a
                                    kinematic or bullet body: its events are solved one at a time */
    uint32_t* b_sync;            /* pending advance of the body's sweep (alpha bits; 0: none) */
    uint32_t* b_best;            /* the body's earliest event candidate this iteration (alpha bits) */
    unsigned long long* b_bkey;  /* and its contact key */
    int* f_leaf;                 /* the proxy's leaf in the step's LBVH */
    float* t_toi;                /* per contact: cached time of impact (alpha) */
    int* t_when;                 /* per contact: iteration that computed t_toi, -1 none */
    int* t_count;                /* per contact: time-of-impact events (toi_count) */
    uint8_t* t_elig;             /* per contact: non-sensor with a bullet or non-dynamic body */
    int* t_hits;                 /* contacts with an event-candidate alpha this iteration */
    int* t_hitx;                 /* per hit: the dynamic body of a simple hit, -1 for others */
    int* t_sync;                 /* bodies with a pending sweep advance */
    int* t_moved;                /* proxies moved by this iteration's islands */
    unsigned long long* t_nkey;  /* the pass's new contacts sorted by key (key, then table slot) */
    int* t_nslot;
    int* ev_contact;             /* per event of the iteration: its contact, alpha, and the iteration */
    float* ev_alpha;             /* if the contact touched (a solid event), else -1 */
    int* ev_solid;
    int* ev_cand;                /* per event: count, then its bodies' partner contacts */
    uint32_t* tw_alpha;          /* per world: earliest one-at-a-time candidate (alpha bits; ~0: none) */
    unsigned long long* tw_key;  /* and its key */
    uint32_t* tw_salpha;         /* per world: earliest candidate of a body solved side by side */
    unsigned long long* tw_skey;
    float4 *s_xf, *s_pos, *s_pos0, *s_vel;  /* the pass's snapshot of the bodies and proxies */
    uint32_t* s_flags;
    float4* s_fat;
    /* outputs for the host */
    int4* events;                /* kind, fixture a, fixture b, - */
    uint2* pairs;                /* recorded emitted pairs (fixture ids) */
    /* scratch for the primitives */
    uint32_t* scan_tmp;
    uint32_t* sort_hist;
    int sort_hist_cap;
    int* cnt;
};

/* After a grid-barrier wait ran out, the step's buffers may be half-written: every later kernel of
 * the world returns at once (it reads no index another kernel computed) until the host reads and
 * clears the status (B2G_ERR_TIMEOUT). The status word is written only by the world's own kernels and
 * the host between launches, so all blocks of one launch see the same value. */
__device__ __forceinline__ bool world_aborted(const int* cnt) {
    return (((volatile const int*)cnt)[CNT_STATUS] & ST_BARRIER_TIMEOUT) != 0;
}
#define B2G_RETURN_IF_ABORTED(w) \
    do {                          \
        if (world_aborted((w).cnt)) return; \
    } while (0)

/* Programmatic dependent launch: a kernel launched with launch_pdl may be scheduled while the
 * kernel before it on the stream drains (its launch no longer waits behind that kernel's last
 * block). pdl_entry() waits until that kernel has completed and its writes are visible (at once for
 * a kernel launched without the attribute) and lets the next kernel be scheduled in turn; every
 * kernel launched with launch_pdl calls it before it reads memory. */
__device__ __forceinline__ void pdl_entry() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

/* kernel-file launchers */
/* may_sleep: some body may be asleep (sleeping allowed, or a body made asleep): contacts then see
 * the bodies woken by contacts before them in the table's key order, as in the reference's list */
void launch_collide(const DevWorld& w, const StepParams& sp, cudaStream_t s, bool may_sleep, int num_sms);
void launch_shape_rows(const DevWorld& w, int n_fixtures, cudaStream_t s);
/* contact edits of destroy / refilter calls between steps (k_edit_contacts in k_collide.cu): fix_mark
 * per fixture, bit 0 destroyed (its contacts are destroyed), bit 1 refiltered (its contacts are flagged
 * for filtering); body_pairs: contacts between these bodies are flagged for filtering */
void launch_edit_contacts(const DevWorld& w, const uint8_t* fix_mark, const int2* body_pairs, int n_pairs,
                          bool record_events, cudaStream_t s);
/* marks every proxy moved, so the next broadphase queries them all (a repeated pass after a capacity
 * grew finds the same new contacts as the pass it replaces) */
void launch_touch_all_proxies(const DevWorld& w, cudaStream_t s);
/* flags the contacts of bodies a joint keeps apart (after joints were created) */
void launch_flag_joint_contacts(const DevWorld& w, cudaStream_t s, int num_sms);
void launch_islands_and_constraints(const DevWorld& w, const StepParams& sp, cudaStream_t s);
/* parts: allow the part-local solve (used where the world's size suits it) */
void launch_colouring(const DevWorld& w, cudaStream_t s, int num_sms, bool parts);
int launch_solver(const DevWorld& w, const StepParams& sp, cudaStream_t s, int num_sms, bool parts);
/* time of impact of n shape pairs (sweeps as 2 float4: (lc, c0), (c, a0, a)); out = (state, t bits) */
void launch_time_of_impact(const ShapeRec* sa, const float4* swa, const ShapeRec* sb, const float4* swb,
                           const float* t_max, int n, int2* out, cudaStream_t s);
/* continuous physics of a step (B2world::solve_toi) as one cooperative launch; returns a CUDA error */
int launch_continuous(const DevWorld& w, const StepParams& sp, cudaStream_t s, int num_sms);
/* whether the part-local solve applies to this world (parts allowed and the world's size suits it) */
bool use_parts(const DevWorld& w, int num_sms, bool allowed);
/* mark (optional) is called with 0 after the keys and their sort, 1 after the hierarchy (build,
 * refit, four-way records, contact rows), 2 after the traversal (before the contact merge), so the
 * caller can record profiling events there */
/* mode: BP_AUTO (the pass decides whether to rebuild the hierarchy), BP_REBUILD, or BP_REPEAT (the
 * same pass again, after a capacity overflow: the previous decision holds) */
enum { BP_AUTO = 0, BP_REBUILD = 1, BP_REPEAT = 2 };
void launch_broadphase(const DevWorld& w, const StepParams& sp, cudaStream_t s, int num_sms,
                       const std::function<void(int)>& mark = nullptr, int mode = BP_AUTO);
void launch_set_transform(const DevWorld& w, int body, float px, float py, float angle, cudaStream_t s);
void launch_clear_forces(const DevWorld& w, cudaStream_t s);
void launch_collide_pairs(const ShapeRec* a, const float4* xa, const ShapeRec* b, const float4* xb, const int* kind,
                          int n, float4* geo, float4* pts, uint4* ids, cudaStream_t s);

/* world queries on the last step's LBVH (k_query.cu) */
void launch_ray_cast(const DevWorld& w, const float4* rays, const uint32_t* ray_world, int n, float4* out_a,
                     float4* out_b, cudaStream_t s);
void launch_query_aabb(const DevWorld& w, const float4* boxes, const uint32_t* box_world, int n, uint2* out, int cap,
                       int* count, cudaStream_t s);

/* primitives (k_prims.cu) */
void scan_exclusive_u32(const uint32_t* in, uint32_t* out, const int* d_n, int max_n, uint32_t* tmp, int* d_total,
                        cudaStream_t s);
/* stable LSD radix sort of (key, value) pairs by key bits [0, bits); n from device; result in *_a. */
void radix_sort_pairs(unsigned long long* key_a, uint32_t* val_a, unsigned long long* key_b, uint32_t* val_b,
                      const int* d_n, int max_n, int bits, uint32_t* hist, cudaStream_t s);
/* the same sort as one cooperative launch (2 grid barriers per 8-bit pass; inputs of at most
 * 2048 items are sorted by a single block, inputs of at most 8192 by a rank count in three small
 * kernels); uses cnt's barrier words. zero_or_max: the count is known to be 0 or max_n (no
 * rank-count launches when max_n is large). */
void radix_sort_pairs_coop(unsigned long long* key_a, uint32_t* val_a, unsigned long long* key_b, uint32_t* val_b,
                           const int* d_n, int max_n, int bits, uint32_t* hist, int* cnt, cudaStream_t s, int num_sms,
                           bool zero_or_max = false);
size_t radix_sort_hist_size(int max_n);
size_t scan_tmp_size(int max_n);

/* Host-side count of the kernels this library has launched (bench.py reports it per step). */
extern unsigned long long g_kernel_launches;
#define B2G_LAUNCHED(n) (::b2g::g_kernel_launches += (unsigned long long)(n))

/* multiprocessors of the current device, queried once per device ordinal (for the launchers of the
 * stand-alone routines, which have no world) */
int current_sm_count();

inline int grid_for(int n, int block, int max_blocks) {
    int g = (n + block - 1) / block;
    if (g < 1) g = 1;
    return g < max_blocks ? g : max_blocks;
}

}  // namespace b2g
#endif
