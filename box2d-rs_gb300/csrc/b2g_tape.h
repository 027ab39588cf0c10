/*
 * b2g_tape.h — device layout of the step tape (recorded during forward steps) and of the
 * work buffers of the backward pass.
 *
 * Per taped step the tape holds the solver's frozen structure: one TapeSlot per contact
 * constraint in solver order (slots grouped by colour), the colour offsets, the step
 * parameters, and every `ckpt_every` steps a checkpoint of all bodies' solver state
 * (centre of mass, angle, linear and angular velocity). The backward pass replays each
 * checkpoint segment forward in f32 (bit-identical to the solver kernel), keeping every
 * intermediate of the segment, then runs the hand-written adjoint in reverse.
 */
#ifndef B2G_TAPE_H
#define B2G_TAPE_H

#include "b2g_adjoint.cuh"
#include "b2g_internal.h"

namespace b2g {

/* one constraint of one taped step; 144 bytes, the layout of b2g_tape_slot */
struct TapeSlot {
    int4 idx;      /* body A, body B, count | manifold type << 8 | dynamic flags << 16, colour */
    float4 geo;    /* local normal, local point */
    float4 lp;     /* manifold point 0, point 1 (local) */
    float4 inv;    /* inverse masses and inertias of A and B */
    float4 lc;     /* local centres of A and B */
    float4 mat;    /* friction, restitution, restitution threshold, tangent speed */
    float4 rad;    /* radius A, radius B, island (int bits), position iterations run (int bits) */
    float4 imp;    /* warm-start impulses as carried into the step (before dt_ratio) */
    int4 carry;    /* per point: previous step's slot * 2 + point the impulse came from, or -1;
                      feature ids of points 0 and 1 */
};
static_assert(sizeof(TapeSlot) == 144, "TapeSlot layout");

/* 48 bytes, the layout of b2g_tape_step */
struct TapeStep {
    float dt, dt_ratio, gx, gy;
    int vi, pi, warm, nslots;
    long long slot_off;
    int ncol, ncontacts;
};
static_assert(sizeof(TapeStep) == 48, "TapeStep layout");

enum { TAPE_CNT_STEPS = 0, TAPE_CNT_SLOTS = 1, TAPE_CNT_STATUS = 2, TAPE_CNT_POOL = 3, TAPE_CNT_SIZE = 4 };
enum : unsigned long long { TAPE_ST_OVERFLOW = 1ull };

struct TapeDev {
    TapeSlot* slots;
    long long slot_cap;
    TapeStep* steps;
    int step_cap;
    int ckpt_every;
    int* col_off;                    /* step_cap x (kMaxColours + 1): boundary colour offsets (all
                                        colours of a step solved without parts) */
    int* part_np;                    /* step_cap: parts of the step's part-local solve (0: none) */
    int* part_row;                   /* step_cap x max_parts: each part's row in part_pool */
    int* part_pool;                  /* rows [colours n, offset 0 .. offset n] of the parts' interior
                                        colours */
    long long pool_cap;
    int max_parts;
    unsigned long long* cmap[2];     /* per step parity, per contact: (step + 1) << 32 | slot */
    float4* ckpt_pos;                /* (step_cap / ckpt_every + 2) x n_bodies: c.x, c.y, a, - */
    float4* ckpt_vel;                /* v.x, v.y, w, - */
    int n_bodies;
    long long* cnt;                  /* TAPE_CNT_* */
};

/* work buffers of one backward pass (sized for one segment of `seg` steps) */
struct AdjWork {
    TapeDev t;
    const float4* b_mass;
    const float4* b_damp;
    const uint32_t* b_flags;
    const float2* b_lc;
    int nb;
    int t0, t1;                      /* the segment [t0, t1) */
    int max_slots, max_vi, max_pi;
    const float4* end_pos;           /* state after the segment's last step (checkpoint or final) */
    const float4* end_vel;
    /* forward replay */
    float4 *cur_pos, *cur_vel;       /* nb */
    float4 *ws_pos, *ws_vel1, *ws_vel2;  /* seg x nb: start pose, velocity after integration,
                                            velocity before position integration */
    adj::VC<float>* vc;              /* max_slots */
    float4* imp;                     /* max_slots */
    float4* wv;                      /* seg x max_vi x max_slots x 3: pre-update velocities and
                                        impulses, decisions */
    float4* ww;                      /* seg x max_slots x 2: velocities before the warm start */
    float4* wp;                      /* seg x max_pi x max_slots x 2: poses before each position
                                        update, decisions */
    /* reverse */
    float4 *g_pos, *g_vel;           /* nb */
    adj::VCGrad<float>* gvc;         /* max_slots */
    float4* g_imp;                   /* max_slots */
    float4* g_end[2];                /* per step parity, max_slots: adjoint of the stored impulses */
    int* cnt;                        /* barrier block (CNT_SIZE ints) */
    unsigned* mismatch;              /* replayed state differing from the recorded one (bodies) */
};

/* forward recording, around the solver launch of a taped step */
void launch_tape_record(const DevWorld& w, const TapeDev& t, const StepParams& sp, cudaStream_t s, int num_sms);
void launch_tape_post(const DevWorld& w, const TapeDev& t, const StepParams& sp, cudaStream_t s, int num_sms);
/* copy the current body state into checkpoint slot `index` */
void launch_tape_snapshot(const DevWorld& w, const TapeDev& t, int index, cudaStream_t s);
/* one backward segment: replay [t0, t1) forward, then reverse it */
int launch_adjoint_segment(const AdjWork& a, cudaStream_t s, int num_sms);

}  // namespace b2g
#endif
