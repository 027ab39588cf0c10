/*
 * k_adjoint.cu — the step tape (recorded around the solver launch of each taped forward
 * step) and the backward pass over it.
 *
 * Recording (three small kernels per step, inside the step's CUDA graph):
 *   k_tape_record  after colouring: the solver slots in colour order with their frozen
 *                  manifolds, materials, masses and carried impulses; the colour offsets; the
 *                  step parameters; a checkpoint of every body every `ckpt_every` steps; and
 *                  for each manifold point the previous step's slot point its warm-start
 *                  impulse came from (the same feature-id match the narrowphase made).
 *   k_tape_post    after the solver: the number of position iterations each slot's island ran
 *                  (the per-island early exit of b2_island_private.rs:257-274).
 *   k_tape_advance one thread: step and slot counters.
 *
 * Backward, per checkpoint segment from the last to the first (one cooperative launch each):
 *   k_adj_replay   restores the segment's checkpoint and re-runs its steps with the templated
 *                  forward functions in f32 — the same IEEE operations in the same order as the
 *                  solver kernel, colour by colour — keeping every intermediate the reverse
 *                  sweep needs, and counts bodies whose replayed end state differs bit-wise
 *                  from the recorded one.
 *   k_adj_reverse  walks the segment backwards: position iterations, position integration,
 *                  velocity iterations, warm start, impulse carry to the previous step,
 *                  constraint initialisation, velocity integration.
 * Gauss-Seidel order is preserved in reverse: within a colour no dynamic body appears twice, so
 * the adjoints of dynamic bodies are updated without atomics; static and kinematic bodies,
 * which several slots of one colour may share, accumulate with atomicAdd.
 */
#include "b2g_sync.cuh"
#include "b2g_tape.h"

namespace b2g {
namespace {

using namespace adj;

constexpr int kBlock = 256;

__device__ __forceinline__ bool sync_all(int* cnt) {
    if (gridDim.x == 1) {
        __syncthreads();
        return true;
    }
    return grid_barrier(cnt);
}

/* ---------------- recording ---------------- */

__device__ __forceinline__ bool tape_ok(const TapeDev& t, long long step, long long base, int ncons) {
    return t.cnt[TAPE_CNT_STATUS] == 0 && step < t.step_cap && base + ncons <= t.slot_cap;
}

__global__ void k_tape_record(DevWorld w, TapeDev t, StepParams sp) {
    B2G_RETURN_IF_ABORTED(w);
    const long long step = t.cnt[TAPE_CNT_STEPS];
    const long long base = t.cnt[TAPE_CNT_SLOTS];
    const int ncons = w.cnt[CNT_CONS];
    const int ncol = w.cnt[CNT_COLOURS];
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gsize = gridDim.x * blockDim.x;
    if (!tape_ok(t, step, base, ncons)) {
        if (gtid == 0) t.cnt[TAPE_CNT_STATUS] |= (long long)TAPE_ST_OVERFLOW;
        return;
    }
    if (gtid == 0) {
        TapeStep s;
        s.dt = sp.dt;
        s.dt_ratio = sp.dt_ratio;
        s.gx = sp.gx;
        s.gy = sp.gy;
        s.vi = sp.vi;
        s.pi = sp.pi;
        s.warm = sp.warm;
        s.nslots = ncons;
        s.slot_off = base;
        s.ncol = ncol;
        s.ncontacts = w.cnt[CNT_CONTACTS];
        t.steps[step] = s;
    }
    for (int c = gtid; c <= ncol; c += gsize) t.col_off[(size_t)step * (kMaxColours + 1) + c] = w.col_off[c];
    if (blockIdx.x == 0) {
        /* the part-local layout: one row [n, offsets 0..n] per part, packed into the pool */
        __shared__ int s_row[kMaxParts + 2];
        const int np = w.cnt[CNT_INTERIOR] > 0 ? min(w.cnt[CNT_PARTS], t.max_parts) : 0;
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int q = 0; q < np; ++q) {
                s_row[q] = acc;
                acc += w.part_ncol[q] + 2;
            }
            const long long at = t.cnt[TAPE_CNT_POOL];
            if (w.cnt[CNT_INTERIOR] > 0 && w.cnt[CNT_PARTS] > t.max_parts) t.cnt[TAPE_CNT_STATUS] |= (long long)TAPE_ST_OVERFLOW;
            if (at + acc > t.pool_cap) {
                t.cnt[TAPE_CNT_STATUS] |= (long long)TAPE_ST_OVERFLOW;
                s_row[kMaxParts + 1] = -1;
            } else {
                t.cnt[TAPE_CNT_POOL] = at + acc;
                s_row[kMaxParts + 1] = (int)at;
                t.part_np[step] = np;
            }
        }
        __syncthreads();
        const int at = s_row[kMaxParts + 1];
        if (at >= 0) {
            for (int q = threadIdx.x; q < np; q += blockDim.x) {
                const int nc = w.part_ncol[q];
                int* row = t.part_pool + at + s_row[q];
                t.part_row[(size_t)step * t.max_parts + q] = at + s_row[q];
                row[0] = nc;
                for (int c = 0; c <= nc; ++c) row[1 + c] = w.part_off[(size_t)q * (kMaxColours + 1) + c];
            }
        }
    }
    if (step % t.ckpt_every == 0) {
        const size_t o = (size_t)(step / t.ckpt_every) * t.n_bodies;
        for (int b = gtid; b < t.n_bodies; b += gsize) {
            const float4 p = w.b_pos[b], v = w.b_vel[b];
            t.ckpt_pos[o + b] = make_float4(p.x, p.y, p.z, 0.0f);
            t.ckpt_vel[o + b] = make_float4(v.x, v.y, v.z, 0.0f);
        }
    }
    int nprev = 0;
    long long prev_off = 0;
    if (step > 0) {
        nprev = t.steps[step - 1].ncontacts;
        prev_off = t.steps[step - 1].slot_off;
    }
    unsigned long long* cur = t.cmap[step & 1];
    const unsigned long long* prev = t.cmap[(step + 1) & 1];
    for (int k = gtid; k < ncons; k += gsize) {
        const int ci = w.s_contact[k];
        const int2 bd = w.c.body[ci];
        const int2 fx = w.c.fix[ci];
        const uint4 ids = w.c.mids[ci];
        const int mtype = (int)(ids.z & 0xffu);
        const int count = (int)((ids.z >> 8) & 0xffu);
        const float4 massA = w.b_mass[bd.x], massB = w.b_mass[bd.y];
        const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
        const int dyn = ((w.b_flags[bd.x] & BF_TYPE_MASK) == BODY_DYNAMIC ? 1 : 0) |
                        ((w.b_flags[bd.y] & BF_TYPE_MASK) == BODY_DYNAMIC ? 2 : 0);
        int lo = 0, hi = ncol - 1;
        while (lo < hi) { /* last colour whose offset is <= k */
            const int mid = (lo + hi + 1) >> 1;
            if (w.col_off[mid] <= k) lo = mid;
            else hi = mid - 1;
        }
        TapeSlot s;
        s.idx = make_int4(bd.x, bd.y, count | (mtype << 8) | (dyn << 16), lo);
        s.geo = w.c.mgeo[ci];
        s.lp = w.c.mpts[ci];
        s.inv = make_float4(massA.y, massB.y, massA.w, massB.w);
        s.lc = make_float4(lcA.x, lcA.y, lcB.x, lcB.y);
        s.mat = w.c.mat[ci];
        s.rad = make_float4(w.f_shape[fx.x].radius, w.f_shape[fx.y].radius, __int_as_float(w.cons_island[w.s_cons[k]]),
                            __int_as_float(sp.pi));
        s.imp = w.c.mimp[ci];
        int carry[2] = {-1, -1};
        if (step > 0 && count > 0 && nprev > 0) {
            const unsigned long long key = w.c.key[ci];
            int a = 0, b = nprev - 1, found = -1;
            while (a <= b) {
                const int mid = (a + b) >> 1;
                const unsigned long long kk = w.c_alt.key[mid];
                if (kk == key) {
                    found = mid;
                    break;
                }
                if (kk < key) a = mid + 1;
                else b = mid - 1;
            }
            if (found >= 0) {
                const unsigned long long m = prev[found];
                if ((m >> 32) == (unsigned long long)step) {
                    const int pk = (int)(m & 0xffffffffull);
                    const int4 pc = t.slots[prev_off + pk].carry;
                    const int pcount = t.slots[prev_off + pk].idx.z & 0xff;
                    /* the narrowphase's impulse match (b2_contact.rs:277-298) */
                    for (int p = 0; p < count; ++p) {
                        const uint32_t id = p == 0 ? ids.x : ids.y;
                        if (pcount > 0 && (uint32_t)pc.z == id) carry[p] = pk * 2;
                        else if (pcount > 1 && (uint32_t)pc.w == id) carry[p] = pk * 2 + 1;
                    }
                }
            }
        }
        s.carry = make_int4(carry[0], carry[1], (int)ids.x, (int)ids.y);
        t.slots[base + k] = s;
        cur[ci] = ((unsigned long long)(step + 1) << 32) | (unsigned long long)(unsigned)k;
    }
}

__global__ void k_tape_post(DevWorld w, TapeDev t, StepParams sp) {
    B2G_RETURN_IF_ABORTED(w);
    const long long step = t.cnt[TAPE_CNT_STEPS];
    const long long base = t.cnt[TAPE_CNT_SLOTS];
    const int ncons = w.cnt[CNT_CONS];
    if (!tape_ok(t, step, base, ncons)) return;
    const float tol = 3.0f * kLinearSlop;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncons; k += gridDim.x * blockDim.x) {
        const int isl = w.vc_island[k];
        int n = sp.pi;
        for (int j = 0; j < sp.pi; ++j) {
            if (__uint_as_float(w.isl_minsep[(size_t)j * w.body_cap + isl]) <= tol) {
                n = j + 1;
                break;
            }
        }
        t.slots[base + k].rad.w = __int_as_float(n);
    }
}

__global__ void k_tape_advance(DevWorld w, TapeDev t) {
    B2G_RETURN_IF_ABORTED(w);
    const long long step = t.cnt[TAPE_CNT_STEPS];
    const long long base = t.cnt[TAPE_CNT_SLOTS];
    const int ncons = w.cnt[CNT_CONS];
    if (!tape_ok(t, step, base, ncons)) return;
    t.cnt[TAPE_CNT_STEPS] = step + 1;
    t.cnt[TAPE_CNT_SLOTS] = base + ncons;
}

__global__ void k_tape_snapshot(DevWorld w, TapeDev t, int index) {
    B2G_RETURN_IF_ABORTED(w);
    const size_t o = (size_t)index * t.n_bodies;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < t.n_bodies; b += gridDim.x * blockDim.x) {
        const float4 p = w.b_pos[b], v = w.b_vel[b];
        t.ckpt_pos[o + b] = make_float4(p.x, p.y, p.z, 0.0f);
        t.ckpt_vel[o + b] = make_float4(v.x, v.y, v.z, 0.0f);
    }
}

/* ---------------- backward ---------------- */

__device__ __forceinline__ SlotStatic slot_static(const TapeSlot& t) {
    SlotStatic s;
    s.a = t.idx.x;
    s.b = t.idx.y;
    s.count = t.idx.z & 0xff;
    s.mtype = (t.idx.z >> 8) & 0xff;
    s.flags = (t.idx.z >> 16) & 3;
    s.colour = t.idx.w;
    s.island = __float_as_int(t.rad.z);
    s.carry[0] = t.carry.x;
    s.carry[1] = t.carry.y;
    s.ln[0] = t.geo.x;
    s.ln[1] = t.geo.y;
    s.lpt[0] = t.geo.z;
    s.lpt[1] = t.geo.w;
    s.lp[0] = t.lp.x;
    s.lp[1] = t.lp.y;
    s.lp[2] = t.lp.z;
    s.lp[3] = t.lp.w;
    s.mA = t.inv.x;
    s.mB = t.inv.y;
    s.iA = t.inv.z;
    s.iB = t.inv.w;
    s.rA = t.rad.x;
    s.rB = t.rad.y;
    s.friction = t.mat.x;
    s.restitution = t.mat.y;
    s.threshold = t.mat.z;
    return s;
}

__device__ __forceinline__ BodyStatic body_static(const AdjWork& a, int b) {
    const float4 m = a.b_mass[b], d = a.b_damp[b];
    const float2 lc = a.b_lc[b];
    BodyStatic s;
    s.m = m.x;
    s.invm = m.y;
    s.I = m.z;
    s.invI = m.w;
    s.lin_damp = d.x;
    s.ang_damp = d.y;
    s.gscale = d.z;
    s.lcx = lc.x;
    s.lcy = lc.y;
    s.type = (int)(a.b_flags[b] & BF_TYPE_MASK);
    return s;
}

__device__ __forceinline__ int body_type(const AdjWork& a, int b) { return (int)(a.b_flags[b] & BF_TYPE_MASK); }

/* write back a body adjoint: dynamic bodies were loaded and are exclusive to this slot within
 * the colour; others were passed in as zero and their contributions are added atomically */
__device__ __forceinline__ void put_g(float4* g, int b, bool dyn, P2<float> gc, float ga) {
    if (dyn) {
        g[b] = make_float4(gc.x, gc.y, ga, 0.0f);
    } else {
        atomicAdd(&g[b].x, gc.x);
        atomicAdd(&g[b].y, gc.y);
        atomicAdd(&g[b].z, ga);
    }
}
__device__ __forceinline__ void get_g(const float4* g, int b, bool dyn, P2<float>& gc, float& ga) {
    if (dyn) {
        const float4 v = g[b];
        gc = p2(v.x, v.y);
        ga = v.z;
    } else {
        gc = p2(0.0f, 0.0f);
        ga = 0.0f;
    }
}

__device__ __forceinline__ float4* wv_rec(const AdjWork& a, int s, int it, int k) {
    return a.wv + (((size_t)s * a.max_vi + it) * a.max_slots + k) * 3;
}
__device__ __forceinline__ float4* wp_rec(const AdjWork& a, int s, int it, int k) {
    return a.wp + (((size_t)s * a.max_pi + it) * a.max_slots + k) * 2;
}

/* A taped step's solve order: the interior colours of each part (the parts are independent, so a
 * block sweeps whole parts, separated by __syncthreads), then the boundary colours grid-wide. */
struct StepOrder {
    const int* co;      /* boundary colour offsets */
    int ncol;
    int np;             /* parts (0: the step ran without) */
    const int* rows;    /* per part: its row in the pool */
    const int* pool;
};

__device__ __forceinline__ StepOrder step_order(const AdjWork& a, int t, const TapeStep& st) {
    StepOrder o;
    o.co = a.t.col_off + (size_t)t * (kMaxColours + 1);
    o.ncol = st.ncol;
    o.np = a.t.part_np[t];
    o.rows = a.t.part_row + (size_t)t * a.t.max_parts;
    o.pool = a.t.part_pool;
    return o;
}

/* fn(k) for every slot in solve order, each colour complete before the next */
template <class F>
__device__ __forceinline__ bool sweep_forward(const StepOrder& o, int* cnt, F&& fn) {
    if (o.np > 0) {
        for (int p = blockIdx.x; p < o.np; p += gridDim.x) {
            const int* row = o.pool + o.rows[p];
            const int nc = row[0];
            for (int c = 0; c < nc; ++c) {
                for (int k = row[1 + c] + threadIdx.x; k < row[2 + c]; k += blockDim.x) fn(k);
                __syncthreads();
            }
        }
        if (!sync_all(cnt)) return false;
    }
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gsize = gridDim.x * blockDim.x;
    for (int c = 0; c < o.ncol; ++c) {
        for (int k = o.co[c] + gtid; k < o.co[c + 1]; k += gsize) fn(k);
        if (!sync_all(cnt)) return false;
    }
    return true;
}

/* the same colours in the reverse order */
template <class F>
__device__ __forceinline__ bool sweep_reverse(const StepOrder& o, int* cnt, F&& fn) {
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x, gsize = gridDim.x * blockDim.x;
    for (int c = o.ncol - 1; c >= 0; --c) {
        for (int k = o.co[c] + gtid; k < o.co[c + 1]; k += gsize) fn(k);
        if (!sync_all(cnt)) return false;
    }
    if (o.np > 0) {
        for (int p = blockIdx.x; p < o.np; p += gridDim.x) {
            const int* row = o.pool + o.rows[p];
            for (int c = row[0] - 1; c >= 0; --c) {
                for (int k = row[1 + c] + threadIdx.x; k < row[2 + c]; k += blockDim.x) fn(k);
                __syncthreads();
            }
        }
        if (!sync_all(cnt)) return false;
    }
    return true;
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_adj_replay(AdjWork a) {
    grid_barrier_start();
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gsize = gridDim.x * blockDim.x;
    const int nb = a.nb;
    {
        const size_t o = (size_t)(a.t0 / a.t.ckpt_every) * nb;
        for (int b = gtid; b < nb; b += gsize) {
            a.cur_pos[b] = a.t.ckpt_pos[o + b];
            a.cur_vel[b] = a.t.ckpt_vel[o + b];
        }
    }
    if (!sync_all(a.cnt)) return;
    for (int t = a.t0; t < a.t1; ++t) {
        const int s = t - a.t0;
        const TapeStep st = a.t.steps[t];
        const TapeSlot* sl = a.t.slots + st.slot_off;
        const StepOrder order = step_order(a, t, st);
        const float h = st.dt;
        const int ns = st.nslots;
        float4* wsp = a.ws_pos + (size_t)s * nb;
        float4* wv1 = a.ws_vel1 + (size_t)s * nb;
        float4* wv2 = a.ws_vel2 + (size_t)s * nb;
        /* velocity integration (b2_island_private.rs:136-170) */
        for (int b = gtid; b < nb; b += gsize) {
            const float4 p = a.cur_pos[b];
            float4 v = a.cur_vel[b];
            wsp[b] = p;
            if (body_type(a, b) == BODY_DYNAMIC) {
                const BodyStatic bs = body_static(a, b);
                P2<float> vv = p2(v.x, v.y);
                float w = v.z;
                integrate_velocity(bs, h, st.gx, st.gy, vv, w);
                v = make_float4(vv.x, vv.y, w, v.w);
                a.cur_vel[b] = v;
            }
            wv1[b] = v;
        }
        if (!sync_all(a.cnt)) return;
        /* constraint initialisation and warm-start impulses */
        for (int k = gtid; k < ns; k += gsize) {
            const TapeSlot ts = sl[k];
            const SlotStatic ss = slot_static(ts);
            const float4 pA = a.cur_pos[ss.a], pB = a.cur_pos[ss.b];
            const float4 vA = a.cur_vel[ss.a], vB = a.cur_vel[ss.b];
            VC<float> vc;
            init_slot(ss, p2(pA.x, pA.y), pA.z, p2(pB.x, pB.y), pB.z, p2(vA.x, vA.y), vA.z, p2(vB.x, vB.y), vB.z,
                      p2(ts.lc.x, ts.lc.y), p2(ts.lc.z, ts.lc.w), vc);
            a.vc[k] = vc;
            float4 im = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (st.warm) {
                im.x = st.dt_ratio * ts.imp.x;
                im.y = st.dt_ratio * ts.imp.y;
                if (ss.count > 1) {
                    im.z = st.dt_ratio * ts.imp.z;
                    im.w = st.dt_ratio * ts.imp.w;
                }
            }
            a.imp[k] = im;
        }
        if (!sync_all(a.cnt)) return;
        if (st.warm) {
            const bool ok = sweep_forward(order, a.cnt, [&](int k) {
                    const SlotStatic ss = slot_static(sl[k]);
                    const float4 vA = a.cur_vel[ss.a], vB = a.cur_vel[ss.b];
                    float4* rec = a.ww + ((size_t)s * a.max_slots + k) * 2;
                    rec[0] = vA;
                    rec[1] = vB;
                    const VC<float> vc = a.vc[k];
                    const float4 im = a.imp[k];
                    const float ni[2] = {im.x, im.z}, ti[2] = {im.y, im.w};
                    P2<float> va = p2(vA.x, vA.y), vb = p2(vB.x, vB.y);
                    float wa = vA.z, wb = vB.z;
                    warm_slot(ss, vc, ni, ti, va, wa, vb, wb);
                    if (ss.flags & 1) a.cur_vel[ss.a] = make_float4(va.x, va.y, wa, vA.w);
                    if (ss.flags & 2) a.cur_vel[ss.b] = make_float4(vb.x, vb.y, wb, vB.w);
            });
            if (!ok) return;
        }
        /* velocity iterations */
        for (int it = 0; it < st.vi; ++it) {
            const bool ok = sweep_forward(order, a.cnt, [&](int k) {
                    const SlotStatic ss = slot_static(sl[k]);
                    const float4 vA = a.cur_vel[ss.a], vB = a.cur_vel[ss.b];
                    const float4 im = a.imp[k];
                    const VC<float> vc = a.vc[k];
                    float ni[2] = {im.x, im.z}, ti[2] = {im.y, im.w};
                    P2<float> va = p2(vA.x, vA.y), vb = p2(vB.x, vB.y);
                    float wa = vA.z, wb = vB.z;
                    VelDecision dec;
                    dec.fr[0] = dec.fr[1] = 0;
                    dec.nrm = 0;
                    solve_velocity(ss, vc, ni, ti, va, wa, vb, wb, dec, false);
                    float4* rec = wv_rec(a, s, it, k);
                    rec[0] = make_float4(vA.x, vA.y, vA.z, vB.x);
                    rec[1] = make_float4(vB.y, vB.z, __int_as_float(dec.fr[0] | (dec.fr[1] << 8) | (dec.nrm << 16)), 0.0f);
                    rec[2] = im;
                    a.imp[k] = make_float4(ni[0], ti[0], ni[1], ti[1]);
                    if (ss.flags & 1) a.cur_vel[ss.a] = make_float4(va.x, va.y, wa, vA.w);
                    if (ss.flags & 2) a.cur_vel[ss.b] = make_float4(vb.x, vb.y, wb, vB.w);
            });
            if (!ok) return;
        }
        /* position integration with the translation / rotation clamps */
        for (int b = gtid; b < nb; b += gsize) {
            if (body_type(a, b) == BODY_STATIC) continue;
            const float4 p = a.cur_pos[b];
            const float4 v = a.cur_vel[b];
            wv2[b] = v;
            P2<float> c = p2(p.x, p.y), vv = p2(v.x, v.y);
            float ang = p.z, w = v.z;
            unsigned char cl = 0;
            integrate_position(h, c, ang, vv, w, cl, false);
            a.cur_pos[b] = make_float4(c.x, c.y, ang, p.w);
            a.cur_vel[b] = make_float4(vv.x, vv.y, w, v.w);
        }
        if (!sync_all(a.cnt)) return;
        /* position iterations, each island for the number of iterations it ran */
        for (int it = 0; it < st.pi; ++it) {
            const bool ok = sweep_forward(order, a.cnt, [&](int k) {
                    const TapeSlot ts = sl[k];
                    if (it >= __float_as_int(ts.rad.w)) return;
                    const SlotStatic ss = slot_static(ts);
                    const float4 pA = a.cur_pos[ss.a], pB = a.cur_pos[ss.b];
                    P2<float> cA = p2(pA.x, pA.y), cB = p2(pB.x, pB.y);
                    float aA = pA.z, aB = pB.z;
                    unsigned char dec[2] = {0, 0};
                    solve_position(ss, p2(ts.lc.x, ts.lc.y), p2(ts.lc.z, ts.lc.w), cA, aA, cB, aB, dec, false);
                    float4* rec = wp_rec(a, s, it, k);
                    rec[0] = make_float4(pA.x, pA.y, pA.z, pB.x);
                    rec[1] = make_float4(pB.y, pB.z, __int_as_float(dec[0] | (dec[1] << 8)), 0.0f);
                    if (ss.flags & 1) a.cur_pos[ss.a] = make_float4(cA.x, cA.y, aA, pA.w);
                    if (ss.flags & 2) a.cur_pos[ss.b] = make_float4(cB.x, cB.y, aB, pB.w);
            });
            if (!ok) return;
        }
    }
    /* the replay must land on the recorded state bit for bit */
    for (int b = gtid; b < nb; b += gsize) {
        const float4 p = a.cur_pos[b], v = a.cur_vel[b];
        const float4 ep = a.end_pos[b], ev = a.end_vel[b];
        if (__float_as_uint(p.x) != __float_as_uint(ep.x) || __float_as_uint(p.y) != __float_as_uint(ep.y) ||
            __float_as_uint(p.z) != __float_as_uint(ep.z) || __float_as_uint(v.x) != __float_as_uint(ev.x) ||
            __float_as_uint(v.y) != __float_as_uint(ev.y) || __float_as_uint(v.z) != __float_as_uint(ev.z))
            atomicAdd(a.mismatch, 1u);
    }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_adj_reverse(AdjWork a) {
    grid_barrier_start();
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gsize = gridDim.x * blockDim.x;
    const int nb = a.nb;
    for (int t = a.t1 - 1; t >= a.t0; --t) {
        const int s = t - a.t0;
        const TapeStep st = a.t.steps[t];
        const TapeSlot* sl = a.t.slots + st.slot_off;
        const StepOrder order = step_order(a, t, st);
        const float h = st.dt;
        const int ns = st.nslots;
        const int nprev = t > 0 ? a.t.steps[t - 1].nslots : 0;
        const float4* wsp = a.ws_pos + (size_t)s * nb;
        const float4* wv1 = a.ws_vel1 + (size_t)s * nb;
        const float4* wv2 = a.ws_vel2 + (size_t)s * nb;
        float4* gend_cur = a.g_end[t & 1];
        float4* gend_prev = a.g_end[(t + 1) & 1];
        /* position iterations, last to first */
        for (int it = st.pi - 1; it >= 0; --it) {
            const bool ok = sweep_reverse(order, a.cnt, [&](int k) {
                    const TapeSlot ts = sl[k];
                    if (it >= __float_as_int(ts.rad.w)) return;
                    const SlotStatic ss = slot_static(ts);
                    const float4* rec = wp_rec(a, s, it, k);
                    const float4 r0 = rec[0], r1 = rec[1];
                    const int db = __float_as_int(r1.z);
                    const unsigned char dec[2] = {(unsigned char)(db & 0xff), (unsigned char)((db >> 8) & 0xff)};
                    const bool dA = ss.flags & 1, dB = ss.flags & 2;
                    P2<float> gcA, gcB;
                    float gaA, gaB;
                    get_g(a.g_pos, ss.a, dA, gcA, gaA);
                    get_g(a.g_pos, ss.b, dB, gcB, gaB);
                    solve_position_bwd(ss, p2(ts.lc.x, ts.lc.y), p2(ts.lc.z, ts.lc.w), p2(r0.x, r0.y), r0.z,
                                       p2(r0.w, r1.x), r1.y, dec, gcA, gaA, gcB, gaB);
                    put_g(a.g_pos, ss.a, dA, gcA, gaA);
                    put_g(a.g_pos, ss.b, dB, gcB, gaB);
            });
            if (!ok) return;
        }
        /* position integration; constraint data of the step again; impulse adjoints */
        for (int b = gtid; b < nb; b += gsize) {
            if (body_type(a, b) == BODY_STATIC) continue;
            const float4 v = wv2[b];
            P2<float> c0 = p2(0.0f, 0.0f), vv = p2(v.x, v.y);
            float a0 = 0.0f, w = v.z;
            unsigned char cl = 0;
            integrate_position(h, c0, a0, vv, w, cl, false);
            const float4 gp = a.g_pos[b], gv = a.g_vel[b];
            P2<float> gc = p2(gp.x, gp.y), gvv = p2(gv.x, gv.y);
            float ga = gp.z, gw = gv.z;
            integrate_position_bwd(h, p2(v.x, v.y), v.z, cl, gc, ga, gvv, gw);
            a.g_vel[b] = make_float4(gvv.x, gvv.y, gw, 0.0f);
        }
        for (int k = gtid; k < ns; k += gsize) {
            const TapeSlot ts = sl[k];
            const SlotStatic ss = slot_static(ts);
            const float4 pA = wsp[ss.a], pB = wsp[ss.b];
            const float4 vA = wv1[ss.a], vB = wv1[ss.b];
            VC<float> vc;
            init_slot(ss, p2(pA.x, pA.y), pA.z, p2(pB.x, pB.y), pB.z, p2(vA.x, vA.y), vA.z, p2(vB.x, vB.y), vB.z,
                      p2(ts.lc.x, ts.lc.y), p2(ts.lc.z, ts.lc.w), vc);
            a.vc[k] = vc;
            VCGrad<float> g;
            zero(g);
            a.gvc[k] = g;
            a.g_imp[k] = gend_cur[k];
        }
        for (int k = gtid; k < nprev; k += gsize) gend_prev[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (!sync_all(a.cnt)) return;
        /* velocity iterations, last to first */
        for (int it = st.vi - 1; it >= 0; --it) {
            const bool ok = sweep_reverse(order, a.cnt, [&](int k) {
                    const SlotStatic ss = slot_static(sl[k]);
                    const float4* rec = wv_rec(a, s, it, k);
                    const float4 r0 = rec[0], r1 = rec[1], r2 = rec[2];
                    const int db = __float_as_int(r1.z);
                    VelDecision dec;
                    dec.fr[0] = (unsigned char)(db & 0xff);
                    dec.fr[1] = (unsigned char)((db >> 8) & 0xff);
                    dec.nrm = (unsigned char)((db >> 16) & 0xff);
                    const float ni[2] = {r2.x, r2.z}, ti[2] = {r2.y, r2.w};
                    const VC<float> vc = a.vc[k];
                    VCGrad<float> g = a.gvc[k];
                    const float4 gi = a.g_imp[k];
                    float gni[2] = {gi.x, gi.z}, gti[2] = {gi.y, gi.w};
                    const bool dA = ss.flags & 1, dB = ss.flags & 2;
                    P2<float> gvA, gvB;
                    float gwA, gwB;
                    get_g(a.g_vel, ss.a, dA, gvA, gwA);
                    get_g(a.g_vel, ss.b, dB, gvB, gwB);
                    solve_velocity_bwd(ss, vc, dec, ni, ti, p2(r0.x, r0.y), r0.z, p2(r0.w, r1.x), r1.y, gni, gti, gvA,
                                       gwA, gvB, gwB, g);
                    a.gvc[k] = g;
                    a.g_imp[k] = make_float4(gni[0], gti[0], gni[1], gti[1]);
                    put_g(a.g_vel, ss.a, dA, gvA, gwA);
                    put_g(a.g_vel, ss.b, dB, gvB, gwB);
            });
            if (!ok) return;
        }
        /* warm start (reads the body adjoints only) and the impulse carry to the previous step */
        for (int k = gtid; k < ns; k += gsize) {
            const TapeSlot ts = sl[k];
            const SlotStatic ss = slot_static(ts);
            const VC<float> vc = a.vc[k];
            const float4 gi = a.g_imp[k];
            float gni[2] = {gi.x, gi.z}, gti[2] = {gi.y, gi.w};
            if (st.warm) {
                VCGrad<float> g = a.gvc[k];
                const float4 ga = a.g_vel[ss.a], gb = a.g_vel[ss.b];
                float ni0[2] = {st.dt_ratio * ts.imp.x, 0.0f}, ti0[2] = {st.dt_ratio * ts.imp.y, 0.0f};
                if (ss.count > 1) {
                    ni0[1] = st.dt_ratio * ts.imp.z;
                    ti0[1] = st.dt_ratio * ts.imp.w;
                }
                warm_slot_bwd(ss, vc, ni0, ti0, p2(ga.x, ga.y), ga.z, p2(gb.x, gb.y), gb.z, gni, gti, g);
                a.gvc[k] = g;
            }
            const float4 ge = gend_cur[k];
            const float pass[4] = {ge.x, ge.y, ge.z, ge.w};
            float* gp = (float*)gend_prev;
            for (int j = 0; j < ss.count; ++j) {
                float gn, gt;
                if (j < vc.vcount) {
                    gn = st.warm ? st.dt_ratio * gni[j] : 0.0f;
                    gt = st.warm ? st.dt_ratio * gti[j] : 0.0f;
                } else {
                    /* a point the reduced block solver left alone keeps its carried impulse */
                    gn = pass[2 * j];
                    gt = pass[2 * j + 1];
                }
                const int cj = ss.carry[j];
                if (cj >= 0 && t > 0) {
                    atomicAdd(gp + (size_t)cj * 2, gn);
                    atomicAdd(gp + (size_t)cj * 2 + 1, gt);
                }
            }
        }
        if (!sync_all(a.cnt)) return;
        /* constraint initialisation, colour by colour */
        {
            const bool ok = sweep_reverse(order, a.cnt, [&](int k) {
                const TapeSlot ts = sl[k];
                const SlotStatic ss = slot_static(ts);
                const float4 pA = wsp[ss.a], pB = wsp[ss.b];
                const float4 vA = wv1[ss.a], vB = wv1[ss.b];
                const bool dA = ss.flags & 1, dB = ss.flags & 2;
                P2<float> gcA, gcB, gvA, gvB;
                float gaA, gaB, gwA, gwB;
                get_g(a.g_pos, ss.a, dA, gcA, gaA);
                get_g(a.g_pos, ss.b, dB, gcB, gaB);
                get_g(a.g_vel, ss.a, dA, gvA, gwA);
                get_g(a.g_vel, ss.b, dB, gvB, gwB);
                init_slot_bwd(ss, p2(pA.x, pA.y), pA.z, p2(pB.x, pB.y), pB.z, p2(vA.x, vA.y), vA.z, p2(vB.x, vB.y),
                              vB.z, p2(ts.lc.x, ts.lc.y), p2(ts.lc.z, ts.lc.w), a.vc[k], a.gvc[k], gcA, gaA, gcB, gaB,
                              gvA, gwA, gvB, gwB);
                put_g(a.g_pos, ss.a, dA, gcA, gaA);
                put_g(a.g_pos, ss.b, dB, gcB, gaB);
                put_g(a.g_vel, ss.a, dA, gvA, gwA);
                put_g(a.g_vel, ss.b, dB, gvB, gwB);
            });
            if (!ok) return;
        }
        /* velocity integration */
        for (int b = gtid; b < nb; b += gsize) {
            if (body_type(a, b) != BODY_DYNAMIC) continue;
            const BodyStatic bs = body_static(a, b);
            const float4 gv = a.g_vel[b];
            P2<float> gvv = p2(gv.x, gv.y);
            float gw = gv.z;
            integrate_velocity_bwd(bs, h, gvv, gw);
            a.g_vel[b] = make_float4(gvv.x, gvv.y, gw, 0.0f);
        }
        if (!sync_all(a.cnt)) return;
    }
}

/* one block per SM, like the forward solver: the sweeps are bound by grid-barrier latency, which
 * grows with the number of arriving blocks */
int coop_blocks_for(const void* fn, int block, int num_sms) {
    (void)fn;
    (void)block;
    return num_sms;
}

}  // namespace

void launch_tape_record(const DevWorld& w, const TapeDev& t, const StepParams& sp, cudaStream_t s, int num_sms) {
    k_tape_record<<<num_sms * 2, kBlock, 0, s>>>(w, t, sp);
    B2G_LAUNCHED(1);
}

void launch_tape_post(const DevWorld& w, const TapeDev& t, const StepParams& sp, cudaStream_t s, int num_sms) {
    k_tape_post<<<num_sms * 2, kBlock, 0, s>>>(w, t, sp);
    k_tape_advance<<<1, 1, 0, s>>>(w, t);
    B2G_LAUNCHED(2);
}

void launch_tape_snapshot(const DevWorld& w, const TapeDev& t, int index, cudaStream_t s) {
    k_tape_snapshot<<<grid_for(t.n_bodies, kBlock, w.num_sms * 4), kBlock, 0, s>>>(w, t, index);
    B2G_LAUNCHED(1);
}

/* Small problems run in one block (block-level barriers); larger ones as a cooperative grid of
 * at most two blocks per SM. */
int launch_adjoint_segment(const AdjWork& a, cudaStream_t s, int num_sms) {
    AdjWork ac = a;
    void* args[] = {&ac};
    const bool single = a.max_slots <= 4096 && a.nb <= 16384;
    cudaError_t e;
    int* bar = a.cnt + CNT_BARRIER;
    if (single) {
        e = cudaLaunchCooperativeKernel((const void*)k_adj_replay<512>, dim3(1), dim3(512), args, 0, s);
        if (e == cudaSuccess)
            e = cudaLaunchCooperativeKernel((const void*)k_adj_reverse<512>, dim3(1), dim3(512), args, 0, s);
    } else {
        static int br = 0, bv = 0;
        if (!br) br = coop_blocks_for((const void*)k_adj_replay<kBlock>, kBlock, num_sms);
        if (!bv) bv = coop_blocks_for((const void*)k_adj_reverse<kBlock>, kBlock, num_sms);
        e = cudaMemsetAsync(bar, 0, sizeof(int), s);
        if (e == cudaSuccess)
            e = cudaLaunchCooperativeKernel((const void*)k_adj_replay<kBlock>, dim3(br), dim3(kBlock), args, 0, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(bar, 0, sizeof(int), s);
        if (e == cudaSuccess)
            e = cudaLaunchCooperativeKernel((const void*)k_adj_reverse<kBlock>, dim3(bv), dim3(kBlock), args, 0, s);
    }
    B2G_LAUNCHED(2);
    return (int)e;
}

}  // namespace b2g
